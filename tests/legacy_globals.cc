// Test harness for steps_gb300/legacy/forces_gb300.cc: defines the StePS
// globals the shim reads (types as StePS/src/global_variables.h declares
// them) and a C API to fill them and call the driver-facing force symbol.
#include <stdlib.h>
#include <string.h>

#include <vector>

#ifdef USE_SINGLE_PRECISION
typedef float REAL;
#else
typedef double REAL;
#endif

int IS_PERIODIC, COSMOLOGY, COMOVING_INTEGRATION;
REAL L, Rsim;
bool ForceError;
int n_GPU = 1, rank = 0;
REAL *M, *SOFT_LENGTH;
int N;
REAL beta, ParticleRadi, rho_part, M_min, mass_in_unit_sphere;
double Omega_lambda, H0;
#ifdef PERIODIC
REAL *T3_EWALD_FORCE_TABLE;
int N_EWALD_FORCE_GRID;
#elif defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
REAL *S1R2_EWALD_FORCE_TABLE;
int Nz_EWALD_FORCE_GRID, Nrho_EWALD_FORCE_GRID;
#endif
#if defined(PERIODIC_Z)
int RADIAL_FORCE_TABLE_SIZE;
REAL *RADIAL_FORCE_TABLE;
#endif

void forces(REAL *x, REAL *F, int ID_min, int ID_max);
void forces_periodic(REAL *x, REAL *F, int ID_min, int ID_max);
void forces_periodic_z(REAL *x, REAL *F, int ID_min, int ID_max);
void recalculate_softening();
extern "C" void steps_gb300_legacy_precision(int precision);

extern "C" {
void h_set(int n, const double *m, const double *eps, int is_periodic, double l, double rsim, int cosmology,
           int comoving, double mius)
{
    N = n;
    M = (REAL *)realloc(M, sizeof(REAL) * n);
    SOFT_LENGTH = (REAL *)realloc(SOFT_LENGTH, sizeof(REAL) * n);
    for (int i = 0; i < n; i++) { M[i] = m[i]; SOFT_LENGTH[i] = eps[i]; }
    IS_PERIODIC = is_periodic;
    L = l;
    Rsim = rsim;
    COSMOLOGY = cosmology;
    COMOVING_INTEGRATION = comoving;
    mass_in_unit_sphere = mius;
}
void h_table(const double *t, int a, int b)
{
#ifdef PERIODIC
    size_t cnt = 3ull * a * a * a;
    T3_EWALD_FORCE_TABLE = (REAL *)realloc(T3_EWALD_FORCE_TABLE, sizeof(REAL) * cnt);
    for (size_t i = 0; i < cnt; i++) T3_EWALD_FORCE_TABLE[i] = t[i];
    N_EWALD_FORCE_GRID = a;
#elif defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
    size_t cnt = 2ull * a * b;
    S1R2_EWALD_FORCE_TABLE = (REAL *)realloc(S1R2_EWALD_FORCE_TABLE, sizeof(REAL) * cnt);
    for (size_t i = 0; i < cnt; i++) S1R2_EWALD_FORCE_TABLE[i] = t[i];
    Nrho_EWALD_FORCE_GRID = a;
    Nz_EWALD_FORCE_GRID = b;
#else
    (void)t; (void)a; (void)b;
#endif
}
void h_precision(int p) { steps_gb300_legacy_precision(p); }
// Sets the globals recalculate_softening reads, calls it, returns beta and
// rho_part (host only: no GPU context is created).
void h_softening(double radius, double m_min, int cosmology, double *beta_out, double *rho_out)
{
    ParticleRadi = radius;
    M_min = m_min;
    COSMOLOGY = cosmology;
    rho_part = 0;
    recalculate_softening();
    *beta_out = beta;
    *rho_out = rho_part;
}
// Positions and forces pass through REAL arrays, as the driver holds them
// (float in a USE_SINGLE_PRECISION build, StePS/src/global_variables.h:26-32).
int h_forces(double *x, double *F, int id_min, int id_max)
{
    ForceError = false;
    const int ni = id_max - id_min + 1;
    std::vector<REAL> xr(x, x + 3 * (size_t)N), Fr(3 * (size_t)(ni > 0 ? ni : 1));
    for (int k = 0; k < 3 * (ni > 0 ? ni : 1); k++) Fr[k] = (REAL)F[k];
#if defined(PERIODIC)
    forces_periodic(xr.data(), Fr.data(), id_min, id_max);
#elif defined(PERIODIC_Z)
    forces_periodic_z(xr.data(), Fr.data(), id_min, id_max);
#else
    forces(xr.data(), Fr.data(), id_min, id_max);
#endif
    for (int k = 0; k < 3 * (ni > 0 ? ni : 0); k++) F[k] = Fr[k];
    return ForceError ? 1 : 0;
}
}
