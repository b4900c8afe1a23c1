/* Test-infrastructure harness around the UNMODIFIED reference StePS CPU
 * force path (StePS/src/forces.cc, ewald_space.cc, utils.cc, step.cc,
 * friedmann_solver.cc), compiled from the reference tree by oracle/Makefile
 * into oracle/_ref/libref_<variant>.so.
 *
 * The reference keeps all state in globals that StePS/src/main.cc defines
 * (StePS/src/main.cc:37-146); this file defines that storage and exposes a
 * small extern "C" API so the tests can drive the reference's own
 * forces / forces_periodic / forces_periodic_z (forces.cc:510, :776, :1221),
 * step() (step.cc:100) and the Ewald table builders (ewald_space.cc:118,
 * :288, :754) on seeded inputs. Nothing here is shipped or timed as product.
 */
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "mpi.h"
#include "global_variables.h"

/* ---- storage for the reference's globals (main.cc:37-146) ---- */
int t, N;
REAL SOFT_CONST[8];
REAL w[3];
double a_max;
REAL *x, *v, *F;
double h, h_min, h_max, T, t_next, t_bigbang;
REAL ACC_PARAM;
double rho_crit;
REAL mass_in_unit_sphere;
int n_GPU = 1;
int numtasks = 1, rank = 0;
int N_mpi_thread;
int ID_MPI_min, ID_MPI_max;
MPI_Status Stat;
int BUFFER_start_ID;
REAL *F_buffer;
REAL x4, err, errmax;
REAL beta, ParticleRadi, rho_part, M_min;
int IS_PERIODIC, COSMOLOGY;
int COMOVING_INTEGRATION;
REAL L, Rsim;
double Omega_b, Omega_lambda, Omega_dm, Omega_r, Omega_k, Omega_m, H0, Hubble_param, Decel_param, delta_Hubble_param;
REAL *M;
REAL *SOFT_LENGTH;
REAL M_tmp;
double a = 1.0, a_start, a_prev, a_tmp;
double Omega_m_eff;
double delta_a;
int e[2202][4];
int el;
bool ForceError;
#ifdef PERIODIC
REAL *T3_EWALD_FORCE_TABLE;
int N_EWALD_FORCE_GRID;
#endif
#if defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
REAL *S1R2_EWALD_FORCE_TABLE;
int Nz_EWALD_FORCE_GRID;
int Nrho_EWALD_FORCE_GRID;
#endif
#if defined(PERIODIC_Z) && defined(PERIODIC_Z_NOLOOKUP)
int ewald_max;
REAL ewald_cut;
#endif
#if defined(PERIODIC_Z)
int RADIAL_FORCE_TABLE_SIZE;
int RADIAL_FORCE_ACCURACY;
REAL *RADIAL_FORCE_TABLE;
#endif

/* ---- reference functions defined in the other reference objects ---- */
void forces(REAL *x, REAL *F, int ID_min, int ID_max);
void forces_periodic(REAL *x, REAL *F, int ID_min, int ID_max);
void forces_periodic_z(REAL *x, REAL *F, int ID_min, int ID_max);
void step(REAL *x, REAL *v, REAL *F);
void calculate_softening_length(REAL *SOFT_LENGTH, REAL *M, int N);
REAL force_softening(REAL r, REAL beta);
#ifdef PERIODIC
int ewald_space(REAL R, int ewald_index[][4]);
void calculate_t3_ewald_lookup_table(int Ngrid, REAL L, REAL alpha, int realspace_el, int recspace_el,
                                     int realspace_ewald_index[][4], int recspace_ewald_index[][4],
                                     REAL rel_cut, REAL rec_cut, REAL *T3_EWALD_FORCE_TABLE);
void ewald_interpolate_D(int Ngrid, REAL L, const REAL *T3_EWALD_FORCE_TABLE, const REAL dx, const REAL dy,
                         const REAL dz, REAL D[3], int order);
#endif
#if defined(PERIODIC_Z)
void get_cylindrical_force_table(REAL *FORCE_TABLE, REAL R, REAL Lz, int TABLE_SIZE, int RADIAL_FORCE_ACCURACY);
#endif
#if defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
void calculate_S1R2ewald_correction_table(int Nrho, int Nz, REAL rho_max, REAL Lz, REAL alpha, int nmax, int mmax,
                                          REAL *&S1R2_EWALD_FORCE_TABLE);
void S1R2ewald_force_pair(double dx, double dy, double dz, double Lz, double alpha, int nmax, int mmax, double &Fx,
                          double &Fy, double &Fz);
void ewald_interpolate_D(const REAL *T, int Nrho, int Nz, REAL rho_max, REAL Lz, REAL dx, REAL dy, REAL dz, REAL &Dx,
                         REAL &Dy, REAL &Dz);
#endif

static void *xrealloc(void *p, size_t n) { return realloc(p, n ? n : 1); }

extern "C" {

/* Topology compiled into this variant: 0 = R^3, 1 = T^3, 2 = S1xR2 table, 3 = S1xR2 image sum. */
int ref_topology(void)
{
#if defined(PERIODIC)
    return 1;
#elif defined(PERIODIC_Z) && defined(PERIODIC_Z_NOLOOKUP)
    return 3;
#elif defined(PERIODIC_Z)
    return 2;
#else
    return 0;
#endif
}

int ref_interp_order(void)
{
#ifdef EWALD_INTERPOLATION_ORDER
    return EWALD_INTERPOLATION_ORDER;
#else
    return -1;
#endif
}

void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

/* Copies N particles (AoS x[3N], masses, softening lengths) into the globals. */
void ref_set_particles(int n, const double *xin, const double *m, const double *eps)
{
    N = n;
    x = (REAL *)xrealloc(x, sizeof(REAL) * 3 * (size_t)n);
    v = (REAL *)xrealloc(v, sizeof(REAL) * 3 * (size_t)n);
    F = (REAL *)xrealloc(F, sizeof(REAL) * 3 * (size_t)n);
    M = (REAL *)xrealloc(M, sizeof(REAL) * (size_t)n);
    SOFT_LENGTH = (REAL *)xrealloc(SOFT_LENGTH, sizeof(REAL) * (size_t)n);
    for (int i = 0; i < 3 * n; i++) { x[i] = (REAL)xin[i]; v[i] = 0; F[i] = 0; }
    for (int i = 0; i < n; i++) { M[i] = (REAL)m[i]; SOFT_LENGTH[i] = (REAL)eps[i]; }
}

/* Overwrites the velocities v[3N] (set_particles starts them at zero). */
void ref_set_velocities(const double *vin)
{
    for (int i = 0; i < 3 * N; i++) v[i] = (REAL)vin[i];
}

/* The reference's own softening law (utils.cc:59-82) with PARTICLE_RADII = radius.
 * Overwrites SOFT_LENGTH and returns it in eps_out; also sets M_min and rho_part. */
void ref_softening(double radius, double *eps_out)
{
    ParticleRadi = (REAL)radius;
    calculate_softening_length(SOFT_LENGTH, M, N);
    for (int i = 0; i < N; i++) eps_out[i] = SOFT_LENGTH[i];
}

void ref_set_params(int is_periodic, double box_l, double rsim, int cosmology, int comoving, double mius, double h0,
                    double omega_lambda)
{
    IS_PERIODIC = is_periodic;
    L = (REAL)box_l;
    Rsim = (REAL)rsim;
    COSMOLOGY = cosmology;
    COMOVING_INTEGRATION = comoving;
    mass_in_unit_sphere = (REAL)mius;
    H0 = h0;
    Omega_lambda = omega_lambda;
    a = 1.0;
    Hubble_param = 0.0;
#if defined(PERIODIC_Z) && defined(PERIODIC_Z_NOLOOKUP)
    /* main.cc:1270-1271 (the same values forces_cuda.cu:659-660 derives in-kernel). */
    ewald_max = IS_PERIODIC + 1;
    ewald_cut = ((REAL)ewald_max) - 0.4;
#endif
}

/* One reference force evaluation for i in [id_min, id_max]; F_out gets 3*(id_max-id_min+1) values. */
void ref_forces(double *F_out, int id_min, int id_max)
{
    int ni = id_max - id_min + 1;
    N_mpi_thread = ni;
    REAL *Fl = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)(ni > 0 ? ni : 1));
#if defined(PERIODIC)
    forces_periodic(x, Fl, id_min, id_max);
#elif defined(PERIODIC_Z)
    forces_periodic_z(x, Fl, id_min, id_max);
#else
    forces(x, Fl, id_min, id_max);
#endif
    for (int i = 0; i < 3 * ni; i++) F_out[i] = Fl[i];
    free(Fl);
}

/* Fixed-step KDK through the reference's step() (step.cc:100): F must hold the
 * forces of the current positions (call ref_forces_full first). */
void ref_forces_full(void)
{
    N_mpi_thread = N;
    ID_MPI_min = 0;
    ID_MPI_max = N - 1;
#if defined(PERIODIC)
    forces_periodic(x, F, 0, N - 1);
#elif defined(PERIODIC_Z)
    forces_periodic_z(x, F, 0, N - 1);
#else
    forces(x, F, 0, N - 1);
#endif
}

void ref_step(double dt)
{
    h = dt;
    N_mpi_thread = N;
    ID_MPI_min = 0;
    ID_MPI_max = N - 1;
    step(x, v, F);
}

double ref_errmax(void) { return (double)errmax; }

void ref_get_state(double *xo, double *vo, double *Fo)
{
    for (int i = 0; i < 3 * N; i++) { xo[i] = x[i]; vo[i] = v[i]; Fo[i] = F[i]; }
}

#ifndef STEPS_HARNESS_NO_SOFTENING_PROBE
/* force_softening lives in the reference's force TU (forces.cc:52); a build
 * that links another force TU (tests/test_legacy_link.py) leaves it out. */
double ref_force_softening(double r, double b) { return (double)force_softening((REAL)r, (REAL)b); }
#endif

#ifdef PERIODIC
/* Builds the T^3 Ewald correction table exactly as main.cc:467-470 does:
 * index sets ewald_space(real_radius) and ewald_space(rec_radius), then
 * calculate_t3_ewald_lookup_table. Returns ngrid^3*3 doubles in out. */
int ref_build_t3_table(int ngrid, double box_l, double alpha, double rel_cut, double rec_cut, double real_radius,
                       double rec_radius, double *out)
{
    static int real_idx[40000][4];
    static int rec_idx[40000][4];
    int nreal = ewald_space((REAL)real_radius, real_idx);
    int nrec = ewald_space((REAL)rec_radius, rec_idx);
    REAL *tab = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)ngrid * ngrid * ngrid);
    calculate_t3_ewald_lookup_table(ngrid, (REAL)box_l, (REAL)alpha, nreal, nrec, real_idx, rec_idx, (REAL)rel_cut,
                                    (REAL)rec_cut, tab);
    for (size_t i = 0; i < 3 * (size_t)ngrid * ngrid * ngrid; i++) out[i] = tab[i];
    free(tab);
    return nreal * 100000 + nrec;
}

int ref_ewald_space(double radius, int *out4, int cap)
{
    static int idx[40000][4];
    int last = ewald_space((REAL)radius, idx);
    for (int i = 0; i <= last && i < cap; i++)
        for (int k = 0; k < 4; k++) out4[4 * i + k] = idx[i][k];
    return last;
}

void ref_set_t3_table(const double *tab, int ngrid)
{
    N_EWALD_FORCE_GRID = ngrid;
    size_t n = 3 * (size_t)ngrid * ngrid * ngrid;
    T3_EWALD_FORCE_TABLE = (REAL *)xrealloc(T3_EWALD_FORCE_TABLE, sizeof(REAL) * n);
    for (size_t i = 0; i < n; i++) T3_EWALD_FORCE_TABLE[i] = (REAL)tab[i];
}

void ref_t3_interp(double dx, double dy, double dz, double *D3)
{
    REAL D[3];
    ewald_interpolate_D(N_EWALD_FORCE_GRID, L, T3_EWALD_FORCE_TABLE, (REAL)dx, (REAL)dy, (REAL)dz, D,
                        EWALD_INTERPOLATION_ORDER);
    D3[0] = D[0]; D3[1] = D[1]; D3[2] = D[2];
}
#endif

#if defined(PERIODIC_Z)
void ref_cyl_table(double R, double Lz, int size, int accuracy, double *out)
{
    REAL *tab = (REAL *)malloc(sizeof(REAL) * (size_t)size);
    get_cylindrical_force_table(tab, (REAL)R, (REAL)Lz, size, accuracy);
    for (int i = 0; i < size; i++) out[i] = tab[i];
    free(tab);
}

void ref_set_radial_table(const double *tab, int size)
{
    RADIAL_FORCE_TABLE_SIZE = size;
    RADIAL_FORCE_TABLE = (REAL *)xrealloc(RADIAL_FORCE_TABLE, sizeof(REAL) * (size_t)size);
    for (int i = 0; i < size; i++) RADIAL_FORCE_TABLE[i] = (REAL)tab[i];
}
#endif

#if defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
/* S1xR2 (rho,z) correction table as main.cc:649 builds it (Tornberg 2015 Ewald sums). */
void ref_build_s1r2_table(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax, double *out)
{
    REAL *tab = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)nrho * nz);
    calculate_S1R2ewald_correction_table(nrho, nz, (REAL)rho_max, (REAL)lz, (REAL)alpha, nmax, mmax, tab);
    for (size_t i = 0; i < 2 * (size_t)nrho * nz; i++) out[i] = tab[i];
    free(tab);
}

void ref_s1r2_pair(double dx, double dy, double dz, double lz, double alpha, int nmax, int mmax, double *F3)
{
    S1R2ewald_force_pair(dx, dy, dz, lz, alpha, nmax, mmax, F3[0], F3[1], F3[2]);
}

void ref_set_s1r2_table(const double *tab, int nrho, int nz)
{
    Nrho_EWALD_FORCE_GRID = nrho;
    Nz_EWALD_FORCE_GRID = nz;
    size_t n = 2 * (size_t)nrho * nz;
    S1R2_EWALD_FORCE_TABLE = (REAL *)xrealloc(S1R2_EWALD_FORCE_TABLE, sizeof(REAL) * n);
    for (size_t i = 0; i < n; i++) S1R2_EWALD_FORCE_TABLE[i] = (REAL)tab[i];
}

void ref_s1r2_interp(double dx, double dy, double dz, double *D3)
{
    REAL Dx, Dy, Dz;
    ewald_interpolate_D(S1R2_EWALD_FORCE_TABLE, Nrho_EWALD_FORCE_GRID, Nz_EWALD_FORCE_GRID,
                        EWALD_LOOKUP_TABLE_RADIAL_EXTENT_FACTOR * Rsim, L, (REAL)dx, (REAL)dy, (REAL)dz, Dx, Dy, Dz);
    D3[0] = Dx; D3[1] = Dy; D3[2] = Dz;
}
#endif

} /* extern "C" */
