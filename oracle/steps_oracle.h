/* steps_oracle.h -- TEST ORACLE ONLY.
 *
 * Plain-C restatement of the reference StePS direct-summation force path,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker. It is never linked into, called by, or timed as the product
 * (libsteps_gb300.so has no CPU fallback).
 *
 * Parity is pinned against the UNMODIFIED reference CPU sources compiled
 * from the reference tree (oracle/_ref, see oracle/Makefile) by
 * tests/test_oracle_ref.py and against the golden vectors in tests/golden/
 * by tests/test_oracle_golden.py.
 *
 * All arrays are AoS: x[3*i+k]; forces are accelerations with G = 1,
 * overwritten (not accumulated) for i in [id_min, id_max], stored at
 * F[3*(i-id_min)+k], exactly as forces.cc:510/776/1221 return them.
 */
#ifndef STEPS_ORACLE_H
#define STEPS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_params {
    int is_periodic;            /* IS_PERIODIC */
    double L;                   /* box size (T^3) or periodic length L_z (S1xR2) */
    double rsim;                /* Rsim, radius of the simulation volume */
    int cosmology;              /* COSMOLOGY */
    int comoving;               /* COMOVING_INTEGRATION */
    double mass_in_unit_sphere; /* background pull coefficient */
    double h0, omega_lambda;    /* for the non-comoving DE term H0^2*Omega_lambda */
} oracle_params;

double oracle_force_softening(double r, double beta);

void oracle_forces_r3(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                      const oracle_params *p, double *F);

void oracle_t3_interp(int ngrid, double L, const double *table, double dx, double dy, double dz, int order,
                      double D[3]);
void oracle_forces_t3(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                      const oracle_params *p, const double *table, int ngrid, int order, double *F);

double oracle_cyl_correction(double r, double R, const double *table, int size);
void oracle_forces_s1r2_images(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                               const oracle_params *p, const double *radial_table, int radial_size, double *F);

void oracle_s1r2_interp(const double *table, int nrho, int nz, double rho_max, double lz, double dx, double dy,
                        double dz, int order, double D[3]);
void oracle_forces_s1r2_table(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                              const oracle_params *p, const double *table, int nrho, int nz, int order,
                              const double *radial_table, int radial_size, double *F);

int oracle_lattice(double radius, int *out4, int cap);
void oracle_t3_table(int ngrid, double L, double alpha, double rel_cut, double rec_cut, double real_radius,
                     double rec_radius, double *out);

void oracle_s1r2_pair(double dx, double dy, double dz, double lz, double alpha, int nmax, int mmax, double F[3]);
void oracle_s1r2_table(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax, double *out);

void oracle_cyl_table(double R, double lz, int size, int accuracy, double *out);

/* topology: 0 = R^3, 1 = T^3 (table, order), 2 = S1xR2 table (order), 3 = S1xR2 image sum. */
typedef struct oracle_system {
    int topology;
    int n;
    const double *m, *eps;
    oracle_params p;
    const double *table;
    int ngrid, nrho, nz, order;
    const double *radial_table;
    int radial_size;
} oracle_system;

void oracle_forces(const oracle_system *s, const double *x, int id_min, int id_max, double *F);

/* nsteps fixed-h KDK leapfrog steps (step.cc:100-312) with scale factor a and
 * Hubble parameter H held fixed (non-cosmological runs: a = 1, H = 0).
 * On entry F holds the forces of x; on exit x, v, F are advanced. Returns the
 * last step's errmax (step.cc:265-269) with rho_part given by the caller. */
double oracle_kdk(const oracle_system *s, int nsteps, double h, double g, double a, double hubble, double rho_part,
                  double *x, double *v, double *F);

void oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
