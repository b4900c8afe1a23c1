/*
 * forces_gb300.cc -- drop-in replacement of StePS's force translation unit
 * (StePS/src/forces.cc for CPU builds, StePS/src/forces_cuda.cu for CUDA
 * builds) on top of libsteps_gb300 (include/steps_gb300.h).
 *
 * Compile it with the SAME -D switches as the rest of the StePS build
 * (PERIODIC / PERIODIC_Z / PERIODIC_Z_NOLOOKUP / EWALD_INTERPOLATION_ORDER /
 * USE_SINGLE_PRECISION) and link -lsteps_gb300 in place of forces.o or
 * forces_cuda.o; main.cc and step.cc stay byte-identical. It defines exactly
 * the symbols the driver calls:
 *
 *   void forces(REAL*, REAL*, int, int)             StePS/src/forces.cc:510, forces_cuda.cu:74
 *   void forces_periodic(REAL*, REAL*, int, int)    StePS/src/forces.cc:776, forces_cuda.cu:169
 *   void forces_periodic_z(REAL*, REAL*, int, int)  StePS/src/forces.cc:1221, forces_cuda.cu:457
 *   void recalculate_softening(void)                StePS/src/forces.cc:43, forces_cuda.cu:868
 *
 * and reads the driver's globals (StePS/src/global_variables.h:42-147). The
 * first call creates the GPU context (device STEPS_GB300_DEVICE, default 0);
 * masses/softening are re-uploaded when they change; tables when their
 * pointer or size changes. Failures set ForceError = true and print to
 * stderr, which makes the StePS main loop stop (StePS/src/main.cc:1851-1856).
 *
 * Precision: STEPS_GB300_PRECISION=fp64|mixed in the environment, default
 * mixed (FP32 pair arithmetic, FP64 accumulation, p99 error <= 1e-5).
 * Each call prints the reference CUDA build's wall-clock line to stdout
 * unless STEPS_GB300_QUIET=1.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "steps_gb300.h"

#ifdef USE_SINGLE_PRECISION
typedef float REAL;
#else
typedef double REAL;
#endif

/* ---- the StePS globals this file reads (StePS/src/global_variables.h) ---- */
extern int IS_PERIODIC;          /* :42 */
extern int COSMOLOGY;            /* :43 */
extern int COMOVING_INTEGRATION; /* :44 */
extern REAL L;                   /* :45 */
extern REAL Rsim;                /* :46 */
extern bool ForceError;          /* :62 */
extern int n_GPU;                /* :65 */
extern int rank;                 /* :67 */
extern REAL *M;                  /* :98 */
extern REAL *SOFT_LENGTH;        /* :99 */
extern int N;                    /* :101 */
extern REAL beta;                /* :106 */
extern REAL ParticleRadi;        /* :107 */
extern REAL rho_part;            /* :108 */
extern REAL M_min;               /* :110 */
extern REAL mass_in_unit_sphere; /* :111 */
extern double Omega_lambda, H0;  /* :117 */
#ifdef PERIODIC
extern REAL *T3_EWALD_FORCE_TABLE; /* :49 */
extern int N_EWALD_FORCE_GRID;     /* :50 */
#elif defined(PERIODIC_Z) && !defined(PERIODIC_Z_NOLOOKUP)
extern REAL *S1R2_EWALD_FORCE_TABLE; /* :53 */
extern int Nz_EWALD_FORCE_GRID;      /* :54 */
extern int Nrho_EWALD_FORCE_GRID;    /* :55 */
#endif
#if defined(PERIODIC_Z)
extern int RADIAL_FORCE_TABLE_SIZE; /* :139 */
extern REAL *RADIAL_FORCE_TABLE;    /* :141 */
#endif

#ifndef EWALD_INTERPOLATION_ORDER
#define EWALD_INTERPOLATION_ORDER 4
#endif

namespace {

struct LegacyState {
    bool ready = false;
    int precision = STEPS_MIXED;
    bool tune = true;  // autotune the mixed kernel after the first mixed force call
    std::vector<double> m, eps;  // what the device holds
    const void *table_ptr = nullptr;
    long long table_size = -1;
    const void *radial_ptr = nullptr;
    int radial_size = -1;
    std::vector<double> xbuf, Fbuf;
};

LegacyState S;

void report(const char *where)
{
    fprintf(stderr, "MPI rank %i: steps_gb300 %s failed: %s\n", rank, where, steps_gpu_error_string());
    ForceError = true;
}

bool ensure_context()
{
    if (S.ready) return true;
    const char *dev = getenv("STEPS_GB300_DEVICE");
    const char *prec = getenv("STEPS_GB300_PRECISION");
    if (prec && strcmp(prec, "fp64") == 0) S.precision = STEPS_FP64;
    const char *tune = getenv("STEPS_GB300_AUTOTUNE");
    if (tune && strcmp(tune, "0") == 0) S.tune = false;
    if (n_GPU > 1 && rank == 0)
        fprintf(stderr, "steps_gb300: using one GPU per rank (n_GPU = %i requested)\n", n_GPU);
    if (steps_gpu_init(dev ? atoi(dev) : 0) != STEPS_OK) {
        report("init");
        return false;
    }
    S.ready = true;
    return true;
}

bool sync_particles()
{
    size_t n = (size_t)N;
    bool changed = S.m.size() != n;
    if (!changed)
        for (size_t i = 0; i < n; i++)
            if (S.m[i] != (double)M[i] || S.eps[i] != (double)SOFT_LENGTH[i]) { changed = true; break; }
    if (!changed) return true;
    S.m.resize(n);
    S.eps.resize(n);
    for (size_t i = 0; i < n; i++) { S.m[i] = M[i]; S.eps[i] = SOFT_LENGTH[i]; }
    if (steps_gpu_set_particles(N, S.m.data(), S.eps.data()) != STEPS_OK) {
        report("set_particles");
        S.m.clear();
        return false;
    }
    return true;
}

[[maybe_unused]] bool upload_table(const REAL *tab, long long count, int (*setter)(int, int, const double *), int a, int b)
{
    if (tab == S.table_ptr && count == S.table_size) return true;
    std::vector<double> t((size_t)count);
    for (long long i = 0; i < count; i++) t[(size_t)i] = tab[i];
    if (setter(a, b, t.data()) != STEPS_OK) {
        report("table upload");
        return false;
    }
    S.table_ptr = tab;
    S.table_size = count;
    return true;
}

[[maybe_unused]] int set_t3(int ng, int, const double *t) { return steps_gpu_set_table_t3(ng, t); }
[[maybe_unused]] int set_s1(int nrho, int nz, const double *t) { return steps_gpu_set_table_s1r2(nrho, nz, t); }

// The per-call timing line the reference's CUDA build prints to stdout
// (StePS/src/forces_cuda.cu:1115, :1372 "Force calculation finished ...", :1702
// "Z-periodic force calculation finished ..."), so logs read the same.
// STEPS_GB300_QUIET=1 silences it.
struct CallTimer {
    const char *prefix;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    explicit CallTimer(const char *pre) : prefix(pre) {}
    ~CallTimer()
    {
        static const bool quiet = getenv("STEPS_GB300_QUIET") && strcmp(getenv("STEPS_GB300_QUIET"), "1") == 0;
        if (quiet) return;
        double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        printf("%sorce calculation finished on MPI task %i. Force calculation wall-clock time = %fs.\n", prefix, rank,
               s);
    }
};

void run(const steps_params &p, REAL *x, REAL *F, int ID_min, int ID_max)
{
    if (ID_max < ID_min) return;  // an empty range: the reference's loops do nothing (forces.cc:520-556)
    if (!ensure_context() || !sync_particles()) return;
    [[maybe_unused]] const int ni = ID_max - ID_min + 1;  // the FP32 build's conversion
    const double *xd;
    double *Fd;
#ifdef USE_SINGLE_PRECISION
    S.xbuf.resize(3 * (size_t)N);
    S.Fbuf.resize(3 * (size_t)(ni > 0 ? ni : 1));
    for (size_t i = 0; i < 3 * (size_t)N; i++) S.xbuf[i] = x[i];
    xd = S.xbuf.data();
    Fd = S.Fbuf.data();
#else
    xd = x;
    Fd = F;
#endif
    if (steps_gpu_forces(&p, S.precision, xd, Fd, ID_min, ID_max) != STEPS_OK) {
        report("force evaluation");
        return;
    }
    if (S.tune && S.precision == STEPS_MIXED) {
        // Once per run, on the positions just uploaded: time every kernel shape
        // and keep the fastest for the following steps.
        S.tune = false;
        int shape[3];
        if (steps_gpu_autotune(&p, ID_min, ID_max, shape) != STEPS_OK) report("autotune");
    }
#ifdef USE_SINGLE_PRECISION
    for (size_t i = 0; i < 3 * (size_t)ni; i++) F[i] = (REAL)Fd[i];
#endif
}

steps_params base_params(int topology)
{
    steps_params p;
    memset(&p, 0, sizeof p);
    p.topology = topology;
    p.is_periodic = IS_PERIODIC;
    p.L = L;
    p.rsim = Rsim;
    p.cosmology = COSMOLOGY;
    p.comoving = COMOVING_INTEGRATION;
    p.mass_in_unit_sphere = mass_in_unit_sphere;
    p.h0 = H0;
    p.omega_lambda = Omega_lambda;
    p.ewald_order = EWALD_INTERPOLATION_ORDER;
    p.s1r2_images = 0;
    return p;
}

}  // namespace

/* Overrides the precision chosen at the first call (STEPS_GB300_PRECISION):
 * STEPS_FP64 or STEPS_MIXED. */
extern "C" void steps_gb300_legacy_precision(int precision)
{
    if (precision == STEPS_FP64 || precision == STEPS_MIXED) {
        ensure_context();
        S.precision = precision;
    }
}

/* forces.cc:43-50: the same expression (pow, and pi rounded to the same
 * double), so rho_part -- and with it step.cc's errmax -- is bit-identical. */
void recalculate_softening()
{
    beta = ParticleRadi;
    if (COSMOLOGY == 1) rho_part = M_min / (4.0 * 3.14159265358979323846 * pow(beta, 3.0) / 3.0);
}

#if !defined(PERIODIC) && !defined(PERIODIC_Z)
void forces(REAL *x, REAL *F, int ID_min, int ID_max)
{
    CallTimer timer("F");
    steps_params p = base_params(STEPS_R3);
    run(p, x, F, ID_min, ID_max);
}
#endif

#ifdef PERIODIC
void forces_periodic(REAL *x, REAL *F, int ID_min, int ID_max)
{
    CallTimer timer("F");
    steps_params p = base_params(STEPS_T3);
    if (ID_max < ID_min) return;  // empty range: no work, no table upload
    if (IS_PERIODIC >= 2) {
        if (!ensure_context()) return;
        long long cnt = 3LL * N_EWALD_FORCE_GRID * N_EWALD_FORCE_GRID * N_EWALD_FORCE_GRID;
        if (!upload_table(T3_EWALD_FORCE_TABLE, cnt, set_t3, N_EWALD_FORCE_GRID, 0)) return;
    }
    run(p, x, F, ID_min, ID_max);
}
#endif

#ifdef PERIODIC_Z
void forces_periodic_z(REAL *x, REAL *F, int ID_min, int ID_max)
{
    CallTimer timer("Z-periodic f");
    steps_params p = base_params(STEPS_S1R2);
    if (ID_max < ID_min) return;  // empty range: no work, no table upload
    if (!ensure_context()) return;
#ifdef PERIODIC_Z_NOLOOKUP
    p.s1r2_images = 1;
#else
    if (IS_PERIODIC >= 2) {
        long long cnt = 2LL * Nrho_EWALD_FORCE_GRID * Nz_EWALD_FORCE_GRID;
        if (!upload_table(S1R2_EWALD_FORCE_TABLE, cnt, set_s1, Nrho_EWALD_FORCE_GRID, Nz_EWALD_FORCE_GRID)) return;
    }
#endif
    if (COSMOLOGY == 1 && COMOVING_INTEGRATION == 1 && RADIAL_FORCE_TABLE &&
        (RADIAL_FORCE_TABLE != S.radial_ptr || RADIAL_FORCE_TABLE_SIZE != S.radial_size)) {
        std::vector<double> t(RADIAL_FORCE_TABLE, RADIAL_FORCE_TABLE + RADIAL_FORCE_TABLE_SIZE);
        if (steps_gpu_set_radial_table(RADIAL_FORCE_TABLE_SIZE, t.data()) != STEPS_OK) {
            report("radial table upload");
            return;
        }
        S.radial_ptr = RADIAL_FORCE_TABLE;
        S.radial_size = RADIAL_FORCE_TABLE_SIZE;
    }
    run(p, x, F, ID_min, ID_max);
}
#endif
