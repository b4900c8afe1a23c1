/*
 * steps_gb300.h -- C-ABI of libsteps_gb300.so, a GB300-native (sm_103a)
 * implementation of the StePS direct O(N^2) gravity force evaluation.
 *
 * The library replaces the three direct-summation force functions of StePS
 * behind their own interface:
 *
 *   void forces(REAL* x, REAL* F, int ID_min, int ID_max);             R^3
 *        StePS/src/forces.cc:510, StePS/src/forces_cuda.cu:74
 *   void forces_periodic(REAL* x, REAL* F, int ID_min, int ID_max);    T^3
 *        StePS/src/forces.cc:776, StePS/src/forces_cuda.cu:169
 *   void forces_periodic_z(REAL* x, REAL* F, int ID_min, int ID_max);  S1xR2
 *        StePS/src/forces.cc:1221, StePS/src/forces_cuda.cu:457
 *
 * Those three symbols themselves are provided, on top of this C-ABI, by
 * steps_gb300/legacy/forces_gb300.cc, which reads the StePS globals
 * (N, M, SOFT_LENGTH, L, Rsim, IS_PERIODIC, COSMOLOGY, ... declared in
 * StePS/src/global_variables.h:42-147) and is linked into the unchanged
 * StePS driver in place of forces.cc / forces_cuda.cu.
 *
 * Conventions (all entry points):
 *   - every call returns an int status (STEPS_OK = 0); the text of the last
 *     failure is available from steps_gpu_error_string();
 *   - positions x are AoS double[3*n] (x[3*i+k]), the layout of the StePS
 *     global x (StePS/src/global_variables.h:107);
 *   - forces are accelerations with G = 1, OVERWRITTEN (not accumulated) for
 *     i in [id_min, id_max] and stored at F[3*(i-id_min)+k], as
 *     forces.cc:520-526 and forces_cuda.cu:1045,1078-1097 return them: the
 *     reference's CPU loop adds into F with += (forces.cc:550-556) but zeroes
 *     F first, so values a caller pre-loads into F are lost there too;
 *   - one GPU, one internal CUDA stream; calls are synchronous from the
 *     caller's view (unless documented otherwise) and not re-entrant.
 */
#ifndef STEPS_GB300_H
#define STEPS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define STEPS_GB300_ABI_VERSION 1

/* Status codes. */
#define STEPS_OK 0
#define STEPS_E_ARG 1     /* invalid argument: null pointer, bad size or range */
#define STEPS_E_STATE 2   /* call out of order: not initialised, no particles, no table */
#define STEPS_E_CUDA 3    /* a CUDA runtime call or kernel launch failed */
#define STEPS_E_NOMEM 4   /* device allocation failed */
#define STEPS_E_TABLE 5   /* table shape does not match the request */
#define STEPS_E_TIMEOUT 6 /* a bounded device-side wait gave up (status written by the kernel) */
#define STEPS_E_BOUNDS 7  /* debug build (libsteps_gb300_check.so) only: an index failed its bounds check */

/* Topologies (compile-time PERIODIC / PERIODIC_Z switches in StePS,
 * StePS/Template-LinuxGCC-Makefile:29-32). */
#define STEPS_R3 0   /* compactified non-periodic R^3 */
#define STEPS_T3 1   /* T^3: nearest image + Ewald correction table */
#define STEPS_S1R2 2 /* S1xR2: periodic along z */

/* Precision modes. */
#define STEPS_FP64 0  /* plain FP64 end to end (correctness reference on the GPU) */
#define STEPS_MIXED 1 /* FP32 pair arithmetic on tile-centred coordinates, FP64 accumulation */

/* Per-call physics parameters: the StePS globals the force functions read.
 * Mirrors StePS/src/global_variables.h:42-47,98,104,118-147. */
typedef struct steps_params {
    int topology;               /* STEPS_R3 / STEPS_T3 / STEPS_S1R2 */
    int is_periodic;            /* IS_PERIODIC: T3 1 = nearest image only, >= 2 Ewald table;
                                   S1R2: 1 = nearest image, >= 2 periodic images / table */
    double L;                   /* L: box size (T3) or periodic length L_z (S1R2) */
    double rsim;                /* Rsim: radius of the simulation volume */
    int cosmology;              /* COSMOLOGY */
    int comoving;               /* COMOVING_INTEGRATION */
    double mass_in_unit_sphere; /* mass_in_unit_sphere (background pull, comoving runs) */
    double h0;                  /* H0 (non-comoving background term H0^2 * Omega_lambda) */
    double omega_lambda;        /* Omega_lambda */
    int ewald_order;            /* T3: 2 (trilinear) or 4 (Catmull-Rom tricubic);
                                   S1R2 table: 0 (NGP), 2 (CIC), 4 (TSC) -- EWALD_INTERPOLATION_ORDER */
    int s1r2_images;            /* S1R2 with is_periodic >= 2: 1 = explicit image sum
                                   (PERIODIC_Z_NOLOOKUP), 0 = (rho, z) correction table */
} steps_params;

/* ---- lifetime ----------------------------------------------------------- */

/* Selects the GPU and creates the persistent device context (stream, events,
 * buffers). Replaces the per-call cudaSetDevice/cudaMalloc/cudaFree of
 * forces_cuda.cu:959-1105. Idempotent for the same device. */
int steps_gpu_init(int device);

/* Frees every device buffer and the stream. Safe to call twice. */
int steps_gpu_shutdown(void);

/* Text of the last failure on this thread ("" if none). Never NULL. */
const char *steps_gpu_error_string(void);

int steps_gpu_abi_version(void);

/* ---- particle data ------------------------------------------------------ */

/* Uploads the per-particle masses M[n] and softening lengths SOFT_LENGTH[n]
 * (host arrays, StePS/src/global_variables.h:98-99; softening from
 * calculate_softening_length, StePS/src/utils.cc:59-82). Call again whenever
 * either changes; n fixes the particle count for the following force calls. */
int steps_gpu_set_particles(int n, const double *m, const double *eps);

/* ---- tables ------------------------------------------------------------- */

/* T^3 Ewald correction table D(r) on the cell-centred ngrid^3 grid over
 * [-L/2, L/2]^3, layout table[((ix*ngrid+iy)*ngrid+iz)*3+c]
 * (T3_EWALD_FORCE_TABLE, StePS/src/ewald_space.cc:45-48, :288). Host FP64. */
int steps_gpu_set_table_t3(int ngrid, const double *table);

/* Builds the T^3 table on the GPU in FP64 (StePS/src/ewald_space.cc:210-383
 * computed at every grid point): real-space images n with |n|^2 < real_radius^2
 * and |r + nL| <= rel_cut*L; reciprocal vectors h with |h|^2 < rec_radius^2 and
 * |2 pi h / L| <= rec_cut; Ewald parameter alpha. main.cc:416-470 uses
 * alpha = 2/L, real_radius = rel_cut + 1, rec_radius = rec_cut + 2. */
int steps_gpu_build_table_t3(int ngrid, double L, double alpha, double rel_cut, double rec_cut, double real_radius,
                             double rec_radius);

/* Copies the current T^3 table (ngrid^3*3 doubles) to the host. */
int steps_gpu_get_table_t3(double *out);

/* S1xR2 (rho, z) correction table, layout table[(ir*nz+iz)*2+c], c = 0: D_rho,
 * 1: D_z (S1R2_EWALD_FORCE_TABLE, StePS/src/ewald_space.cc:612-616, :754). */
int steps_gpu_set_table_s1r2(int nrho, int nz, const double *table);

/* Builds the S1xR2 table on the GPU (StePS/src/ewald_space.cc:618-798,
 * Tornberg 2015 singly periodic Ewald sums) for rho in [0, rho_max].
 * alpha = 0 with mmax = 0 -- the arguments of the reference's
 * PERIODIC_Z_RSPACELOOKUP build (StePS/src/main.cc:650) -- builds it from
 * direct real-space sums over nmax images per side instead, in that build's
 * summation order (ewald_space.cc:710-750). */
int steps_gpu_build_table_s1r2(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax);
int steps_gpu_get_table_s1r2(double *out);

/* Loads a T^3 table file written by the reference's driver
 * (save_t3_ewald_lookup_table, StePS/src/inputoutput.cc:1792: dataset
 * /t3_ewald/T3_EWALD_FORCE_TABLE of (Ng, Ng, Ng, 3) doubles, or floats from a
 * single-precision build) and makes it the current table, as
 * steps_gpu_set_table_t3 does; *ngrid_out (may be NULL) receives Ng. Reads the
 * file layout the HDF5 library writes with default properties (no HDF5
 * installation needed); other layouts return STEPS_E_ARG with the reason. */
int steps_gpu_load_table_t3_hdf5(const char *path, int *ngrid_out);

/* The same for an S1xR2 table file (save_s1r2_ewald_lookup_table,
 * StePS/src/inputoutput.cc:2102: /s1r2_ewald/S1R2_EWALD_FORCE_TABLE of
 * (Nrho, Nz, 2)). */
int steps_gpu_load_table_s1r2_hdf5(const char *path, int *nrho_out, int *nz_out);

/* The reader behind the two loaders, for any dataset of such a file (no GPU
 * needed): `dataset` is an absolute path ("/group/name"); integer and
 * floating-point elements are converted to double. Writes *rank, dims[rank]
 * (up to 32) and *count (any may be NULL); copies the elements into out when
 * out is non-NULL and capacity >= count. */
int steps_h5_read_f64(const char *path, const char *dataset, double *out, long long capacity, long long *count,
                      int *rank, long long *dims);

/* Cylindrical background multiplier table RADIAL_FORCE_TABLE[size]
 * (StePS/src/utils.cc:162-228), used by S1xR2 comoving runs. */
int steps_gpu_set_radial_table(int size, const double *table);

/* Builds that table on the GPU in FP64 -- get_cylindrical_force_table
 * (StePS/src/utils.cc:162-228): the pull at r_i = rsim i / (size - 1) of a
 * finite cylinder of half length lz by the trapezoid rule over `accuracy`
 * intervals (RADIAL_FORCE_TABLE_SIZE, RADIAL_FORCE_ACCURACY; the reference's
 * driver passes lz = L/2 at IS_PERIODIC = 1 and L (IS_PERIODIC + 0.6) above,
 * StePS/src/main.cc:905-917) -- and keeps it as the radial table. */
int steps_gpu_build_radial_table(int size, double rsim, double lz, int accuracy);

/* Copies the current radial table (size doubles) to the host. */
int steps_gpu_get_radial_table(double *out);

/* ---- force evaluation --------------------------------------------------- */

/* The drop-in force call with HOST buffers: uploads x (double[3n]), computes
 * the accelerations of particles id_min..id_max against all n particles and
 * downloads them into F (double[3*(id_max-id_min+1)], overwritten).
 * id_max = id_min - 1 is the empty range: nothing is computed or written (F
 * may then be NULL), as the reference's loop over an empty range does.
 * Equivalent of forces()/forces_periodic()/forces_periodic_z()
 * (forces.cc:510/776/1221, forces_cuda.cu:878/1121/1378). */
int steps_gpu_forces(const steps_params *p, int precision, const double *x, double *F, int id_min, int id_max);

/* Device-resident variant: positions already uploaded with
 * steps_gpu_upload_positions (or advanced by steps_gpu_kdk); the result
 * stays on the device until steps_gpu_download_forces. No host copies. */
int steps_gpu_upload_positions(const double *x);
int steps_gpu_forces_resident(const steps_params *p, int precision, int id_min, int id_max);
/* Copies the forces of the last successful force call (any entry point of
 * this context, the KDK steps included) into F, double[3 * count] with count
 * from steps_gpu_forces_range. New masses (steps_gpu_set_particles) and a
 * failed force call leave no range: STEPS_E_STATE. */
int steps_gpu_download_forces(double *F);
/* The i range the resident forces cover: *id_min and *count (0 when none). */
int steps_gpu_forces_range(int *id_min, int *count);

/* ---- leapfrog (device resident) ----------------------------------------- */

/* Uploads velocities v[3n] (host). */
int steps_gpu_upload_velocities(const double *v);

/* nsteps fixed-h KDK steps of StePS's step() (StePS/src/step.cc:100-312) on
 * the resident x, v: kick h/2 + drift h, periodic wrap, force, kick h/2, with
 * acceleration g*F*a^-3 - 2*hubble*v. Computes the forces of the current
 * positions first if none are resident. errmax (step.cc:265-269, with
 * rho_part) of the last step is written to *errmax_out when non-NULL.
 * Mixed-precision R^3 steps re-sort the particles every 8th step and in
 * between rebuild the tiles in the previous order (same forces, less
 * preparation); periodic topologies re-sort every step. */
int steps_gpu_kdk(const steps_params *p, int precision, int nsteps, double h, double g, double a, double hubble,
                  double rho_part, double *errmax_out);

/* Downloads the resident positions, velocities and forces (any may be NULL). */
int steps_gpu_download_state(double *x, double *v, double *F);

/* ---- batched ensembles (independent realisations, uneven N) ------------- */

/* Registers `count` independent R^3 realisations; realisation k has n[k]
 * particles whose positions, masses and softening lengths are the host arrays
 * x[k] (double[3 n[k]]), m[k], eps[k]. Velocities start at zero. Registering
 * the same count and n[] again replaces the data only: the tuned tile shape
 * and the captured graph of the previous batch are kept. */
int steps_gpu_batch_set(int count, const int *n, const double *const *x, const double *const *m,
                        const double *const *eps);

/* One force evaluation followed by nsteps fixed-h KDK steps of every
 * realisation (StePS/src/step.cc:100-312 with g = 1, a = 1, no Hubble drag).
 * graph = 1 runs the whole of it as ONE persistent kernel, after a single
 * ordering pass, captured into a CUDA graph: (stage, item) tasks from one
 * queue, each stage of a realisation starting when its previous stage is
 * done (bounded waits: STEPS_E_TIMEOUT if one gives up), the kicks, drift and
 * re-tiling done by the block that completes each tile; tile shape, j-chunk
 * length and grid size autotuned on the first run. graph = 2 runs it as a
 * CUDA graph of per-phase kernels (re-ordering every step); graph = 0 as
 * `count` separate plain launches per phase. */
int steps_gpu_batch_run(const steps_params *p, int precision, int nsteps, double h, int graph);

/* Downloads realisation k's positions/velocities/forces (any may be NULL). */
int steps_gpu_batch_get(int k, double *x, double *v, double *F);

/* ---- tuning and instrumentation ----------------------------------------- */

/* Fixes the mixed-precision kernel shape: threads per block (64/128/256),
 * i-particles per thread (1/2/4) and j-range split (0 = automatic). Tile size
 * is threads*ipt. Returns STEPS_E_ARG for an unsupported shape. */
int steps_gpu_set_tuning(int threads, int ipt, int jsplit);

/* R^3 mixed-precision pair loop: 0 = scalar FP32 instructions, 1 = packed
 * FP32x2 instructions (two pairs per instruction, sm_100+), 2 / 3 = packed
 * with 768 / 1024 resident threads per SM asked of the register allocator,
 * 4 = packed with the j tiles streamed by bulk copies (TMA) through an
 * mbarrier ring (bounded waits; STEPS_E_TIMEOUT if one gives up). Same results
 * to rounding; the autotuner picks among them. T^3 with a trilinear table reads
 * the same setting as 1 = quad lanes (one i per thread; the 4 lanes of a quad take one
 * i against 4 neighbouring j per step, so table loads share cache lines), any
 * other value = one i per lane. */
int steps_gpu_set_kernel_variant(int variant);

/* T^3 mixed precision: capacity, in table cells (16 bytes each), of the
 * shared-memory window of the Ewald table that each block stages per tile
 * pair. Without a window (0, the default), or when a tile pair's window does
 * not fit, pairs read an FP32 copy of the table with a periodic halo through
 * L1/L2. At most STEPS_T3_WINDOW_MAX. */
#define STEPS_T3_WINDOW_MAX 12288
int steps_gpu_set_t3_window(int cells);

/* Mixed precision: tile pairs whose coordinate scale (centre distance plus
 * half extents) exceeds `ratio` times their box gap run the double-float
 * near-field path instead of the FP32 far-field loop. Lower = more accurate
 * and slower. Range [1, 1e6]. */
int steps_gpu_set_precision_guard(double ratio);

/* Times every supported mixed-precision shape on the resident particles for
 * the given topology -- for R^3 with each pair-loop variant -- and keeps the
 * fastest; writes threads, ipt, variant to out[3]. Each candidate is first
 * timed on a strided sample of the range's i tiles against all j, 24 waves
 * of work (after one untimed launch); the three best are timed again on 96
 * waves (or the whole range when it is smaller). Leaves no resident forces. */
int steps_gpu_autotune(const steps_params *p, int id_min, int id_max, int *out);

/* Number of kernels this library has launched since init. */
long long steps_gpu_launch_count(void);

/* Device time (CUDA events on the library stream) of the phases of the last
 * force evaluation: 0 = preparation (packing, ordering, tiling), 1 = pair
 * kernel, 2 = reduction/epilogue. Synchronises the stream. */
double steps_gpu_last_phase_ms(int phase);

/* Pairs the last pair kernel evaluated: (id_max-id_min+1) * n. */
double steps_gpu_last_pairs(void);

/* Event markers on the library stream for callers that time a sequence of
 * calls: mark(slot) records event `slot` (0..15); elapsed(a, b) synchronises
 * and returns milliseconds between two recorded marks. */
int steps_gpu_timer_mark(int slot);
double steps_gpu_timer_elapsed_ms(int a, int b);

/* Overwrites a device buffer of `bytes` bytes on the library stream (evicts
 * L2 between timed steps). */
int steps_gpu_flush_l2(long long bytes);

/* Measures this GPU's FP32 FMA and FP64 FMA issue peaks (FLOP/s, an FMA
 * counted as 2) with dependent-chain kernels; either pointer may be NULL. */
int steps_gpu_measure_peaks(double *fp32_flops, double *fp64_flops);

/* Blocks until the library stream is idle; returns a pending kernel error. */
int steps_gpu_synchronize(void);

/* Page-locked host memory for the host-buffer calls (x, F of steps_gpu_forces,
 * steps_gpu_upload_positions, ...): copies from and to it run at full DMA
 * speed. The reference's driver arrays are ordinary malloc memory, which also
 * works. *p is NULL on failure. */
int steps_gpu_host_alloc(long long bytes, void **p);
int steps_gpu_host_free(void *p);

/* Test hook for the bounded waits (no counterpart in the reference): in the
 * next mixed R^3 force evaluation with pair-loop variant 4, block 0 withholds
 * the bulk copy of its tile number tile_seq (0-based, counted over the block's
 * work), so the waits on that tile run out after about a second. The call then
 * returns STEPS_E_TIMEOUT, the kernel having left cleanly, and the context
 * stays usable. -1 cancels. One shot. */
int steps_gpu_test_stall_copy(long long tile_seq);

/* Test hook for the persistent ensemble kernel's bounded waits (no
 * counterpart in the reference): in the next steps_gpu_batch_run with
 * graph = 1 (run directly, not from the captured graph), realisation
 * `realisation` never reports its first stage done, so the waits of its next
 * stage run out after about a second; the call returns STEPS_E_TIMEOUT and the
 * context stays usable. -1 cancels. One shot. */
int steps_gpu_test_stall_ensemble(int realisation);

/* Debug bounds checks. libsteps_gb300_check.so is the same library built with
 * -DSTEPS_CHECK: every kernel compares its tile, chunk, slot, output-row,
 * table-cell and ordering indices with their bounds, records the first one out
 * of range, keeps the access inside its buffer, and the call returns
 * STEPS_E_BOUNDS with the site, index and bound in steps_gpu_error_string().
 * steps_gpu_checks_compiled() is 1 in that build, 0 in the normal one.
 * steps_gpu_test_bounds_check() checks the mechanism itself: in the checked
 * build it launches one kernel that submits `index` against the bound 16 (the
 * index is never dereferenced) and returns STEPS_E_BOUNDS when index is outside
 * [0, 16), STEPS_OK otherwise; in the normal build it returns STEPS_E_STATE. */
int steps_gpu_checks_compiled(void);
int steps_gpu_test_bounds_check(int index);

/* ---- allocation-free entry point ----------------------------------------- */

/* No counterpart in the reference. Plain FP64 R^3 forces for callers that
 * cannot allocate device memory: applications that give all device memory to
 * their own pool allocator, and loops that must not pay the implicit device
 * synchronisation of cudaMalloc/cudaFree. The caller owns every buffer, all
 * in device memory of the current device: x[3n] (AoS), m[n], eps[n] and
 * F[3*(id_max-id_min+1)] (overwritten). Calls no cudaMalloc, cudaFree or
 * allocating library routine and needs no steps_gpu_init. Asynchronous on
 * `stream` (a cudaStream_t; NULL = legacy default stream). id_max = id_min - 1
 * is the empty range: STEPS_OK with nothing computed (F may then be NULL).
 * Working memory is one static 32 MiB device array per GPU that loads the
 * library, held until exit: the i range is limited to 1,398,101 particles
 * (larger ranges return STEPS_E_ARG). The array's device address is looked
 * up by the first call on each device, and again by the first call after a
 * cudaDeviceReset -- make those calls before any stream capture. All calls
 * share the array (it keeps the last call's contents; each call writes what
 * it reads): calls that overlap on the GPU race, so the caller serialises
 * them. */
int steps_gpu_forces_fp64_noalloc(const steps_params *p, const double *x, const double *m, const double *eps, int n,
                                  double *F, int id_min, int id_max, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* STEPS_GB300_H */
