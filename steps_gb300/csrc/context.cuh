// The single persistent device context of libsteps_gb300 and the internal
// entry points the translation units share.
#pragma once

#include "common.cuh"

namespace steps {

struct Batch;  // batched ensembles (batch.cu)

struct Ctx {
    int device = -1;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t marks[16] = {};
    bool mark_set[16] = {};
    cudaEvent_t phase[4] = {};
    bool phase_valid = false;

    int n = 0;                       // particle count fixed by set_particles
    DevBuf m64, eps64;               // masses, softening (FP64, original order)
    DevBuf x, v, F;                  // positions/velocities (AoS FP64), last forces
    bool have_x = false, have_v = false;
    bool F_valid = false;            // F holds full-range forces of the current x
    int F_lo = 0, F_ni = 0;          // range F currently holds
    DevBuf pack64;                   // FP64 kernel j stream: (x, y, z, m) per particle
    DevBuf partial;                  // per-j-chunk partial forces (FP64)
    DevBuf bbox, counter, status, flush, peaks;
    DevBuf kstatus;                  // int written by kernels whose bounded waits give up
    int *kstatus_host = nullptr;     // page-locked mirror of kstatus
    bool status_pending = false;     // a kernel that can write kstatus ran since it was last read
    long long stall_seq = -1;        // test hook for the next pipelined launch (one shot)
    TileSet tj, ti;                  // j set (all particles) and i subset tiles

    DevBuf t3;
    int t3_ng = 0;
    long long t3_version = 0;  // bumped whenever the table changes
    DevBuf t3f;                // FP32 float4-per-cell haloed copy for the mixed kernels
    long long t3f_version = -1;
    DevBuf t3r;                // stencil records of the haloed copy (z rows / yz quads)
    long long t3r_version = -1;
    int t3r_order = 0;
    DevBuf s1rec;              // S1xR2 table records: whole CIC stencils or TSC z triplets
    long long s1rec_version = -1;
    int s1rec_order = -1;             // layout of s1rec: CIC (2) or TSC (4)
    DevBuf s1r2;
    int nrho = 0, nz = 0;
    long long s1r2_version = 0;
    DevBuf s1f;  // FP32 float2 copy for the mixed kernel
    long long s1f_version = -1;
    DevBuf radial;
    int radial_size = 0;

    Shape shape;
    bool shape_fixed = false;
    int tune_sample = 0;  // the autotuner's timing runs: tune_sample waves of items over a strided sample of
                          // i tiles (0: off), no reduction
    bool tune_sampled = false;  // the last timing run was cut to a sample (else it covered the whole range)
    double last_pairs = 0.0;
    int last_S = 0;             // j chunks per i tile of the last mixed launch
    double last_waves = 0.0;    // its full-range items over the resident blocks

    Batch *batch = nullptr;
};

Ctx &ctx();
void require_init();
// The device status word kernels with bounded waits write STEPS_E_TIMEOUT to
// (zero until a wait gives up; zeroed when allocated).
int *kernel_status_word();
// Reads that word (synchronising the stream) when such a kernel ran since it
// was last read; fails with STEPS_E_TIMEOUT, clearing the word and the
// resident force range, when a wait gave up.
void check_kernel_status();
// Runs body(arg), turning a thrown Error into its status code (and message).
int run_guarded(void (*body)(void *), void *arg);
void batch_release();
KParams derive_params(const steps_params *p);
Tables device_tables(const KParams &kp);

// order.cu
// Padding ids: j padding and i padding differ so a padded i never meets a padded j.
constexpr uint32_t PAD_J = 0xffffffffu, PAD_I = 0xfffffffeu;
void build_tiles(TileSet &ts, const double *x, const double *m64, const double *eps64, int lo, int count, int T,
                 bool reuse, cudaStream_t st, unsigned long long *bbox_scratch, uint32_t pad_id);
// Stable LSD radix sort of (keys, vals) on key bits [lo_bit, 64).
void sort_pairs(TileSet &ts, int n, cudaStream_t st, int lo_bit = 0);
int morton_sort_bits(int n);
void batch_keys(const double *x, int lo, int count, unsigned long long prefix, unsigned long long *keys, uint32_t *vals,
                unsigned long long *bbox_scratch, cudaStream_t st);
void tile_build_range(const double *x, const double *m64, const double *eps64, const uint32_t *perm, int count, int T,
                      float4 *pack, float *epsf, float4 *meta, uint32_t *idx, uint32_t pad_id, float4 *lo, float *soa,
                      const int2 *tdesc, int ntiles, cudaStream_t st, float4 *sub);

// pair_fp64.cu: FP64 forces of i in [id_min, id_min+ni) into F[3*ni] (with background).
void forces_fp64(const KParams &kp, const Tables &tb, const double *x, int n, int id_min, int ni, double *F);

// pair_mixed.cu
struct MixedLaunch;
void forces_mixed(const KParams &kp, const Tables &tb, const double *x, const double *m64, const double *eps64,
                  int n, int id_min, int ni, double *F, bool reuse_order);
bool shape_supported(int threads, int ipt);
bool shape_supported_for(const KParams &kp, int threads, int ipt);

// Shared force driver used by the C-ABI, the KDK loop and the batch code.
void compute_forces(const steps_params *p, int precision, int id_min, int id_max, bool reuse_order);

// kdk.cu
void kdk_kick_drift(double *x, double *v, const double *F, int n, double h, double g, double a3, double hubble,
                    int wrap_mode, double L, cudaStream_t st);
double kdk_kick_err(double *v, const double *F, const double *m, int n, double h, double g, double a3, double hubble,
                    double rho_part, double *err_scratch, cudaStream_t st, bool fetch);

// background epilogue shared by the reductions
struct Background {
    int mode;        // 0 none, 1 coef * (x, y, z), 2 coef * (x, y) (S1R2), 3 cylindrical table * coef * (x, y)
    double coef;
    double rsim;
    const double *radial;
    int radial_size;
};
Background background_of(const KParams &kp, const Tables &tb);

// Background pull of the matter outside the simulation volume, added after the
// j sum: R^3 StePS/src/forces.cc:557-568; S1xR2 forces.cc:1293-1304 with the
// cylindrical multiplier (forces.cc:279-316, linear) and :1336-1346 (table mode).
__device__ __forceinline__ void add_background(const Background &bg, const double *xi, double *Fi)
{
    if (bg.mode == 1) {
        for (int k = 0; k < 3; k++) Fi[k] += bg.coef * xi[k];
    } else if (bg.mode == 2) {
        Fi[0] += bg.coef * xi[0];
        Fi[1] += bg.coef * xi[1];
    } else if (bg.mode == 3) {
        double r = sqrt(xi[0] * xi[0] + xi[1] * xi[1]);
        int sz = bg.radial_size;
        double step = bg.rsim / (double)sz;
        int i = (int)floor(r / bg.rsim * (sz - 1));
        double c = bg.radial[sz - 1];
        if (i < sz - 1) {
            STEPS_CHECK_IDX(i, sz - 1, CK_RADIAL);
            double x1 = step * i, y1 = bg.radial[i], x2 = step * (i + 1), y2 = bg.radial[i + 1];
            double A = (y2 - y1) / (x2 - x1);
            double B = y1 - A * x1;
            c = A * r + B;
        }
        Fi[0] += bg.coef * xi[0] * c;
        Fi[1] += bg.coef * xi[1] * c;
    }
}

}  // namespace steps
