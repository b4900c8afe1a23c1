// Shared declarations of libsteps_gb300: the persistent device context,
// error handling, kernel parameter blocks and device math helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "steps_gb300.h"

namespace steps {

// ---------------------------------------------------------------- errors --

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg);
void check_cuda(cudaError_t e, const char *what, const char *file, int line);
#define STEPS_CUDA(expr) ::steps::check_cuda((expr), #expr, __FILE__, __LINE__)

// ------------------------------------------------------------ device buf --

// A growable device allocation owned by the context. Grows (free + malloc)
// only when a request exceeds its capacity; never shrinks until shutdown.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    template <class T>
    T *as() const { return static_cast<T *>(p); }
    template <class T>
    T *ensure(size_t count) { grow(count * sizeof(T)); return static_cast<T *>(p); }
    void grow(size_t want);
    void release();
};

// ------------------------------------------------- kernel parameter blocks --

// Physics parameters as the kernels read them (derived once per call).
struct KParams {
    int topology;
    int is_periodic;
    int comoving_bg;   // 0 none, 1 mass_in_unit_sphere * x, 2 H0^2 Omega_L * x
    int s1r2_images;   // S1R2 with is_periodic >= 2: explicit images (1) or table (0)
    int emax;          // S1R2 image range [-emax, emax] (ewald_max = IS_PERIODIC + 1)
    int order;         // interpolation order of the active table
    double L, halfL, cutL;  // cutL = (emax - 0.4) * L
    double bg_coef;
    double rsim;
};

// Tables resident on the device (FP64 as StePS builds them).
struct Tables {
    const double *t3;  // ngrid^3 * 3
    int t3_ng;
    const double *s1r2;  // nrho * nz * 2
    int nrho, nz;
    double rho_max;
    const double *radial;  // cylindrical background multiplier
    int radial_size;
};

// A set of particles ordered along a Morton curve and cut into tiles of T.
// pack[q] = (x - c, y - c, z - c, m) of the q-th particle in curve order,
// relative to its tile's centre c (exactly representable in FP32);
// meta[2t] = (c.x, c.y, c.z, eps_max), meta[2t+1] = (half extents, 0).
struct TileSet {
    int lo = 0, count = 0;  // original index range [lo, lo + count)
    int T = 0, ntiles = 0;
    DevBuf keys[2], vals[2], hist;
    DevBuf pack, eps, meta;
    DevBuf idx;  // idx[q] = original index of curve position q; padding holds pad_id
    DevBuf resid;  // resid[q] = (x - c) - pack[q].xyz, the FP32 residual of the offset
    DevBuf soa;    // tile-blocked SoA copy of pack: X[T], Y[T], Z[T], M[T] per tile
    DevBuf sub;    // per SUBTILE particles: (box centre offset, eps_max), (half extents, 0)
    int perm_sel = 0;  // vals[perm_sel] holds curve position -> original index
    bool ordered = false;
    const uint32_t *perm() const { return vals[perm_sel].as<uint32_t>(); }
};

// Mixed-kernel launch shape.
struct Shape {
    int threads = 128;
    int ipt = 2;
    int jsplit = 0;
    int variant = 0;  // R^3: 0 scalar FP32 pair loop; 1, 2, 3 packed FP32x2 (0, 768, 1024 threads/SM
                      // asked); 4 packed with the bulk-copy (TMA) + mbarrier pipeline
    float guard = 30.0f;  // tile-pair scale / gap above which the double-float path runs
    int t3_cells = 0;  // T^3: shared-memory table window capacity in cells (0 = haloed table via L1/L2)
};

// ------------------------------------------------------------- utilities --

inline __host__ __device__ int div_up(int a, int b) { return (a + b - 1) / b; }

// Particles per j sub-tile: the near/far decision of the packed R^3 kernel is
// taken per (warp, sub-tile) from the sub-tile boxes the tile build writes.
constexpr int SUBTILE = 16;

// Kernel-launch bookkeeping: counts launches and surfaces launch errors.
void note_launch(const char *name);
// Adds kernels launched by other means (the kernel nodes of a graph launch).
void add_launches(long long k);

// ------------------------------------------------- debug bounds checks --
//
// Compiled with -DSTEPS_CHECK (libsteps_gb300_check.so), STEPS_CHECK_IDX(v,
// bound, site) compares the index variable v with [0, bound). The first index
// out of range in this translation unit is recorded (site, index, bound), v
// is set to 0 so that the access it guards stays inside its buffer, and the
// C-ABI call that launched the kernel returns STEPS_E_BOUNDS with the record
// in its message. In the normal build the macro is empty.
enum CheckSite {
    CK_NONE = 0,
    CK_I_TILE,      // i tile of a work item
    CK_J_TILE,      // j tile range of a work item
    CK_CHUNK,       // j chunk (partial slab) of a work item
    CK_SLOT,        // partial slot of a work-list item or of an i tile
    CK_OUTPUT,      // caller-order output row (curve position -> original index - id_min)
    CK_T3_CELL,     // cell of the FP32 T^3 table (haloed copy, window or wrapped read)
    CK_T3_FP64,     // cell of the FP64 T^3 table
    CK_S1_CELL,     // (rho, z) cell of the S1xR2 table or of its records
    CK_RADIAL,      // entry of the cylindrical radial-force table
    CK_PERM,        // original particle index read from the ordering
    CK_SCATTER,     // destination of a radix-sort scatter
    CK_SELFTEST,    // steps_gpu_test_bounds_check
    CK_NSITES
};

struct CheckRecord {
    int code;  // 0, or STEPS_E_BOUNDS once an index failed
    int site;
    long long index, bound;
};

#ifdef STEPS_CHECK
static __device__ CheckRecord g_check_record;

static __device__ __noinline__ void check_failed(long long index, long long bound, int site)
{
    if (atomicCAS(&g_check_record.code, 0, STEPS_E_BOUNDS) == 0) {
        g_check_record.site = site;
        g_check_record.index = index;
        g_check_record.bound = bound;
        __threadfence();
    }
}

#define STEPS_CHECK_IDX(v, bound, site)                                                          \
    do {                                                                                         \
        if ((unsigned long long)(long long)(v) >= (unsigned long long)(long long)(bound)) {     \
            ::steps::check_failed((long long)(v), (long long)(bound), (site));                   \
            (v) = 0;                                                                             \
        }                                                                                        \
    } while (0)

// True when the cells [first, last] lie in [0, bound); otherwise records the
// offending end and returns false (the caller then moves the access to 0).
static __device__ __forceinline__ bool check_span(long long first, long long last, long long bound, int site)
{
    if (first >= 0 && last < bound) return true;
    check_failed(first < 0 ? first : last, bound, site);
    return false;
}

// Each translation unit registers where its record lives; the C-ABI reads
// every record after each call.
int register_check_record(void *(*where)());
static void *check_record_address()
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_check_record) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
static const int g_check_registered = register_check_record(&check_record_address);
#else
#define STEPS_CHECK_IDX(v, bound, site) ((void)0)
#endif

// ---------------------------------------------------- device math helpers --

// Order-preserving integer image of a double (atomic min/max of bounding boxes).
__device__ __forceinline__ unsigned long long ordered_bits(double d)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double from_ordered_bits(unsigned long long u)
{
    unsigned long long b = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ unsigned long long spread3(unsigned long long v)
{
    // Spread the low 21 bits of v to every third bit.
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}



// MUFU reciprocal square root, approximate (relative error < 2^-22), FTZ.
__device__ __forceinline__ float rsqrt_mufu(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float sqrt_mufu(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float rcp_mufu(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// FP64 1/sqrt(x) for 1e-36 < x < 1e36: a single-precision MUFU seed (relative
// error e0 < 2^-22) refined by one third-order Householder step of Newton's
// iteration for f(y) = y^-2 - x, i.e. the binomial series of (1 - e)^(-1/2):
//   e = 1 - x y^2,  y' = y (1 + e/2 + 3 e^2 / 8),  error O(e0^3) < 1e-19,
// so the result is within a couple of ulp of 1/sqrt(x).
__device__ __forceinline__ double rsqrt_fp64(double x)
{
    double y = (double)rsqrt_mufu(__double2float_rn(x));
    double t = x * y;
    double e = fma(-t, y, 1.0);
    double p = fma(0.375, e, 0.5);
    return fma(y * e, p, y);
}

// Cubic-spline softened force coefficient w(r, beta) for r < beta (the
// r >= beta branch is 1/r^3). StePS/src/forces.cc:52-87,
// StePS/src/forces_cuda.cu:466-519, written in u = r / beta:
//   u <= 1/2 : (32 u^3 - 38.4 u^2 + 32/3) / beta^3
//   u >  1/2 : (-32/3 u^3 + 38.4 u^2 - 48 u + 64/3) / beta^3 - (1/15) / r^3
__device__ __forceinline__ double spline_inner_fp64(double r, double beta)
{
    double ib = 1.0 / beta;
    double u = r * ib;
    double ib3 = ib * ib * ib;
    if (u <= 0.5) return ib3 * (u * u * (32.0 * u - 38.4) + 32.0 / 3.0);
    double r3 = r * r * r;
    return ib3 * (u * (u * (-32.0 / 3.0 * u + 38.4) - 48.0) + 64.0 / 3.0) - (1.0 / 15.0) / r3;
}

__device__ __forceinline__ double softening_fp64(double r2, double beta)
{
    if (r2 >= beta * beta) {
        double y = rsqrt_fp64(r2);
        return y * y * y;
    }
    return spline_inner_fp64(sqrt(r2), beta);
}

__device__ __forceinline__ float spline_inner_f32(float r2, float beta)
{
    float r = sqrt_mufu(r2);
    float ib = rcp_mufu(beta);
    float u = r * ib;
    float ib3 = ib * ib * ib;
    if (u <= 0.5f) return ib3 * (u * u * (32.0f * u - 38.4f) + (32.0f / 3.0f));
    float ir = rcp_mufu(r);
    return ib3 * (u * (u * (-32.0f / 3.0f * u + 38.4f) - 48.0f) + (64.0f / 3.0f)) -
           (1.0f / 15.0f) * ir * ir * ir;
}

}  // namespace steps
