// Shared pieces of the mixed-precision pair kernels (pair_mixed.cu, pair_t3.cu):
// the argument block, cp.async staging of j tiles, TwoSum and box gaps.
#pragma once

#include "common.cuh"

namespace steps {
namespace mixed {

enum Kind { K_R3 = 0, K_S1_IMG = 1, K_S1_GEN = 2 };

struct MixedArgs {
    const float4 *jpack;
    const float *jeps;
    const float4 *jmeta;
    const uint32_t *jidx;
    const float4 *jres;  // FP32 residuals of the j offsets (double-float near path)
    const float *jsoa;   // tile-blocked SoA copy of jpack (packed-FP32 kernel)
    const float4 *jsub;  // j sub-tile boxes, 2 float4 per SUBTILE particles (packed-FP32 kernel)
    int njt;
    const float4 *ipack;
    const float *ieps;
    const float4 *imeta;
    const uint32_t *iidx;
    const float4 *ilo;
    int nit;
    int S, tpc;  // j chunks per i tile, j tiles per chunk
    int nitems;
    int istride;  // item -> i tile (item / S) * istride: 1, or > 1 when the autotuner times a sample of i tiles
    unsigned *counter;
    int *status;        // STEPS_E_TIMEOUT written here by a pipeline wait that gave up
    long long stall_seq;  // test hook: block 0 withholds the copy of its tile number stall_seq (-1: none)
    const int4 *items;  // work list (batches): i tile, j tile begin, j tile end, partial slot
    int nslots;         // partial slots of the work list (bounds checks)
    double *part;       // [S][nit*T][3]
    size_t part_stride; // nit*T*3
    float L, halfL, cutL;
    float L_lo, halfL_lo;  // L - fl(L), L/2 - fl(L/2): the FP32 residuals of the period
    float wrap_tol;     // |d| this close to L/2 takes the nearest-image decision on an exact d
    float cut_tol;      // |dz + mL| this close to cutL is re-decided on an exact dz
    float guard2;       // square of the precision guard ratio (coarse_for_gap)
    int emax;
    int nearest;        // S1R2 IS_PERIODIC == 1: nearest image along z only
    // T^3 Ewald table (FP32 copy, one float4 per cell) and its geometry
    const float4 *t3f;
    int ng;
    float ih, u0;       // continuous cell index u(d) = d * ih + u0, ih = ng / L, u0 = ng/2 - 1/2
    int wcap;           // cells of the shared-memory table window
    int halo, ext;      // the FP32 copy is haloed: ext^3 cells, ext = ng + 2 halo
    const float4 *t3r;  // stencil records of the haloed copy: x, y components (2 float4 per cell)
    const float4 *t3rz; // ... and the z component (1 float4 per cell)
    // S1xR2 (rho, z) correction table (FP32 float2 copy) and its geometry
    const float2 *s1tab;
    const float4 *s1rec;  // records of s1tab: whole CIC stencils (32 bytes), TSC z triplets
    int nrho, nz;
    float irho, iz, rho_max;  // 1 / drho, nz / L_z
    double s1_drho, s1_dzc, s1_L;  // rho and z cell sizes and L in FP64 (exact NGP face decisions)
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <int BLOCK, int IPT>
__device__ __forceinline__ void stage_tile(const MixedArgs &a, int J, float4 *sp, float *se, uint32_t *sid,
                                           float4 *sres)
{
    constexpr int T = BLOCK * IPT;
    STEPS_CHECK_IDX(J, a.njt, CK_J_TILE);
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        int e = k * BLOCK + threadIdx.x;
        size_t q = (size_t)J * T + e;
        cp_async16(sp + e, a.jpack + q);
        cp_async4(se + e, a.jeps + q);
        cp_async4(sid + e, a.jidx + q);
        cp_async16(sres + e, a.jres + q);
    }
    cp_commit();
}

// a - b = s + e exactly (Knuth's TwoSum on a + (-b)); returns s, writes e.
__device__ __forceinline__ float two_diff(float a, float b, float &e)
{
    const float s = a - b;
    const float bb = s - a;
    e = (a - (s - bb)) + (-b - bb);
    return s;
}

// The FP32 tile offsets carry ~6e-8 of the tile-pair scale |d_O| + h_I + h_J,
// so a pair at distance r gets a relative error ~6e-8 * scale / r. Where the
// scale exceeds `guard` times the box gap (guard2 = guard^2), the block takes
// the double-float (full) path instead.
__device__ __forceinline__ bool coarse_for_gap(float dOx, float dOy, float dOz, float4 hI, float4 hJ, float g2,
                                               float guard2)
{
    const float s = sqrtf(dOx * dOx + dOy * dOy + dOz * dOz) + sqrtf(hI.x * hI.x + hI.y * hI.y + hI.z * hI.z) +
                    sqrtf(hJ.x * hJ.x + hJ.y * hJ.y + hJ.z * hJ.z);
    return s * s > guard2 * g2;
}

// i particle k in J's frame as an unevaluated sum ph + pl: ph = fl(x_hi - dO),
// pl = its rounding error (exact) - eO + x_lo.
__device__ __forceinline__ void frame_split(float xh, float xl, float dO, float eO, float &ph, float &pl)
{
    float e;
    ph = two_diff(xh, dO, e);
    pl = (e - eO) + xl;
}

// Moves J's centre to its image nearest I's along one axis: d_O + e_O
// becomes d_O + e_O - k L with k = rint(d_O / L). The subtraction's rounding
// and the FP32 residual of L go into e_O, so the frame change stays exact.
__device__ __forceinline__ void shift_frame(float &dO, float &eO, float L, float L_lo)
{
    const float k = rintf(dO / L);
    if (k != 0.0f) {
        float e;
        dO = two_diff(dO, k * L, e);
        eO = (eO + e) - k * L_lo;
    }
}

// Nearest image along one axis, |d| > L/2 -> d - sign(d) L
// (StePS/src/forces.cc:812-817), for the double-float separation
// d = (q + ql) - (ph + pl) whose FP32 rounding is d. Within wrap_tol of L/2
// the decision is taken on the unrounded sum, so FP32 rounding never picks
// another image than the FP64 reference (a flip reverses the pair's force).
__device__ __forceinline__ float nearest_image(float d, float q, float ph, float ql, float pl, float L, float halfL,
                                               float halfL_lo, float wrap_tol)
{
    const float ad = fabsf(d);
    bool w = ad > halfL;
    if (fabsf(ad - halfL) < wrap_tol) {
        float e;
        const float s = two_diff(q, ph, e);
        const float t = e + (ql - pl);
        // |s + t| - L/2 with |s| - fl(L/2) exact (Sterbenz); its sign is the decision.
        w = (fabsf(s) - halfL) + (copysignf(1.0f, s) * t - halfL_lo) > 0.0f;
    }
    return w ? d - copysignf(L, d) : d;
}

// The S1xR2 image cut |dz + sh| <= cutL (StePS/src/forces.cc:1274) decided on
// the double-float dz = (qz + qlz) - (phz + plz): a hard cut, so within FP32
// rounding of it the rounded dz could decide differently than FP64.
__device__ __forceinline__ bool cut_in_exact(float qz, float qlz, float phz, float plz, float sh, float cutL)
{
    float e1, e2;
    const float s1 = two_diff(qz, phz, e1);
    const float hh = two_diff(s1, -sh, e2);
    const float tail = e2 + (e1 + (qlz - plz));
    return (fabsf(hh) - cutL) + copysignf(1.0f, hh) * tail <= 0.0f;
}

// Lower bound of |d| over the separations of two boxes along one axis.
__device__ __forceinline__ float axis_gap(float dO, float hI, float hJ) { return fmaxf(fabsf(dO) - hI - hJ, 0.0f); }

// Box of the i particles of this warp (FP32 offsets from I's centre, IPT per
// lane): centre c and half extents h, widened by 1e-6 relative so that it also
// holds the exact positions (offset + residual) whatever the FP32 rounding.
template <int IPT>
__device__ __forceinline__ void warp_box(const float *xi, const float *yi, const float *zi, float4 &c, float4 &h)
{
    float lo[3] = {xi[0], yi[0], zi[0]}, hi[3] = {xi[0], yi[0], zi[0]};
#pragma unroll
    for (int k = 1; k < IPT; k++) {
        lo[0] = fminf(lo[0], xi[k]); hi[0] = fmaxf(hi[0], xi[k]);
        lo[1] = fminf(lo[1], yi[k]); hi[1] = fmaxf(hi[1], yi[k]);
        lo[2] = fminf(lo[2], zi[k]); hi[2] = fmaxf(hi[2], zi[k]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    float cc[3], hh[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        cc[d] = 0.5f * (lo[d] + hi[d]);
        hh[d] = fmaxf(hi[d] - cc[d], cc[d] - lo[d]) * 1.000001f + 1e-6f * fabsf(cc[d]);
    }
    c = make_float4(cc[0], cc[1], cc[2], 0.0f);
    h = make_float4(hh[0], hh[1], hh[2], 0.0f);
}

// Whether a warp with i box (c, h) in I's frame needs the near-field path
// against tile J (offset d_O from I's centre, half extents hJ): some pair may
// be closer than bmax = eps_max(I) + eps_max(J), or the FP32 scale of its
// offsets is coarse for its gap (coarse_for_gap). The box offset carries the
// FP32 rounding of d_O - c, covered by 1e-6 of |d_O| + |c|.
__device__ __forceinline__ bool warp_full(float dOx, float dOy, float dOz, float4 c, float4 h, float4 hJ, float bmax,
                                          float guard2)
{
    const float dx = dOx - c.x, dy = dOy - c.y, dz = dOz - c.z;
    const float4 hw = make_float4(h.x + 1e-6f * (fabsf(dOx) + fabsf(c.x)), h.y + 1e-6f * (fabsf(dOy) + fabsf(c.y)),
                                  h.z + 1e-6f * (fabsf(dOz) + fabsf(c.z)), 0.0f);
    const float gx = axis_gap(dx, hw.x, hJ.x), gy = axis_gap(dy, hw.y, hJ.y), gz = axis_gap(dz, hw.z, hJ.z);
    const float g2 = gx * gx + gy * gy + gz * gz;
    return g2 <= bmax * bmax * 1.0001f + 1e-30f || coarse_for_gap(dx, dy, dz, hw, hJ, g2, guard2);
}

// warp_full for one j sub-tile: box centre s (offset from J's centre, with
// the sub-tile's largest softening in s.w) and half extents hs. The gap is the
// sub-tile's; the FP32 error scale stays that of the offsets actually used --
// i in J's frame (|d_O - c| + |h|) and j relative to J's centre (|s| + |hs|).
__device__ __forceinline__ bool warp_full_sub(float dOx, float dOy, float dOz, float4 s, float4 hs, float4 c,
                                              float4 h, float wemax, float guard2)
{
    const float ex = dOx - c.x, ey = dOy - c.y, ez = dOz - c.z;  // J's centre from the warp box centre
    const float dx = ex + s.x, dy = ey + s.y, dz = ez + s.z;
    const float4 hw = make_float4(h.x + 1e-6f * (fabsf(ex) + fabsf(s.x) + fabsf(c.x)),
                                  h.y + 1e-6f * (fabsf(ey) + fabsf(s.y) + fabsf(c.y)),
                                  h.z + 1e-6f * (fabsf(ez) + fabsf(s.z) + fabsf(c.z)), 0.0f);
    const float gx = axis_gap(dx, hw.x, hs.x), gy = axis_gap(dy, hw.y, hs.y), gz = axis_gap(dz, hw.z, hs.z);
    const float g2 = gx * gx + gy * gy + gz * gz;
    const float bmax = wemax + s.w;
    const float sc = sqrtf(ex * ex + ey * ey + ez * ez) + sqrtf(hw.x * hw.x + hw.y * hw.y + hw.z * hw.z) +
                     sqrtf(s.x * s.x + s.y * s.y + s.z * s.z) + sqrtf(hs.x * hs.x + hs.y * hs.y + hs.z * hs.z);
    return g2 <= bmax * bmax * 1.0001f + 1e-30f || sc * sc > guard2 * g2;
}

// Packed FP32 pairs (PTX .f32x2, sm_100+).
typedef unsigned long long f2;  // two FP32 values in a 64-bit register pair; low half = first

__device__ __forceinline__ f2 f2_bcast(float v)
{
    f2 r;
    asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// ---- mbarrier + bulk-copy (TMA) pipeline helpers -------------------------

// SM clock cycles a bounded mbarrier wait lasts before the kernel gives up,
// records STEPS_E_TIMEOUT and returns (about a second; a healthy wait in these
// kernels takes microseconds).
constexpr long long MBAR_WAIT_CYCLES = 2000000000LL;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity to complete; false after
// MBAR_WAIT_CYCLES (the caller records the error and leaves).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > MBAR_WAIT_CYCLES) return false;
    return true;
}
// Bulk copy global -> shared of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completion counted on the mbarrier as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

using KernelFn = void (*)(MixedArgs);

// The persistent ensemble kernel (pair_r3x2.cu): every force evaluation and
// KDK step of a batch of realisations in one launch. Tasks are (stage, item)
// for stage 0 .. nstages - 1 (stage 0: the initial force; stage s >= 1: the
// force after step s) over the batch's work list, largest realisation first.
// Tile data that the run rewrites (offsets, residuals, metadata, sub-tile
// boxes) are double-buffered: stage s reads buffer s & 1.
struct EnsembleArgs {
    const float4 *pack[2];  // i offsets (x - c, y - c, z - c, m)
    const float *soa[2];    // tile-blocked SoA j copy
    const float4 *resid[2];
    const float4 *meta[2];
    const float4 *sub[2];
    float4 *pack_w[2];      // the same buffers, written by the rebuild
    float *soa_w[2];
    float4 *resid_w[2];
    float4 *meta_w[2];
    float4 *sub_w[2];
    const float *jeps;      // softening (constant over the run)
    const uint32_t *jidx;   // original index of each padded position (constant)
    float *epsf_w;
    const int4 *items;      // work list: i tile, j tile begin, j tile end, partial slot
    int nitems, nstages;
    const int *tile_rel;    // realisation of each tile
    const int2 *tdesc;      // per tile: first sorted position, particle count
    const int2 *tslot;      // per tile: first partial slot, number of slots
    const int *rel_ntiles;  // tiles of each realisation
    const uint32_t *perm;   // sorted position -> original index
    double *part;           // partial slots [slot][T][3]
    unsigned *queue;        // task counter
    unsigned *tile_cnt;     // per tile: items finished, over all stages
    unsigned *rel_done;     // per realisation: tiles finished (forces, kicks, drift, rebuild), over all stages
    double *x, *v, *F;      // caller-order FP64 positions, velocities, forces
    const double *m64, *eps64;
    double h;               // fixed step; acceleration g F a^-3 - 2 H v with g = 1, a = 1, H = 0
    float guard2;
    int *status;            // STEPS_E_TIMEOUT when a stage wait gave up
    int stall_rel;          // test hook: this realisation's stage-0 tiles are never reported done (-1: none)
    int ntiles, nslots, nrel, n;  // tiles, partial slots, realisations, particles (bounds checks)
};
using EnsembleFn = void (*)(EnsembleArgs);

}  // namespace mixed

// pair_t3.cu: T^3 kernel for a shape (dynamic shared memory returned) and its
// table arguments (FP32 table copy, grid geometry).
// variant 0: one i per lane (optionally with the shared-memory window);
// variant 1: quad lanes where t3_quad_kernel has them (trilinear, one i per
// thread), else as 0.
mixed::KernelFn t3_kernel(const KParams &kp, int threads, int ipt, size_t *dyn_smem, int variant = 0);
mixed::KernelFn t3_quad_kernel(const KParams &kp, int threads, int ipt);
constexpr int T3_VARIANTS = 2;
void t3_args(mixed::MixedArgs &a, const KParams &kp, const Tables &tb, cudaStream_t st);
// pair_r3x2.cu: R^3 kernel on packed FP32 pairs; occ = 0, 768 or 1024
// resident threads per SM requested from the register allocator.
mixed::KernelFn r3x2_kernel(int threads, int ipt, bool list = false, int occ = 0);
// Resident-thread request of a packed R^3 kernel variant (1, 2, 3).
inline int r3x2_occ(int variant) { return variant == 2 ? 768 : variant == 3 ? 1024 : 0; }
// pair_r3x2.cu: the packed R^3 kernel with its j tiles streamed by bulk
// copies through an mbarrier ring (variant 4).
mixed::KernelFn r3x2_pipe_kernel(int threads, int ipt);
constexpr int R3_VARIANTS = 5;  // 0 scalar, 1-3 packed, 4 packed + bulk-copy pipeline
// pair_r3x2.cu: the persistent ensemble kernel for a shape.
mixed::EnsembleFn ensemble_kernel(int threads, int ipt);
// S1xR2 with the (rho, z) table (IS_PERIODIC >= 2, no explicit images).
mixed::KernelFn s1tab_kernel(const KParams &kp, int threads, int ipt);
void s1tab_args(mixed::MixedArgs &a, const KParams &kp, const Tables &tb, cudaStream_t st);

}  // namespace steps
