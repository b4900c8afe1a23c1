// Mixed-precision R^3 kernel on packed FP32 pairs (PTX .f32x2 add/sub/mul/fma,
// sm_100+): the same algorithm, tiling and accuracy as k_pair_mixed<K_R3>
// (pair_mixed.cu), with the far-field pair arithmetic issued two pairs per
// instruction.
//
// The scalar far-field loop needs 12 FP32 instructions + 1 MUFU + 1/ipt LDS
// per pair and is issue-bound (one instruction per cycle per SM sub-partition).
// Packed, one thread holds each i as a broadcast pair {p, p} and meets two j
// particles at a time: X[jj..jj+1] from the tile's SoA block in shared memory
// is already the packed operand {q_jj, q_jj+1}. Per two pairs: 3 FADD2 (d),
// FMUL2 + 2 FFMA2 (r^2), 2 MUFU rsqrt, 3 FMUL2 (m r^-3), 3 FFMA2 (accumulate)
// -- 14 issue slots, so the FMA pipe rather than issue becomes the limit.
// Near-field tile pairs (and tile pairs whose FP32 scale is coarse for their
// gap) run the scalar double-float spline path, reading the same SoA block.
#include "common.cuh"
#include "context.cuh"
#include "mixed.cuh"
#include "tile.cuh"

namespace steps {

namespace {

using namespace mixed;

template <int BLOCK, int IPT>
__device__ __forceinline__ void stage_soa(const MixedArgs &a, int J, float *sx, float *se, uint32_t *sid, float4 *sres,
                                          float4 *ssub)
{
    constexpr int T = BLOCK * IPT;
    constexpr int NS2 = 2 * (T / SUBTILE);  // float4 of sub-tile boxes per tile
    STEPS_CHECK_IDX(J, a.njt, CK_J_TILE);
    const float4 *src = reinterpret_cast<const float4 *>(a.jsoa + (size_t)J * 4 * T);
    float4 *dst = reinterpret_cast<float4 *>(sx);
    for (int e = threadIdx.x; e < NS2; e += BLOCK) cp_async16(ssub + e, a.jsub + (size_t)J * NS2 + e);
#pragma unroll
    for (int k = 0; k < IPT; k++) {  // 4T floats = T float4 chunks
        const int e = k * BLOCK + threadIdx.x;
        const size_t q = (size_t)J * T + e;
        cp_async16(dst + e, src + e);
        cp_async4(se + e, a.jeps + q);
        cp_async4(sid + e, a.jidx + q);
        cp_async16(sres + e, a.jres + q);
    }
    cp_commit();
}

// v, made to depend on dep (an opaque move): keeps a computation from v
// inside the loop that dep varies in.
__device__ __forceinline__ float pin_to(float v, int dep)
{
    float r;
    asm("mov.b32 %0, %1; // %2" : "=f"(r) : "f"(v), "r"(dep));
    return r;
}

// One j tile J against this thread's i particles: the staged tile is sxb
// (X[T], Y[T], Z[T], M[T]), seb (softening), sidb (ids), sresb (residuals).
// The near/far decision is taken per (warp, j sub-tile of SUBTILE particles)
// from the sub-tile boxes: lane s classifies sub-tile s, a ballot gathers the
// warp-uniform mask, and runs of far sub-tiles take the packed loop while
// near (or coarse-scale) sub-tiles take the scalar double-float path.
// mJ0: tile J's FP32 centre and largest softening (its first metadata float4).
template <int BLOCK, int IPT>
__device__ __forceinline__ void r3x2_tile(float4 mJ0, float guard2, const float *sxb, const float *seb,
                                          const uint32_t *sidb, const float4 *sresb, const float4 *ssubb, float4 mI0,
                                          float4 wc, float4 wh, float wemax, const float *xi, const float *yi,
                                          const float *zi, const float *ei, const float *lx, const float *ly,
                                          const float *lz, const uint32_t *ii, double *ax, double *ay, double *az)
{
    constexpr int T = BLOCK * IPT;
    constexpr int NS = T / SUBTILE;  // 4 .. 32 sub-tiles
    constexpr unsigned ALL = NS == 32 ? 0xffffffffu : (1u << NS) - 1u;
    float eOx, eOy, eOz;
    const float dOx = two_diff(mJ0.x, mI0.x, eOx), dOy = two_diff(mJ0.y, mI0.y, eOy),
                dOz = two_diff(mJ0.z, mI0.z, eOz);
    // Near field / coarse FP32 scale per (warp, sub-tile), warp-uniform.
    const int lane = threadIdx.x & 31;
    bool f = false;
    if (lane < NS) f = warp_full_sub(dOx, dOy, dOz, ssubb[2 * lane], ssubb[2 * lane + 1], wc, wh, wemax, guard2);
    const unsigned full = __ballot_sync(0xffffffffu, f) & ALL;
    const float *X = sxb;
    const float *Y = X + T;
    const float *Z = X + 2 * T;
    const float *Mq = X + 3 * T;

    // Segments of consecutive sub-tiles with the same decision, in order;
    // each takes one path and folds its FP32 sums into the FP64 accumulators.
    unsigned rem = ALL;
    while (rem) {
        const int s0 = __ffs(rem) - 1;
        const bool nearseg = (full >> s0) & 1u;
        const unsigned same = (nearseg ? full : ~full) & ALL;
        const unsigned rest = ~(same >> s0);
        const int s1 = rest ? s0 + __ffs(rest) - 1 : 32;
        rem = s1 >= 32 ? 0u : rem & ~((1u << s1) - 1u);
        // The frame offsets pass through a move that depends on the segment,
        // so neither path's set-up is hoisted out of this loop (both would
        // then stay live across the other path and cost registers).
        const float oX = pin_to(dOx, s0), oY = pin_to(dOy, s0), oZ = pin_to(dOz, s0);
        if (!nearseg) {
            // Far field: packed FP32x2.
            f2 PX[IPT], PY[IPT], PZ[IPT], AX[IPT], AY[IPT], AZ[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                PX[k] = f2_bcast(((xi[k] - oX) - eOx) + lx[k]);
                PY[k] = f2_bcast(((yi[k] - oY) - eOy) + ly[k]);
                PZ[k] = f2_bcast(((zi[k] - oZ) - eOz) + lz[k]);
                AX[k] = AY[k] = AZ[k] = 0ull;  // {+0, +0}
            }
#pragma unroll 2
            for (int jj = s0 * SUBTILE; jj < s1 * SUBTILE; jj += 4) {
                const ulonglong2 qx4 = *reinterpret_cast<const ulonglong2 *>(X + jj);
                const ulonglong2 qy4 = *reinterpret_cast<const ulonglong2 *>(Y + jj);
                const ulonglong2 qz4 = *reinterpret_cast<const ulonglong2 *>(Z + jj);
                const ulonglong2 qm4 = *reinterpret_cast<const ulonglong2 *>(Mq + jj);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const f2 qx = h ? qx4.y : qx4.x, qy = h ? qy4.y : qy4.x, qz = h ? qz4.y : qz4.x;
                    const f2 qm = h ? qm4.y : qm4.x;
#pragma unroll
                    for (int k = 0; k < IPT; k++) {
                        const f2 dx = f2_sub(qx, PX[k]), dy = f2_sub(qy, PY[k]), dz = f2_sub(qz, PZ[k]);
                        const f2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
                        float r2a, r2b;
                        f2_unpack(r2, r2a, r2b);
                        const f2 ri = f2_pack(rsqrt_mufu(r2a), rsqrt_mufu(r2b));
                        const f2 w = f2_mul(f2_mul(qm, ri), f2_mul(ri, ri));
                        AX[k] = f2_fma(w, dx, AX[k]);
                        AY[k] = f2_fma(w, dy, AY[k]);
                        AZ[k] = f2_fma(w, dz, AZ[k]);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                float l0, l1;
                f2_unpack(AX[k], l0, l1);
                ax[k] += (double)(l0 + l1);
                f2_unpack(AY[k], l0, l1);
                ay[k] += (double)(l0 + l1);
                f2_unpack(AZ[k], l0, l1);
                az[k] += (double)(l0 + l1);
            }
        } else {
            // Near field: scalar double-float path with the spline
            // (StePS/src/forces.cc:52-87); the self pair gets d = 0.
            float phx[IPT], phy[IPT], phz[IPT], plx[IPT], ply[IPT], plz[IPT], fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                frame_split(xi[k], lx[k], oX, eOx, phx[k], plx[k]);
                frame_split(yi[k], ly[k], oY, eOy, phy[k], ply[k]);
                frame_split(zi[k], lz[k], oZ, eOz, phz[k], plz[k]);
                fx[k] = fy[k] = fz[k] = 0.0f;
            }
            for (int jj = s0 * SUBTILE; jj < s1 * SUBTILE; ++jj) {
                const float qx = X[jj], qy = Y[jj], qz = Z[jj], qm = Mq[jj];
                const float ej = seb[jj];
                const uint32_t jid = sidb[jj];
                const float4 ql = sresb[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const bool self = jid == ii[k];
                    const float dx = self ? 0.0f : (qx - phx[k]) + (ql.x - plx[k]);
                    const float dy = self ? 0.0f : (qy - phy[k]) + (ql.y - ply[k]);
                    const float dz = self ? 0.0f : (qz - phz[k]) + (ql.z - plz[k]);
                    const float b = ei[k] + ej;
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float ri = rsqrt_mufu(r2);
                    float w = ri * ri * ri;
                    if (r2 < b * b) w = spline_inner_f32(r2, b);
                    w *= qm;
                    fx[k] = fmaf(w, dx, fx[k]);
                    fy[k] = fmaf(w, dy, fy[k]);
                    fz[k] = fmaf(w, dz, fz[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                ax[k] += (double)fx[k];
                ay[k] += (double)fy[k];
                az[k] += (double)fz[k];
            }
        }
    }
}

// Largest softening length of this warp's i particles.
template <int IPT>
__device__ __forceinline__ float warp_eps_max(const float *ei)
{
    float e = ei[0];
#pragma unroll
    for (int k = 1; k < IPT; k++) e = fmaxf(e, ei[k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    return e;
}

template <int BLOCK, int IPT, bool LIST>
__device__ __forceinline__ void r3x2_body(const MixedArgs &a)
{
    constexpr int T = BLOCK * IPT;
    __shared__ __align__(16) float sx[2][4 * T];  // X[T], Y[T], Z[T], M[T]
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ __align__(16) float4 sres[2][T];
    __shared__ __align__(16) float4 ssub[2][2 * (T / SUBTILE)];
    __shared__ int s_item;
    const int tid = threadIdx.x;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.nitems) return;
        int I, J0, J1;
        size_t base;  // where this item's T partial forces go
        if (LIST) {
            const int4 d = __ldg(a.items + item);
            I = d.x;
            J0 = d.y;
            J1 = d.z;
            int slot = d.w;
            STEPS_CHECK_IDX(slot, a.nslots, CK_SLOT);
            STEPS_CHECK_IDX(I, a.nit, CK_I_TILE);
            base = (size_t)slot * 3 * T;
        } else {
            I = (item / a.S) * a.istride;
            const int chunk = item % a.S;
            J0 = chunk * a.tpc;
            J1 = min(a.njt, J0 + a.tpc);
            STEPS_CHECK_IDX(I, a.nit, CK_I_TILE);
            base = (size_t)chunk * a.part_stride + 3 * (size_t)I * T;
        }

        const float4 mI0 = __ldg(a.imeta + 2 * I);
        const float4 mI1 = __ldg(a.imeta + 2 * I + 1);
        float xi[IPT], yi[IPT], zi[IPT], ei[IPT], lx[IPT], ly[IPT], lz[IPT];
        uint32_t ii[IPT];
        double ax[IPT], ay[IPT], az[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t q = (size_t)I * T + k * BLOCK + tid;
            const float4 p = __ldg(a.ipack + q);
            xi[k] = p.x;
            yi[k] = p.y;
            zi[k] = p.z;
            ei[k] = __ldg(a.ieps + q);
            ii[k] = __ldg(a.iidx + q);
            const float4 l = __ldg(a.ilo + q);
            lx[k] = l.x;
            ly[k] = l.y;
            lz[k] = l.z;
            ax[k] = ay[k] = az[k] = 0.0;
        }

        float4 wc, wh;  // this warp's i box in I's frame
        warp_box<IPT>(xi, yi, zi, wc, wh);
        const float wemax = warp_eps_max<IPT>(ei);

        if (J0 < J1) stage_soa<BLOCK, IPT>(a, J0, sx[0], se[0], sid[0], sres[0], ssub[0]);
        for (int J = J0; J < J1; ++J) {
            const int buf = (J - J0) & 1;
            if (J + 1 < J1) {
                stage_soa<BLOCK, IPT>(a, J + 1, sx[buf ^ 1], se[buf ^ 1], sid[buf ^ 1], sres[buf ^ 1], ssub[buf ^ 1]);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();

            r3x2_tile<BLOCK, IPT>(__ldg(a.jmeta + 2 * J), a.guard2, sx[buf], se[buf], sid[buf], sres[buf], ssub[buf], mI0, wc, wh, wemax, xi, yi,
                                  zi, ei, lx, ly, lz, ii, ax, ay, az);
            __syncthreads();
        }

        double *o = a.part + base;
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t e = k * BLOCK + tid;
            o[3 * e] = ax[k];
            o[3 * e + 1] = ay[k];
            o[3 * e + 2] = az[k];
        }
    }
}

// The same work as r3x2_body with the j tiles streamed through an S-stage
// shared-memory ring filled by bulk copies (cp.async.bulk, the TMA engine)
// and tracked by mbarriers: full[s] completes when stage s has landed,
// empty[s] when every warp has finished with it. Thread 0 issues the copy of
// tile J + S - 1 when it starts tile J, so warps wait only for their data,
// never for each other, and drift up to S - 1 tiles apart (no block-wide
// barrier per tile). Every wait is bounded: a wait that gives up writes
// STEPS_E_TIMEOUT to a.status, the block stops taking work, and thread 0
// waits (bounded) for its copies in flight before the block exits.
template <int BLOCK, int IPT>
__device__ __forceinline__ void r3x2_pipe_body(const MixedArgs &a)
{
    constexpr int T = BLOCK * IPT;
    constexpr int S = T <= 256 ? 4 : 2;
    constexpr int NW = BLOCK / 32;
    constexpr int NS2 = 2 * (T / SUBTILE);
    // SoA 16T + softening 4T + ids 4T + residuals 16T + sub-tile boxes 2T
    constexpr unsigned BYTES = 40u * T + 16u * NS2;
    __shared__ __align__(128) float sx[S][4 * T];  // per stage X[T], Y[T], Z[T], M[T]
    __shared__ __align__(16) float se[S][T];
    __shared__ __align__(16) uint32_t sid[S][T];
    __shared__ __align__(16) float4 sres[S][T];
    __shared__ __align__(16) float4 ssub[S][NS2];
    __shared__ __align__(8) unsigned long long full[S], empty[S];
    __shared__ int s_item, s_abort;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) {
        for (int st = 0; st < S; st++) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], NW);
        }
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();
    unsigned long long issued = 0;    // tiles whose copy thread 0 has issued
    unsigned long long consumed = 0;  // tiles this thread's warp has finished (the same in every warp)
    auto issue = [&](int J) -> bool {  // thread 0
        STEPS_CHECK_IDX(J, a.njt, CK_J_TILE);
        const int st = (int)(issued % S);
        if (issued >= S && !mbar_wait(&empty[st], (unsigned)((issued / S - 1) & 1))) return false;
        mbar_arrive_expect_tx(&full[st], BYTES);
        // test hook: withhold one copy so that the waits on it run out
        if (!(blockIdx.x == 0 && (long long)issued == a.stall_seq)) {
            bulk_g2s(sx[st], a.jsoa + (size_t)J * 4 * T, 16u * T, &full[st]);
            bulk_g2s(se[st], a.jeps + (size_t)J * T, 4u * T, &full[st]);
            bulk_g2s(sid[st], a.jidx + (size_t)J * T, 4u * T, &full[st]);
            bulk_g2s(sres[st], a.jres + (size_t)J * T, 16u * T, &full[st]);
            bulk_g2s(ssub[st], a.jsub + (size_t)J * NS2, 16u * NS2, &full[st]);
        }
        issued++;
        return true;
    };
    auto abort_block = [&]() {
        s_abort = 1;
        atomicExch(a.status, STEPS_E_TIMEOUT);
    };

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = s_abort ? a.nitems : (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.nitems) break;
        int I = (item / a.S) * a.istride;
        STEPS_CHECK_IDX(I, a.nit, CK_I_TILE);
        const int chunk = item % a.S;
        const int J0 = chunk * a.tpc;
        const int J1 = min(a.njt, J0 + a.tpc);
        const size_t base = (size_t)chunk * a.part_stride + 3 * (size_t)I * T;

        const float4 mI0 = __ldg(a.imeta + 2 * I);
        float xi[IPT], yi[IPT], zi[IPT], ei[IPT], lx[IPT], ly[IPT], lz[IPT];
        uint32_t ii[IPT];
        double ax[IPT], ay[IPT], az[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t q = (size_t)I * T + k * BLOCK + tid;
            const float4 p = __ldg(a.ipack + q);
            xi[k] = p.x;
            yi[k] = p.y;
            zi[k] = p.z;
            ei[k] = __ldg(a.ieps + q);
            ii[k] = __ldg(a.iidx + q);
            const float4 l = __ldg(a.ilo + q);
            lx[k] = l.x;
            ly[k] = l.y;
            lz[k] = l.z;
            ax[k] = ay[k] = az[k] = 0.0;
        }
        float4 wc, wh;
        warp_box<IPT>(xi, yi, zi, wc, wh);
        const float wemax = warp_eps_max<IPT>(ei);

        bool ok = true;
        if (tid == 0)
            for (int J = J0; J < J1 && J < J0 + S - 1 && ok; J++) ok = issue(J);
        for (int J = J0; J < J1; ++J) {
            bool mine = true;
            if (tid == 0 && ok && J + S - 1 < J1) mine = ok = issue(J + S - 1);
            if (tid == 0 && !ok) mine = false;
            const int st = (int)(consumed % S);
            mine = mine && mbar_wait(&full[st], (unsigned)((consumed / S) & 1));
            if (!__all_sync(0xffffffffu, mine)) {  // warp-uniform
                if (lane == 0) abort_block();
                break;
            }
            r3x2_tile<BLOCK, IPT>(__ldg(a.jmeta + 2 * J), a.guard2, sx[st], se[st], sid[st], sres[st], ssub[st], mI0, wc, wh, wemax, xi, yi, zi, ei,
                                  lx, ly, lz, ii, ax, ay, az);
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            consumed++;
        }

        double *o = a.part + base;
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t e = k * BLOCK + tid;
            o[3 * e] = ax[k];
            o[3 * e + 1] = ay[k];
            o[3 * e + 2] = az[k];
        }
    }
    // After an abort, copies may still be in flight into this block's shared
    // memory: thread 0 waits for them (bounded) before the block exits.
    if (tid == 0)
        for (unsigned long long q = consumed; q < issued; q++) mbar_wait(&full[q % S], (unsigned)((q / S) & 1));
}

template <int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK) k_pair_r3x2_pipe(MixedArgs a)
{
    r3x2_pipe_body<BLOCK, IPT>(a);
}

// Default packed kernel: for blocks of 64 or 128 threads with up to two i
// particles a thread, at least 640 resident threads per SM asked of the
// register allocator (102 registers a thread).
template <int BLOCK, int IPT, bool LIST>
__global__ void __launch_bounds__(BLOCK, BLOCK <= 128 && IPT <= 2 ? 640 / BLOCK : 1) k_pair_r3x2(MixedArgs a)
{
    r3x2_body<BLOCK, IPT, LIST>(a);
}

// The same kernel with OCC resident threads per SM asked of the register
// allocator (65536 / OCC registers a thread): more warps to hide the FP32x2
// and MUFU latencies, at the price of spills for the larger tiles.
template <int BLOCK, int IPT, int OCC>
__global__ void __launch_bounds__(BLOCK, OCC / BLOCK) k_pair_r3x2_occ(MixedArgs a)
{
    r3x2_body<BLOCK, IPT, false>(a);
}

// ---- persistent ensemble kernel --------------------------------------------
//
// One launch runs every stage of a batch run (EnsembleArgs): the initial force
// evaluation and, per KDK step, the force at the drifted positions. A block
// takes (stage, item) tasks from one atomic counter in queue order (stage by
// stage, each stage's items largest realisation first). A stage-s task of
// realisation k may start once all of k's tiles have been finished at stage
// s - 1 -- a bounded wait, which in queue order rarely waits at all, since
// k's previous-stage items were queued long before. The block that completes
// the last item of an i tile at stage s adds the tile's partial slots in
// order (deterministic), writes F, applies the kick of the step that stage
// ends (StePS/src/step.cc:256-262), then the next step's kick and drift
// (step.cc:131-149), and rebuilds the tile into the other buffer; then it
// counts the tile done for its realisation. Particles keep the order of the
// initial sort for the whole run (the forces do not depend on the order).
//
// A wait that gives up (about a second) records STEPS_E_TIMEOUT; every block
// then stops taking tasks, and waits in progress give up at once.

// Bounded spin on a counter another block increments: true once it reaches
// target; false after MBAR_WAIT_CYCLES or as soon as the status word is set.
__device__ __forceinline__ bool wait_counter(const unsigned *cnt, unsigned target, const int *status)
{
    const volatile unsigned *c = cnt;
    const volatile int *st = status;
    if (*c >= target) return true;
    const long long t0 = clock64();
    while (*c < target)
        if (*st != 0 || clock64() - t0 > MBAR_WAIT_CYCLES) return false;
    return true;
}

template <int BLOCK, int IPT>
__device__ __forceinline__ void ensemble_finish_tile(const EnsembleArgs &e, int I, int stage)
{
    constexpr int T = BLOCK * IPT;
    const int tid = threadIdx.x;
    const int2 sl = __ldg(e.tslot + I), td = __ldg(e.tdesc + I);
    const bool kick2 = stage >= 1, kick1 = stage < e.nstages - 1;
    const double h2 = e.h / 2.0;
    for (int p = tid; p < T; p += BLOCK) {
        uint32_t o = __ldg(e.jidx + (size_t)I * T + p);
        if (o == 0xffffffffu) continue;  // padding
        STEPS_CHECK_IDX(o, e.n, CK_PERM);
        double f[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < sl.y; s++) {
            int slot = sl.x + s;
            STEPS_CHECK_IDX(slot, e.nslots, CK_SLOT);
            const double *pc = e.part + ((size_t)slot * T + p) * 3;
            f[0] += __ldcg(pc);
            f[1] += __ldcg(pc + 1);
            f[2] += __ldcg(pc + 2);
        }
        for (int c = 0; c < 3; c++) {
            const size_t q = 3 * (size_t)o + c;
            e.F[q] = f[c];
            double vv = __ldcg(e.v + q);
            // acceleration g F a^-3 - 2 H v at g = 1, a = 1, H = 0, as the batch's KDK kernels evaluate it
            if (kick2) vv += (1.0 * f[c] * 1.0 - 2.0 * 0.0 * vv) * h2;
            if (kick1) {
                vv = vv + (1.0 * f[c] * 1.0 - 2.0 * 0.0 * vv) * h2;
                e.x[q] = __ldcg(e.x + q) + vv * e.h;
            }
            e.v[q] = vv;
        }
    }
    __syncthreads();
    if (kick1) {
        const int nb = (stage + 1) & 1;
        build_tile<BLOCK, true>(I, td.x, td.y, e.x, e.m64, e.eps64, e.perm, e.n, T, e.pack_w[nb], e.epsf_w, e.meta_w[nb],
                                nullptr, 0xffffffffu, e.resid_w[nb], e.soa_w[nb], e.sub_w[nb]);
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        int k = __ldg(e.tile_rel + I);
        STEPS_CHECK_IDX(k, e.nrel, CK_I_TILE);
        if (!(stage == 0 && k == e.stall_rel)) atomicAdd(e.rel_done + k, 1u);
    }
}

template <int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK, BLOCK <= 128 && IPT <= 2 ? 640 / BLOCK : 1) k_ensemble(EnsembleArgs e)
{
    constexpr int T = BLOCK * IPT;
    __shared__ __align__(16) float sx[2][4 * T];
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ __align__(16) float4 sres[2][T];
    __shared__ __align__(16) float4 ssub[2][2 * (T / SUBTILE)];
    __shared__ __align__(16) float4 smeta[2];  // the staged j tile's centre and largest softening
    __shared__ int s_task, s_last;
    const int tid = threadIdx.x;
    const int ntasks = e.nitems * e.nstages;
    // A j tile with its metadata, in one cp.async group, all through L2.
    auto stage_j = [&](const MixedArgs &sa, const float4 *jmeta, int J, int buf) {
        if (tid == 0) cp_async16(&smeta[buf], jmeta + 2 * J);
        stage_soa<BLOCK, IPT>(sa, J, sx[buf], se[buf], sid[buf], sres[buf], ssub[buf]);
    };

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            const volatile int *st = e.status;
            int task = *st != 0 ? ntasks : (int)atomicAdd(e.queue, 1u);
            if (task < ntasks && task >= e.nitems) {  // stage >= 1: wait for the previous stage of this realisation
                const int stage = task / e.nitems;
                int it = __ldg(e.items + task % e.nitems).x;
                STEPS_CHECK_IDX(it, e.ntiles, CK_I_TILE);
                int k = __ldg(e.tile_rel + it);
                STEPS_CHECK_IDX(k, e.nrel, CK_I_TILE);
                if (!wait_counter(e.rel_done + k, (unsigned)(__ldg(e.rel_ntiles + k) * stage), e.status)) {
                    atomicExch(e.status, STEPS_E_TIMEOUT);
                    task = ntasks;
                }
            }
            __threadfence();
            s_task = task;
        }
        __syncthreads();
        const int task = s_task;
        if (task >= ntasks) break;
        const int stage = task / e.nitems;
        const int b = stage & 1;
        const int4 d = __ldg(e.items + task % e.nitems);
        int I = d.x, slot = d.w;
        const int J0 = d.y, J1 = d.z;
        STEPS_CHECK_IDX(I, e.ntiles, CK_I_TILE);
        STEPS_CHECK_IDX(slot, e.nslots, CK_SLOT);
        const float4 *ipack = e.pack[b], *ilo = e.resid[b], *imeta = e.meta[b];

        const float4 mI0 = __ldcg(imeta + 2 * I);
        float xi[IPT], yi[IPT], zi[IPT], ei[IPT], lx[IPT], ly[IPT], lz[IPT];
        uint32_t ii[IPT];
        double ax[IPT], ay[IPT], az[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t q = (size_t)I * T + k * BLOCK + tid;
            const float4 p = __ldcg(ipack + q);
            xi[k] = p.x;
            yi[k] = p.y;
            zi[k] = p.z;
            ei[k] = __ldg(e.jeps + q);
            ii[k] = __ldg(e.jidx + q);
            const float4 l = __ldcg(ilo + q);
            lx[k] = l.x;
            ly[k] = l.y;
            lz[k] = l.z;
            ax[k] = ay[k] = az[k] = 0.0;
        }
        float4 wc, wh;
        warp_box<IPT>(xi, yi, zi, wc, wh);
        const float wemax = warp_eps_max<IPT>(ei);

        MixedArgs a;  // the fields stage_soa reads
        a.njt = e.ntiles;
        a.jsoa = e.soa[b];
        a.jeps = e.jeps;
        a.jidx = e.jidx;
        a.jres = e.resid[b];
        a.jsub = e.sub[b];
        if (J0 < J1) stage_j(a, e.meta[b], J0, 0);
        for (int J = J0; J < J1; ++J) {
            const int buf = (J - J0) & 1;
            if (J + 1 < J1) {
                stage_j(a, e.meta[b], J + 1, buf ^ 1);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();
            r3x2_tile<BLOCK, IPT>(smeta[buf], e.guard2, sx[buf], se[buf], sid[buf], sres[buf], ssub[buf], mI0, wc, wh,
                                  wemax, xi, yi, zi, ei, lx, ly, lz, ii, ax, ay, az);
            __syncthreads();
        }

        double *o = e.part + (size_t)slot * 3 * T;
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const size_t q = k * BLOCK + tid;
            o[3 * q] = ax[k];
            o[3 * q + 1] = ay[k];
            o[3 * q + 2] = az[k];
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned slots = (unsigned)__ldg(e.tslot + I).y;
            s_last = atomicAdd(e.tile_cnt + I, 1u) == slots * (unsigned)(stage + 1) - 1u;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            ensemble_finish_tile<BLOCK, IPT>(e, I, stage);
        }
    }
}

}  // namespace

EnsembleFn ensemble_kernel(int threads, int ipt)
{
#define STEPS_SHAPE(B, P) \
    if (threads == B && ipt == P) return k_ensemble<B, P>;
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(64, 4)
    STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(128, 4)
    STEPS_SHAPE(256, 1) STEPS_SHAPE(256, 2)
#undef STEPS_SHAPE
    return nullptr;
}

KernelFn r3x2_pipe_kernel(int threads, int ipt)
{
#define STEPS_SHAPE(B, P) \
    if (threads == B && ipt == P) return k_pair_r3x2_pipe<B, P>;
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(64, 4)
    STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(128, 4)
    STEPS_SHAPE(256, 1) STEPS_SHAPE(256, 2)
#undef STEPS_SHAPE
    return nullptr;
}

KernelFn r3x2_kernel(int threads, int ipt, bool list, int occ)
{
#define STEPS_SHAPE(B, P)                                                         \
    if (threads == B && ipt == P) {                                              \
        if (list) return occ == 0 ? k_pair_r3x2<B, P, true> : nullptr;          \
        if (occ == 0) return k_pair_r3x2<B, P, false>;                          \
        if (occ == 768) return k_pair_r3x2_occ<B, P, 768>;                      \
        if (occ == 1024) return k_pair_r3x2_occ<B, P, 1024>;                    \
        return nullptr;                                                          \
    }
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(64, 4)
    STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(128, 4)
    STEPS_SHAPE(256, 1) STEPS_SHAPE(256, 2)
#undef STEPS_SHAPE
    return nullptr;
}

}  // namespace steps
