// Mixed-precision direct-summation kernels: FP32 pair arithmetic on
// tile-centred coordinates, FP64 accumulation per i particle.
//
// Layout (built by order.cu): particles sorted along a Morton curve and cut
// into tiles of T = threads * ipt. Each particle is stored as an FP32 offset
// from its tile's centre c (c exactly representable in FP32, the offset
// computed in FP64 then rounded), so an FP32 offset carries ~1e-7 of the
// tile's extent, not of the box.
//
// Work item = (i tile I, j chunk): a persistent block takes items from an
// atomic counter, holds its T i particles in registers (ipt per thread) and
// streams the chunk's j tiles through a double-buffered shared-memory ring
// filled by cp.async. For a tile pair the block forms d_O = c_J - c_I in FP32
// (one rounding), moves its i particles into J's frame (x_i - d_O) and then
// every pair is d = x_j - (x_i - d_O): no FP64 operation per pair and none per
// (i, J) beyond one FP32 subtraction. Per tile pair the FP32 sums are folded
// into FP64 accumulators; partial sums per j chunk go to an FP64 buffer that
// a reduction adds in chunk order (deterministic, no atomics on forces).
//
// Per tile pair the block classifies, from the tiles' boxes and largest
// softening lengths, whether any pair can be closer than its softening
// support beta = eps_i + eps_j (StePS/src/forces.cc:540). Far tile pairs run
// the plain 1/r^3 loop (3 FADD, 3 FMUL/FFMA for r^2, 1 MUFU rsqrt, 3 FMUL,
// 3 FFMA per pair); near ones run the full spline (forces.cc:52-87).
#include <algorithm>

#include "common.cuh"
#include "context.cuh"
#include "mixed.cuh"

namespace steps {

namespace {

using namespace mixed;

template <int KIND, int BLOCK, int IPT, int EMAX>
__global__ void __launch_bounds__(BLOCK, KIND == K_R3 && IPT == 1 ? 1024 / BLOCK : 1) k_pair_mixed(MixedArgs a)
{
    constexpr int T = BLOCK * IPT;
    constexpr int NIMG = KIND == K_S1_IMG ? 2 * EMAX + 1 : 1;
    __shared__ __align__(16) float4 sp[2][T];
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ __align__(16) float4 sres[2][T];
    __shared__ int s_item;
    const int tid = threadIdx.x;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.nitems) return;
        int I = (item / a.S) * a.istride;
        STEPS_CHECK_IDX(I, a.nit, CK_I_TILE);
        const int chunk = item % a.S;
        const int J0 = chunk * a.tpc;
        const int J1 = min(a.njt, J0 + a.tpc);

        const float4 mI0 = __ldg(a.imeta + 2 * I);
        const float4 mI1 = __ldg(a.imeta + 2 * I + 1);
        float xi[IPT], yi[IPT], zi[IPT], ei[IPT], lx[IPT], ly[IPT], lz[IPT];
        uint32_t ii[IPT];
        double ax[IPT], ay[IPT], az[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            size_t q = (size_t)I * T + k * BLOCK + tid;
            float4 p = __ldg(a.ipack + q);
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

        float4 wc = make_float4(0.f, 0.f, 0.f, 0.f), wh = wc;  // this warp's i box in I's frame (R^3)
        if (KIND == K_R3) warp_box<IPT>(xi, yi, zi, wc, wh);

        if (J0 < J1) stage_tile<BLOCK, IPT>(a, J0, sp[0], se[0], sid[0], sres[0]);
        for (int J = J0; J < J1; ++J) {
            const int buf = (J - J0) & 1;
            if (J + 1 < J1) {
                stage_tile<BLOCK, IPT>(a, J + 1, sp[buf ^ 1], se[buf ^ 1], sid[buf ^ 1], sres[buf ^ 1]);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();

            const float4 mJ0 = __ldg(a.jmeta + 2 * J);
            const float4 mJ1 = __ldg(a.jmeta + 2 * J + 1);
            // d_O = c_J - c_I as an unevaluated FP32 sum dO + eO (TwoSum,
            // exact): the i particles' positions in J's frame then carry
            // ~1e-7 of |x_i - c_J| whatever the size of the i tile.
            float eOx, eOy, eOz;
            const float dOx = two_diff(mJ0.x, mI0.x, eOx), dOy = two_diff(mJ0.y, mI0.y, eOy);
            float dOz = two_diff(mJ0.z, mI0.z, eOz);
            const float bmax = mI0.w + mJ0.w;
            const float bmax2 = bmax * bmax * 1.0001f + 1e-30f;
            const float gx = axis_gap(dOx, mI1.x, mJ1.x), gy = axis_gap(dOy, mI1.y, mJ1.y);

            bool full;  // near-field tile pair: softening and every test per pair
            float off[NIMG];
            unsigned long long strad = 0ull;  // S1 images straddling the cut over this tile pair
            // K_S1_GEN with explicit images (any count): the images not entirely
            // outside the cut form [mfirst, mlast]; bit m - mfirst of stradl marks
            // those straddling it.
            int mfirst = 0, mlast = -1;
            unsigned long long stradl = 0ull;
            if (KIND == K_R3) {  // per warp: warps away from a near J keep the far loop
                full = warp_full(dOx, dOy, dOz, wc, wh, mJ1, bmax, a.guard2);
            } else if (KIND == K_S1_IMG) {
                // Range of dz over the tile pair, then per image m: entirely
                // inside the cut (offset m L), entirely outside (offset 1e18,
                // whose 1/r^3 underflows to 0), or straddling (offset m L and
                // a per-pair cut test, bit m of `strad`).
                const float hz = mI1.z + mJ1.z;
                const float lo = dOz - hz, hi = dOz + hz;
                const float g2xy = gx * gx + gy * gy;
                bool near = false;
                float g2min = 3.0e38f;
                const float cin = a.cutL * (1.0f - 1e-6f), cout = a.cutL * (1.0f + 1e-6f);
                strad = 0ull;
#pragma unroll
                for (int m = 0; m < NIMG; m++) {
                    const float sh = (float)(m - EMAX) * a.L;
                    const float l = lo + sh, h = hi + sh;
                    const bool in = fmaxf(fabsf(l), fabsf(h)) <= cin;
                    const bool out = l > cout || h < -cout;
                    strad |= (in || out) ? 0ull : 1ull << m;
                    off[m] = out ? 1e18f : sh;
                    const float gz = (l <= 0.0f && h >= 0.0f) ? 0.0f : fminf(fabsf(l), fabsf(h));
                    near |= !out && (g2xy + gz * gz <= bmax2);
                    if (!out) g2min = fminf(g2min, g2xy + gz * gz);
                }
                full = near || coarse_for_gap(dOx, dOy, dOz, mI1, mJ1, g2min, a.guard2);
            } else if (a.nearest) {
                // S1xR2 nearest image along z: J's centre moves to the image
                // nearest I's; tile pairs whose dz range stays inside +-L/2 need
                // no per-pair wrap and take the R^3 far path.
                shift_frame(dOz, eOz, a.L, a.L_lo);
                const float gz = axis_gap(dOz, mI1.z, mJ1.z);
                const float g2 = gx * gx + gy * gy + gz * gz;
                full = fabsf(dOz) + mI1.z + mJ1.z > a.halfL - a.wrap_tol || g2 <= bmax2 ||
                       coarse_for_gap(dOx, dOy, dOz, mI1, mJ1, g2, a.guard2);
            } else {
                const float hz = mI1.z + mJ1.z;
                const float lo = dOz - hz, hi = dOz + hz;
                const float g2xy = gx * gx + gy * gy;
                const float cin = a.cutL * (1.0f - 1e-6f), cout = a.cutL * (1.0f + 1e-6f);
                bool near = false, many = false;
                float g2min = 3.0e38f;
                mfirst = a.emax + 1;
                for (int m = -a.emax; m <= a.emax; m++) {
                    const float sh = (float)m * a.L;
                    const float l = lo + sh, h = hi + sh;
                    if (l > cout || h < -cout) continue;  // entirely outside the cut
                    if (mfirst > a.emax) mfirst = m;
                    mlast = m;
                    if (fmaxf(fabsf(l), fabsf(h)) > cin) {  // straddles the cut
                        if (m - mfirst < 64) stradl |= 1ull << (m - mfirst);
                        else many = true;
                    }
                    const float gz = (l <= 0.0f && h >= 0.0f) ? 0.0f : fminf(fabsf(l), fabsf(h));
                    near |= g2xy + gz * gz <= bmax2;
                    g2min = fminf(g2min, g2xy + gz * gz);
                }
                full = many || near || coarse_for_gap(dOx, dOy, dOz, mI1, mJ1, g2min, a.guard2);
            }

            // i in J's frame, rounded to FP32 for the far path.
            float px[IPT], py[IPT], pz[IPT], fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                px[k] = ((xi[k] - dOx) - eOx) + lx[k];
                py[k] = ((yi[k] - dOy) - eOy) + ly[k];
                pz[k] = ((zi[k] - dOz) - eOz) + lz[k];
                fx[k] = fy[k] = fz[k] = 0.0f;
            }
            const float4 *spb = sp[buf];
            const float *seb = se[buf];
            const uint32_t *sidb = sid[buf];
            const float4 *sresb = sres[buf];

            if (!full && KIND == K_S1_GEN && !a.nearest) {
                // explicit images, any count: a runtime loop over [mfirst, mlast]
#pragma unroll 2
                for (int jj = 0; jj < T; ++jj) {
                    const float4 q = spb[jj];
#pragma unroll
                    for (int k = 0; k < IPT; k++) {
                        const float dx = q.x - px[k], dy = q.y - py[k], dz = q.z - pz[k];
                        const float rho2 = fmaf(dx, dx, dy * dy);
                        float sw = 0.0f, swz = 0.0f, fm = (float)mfirst;
                        for (int m = mfirst; m <= mlast; m++, fm += 1.0f) {
                            const float sh = fm * a.L;
                            const float dzm = dz + sh;
                            const float ri = rsqrt_mufu(fmaf(dzm, dzm, rho2));
                            float ri3 = ri * ri * ri;
                            if (stradl >> (m - mfirst) & 1ull) {  // block-uniform
                                bool in = fabsf(dzm) <= a.cutL;
                                if (fabsf(fabsf(dzm) - a.cutL) < a.cut_tol) {
                                    float phz, plz;
                                    frame_split(zi[k], lz[k], dOz, eOz, phz, plz);
                                    in = cut_in_exact(q.z, sresb[jj].z, phz, plz, sh, a.cutL);
                                }
                                ri3 = in ? ri3 : 0.0f;
                            }
                            sw += ri3;
                            swz = fmaf(ri3, dzm, swz);
                        }
                        const float t = q.w * sw;
                        fx[k] = fmaf(t, dx, fx[k]);
                        fy[k] = fmaf(t, dy, fy[k]);
                        fz[k] = fmaf(q.w, swz, fz[k]);
                    }
                }
            } else if (!full) {
                if (KIND == K_R3 || KIND == K_S1_GEN) {  // K_S1_GEN here: nearest-image tile pairs
#pragma unroll 8
                    for (int jj = 0; jj < T; ++jj) {
                        const float4 q = spb[jj];
#pragma unroll
                        for (int k = 0; k < IPT; k++) {
                            const float dx = q.x - px[k], dy = q.y - py[k], dz = q.z - pz[k];
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            const float ri = rsqrt_mufu(r2);
                            const float w = (q.w * ri) * (ri * ri);
                            fx[k] = fmaf(w, dx, fx[k]);
                            fy[k] = fmaf(w, dy, fy[k]);
                            fz[k] = fmaf(w, dz, fz[k]);
                        }
                    }
                } else if (KIND == K_S1_IMG) {
                    if (strad == 0ull) {  // every image entirely in or out of the cut
#pragma unroll 2
                        for (int jj = 0; jj < T; ++jj) {
                            const float4 q = spb[jj];
#pragma unroll
                            for (int k = 0; k < IPT; k++) {
                                const float dx = q.x - px[k], dy = q.y - py[k], dz = q.z - pz[k];
                                const float rho2 = fmaf(dx, dx, dy * dy);
                                float sw = 0.0f, swz = 0.0f;
#pragma unroll
                                for (int m = 0; m < NIMG; m++) {
                                    const float dzm = dz + off[m];
                                    const float ri = rsqrt_mufu(fmaf(dzm, dzm, rho2));
                                    const float ri3 = ri * ri * ri;
                                    sw += ri3;
                                    swz = fmaf(ri3, dzm, swz);
                                }
                                const float t = q.w * sw;
                                fx[k] = fmaf(t, dx, fx[k]);
                                fy[k] = fmaf(t, dy, fy[k]);
                                fz[k] = fmaf(q.w, swz, fz[k]);
                            }
                        }
                    } else {  // some image straddles the cut: a per-pair test for those
                        for (int jj = 0; jj < T; ++jj) {
                            const float4 q = spb[jj];
#pragma unroll
                            for (int k = 0; k < IPT; k++) {
                                const float dx = q.x - px[k], dy = q.y - py[k], dz = q.z - pz[k];
                                const float rho2 = fmaf(dx, dx, dy * dy);
                                float sw = 0.0f, swz = 0.0f;
#pragma unroll
                                for (int m = 0; m < NIMG; m++) {
                                    const float dzm = dz + off[m];
                                    const float ri = rsqrt_mufu(fmaf(dzm, dzm, rho2));
                                    float ri3 = ri * ri * ri;
                                    if (strad & (1ull << m)) {  // block-uniform
                                        bool in = fabsf(dzm) <= a.cutL;
                                        if (fabsf(fabsf(dzm) - a.cutL) < a.cut_tol) {
                                            float phz, plz;
                                            frame_split(zi[k], lz[k], dOz, eOz, phz, plz);
                                            in = cut_in_exact(q.z, sresb[jj].z, phz, plz, off[m], a.cutL);
                                        }
                                        ri3 = in ? ri3 : 0.0f;
                                    }
                                    sw += ri3;
                                    swz = fmaf(ri3, dzm, swz);
                                }
                                const float t = q.w * sw;
                                fx[k] = fmaf(t, dx, fx[k]);
                                fy[k] = fmaf(t, dy, fy[k]);
                                fz[k] = fmaf(q.w, swz, fz[k]);
                            }
                        }
                    }
                }
            } else {
                // Full path: softening per pair (and per image with the cut test).
                // i in J's frame as a double-float ph + pl.
                float phx[IPT], phy[IPT], phz[IPT], plx[IPT], ply[IPT], plz[IPT];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    frame_split(xi[k], lx[k], dOx, eOx, phx[k], plx[k]);
                    frame_split(yi[k], ly[k], dOy, eOy, phy[k], ply[k]);
                    frame_split(zi[k], lz[k], dOz, eOz, phz[k], plz[k]);
                }
                // The self pair gets d = 0 exactly, as in the reference: after
                // the change of tile frame its FP32 separation is a rounding
                // residue, which the spline core would turn into a force.
                for (int jj = 0; jj < T; ++jj) {
                    const float4 q = spb[jj];
                    const float ej = seb[jj];
                    const uint32_t jid = sidb[jj];
                    const float4 ql = sresb[jj];
#pragma unroll
                    for (int k = 0; k < IPT; k++) {
                        const bool self = jid == ii[k];
                        // double-float separation: ~1e-7 of |d| whatever the tile size
                        const float dx = self ? 0.0f : (q.x - phx[k]) + (ql.x - plx[k]);
                        const float dy = self ? 0.0f : (q.y - phy[k]) + (ql.y - ply[k]);
                        float dz = self ? 0.0f : (q.z - phz[k]) + (ql.z - plz[k]);
                        const float b = ei[k] + ej;
                        const float b2 = b * b;
                        if (KIND == K_R3) {
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            const float ri = rsqrt_mufu(r2);
                            float w = ri * ri * ri;
                            if (r2 < b2) w = spline_inner_f32(r2, b);
                            w *= q.w;
                            fx[k] = fmaf(w, dx, fx[k]);
                            fy[k] = fmaf(w, dy, fy[k]);
                            fz[k] = fmaf(w, dz, fz[k]);
                        } else {
                            const float rho2 = fmaf(dx, dx, dy * dy);
                            int mlo = -a.emax, mhi = a.emax;
                            if (KIND == K_S1_GEN && a.nearest) {
                                if (!self)
                                    dz = nearest_image(dz, q.z, phz[k], ql.z, plz[k], a.L, a.halfL, a.halfL_lo,
                                                       a.wrap_tol);
                                mlo = mhi = 0;
                            }
                            float sw = 0.0f, swz = 0.0f;
                            for (int m = mlo; m <= mhi; m++) {
                                const float sh = (float)m * a.L;
                                const float dzm = dz + sh;
                                const float r2 = fmaf(dzm, dzm, rho2);
                                const float ri = rsqrt_mufu(r2);
                                float w = ri * ri * ri;
                                if (r2 < b2) w = spline_inner_f32(r2, b);
                                if (!a.nearest) {
                                    // |dz + mL| <= (e - 0.4) L (StePS/src/forces.cc:1274), a hard
                                    // cut: within a hair of it, decide on a TwoSum-exact dz.
                                    bool in = fabsf(dzm) <= a.cutL;
                                    if (!self && fabsf(fabsf(dzm) - a.cutL) < a.cut_tol)
                                        in = cut_in_exact(q.z, ql.z, phz[k], plz[k], sh, a.cutL);
                                    if (!in) w = 0.0f;
                                }
                                sw += w;
                                swz = fmaf(w, dzm, swz);
                            }
                            const float t = q.w * sw;
                            fx[k] = fmaf(t, dx, fx[k]);
                            fy[k] = fmaf(t, dy, fy[k]);
                            fz[k] = fmaf(q.w, swz, fz[k]);
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                ax[k] += (double)fx[k];
                ay[k] += (double)fy[k];
                az[k] += (double)fz[k];
            }
            __syncthreads();
        }

        double *o = a.part + (size_t)chunk * a.part_stride;
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            size_t q = (size_t)I * T + k * BLOCK + tid;
            o[3 * q] = ax[k];
            o[3 * q + 1] = ay[k];
            o[3 * q + 2] = az[k];
        }
    }
}

// Sum the chunk partials in chunk order, add the background term and scatter
// from curve order back to the caller's order F[3*(orig - id_min) + k].
__global__ void k_reduce_mixed(const double *__restrict__ part, int S, size_t stride, const uint32_t *__restrict__ perm,
                               int count, int id_min, const double *__restrict__ x, Background bg,
                               double *__restrict__ F)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    double f[3] = {0, 0, 0};
    for (int s = 0; s < S; s++)
        for (int k = 0; k < 3; k++) f[k] += part[(size_t)s * stride + 3 * (size_t)q + k];
    uint32_t o = perm[q];
    long long row = (long long)o - id_min;
    STEPS_CHECK_IDX(row, count, CK_OUTPUT);
    o = (uint32_t)(row + id_min);
    add_background(bg, x + 3 * (size_t)o, f);
    for (int k = 0; k < 3; k++) F[3 * (size_t)row + k] = f[k];
}

template <int KIND, int EMAX>
KernelFn pick(int threads, int ipt)
{
#define STEPS_SHAPE(B, P) \
    if (threads == B && ipt == P) return k_pair_mixed<KIND, B, P, EMAX>;
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(64, 4)
    STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(128, 4)
    STEPS_SHAPE(256, 1) STEPS_SHAPE(256, 2)
#undef STEPS_SHAPE
    return nullptr;
}

KernelFn select_kernel(const KParams &kp, int threads, int ipt)
{
    if (kp.topology == STEPS_R3) return pick<K_R3, 0>(threads, ipt);
    if (kp.topology == STEPS_S1R2 && kp.s1r2_images && kp.is_periodic >= 2) {
        switch (kp.emax) {
        case 3: return pick<K_S1_IMG, 3>(threads, ipt);
        case 4: return pick<K_S1_IMG, 4>(threads, ipt);
        case 5: return pick<K_S1_IMG, 5>(threads, ipt);
        case 16: return pick<K_S1_IMG, 16>(threads, ipt);  // IS_PERIODIC = 15, the cylindrical example
        default: return pick<K_S1_GEN, 0>(threads, ipt);
        }
    }
    if (kp.topology == STEPS_S1R2 && kp.is_periodic < 2) return pick<K_S1_GEN, 0>(threads, ipt);
    return nullptr;
}

}  // namespace

bool shape_supported(int threads, int ipt)
{
    KParams kp{};
    kp.topology = STEPS_R3;
    return select_kernel(kp, threads, ipt) != nullptr;
}

bool shape_supported_for(const KParams &kp, int threads, int ipt)
{
    size_t dyn;
    if (kp.topology == STEPS_T3) return t3_kernel(kp, threads, ipt, &dyn) != nullptr;
    if (kp.topology == STEPS_S1R2 && kp.is_periodic >= 2 && !kp.s1r2_images)
        return s1tab_kernel(kp, threads, ipt) != nullptr;
    return select_kernel(kp, threads, ipt) != nullptr;
}

bool mixed_supported(const KParams &kp) { return select_kernel(kp, 128, 2) != nullptr; }

void forces_mixed(const KParams &kp, const Tables &tb, const double *x, const double *m64, const double *eps64,
                  int n, int id_min, int ni, double *F, bool reuse_order)
{
    Ctx &c = ctx();
    cudaStream_t st = c.stream;
    const int threads = c.shape.threads, ipt = c.shape.ipt;
    const int T = threads * ipt;
    size_t dyn = 0;
    const bool s1tab = kp.topology == STEPS_S1R2 && kp.is_periodic >= 2 && !kp.s1r2_images;
    const bool packed = kp.topology == STEPS_R3 && c.shape.variant >= 1;
    // T^3 reads the variant as 0 (one i per lane) or 1 (quad lanes); the R^3
    // pair loops 2-4 have no T^3 counterpart and mean 0 there.
    KernelFn fn = kp.topology == STEPS_T3 ? t3_kernel(kp, threads, ipt, &dyn, c.shape.variant == 1 ? 1 : 0)
                  : s1tab              ? s1tab_kernel(kp, threads, ipt)
                  : packed             ? (c.shape.variant == 4 ? r3x2_pipe_kernel(threads, ipt)
                                                               : r3x2_kernel(threads, ipt, false, r3x2_occ(c.shape.variant)))
                                       : select_kernel(kp, threads, ipt);
    if (!fn) fail(STEPS_E_ARG, "mixed precision: unsupported topology/mode or kernel shape");

    unsigned long long *bb = c.bbox.ensure<unsigned long long>(8);
    STEPS_CUDA(cudaEventRecord(c.phase[0], st));
    build_tiles(c.tj, x, m64, eps64, 0, n, T, reuse_order, st, bb, PAD_J);
    const bool full_i = id_min == 0 && ni == n;
    TileSet &ti = full_i ? c.tj : c.ti;
    if (!full_i)
        build_tiles(c.ti, x, m64, eps64, id_min, ni, T, reuse_order, st, bb, PAD_I);
    STEPS_CUDA(cudaEventRecord(c.phase[1], st));

    // Work decomposition: items = i tiles x j chunks, sized so the persistent
    // grid sees several waves with a small last-wave remainder.
    if (dyn > 0) STEPS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int occ = 0;
    STEPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, dyn));
    if (occ < 1) occ = 1;
    const int resident = c.nsm * occ;
    const int nit = ti.ntiles, njt = c.tj.ntiles;
    int S = c.shape.jsplit;
    // The FP64 chunk partials (S x N_i x 24 B) stay within 4 GiB.
    const long long smax = std::max(1LL, (4LL << 30) / ((long long)nit * T * 24));
    if (S <= 0) {
        // Items of at most 64 and at least 4 j tiles, aiming at 16 or more
        // waves of items over the persistent grid: long items balance badly
        // (near-field tile pairs make their lengths uneven), very short ones
        // pay the per-item set-up.
        const long long pairs = (long long)nit * njt;
        const long long tpc = std::min(64LL, std::max(4LL, pairs / (16LL * resident)));
        S = (int)std::min<long long>(smax, (njt + tpc - 1) / tpc);
        if (S < 1) S = 1;
    }
    if (S > njt) S = njt;
    if (S > smax) S = (int)smax;
    const int tpc = div_up(njt, S);
    S = div_up(njt, tpc);

    MixedArgs a;
    a.jpack = c.tj.pack.as<float4>();
    a.jeps = c.tj.eps.as<float>();
    a.jmeta = c.tj.meta.as<float4>();
    a.jidx = c.tj.idx.as<uint32_t>();
    a.jres = c.tj.resid.as<float4>();
    a.jsoa = c.tj.soa.as<float>();
    a.jsub = c.tj.sub.as<float4>();
    a.njt = njt;
    a.ipack = ti.pack.as<float4>();
    a.ieps = ti.eps.as<float>();
    a.imeta = ti.meta.as<float4>();
    a.iidx = ti.idx.as<uint32_t>();
    a.ilo = ti.resid.as<float4>();
    a.nit = nit;
    a.S = S;
    a.tpc = tpc;
    a.nitems = nit * S;
    a.istride = 1;
    // The autotuner times a strided sample of the real i tiles (dense tiles,
    // the same j split): tune_sample waves of items.
    const bool sample = c.tune_sample > 0;
    c.tune_sampled = false;
    if (sample) {
        const long long want = (long long)c.tune_sample * resident;
        if (want < (long long)a.nitems) {
            const int tiles = (int)((want + S - 1) / S);
            a.istride = std::max(1, nit / tiles);
            a.nitems = (int)want;  // the last sampled tile may run only some of its chunks
            c.tune_sampled = true;
        }
    }
    a.counter = c.counter.ensure<unsigned>(4);
    a.items = nullptr;
    a.part_stride = (size_t)nit * T * 3;
    a.part = c.partial.ensure<double>((size_t)S * a.part_stride);
    a.L = (float)kp.L;
    a.halfL = (float)kp.halfL;
    a.cutL = (float)kp.cutL;
    a.cut_tol = (float)(kp.cutL * 1e-5);
    a.L_lo = (float)(kp.L - (double)a.L);
    a.halfL_lo = (float)(kp.halfL - (double)a.halfL);
    a.wrap_tol = (float)(kp.halfL * 1e-5);
    a.guard2 = c.shape.guard * c.shape.guard;
    a.emax = kp.emax;
    a.nearest = kp.topology == STEPS_S1R2 && kp.is_periodic < 2;
    a.t3f = nullptr;
    a.ng = 0;
    a.ih = a.u0 = 0.0f;
    a.wcap = 0;
    a.halo = a.ext = 0;
    a.t3r = nullptr;
    a.t3rz = nullptr;
    a.s1tab = nullptr;
    a.s1rec = nullptr;
    a.nrho = a.nz = 0;
    a.irho = a.iz = a.rho_max = 0.0f;
    if (kp.topology == STEPS_T3) t3_args(a, kp, tb, st);
    if (s1tab) s1tab_args(a, kp, tb, st);

    a.status = kernel_status_word();
    a.stall_seq = c.stall_seq;
    c.stall_seq = -1;
    STEPS_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st));
    const bool bounded_waits = packed && c.shape.variant == 4;
    if (bounded_waits) STEPS_CUDA(cudaMemsetAsync(a.status, 0, sizeof(int), st));
    int grid = resident < a.nitems ? resident : a.nitems;
    fn<<<grid, threads, dyn, st>>>(a);
    note_launch("k_pair_mixed");
    if (bounded_waits) {
        // A kernel whose bounded waits gave up has left and written its status.
        if (!c.kstatus_host) STEPS_CUDA(cudaMallocHost(&c.kstatus_host, sizeof(int)));
        STEPS_CUDA(cudaMemcpyAsync(c.kstatus_host, a.status, sizeof(int), cudaMemcpyDeviceToHost, st));
        STEPS_CUDA(cudaStreamSynchronize(st));
        if (*c.kstatus_host != 0) fail(STEPS_E_TIMEOUT, "pair kernel: a pipeline wait timed out (status written by the kernel)");
    }
    STEPS_CUDA(cudaEventRecord(c.phase[2], st));
    if (!sample) {
        k_reduce_mixed<<<div_up(ni, 256), 256, 0, st>>>(a.part, S, a.part_stride, ti.perm(), ni, id_min, x,
                                                       background_of(kp, tb), F);
        note_launch("k_reduce_mixed");
    }
    STEPS_CUDA(cudaEventRecord(c.phase[3], st));
    c.phase_valid = true;
    c.last_pairs = c.tune_sampled ? (double)a.nitems * T * ((double)tpc * T) : (double)ni * (double)n;
    c.last_S = S;
    c.last_waves = (double)nit * S / resident;
}

}  // namespace steps
