// Mixed-precision T^3 kernel: nearest-image softened direct sum plus the
// Ewald correction -m_j D(d) interpolated from the FP64-built table
// (StePS/src/forces.cc:776-876, interpolation StePS/src/ewald_space.cc:452-523).
//
// Same tiling as pair_mixed.cu (FP32 tile-relative pairs, FP64 accumulation).
// Per tile pair the block
//   * moves J's centre to the image nearest I's (d_O - L rint(d_O / L)) and
//     flags the axes along which the pair box crosses +-L/2: only there is
//     the nearest-image wrap applied per pair (StePS/src/forces.cc:812-817);
//   * stages the part of the correction table that the pair box can reach
//     into shared memory as FP32 float4 cells (a "window", cell-centred grid
//     over [-L/2, L/2], indices taken modulo ngrid); the per-pair
//     interpolation then reads shared memory only. A window larger than the
//     staging area falls back to reading the FP32 table copy from L2.
// The table lookup uses the unwrapped separation: the table is periodic in
// its index, so it is the lookup the reference does at the wrapped one.
#include "common.cuh"
#include "context.cuh"
#include "mixed.cuh"

namespace steps {

namespace {

using namespace mixed;

__device__ __forceinline__ int pmod(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

template <int ORDER>
__device__ __forceinline__ void weights(float t, float *w)
{
    if (ORDER == 4) {  // Catmull-Rom, StePS/src/ewald_space.cc:440-449
        const float t2 = t * t, t3 = t2 * t;
        w[0] = -0.5f * t3 + t2 - 0.5f * t;
        w[1] = 1.5f * t3 - 2.5f * t2 + 1.0f;
        w[2] = -1.5f * t3 + 2.0f * t2 + 0.5f * t;
        w[3] = 0.5f * t3 - 0.5f * t2;
    } else {  // 2-point Lagrange (trilinear)
        w[0] = 1.0f - t;
        w[1] = t;
    }
}

// ORDER 0: IS_PERIODIC == 1, nearest image only (no table).
template <int BLOCK, int IPT, int ORDER>
__global__ void __launch_bounds__(BLOCK) k_pair_t3(MixedArgs a)
{
    constexpr int T = BLOCK * IPT;
    constexpr int NT = ORDER == 0 ? 1 : ORDER;  // stencil width
    constexpr int OFF = ORDER == 4 ? 1 : 0;     // stencil starts OFF cells left of floor(u)
    __shared__ __align__(16) float4 sp[2][T];
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ int s_item;
    extern __shared__ float4 win[];
    const int tid = threadIdx.x;
    const float L = a.L, halfL = a.halfL;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.nitems) return;
        const int I = item / a.S;
        const int chunk = item - I * a.S;
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

        if (J0 < J1) stage_tile<BLOCK, IPT>(a, J0, sp[0], se[0], sid[0]);
        for (int J = J0; J < J1; ++J) {
            const int buf = (J - J0) & 1;
            const float4 mJ0 = __ldg(a.jmeta + 2 * J);
            const float4 mJ1 = __ldg(a.jmeta + 2 * J + 1);
            float eO[3];
            float dO[3] = {two_diff(mJ0.x, mI0.x, eO[0]), two_diff(mJ0.y, mI0.y, eO[1]),
                           two_diff(mJ0.z, mI0.z, eO[2])};
            const float hs[3] = {mI1.x + mJ1.x, mI1.y + mJ1.y, mI1.z + mJ1.z};
            bool wrap[3];
            float g2 = 0.0f;
            int w0[3], wn[3];
            float uc[3];
#pragma unroll
            for (int ax3 = 0; ax3 < 3; ax3++) {
                dO[ax3] -= L * rintf(dO[ax3] / L);  // nearest image of J's centre
                wrap[ax3] = fabsf(dO[ax3]) + hs[ax3] > halfL;
                const float g = fmaxf(fabsf(dO[ax3]) - hs[ax3], 0.0f);
                g2 += g * g;
                if (ORDER != 0) {
                    const float ulo = (dO[ax3] - hs[ax3]) * a.ih + a.u0;
                    const float uhi = (dO[ax3] + hs[ax3]) * a.ih + a.u0;
                    w0[ax3] = (int)floorf(ulo - 1e-3f) - OFF;
                    wn[ax3] = (int)floorf(uhi + 1e-3f) - OFF + NT - w0[ax3];
                    uc[ax3] = a.u0 - (float)w0[ax3];  // window-local continuous index offset
                }
            }
            // Pairs closer than some beta = eps_i + eps_j need the spline; a
            // wrapped axis makes the box gap meaningless, so take the full path.
            const float bmax = mI0.w + mJ0.w;
            const bool full = g2 <= bmax * bmax * 1.0001f + 1e-30f || wrap[0] || wrap[1] || wrap[2];
            const int ncell = ORDER != 0 ? wn[0] * wn[1] * wn[2] : 0;
            const bool use_win = ORDER != 0 && ncell <= a.wcap;

            if (J + 1 < J1) {
                stage_tile<BLOCK, IPT>(a, J + 1, sp[buf ^ 1], se[buf ^ 1], sid[buf ^ 1]);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            if (use_win) {
                for (int cidx = tid; cidx < ncell; cidx += BLOCK) {
                    const int cz = cidx % wn[2];
                    const int cy = (cidx / wn[2]) % wn[1];
                    const int cx = cidx / (wn[2] * wn[1]);
                    const int gx = pmod(w0[0] + cx, a.ng), gy = pmod(w0[1] + cy, a.ng), gz = pmod(w0[2] + cz, a.ng);
                    win[cidx] = __ldg(a.t3f + ((size_t)gx * a.ng + gy) * a.ng + gz);
                }
            }
            __syncthreads();

            float px[IPT], py[IPT], pz[IPT], fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                px[k] = ((xi[k] - dO[0]) - eO[0]) + lx[k];
                py[k] = ((yi[k] - dO[1]) - eO[1]) + ly[k];
                pz[k] = ((zi[k] - dO[2]) - eO[2]) + lz[k];
                fx[k] = fy[k] = fz[k] = 0.0f;
            }
            const float4 *spb = sp[buf];
            const float *seb = se[buf];
            const uint32_t *sidb = sid[buf];
            const int sy = ORDER != 0 ? wn[2] : 0, sx = ORDER != 0 ? wn[1] * wn[2] : 0;

#pragma unroll 2
            for (int jj = 0; jj < T; ++jj) {
                const float4 q = spb[jj];
                const float ej = seb[jj];
                const uint32_t jid = sidb[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const bool self = full && jid == ii[k];
                    const float dx = self ? 0.0f : q.x - px[k];
                    const float dy = self ? 0.0f : q.y - py[k];
                    const float dz = self ? 0.0f : q.z - pz[k];
                    float nx = dx, ny = dy, nz = dz;
                    if (wrap[0]) nx = fabsf(nx) > halfL ? nx - copysignf(L, nx) : nx;
                    if (wrap[1]) ny = fabsf(ny) > halfL ? ny - copysignf(L, ny) : ny;
                    if (wrap[2]) nz = fabsf(nz) > halfL ? nz - copysignf(L, nz) : nz;
                    const float r2 = fmaf(nx, nx, fmaf(ny, ny, nz * nz));
                    const float ri = rsqrt_mufu(r2);
                    float w = ri * ri * ri;
                    if (full) {
                        const float b = ei[k] + ej;
                        if (r2 < b * b) w = spline_inner_f32(r2, b);
                    }
                    float Dx = 0.0f, Dy = 0.0f, Dz = 0.0f;
                    if (ORDER != 0) {
                        float wx[4], wy[4], wz[4];
                        int bx, by, bz;
                        if (use_win) {
                            const float ux = fmaf(dx, a.ih, uc[0]), uy = fmaf(dy, a.ih, uc[1]),
                                        uz = fmaf(dz, a.ih, uc[2]);
                            const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
                            weights<ORDER>(ux - fxl, wx);
                            weights<ORDER>(uy - fyl, wy);
                            weights<ORDER>(uz - fzl, wz);
                            bx = (int)fxl - OFF;
                            by = (int)fyl - OFF;
                            bz = (int)fzl - OFF;
                            const float4 *base = win + (bx * sx + by * sy + bz);
#pragma unroll
                            for (int aa = 0; aa < NT; aa++)
#pragma unroll
                                for (int bb = 0; bb < NT; bb++) {
                                    const float wxy = wx[aa] * wy[bb];
#pragma unroll
                                    for (int cc = 0; cc < NT; cc++) {
                                        const float4 v = base[aa * sx + bb * sy + cc];
                                        const float ww = wxy * wz[cc];
                                        Dx = fmaf(ww, v.x, Dx);
                                        Dy = fmaf(ww, v.y, Dy);
                                        Dz = fmaf(ww, v.z, Dz);
                                    }
                                }
                        } else {
                            const float ux = fmaf(dx, a.ih, a.u0), uy = fmaf(dy, a.ih, a.u0),
                                        uz = fmaf(dz, a.ih, a.u0);
                            const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
                            weights<ORDER>(ux - fxl, wx);
                            weights<ORDER>(uy - fyl, wy);
                            weights<ORDER>(uz - fzl, wz);
                            bx = (int)fxl - OFF;
                            by = (int)fyl - OFF;
                            bz = (int)fzl - OFF;
                            for (int aa = 0; aa < NT; aa++) {
                                const int gx = pmod(bx + aa, a.ng);
                                for (int bb = 0; bb < NT; bb++) {
                                    const int gy = pmod(by + bb, a.ng);
                                    const float wxy = wx[aa] * wy[bb];
                                    for (int cc = 0; cc < NT; cc++) {
                                        const int gz = pmod(bz + cc, a.ng);
                                        const float4 v = __ldg(a.t3f + ((size_t)gx * a.ng + gy) * a.ng + gz);
                                        const float ww = wxy * wz[cc];
                                        Dx = fmaf(ww, v.x, Dx);
                                        Dy = fmaf(ww, v.y, Dy);
                                        Dz = fmaf(ww, v.z, Dz);
                                    }
                                }
                            }
                        }
                    }
                    fx[k] = fmaf(q.w, fmaf(w, nx, -Dx), fx[k]);
                    fy[k] = fmaf(q.w, fmaf(w, ny, -Dy), fy[k]);
                    fz[k] = fmaf(q.w, fmaf(w, nz, -Dz), fz[k]);
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

__global__ void k_table_f32(const double *__restrict__ t, size_t ncell, float4 *__restrict__ out)
{
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncell) out[c] = make_float4((float)t[3 * c], (float)t[3 * c + 1], (float)t[3 * c + 2], 0.0f);
}

template <int ORDER>
KernelFn pick_t3(int threads, int ipt)
{
#define STEPS_SHAPE(B, P) \
    if (threads == B && ipt == P) return k_pair_t3<B, P, ORDER>;
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(256, 1)
#undef STEPS_SHAPE
    return nullptr;
}

}  // namespace

// Window capacity (cells) of the T^3 kernels' shared-memory table staging.
constexpr int T3_WINDOW_CELLS = 2048;

KernelFn t3_kernel(const KParams &kp, int threads, int ipt, size_t *dyn_smem)
{
    *dyn_smem = 0;
    if (kp.is_periodic < 2) return pick_t3<0>(threads, ipt);
    *dyn_smem = T3_WINDOW_CELLS * sizeof(float4);
    return kp.order == 4 ? pick_t3<4>(threads, ipt) : pick_t3<2>(threads, ipt);
}

// FP32 float4 copy of the FP64 table, rebuilt whenever the table changes.
const float4 *t3_table_f32(const Tables &tb, cudaStream_t st)
{
    Ctx &c = ctx();
    size_t ncell = (size_t)tb.t3_ng * tb.t3_ng * tb.t3_ng;
    if (c.t3f_version != c.t3_version || !c.t3f.p) {
        float4 *o = c.t3f.ensure<float4>(ncell);
        k_table_f32<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.t3, ncell, o);
        note_launch("k_table_f32");
        c.t3f_version = c.t3_version;
    }
    return c.t3f.as<float4>();
}

void t3_args(MixedArgs &a, const KParams &kp, const Tables &tb, cudaStream_t st)
{
    a.t3f = nullptr;
    a.ng = tb.t3_ng;
    a.ih = 0.0f;
    a.u0 = 0.0f;
    a.wcap = T3_WINDOW_CELLS;
    if (kp.is_periodic >= 2) {
        a.t3f = t3_table_f32(tb, st);
        a.ih = (float)((double)tb.t3_ng / kp.L);
        a.u0 = (float)((double)tb.t3_ng * 0.5 - 0.5);
    }
}

}  // namespace steps
