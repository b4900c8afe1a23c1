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

// i mod n for i in [-2n, 3n), without a division; any other i (positions
// outside the box, NaN) is clamped into [0, n) so the read stays in the table.
__device__ __forceinline__ int wrap_index(int i, int n)
{
    i += i < 0 ? n : 0;
    i += i < 0 ? n : 0;
    i -= i >= n ? n : 0;
    i -= i >= n ? n : 0;
    return min(max(i, 0), n - 1);
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

// T^3 stencil records, one float4 per component, in two arrays of the same
// cell index: the x and y components as one 32-byte record (a.t3r, read with
// one 256-bit load) and the z component as one 16-byte record (a.t3rz): two
// L1 requests per record instead of three, in the same 48 bytes per cell.
// (Records padded to 64 bytes for the same purpose were 13-17 % slower: the
// larger table loses L1 hits.)

// Two float4 of a 32-byte aligned record in one 256-bit load (sm_100+):
// the L1 data path, which bounds the table kernels, sees one request per
// record instead of two. The S1xR2 CIC and TSC records are 32 bytes: CIC
// 2.71e11 -> 3.53e11 and TSC 1.06e11 -> 1.31e11 pairs/s at N = 2^20.
__device__ __forceinline__ void ldg_v8(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// w . v for the 4 z taps of a z-row record.
__device__ __forceinline__ float dot4(const float *w, float4 v)
{
    return fmaf(w[3], v.w, fmaf(w[2], v.z, fmaf(w[1], v.y, w[0] * v.x)));
}

// Sum of the NT^3 stencil taps fetch(a, b, c) weighted by wx[a] wy[b] wz[c].
// Trilinear: 8 products of the three weights (36 FP ops). Tricubic: nested,
// sum_a wx_a sum_b wy_b sum_c wz_c T_abc (252 FP ops instead of 272).
template <int ORDER, class Fetch>
__device__ __forceinline__ void stencil(const float *wx, const float *wy, const float *wz, Fetch fetch, float &Dx,
                                        float &Dy, float &Dz)
{
    constexpr int NT = ORDER;
    if constexpr (ORDER == 4) {
#pragma unroll
        for (int aa = 0; aa < NT; aa++) {
            float rx = 0.0f, ry = 0.0f, rz = 0.0f;
#pragma unroll
            for (int bb = 0; bb < NT; bb++) {
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
                for (int cc = 0; cc < NT; cc++) {
                    const float4 v = fetch(aa, bb, cc);
                    sx = fmaf(wz[cc], v.x, sx);
                    sy = fmaf(wz[cc], v.y, sy);
                    sz = fmaf(wz[cc], v.z, sz);
                }
                rx = fmaf(wy[bb], sx, rx);
                ry = fmaf(wy[bb], sy, ry);
                rz = fmaf(wy[bb], sz, rz);
            }
            Dx = fmaf(wx[aa], rx, Dx);
            Dy = fmaf(wx[aa], ry, Dy);
            Dz = fmaf(wx[aa], rz, Dz);
        }
    } else {
#pragma unroll
        for (int aa = 0; aa < NT; aa++)
#pragma unroll
            for (int bb = 0; bb < NT; bb++) {
                const float wxy = wx[aa] * wy[bb];
#pragma unroll
                for (int cc = 0; cc < NT; cc++) {
                    const float4 v = fetch(aa, bb, cc);
                    const float ww = wxy * wz[cc];
                    Dx = fmaf(ww, v.x, Dx);
                    Dy = fmaf(ww, v.y, Dy);
                    Dz = fmaf(ww, v.z, Dz);
                }
            }
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
    __shared__ __align__(16) float4 sres[2][T];
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

        if (J0 < J1) stage_tile<BLOCK, IPT>(a, J0, sp[0], se[0], sid[0], sres[0]);
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
                shift_frame(dO[ax3], eO[ax3], L, a.L_lo);  // nearest image of J's centre
                wrap[ax3] = fabsf(dO[ax3]) + hs[ax3] > halfL - a.wrap_tol;  // conservative by wrap_tol
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
            const bool full = g2 <= bmax * bmax * 1.0001f + 1e-30f || wrap[0] || wrap[1] || wrap[2] ||
                              coarse_for_gap(dO[0], dO[1], dO[2], mI1, mJ1, g2, a.guard2);
            // Window strides are odd so that neighbouring cells fall in
            // different shared-memory banks; cells past wn[] are padding.
            // Non-finite or out-of-box input can make wn[] anything: the
            // window is used only when every extent is in [NT, wcap].
            bool use_win = ORDER != 0;
#pragma unroll
            for (int ax3 = 0; ax3 < 3; ax3++) use_win = use_win && wn[ax3] >= NT && wn[ax3] <= a.wcap;
            const int sy = use_win ? (wn[2] | 1) : 0;
            const int sx = use_win ? ((wn[1] * sy) | 1) : 0;
            use_win = use_win && (long long)wn[0] * sx <= (long long)a.wcap;
            const int ncell = use_win ? wn[0] * sx : 0;
            // Otherwise the stencils of this tile pair lie inside the table's
            // periodic halo (no per-pair wrap), or take the wrapped lookup.
            bool halo = ORDER != 0 && !use_win;
#pragma unroll
            for (int ax3 = 0; ax3 < 3; ax3++)
                halo = halo && w0[ax3] >= -a.halo && w0[ax3] + wn[ax3] <= a.ng + a.halo;

            if (J + 1 < J1) {
                stage_tile<BLOCK, IPT>(a, J + 1, sp[buf ^ 1], se[buf ^ 1], sid[buf ^ 1], sres[buf ^ 1]);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            if (use_win) {
                for (int cidx = tid; cidx < ncell; cidx += BLOCK) {
                    const int cx = cidx / sx;
                    const int rem = cidx - cx * sx;
                    const int cy = rem / sy;
                    const int cz = rem - cy * sy;
                    const int gx = pmod(w0[0] + cx, a.ng), gy = pmod(w0[1] + cy, a.ng), gz = pmod(w0[2] + cz, a.ng);
                    long long cell = ((long long)(gx + a.halo) * a.ext + gy + a.halo) * a.ext + gz + a.halo;
                    STEPS_CHECK_IDX(cell, (long long)a.ext * a.ext * a.ext, CK_T3_CELL);
                    win[cidx] = __ldg(a.t3f + cell);
                }
            }
            __syncthreads();

            float phx[IPT], phy[IPT], phz[IPT], plx[IPT], ply[IPT], plz[IPT];
            float px[IPT], py[IPT], pz[IPT], fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                frame_split(xi[k], lx[k], dO[0], eO[0], phx[k], plx[k]);
                frame_split(yi[k], ly[k], dO[1], eO[1], phy[k], ply[k]);
                frame_split(zi[k], lz[k], dO[2], eO[2], phz[k], plz[k]);
                px[k] = phx[k] + plx[k];
                py[k] = phy[k] + ply[k];
                pz[k] = phz[k] + plz[k];
                fx[k] = fy[k] = fz[k] = 0.0f;
            }
            const float4 *spb = sp[buf];
            const float *seb = se[buf];
            const uint32_t *sidb = sid[buf];
            const float4 *sresb = sres[buf];

#pragma unroll 2
            for (int jj = 0; jj < T; ++jj) {
                const float4 q = spb[jj];
                const float ej = seb[jj];
                const uint32_t jid = sidb[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const bool self = full && jid == ii[k];
                    float dx, dy, dz;
                    if (full) {  // double-float separation
                        const float4 ql = sresb[jj];
                        dx = self ? 0.0f : (q.x - phx[k]) + (ql.x - plx[k]);
                        dy = self ? 0.0f : (q.y - phy[k]) + (ql.y - ply[k]);
                        dz = self ? 0.0f : (q.z - phz[k]) + (ql.z - plz[k]);
                    } else {
                        dx = q.x - px[k];
                        dy = q.y - py[k];
                        dz = q.z - pz[k];
                    }
                    float nx = dx, ny = dy, nz = dz;
                    if (full && !self) {  // wrapped axes are full-path tile pairs
                        const float4 ql = sresb[jj];
                        if (wrap[0]) nx = nearest_image(dx, q.x, phx[k], ql.x, plx[k], L, halfL, a.halfL_lo, a.wrap_tol);
                        if (wrap[1]) ny = nearest_image(dy, q.y, phy[k], ql.y, ply[k], L, halfL, a.halfL_lo, a.wrap_tol);
                        if (wrap[2]) nz = nearest_image(dz, q.z, phz[k], ql.z, plz[k], L, halfL, a.halfL_lo, a.wrap_tol);
                    }
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
                        if (use_win) {  // shared-memory window, window-local cell index
                            const float ux = fmaf(dx, a.ih, uc[0]), uy = fmaf(dy, a.ih, uc[1]),
                                        uz = fmaf(dz, a.ih, uc[2]);
                            const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
                            weights<ORDER>(ux - fxl, wx);
                            weights<ORDER>(uy - fyl, wy);
                            weights<ORDER>(uz - fzl, wz);
                            // The window covers every stencil of the tile pair; the
                            // clamps only keep non-finite input inside it.
                            bx = min(max((int)fxl - OFF, 0), wn[0] - NT);
                            by = min(max((int)fyl - OFF, 0), wn[1] - NT);
                            bz = min(max((int)fzl - OFF, 0), wn[2] - NT);
#ifdef STEPS_CHECK
                            const long long wfirst = bx * sx + by * sy + bz;
                            if (!check_span(wfirst, wfirst + (NT - 1) * (sx + sy + 1), ncell, CK_T3_CELL))
                                bx = by = bz = 0;
#endif
                            const float4 *base = win + (bx * sx + by * sy + bz);
                            stencil<ORDER>(wx, wy, wz, [&](int aa, int bb, int cc) { return base[aa * sx + bb * sy + cc]; },
                                           Dx, Dy, Dz);
                        } else if (halo) {  // haloed table in L1/L2, no wrap
                            const float uh = a.u0 + (float)a.halo;
                            const float ux = fmaf(dx, a.ih, uh), uy = fmaf(dy, a.ih, uh), uz = fmaf(dz, a.ih, uh);
                            const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
                            weights<ORDER>(ux - fxl, wx);
                            weights<ORDER>(uy - fyl, wy);
                            weights<ORDER>(uz - fzl, wz);
                            const int E = a.ext;
                            bx = min(max((int)fxl - OFF, 0), E - NT);
                            by = min(max((int)fyl - OFF, 0), E - NT);
                            bz = min(max((int)fzl - OFF, 0), E - NT);
#ifdef STEPS_CHECK
                            const long long hfirst = ((long long)bx * E + by) * E + bz;
                            if (!check_span(hfirst, hfirst + (long long)(NT - 1) * ((long long)E * E + E + 1),
                                            (long long)E * E * E, CK_T3_CELL))
                                bx = by = bz = 0;
#endif
                            if (ORDER == 4) {
                                // z-row records: the 4 z taps of one (x, y) row, per
                                // component, in 3 float4 (48 B), 16 rows per pair
                                const int cb = (bx * E + by) * E + bz;
#pragma unroll
                                for (int aa = 0; aa < 4; aa++) {
                                    float rx = 0.0f, ry = 0.0f, rz = 0.0f;
#pragma unroll
                                    for (int bb = 0; bb < 4; bb++) {
                                        const int cr = cb + (aa * E + bb) * E;
                                        float4 vx, vy;
                                        ldg_v8(a.t3r + 2 * (size_t)cr, vx, vy);
                                        const float4 vz = __ldg(a.t3rz + cr);
                                        rx = fmaf(wy[bb], dot4(wz, vx), rx);
                                        ry = fmaf(wy[bb], dot4(wz, vy), ry);
                                        rz = fmaf(wy[bb], dot4(wz, vz), rz);
                                    }
                                    Dx = fmaf(wx[aa], rx, Dx);
                                    Dy = fmaf(wx[aa], ry, Dy);
                                    Dz = fmaf(wx[aa], rz, Dz);
                                }
                            } else {
                                // (y, z) quad records: cells (x, y..y+1, z..z+1), per
                                // component, in 3 float4 (48 B), 2 records per pair
                                const float q00 = wy[0] * wz[0], q01 = wy[0] * wz[1], q10 = wy[1] * wz[0],
                                            q11 = wy[1] * wz[1];
                                const int cb = (bx * E + by) * E + bz;
#pragma unroll
                                for (int aa = 0; aa < 2; aa++) {
                                    const int cr = cb + aa * E * E;
                                    float4 vx, vy;
                                    ldg_v8(a.t3r + 2 * (size_t)cr, vx, vy);
                                    const float4 vz = __ldg(a.t3rz + cr);
                                    Dx = fmaf(wx[aa], fmaf(q11, vx.w, fmaf(q10, vx.z, fmaf(q01, vx.y, q00 * vx.x))), Dx);
                                    Dy = fmaf(wx[aa], fmaf(q11, vy.w, fmaf(q10, vy.z, fmaf(q01, vy.y, q00 * vy.x))), Dy);
                                    Dz = fmaf(wx[aa], fmaf(q11, vz.w, fmaf(q10, vz.z, fmaf(q01, vz.y, q00 * vz.x))), Dz);
                                }
                            }
                        } else {  // wrapped lookup (tile pairs wider than the halo)
                            const float ux = fmaf(dx, a.ih, a.u0), uy = fmaf(dy, a.ih, a.u0),
                                        uz = fmaf(dz, a.ih, a.u0);
                            const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
                            weights<ORDER>(ux - fxl, wx);
                            weights<ORDER>(uy - fyl, wy);
                            weights<ORDER>(uz - fzl, wz);
                            bx = (int)fxl - OFF;
                            by = (int)fyl - OFF;
                            bz = (int)fzl - OFF;
                            // Stencil indices wrapped once per axis: |d| < 3L/2,
                            // so every index lies in [-2 ng, 3 ng).
                            int gx[NT], gy[NT], gz[NT];
#pragma unroll
                            for (int t = 0; t < NT; t++) {
                                gx[t] = wrap_index(bx + t, a.ng) + a.halo;
                                gy[t] = wrap_index(by + t, a.ng) + a.halo;
                                gz[t] = wrap_index(bz + t, a.ng) + a.halo;
                                STEPS_CHECK_IDX(gx[t], a.ext, CK_T3_CELL);
                                STEPS_CHECK_IDX(gy[t], a.ext, CK_T3_CELL);
                                STEPS_CHECK_IDX(gz[t], a.ext, CK_T3_CELL);
                            }
                            stencil<ORDER>(wx, wy, wz,
                                           [&](int aa, int bb, int cc) {
                                               return __ldg(a.t3f + (gx[aa] * a.ext + gy[bb]) * a.ext + gz[cc]);
                                           },
                                           Dx, Dy, Dz);
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

// Cell index of a nearest-image z in [-L/2, L/2]: floor(uz) lies in [-1, nz]
// up to rounding, so one conditional shift wraps it; anything else
// (non-finite input) is clamped into [0, nz).
__device__ __forceinline__ int wrap_near(float f, int nz)
{
    int i = (int)f;
    i += i < 0 ? nz : 0;
    i -= i >= nz ? nz : 0;
    return min(max(i, 0), nz - 1);
}

// (rho, z) table interpolation in FP32 from the float2 copy of the S1xR2
// table: NGP / CIC / TSC exactly as StePS/src/ewald_space.cc:803-1000
// (rho clamped to [0, rho_max], z index periodic).
// CIC reads whole-stencil records (k_table2_cic): 2 loads from one 32-byte
// sector per pair. TSC reads z-triplet records (k_table2_zrec): record
// (ir, iz) = cells (ir, iz-1), (ir, iz), (ir, iz+1), z periodic, as (Dr, Dz)
// pairs in 2 float4, so one rho row of its stencil is 2 loads instead of 3.
// (Whole TSC stencils in 128-byte records -- 5 loads from one line -- were
// 20 % slower: the table grows 4x and falls out of L1.)
template <int ORDER>
__device__ __forceinline__ void s1r2_interp_f32(const float2 *__restrict__ T, const float4 *__restrict__ R, int nrho,
                                                int nz, float irho, float rho_max, float iz, float halfL, float rho,
                                                float z, float &Dr, float &Dz)
{
    const float rr = fminf(fmaxf(rho, 0.0f), rho_max);
    const float ur = rr * irho;
    const float uz = (z + halfL) * iz - 0.5f;
    Dr = 0.0f;
    Dz = 0.0f;
    if (ORDER == 0) {
        int ir = (int)floorf(ur + 0.5f);
        ir = ir < 0 ? 0 : (ir > nrho - 1 ? nrho - 1 : ir);
        int izc = wrap_near(floorf(uz + 0.5f), nz);
        STEPS_CHECK_IDX(ir, nrho, CK_S1_CELL);
        STEPS_CHECK_IDX(izc, nz, CK_S1_CELL);
        const float2 v = __ldg(T + (size_t)ir * nz + izc);
        Dr = v.x;
        Dz = v.y;
    } else if (ORDER == 2) {
        int ir0 = (int)floorf(ur);
        float fr = ur - (float)ir0;
        if (ir0 < 0) { ir0 = 0; fr = 0.0f; }
        if (ir0 > nrho - 2) { ir0 = nrho - 2 > 0 ? nrho - 2 : 0; fr = 1.0f; }
        const float iz0r = floorf(uz);
        const float fz = uz - iz0r;
        int iz0 = wrap_near(iz0r, nz);
        int ra = ir0;
        STEPS_CHECK_IDX(ra, nrho - 1, CK_S1_CELL);
        STEPS_CHECK_IDX(iz0, nz, CK_S1_CELL);
        // record (ir0, iz0): rows ir0, ir0 + 1 x cells iz0, iz0 + 1 (periodic)
        float4 r0, r1;
        ldg_v8(R + 2 * ((size_t)ra * nz + iz0), r0, r1);  // 32-byte records, 256-byte aligned base
        const float w00 = (1.0f - fr) * (1.0f - fz), w10 = fr * (1.0f - fz), w01 = (1.0f - fr) * fz, w11 = fr * fz;
        Dr = w00 * r0.x + w10 * r1.x + w01 * r0.z + w11 * r1.z;
        Dz = w00 * r0.y + w10 * r1.y + w01 * r0.w + w11 * r1.w;
    } else {
        const int jr = (int)floorf(ur + 0.5f), jz = (int)floorf(uz + 0.5f);
        const float sr = ur - (float)jr, sz = uz - (float)jz;
        const float wr[3] = {0.5f * (0.5f - sr) * (0.5f - sr), 0.75f - sr * sr, 0.5f * (0.5f + sr) * (0.5f + sr)};
        const float wz[3] = {0.5f * (0.5f - sz) * (0.5f - sz), 0.75f - sz * sz, 0.5f * (0.5f + sz) * (0.5f + sz)};
        int ir[3] = {jr - 1, jr, jr + 1};
        if (ir[0] < 0) ir[0] = 0;
        if (ir[1] < 0) ir[1] = 0;
        if (ir[1] > nrho - 1) ir[1] = nrho - 1;
        if (ir[2] > nrho - 1) ir[2] = nrho - 1;
        int iz1 = wrap_near((float)jz, nz);
        STEPS_CHECK_IDX(iz1, nz, CK_S1_CELL);
#pragma unroll
        for (int r = 0; r < 3; r++) STEPS_CHECK_IDX(ir[r], nrho, CK_S1_CELL);
#pragma unroll
        for (int r = 0; r < 3; r++) {  // record (ir, iz1): cells iz1 - 1, iz1, iz1 + 1
            float4 v01, v2;
            ldg_v8(R + 2 * ((size_t)ir[r] * nz + iz1), v01, v2);  // 32-byte records
            const float sr_ = fmaf(wz[2], v2.x, fmaf(wz[1], v01.z, wz[0] * v01.x));
            const float sz_ = fmaf(wz[2], v2.y, fmaf(wz[1], v01.w, wz[0] * v01.y));
            Dr = fmaf(wr[r], sr_, Dr);
            Dz = fmaf(wr[r], sz_, Dz);
        }
    }
}

// The separation (q + ql) - (ph + pl) of a double-float pair in FP64 (exact
// up to the FP64 rounding of the sum).
__device__ __forceinline__ double exact_sep(float q, float ph, float ql, float pl)
{
    float e;
    const float s = two_diff(q, ph, e);
    return (double)s + ((double)e + ((double)ql - (double)pl));
}

// NGP cell within FP32 rounding of a face, decided on the FP64 separation
// without a square root. The reference's index is floor(rho / drho + 1/2)
// (StePS/src/ewald_space.cc:803-840); with K the integer nearest to the FP32
// estimate of rho / drho + 1/2, it is K when rho >= (K - 1/2) drho, else K - 1,
// and rho >= f >= 0 is rho^2 >= f^2. Exact up to the FP64 rounding of rho^2
// and of the face: a pair within an ulp or so of a face may differ from the
// reference's own FP64 rounding.
__device__ __forceinline__ int ngp_rho_index(double dx, double dy, float ur_half, const MixedArgs &a)
{
    const float K = rintf(ur_half);
    if (!(K > 0.0f)) return 0;
    const double face = ((double)K - 0.5) * a.s1_drho;
    const int ir = fma(dx, dx, dy * dy) >= face * face ? (int)K : (int)K - 1;
    return min(max(ir, 0), a.nrho - 1);
}

// The same along z: floor((dz + L/2) / dz_cell) is K when dz + L/2 >= K dz_cell.
__device__ __forceinline__ int ngp_z_index(double dz, float uz_half, const MixedArgs &a)
{
    const float K = rintf(uz_half);
    const int iz = dz + 0.5 * a.s1_L >= (double)K * a.s1_dzc ? (int)K : (int)K - 1;
    return wrap_near((float)iz, a.nz);
}

// S1xR2 with the (rho, z) correction table (StePS/src/forces.cc:1307-1350):
// nearest image along z, softened Newton, minus m_j D(rho, dz).
template <int BLOCK, int IPT, int ORDER>
__global__ void __launch_bounds__(BLOCK) k_pair_s1tab(MixedArgs a)
{
    constexpr int T = BLOCK * IPT;
    __shared__ __align__(16) float4 sp[2][T];
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ __align__(16) float4 sres[2][T];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const float L = a.L, halfL = a.halfL;
    const float2 *tab = a.s1tab;
    const float irho = a.irho, iz = a.iz, rho_max = a.rho_max;

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
            float eOx, eOy, eOz;
            const float dOx = two_diff(mJ0.x, mI0.x, eOx), dOy = two_diff(mJ0.y, mI0.y, eOy);
            float dOz = two_diff(mJ0.z, mI0.z, eOz);
            shift_frame(dOz, eOz, L, a.L_lo);  // nearest image of J's centre along z
            const float hz = mI1.z + mJ1.z;
            const bool wrapz = fabsf(dOz) + hz > halfL - a.wrap_tol;
            const float gx = axis_gap(dOx, mI1.x, mJ1.x), gy = axis_gap(dOy, mI1.y, mJ1.y);
            const float gz = axis_gap(dOz, mI1.z, mJ1.z);
            const float bmax = mI0.w + mJ0.w;
            const float g2 = gx * gx + gy * gy + gz * gz;
            const bool full = wrapz || g2 <= bmax * bmax * 1.0001f + 1e-30f || coarse_for_gap(dOx, dOy, dOz, mI1, mJ1, g2, a.guard2);

            // Far tile pairs of the continuous interpolants take the single-rounding
            // separation, as the R^3 and T^3 kernels do; NGP picks a cell, so it
            // keeps the double-float one everywhere.
            const bool dfs = ORDER == 0 || full;
            float phx[IPT], phy[IPT], phz[IPT], plx[IPT], ply[IPT], plz[IPT];
            float px[IPT], py[IPT], pz[IPT], fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                frame_split(xi[k], lx[k], dOx, eOx, phx[k], plx[k]);
                frame_split(yi[k], ly[k], dOy, eOy, phy[k], ply[k]);
                frame_split(zi[k], lz[k], dOz, eOz, phz[k], plz[k]);
                px[k] = phx[k] + plx[k];
                py[k] = phy[k] + ply[k];
                pz[k] = phz[k] + plz[k];
                fx[k] = fy[k] = fz[k] = 0.0f;
            }
            const float4 *spb = sp[buf];
            const float *seb = se[buf];
            const uint32_t *sidb = sid[buf];
            const float4 *sresb = sres[buf];
            for (int jj = 0; jj < T; ++jj) {
                const float4 q = spb[jj];
                const float ej = seb[jj];
                const uint32_t jid = sidb[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const bool self = full && jid == ii[k];
                    float dx, dy, dz;
                    if (dfs) {
                        const float4 ql = sresb[jj];
                        dx = self ? 0.0f : (q.x - phx[k]) + (ql.x - plx[k]);
                        dy = self ? 0.0f : (q.y - phy[k]) + (ql.y - ply[k]);
                        dz = self ? 0.0f : (q.z - phz[k]) + (ql.z - plz[k]);
                        if (wrapz && !self)
                            dz = nearest_image(dz, q.z, phz[k], ql.z, plz[k], L, halfL, a.halfL_lo, a.wrap_tol);
                    } else {
                        dx = q.x - px[k];
                        dy = q.y - py[k];
                        dz = q.z - pz[k];
                    }
                    const float rho2 = fmaf(dx, dx, dy * dy);
                    const float r2 = fmaf(dz, dz, rho2);
                    const float ri = rsqrt_mufu(r2);
                    float w = ri * ri * ri;
                    if (full) {
                        const float b = ei[k] + ej;
                        if (r2 < b * b) w = spline_inner_f32(r2, b);
                    }
                    const float rho = sqrt_mufu(rho2);
                    float Dr, Dz;
                    if (ORDER == 0) {
                        // NGP picks a cell, a hard decision: within FP32 rounding of
                        // a cell face it is taken on the FP64 separation.
                        const float ur = fminf(fmaxf(rho, 0.0f), rho_max) * irho + 0.5f;
                        const float uzc = (dz + halfL) * iz;
                        const float flr = floorf(ur), flz = floorf(uzc);
                        // FP32 (rho, z) carry < 3e-7 relative error; margin 2x
                        const float tr = 6e-7f * ur + 2e-6f, tz = 6e-7f * uzc + 2e-6f;
                        int ir = min(max((int)flr, 0), a.nrho - 1);
                        int izc = wrap_near(flz, a.nz);
                        const bool amb_r = fabsf(ur - flr - 0.5f) > 0.5f - tr;
                        const bool amb_z = fabsf(uzc - flz - 0.5f) > 0.5f - tz;
                        if (!self && (amb_r || amb_z)) {
                            const float4 ql = sresb[jj];
                            if (amb_r)
                                ir = ngp_rho_index(exact_sep(q.x, phx[k], ql.x, plx[k]),
                                                   exact_sep(q.y, phy[k], ql.y, ply[k]), ur, a);
                            if (amb_z) {
                                double dz64 = exact_sep(q.z, phz[k], ql.z, plz[k]);
                                if (dz != (q.z - phz[k]) + (ql.z - plz[k])) dz64 -= copysign(a.s1_L, dz64);  // wrapped
                                izc = ngp_z_index(dz64, uzc, a);
                            }
                        }
                        STEPS_CHECK_IDX(ir, a.nrho, CK_S1_CELL);
                        STEPS_CHECK_IDX(izc, a.nz, CK_S1_CELL);
                        const float2 v = __ldg(tab + (size_t)ir * a.nz + izc);
                        Dr = v.x;
                        Dz = v.y;
                    } else {
                        s1r2_interp_f32<ORDER>(tab, a.s1rec, a.nrho, a.nz, irho, rho_max, iz, halfL, rho, dz, Dr, Dz);
                    }
                    const float er = rho > 0.0f ? Dr * rcp_mufu(rho) : 0.0f;
                    fx[k] = fmaf(q.w, fmaf(w, dx, -er * dx), fx[k]);
                    fy[k] = fmaf(q.w, fmaf(w, dy, -er * dy), fy[k]);
                    fz[k] = fmaf(q.w, fmaf(w, dz, -Dz), fz[k]);
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

// CIC stencil records of the (rho, z) table: record (ir, iz) holds rows ir,
// ir + 1 (clamped to the table) x cells iz, iz + 1 (periodic) as (D_rho, D_z)
// pairs in 2 float4.
__global__ void k_table2_cic(const double *__restrict__ t, int nrho, int nz, float4 *__restrict__ out)
{
    const size_t ncell = (size_t)nrho * nz;
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int iz = (int)(c % nz), ir = (int)(c / nz);
    const int ir1 = ir + 1 < nrho ? ir + 1 : nrho - 1, iz1 = iz + 1 < nz ? iz + 1 : 0;
    const size_t a = (size_t)ir * nz + iz, b = (size_t)ir * nz + iz1, d = (size_t)ir1 * nz + iz,
                 e = (size_t)ir1 * nz + iz1;
    out[2 * c] = make_float4((float)t[2 * a], (float)t[2 * a + 1], (float)t[2 * b], (float)t[2 * b + 1]);
    out[2 * c + 1] = make_float4((float)t[2 * d], (float)t[2 * d + 1], (float)t[2 * e], (float)t[2 * e + 1]);
}

// z-triplet records of the (rho, z) table for TSC (see s1r2_interp_f32).
__global__ void k_table2_zrec(const double *__restrict__ t, int nrho, int nz, float4 *__restrict__ out)
{
    const size_t ncell = (size_t)nrho * nz;
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int iz = (int)(c % nz);
    const size_t row = c - iz;
    const size_t m = row + (iz > 0 ? iz - 1 : nz - 1), p = row + (iz + 1 < nz ? iz + 1 : 0);
    out[2 * c] = make_float4((float)t[2 * m], (float)t[2 * m + 1], (float)t[2 * c], (float)t[2 * c + 1]);
    out[2 * c + 1] = make_float4((float)t[2 * p], (float)t[2 * p + 1], 0.0f, 0.0f);
}

__global__ void k_table2_f32(const double *__restrict__ t, size_t ncell, float2 *__restrict__ out)
{
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncell) out[c] = make_float2((float)t[2 * c], (float)t[2 * c + 1]);
}

template <int ORDER>
KernelFn pick_s1tab(int threads, int ipt)
{
#define STEPS_SHAPE(B, P) \
    if (threads == B && ipt == P) return k_pair_s1tab<B, P, ORDER>;
    STEPS_SHAPE(64, 1) STEPS_SHAPE(64, 2) STEPS_SHAPE(128, 1) STEPS_SHAPE(128, 2) STEPS_SHAPE(256, 1)
#undef STEPS_SHAPE
    return nullptr;
}

// FP32 copy of the ng^3 table with a periodic halo of `halo` cells on every
// side: cell (i, j, k) of the ext^3 copy, ext = ng + 2 halo, is table cell
// ((i - halo) mod ng, (j - halo) mod ng, (k - halo) mod ng).
__global__ void k_table_f32(const double *__restrict__ t, int ng, int halo, float4 *__restrict__ out)
{
    const int ext = ng + 2 * halo;
    const size_t ncell = (size_t)ext * ext * ext;
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int k = (int)(c % ext), j = (int)((c / ext) % ext), i = (int)(c / ((size_t)ext * ext));
    const size_t s = ((size_t)pmod(i - halo, ng) * ng + pmod(j - halo, ng)) * ng + pmod(k - halo, ng);
    out[c] = make_float4((float)t[3 * s], (float)t[3 * s + 1], (float)t[3 * s + 2], 0.0f);
}

// Ewald correction D(d) of one pair from the FP32 table (not the window):
// stencil records of the haloed copy when the tile pair's stencils stay in
// the halo, else taps of the haloed copy at indices wrapped once per axis.
template <int ORDER>
__device__ __forceinline__ void t3_correction(const MixedArgs &a, bool halo, float dx, float dy, float dz, float &Dx,
                                              float &Dy, float &Dz)
{
    constexpr int NT = ORDER;
    constexpr int OFF = ORDER == 4 ? 1 : 0;
    float wx[4], wy[4], wz[4];
    Dx = Dy = Dz = 0.0f;
    if (halo) {
        const float uh = a.u0 + (float)a.halo;
        const float ux = fmaf(dx, a.ih, uh), uy = fmaf(dy, a.ih, uh), uz = fmaf(dz, a.ih, uh);
        const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
        weights<ORDER>(ux - fxl, wx);
        weights<ORDER>(uy - fyl, wy);
        weights<ORDER>(uz - fzl, wz);
        const int E = a.ext;
        int bx = min(max((int)fxl - OFF, 0), E - NT);
        int by = min(max((int)fyl - OFF, 0), E - NT);
        int bz = min(max((int)fzl - OFF, 0), E - NT);
#ifdef STEPS_CHECK
        const long long hfirst = ((long long)bx * E + by) * E + bz;
        if (!check_span(hfirst, hfirst + (long long)(NT - 1) * ((long long)E * E + E + 1), (long long)E * E * E,
                        CK_T3_CELL))
            bx = by = bz = 0;
#endif
        const int cb = (bx * E + by) * E + bz;
        if (ORDER == 4) {  // z-row records
#pragma unroll
            for (int aa = 0; aa < 4; aa++) {
                float rx = 0.0f, ry = 0.0f, rz = 0.0f;
#pragma unroll
                for (int bb = 0; bb < 4; bb++) {
                    const int cr = cb + (aa * E + bb) * E;
                    float4 vx, vy;
                    ldg_v8(a.t3r + 2 * (size_t)cr, vx, vy);
                    const float4 vz = __ldg(a.t3rz + cr);
                    rx = fmaf(wy[bb], dot4(wz, vx), rx);
                    ry = fmaf(wy[bb], dot4(wz, vy), ry);
                    rz = fmaf(wy[bb], dot4(wz, vz), rz);
                }
                Dx = fmaf(wx[aa], rx, Dx);
                Dy = fmaf(wx[aa], ry, Dy);
                Dz = fmaf(wx[aa], rz, Dz);
            }
        } else {  // (y, z) quad records
            const float q00 = wy[0] * wz[0], q01 = wy[0] * wz[1], q10 = wy[1] * wz[0], q11 = wy[1] * wz[1];
#pragma unroll
            for (int aa = 0; aa < 2; aa++) {
                const int cr = cb + aa * E * E;
                float4 vx, vy;
                ldg_v8(a.t3r + 2 * (size_t)cr, vx, vy);
                const float4 vz = __ldg(a.t3rz + cr);
                Dx = fmaf(wx[aa], fmaf(q11, vx.w, fmaf(q10, vx.z, fmaf(q01, vx.y, q00 * vx.x))), Dx);
                Dy = fmaf(wx[aa], fmaf(q11, vy.w, fmaf(q10, vy.z, fmaf(q01, vy.y, q00 * vy.x))), Dy);
                Dz = fmaf(wx[aa], fmaf(q11, vz.w, fmaf(q10, vz.z, fmaf(q01, vz.y, q00 * vz.x))), Dz);
            }
        }
    } else {
        const float ux = fmaf(dx, a.ih, a.u0), uy = fmaf(dy, a.ih, a.u0), uz = fmaf(dz, a.ih, a.u0);
        const float fxl = floorf(ux), fyl = floorf(uy), fzl = floorf(uz);
        weights<ORDER>(ux - fxl, wx);
        weights<ORDER>(uy - fyl, wy);
        weights<ORDER>(uz - fzl, wz);
        const int bx = (int)fxl - OFF, by = (int)fyl - OFF, bz = (int)fzl - OFF;
        int gx[NT], gy[NT], gz[NT];
#pragma unroll
        for (int t = 0; t < NT; t++) {
            gx[t] = wrap_index(bx + t, a.ng) + a.halo;
            gy[t] = wrap_index(by + t, a.ng) + a.halo;
            gz[t] = wrap_index(bz + t, a.ng) + a.halo;
            STEPS_CHECK_IDX(gx[t], a.ext, CK_T3_CELL);
            STEPS_CHECK_IDX(gy[t], a.ext, CK_T3_CELL);
            STEPS_CHECK_IDX(gz[t], a.ext, CK_T3_CELL);
        }
        stencil<ORDER>(wx, wy, wz,
                       [&](int aa, int bb, int cc) { return __ldg(a.t3f + (gx[aa] * a.ext + gy[bb]) * a.ext + gz[cc]); },
                       Dx, Dy, Dz);
    }
}

// Quad lane mapping (T^3 variant 1, one i per thread). The 32 lanes of a warp
// form 8 quads; quad g holds the warp's i particles 4g..4g+3 (one per lane).
// In each step every lane of quad g takes the same i, 4g + s for s = 0..3 in
// turn, against its own j, jb + (lane & 3). One table-record load then serves
// 8 distinct i against 4 neighbouring j instead of 32 i against one j, and
// the lanes' stencils share more L1 lines. Each lane keeps 4 FP32 partial
// forces (one per i of its quad) over a j tile; a 4-lane transpose-reduce
// (3 shuffles per component) leaves every lane the sum for its own i, which
// goes into the FP64 accumulator as in the one-i-per-lane kernel.
template <int BLOCK, int ORDER>
__global__ void __launch_bounds__(BLOCK) k_pair_t3q(MixedArgs a)
{
    constexpr int T = BLOCK;
    constexpr int NT = ORDER;
    constexpr int OFF = ORDER == 4 ? 1 : 0;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ __align__(16) float4 sp[2][T];
    __shared__ __align__(16) float se[2][T];
    __shared__ __align__(16) uint32_t sid[2][T];
    __shared__ __align__(16) float4 sres[2][T];
    __shared__ int s_item;
    const int tid = threadIdx.x, lane = tid & 31, r = lane & 3, qb = lane & ~3;
    const float L = a.L, halfL = a.halfL;

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
        const size_t qi = (size_t)I * T + tid;
        const float4 pi = __ldg(a.ipack + qi);
        const float4 li = __ldg(a.ilo + qi);
        const float eown = __ldg(a.ieps + qi);
        const uint32_t idown = __ldg(a.iidx + qi);
        double ax = 0.0, ay = 0.0, az = 0.0;

        if (J0 < J1) stage_tile<BLOCK, 1>(a, J0, sp[0], se[0], sid[0], sres[0]);
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
            bool halo = ORDER != 0;
#pragma unroll
            for (int ax3 = 0; ax3 < 3; ax3++) {
                shift_frame(dO[ax3], eO[ax3], L, a.L_lo);  // nearest image of J's centre
                wrap[ax3] = fabsf(dO[ax3]) + hs[ax3] > halfL - a.wrap_tol;
                const float g = fmaxf(fabsf(dO[ax3]) - hs[ax3], 0.0f);
                g2 += g * g;
                const int w0 = (int)floorf((dO[ax3] - hs[ax3]) * a.ih + a.u0 - 1e-3f) - OFF;
                const int w1 = (int)floorf((dO[ax3] + hs[ax3]) * a.ih + a.u0 + 1e-3f) - OFF + NT;
                halo = halo && w0 >= -a.halo && w1 <= a.ng + a.halo;
            }
            const float bmax = mI0.w + mJ0.w;
            const bool full = g2 <= bmax * bmax * 1.0001f + 1e-30f || wrap[0] || wrap[1] || wrap[2] ||
                              coarse_for_gap(dO[0], dO[1], dO[2], mI1, mJ1, g2, a.guard2);
            if (J + 1 < J1) {
                stage_tile<BLOCK, 1>(a, J + 1, sp[buf ^ 1], se[buf ^ 1], sid[buf ^ 1], sres[buf ^ 1]);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();

            // own i in J's frame
            float phx, phy, phz, plx, ply, plz;
            frame_split(pi.x, li.x, dO[0], eO[0], phx, plx);
            frame_split(pi.y, li.y, dO[1], eO[1], phy, ply);
            frame_split(pi.z, li.z, dO[2], eO[2], phz, plz);
            float fx[4] = {0.0f, 0.0f, 0.0f, 0.0f}, fy[4] = {0.0f, 0.0f, 0.0f, 0.0f},
                  fz[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            const float4 *spb = sp[buf];
            const float *seb = se[buf];
            const uint32_t *sidb = sid[buf];
            const float4 *sresb = sres[buf];

            if (!full) {
                // far tile pair: the quad's four i as single FP32 positions
                float Px[4], Py[4], Pz[4];
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    Px[s] = __shfl_sync(FULL, phx + plx, qb | s);
                    Py[s] = __shfl_sync(FULL, phy + ply, qb | s);
                    Pz[s] = __shfl_sync(FULL, phz + plz, qb | s);
                }
#pragma unroll 1
                for (int jb = 0; jb < T; jb += 4) {
                    const float4 q = spb[jb + r];
#pragma unroll
                    for (int s = 0; s < 4; s++) {
                        const float dx = q.x - Px[s], dy = q.y - Py[s], dz = q.z - Pz[s];
                        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        const float ri = rsqrt_mufu(r2);
                        const float w = ri * ri * ri;
                        float Dx = 0.0f, Dy = 0.0f, Dz = 0.0f;
                        if (ORDER != 0) t3_correction<ORDER>(a, halo, dx, dy, dz, Dx, Dy, Dz);
                        fx[s] = fmaf(q.w, fmaf(w, dx, -Dx), fx[s]);
                        fy[s] = fmaf(q.w, fmaf(w, dy, -Dy), fy[s]);
                        fz[s] = fmaf(q.w, fmaf(w, dz, -Dz), fz[s]);
                    }
                }
            } else {
                // near tile pair (rare): double-float separations, softening, the
                // exact nearest-image decision; each i fetched from its lane per step
#pragma unroll 1
                for (int jb = 0; jb < T; jb += 4) {
                    const int jj = jb + r;
                    const float4 q = spb[jj];
                    const float ej = seb[jj];
                    const uint32_t jid = sidb[jj];
                    const float4 ql = sresb[jj];
#pragma unroll
                    for (int s = 0; s < 4; s++) {
                        const float hx = __shfl_sync(FULL, phx, qb | s), hy = __shfl_sync(FULL, phy, qb | s),
                                    hz = __shfl_sync(FULL, phz, qb | s);
                        const float lx_ = __shfl_sync(FULL, plx, qb | s), ly_ = __shfl_sync(FULL, ply, qb | s),
                                    lz_ = __shfl_sync(FULL, plz, qb | s);
                        const float ei = __shfl_sync(FULL, eown, qb | s);
                        const uint32_t iid = __shfl_sync(FULL, idown, qb | s);
                        const bool self = jid == iid;
                        const float dx = self ? 0.0f : (q.x - hx) + (ql.x - lx_);
                        const float dy = self ? 0.0f : (q.y - hy) + (ql.y - ly_);
                        const float dz = self ? 0.0f : (q.z - hz) + (ql.z - lz_);
                        float nx = dx, ny = dy, nz = dz;
                        if (!self) {  // wrapped axes are full-path tile pairs
                            if (wrap[0]) nx = nearest_image(dx, q.x, hx, ql.x, lx_, L, halfL, a.halfL_lo, a.wrap_tol);
                            if (wrap[1]) ny = nearest_image(dy, q.y, hy, ql.y, ly_, L, halfL, a.halfL_lo, a.wrap_tol);
                            if (wrap[2]) nz = nearest_image(dz, q.z, hz, ql.z, lz_, L, halfL, a.halfL_lo, a.wrap_tol);
                        }
                        const float r2 = fmaf(nx, nx, fmaf(ny, ny, nz * nz));
                        const float ri = rsqrt_mufu(r2);
                        float w = ri * ri * ri;
                        const float bb = ei + ej;
                        if (r2 < bb * bb) w = spline_inner_f32(r2, bb);
                        float Dx = 0.0f, Dy = 0.0f, Dz = 0.0f;
                        if (ORDER != 0) t3_correction<ORDER>(a, halo, dx, dy, dz, Dx, Dy, Dz);
                        fx[s] = fmaf(q.w, fmaf(w, nx, -Dx), fx[s]);
                        fy[s] = fmaf(q.w, fmaf(w, ny, -Dy), fy[s]);
                        fz[s] = fmaf(q.w, fmaf(w, nz, -Dz), fz[s]);
                    }
                }
            }
            // 4-lane transpose-reduce: lane r = 2b + c ends with the sum of
            // element r over its quad
            const bool b = (r & 2) != 0, c = (r & 1) != 0;
            float h0, h1, tx, ty, tz;
            h0 = (b ? fx[2] : fx[0]) + __shfl_xor_sync(FULL, b ? fx[0] : fx[2], 2);
            h1 = (b ? fx[3] : fx[1]) + __shfl_xor_sync(FULL, b ? fx[1] : fx[3], 2);
            tx = (c ? h1 : h0) + __shfl_xor_sync(FULL, c ? h0 : h1, 1);
            h0 = (b ? fy[2] : fy[0]) + __shfl_xor_sync(FULL, b ? fy[0] : fy[2], 2);
            h1 = (b ? fy[3] : fy[1]) + __shfl_xor_sync(FULL, b ? fy[1] : fy[3], 2);
            ty = (c ? h1 : h0) + __shfl_xor_sync(FULL, c ? h0 : h1, 1);
            h0 = (b ? fz[2] : fz[0]) + __shfl_xor_sync(FULL, b ? fz[0] : fz[2], 2);
            h1 = (b ? fz[3] : fz[1]) + __shfl_xor_sync(FULL, b ? fz[1] : fz[3], 2);
            tz = (c ? h1 : h0) + __shfl_xor_sync(FULL, c ? h0 : h1, 1);
            ax += (double)tx;
            ay += (double)ty;
            az += (double)tz;
            __syncthreads();
        }

        double *o = a.part + (size_t)chunk * a.part_stride;
        o[3 * qi] = ax;
        o[3 * qi + 1] = ay;
        o[3 * qi + 2] = az;
    }
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

KernelFn t3_quad_kernel(const KParams &kp, int threads, int ipt)
{
    if (kp.is_periodic < 2 || kp.order != 2 || ipt != 1) return nullptr;  // trilinear, one i per thread
    if (threads == 64) return k_pair_t3q<64, 2>;
    if (threads == 128) return k_pair_t3q<128, 2>;
    if (threads == 256) return k_pair_t3q<256, 2>;
    return nullptr;
}

KernelFn t3_kernel(const KParams &kp, int threads, int ipt, size_t *dyn_smem, int variant)
{
    *dyn_smem = 0;
    if (kp.is_periodic < 2) return pick_t3<0>(threads, ipt);
    if (variant == 1)  // quad lanes where they exist (no shared-memory window)
        if (KernelFn q = t3_quad_kernel(kp, threads, ipt)) return q;
    *dyn_smem = (size_t)ctx().shape.t3_cells * sizeof(float4);
    return kp.order == 4 ? pick_t3<4>(threads, ipt) : pick_t3<2>(threads, ipt);
}

// Stencil records of the haloed table, one float4 per component, record
// (i, j, k) of the ext^3 grid (x and y in out[2c], out[2c + 1], z in outz[c]):
//   tricubic: z row  -- cells (i, j, k..k+3)
//   trilinear: (y, z) quad -- cells (i, j, k), (i, j, k+1), (i, j+1, k), (i, j+1, k+1)
__global__ void k_table_records(const double *__restrict__ t, int ng, int halo, int order, float4 *__restrict__ out,
                                float4 *__restrict__ outz)
{
    const int ext = ng + 2 * halo;
    const size_t ncell = (size_t)ext * ext * ext;
    size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int k = (int)(c % ext), j = (int)((c / ext) % ext), i = (int)(c / ((size_t)ext * ext));
    float v[3][4];
    for (int q = 0; q < 4; q++) {
        const int dj = order == 4 ? 0 : q >> 1, dk = order == 4 ? q : q & 1;
        const size_t s = ((size_t)pmod(i - halo, ng) * ng + pmod(j + dj - halo, ng)) * ng + pmod(k + dk - halo, ng);
        for (int comp = 0; comp < 3; comp++) v[comp][q] = (float)t[3 * s + comp];
    }
    out[2 * c] = make_float4(v[0][0], v[0][1], v[0][2], v[0][3]);
    out[2 * c + 1] = make_float4(v[1][0], v[1][1], v[1][2], v[1][3]);
    outz[c] = make_float4(v[2][0], v[2][1], v[2][2], v[2][3]);
}

// Halo of the FP32 table copies: tile pairs whose stencils stay within it
// need no per-pair wrap. It grows with the grid (cells shrink as L / ng, tile
// extents do not): 16 cells at ng = 63, ng / 8 above 128.
inline int t3_halo(int ng) { return ng / 8 > 16 ? ng / 8 : 16; }

// FP32 float4 haloed copy of the FP64 table, rebuilt whenever the table changes.
const float4 *t3_table_f32(const Tables &tb, cudaStream_t st)
{
    Ctx &c = ctx();
    const size_t ext = (size_t)tb.t3_ng + 2 * t3_halo(tb.t3_ng);
    const size_t ncell = ext * ext * ext;
    if (c.t3f_version != c.t3_version || !c.t3f.p) {
        float4 *o = c.t3f.ensure<float4>(ncell);
        k_table_f32<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.t3, tb.t3_ng, t3_halo(tb.t3_ng), o);
        note_launch("k_table_f32");
        c.t3f_version = c.t3_version;
    }
    return c.t3f.as<float4>();
}

// The stencil records for the table's interpolation order, rebuilt whenever
// the table or the order changes.
const float4 *t3_table_records(const Tables &tb, int order, cudaStream_t st)
{
    Ctx &c = ctx();
    const size_t ext = (size_t)tb.t3_ng + 2 * t3_halo(tb.t3_ng);
    const size_t ncell = ext * ext * ext;
    if (c.t3r_version != c.t3_version || c.t3r_order != order || !c.t3r.p) {
        float4 *o = c.t3r.ensure<float4>(3 * ncell);  // 2 ncell xy records, then ncell z records
        k_table_records<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.t3, tb.t3_ng, t3_halo(tb.t3_ng), order,
                                                                          o, o + 2 * ncell);
        note_launch("k_table_records");
        c.t3r_version = c.t3_version;
        c.t3r_order = order;
    }
    return c.t3r.as<float4>();
}

void t3_args(MixedArgs &a, const KParams &kp, const Tables &tb, cudaStream_t st)
{
    a.t3f = nullptr;
    a.ng = tb.t3_ng;
    a.ih = 0.0f;
    a.u0 = 0.0f;
    a.wcap = ctx().shape.t3_cells;
    a.halo = t3_halo(tb.t3_ng);
    a.ext = tb.t3_ng + 2 * a.halo;
    a.t3r = nullptr;
    a.t3rz = nullptr;
    if (kp.is_periodic >= 2) {
        a.t3f = t3_table_f32(tb, st);
        a.t3r = t3_table_records(tb, kp.order == 4 ? 4 : 2, st);
        const size_t ext = (size_t)tb.t3_ng + 2 * t3_halo(tb.t3_ng);
        a.t3rz = a.t3r + 2 * ext * ext * ext;
        a.ih = (float)((double)tb.t3_ng / kp.L);
        a.u0 = (float)((double)tb.t3_ng * 0.5 - 0.5);
    }
}

KernelFn s1tab_kernel(const KParams &kp, int threads, int ipt)
{
    if (kp.order == 0) return pick_s1tab<0>(threads, ipt);
    if (kp.order == 2) return pick_s1tab<2>(threads, ipt);
    return pick_s1tab<4>(threads, ipt);
}

void s1tab_args(MixedArgs &a, const KParams &kp, const Tables &tb, cudaStream_t st)
{
    Ctx &c = ctx();
    size_t ncell = (size_t)tb.nrho * tb.nz;
    if (c.s1f_version != c.s1r2_version || !c.s1f.p) {
        float2 *o = c.s1f.ensure<float2>(ncell);
        k_table2_f32<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.s1r2, ncell, o);
        note_launch("k_table2_f32");
        c.s1f_version = c.s1r2_version;
    }
    if (kp.order != 0 && (c.s1rec_version != c.s1r2_version || c.s1rec_order != kp.order || !c.s1rec.p)) {
        if (kp.order == 4) {
            float4 *o = c.s1rec.ensure<float4>(2 * ncell);
            k_table2_zrec<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.s1r2, tb.nrho, tb.nz, o);
            note_launch("k_table2_zrec");
        } else {
            float4 *o = c.s1rec.ensure<float4>(2 * ncell);
            k_table2_cic<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(tb.s1r2, tb.nrho, tb.nz, o);
            note_launch("k_table2_cic");
        }
        c.s1rec_version = c.s1r2_version;
        c.s1rec_order = kp.order;
    }
    a.s1tab = c.s1f.as<float2>();
    a.s1rec = kp.order != 0 ? c.s1rec.as<float4>() : nullptr;
    a.nrho = tb.nrho;
    a.nz = tb.nz;
    const double drho = tb.rho_max / (double)(tb.nrho - 1 > 1 ? tb.nrho - 1 : 1);
    a.irho = (float)(1.0 / drho);
    a.iz = (float)((double)tb.nz / kp.L);
    a.rho_max = (float)tb.rho_max;
    a.s1_drho = drho;
    a.s1_dzc = kp.L / (double)tb.nz;
    a.s1_L = kp.L;
}

}  // namespace steps
