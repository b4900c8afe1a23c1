// The tile builder shared by the ordering pass (order.cu) and the persistent
// ensemble kernel (pair_r3x2.cu), which rebuilds each tile after its kick and
// drift.
#pragma once

#include "common.cuh"

namespace steps {

__device__ __forceinline__ double warp_min(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Builds tile `tile` (the T particles of sorted positions [sbase, sbase + cnt),
// padded to T) with a block of NT threads: FP32-exact centre, half extents and
// largest softening (meta), FP32 offsets (pack, soa), their FP32 residuals
// (lo), softening (epsf), original indices (idx) and the sub-tile boxes (sub).
// perm holds original indices below nx (checked in bounds-checked builds).
// COH: positions are read through L2 (ld.global.cg), for a kernel in which
// other blocks have just written them (L1 is not coherent across SMs).
template <int NT, bool COH>
__device__ __forceinline__ void build_tile(int tile, int sbase, int cnt, const double *__restrict__ x,
                                           const double *__restrict__ m, const double *__restrict__ eps,
                                           const uint32_t *__restrict__ perm, long long nx, int T,
                                           float4 *__restrict__ pack,
                                           float *__restrict__ epsf, float4 *__restrict__ meta,
                                           uint32_t *__restrict__ idx, uint32_t pad_id, float4 *__restrict__ lo,
                                           float *__restrict__ soa, float4 *__restrict__ sub)
{
    __shared__ double red[7][NT / 32];
    __shared__ float s_c[3];
    auto ldx = [&](size_t q) { return COH ? __ldcg(x + q) : x[q]; };
    int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300}, em = 0.0;
    for (int e = t; e < T; e += NT) {
        if (e < cnt) {
            uint32_t o = perm[sbase + e];
            STEPS_CHECK_IDX(o, nx, CK_PERM);
            for (int k = 0; k < 3; k++) {
                double v = ldx(3 * (size_t)o + k);
                mn[k] = fmin(mn[k], v);
                mx[k] = fmax(mx[k], v);
            }
            em = fmax(em, eps[o]);
        }
    }
    for (int k = 0; k < 3; k++) { mn[k] = warp_min(mn[k]); mx[k] = warp_max(mx[k]); }
    em = warp_max(em);
    if (lane == 0) {
        for (int k = 0; k < 3; k++) { red[k][w] = mn[k]; red[3 + k][w] = mx[k]; }
        red[6][w] = em;
    }
    __syncthreads();
    if (t == 0) {
        double a[7];
        for (int k = 0; k < 7; k++) a[k] = red[k][0];
        for (int v = 1; v < NT / 32; v++) {
            for (int k = 0; k < 3; k++) { a[k] = fmin(a[k], red[k][v]); a[3 + k] = fmax(a[3 + k], red[3 + k][v]); }
            a[6] = fmax(a[6], red[6][v]);
        }
        float c[3], h[3];
        for (int k = 0; k < 3; k++) {
            if (a[k] > a[3 + k]) { a[k] = 0.0; a[3 + k] = 0.0; }  // empty tile
            c[k] = __double2float_rn(0.5 * (a[k] + a[3 + k]));
            double ext = fmax(a[3 + k] - (double)c[k], (double)c[k] - a[k]);
            // Round up so the FP32 half extent bounds every FP32 offset.
            h[k] = __double2float_ru(ext * (1.0 + 1e-6)) + 1e-30f;
            s_c[k] = c[k];
        }
        meta[2 * tile] = make_float4(c[0], c[1], c[2], __double2float_ru(a[6]));
        meta[2 * tile + 1] = make_float4(h[0], h[1], h[2], 0.0f);
    }
    __syncthreads();
    double cx = s_c[0], cy = s_c[1], cz = s_c[2];
    for (int e = t; e < T; e += NT) {
        const int q = tile * T + e;
        if (e < cnt) {
            uint32_t o = perm[sbase + e];
            STEPS_CHECK_IDX(o, nx, CK_PERM);
            const double ox = ldx(3 * (size_t)o) - cx, oy = ldx(3 * (size_t)o + 1) - cy, oz = ldx(3 * (size_t)o + 2) - cz;
            const float hx = __double2float_rn(ox), hy = __double2float_rn(oy), hz = __double2float_rn(oz);
            pack[q] = make_float4(hx, hy, hz, __double2float_rn(m[o]));
            if (soa) {  // tile-blocked SoA copy: X[T], Y[T], Z[T], M[T] per tile
                float *b = soa + (size_t)tile * 4 * T;
                b[e] = hx;
                b[T + e] = hy;
                b[2 * T + e] = hz;
                b[3 * T + e] = __double2float_rn(m[o]);
            }
            // What FP32 dropped from the offset: i particles carry it so that
            // their position in another tile's frame keeps full precision.
            if (lo)
                lo[q] = make_float4(__double2float_rn(ox - hx), __double2float_rn(oy - hy), __double2float_rn(oz - hz),
                                    0.f);
            epsf[q] = __double2float_rn(eps[o]);
            if (idx) idx[q] = o;
        } else {
            pack[q] = make_float4(0.f, 0.f, 0.f, 0.f);  // massless padding at the tile centre
            if (soa) {
                float *b = soa + (size_t)tile * 4 * T;
                b[e] = b[T + e] = b[2 * T + e] = b[3 * T + e] = 0.f;
            }
            if (lo) lo[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            epsf[q] = 0.f;
            if (idx) idx[q] = pad_id;
        }
        if (sub) {
            // Sub-tile boxes: the SUBTILE consecutive particles of a half warp
            // (padding included, at the tile centre), in the tile's FP32 offset
            // frame, widened by 1e-6 relative so they hold the exact positions.
            const float4 pq = pack[q];
            float l3[3] = {pq.x, pq.y, pq.z}, h3[3] = {pq.x, pq.y, pq.z};
            float se = epsf[q];
#pragma unroll
            for (int o = SUBTILE / 2; o > 0; o >>= 1) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    l3[k] = fminf(l3[k], __shfl_xor_sync(0xffffffffu, l3[k], o));
                    h3[k] = fmaxf(h3[k], __shfl_xor_sync(0xffffffffu, h3[k], o));
                }
                se = fmaxf(se, __shfl_xor_sync(0xffffffffu, se, o));
            }
            if ((e & (SUBTILE - 1)) == 0) {
                float c3[3], w3[3];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    c3[k] = 0.5f * (l3[k] + h3[k]);
                    const float w = fmaxf(h3[k] - c3[k], c3[k] - l3[k]);
                    w3[k] = w * 1.000001f + 1e-6f * (fabsf(c3[k]) + w) + 1e-30f;
                }
                float4 *d = sub + 2 * ((size_t)tile * (T / SUBTILE) + e / SUBTILE);
                d[0] = make_float4(c3[0], c3[1], c3[2], se);
                d[1] = make_float4(w3[0], w3[1], w3[2], 0.0f);
            }
        }
    }
}


}  // namespace steps
