// Spatial ordering of a particle set for the mixed-precision kernels:
//   1. bounding box (FP64, atomic min/max on order-preserving integer images),
//   2. 63-bit Morton keys (21 bits per axis) of the positions in the box,
//   3. a stable least-significant-digit radix sort of (key, index) pairs,
//   4. tiles of T consecutive particles along the curve: each tile gets an
//      FP32-exact centre c, FP32 offsets x - c computed in FP64, half extents
//      and its largest softening length.
// The order only sets locality (tile size, hence FP32 offset magnitude and
// the near/far split); the forces do not depend on it beyond rounding.
#include "common.cuh"
#include "context.cuh"
#include "tile.cuh"

namespace steps {

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;  // elements per thread per block
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;
constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;

__global__ void k_bbox_init(unsigned long long *bb)
{
    int t = threadIdx.x;
    if (t < 3) bb[t] = ~0ull;        // min
    else if (t < 6) bb[t] = 0ull;    // max
}

__global__ void k_bbox(const double *__restrict__ x, int lo, int count, unsigned long long *bb)
{
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x) {
        const double *p = x + 3 * (size_t)(lo + q);
        for (int k = 0; k < 3; k++) { mn[k] = fmin(mn[k], p[k]); mx[k] = fmax(mx[k], p[k]); }
    }
    for (int k = 0; k < 3; k++)
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmax(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; k++) {
            atomicMin(&bb[k], ordered_bits(mn[k]));
            atomicMax(&bb[3 + k], ordered_bits(mx[k]));
        }
}

// Keys for particles lo..lo+count-1; prefix (the realisation index of a batch)
// occupies the bits above 3*bits.
__global__ void k_keys(const double *__restrict__ x, int lo, int count, const unsigned long long *bb, int bits,
                       unsigned long long prefix, unsigned long long *keys, uint32_t *vals)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    double cells = (double)(1u << bits);
    const double *p = x + 3 * (size_t)(lo + q);
    unsigned long long key = 0;
    for (int k = 0; k < 3; k++) {
        double lo_k = from_ordered_bits(bb[k]);
        double hi_k = from_ordered_bits(bb[3 + k]);
        double span = hi_k - lo_k;
        double u = span > 0 ? (p[k] - lo_k) / span * cells : 0.0;
        long long c = (long long)u;
        c = c < 0 ? 0 : (c >= (long long)cells ? (long long)cells - 1 : c);
        key |= spread3((unsigned long long)c) << k;
    }
    keys[q] = key | (prefix << (3 * bits));
    vals[q] = (uint32_t)(lo + q);
}

// Per-block digit histograms, stored digit-major: hist[d * nblk + b].
__global__ void __launch_bounds__(SORT_THREADS) k_hist(const unsigned long long *__restrict__ keys, int n, int shift,
                                                      uint32_t *hist)
{
    __shared__ uint32_t h[RADIX];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; r++) {
        int q = base + r * SORT_THREADS + threadIdx.x;
        if (q < n) atomicAdd(&h[(keys[q] >> shift) & (RADIX - 1)], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of hist[0..total) in one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan(uint32_t *hist, int total)
{
    __shared__ uint32_t part[1024];
    int t = threadIdx.x;
    int per = div_up(total, 1024);
    int b = t * per, e = min(total, b + per);
    uint32_t s = 0;
    for (int i = b; i < e; i++) s += hist[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t ? part[t - 1] : 0;
    for (int i = b; i < e; i++) {
        uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// Stable scatter: element order inside a block is (round, warp, lane), which is
// the input order, and ranks among equal digits follow that order.
__global__ void __launch_bounds__(SORT_THREADS) k_scatter(const unsigned long long *__restrict__ kin,
                                                         const uint32_t *__restrict__ vin, int n, int shift,
                                                         const uint32_t *__restrict__ hist,
                                                         unsigned long long *__restrict__ kout,
                                                         uint32_t *__restrict__ vout)
{
    constexpr int WARPS = SORT_THREADS / 32;
    __shared__ uint32_t wc[WARPS][RADIX];
    int t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t run = hist[(size_t)t * gridDim.x + blockIdx.x];  // thread t owns digit t
    unsigned lt = (1u << lane) - 1u;
    int base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; r++) {
        for (int k = 0; k < WARPS; k++) wc[k][t] = 0;
        __syncthreads();
        int q = base + r * SORT_THREADS + t;
        bool valid = q < n;
        unsigned long long key = valid ? kin[q] : 0ull;
        uint32_t val = valid ? vin[q] : 0u;
        int d = valid ? (int)((key >> shift) & (RADIX - 1)) : RADIX;  // invalid lanes form their own group
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lt);
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) wc[w][d] = __popc(peers);
        __syncthreads();
        // Per digit: exclusive prefix over warps, continuing from earlier rounds.
        for (int k = 0; k < WARPS; k++) {
            uint32_t c = wc[k][t];
            wc[k][t] = run;
            run += c;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = wc[w][d] + rank;
            STEPS_CHECK_IDX(pos, n, CK_SCATTER);
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

constexpr int TB_THREADS = 256;

// One block per tile of T particles in curve order. Without descriptors the
// tiles cut one sorted set; with them (batches) every tile names its own
// start and count.
__global__ void __launch_bounds__(TB_THREADS) k_tile_build(const double *__restrict__ x, const double *__restrict__ m,
                                                          const double *__restrict__ eps,
                                                          const uint32_t *__restrict__ perm, long long nx,
                                                          int count, int T,
                                                          float4 *__restrict__ pack, float *__restrict__ epsf,
                                                          float4 *__restrict__ meta, uint32_t *__restrict__ idx,
                                                          uint32_t pad_id, float4 *__restrict__ lo,
                                                          float *__restrict__ soa, const int2 *__restrict__ tdesc,
                                                          float4 *__restrict__ sub)
{
    const int tile = blockIdx.x;
    const int sbase = tdesc ? tdesc[tile].x : tile * T;
    int cnt = tdesc ? tdesc[tile].y : min(T, count - tile * T);
#ifdef STEPS_CHECK
    if (!check_span(sbase, (long long)sbase + cnt - 1, count, CK_PERM)) cnt = 0;
#endif
    build_tile<TB_THREADS, false>(tile, sbase, cnt, x, m, eps, perm, nx, T, pack, epsf, meta, idx, pad_id, lo, soa,
                                  sub);
}

}  // namespace

// Leading Morton bits that order a set of n particles into compact tiles:
// 2^(bits/3) cells per axis, at least 2^5 times the mean particle spacing,
// so clustered sets still see about one particle per cell in dense regions.
// Bits below are left in input order (the sort is stable).
int morton_sort_bits(int n)
{
    int lg = 0;
    while ((1LL << lg) < (long long)n) lg++;
    const int bits = 3 * ((lg + 2) / 3 + 5);
    return bits < 63 ? bits : 63;
}

void sort_pairs(TileSet &ts, int n, cudaStream_t st, int lo_bit)
{
    int nblk = div_up(n, SORT_TILE);
    uint32_t *hist = ts.hist.ensure<uint32_t>((size_t)RADIX * (nblk > 0 ? nblk : 1));
    int cur = 0;
    for (int shift = lo_bit / RADIX_BITS * RADIX_BITS; shift < 64; shift += RADIX_BITS) {
        k_hist<<<nblk, SORT_THREADS, 0, st>>>(ts.keys[cur].as<unsigned long long>(), n, shift, hist);
        note_launch("k_hist");
        k_scan<<<1, 1024, 0, st>>>(hist, RADIX * nblk);
        note_launch("k_scan");
        k_scatter<<<nblk, SORT_THREADS, 0, st>>>(ts.keys[cur].as<unsigned long long>(), ts.vals[cur].as<uint32_t>(), n,
                                                 shift, hist, ts.keys[cur ^ 1].as<unsigned long long>(),
                                                 ts.vals[cur ^ 1].as<uint32_t>());
        note_launch("k_scatter");
        cur ^= 1;
    }
    ts.perm_sel = cur;
}

// Orders particles [lo, lo+count) of the AoS FP64 array x along a Morton curve
// (unless reuse is set and an order already exists) and (re)builds the tiles.
void build_tiles(TileSet &ts, const double *x, const double *m64, const double *eps64, int lo, int count, int T,
                 bool reuse, cudaStream_t st, unsigned long long *bbox_scratch, uint32_t pad_id)
{
    if (count <= 0) fail(STEPS_E_ARG, "empty particle set");
    bool same = ts.ordered && ts.lo == lo && ts.count == count;
    ts.T = T;
    ts.ntiles = div_up(count, T);
    size_t padded = (size_t)ts.ntiles * T;
    if (!(reuse && same)) {
        for (int b = 0; b < 2; b++) {
            ts.keys[b].ensure<unsigned long long>(count);
            ts.vals[b].ensure<uint32_t>(count);
        }
        k_bbox_init<<<1, 32, 0, st>>>(bbox_scratch);
        note_launch("k_bbox_init");
        int g = div_up(count, 256);
        k_bbox<<<g < 1024 ? g : 1024, 256, 0, st>>>(x, lo, count, bbox_scratch);
        note_launch("k_bbox");
        k_keys<<<div_up(count, 256), 256, 0, st>>>(x, lo, count, bbox_scratch, 21, 0ull, ts.keys[0].as<unsigned long long>(),
                                                  ts.vals[0].as<uint32_t>());
        note_launch("k_keys");
        sort_pairs(ts, count, st, 63 - morton_sort_bits(count));
        ts.lo = lo;
        ts.count = count;
        ts.ordered = true;
    }
    ts.pack.ensure<float4>(padded);
    ts.eps.ensure<float>(padded);
    ts.meta.ensure<float4>(2 * (size_t)ts.ntiles);
    ts.idx.ensure<uint32_t>(padded);
    ts.resid.ensure<float4>(padded);
    ts.soa.ensure<float4>(padded);
    ts.sub.ensure<float4>(2 * (padded / SUBTILE));
    k_tile_build<<<ts.ntiles, TB_THREADS, 0, st>>>(x, m64, eps64, ts.perm(), (long long)lo + count, count, T,
                                                   ts.pack.as<float4>(),
                                                   ts.eps.as<float>(), ts.meta.as<float4>(), ts.idx.as<uint32_t>(),
                                                   pad_id, ts.resid.as<float4>(), ts.soa.as<float>(), nullptr,
                                                   ts.sub.as<float4>());
    note_launch("k_tile_build");
}

// Batched variant: keys carry the realisation index above the Morton bits, so
// one sort orders every realisation's particles contiguously by realisation.
void batch_keys(const double *x, int lo, int count, unsigned long long prefix, unsigned long long *keys, uint32_t *vals,
                unsigned long long *bbox_scratch, cudaStream_t st)
{
    k_bbox_init<<<1, 32, 0, st>>>(bbox_scratch);
    note_launch("k_bbox_init");
    int g = div_up(count, 256);
    k_bbox<<<g < 1024 ? g : 1024, 256, 0, st>>>(x, lo, count, bbox_scratch);
    note_launch("k_bbox");
    k_keys<<<div_up(count, 256), 256, 0, st>>>(x, lo, count, bbox_scratch, 19, prefix, keys, vals);
    note_launch("k_keys");
}

void tile_build_range(const double *x, const double *m64, const double *eps64, const uint32_t *perm, int count, int T,
                      float4 *pack, float *epsf, float4 *meta, uint32_t *idx, uint32_t pad_id, float4 *lo, float *soa,
                      const int2 *tdesc, int ntiles, cudaStream_t st, float4 *sub)
{
    int nt = tdesc ? ntiles : div_up(count, T);
    k_tile_build<<<nt, TB_THREADS, 0, st>>>(x, m64, eps64, perm, count, count, T, pack, epsf, meta, idx, pad_id, lo,
                                            soa, tdesc, sub);
    note_launch("k_tile_build");
}

}  // namespace steps
