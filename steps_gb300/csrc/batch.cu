// Batched ensembles: many independent compactified R^3 realisations of uneven
// N, advanced together (one force evaluation + fixed-dt KDK steps).
//
// Layout: all realisations' particles are concatenated (positions,
// velocities, forces in caller order, realisation k at offset off[k]). One
// radix sort orders every particle by (realisation, Morton key in that
// realisation's own box), so each realisation occupies a contiguous range of
// the sorted order; tiles never straddle two realisations (each realisation
// is padded to a whole number of tiles).
//
// Work: a host-built list of items (i tile, j tile range, partial slot)
// covering, for every realisation, its i tiles x j chunks; ordered by
// realisation size, largest first, so the persistent kernel's atomic queue
// schedules longest-processing-time first. The pair kernel is the packed
// FP32x2 R^3 kernel in work-list mode; partial sums go to per-item slots and
// a reduction adds each i tile's slots in order (deterministic).
//
// graph = 1: the whole run in ONE persistent kernel (k_ensemble, pair_r3x2.cu)
// after a single ordering pass, captured into a CUDA graph and replayed:
// (stage, item) tasks from one queue, a bounded wait per task on its
// realisation's previous stage, the kicks, drift and tile rebuild done by the
// block that finishes each tile. The tile shape, the j-chunk length and the
// grid size are chosen by timing candidates first.
// graph = 2: the same run as a CUDA graph of per-phase kernels (per step:
// kick+drift, re-order, re-tile, work-list force, reduction, kick).
// graph = 0: the same work as `count` separate single-realisation force calls
// (and KDK kernels) per phase, for comparison.
#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "mixed.cuh"

namespace steps {

struct Batch {
    int count = 0;
    std::vector<int> n, off;  // particles and their offset per realisation
    int ntot = 0;
    DevBuf x, v, F, m64, eps64;
    DevBuf rel;                   // uint16 realisation of each particle (caller order)
    DevBuf bbox;                  // 6 ordered-bit u64 per realisation
    TileSet ts;                   // sort buffers + tile arrays over the padded batch
    DevBuf tdesc;                 // int2 per tile: sorted start, count
    DevBuf items;                 // int4 work list
    DevBuf tslot;                 // int2 per tile: first partial slot, number of slots
    DevBuf part, counter, err;
    int T = 0, ntiles = 0, nitems = 0, threads = 0, ipt = 0, grid = 0;
    int jmax = 256;  // j tiles per work item at most
    long long graph_kernels = 0;
    int nmax = 0;  // largest realisation
    bool tuned = false;     // per-phase graph shape
    bool ens_tuned = false; // persistent kernel shape, j-chunk length, grid
    int threads_pp = 128, ipt_pp = 2;  // per-phase graph shape
    int ens_threads = 128, ens_ipt = 2, ens_jmax = 256, ens_grid = 0;
    double ens_frac = 1.0;
    // persistent path: the second tile buffer, per-tile realisation, counters
    DevBuf pack2, soa2, resid2, meta2, sub2;
    DevBuf tile_rel, rel_ntiles, ens_ctl;
    int stall_rel = -1;  // test hook for the next persistent run (one shot)
    cudaGraphExec_t exec = nullptr;
    int graph_steps = -1, graph_mode = 0;
    double graph_h = 0.0;
};

namespace {

__global__ void k_batch_bbox(const double *__restrict__ x, const uint16_t *__restrict__ rel, int n,
                             unsigned long long *bb)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = rel[i];
        for (int c = 0; c < 3; c++) {
            const double v = x[3 * (size_t)i + c];
            atomicMin(&bb[6 * k + c], ordered_bits(v));
            atomicMax(&bb[6 * k + 3 + c], ordered_bits(v));
        }
    }
}

__global__ void k_batch_bbox_init(unsigned long long *bb, int count)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 6 * count) bb[t] = (t % 6) < 3 ? ~0ull : 0ull;
}

// Key = realisation index (13 bits) above a 51-bit Morton key (17 bits per
// axis) of the particle's position in its realisation's own bounding box.
__global__ void k_batch_keys(const double *__restrict__ x, const uint16_t *__restrict__ rel, int n,
                             const unsigned long long *__restrict__ bb, unsigned long long *keys, uint32_t *vals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = rel[i];
    const double cells = (double)(1u << 17);
    unsigned long long key = 0;
    for (int c = 0; c < 3; c++) {
        const double lo = from_ordered_bits(bb[6 * k + c]), hi = from_ordered_bits(bb[6 * k + 3 + c]);
        const double span = hi - lo;
        const double u = span > 0 ? (x[3 * (size_t)i + c] - lo) / span * cells : 0.0;
        long long q = (long long)u;
        q = q < 0 ? 0 : (q >= (long long)cells ? (long long)cells - 1 : q);
        key |= spread3((unsigned long long)q) << c;
    }
    keys[i] = key | ((unsigned long long)k << 51);
    vals[i] = (uint32_t)i;
}

// Sum each i's slots in order and scatter to caller order.
__global__ void k_batch_reduce(const double *__restrict__ part, const int2 *__restrict__ tslot,
                               const uint32_t *__restrict__ idx, int npad, int T, int n, int nslots,
                               double *__restrict__ F)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npad) return;
    uint32_t o = idx[q];
    if (o == PAD_J) return;
    STEPS_CHECK_IDX(o, n, CK_OUTPUT);
    const int t = q / T, e = q - t * T;
    const int2 s = tslot[t];
    double f[3] = {0, 0, 0};
    for (int k = 0; k < s.y; k++) {
        int slot = s.x + k;
        STEPS_CHECK_IDX(slot, nslots, CK_SLOT);
        for (int c = 0; c < 3; c++) f[c] += part[((size_t)slot * T + e) * 3 + c];
    }
    for (int c = 0; c < 3; c++) F[3 * (size_t)o + c] = f[c];
}

// Tile descriptors and the work list for tile size T (host side, once per shape).
void plan(Batch &b, int threads, int ipt, int jmax = 256)
{
    Ctx &c = ctx();
    const int T = threads * ipt;
    b.jmax = jmax;
    std::vector<int> tstart(b.count), nt(b.count);
    std::vector<int2> desc;
    for (int k = 0; k < b.count; k++) {
        nt[k] = div_up(b.n[k], T);
        tstart[k] = (int)desc.size();
        for (int t = 0; t < nt[k]; t++) desc.push_back(make_int2(b.off[k] + t * T, std::min(T, b.n[k] - t * T)));
    }
    b.ntiles = (int)desc.size();
    // Items: per realisation i tiles x j chunks of at most jmax tiles; largest realisations first.
    std::vector<int> order(b.count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int d) { return b.n[a] > b.n[d]; });
    std::vector<int4> items;
    std::vector<int2> tslot(b.ntiles);
    std::vector<int> trel(b.ntiles);
    for (int k = 0; k < b.count; k++)
        for (int t = 0; t < nt[k]; t++) trel[tstart[k] + t] = k;
    for (int k : order) {
        const int S = div_up(nt[k], jmax);
        const int per = div_up(nt[k], S);
        for (int I = 0; I < nt[k]; I++) {
            const int gI = tstart[k] + I;
            tslot[gI] = make_int2((int)items.size(), 0);
            for (int s = 0; s < S; s++) {
                const int J0 = tstart[k] + s * per, J1 = std::min(tstart[k] + nt[k], J0 + per);
                if (J0 >= J1) continue;
                items.push_back(make_int4(gI, J0, J1, (int)items.size()));
                tslot[gI].y++;
            }
        }
    }
    b.nitems = (int)items.size();
    const size_t padded = (size_t)b.ntiles * T;
    STEPS_CUDA(cudaMemcpyAsync(b.tdesc.ensure<int2>(desc.size()), desc.data(), desc.size() * sizeof(int2),
                               cudaMemcpyHostToDevice, c.stream));
    STEPS_CUDA(cudaMemcpyAsync(b.items.ensure<int4>(items.size()), items.data(), items.size() * sizeof(int4),
                               cudaMemcpyHostToDevice, c.stream));
    STEPS_CUDA(cudaMemcpyAsync(b.tslot.ensure<int2>(tslot.size()), tslot.data(), tslot.size() * sizeof(int2),
                               cudaMemcpyHostToDevice, c.stream));
    STEPS_CUDA(cudaMemcpyAsync(b.tile_rel.ensure<int>(trel.size()), trel.data(), trel.size() * sizeof(int),
                               cudaMemcpyHostToDevice, c.stream));
    STEPS_CUDA(cudaMemcpyAsync(b.rel_ntiles.ensure<int>(nt.size()), nt.data(), nt.size() * sizeof(int),
                               cudaMemcpyHostToDevice, c.stream));
    b.ts.pack.ensure<float4>(padded);
    b.ts.eps.ensure<float>(padded);
    b.ts.meta.ensure<float4>(2 * (size_t)b.ntiles);
    b.ts.idx.ensure<uint32_t>(padded);
    b.ts.resid.ensure<float4>(padded);
    b.ts.soa.ensure<float4>(padded);
    b.ts.sub.ensure<float4>(2 * (padded / SUBTILE));
    b.pack2.ensure<float4>(padded);
    b.soa2.ensure<float4>(padded);
    b.resid2.ensure<float4>(padded);
    b.meta2.ensure<float4>(2 * (size_t)b.ntiles);
    b.sub2.ensure<float4>(2 * (padded / SUBTILE));
    b.ens_ctl.ensure<unsigned>(1 + (size_t)b.ntiles + b.count);
    b.part.ensure<double>((size_t)b.nitems * T * 3);
    b.T = T;
    b.threads = threads;
    b.ipt = ipt;
    mixed::KernelFn fn = r3x2_kernel(threads, ipt, true);
    if (!fn) fail(STEPS_E_ARG, "batch: unsupported kernel shape");
    int occ = 0;
    STEPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, 0));
    b.grid = std::min(c.nsm * std::max(occ, 1), b.nitems);
    STEPS_CUDA(cudaStreamSynchronize(c.stream));
}

// Orders every realisation (one sort) and builds the tiles into the first
// tile buffer (and, for the persistent kernel, the second one as well).
void batch_order(Batch &b, bool both_buffers)
{
    Ctx &c = ctx();
    cudaStream_t st = c.stream;
    unsigned long long *bb = b.bbox.as<unsigned long long>();
    k_batch_bbox_init<<<div_up(6 * b.count, 256), 256, 0, st>>>(bb, b.count);
    note_launch("k_batch_bbox_init");
    k_batch_bbox<<<std::min(div_up(b.ntot, 256), 4 * c.nsm * 8), 256, 0, st>>>(b.x.as<double>(), b.rel.as<uint16_t>(),
                                                                            b.ntot, bb);
    note_launch("k_batch_bbox");
    k_batch_keys<<<div_up(b.ntot, 256), 256, 0, st>>>(b.x.as<double>(), b.rel.as<uint16_t>(), b.ntot, bb,
                                                      b.ts.keys[0].as<unsigned long long>(),
                                                      b.ts.vals[0].as<uint32_t>());
    note_launch("k_batch_keys");
    // realisation bits [51, 64) and the leading Morton bits the largest realisation needs
    sort_pairs(b.ts, b.ntot, st, std::max(0, 51 - std::min(51, morton_sort_bits(b.nmax))));
    tile_build_range(b.x.as<double>(), b.m64.as<double>(), b.eps64.as<double>(), b.ts.perm(), b.ntot, b.T,
                     b.ts.pack.as<float4>(), b.ts.eps.as<float>(), b.ts.meta.as<float4>(), b.ts.idx.as<uint32_t>(),
                     PAD_J, b.ts.resid.as<float4>(), b.ts.soa.as<float>(), b.tdesc.as<int2>(), b.ntiles, st,
                     b.ts.sub.as<float4>());
    if (both_buffers)
        tile_build_range(b.x.as<double>(), b.m64.as<double>(), b.eps64.as<double>(), b.ts.perm(), b.ntot, b.T,
                         b.pack2.as<float4>(), b.ts.eps.as<float>(), b.meta2.as<float4>(), nullptr, PAD_J,
                         b.resid2.as<float4>(), b.soa2.as<float>(), b.tdesc.as<int2>(), b.ntiles, st,
                         b.sub2.as<float4>());
}

// One batched force evaluation on the resident positions (stream-ordered; no
// host synchronisation, so it can be captured into a graph).
void batch_forces(Batch &b)
{
    Ctx &c = ctx();
    cudaStream_t st = c.stream;
    batch_order(b, false);

    mixed::MixedArgs a{};
    a.stall_seq = -1;
    a.istride = 1;
    a.jpack = a.ipack = b.ts.pack.as<float4>();
    a.jeps = a.ieps = b.ts.eps.as<float>();
    a.jmeta = a.imeta = b.ts.meta.as<float4>();
    a.jidx = a.iidx = b.ts.idx.as<uint32_t>();
    a.jres = a.ilo = b.ts.resid.as<float4>();
    a.jsoa = b.ts.soa.as<float>();
    a.jsub = b.ts.sub.as<float4>();
    a.njt = a.nit = b.ntiles;
    a.nitems = b.nitems;
    a.items = b.items.as<int4>();
    a.nslots = b.nitems;
    a.counter = b.counter.as<unsigned>();
    a.part = b.part.as<double>();
    a.guard2 = c.shape.guard * c.shape.guard;
    mixed::KernelFn fn = r3x2_kernel(b.threads, b.ipt, true);
    STEPS_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st));
    fn<<<b.grid, b.threads, 0, st>>>(a);
    note_launch("k_pair_r3x2(list)");
    k_batch_reduce<<<div_up(b.ntiles * b.T, 256), 256, 0, st>>>(b.part.as<double>(), b.tslot.as<int2>(),
                                                                b.ts.idx.as<uint32_t>(), b.ntiles * b.T, b.T, b.ntot,
                                                                b.nitems, b.F.as<double>());
    note_launch("k_batch_reduce");
}

// The whole run in one persistent kernel (stream-ordered, capturable): one
// ordering pass that builds both tile buffers, the counters zeroed, then
// k_ensemble over nsteps + 1 stages.
void ensemble_run(Batch &b, int nsteps, double h, int stall_rel)
{
    Ctx &c = ctx();
    cudaStream_t st = c.stream;
    batch_order(b, true);
    unsigned *ctl = b.ens_ctl.as<unsigned>();
    STEPS_CUDA(cudaMemsetAsync(ctl, 0, sizeof(unsigned) * (1 + (size_t)b.ntiles + b.count), st));
    mixed::EnsembleArgs e{};
    float4 *pk[2] = {b.ts.pack.as<float4>(), b.pack2.as<float4>()};
    float *so[2] = {b.ts.soa.as<float>(), b.soa2.as<float>()};
    float4 *re[2] = {b.ts.resid.as<float4>(), b.resid2.as<float4>()};
    float4 *me[2] = {b.ts.meta.as<float4>(), b.meta2.as<float4>()};
    float4 *su[2] = {b.ts.sub.as<float4>(), b.sub2.as<float4>()};
    for (int k = 0; k < 2; k++) {
        e.pack[k] = e.pack_w[k] = pk[k];
        e.soa[k] = e.soa_w[k] = so[k];
        e.resid[k] = e.resid_w[k] = re[k];
        e.meta[k] = e.meta_w[k] = me[k];
        e.sub[k] = e.sub_w[k] = su[k];
    }
    e.jeps = b.ts.eps.as<float>();
    e.epsf_w = b.ts.eps.as<float>();
    e.jidx = b.ts.idx.as<uint32_t>();
    e.items = b.items.as<int4>();
    e.nitems = b.nitems;
    e.nstages = nsteps + 1;
    e.tile_rel = b.tile_rel.as<int>();
    e.tdesc = b.tdesc.as<int2>();
    e.tslot = b.tslot.as<int2>();
    e.rel_ntiles = b.rel_ntiles.as<int>();
    e.perm = b.ts.perm();
    e.part = b.part.as<double>();
    e.queue = ctl;
    e.tile_cnt = ctl + 1;
    e.rel_done = ctl + 1 + b.ntiles;
    e.x = b.x.as<double>();
    e.v = b.v.as<double>();
    e.F = b.F.as<double>();
    e.m64 = b.m64.as<double>();
    e.eps64 = b.eps64.as<double>();
    e.h = h;
    e.guard2 = c.shape.guard * c.shape.guard;
    e.status = kernel_status_word();
    e.stall_rel = stall_rel;
    e.ntiles = b.ntiles;
    e.nslots = b.nitems;
    e.nrel = b.count;
    e.n = b.ntot;
    mixed::EnsembleFn fn = ensemble_kernel(b.threads, b.ipt);
    if (!fn) fail(STEPS_E_ARG, "batch: unsupported kernel shape");
    fn<<<b.ens_grid, b.threads, 0, st>>>(e);
    note_launch("k_ensemble");
    c.status_pending = true;
}

// Plans the work list for the persistent kernel's shape and sizes its grid:
// `frac` of the blocks that fit on the GPU at once.
void ensemble_plan(Batch &b, int threads, int ipt, int jmax, double frac)
{
    Ctx &c = ctx();
    plan(b, threads, ipt, jmax);
    mixed::EnsembleFn fn = ensemble_kernel(threads, ipt);
    if (!fn) fail(STEPS_E_ARG, "batch: unsupported kernel shape");
    int occ = 0;
    STEPS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, 0));
    const int resident = c.nsm * std::max(occ, 1);
    b.ens_grid = std::max(1, std::min(b.nitems, (int)(frac * resident)));
}

// Times one force evaluation (a one-stage run) per candidate tile shape,
// j-chunk length and grid size, and keeps the fastest.
void ensemble_tune(Batch &b)
{
    Ctx &c = ctx();
    static const int shapes[][2] = {{128, 2}, {128, 1}, {256, 1}, {64, 2}};
    static const int jmaxes[] = {64, 256};
    static const double fracs[] = {1.0, 0.75};
    float best = 1e30f;
    int bt = 128, bi = 2, bj = 256;
    double bf = 1.0;
    for (auto &sh : shapes)
        for (int jm : jmaxes)
            for (double fr : fracs) {
                ensemble_plan(b, sh[0], sh[1], jm, fr);
                ensemble_run(b, 0, 0.0, -1);  // warm
                STEPS_CUDA(cudaEventRecord(c.marks[12], c.stream));
                ensemble_run(b, 0, 0.0, -1);
                STEPS_CUDA(cudaEventRecord(c.marks[13], c.stream));
                STEPS_CUDA(cudaEventSynchronize(c.marks[13]));
                float ms = 0;
                STEPS_CUDA(cudaEventElapsedTime(&ms, c.marks[12], c.marks[13]));
                if (ms < best) { best = ms; bt = sh[0]; bi = sh[1]; bj = jm; bf = fr; }
            }
    check_kernel_status();
    ensemble_plan(b, bt, bi, bj, bf);
    b.ens_threads = bt;
    b.ens_ipt = bi;
    b.ens_jmax = bj;
    b.ens_frac = bf;
    b.ens_tuned = true;
}

void batch_steps(Batch &b, int nsteps, double h)
{
    Ctx &c = ctx();
    batch_forces(b);
    for (int s = 0; s < nsteps; s++) {
        kdk_kick_drift(b.x.as<double>(), b.v.as<double>(), b.F.as<double>(), b.ntot, h, 1.0, 1.0, 0.0, 0, 0.0,
                       c.stream);
        batch_forces(b);
        kdk_kick_err(b.v.as<double>(), b.F.as<double>(), b.m64.as<double>(), b.ntot, h, 1.0, 1.0, 0.0, 1.0,
                     b.err.as<double>(), c.stream, false);
    }
}

// Per-realisation path: the same work as `count` separate force calls.
void plain_steps(Batch &b, const KParams &kp, int precision, int nsteps, double h)
{
    Ctx &c = ctx();
    Tables tb{};
    auto force = [&](int k) {
        const size_t o = (size_t)b.off[k];
        double *x = b.x.as<double>() + 3 * o, *F = b.F.as<double>() + 3 * o;
        const double *m = b.m64.as<double>() + o, *e = b.eps64.as<double>() + o;
        if (precision == STEPS_FP64) fail(STEPS_E_ARG, "batch: FP64 ensembles are not supported");
        forces_mixed(kp, tb, x, m, e, b.n[k], 0, b.n[k], F, false);
    };
    for (int k = 0; k < b.count; k++) force(k);
    for (int s = 0; s < nsteps; s++) {
        for (int k = 0; k < b.count; k++) {
            const size_t o = (size_t)b.off[k];
            kdk_kick_drift(b.x.as<double>() + 3 * o, b.v.as<double>() + 3 * o, b.F.as<double>() + 3 * o, b.n[k], h,
                           1.0, 1.0, 0.0, 0, 0.0, c.stream);
            force(k);
            kdk_kick_err(b.v.as<double>() + 3 * o, b.F.as<double>() + 3 * o, b.m64.as<double>() + o, b.n[k], h, 1.0,
                         1.0, 0.0, 1.0, b.err.as<double>(), c.stream, false);
        }
    }
}

// Kernel nodes of a captured graph (what one launch of it runs).
long long count_kernel_nodes(cudaGraph_t g)
{
    size_t n = 0;
    STEPS_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) STEPS_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    long long k = 0;
    for (size_t i = 0; i < n; i++) {
        cudaGraphNodeType t;
        STEPS_CUDA(cudaGraphNodeGetType(nodes[i], &t));
        k += t == cudaGraphNodeTypeKernel;
    }
    return k;
}

void release_graph(Batch &b)
{
    if (b.exec) cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
    b.graph_steps = -1;
}

}  // namespace

void batch_release()
{
    Ctx &c = ctx();
    Batch *b = c.batch;
    if (!b) return;
    release_graph(*b);
    DevBuf *bufs[] = {&b->x, &b->v, &b->F, &b->m64, &b->eps64, &b->rel, &b->bbox, &b->tdesc, &b->items, &b->tslot,
                      &b->part, &b->counter, &b->err, &b->ts.keys[0], &b->ts.keys[1], &b->ts.vals[0], &b->ts.vals[1],
                      &b->ts.hist, &b->ts.pack, &b->ts.eps, &b->ts.meta, &b->ts.idx, &b->ts.resid, &b->ts.soa,
                      &b->ts.sub, &b->pack2, &b->soa2, &b->resid2, &b->meta2, &b->sub2, &b->tile_rel,
                      &b->rel_ntiles, &b->ens_ctl};
    for (DevBuf *d : bufs) d->release();
    delete b;
    c.batch = nullptr;
}

}  // namespace steps

using namespace steps;

extern "C" {

int steps_gpu_batch_set(int count, const int *n, const double *const *x, const double *const *m,
                        const double *const *eps)
{
    struct A {
        int count;
        const int *n;
        const double *const *x, *const *m, *const *eps;
    } args{count, n, x, m, eps};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            require_init();
            Ctx &c = ctx();
            if (a.count < 1 || a.count > 8191 || !a.n || !a.x || !a.m || !a.eps)
                fail(STEPS_E_ARG, "batch_set: count in [1, 8191] and non-NULL arrays required");
            long long tot = 0;
            for (int k = 0; k < a.count; k++) {
                if (a.n[k] < 1 || !a.x[k] || !a.m[k] || !a.eps[k]) fail(STEPS_E_ARG, "batch_set: empty realisation");
                tot += a.n[k];
            }
            if (tot > (1LL << 30)) fail(STEPS_E_ARG, "batch_set: too many particles");
            // The same realisation sizes as the registered batch: keep its
            // buffers, tuned tile shape and captured graph, replace the data.
            const bool same = c.batch && c.batch->count == a.count &&
                              std::equal(c.batch->n.begin(), c.batch->n.end(), a.n);
            if (!same) {
                batch_release();
                c.batch = new Batch();
                Batch &b = *c.batch;
                b.count = a.count;
                b.n.assign(a.n, a.n + a.count);
                b.off.resize(a.count);
                int o = 0;
                for (int k = 0; k < a.count; k++) { b.off[k] = o; o += a.n[k]; }
                b.ntot = o;
                b.nmax = *std::max_element(b.n.begin(), b.n.end());
                std::vector<uint16_t> rel(b.ntot);
                for (int k = 0; k < a.count; k++) std::fill(rel.begin() + b.off[k], rel.begin() + b.off[k] + b.n[k], k);
                b.x.ensure<double>(3 * (size_t)b.ntot);
                b.m64.ensure<double>(b.ntot);
                b.eps64.ensure<double>(b.ntot);
                b.F.ensure<double>(3 * (size_t)b.ntot);
                b.v.ensure<double>(3 * (size_t)b.ntot);
                STEPS_CUDA(cudaMemcpyAsync(b.rel.ensure<uint16_t>(b.ntot), rel.data(), sizeof(uint16_t) * b.ntot,
                                           cudaMemcpyHostToDevice, c.stream));
                b.bbox.ensure<unsigned long long>(6 * (size_t)a.count);
                for (int k = 0; k < 2; k++) {
                    b.ts.keys[k].ensure<unsigned long long>(b.ntot);
                    b.ts.vals[k].ensure<uint32_t>(b.ntot);
                }
                b.counter.ensure<unsigned>(4);
                b.err.ensure<double>(4);
                STEPS_CUDA(cudaStreamSynchronize(c.stream));  // rel's host copy goes out of scope
            }
            Batch &b = *c.batch;
            double *dx = b.x.as<double>(), *dm = b.m64.as<double>(), *de = b.eps64.as<double>();
            for (int k = 0; k < a.count; k++) {
                const size_t off = (size_t)b.off[k];
                STEPS_CUDA(cudaMemcpyAsync(dx + 3 * off, a.x[k], 3 * sizeof(double) * a.n[k], cudaMemcpyHostToDevice,
                                           c.stream));
                STEPS_CUDA(cudaMemcpyAsync(dm + off, a.m[k], sizeof(double) * a.n[k], cudaMemcpyHostToDevice,
                                           c.stream));
                STEPS_CUDA(cudaMemcpyAsync(de + off, a.eps[k], sizeof(double) * a.n[k], cudaMemcpyHostToDevice,
                                           c.stream));
            }
            STEPS_CUDA(cudaMemsetAsync(b.v.as<double>(), 0, 3 * sizeof(double) * b.ntot, c.stream));
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
        },
        &args);
}

int steps_gpu_batch_run(const steps_params *p, int precision, int nsteps, double h, int graph)
{
    struct A {
        const steps_params *p;
        int precision, nsteps;
        double h;
        int graph;
    } args{p, precision, nsteps, h, graph};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            require_init();
            Ctx &c = ctx();
            Batch *bp = c.batch;
            if (!bp) fail(STEPS_E_STATE, "no batch: call steps_gpu_batch_set first");
            Batch &b = *bp;
            KParams kp = derive_params(a.p);
            if (kp.topology != STEPS_R3 || kp.comoving_bg != 0)
                fail(STEPS_E_ARG, "batch: non-cosmological R^3 realisations only");
            if (a.nsteps < 0) fail(STEPS_E_ARG, "batch: nsteps must be >= 0");
            if (!a.graph) {
                plain_steps(b, kp, a.precision, a.nsteps, a.h);
                STEPS_CUDA(cudaStreamSynchronize(c.stream));
                return;
            }
            if (a.precision != STEPS_MIXED) fail(STEPS_E_ARG, "batch graph: mixed precision only");
            if (a.graph != 1 && a.graph != 2) fail(STEPS_E_ARG, "batch: graph must be 0, 1 or 2");
            const bool persistent = a.graph == 1;
            if (persistent && b.stall_rel >= 0) {
                // the test hook: one direct (uncaptured) run with the stall
                const int k = b.stall_rel;
                b.stall_rel = -1;
                if (!b.ens_tuned) ensemble_tune(b);
                else ensemble_plan(b, b.ens_threads, b.ens_ipt, b.ens_jmax, b.ens_frac);
                release_graph(b);
                ensemble_run(b, a.nsteps, a.h, k);
                STEPS_CUDA(cudaStreamSynchronize(c.stream));
                check_kernel_status();
                return;
            }
            if (persistent && !b.ens_tuned) {
                ensemble_tune(b);
                release_graph(b);
            }
            if (!persistent && !b.tuned) {
                // Time one batched force per candidate shape, keep the fastest.
                static const int shapes[][2] = {{128, 2}, {64, 4}, {128, 1}, {256, 1}, {128, 4}, {256, 2}};
                float best = 1e30f;
                int bt = 128, bi = 2;
                for (auto &s : shapes) {
                    plan(b, s[0], s[1]);
                    batch_forces(b);  // warm
                    STEPS_CUDA(cudaEventRecord(c.marks[12], c.stream));
                    batch_forces(b);
                    STEPS_CUDA(cudaEventRecord(c.marks[13], c.stream));
                    STEPS_CUDA(cudaEventSynchronize(c.marks[13]));
                    float ms = 0;
                    STEPS_CUDA(cudaEventElapsedTime(&ms, c.marks[12], c.marks[13]));
                    if (ms < best) { best = ms; bt = s[0]; bi = s[1]; }
                }
                plan(b, bt, bi);
                b.threads_pp = bt;
                b.ipt_pp = bi;
                b.tuned = true;
                release_graph(b);
            }
            if (!b.exec || b.graph_steps != a.nsteps || b.graph_h != a.h || b.graph_mode != a.graph) {
                release_graph(b);
                // the plan of the chosen path (the two paths keep their own shapes)
                if (persistent) ensemble_plan(b, b.ens_threads, b.ens_ipt, b.ens_jmax, b.ens_frac);
                else plan(b, b.threads_pp, b.ipt_pp);
                if (!persistent) batch_forces(b);  // sizes every buffer before capture
                kernel_status_word();              // allocated outside the capture
                STEPS_CUDA(cudaStreamSynchronize(c.stream));
                cudaGraph_t g;
                STEPS_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
                try {
                    if (persistent) ensemble_run(b, a.nsteps, a.h, -1);
                    else batch_steps(b, a.nsteps, a.h);
                } catch (...) {
                    cudaGraph_t dummy;
                    cudaStreamEndCapture(c.stream, &dummy);
                    if (dummy) cudaGraphDestroy(dummy);
                    throw;
                }
                STEPS_CUDA(cudaStreamEndCapture(c.stream, &g));
                b.graph_kernels = count_kernel_nodes(g);
                cudaError_t e = cudaGraphInstantiate(&b.exec, g, 0);
                cudaGraphDestroy(g);
                STEPS_CUDA(e);
                b.graph_steps = a.nsteps;
                b.graph_h = a.h;
                b.graph_mode = a.graph;
            }
            STEPS_CUDA(cudaGraphLaunch(b.exec, c.stream));
            add_launches(b.graph_kernels);  // the kernels the graph runs
            if (persistent) c.status_pending = true;
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
            check_kernel_status();
        },
        &args);
}

int steps_gpu_test_stall_ensemble(int realisation)
{
    return run_guarded(
        [](void *vp) {
            const int k = *static_cast<int *>(vp);
            Batch *b = ctx().batch;
            if (!b) fail(STEPS_E_STATE, "no batch: call steps_gpu_batch_set first");
            if (k < -1 || k >= b->count) fail(STEPS_E_ARG, "test_stall_ensemble: no such realisation");
            b->stall_rel = k;
        },
        &realisation);
}

int steps_gpu_batch_get(int k, double *x, double *v, double *F)
{
    struct A {
        int k;
        double *x, *v, *F;
    } args{k, x, v, F};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            require_init();
            Ctx &c = ctx();
            Batch *b = c.batch;
            if (!b) fail(STEPS_E_STATE, "no batch: call steps_gpu_batch_set first");
            if (a.k < 0 || a.k >= b->count) fail(STEPS_E_ARG, "batch_get: no such realisation");
            const size_t o = 3 * (size_t)b->off[a.k], bytes = 3 * sizeof(double) * b->n[a.k];
            if (a.x) STEPS_CUDA(cudaMemcpyAsync(a.x, b->x.as<double>() + o, bytes, cudaMemcpyDeviceToHost, c.stream));
            if (a.v) STEPS_CUDA(cudaMemcpyAsync(a.v, b->v.as<double>() + o, bytes, cudaMemcpyDeviceToHost, c.stream));
            if (a.F) STEPS_CUDA(cudaMemcpyAsync(a.F, b->F.as<double>() + o, bytes, cudaMemcpyDeviceToHost, c.stream));
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
        },
        &args);
}

}  // extern "C"
