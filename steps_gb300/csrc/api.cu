// The extern "C" entry points of libsteps_gb300 (declared in
// include/steps_gb300.h) and the persistent single-GPU context behind them.
//
// The reference CUDA path allocates, uploads and frees every device buffer on
// every force call and spreads the i range over an OpenMP team of GPUs
// (StePS/src/forces_cuda.cu:933-1105). Here one context lives from
// steps_gpu_init to steps_gpu_shutdown: masses, softening and tables are
// uploaded once, positions once per call, and all work runs on one stream.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "mixed.cuh"

namespace steps {

static Ctx g_ctx;
static thread_local std::string g_err;
// Kernels launched since steps_gpu_init. Atomic: the allocation-free entry
// point needs no context and may be called from several host threads.
static std::atomic<long long> g_launches{0};

Ctx &ctx() { return g_ctx; }

void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void check_cuda(cudaError_t e, const char *what, const char *file, int line)
{
    if (e == cudaSuccess) return;
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    fail(e == cudaErrorMemoryAllocation ? STEPS_E_NOMEM : STEPS_E_CUDA, buf);
}

void add_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

#ifdef STEPS_CHECK
static std::vector<void *(*)()> &check_registry()
{
    static std::vector<void *(*)()> r;
    return r;
}

int register_check_record(void *(*where)())
{
    check_registry().push_back(where);
    return (int)check_registry().size();
}

static const char *check_site_name(int site)
{
    static const char *names[CK_NSITES] = {"none", "i tile", "j tile range", "j chunk", "partial slot",
                                           "output row", "T3 FP32 table cell", "T3 FP64 table cell",
                                           "S1xR2 table cell", "radial table entry", "particle index",
                                           "radix-sort destination", "self-test index"};
    return site >= 0 && site < CK_NSITES ? names[site] : "unknown site";
}

// Reads the bounds-check record of every translation unit after a call; the
// first one set fails the call with STEPS_E_BOUNDS and is cleared.
static void check_bounds_records()
{
    if (g_ctx.device < 0) return;
    STEPS_CUDA(cudaDeviceSynchronize());
    for (auto where : check_registry()) {
        void *p = where();
        if (!p) continue;
        CheckRecord r;
        STEPS_CUDA(cudaMemcpy(&r, p, sizeof r, cudaMemcpyDeviceToHost));
        if (r.code == 0) continue;
        const CheckRecord none{};
        STEPS_CUDA(cudaMemcpy(p, &none, sizeof none, cudaMemcpyHostToDevice));
        g_ctx.F_ni = 0;
        g_ctx.F_valid = false;
        char buf[200];
        snprintf(buf, sizeof buf, "bounds check failed: %s %lld outside [0, %lld)", check_site_name(r.site), r.index,
                 r.bound);
        fail(STEPS_E_BOUNDS, buf);
    }
}
#endif

__global__ void k_check_selftest(int index)
{
    int v = index;
    STEPS_CHECK_IDX(v, 16, CK_SELFTEST);
    (void)v;
}

void note_launch(const char *name)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof buf, "launch of %s failed: %s", name, cudaGetErrorString(e));
        fail(STEPS_E_CUDA, buf);
    }
}

void DevBuf::grow(size_t want)
{
    if (want <= bytes && p) return;
    if (p) {
        cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    size_t sz = want < 256 ? 256 : want;
    cudaError_t e = cudaMalloc(&p, sz);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        char buf[160];
        snprintf(buf, sizeof buf, "cudaMalloc of %zu bytes failed: %s", sz, cudaGetErrorString(e));
        fail(STEPS_E_NOMEM, buf);
    }
    bytes = sz;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

int *kernel_status_word()
{
    Ctx &c = g_ctx;
    if (!c.kstatus.p) {
        int *w = c.kstatus.ensure<int>(1);
        STEPS_CUDA(cudaMemsetAsync(w, 0, sizeof(int), c.stream));
    }
    return c.kstatus.as<int>();
}

void check_kernel_status()
{
    Ctx &c = g_ctx;
    if (!c.status_pending || !c.kstatus.p) return;
    if (!c.kstatus_host) STEPS_CUDA(cudaMallocHost(&c.kstatus_host, sizeof(int)));
    STEPS_CUDA(cudaMemcpyAsync(c.kstatus_host, c.kstatus.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    STEPS_CUDA(cudaStreamSynchronize(c.stream));
    c.status_pending = false;
    if (*c.kstatus_host != 0) {
        STEPS_CUDA(cudaMemsetAsync(c.kstatus.p, 0, sizeof(int), c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
        c.F_ni = 0;
        c.F_valid = false;
        fail(STEPS_E_TIMEOUT, "a bounded device-side wait gave up (status written by the kernel)");
    }
}

void require_init()
{
    if (g_ctx.device < 0) fail(STEPS_E_STATE, "steps_gpu_init has not been called");
    STEPS_CUDA(cudaSetDevice(g_ctx.device));
}

KParams derive_params(const steps_params *p)
{
    if (!p) fail(STEPS_E_ARG, "params is NULL");
    KParams k{};
    k.topology = p->topology;
    k.is_periodic = p->is_periodic;
    k.s1r2_images = p->s1r2_images;
    k.order = p->ewald_order;
    k.L = p->L;
    k.halfL = 0.5 * p->L;
    k.rsim = p->rsim;
    // ewald_max = IS_PERIODIC + 1, ewald_cut = ewald_max - 0.4 (StePS/src/main.cc:1270-1271,
    // StePS/src/forces_cuda.cu:659-660).
    k.emax = p->is_periodic + 1;
    k.cutL = ((double)k.emax - 0.4) * p->L;
    if (p->topology < STEPS_R3 || p->topology > STEPS_S1R2) fail(STEPS_E_ARG, "unknown topology");
    if (p->topology != STEPS_R3) {
        if (!(p->L > 0)) fail(STEPS_E_ARG, "periodic topology needs L > 0");
        if (p->is_periodic < 1) fail(STEPS_E_ARG, "periodic topology needs IS_PERIODIC >= 1");
    }
    if (p->topology == STEPS_T3 && p->is_periodic >= 2 && p->ewald_order != 2 && p->ewald_order != 4)
        fail(STEPS_E_ARG, "T3 interpolation order must be 2 or 4");
    if (p->topology == STEPS_S1R2 && p->is_periodic >= 2 && !p->s1r2_images && p->ewald_order != 0 &&
        p->ewald_order != 2 && p->ewald_order != 4)
        fail(STEPS_E_ARG, "S1R2 table interpolation order must be 0, 2 or 4");
    if (p->topology == STEPS_S1R2 && p->s1r2_images && k.emax > 64) fail(STEPS_E_ARG, "IS_PERIODIC too large");
    if (p->cosmology == 1 && p->comoving == 1) {
        k.comoving_bg = 1;
        k.bg_coef = p->mass_in_unit_sphere;
    } else if (p->cosmology == 1 && p->comoving == 0) {
        k.comoving_bg = 2;
        k.bg_coef = p->h0 * p->h0 * p->omega_lambda;
    }
    if (p->topology == STEPS_T3) k.comoving_bg = 0;  // T^3 has no background term
    return k;
}

Tables device_tables(const KParams &kp)
{
    Ctx &c = g_ctx;
    Tables t{};
    t.t3 = c.t3.as<double>();
    t.t3_ng = c.t3_ng;
    t.s1r2 = c.s1r2.as<double>();
    t.nrho = c.nrho;
    t.nz = c.nz;
    t.rho_max = 2.25 * kp.rsim;  // EWALD_LOOKUP_TABLE_RADIAL_EXTENT_FACTOR, StePS/src/global_variables.h:39
    t.radial = c.radial.as<double>();
    t.radial_size = c.radial_size;
    if (kp.topology == STEPS_T3 && kp.is_periodic >= 2 && c.t3_ng <= 0)
        fail(STEPS_E_STATE, "T3 Ewald run needs a table (steps_gpu_set_table_t3 / steps_gpu_build_table_t3)");
    if (kp.topology == STEPS_S1R2 && kp.is_periodic >= 2 && !kp.s1r2_images && c.nrho <= 0)
        fail(STEPS_E_STATE, "S1R2 table run needs a table (steps_gpu_set_table_s1r2 / steps_gpu_build_table_s1r2)");
    if (kp.topology == STEPS_S1R2 && kp.is_periodic >= 2 && !kp.s1r2_images && c.nrho < 2)
        fail(STEPS_E_TABLE, "S1R2 table needs at least 2 radial points");
    return t;
}

void compute_forces(const steps_params *p, int precision, int id_min, int id_max, bool reuse_order)
{
    Ctx &c = g_ctx;
    require_init();
    if (c.n <= 0) fail(STEPS_E_STATE, "no particles: call steps_gpu_set_particles first");
    if (!c.have_x) fail(STEPS_E_STATE, "no positions uploaded");
    // id_max = id_min - 1 is the empty range: no work, as in the reference's
    // loop over [ID_min, ID_max] (StePS/src/forces.cc:520-556).
    if (id_min < 0 || id_min > c.n || id_max >= c.n || id_max < id_min - 1)
        fail(STEPS_E_ARG, "i range outside [0, n)");
    if (precision != STEPS_FP64 && precision != STEPS_MIXED) fail(STEPS_E_ARG, "unknown precision mode");
    KParams kp = derive_params(p);
    Tables tb = device_tables(kp);
    int ni = id_max - id_min + 1;
    // Until this call succeeds the force buffer holds no valid range.
    c.F_ni = 0;
    c.F_valid = false;
    if (ni == 0) {
        c.F_lo = id_min;
        return;
    }
    double *F = c.F.ensure<double>(3 * (size_t)c.n);
    if (precision == STEPS_FP64)
        forces_fp64(kp, tb, c.x.as<double>(), c.n, id_min, ni, F);
    else
        forces_mixed(kp, tb, c.x.as<double>(), c.m64.as<double>(), c.eps64.as<double>(), c.n, id_min, ni, F,
                     reuse_order);
    c.F_lo = id_min;
    c.F_ni = ni;
    c.F_valid = id_min == 0 && ni == c.n;
}

}  // namespace steps

using namespace steps;

template <class Fn>
static int guarded(Fn &&fn)
{
    try {
        fn();
#ifdef STEPS_CHECK
        check_bounds_records();
#endif
        return STEPS_OK;
    } catch (const Error &e) {
        g_err = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        g_err = e.what();
        return STEPS_E_STATE;
    }
}

namespace steps {
int run_guarded(void (*body)(void *), void *arg)
{
    return guarded([&] { body(arg); });
}
}  // namespace steps

extern "C" {

int steps_gpu_abi_version(void) { return STEPS_GB300_ABI_VERSION; }

const char *steps_gpu_error_string(void) { return g_err.c_str(); }

int steps_gpu_checks_compiled(void)
{
#ifdef STEPS_CHECK
    return 1;
#else
    return 0;
#endif
}

int steps_gpu_test_bounds_check(int index)
{
    return guarded([&] {
        require_init();
#ifndef STEPS_CHECK
        fail(STEPS_E_STATE, "bounds checks are compiled into libsteps_gb300_check.so only");
#endif
        k_check_selftest<<<1, 1, 0, g_ctx.stream>>>(index);
        note_launch("k_check_selftest");
    });
}

int steps_gpu_init(int device)
{
    return guarded([&] {
        Ctx &c = g_ctx;
        if (c.device == device) return;
        if (c.device >= 0) fail(STEPS_E_STATE, "already initialised on another device; call steps_gpu_shutdown first");
        int count = 0;
        STEPS_CUDA(cudaGetDeviceCount(&count));
        if (device < 0 || device >= count) fail(STEPS_E_ARG, "no such CUDA device");
        STEPS_CUDA(cudaSetDevice(device));
        STEPS_CUDA(cudaDeviceGetAttribute(&c.nsm, cudaDevAttrMultiProcessorCount, device));
        STEPS_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        for (auto &e : c.marks) STEPS_CUDA(cudaEventCreate(&e));
        for (auto &e : c.phase) STEPS_CUDA(cudaEventCreate(&e));
        c.device = device;
        g_launches.store(0);
    });
}

int steps_gpu_shutdown(void)
{
    return guarded([&] {
        Ctx &c = g_ctx;
        if (c.device < 0) return;
        cudaSetDevice(c.device);
        cudaStreamSynchronize(c.stream);
        batch_release();
        DevBuf *bufs[] = {&c.m64, &c.eps64, &c.x, &c.v, &c.F, &c.pack64, &c.partial, &c.bbox, &c.counter,
                          &c.status, &c.flush, &c.peaks, &c.t3, &c.t3f, &c.t3r, &c.s1r2, &c.s1f, &c.s1rec,
                          &c.radial, &c.kstatus};
        for (DevBuf *b : bufs) b->release();
        if (c.kstatus_host) cudaFreeHost(c.kstatus_host);
        TileSet *ts[] = {&c.tj, &c.ti};
        for (TileSet *t : ts) {
            for (int k = 0; k < 2; k++) { t->keys[k].release(); t->vals[k].release(); }
            t->hist.release(); t->pack.release(); t->eps.release(); t->meta.release(); t->idx.release(); t->resid.release(); t->soa.release(); t->sub.release();
            *t = TileSet();
        }
        for (auto &e : c.marks) cudaEventDestroy(e);
        for (auto &e : c.phase) cudaEventDestroy(e);
        cudaStreamDestroy(c.stream);
        g_ctx = Ctx();
    });
}

int steps_gpu_set_particles(int n, const double *m, const double *eps)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (n <= 0 || !m || !eps) fail(STEPS_E_ARG, "set_particles: n must be > 0 and m, eps non-NULL");
        if (n > (1 << 30)) fail(STEPS_E_ARG, "set_particles: n too large");
        if (n != c.n) {
            c.have_x = c.have_v = false;
            c.tj.ordered = c.ti.ordered = false;
        }
        // New masses or softening make the last forces stale, and a smaller n
        // must not let steps_gpu_download_forces copy the old, longer range.
        c.F_valid = false;
        c.F_lo = c.F_ni = 0;
        STEPS_CUDA(cudaMemcpyAsync(c.m64.ensure<double>(n), m, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
        STEPS_CUDA(cudaMemcpyAsync(c.eps64.ensure<double>(n), eps, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
        c.n = n;
    });
}

int steps_gpu_upload_positions(const double *x)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (c.n <= 0) fail(STEPS_E_STATE, "no particles: call steps_gpu_set_particles first");
        if (!x) fail(STEPS_E_ARG, "x is NULL");
        STEPS_CUDA(cudaMemcpyAsync(c.x.ensure<double>(3 * (size_t)c.n), x, sizeof(double) * 3 * c.n,
                                   cudaMemcpyHostToDevice, c.stream));
        c.have_x = true;
        c.F_valid = false;
    });
}

int steps_gpu_upload_velocities(const double *v)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (c.n <= 0) fail(STEPS_E_STATE, "no particles: call steps_gpu_set_particles first");
        if (!v) fail(STEPS_E_ARG, "v is NULL");
        STEPS_CUDA(cudaMemcpyAsync(c.v.ensure<double>(3 * (size_t)c.n), v, sizeof(double) * 3 * c.n,
                                   cudaMemcpyHostToDevice, c.stream));
        c.have_v = true;
    });
}

int steps_gpu_forces_resident(const steps_params *p, int precision, int id_min, int id_max)
{
    return guarded([&] { compute_forces(p, precision, id_min, id_max, false); });
}

int steps_gpu_download_forces(double *F)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (!F) fail(STEPS_E_ARG, "F is NULL");
        if (c.F_ni <= 0) fail(STEPS_E_STATE, "no forces computed");
        STEPS_CUDA(cudaMemcpyAsync(F, c.F.as<double>(), sizeof(double) * 3 * c.F_ni, cudaMemcpyDeviceToHost, c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int steps_gpu_forces_range(int *id_min, int *count)
{
    return guarded([&] {
        if (!id_min || !count) fail(STEPS_E_ARG, "id_min and count must be non-NULL");
        *id_min = g_ctx.F_lo;
        *count = g_ctx.F_ni;
    });
}

int steps_gpu_forces(const steps_params *p, int precision, const double *x, double *F, int id_min, int id_max)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (!x || (!F && id_max >= id_min)) fail(STEPS_E_ARG, "x and F must be non-NULL");
        if (c.n <= 0) fail(STEPS_E_STATE, "no particles: call steps_gpu_set_particles first");
        STEPS_CUDA(cudaMemcpyAsync(c.x.ensure<double>(3 * (size_t)c.n), x, sizeof(double) * 3 * c.n,
                                   cudaMemcpyHostToDevice, c.stream));
        c.have_x = true;
        compute_forces(p, precision, id_min, id_max, false);
        int ni = id_max - id_min + 1;
        if (ni > 0)
            STEPS_CUDA(cudaMemcpyAsync(F, c.F.as<double>(), sizeof(double) * 3 * (size_t)ni, cudaMemcpyDeviceToHost,
                                       c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int steps_gpu_download_state(double *x, double *v, double *F)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        size_t b = sizeof(double) * 3 * (size_t)c.n;
        if (x) {
            if (!c.have_x) fail(STEPS_E_STATE, "no positions");
            STEPS_CUDA(cudaMemcpyAsync(x, c.x.as<double>(), b, cudaMemcpyDeviceToHost, c.stream));
        }
        if (v) {
            if (!c.have_v) fail(STEPS_E_STATE, "no velocities");
            STEPS_CUDA(cudaMemcpyAsync(v, c.v.as<double>(), b, cudaMemcpyDeviceToHost, c.stream));
        }
        if (F) {
            if (c.F_ni <= 0) fail(STEPS_E_STATE, "no forces computed");
            STEPS_CUDA(cudaMemcpyAsync(F, c.F.as<double>(), sizeof(double) * 3 * c.F_ni, cudaMemcpyDeviceToHost,
                                       c.stream));
        }
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int steps_gpu_set_table_t3(int ngrid, const double *table)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (ngrid < 2 || ngrid > 1024 || !table) fail(STEPS_E_ARG, "set_table_t3: ngrid in [2, 1024], table non-NULL");
        size_t cnt = 3 * (size_t)ngrid * ngrid * ngrid;
        STEPS_CUDA(cudaMemcpyAsync(c.t3.ensure<double>(cnt), table, cnt * sizeof(double), cudaMemcpyHostToDevice,
                                   c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
        c.t3_ng = ngrid;
        c.t3_version++;
    });
}

int steps_gpu_get_table_t3(double *out)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (!out) fail(STEPS_E_ARG, "out is NULL");
        if (c.t3_ng <= 0) fail(STEPS_E_STATE, "no T3 table");
        size_t cnt = 3 * (size_t)c.t3_ng * c.t3_ng * c.t3_ng;
        STEPS_CUDA(cudaMemcpyAsync(out, c.t3.as<double>(), cnt * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int steps_gpu_set_table_s1r2(int nrho, int nz, const double *table)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (nrho < 1 || nz < 1 || !table || (long long)nrho * nz > (1LL << 28))
            fail(STEPS_E_ARG, "set_table_s1r2: bad shape or NULL table");
        size_t cnt = 2 * (size_t)nrho * nz;
        STEPS_CUDA(cudaMemcpyAsync(c.s1r2.ensure<double>(cnt), table, cnt * sizeof(double), cudaMemcpyHostToDevice,
                                   c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
        c.nrho = nrho;
        c.nz = nz;
        c.s1r2_version++;
    });
}

int steps_gpu_get_table_s1r2(double *out)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (!out) fail(STEPS_E_ARG, "out is NULL");
        if (c.nrho <= 0) fail(STEPS_E_STATE, "no S1R2 table");
        size_t cnt = 2 * (size_t)c.nrho * c.nz;
        STEPS_CUDA(cudaMemcpyAsync(out, c.s1r2.as<double>(), cnt * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int steps_gpu_set_radial_table(int size, const double *table)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        if (size < 2 || !table) fail(STEPS_E_ARG, "set_radial_table: size >= 2 and table non-NULL");
        STEPS_CUDA(cudaMemcpyAsync(c.radial.ensure<double>(size), table, size * sizeof(double), cudaMemcpyHostToDevice,
                                   c.stream));
        STEPS_CUDA(cudaStreamSynchronize(c.stream));
        c.radial_size = size;
    });
}

int steps_gpu_set_tuning(int threads, int ipt, int jsplit)
{
    return guarded([&] {
        if (!shape_supported(threads, ipt)) fail(STEPS_E_ARG, "unsupported kernel shape");
        if (jsplit < 0) fail(STEPS_E_ARG, "jsplit must be >= 0");
        g_ctx.shape.threads = threads;
        g_ctx.shape.ipt = ipt;
        g_ctx.shape.jsplit = jsplit;
        g_ctx.shape_fixed = true;
    });
}

int steps_gpu_autotune(const steps_params *p, int id_min, int id_max, int *out)
{
    return guarded([&] {
        require_init();
        Ctx &c = g_ctx;
        static const int shapes[][2] = {{64, 1}, {64, 2}, {64, 4}, {128, 1}, {128, 2}, {128, 4}, {256, 1}, {256, 2}};
        Shape keep = c.shape;
        Shape bestS = keep;
        KParams kp = derive_params(p);
        // R^3: the scalar and packed pair loops as well; T^3 with a table: the
        // one-i-per-lane and quad-lane kernels.
        const int nvar = kp.topology == STEPS_R3                          ? R3_VARIANTS
                         : kp.topology == STEPS_T3 && kp.is_periodic >= 2 ? T3_VARIANTS
                                                                          : 1;
        // Stage 1: each candidate is scored by its time per pair on a strided
        // sample of the real i tiles, 24 waves of items (one untimed one-wave
        // launch, then one timed; the whole range if it is smaller). Fewer
        // waves misrank the candidates: the launch ramp and the last wave
        // weigh in.
        // Stage 2: the three best are timed on 96 waves (or the whole range).
        struct SampleMode {
            Ctx &c;
            explicit SampleMode(Ctx &cc) : c(cc) {}
            ~SampleMode()
            {
                c.tune_sample = 0;
                c.F_ni = 0;  // the timing runs leave no usable forces
                c.F_valid = false;
            }
        } mode(c);
        // time per pair of one timed launch at a sample size; warm: after an
        // untimed one-wave launch (module load, caches)
        auto score = [&](const Shape &sh, int waves, bool warm) {
            c.shape = sh;
            if (warm) {
                c.tune_sample = 1;
                compute_forces(p, STEPS_MIXED, id_min, id_max, true);
            }
            c.tune_sample = waves;
            float ms = 0.0f;
            // the phase events bracket the pair kernel only
            compute_forces(p, STEPS_MIXED, id_min, id_max, true);
            STEPS_CUDA(cudaEventSynchronize(c.phase[2]));
            STEPS_CUDA(cudaEventElapsedTime(&ms, c.phase[1], c.phase[2]));
            return (double)ms / c.last_pairs;
        };
        c.tune_sample = 1;
        compute_forces(p, STEPS_MIXED, id_min, id_max, false);  // orders the particles, loads modules
        std::vector<std::pair<double, Shape>> scored;
        for (int v = 0; v < nvar; v++)
            for (auto &s : shapes) {
                if (!shape_supported_for(kp, s[0], s[1])) continue;
                if (kp.topology == STEPS_R3 && v >= 1 && v <= 3 && !r3x2_kernel(s[0], s[1], false, r3x2_occ(v)))
                    continue;
                if (kp.topology == STEPS_R3 && v == 4 && !r3x2_pipe_kernel(s[0], s[1])) continue;
                if (kp.topology == STEPS_T3 && v == 1 && !t3_quad_kernel(kp, s[0], s[1])) continue;
                Shape sh = keep;
                sh.threads = s[0];
                sh.ipt = s[1];
                sh.jsplit = 0;
                sh.variant = v;
                scored.emplace_back(score(sh, 24, true), sh);
                // A range of few waves is balanced by its shortest items:
                // there the j split is timed too (2x and 4x the rule's chunks).
                const int rule_S = c.last_S;
                if (c.last_waves < 32.0)
                    for (int f = 2; f <= 4; f *= 2) {
                        sh.jsplit = rule_S * f;
                        scored.emplace_back(score(sh, 24, true), sh);
                    }
            }
        std::stable_sort(scored.begin(), scored.end(), [](const std::pair<double, Shape> &a,
                                                          const std::pair<double, Shape> &b) { return a.first < b.first; });
        double best = 1e300;
        for (size_t k = 0; k < scored.size() && k < 3; k++) {
            const double sc = score(scored[k].second, 96, false);
            if (sc < best) { best = sc; bestS = scored[k].second; }
        }
        c.shape = bestS;
        c.shape_fixed = true;
        if (out) { out[0] = bestS.threads; out[1] = bestS.ipt; out[2] = bestS.variant; }
    });
}

int steps_gpu_set_precision_guard(double ratio)
{
    return guarded([&] {
        if (!(ratio >= 1.0 && ratio <= 1e6)) fail(STEPS_E_ARG, "precision guard ratio must be in [1, 1e6]");
        g_ctx.shape.guard = (float)ratio;
    });
}

int steps_gpu_set_t3_window(int cells)
{
    return guarded([&] {
        if (cells < 0 || cells > STEPS_T3_WINDOW_MAX)
            fail(STEPS_E_ARG, "T3 window capacity must be in [0, " + std::to_string(STEPS_T3_WINDOW_MAX) + "] cells");
        g_ctx.shape.t3_cells = cells;
    });
}

int steps_gpu_set_kernel_variant(int variant)
{
    return guarded([&] {
        if (variant < 0 || variant >= R3_VARIANTS)
            fail(STEPS_E_ARG, "kernel variant must be 0 (scalar), 1 (packed FP32x2), 2 or 3 (packed, 768 or 1024 "
                              "threads per SM) or 4 (packed, bulk-copy pipeline); for T3, 1 selects quad lanes");
        g_ctx.shape.variant = variant;
    });
}

long long steps_gpu_launch_count(void) { return g_launches.load(); }

double steps_gpu_last_phase_ms(int phase)
{
    Ctx &c = g_ctx;
    if (c.device < 0 || !c.phase_valid || phase < 0 || phase > 2) return -1.0;
    if (cudaEventSynchronize(c.phase[phase + 1]) != cudaSuccess) return -1.0;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c.phase[phase], c.phase[phase + 1]) != cudaSuccess) return -1.0;
    return ms;
}

double steps_gpu_last_pairs(void) { return g_ctx.last_pairs; }

int steps_gpu_timer_mark(int slot)
{
    return guarded([&] {
        require_init();
        if (slot < 0 || slot >= 16) fail(STEPS_E_ARG, "timer slot must be in [0, 16)");
        STEPS_CUDA(cudaEventRecord(g_ctx.marks[slot], g_ctx.stream));
        g_ctx.mark_set[slot] = true;
    });
}

double steps_gpu_timer_elapsed_ms(int a, int b)
{
    Ctx &c = g_ctx;
    if (c.device < 0 || a < 0 || b < 0 || a >= 16 || b >= 16 || !c.mark_set[a] || !c.mark_set[b]) return -1.0;
    if (cudaEventSynchronize(c.marks[b]) != cudaSuccess) return -1.0;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c.marks[a], c.marks[b]) != cudaSuccess) return -1.0;
    return ms;
}

int steps_gpu_flush_l2(long long bytes)
{
    return guarded([&] {
        require_init();
        if (bytes <= 0 || bytes > (8LL << 30)) fail(STEPS_E_ARG, "flush size out of range");
        void *p = g_ctx.flush.ensure<char>((size_t)bytes);
        STEPS_CUDA(cudaMemsetAsync(p, (int)(g_launches.load() & 0xff), (size_t)bytes, g_ctx.stream));
    });
}

int steps_gpu_test_stall_copy(long long tile_seq)
{
    return guarded([&] {
        if (tile_seq < -1) fail(STEPS_E_ARG, "tile_seq must be >= -1");
        g_ctx.stall_seq = tile_seq;
    });
}

int steps_gpu_host_alloc(long long bytes, void **p)
{
    return guarded([&] {
        if (!p || bytes <= 0) fail(STEPS_E_ARG, "host_alloc: positive size and a result pointer required");
        *p = nullptr;
        require_init();
        if (cudaMallocHost(p, (size_t)bytes) != cudaSuccess) {
            *p = nullptr;
            cudaGetLastError();
            fail(STEPS_E_NOMEM, "cudaMallocHost failed");
        }
    });
}

int steps_gpu_host_free(void *p)
{
    return guarded([&] {
        if (p) STEPS_CUDA(cudaFreeHost(p));
    });
}

int steps_gpu_synchronize(void)
{
    return guarded([&] {
        require_init();
        STEPS_CUDA(cudaStreamSynchronize(g_ctx.stream));
        STEPS_CUDA(cudaGetLastError());
    });
}

}  // extern "C"
