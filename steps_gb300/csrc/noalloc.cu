// steps_gpu_forces_fp64_noalloc: the plain FP64 R^3 force evaluation for
// callers that cannot allocate device memory.
//
// Who needs it: applications that hand all device memory to their own pool
// allocator at start-up (a cudaMalloc from the library would then fail or
// fragment their pool), and loops that must not pay the implicit device-wide
// synchronisation a cudaMalloc/cudaFree can cause. Such callers own every
// buffer they pass (positions, masses, softening lengths, forces); this entry
// point calls no cudaMalloc, cudaFree or allocating library routine and needs
// no steps_gpu_init context.
//
// Its only working memory is the file-scope device array below, of
// STEPS_NOALLOC_SCRATCH_BYTES (32 MiB). Every GPU that loads the library
// holds it until the process exits. It holds the per-j-chunk FP64 partial
// forces, 24 bytes per i particle per chunk, so an i range is limited to
// STEPS_NOALLOC_SCRATCH_BYTES / 24 = 1,398,101 particles; larger ranges are
// rejected with STEPS_E_ARG. Every call writes every scratch word it later
// reads, so nothing needs clearing between calls; the array keeps the last
// call's contents. All calls share the one array: calls whose kernels overlap
// on the GPU (different streams, or several host threads) race on it and
// must be serialised by the caller.
//
// The device address of the array is looked up once per device with
// cudaGetSymbolAddress, by the first call made while that device is current;
// make that first call before any stream capture. The address is kept
// together with the CUDA context it was found in: after a cudaDeviceReset
// (which unloads the library's device code with the context) the next call
// finds a new context and looks the address up again, so that call too
// belongs before any stream capture.
//
// The empty i range id_max = id_min - 1 is accepted and does nothing (F may
// then be NULL), as in every other force entry point.
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "context.cuh"

#define STEPS_NOALLOC_SCRATCH_BYTES (32u << 20)

namespace steps {

namespace {

static __device__ __align__(256) double g_noalloc_scratch[STEPS_NOALLOC_SCRATCH_BYTES / sizeof(double)];

constexpr int NA_THREADS = 128;
constexpr int NA_MAX_DEVICES = 64;

std::mutex g_na_mutex;
double *g_na_ptr[NA_MAX_DEVICES] = {};
CUcontext g_na_ctx[NA_MAX_DEVICES] = {};  // the context each cached address belongs to

// cuCtxGetCurrent through the runtime's driver entry-point query (no link
// dependency on libcuda). Called with g_na_mutex held.
CUcontext current_context()
{
    using Fn = CUresult (*)(CUcontext *);
    static Fn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p) {
            cudaGetLastError();
            fail(STEPS_E_CUDA, "noalloc: cuCtxGetCurrent is not available from the driver");
        }
        fn = reinterpret_cast<Fn>(p);
    }
    CUcontext c = nullptr;
    if (fn(&c) != CUDA_SUCCESS) fail(STEPS_E_CUDA, "noalloc: cuCtxGetCurrent failed");
    return c;  // NULL while this thread has made no CUDA runtime call yet
}

double *lookup_scratch()
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        fail(STEPS_E_CUDA,
             std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") + cudaGetErrorString(e));
    }
    return static_cast<double *>(p);
}

// Host-side address of the scratch array on the current device. In host code
// the symbol itself is only a stand-in, never a device address.
double *scratch_on_current_device()
{
    int dev = 0;
    STEPS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NA_MAX_DEVICES) fail(STEPS_E_ARG, "device index out of range for the no-allocation path");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    CUcontext cur = current_context();
    if (cur && g_na_ptr[dev] && g_na_ctx[dev] == cur) return g_na_ptr[dev];
    // First call on this device, or a new context: the lookup also binds the
    // device's primary context to this thread when none is current yet.
    double *p = lookup_scratch();
    if (!cur) cur = current_context();
    g_na_ptr[dev] = p;
    g_na_ctx[dev] = cur;
    return p;
}

// Same pair arithmetic as the plain FP64 R^3 kernel (ascending j per i,
// spline softening StePS/src/forces.cc:52-87), reading the caller's AoS
// positions and mass/softening arrays directly.
__global__ void __launch_bounds__(NA_THREADS)
    k_noalloc_fp64_r3(const double *__restrict__ x, const double *__restrict__ m, const double *__restrict__ eps,
                      int n, int id_min, int ni, int jchunk, double *__restrict__ part)
{
    __shared__ double4_16a sp[NA_THREADS];
    __shared__ double se[NA_THREADS];
    const int t = threadIdx.x;
    const int li = blockIdx.x * NA_THREADS + t;
    const bool active = li < ni;
    const size_t i = (size_t)id_min + (active ? li : 0);
    const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2], ei = eps[i];
    const int j0 = blockIdx.y * jchunk;
    const int j1 = min(n, j0 + jchunk);
    double ax = 0, ay = 0, az = 0;
    for (int jb = j0; jb < j1; jb += NA_THREADS) {
        const int cnt = min(NA_THREADS, j1 - jb);
        __syncthreads();
        if (t < cnt) {
            const size_t j = (size_t)jb + t;
            sp[t] = make_double4_16a(x[3 * j], x[3 * j + 1], x[3 * j + 2], m[j]);
            se[t] = eps[j];
        }
        __syncthreads();
        for (int jj = 0; jj < cnt; ++jj) {
            const double4_16a q = sp[jj];
            const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
            const double w = q.w * softening_fp64(dx * dx + dy * dy + dz * dz, ei + se[jj]);
            ax = fma(w, dx, ax);
            ay = fma(w, dy, ay);
            az = fma(w, dz, az);
        }
    }
    if (active) {
        double *o = part + ((size_t)blockIdx.y * ni + li) * 3;
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

__global__ void k_noalloc_reduce(const double *__restrict__ part, int S, int ni, int id_min,
                                 const double *__restrict__ x, Background bg, double *__restrict__ F)
{
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= ni) return;
    double f[3] = {0, 0, 0};
    for (int s = 0; s < S; s++)
        for (int k = 0; k < 3; k++) f[k] += part[((size_t)s * ni + li) * 3 + k];
    add_background(bg, x + 3 * (size_t)(id_min + li), f);
    for (int k = 0; k < 3; k++) F[3 * (size_t)li + k] = f[k];
}

}  // namespace

}  // namespace steps

using namespace steps;

extern "C" int steps_gpu_forces_fp64_noalloc(const steps_params *p, const double *x, const double *m,
                                             const double *eps, int n, double *F, int id_min, int id_max,
                                             void *stream)
{
    struct A {
        const steps_params *p;
        const double *x, *m, *eps;
        int n;
        double *F;
        int id_min, id_max;
        void *stream;
    } args{p, x, m, eps, n, F, id_min, id_max, stream};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            if (!a.p) fail(STEPS_E_ARG, "noalloc: params is NULL");
            if (a.p->topology != STEPS_R3) fail(STEPS_E_ARG, "noalloc: only the R^3 topology is available");
            // id_max = id_min - 1 is the empty range (StePS/src/forces.cc:520-556
            // loops over nothing): no work, F may be NULL.
            if (a.n <= 0 || a.id_min < 0 || a.id_min > a.n || a.id_max >= a.n || a.id_max < a.id_min - 1)
                fail(STEPS_E_ARG, "noalloc: i range outside [0, n)");
            const int ni = a.id_max - a.id_min + 1;
            if (ni == 0) return;
            if (!a.x || !a.m || !a.eps || !a.F) fail(STEPS_E_ARG, "noalloc: every pointer must be non-NULL");
            const size_t cap = STEPS_NOALLOC_SCRATCH_BYTES / (3 * sizeof(double));  // i-rows of partial forces
            if ((size_t)ni > cap)
                fail(STEPS_E_ARG, "noalloc: i range of " + std::to_string(ni) + " particles exceeds the " +
                                      std::to_string(cap) + " that the 32 MiB scratch holds");
            KParams kp = derive_params(a.p);
            Tables tb{};
            double *part = scratch_on_current_device();
            int sms = 0, dev = 0;
            STEPS_CUDA(cudaGetDevice(&dev));
            STEPS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            // Split the j range for enough blocks, within the scratch capacity.
            const int bx = div_up(ni, NA_THREADS);
            int S = div_up(sms * 16, bx);
            const int maxS = (int)(cap / (size_t)ni);
            if (S > maxS) S = maxS;
            if (S > div_up(a.n, NA_THREADS)) S = div_up(a.n, NA_THREADS);
            if (S < 1) S = 1;
            const int jchunk = div_up(div_up(a.n, S), NA_THREADS) * NA_THREADS;
            S = div_up(a.n, jchunk);
            cudaStream_t st = static_cast<cudaStream_t>(a.stream);
            k_noalloc_fp64_r3<<<dim3(bx, S), NA_THREADS, 0, st>>>(a.x, a.m, a.eps, a.n, a.id_min, ni, jchunk, part);
            note_launch("k_noalloc_fp64_r3");
            k_noalloc_reduce<<<div_up(ni, 256), 256, 0, st>>>(part, S, ni, a.id_min, a.x, background_of(kp, tb), a.F);
            note_launch("k_noalloc_reduce");
        },
        &args);
}
