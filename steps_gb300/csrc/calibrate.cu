// Issue-peak calibration: dependent FMA chains that keep the FP32 (and FP64)
// pipes full, timed with CUDA events. Gives the denominator of the FP32/FP64
// roofline fraction on the GPU the library runs on, at the clocks it runs at.
#include "common.cuh"
#include "context.cuh"

namespace steps {

namespace {

constexpr int CHAINS = 8;
constexpr int ITERS = 4096;

template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T *out, T seed)
{
    T a[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++) a[c] = seed + (T)(threadIdx.x + c);
    const T mul = (T)0.999999, add = (T)1e-7;
    for (int it = 0; it < ITERS; it++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) a[c] = a[c] * mul + add;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; c++) s += a[c];
    if (s == (T)-1) out[blockIdx.x] = s;  // keeps the chains live
}

template <class T>
double time_chains(Ctx &c, int blocks_per_sm)
{
    T *out = c.peaks.ensure<T>(65536);
    int blocks = c.nsm * blocks_per_sm;
    k_fma_chains<T><<<blocks, 256, 0, c.stream>>>(out, (T)1);  // warm-up
    note_launch("k_fma_chains");
    STEPS_CUDA(cudaEventRecord(c.marks[14], c.stream));
    const int reps = 5;
    for (int r = 0; r < reps; r++) {
        k_fma_chains<T><<<blocks, 256, 0, c.stream>>>(out, (T)1);
        note_launch("k_fma_chains");
    }
    STEPS_CUDA(cudaEventRecord(c.marks[15], c.stream));
    STEPS_CUDA(cudaEventSynchronize(c.marks[15]));
    float ms = 0;
    STEPS_CUDA(cudaEventElapsedTime(&ms, c.marks[14], c.marks[15]));
    double flops = 2.0 * CHAINS * (double)ITERS * 256.0 * blocks * reps;
    return flops / (ms * 1e-3);
}

}  // namespace

}  // namespace steps

using namespace steps;

extern "C" int steps_gpu_measure_peaks(double *fp32_flops, double *fp64_flops)
{
    struct A {
        double *f32, *f64;
    } a{fp32_flops, fp64_flops};
    return run_guarded(
        [](void *p) {
            A &q = *static_cast<A *>(p);
            require_init();
            Ctx &c = ctx();
            if (q.f32) q.f32[0] = time_chains<float>(c, 16);
            if (q.f64) q.f64[0] = time_chains<double>(c, 2);
        },
        &a);
}
