// Device-resident KDK leapfrog (StePS/src/step.cc:100-312): positions,
// velocities and forces stay in HBM across steps; only errmax comes back.
// Positions and velocities are FP64 whatever the force precision.
#include "common.cuh"
#include "context.cuh"

namespace steps {

namespace {

// acceleration = g F a^-3 - 2 H v (step.cc:131-136); kick h/2, drift h, then
// the periodic wrap of step.cc:151-180 (wrap_mode 1: all axes, 2: z only).
__global__ void k_kick_drift(double *__restrict__ x, double *__restrict__ v, const double *__restrict__ F, int n,
                             double h, double g, double a3, double hubble, int wrap_mode, double L)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 3; k++) {
        size_t q = 3 * (size_t)i + k;
        double acc = g * F[q] * a3 - 2.0 * hubble * v[q];
        double vv = v[q] + acc * (h / 2.0);
        double xx = x[q] + vv * h;
        if (wrap_mode == 1 || (wrap_mode == 2 && k == 2)) {
            if (xx < 0) xx += L;
            else if (xx >= L) xx -= L;
        }
        v[q] = vv;
        x[q] = xx;
    }
}

// Second kick and err_i = |acc| / cbrt(m_i * 3 / (4 pi rho_part)) (step.cc:256-269);
// errmax by atomicMax on the bit pattern (monotone for non-negative doubles).
__global__ void k_kick_err(double *__restrict__ v, const double *__restrict__ F, const double *__restrict__ m, int n,
                           double h, double g, double a3, double hubble, double cb, unsigned long long *errmax)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < n) {
        double acc[3];
        for (int k = 0; k < 3; k++) {
            size_t q = 3 * (size_t)i + k;
            acc[k] = g * F[q] * a3 - 2.0 * hubble * v[q];
            v[q] += acc[k] * (h / 2.0);
        }
        e = sqrt(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]) / cbrt(m[i] * cb);
    }
    for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0 && e > 0.0) atomicMax(errmax, (unsigned long long)__double_as_longlong(e));
}

}  // namespace

void kdk_kick_drift(double *x, double *v, const double *F, int n, double h, double g, double a3, double hubble,
                    int wrap_mode, double L, cudaStream_t st)
{
    k_kick_drift<<<div_up(n, 256), 256, 0, st>>>(x, v, F, n, h, g, a3, hubble, wrap_mode, L);
    note_launch("k_kick_drift");
}

double kdk_kick_err(double *v, const double *F, const double *m, int n, double h, double g, double a3, double hubble,
                    double rho_part, double *err_scratch, cudaStream_t st, bool fetch)
{
    const double cb = 3.0 / rho_part / (4.0 * 3.14159265358979323846264338327950288419716939937510);
    unsigned long long *em = reinterpret_cast<unsigned long long *>(err_scratch);
    STEPS_CUDA(cudaMemsetAsync(em, 0, sizeof(unsigned long long), st));
    k_kick_err<<<div_up(n, 256), 256, 0, st>>>(v, F, m, n, h, g, a3, hubble, cb, em);
    note_launch("k_kick_err");
    if (!fetch) return 0.0;
    unsigned long long bits = 0;
    STEPS_CUDA(cudaMemcpyAsync(&bits, em, sizeof bits, cudaMemcpyDeviceToHost, st));
    STEPS_CUDA(cudaStreamSynchronize(st));
    double e;
    memcpy(&e, &bits, sizeof e);
    return e;
}

}  // namespace steps

using namespace steps;

// Mixed R^3 steps keep the Morton order of the last sort for
// KDK_RESORT_EVERY - 1 steps and only rebuild the tiles (centres, extents,
// offsets, sub-tile boxes) from the drifted positions: one leapfrog step moves
// a particle a small fraction of its tile, the forces do not depend on the
// order (a looser tile only sends more tile pairs down the exact near path),
// and the sort is most of the preparation at small N. Periodic topologies
// re-sort every step: a particle wrapped across the box would stretch its
// tile over the whole period.
static constexpr int KDK_RESORT_EVERY = 8;

extern "C" int steps_gpu_kdk(const steps_params *p, int precision, int nsteps, double h, double g, double a,
                             double hubble, double rho_part, double *errmax_out)
{
    struct A {
        const steps_params *p;
        int precision, nsteps;
        double h, g, a, hubble, rho_part;
        double *errmax_out;
    } args{p, precision, nsteps, h, g, a, hubble, rho_part, errmax_out};
    return run_guarded(
        [](void *vp) {
            A &q = *static_cast<A *>(vp);
            require_init();
            Ctx &c = ctx();
            if (!q.p) fail(STEPS_E_ARG, "params is NULL");
            if (q.nsteps < 0) fail(STEPS_E_ARG, "nsteps must be >= 0");
            if (!(q.rho_part > 0)) fail(STEPS_E_ARG, "rho_part must be > 0");
            if (!c.have_x || !c.have_v) fail(STEPS_E_STATE, "kdk needs resident positions and velocities");
            int wrap = q.p->topology == STEPS_T3 ? 1 : (q.p->topology == STEPS_S1R2 ? 2 : 0);
            double a3 = pow(q.a, -3.0);
            if (!c.F_valid) compute_forces(q.p, q.precision, 0, c.n - 1, false);
            double *es = c.status.ensure<double>(4);
            double e = 0.0;
            for (int s = 0; s < q.nsteps; s++) {
                kdk_kick_drift(c.x.as<double>(), c.v.as<double>(), c.F.as<double>(), c.n, q.h, q.g, a3, q.hubble,
                               wrap, q.p->L, c.stream);
                const bool reuse = q.p->topology == STEPS_R3 && (s + 1) % KDK_RESORT_EVERY != 0;
                compute_forces(q.p, q.precision, 0, c.n - 1, reuse);
                e = kdk_kick_err(c.v.as<double>(), c.F.as<double>(), c.m64.as<double>(), c.n, q.h, q.g, a3, q.hubble,
                                 q.rho_part, es, c.stream, s == q.nsteps - 1);
            }
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
            if (q.errmax_out) *q.errmax_out = e;
        },
        &args);
}
