// Batched ensembles of independent R^3 realisations (placeholder until the
// persistent work-queue kernel lands; every entry point reports STEPS_E_STATE).
#include "common.cuh"
#include "context.cuh"

namespace steps {
void batch_release() {}
}  // namespace steps

using namespace steps;

extern "C" {

int steps_gpu_batch_set(int, const int *, const double *const *, const double *const *, const double *const *)
{
    return run_guarded([](void *) { fail(STEPS_E_STATE, "batched ensembles are not available in this build"); },
                       nullptr);
}

int steps_gpu_batch_run(const steps_params *, int, int, double, int)
{
    return run_guarded([](void *) { fail(STEPS_E_STATE, "batched ensembles are not available in this build"); },
                       nullptr);
}

int steps_gpu_batch_get(int, double *, double *, double *)
{
    return run_guarded([](void *) { fail(STEPS_E_STATE, "batched ensembles are not available in this build"); },
                       nullptr);
}

}  // extern "C"
