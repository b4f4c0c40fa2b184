#include "context.cuh"
namespace nbg {
int precise_accelerate(nbody_cuda* ctx, const nbody_step_params*) { return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "compensated/FP64 precision not built yet"); }
int precise_integrate(nbody_cuda* ctx, const nbody_step_params*) { return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "compensated precision not built yet"); }
int sync_precise_positions(nbody_cuda*) { return NBODY_OK; }
void release_precise(nbody_cuda*) {}
}
