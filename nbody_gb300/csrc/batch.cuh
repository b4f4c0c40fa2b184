// Internal interface of the batched direct sums (batch.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include "nbody_cuda.h"

struct nbody_cuda;

namespace nbg
{
    struct BatchState;

    int batch_set_systems(nbody_cuda* ctx, const int64_t* offsets, size_t nsys);
    int batch_accelerate(nbody_cuda* ctx, const nbody_step_params* p);
    int batch_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms, int* best);
    int batch_set_config(nbody_cuda* ctx, int index);
    int batch_get_config(const nbody_cuda* ctx);
    int batch_config_count();
    void batch_config_describe(int index, int* block, int* t, int* chunk);
    int batch_energy(nbody_cuda* ctx, const nbody_step_params* p, double* out);
    size_t batch_system_count(const nbody_cuda* ctx);
    void release_batch(nbody_cuda* ctx);
}
