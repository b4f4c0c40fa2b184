// Internal interface of the direct-sum kernels (direct.cu, direct_precise.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace nbg
{
    // Launch shape of one direct-sum accelerate.
    struct DirectPlan
    {
        int variant;    // index into the instantiated (targets/thread, block) table
        int T;          // targets per thread
        int block;      // threads per CTA
        int tile;       // sources per shared-memory tile
        int jsplit;     // source chunks (grid.y); >1 means partials + a fixed-order sum
        int chunk;      // sources per chunk (a multiple of tile)
        int grid_x;     // target blocks
        int law;
        bool aos;
    };

    // Pick a launch shape for n bodies. force_variant >= 0 pins the (T, block) entry.
    DirectPlan plan_direct(size_t n, int law, bool aos, int force_variant = -1);

    // The instantiated kernel shapes: targets per thread, threads per CTA, packed FP32x2 or not.
    int direct_variant_count();
    void direct_variant_describe(int i, int* T, int* block, int* packed);

    // Queue the accelerate. src is pos_mass (SoA) or the Body array viewed as float4
    // (AoS). Results: acc (SoA) or Body::acc in body_out (AoS). scratch must hold
    // plan.jsplit * n float4 when plan.jsplit > 1; with reduce == false the partials are
    // left there for the fused integrate to sum.
    cudaError_t launch_direct(const DirectPlan& plan, const float4* src, const float4* vel_radius,
                              float4* acc, float* body_out, float4* scratch, int n, float G,
                              float eps2, unsigned* err, cudaStream_t stream, uint64_t* launches,
                              bool reduce = true);

    cudaError_t launch_reduce(const float4* scratch, int jsplit, int n, float4* acc,
                              float* body_out, cudaStream_t stream, uint64_t* launches);

    // Semi-implicit Euler (integrate.cu). When part != nullptr the accelerations are the
    // fixed-order sum of jsplit partials, also written to acc / Body::acc.
    cudaError_t launch_integrate_soa(float4* pos_mass, float4* vel_radius, float4* acc,
                                     const float4* part, int jsplit, int n, float dt, float size,
                                     int wrap, cudaStream_t stream, uint64_t* launches);
    cudaError_t launch_integrate_aos(float* bodies, const float4* part, int jsplit, int n,
                                     float dt, float size, int wrap, cudaStream_t stream,
                                     uint64_t* launches);

    // Body (48 B) <-> split streams (integrate.cu).
    cudaError_t launch_split(const float* bodies, float4* pos_mass, float4* vel_radius,
                             float4* acc, int n, cudaStream_t stream, uint64_t* launches);
    cudaError_t launch_join(const float4* pos_mass, const float4* vel_radius, const float4* acc,
                            float* bodies, int n, cudaStream_t stream, uint64_t* launches);
}
