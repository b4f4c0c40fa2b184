// Internal interface of the direct-sum kernels (direct.cu, direct_precise.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

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
        int chunk;      // sources per chunk (a multiple of tile * fold)
        int fold;       // tiles per exact fold of the running sums (a function of n only)
        int grid_x;     // target blocks
        int law;
        bool aos;
    };

    // Bytes of j-split scratch one accelerate needs: per chunk and body, the chunk's FP32 sum
    // S and its compensation C (two float4). None without a split.
    inline size_t direct_scratch_bytes(const DirectPlan& plan, const size_t n)
    {
        return plan.jsplit > 1 ? 2 * static_cast<size_t>(plan.jsplit) * n * 16 : 0;
    }

    // The accelerations from the chunk partials of the FP32 direct sum: chunk c of body i
    // holds its (S, C) at S[2 c n + i] and C[2 c n + i] (C = S + n in the scratch layout).
    // The pairs are added over the chunks in chunk order as a double-float sum (TwoSum into
    // a running (s, e), the compensations added to e), then s + e is rounded to FP32 and
    // scaled by G: the same formula for one chunk or many, so the result does not depend on
    // how the sources were split. FP32 only: GB300's FP64 pipe runs at 1/64 of the FP32
    // rate, and a small system's few bodies would put that work on a few SMs.
    // W lanes per body (consecutive lanes of one warp, g = lane % W): lane g sums chunks g,
    // g + W, ... as above, and the lanes' double-float sums are then merged pairwise in a
    // fixed order (the same TwoSum step). Every lane of the warp must call it; the result is
    // lane g = 0's. W = 1 is the plain sequential sum.
    template <int W>
    __device__ __forceinline__ float3 combine_partials_w(const float4* __restrict__ S, const float4* __restrict__ C,
                                                         const int js, const int n, const int i, const int g,
                                                         const float G)
    {
        float sx = 0.f, sy = 0.f, sz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll 4
        for (int c = g; c < js; c += W)
        {
            const size_t k = 2 * static_cast<size_t>(c) * n + i;
            const float4 s = S[k], e = C[k];
            float t, r;
            two_sum(sx, s.x, t, r);
            sx = t;
            ex = __fadd_rn(ex, __fadd_rn(r, e.x));
            two_sum(sy, s.y, t, r);
            sy = t;
            ey = __fadd_rn(ey, __fadd_rn(r, e.y));
            two_sum(sz, s.z, t, r);
            sz = t;
            ez = __fadd_rn(ez, __fadd_rn(r, e.z));
        }
#pragma unroll
        for (int off = W / 2; off > 0; off >>= 1)
        {
            const float osx = __shfl_down_sync(0xffffffffu, sx, off, W), oex = __shfl_down_sync(0xffffffffu, ex, off, W);
            const float osy = __shfl_down_sync(0xffffffffu, sy, off, W), oey = __shfl_down_sync(0xffffffffu, ey, off, W);
            const float osz = __shfl_down_sync(0xffffffffu, sz, off, W), oez = __shfl_down_sync(0xffffffffu, ez, off, W);
            float t, r;
            two_sum(sx, osx, t, r);
            sx = t;
            ex = __fadd_rn(ex, __fadd_rn(r, oex));
            two_sum(sy, osy, t, r);
            sy = t;
            ey = __fadd_rn(ey, __fadd_rn(r, oey));
            two_sum(sz, osz, t, r);
            sz = t;
            ez = __fadd_rn(ez, __fadd_rn(r, oez));
        }
        return make_float3(G * __fadd_rn(sx, ex), G * __fadd_rn(sy, ey), G * __fadd_rn(sz, ez));
    }

    __device__ __forceinline__ float3 combine_partials(const float4* __restrict__ S, const float4* __restrict__ C,
                                                       const int js, const int n, const int i, const float G)
    {
        return combine_partials_w<1>(S, C, js, n, i, 0, G);
    }

    // Lanes per body for the combine: a small system has many chunks and few bodies, so eight
    // lanes a body spread the combine over eight times the SMs. A function of (n, js) only,
    // so the sums do not depend on which kernel combines them.
    inline int combine_width(const int n, const int js) { return (js >= 8 && n <= (1 << 16)) ? 8 : 1; }

    // Pick a launch shape for n bodies. force_variant >= 0 pins the (T, block) entry.
    DirectPlan plan_direct(size_t n, int law, bool aos, int force_variant = -1);

    // The instantiated kernel shapes: targets per thread, threads per CTA, packed FP32x2 or not.
    int direct_variant_count();
    void direct_variant_describe(int i, int* T, int* block, int* packed);

    // Queue the accelerate. src is pos_mass (SoA) or the Body array viewed as float4
    // (AoS). Results: acc (SoA) or Body::acc in body_out (AoS). scratch must hold
    // direct_scratch_bytes(plan, n); with reduce == false the partials are left there for
    // the fused integrate to sum.
    cudaError_t launch_direct(const DirectPlan& plan, const float4* src, const float4* vel_radius,
                              float4* acc, float* body_out, float4* scratch, int n, float G,
                              float eps2, unsigned* err, cudaStream_t stream, uint64_t* launches,
                              bool reduce = true);

    cudaError_t launch_reduce(const float4* scratch, int jsplit, int n, float G, float4* acc,
                              float* body_out, cudaStream_t stream, uint64_t* launches);

    // Semi-implicit Euler (integrate.cu). When part != nullptr the accelerations are
    // combine_partials over its jsplit chunks (with G), also written to acc / Body::acc.
    cudaError_t launch_integrate_soa(float4* pos_mass, float4* vel_radius, float4* acc,
                                     const float4* part, int jsplit, int n, float G, float dt,
                                     float size, int wrap, cudaStream_t stream, uint64_t* launches);
    cudaError_t launch_integrate_aos(float* bodies, const float4* part, int jsplit, int n,
                                     float G, float dt, float size, int wrap, cudaStream_t stream,
                                     uint64_t* launches);

    // Body (48 B) <-> split streams (integrate.cu).
    cudaError_t launch_split(const float* bodies, float4* pos_mass, float4* vel_radius,
                             float4* acc, int n, cudaStream_t stream, uint64_t* launches);
    cudaError_t launch_join(const float4* pos_mass, const float4* vel_radius, const float4* acc,
                            float* bodies, int n, cudaStream_t stream, uint64_t* launches);
}
