// Semi-implicit Euler and the Body <-> split-stream conversions, for sm_103a.
//
// Reference: detail::integrate_euler and detail::wrap (source/detail/physics.h:50-70),
// run per body by CpuSolver::integrate (source/solvers/cpu_solver.h:29-42); the shader
// twins are shaders/integrate.comp and integrate_split.comp. The arithmetic here is the
// CPU form operation for operation -- v = v + a*dt and x = x + v*dt as separate
// round-to-nearest multiply and add (no FMA contraction), wrap with two exact fmodf --
// so the result is bit-identical to the reference CPU integrator.
//
// Memory-bound: one 16-byte load per stream per body and one store per written stream,
// fully coalesced. When the accelerate left j-split partials, their fixed-order sum is
// fused in here (the reduction and the update share one pass over the bodies).
#include "common.cuh"
#include "direct.cuh"

namespace nbg
{
    __device__ __forceinline__ float wrap1(const float x, const float size)
    {
        const float half = __fmul_rn(size, .5f);
        return __fsub_rn(fmodf(__fadd_rn(fmodf(__fadd_rn(x, half), size), size), size), half);
    }

    __device__ __forceinline__ void euler(float& x, float& v, const float a, const float dt)
    {
        v = __fadd_rn(v, __fmul_rn(a, dt));
        x = __fadd_rn(x, __fmul_rn(v, dt));
    }

    // W lanes per body combine the partials (combine_partials_w); lane 0 integrates
    template <int W>
    __global__ void integrate_soa_kernel(float4* __restrict__ pm, float4* __restrict__ vr,
                                         float4* __restrict__ acc, const float4* __restrict__ part,
                                         const int js, const int n, const float G, const float dt,
                                         const float size, const int wrap)
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        const int i = t / W, g = t % W;
        if (W == 1 && i >= n)
            return;
        float3 a = make_float3(0.f, 0.f, 0.f);
        if (part)
            a = combine_partials_w<W>(part, part + n, js, n, min(i, n - 1), g, G);
        if (i >= n || g != 0)
            return;
        float4 p = pm[i];
        float4 v = vr[i];
        if (part)
            acc[i] = make_float4(a.x, a.y, a.z, 0.f);
        else
        {
            const float4 t4 = acc[i];
            a = make_float3(t4.x, t4.y, t4.z);
        }
        euler(p.x, v.x, a.x, dt);
        euler(p.y, v.y, a.y, dt);
        euler(p.z, v.z, a.z, dt);
        if (wrap && size > 0.f)
        {
            p.x = wrap1(p.x, size);
            p.y = wrap1(p.y, size);
            p.z = wrap1(p.z, size);
        }
        pm[i] = p;
        vr[i] = v;
    }

    template <int W>
    __global__ void integrate_aos_kernel(float* __restrict__ bodies, const float4* __restrict__ part,
                                         const int js, const int n, const float G, const float dt,
                                         const float size, const int wrap)
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        const int i = t / W, g = t % W;
        if (W == 1 && i >= n)
            return;
        float3 s = make_float3(0.f, 0.f, 0.f);
        if (part)
            s = combine_partials_w<W>(part, part + n, js, n, min(i, n - 1), g, G);
        if (i >= n || g != 0)
            return;
        float4* b = reinterpret_cast<float4*>(bodies) + static_cast<size_t>(i) * 3;
        float4 p = b[0];    // pos, radius
        float4 v = b[1];    // vel, mass
        float4 a = b[2];    // acc, pad
        if (part)
        {
            a.x = s.x;
            a.y = s.y;
            a.z = s.z;
            b[2] = a;
        }
        euler(p.x, v.x, a.x, dt);
        euler(p.y, v.y, a.y, dt);
        euler(p.z, v.z, a.z, dt);
        if (wrap && size > 0.f)
        {
            p.x = wrap1(p.x, size);
            p.y = wrap1(p.y, size);
            p.z = wrap1(p.z, size);
        }
        b[0] = p;
        b[1] = v;
    }

    // Body -> {pos, mass}, {vel, radius}, {acc, 0}: gpu_solver_split.h:163-172 on the device.
    __global__ void split_kernel(const float4* __restrict__ bodies, float4* __restrict__ pm,
                                 float4* __restrict__ vr, float4* __restrict__ acc, const int n)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        const float4 p = bodies[3 * static_cast<size_t>(i)];
        const float4 v = bodies[3 * static_cast<size_t>(i) + 1];
        const float4 a = bodies[3 * static_cast<size_t>(i) + 2];
        pm[i] = make_float4(p.x, p.y, p.z, v.w);
        vr[i] = make_float4(v.x, v.y, v.z, p.w);
        acc[i] = make_float4(a.x, a.y, a.z, 0.f);
    }

    // The inverse (materialize(), gpu_solver_split.h:203-218); Body::pad is written as 0.
    __global__ void join_kernel(const float4* __restrict__ pm, const float4* __restrict__ vr,
                                const float4* __restrict__ acc, float4* __restrict__ bodies,
                                const int n)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        const float4 p = pm[i];
        const float4 v = vr[i];
        const float4 a = acc[i];
        bodies[3 * static_cast<size_t>(i)] = make_float4(p.x, p.y, p.z, v.w);
        bodies[3 * static_cast<size_t>(i) + 1] = make_float4(v.x, v.y, v.z, p.w);
        bodies[3 * static_cast<size_t>(i) + 2] = make_float4(a.x, a.y, a.z, 0.f);
    }

    namespace
    {
        constexpr int kBlock = 256;
    }

    cudaError_t launch_integrate_soa(float4* pm, float4* vr, float4* acc, const float4* part,
                                     const int js, const int n, const float G, const float dt, const float size,
                                     const int wrap, cudaStream_t stream, uint64_t* launches)
    {
        if (n <= 0)
            return cudaSuccess;
        if (part && combine_width(n, js) == 8)
            integrate_soa_kernel<8><<<ceil_div(static_cast<size_t>(n) * 8, kBlock), kBlock, 0, stream>>>(
                pm, vr, acc, part, js, n, G, dt, size, wrap);
        else
            integrate_soa_kernel<1><<<ceil_div(n, kBlock), kBlock, 0, stream>>>(pm, vr, acc, part, js, n, G, dt, size,
                                                                             wrap);
        ++*launches;
        return cudaGetLastError();
    }

    cudaError_t launch_integrate_aos(float* bodies, const float4* part, const int js, const int n,
                                     const float G, const float dt, const float size, const int wrap,
                                     cudaStream_t stream, uint64_t* launches)
    {
        if (n <= 0)
            return cudaSuccess;
        if (part && combine_width(n, js) == 8)
            integrate_aos_kernel<8><<<ceil_div(static_cast<size_t>(n) * 8, kBlock), kBlock, 0, stream>>>(
                bodies, part, js, n, G, dt, size, wrap);
        else
            integrate_aos_kernel<1><<<ceil_div(n, kBlock), kBlock, 0, stream>>>(bodies, part, js, n, G, dt, size,
                                                                             wrap);
        ++*launches;
        return cudaGetLastError();
    }

    cudaError_t launch_split(const float* bodies, float4* pm, float4* vr, float4* acc, const int n,
                             cudaStream_t stream, uint64_t* launches)
    {
        if (n <= 0)
            return cudaSuccess;
        split_kernel<<<ceil_div(n, kBlock), kBlock, 0, stream>>>(reinterpret_cast<const float4*>(bodies), pm, vr, acc, n);
        ++*launches;
        return cudaGetLastError();
    }

    cudaError_t launch_join(const float4* pm, const float4* vr, const float4* acc, float* bodies,
                            const int n, cudaStream_t stream, uint64_t* launches)
    {
        if (n <= 0)
            return cudaSuccess;
        join_kernel<<<ceil_div(n, kBlock), kBlock, 0, stream>>>(pm, vr, acc, reinterpret_cast<float4*>(bodies), n);
        ++*launches;
        return cudaGetLastError();
    }
}
