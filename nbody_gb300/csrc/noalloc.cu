// Direct-sum accelerate for callers that cannot allocate device memory.
//
// Who needs it: code that runs inside someone else's frame loop or memory budget -- a
// renderer or game engine calling the solver once per frame, a plugin host that owns
// every device allocation itself, a real-time loop that must never stall. cudaMalloc and
// cudaFree synchronise the whole device and may fail under a fixed budget, so such a
// caller cannot let the library allocate the j-split scratch on first use, as
// nbody_cuda_dev_accel_soa does through its context.
//
// This entry point keeps that scratch in a file-scope __device__ array instead. The array
// is part of the loaded module: every GPU that loads the library holds it (16 MiB of
// partial sums plus one error word) until the process exits. Host code cannot pass the
// array's name to a kernel -- on the host that name is only a stand-in for the symbol,
// not a device address -- so the address is looked up with cudaGetSymbolAddress once per
// device, with that device current, and cached.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "direct.cuh"

namespace
{
    // Partial accelerations of the source chunks: jsplit * n float4 must fit.
    constexpr size_t kNoAllocPartials = size_t(1) << 20;   // 16 MiB of float4
    constexpr int kMaxDevices = 64;

    static __device__ __align__(256) float4 g_noalloc_partials[kNoAllocPartials];
    static __device__ __align__(256) unsigned g_noalloc_error;

    struct DeviceScratch
    {
        float4* partials = nullptr;
        unsigned* error = nullptr;
    };

    std::mutex g_setup_mutex;
    DeviceScratch g_scratch[kMaxDevices];

    // Resolve the device addresses of the two arrays on the current device (first call on
    // each device only). Returns a cudaError_t.
    cudaError_t device_scratch(const int dev, DeviceScratch* out)
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        DeviceScratch& s = g_scratch[dev];
        if (!s.partials)
        {
            void* p = nullptr;
            void* e = nullptr;
            cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (err != cudaSuccess)
                return err;
            err = cudaGetSymbolAddress(&e, g_noalloc_error);
            if (err != cudaSuccess)
                return err;
            s.partials = static_cast<float4*>(p);
            s.error = static_cast<unsigned*>(e);
        }
        *out = s;
        return cudaSuccess;
    }
}

extern "C" int nbody_cuda_dev_accel_soa_noalloc(const void* pos_mass, const void* vel_radius, void* acc,
                                                const size_t n, const nbody_step_params* p, void* stream)
{
    using namespace nbg;
    if (!p)
        return NBODY_ERR_INVALID;
    if (p->law != NBODY_LAW_CUTOFF && p->law != NBODY_LAW_SOFTENED)
        return NBODY_ERR_INVALID;
    if (p->law == NBODY_LAW_SOFTENED && !(p->eps2 > 0.f))
        return NBODY_ERR_INVALID;
    if (p->mode != NBODY_MODE_N2 || p->precision != NBODY_PREC_FP32)
        return NBODY_ERR_UNSUPPORTED;
    if (n > kNoAllocPartials)
        return NBODY_ERR_INVALID;     // beyond the fixed scratch: at most 2^20 bodies
    if (n == 0)
        return NBODY_OK;
    if (!pos_mass || !acc || (p->law == NBODY_LAW_CUTOFF && !vel_radius))
        return NBODY_ERR_INVALID;
    if ((reinterpret_cast<uintptr_t>(pos_mass) | reinterpret_cast<uintptr_t>(acc)) & 15u)
        return NBODY_ERR_INVALID;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return NBODY_ERR_NO_DEVICE;
    DeviceScratch s;
    if (device_scratch(dev, &s) != cudaSuccess)
        return NBODY_ERR_CUDA;

    // The usual launch shape, with the source split capped so its partials fit.
    DirectPlan plan = plan_direct(n, p->law, false);
    if (static_cast<size_t>(plan.jsplit) * n > kNoAllocPartials)
    {
        const size_t js = std::max<size_t>(1, kNoAllocPartials / n);
        size_t chunk = (n + js - 1) / js;
        chunk = (chunk + plan.tile - 1) / plan.tile * plan.tile;
        plan.chunk = static_cast<int>(chunk);
        plan.jsplit = static_cast<int>((n + chunk - 1) / chunk);
    }

    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The error word keeps the previous call's value: clear it first.
    if (cudaMemsetAsync(s.error, 0, sizeof(unsigned), st) != cudaSuccess)
        return NBODY_ERR_CUDA;
    uint64_t launches = 0;
    if (launch_direct(plan, static_cast<const float4*>(pos_mass), static_cast<const float4*>(vel_radius),
                      static_cast<float4*>(acc), nullptr, s.partials, static_cast<int>(n), p->G, p->eps2,
                      s.error, st, &launches) != cudaSuccess)
        return NBODY_ERR_CUDA;
    unsigned word = 0;
    if (cudaMemcpyAsync(&word, s.error, sizeof word, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return NBODY_ERR_CUDA;
    return word ? NBODY_ERR_TIMEOUT : NBODY_OK;
}
