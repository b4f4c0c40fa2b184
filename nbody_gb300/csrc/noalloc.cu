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
// not a device address -- so the address is looked up with cudaGetSymbolAddress, with
// the device current, once per CUDA context, and cached under that context's unique id.
// The module is loaded anew in every context (a second context on the same device, or
// the primary context re-created after cudaDeviceReset), so an address is never reused
// outside the context it came from.
#include <algorithm>
#include <mutex>

#include <cuda.h>       // CUcontext and CUresult only: the two driver calls are resolved at run time

#include "common.cuh"
#include "direct.cuh"

namespace
{
    // Partial accelerations of the source chunks: jsplit * n float4 must fit.
    constexpr size_t kNoAllocPartials = size_t(1) << 20;   // 16 MiB of float4
    constexpr int kCacheSlots = 64;

    static __device__ __align__(256) float4 g_noalloc_partials[kNoAllocPartials];
    static __device__ __align__(256) unsigned g_noalloc_error;

    struct DeviceScratch
    {
        unsigned long long ctx_id = 0;      // 0: an empty slot (context ids start at 1)
        float4* partials = nullptr;
        unsigned* error = nullptr;
    };

    using CtxGetCurrentFn = CUresult (*)(CUcontext*);
    using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

    std::mutex g_setup_mutex;
    DeviceScratch g_cache[kCacheSlots];
    int g_next_slot = 0;
    bool g_driver_resolved = false;
    CtxGetCurrentFn g_get_current = nullptr;
    CtxGetIdFn g_get_id = nullptr;

    cudaError_t lookup(DeviceScratch* out)
    {
        void* p = nullptr;
        void* e = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (err != cudaSuccess)
            return err;
        err = cudaGetSymbolAddress(&e, g_noalloc_error);
        if (err != cudaSuccess)
            return err;
        out->partials = static_cast<float4*>(p);
        out->error = static_cast<unsigned*>(e);
        return cudaSuccess;
    }

    // The device addresses of the two arrays in the calling thread's current context
    // (the device's primary context unless the caller made another one current). The
    // lookup runs on the first call in each context; later calls in the same context take
    // the cached addresses. Where the driver cannot name the context, every call looks
    // the addresses up again. Returns a cudaError_t.
    cudaError_t device_scratch(DeviceScratch* out)
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_driver_resolved)
        {
            g_driver_resolved = true;
            void* f = nullptr;
            void* g = nullptr;
            cudaDriverEntryPointQueryResult q1{}, q2{};
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
                cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
                q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess && f && g)
            {
                g_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
                g_get_id = reinterpret_cast<CtxGetIdFn>(g);
            }
            cudaGetLastError();
        }
        if (!g_get_current || !g_get_id)
            return lookup(out);
        CUcontext c = nullptr;
        if (g_get_current(&c) != CUDA_SUCCESS || !c)
        {
            // no context current yet: the runtime call creates the primary context
            if (const cudaError_t err = lookup(out))
                return err;
            if (g_get_current(&c) != CUDA_SUCCESS || !c)
                return cudaSuccess;     // addresses looked up, but nothing to key them on
        }
        unsigned long long id = 0;
        if (g_get_id(c, &id) != CUDA_SUCCESS || id == 0)
            return lookup(out);
        for (const DeviceScratch& s : g_cache)
            if (s.ctx_id == id)
            {
                *out = s;
                return cudaSuccess;
            }
        DeviceScratch s;
        if (const cudaError_t err = lookup(&s))
            return err;
        s.ctx_id = id;
        g_cache[g_next_slot] = s;
        g_next_slot = (g_next_slot + 1) % kCacheSlots;
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
    // every stream the kernel reads as float4 must be 16-byte aligned: the radii only under
    // the CUTOFF law
    const uintptr_t vr = p->law == NBODY_LAW_CUTOFF ? reinterpret_cast<uintptr_t>(vel_radius) : 0;
    if ((reinterpret_cast<uintptr_t>(pos_mass) | reinterpret_cast<uintptr_t>(acc) | vr) & 15u)
        return NBODY_ERR_INVALID;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return NBODY_ERR_NO_DEVICE;
    DeviceScratch s;
    if (device_scratch(&s) != cudaSuccess)
        return NBODY_ERR_CUDA;

    // The usual launch shape, with the source split capped so its partials fit: a chunk
    // leaves two float4 per body (its sum and the sum's compensation).
    DirectPlan plan = plan_direct(n, p->law, false);
    if (direct_scratch_bytes(plan, n) > kNoAllocPartials * sizeof(float4))
    {
        const size_t js = std::max<size_t>(1, kNoAllocPartials / (2 * n));
        size_t chunk = (n + js - 1) / js;
        const size_t unit = static_cast<size_t>(plan.tile) * plan.fold;
        chunk = (chunk + unit - 1) / unit * unit;
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
