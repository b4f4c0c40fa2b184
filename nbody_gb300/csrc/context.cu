// The nbody_cuda context and the C ABI (include/nbody_cuda.h).
//
// A context owns the device copy of one simulation's bodies in one layout, a stream,
// pinned staging for host transfers, the scratch the kernels need, and a device error
// word. It plays the part GpuDevice plays for the reference's Vulkan variants
// (source/gpu.h:72-353): grow-only buffers with a live count (gpu.h:76-80), uploads of
// whole body arrays, downloads of selected streams (Readback, gpu.h:52-58).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "batch.cuh"
#include "bh.cuh"
#include "common.cuh"
#include "context.cuh"
#include "direct.cuh"

using namespace nbg;

namespace
{
    thread_local std::string g_create_error;
    thread_local int g_create_status = NBODY_OK;

    int fail(nbody_cuda* ctx, const int status, const char* fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        if (ctx)
        {
            ctx->last_error = buf;
            ctx->last_status = status;
        }
        else
        {
            g_create_error = buf;
            g_create_status = status;
        }
        if (std::getenv("NBODY_CUDA_VERBOSE"))
            std::fprintf(stderr, "nbody_cuda: %s\n", buf);
        return status;
    }

    int cuda_fail(nbody_cuda* ctx, const cudaError_t e, const char* what)
    {
        const int st = (e == cudaErrorMemoryAllocation) ? NBODY_ERR_ALLOC : NBODY_ERR_CUDA;
        return fail(ctx, st, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    }

#define NBG_CUDA(ctx, call, what)                       \
    do                                                  \
    {                                                   \
        const cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess)                          \
            return cuda_fail((ctx), e_, (what));        \
    } while (0)

    bool fault_injected(const char* what)
    {
        const char* f = std::getenv("NBODY_CUDA_FAULT");
        return f && std::strcmp(f, what) == 0;
    }

    int check_params(nbody_cuda* ctx, const nbody_step_params* p)
    {
        if (!p)
            return fail(ctx, NBODY_ERR_INVALID, "null step parameters");
        if (p->law != NBODY_LAW_CUTOFF && p->law != NBODY_LAW_SOFTENED)
            return fail(ctx, NBODY_ERR_INVALID, "unknown force law %d", p->law);
        if (p->law == NBODY_LAW_SOFTENED && !(p->eps2 > 0.f))
            return fail(ctx, NBODY_ERR_INVALID, "the softened law needs eps2 > 0 (got %g)", p->eps2);
        if (p->mode != NBODY_MODE_N2 && p->mode != NBODY_MODE_NLOGN && p->mode != NBODY_MODE_BATCHED)
            return fail(ctx, NBODY_ERR_INVALID, "unknown mode %d", p->mode);
        if (p->precision < NBODY_PREC_FP32 || p->precision > NBODY_PREC_FP64)
            return fail(ctx, NBODY_ERR_INVALID, "unknown precision %d", p->precision);
        if (p->walk != NBODY_WALK_TARGET && p->walk != NBODY_WALK_GROUP)
            return fail(ctx, NBODY_ERR_INVALID, "unknown Barnes-Hut walk %d", p->walk);
        return NBODY_OK;
    }
}

// ---------------------------------------------------------------------------------------
// internal helpers shared with the other translation units
// ---------------------------------------------------------------------------------------
namespace nbg
{
    bool is_pinned(const void* p)
    {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeHost;
    }

    int ctx_fail(nbody_cuda* ctx, const int status, const char* msg)
    {
        return fail(ctx, status, "%s", msg);
    }

    int ctx_cuda_fail(nbody_cuda* ctx, const cudaError_t e, const char* what)
    {
        return cuda_fail(ctx, e, what);
    }

    int before_allocation(nbody_cuda* ctx)
    {
        if (ctx->capturing)
            return fail(ctx, NBODY_ERR_UNSUPPORTED, "a device buffer would grow during graph capture");
        if (fault_injected("alloc"))
            return fail(ctx, NBODY_ERR_ALLOC, "injected allocation failure (NBODY_CUDA_FAULT=alloc)");
        ++ctx->generation;
        return NBODY_OK;
    }

    int ensure_scratch(nbody_cuda* ctx, const size_t bytes)
    {
        if (bytes <= ctx->scratch_bytes)
            return NBODY_OK;
        if (const int st = before_allocation(ctx))
            return st;
        if (ctx->scratch)
            cudaFreeAsync(ctx->scratch, ctx->stream);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        const size_t grow = std::max(bytes, ctx->scratch_bytes + ctx->scratch_bytes / 2);
        NBG_CUDA(ctx, cudaMallocAsync(&ctx->scratch, grow, ctx->stream), "scratch allocation");
        ctx->scratch_bytes = grow;
        return NBODY_OK;
    }

    int check_device_error(nbody_cuda* ctx)
    {
        unsigned word = 0;
        NBG_CUDA(ctx, cudaMemcpyAsync(&word, ctx->dev_error, sizeof word, cudaMemcpyDeviceToHost, ctx->stream),
                 "device error word readback");
        NBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize");
        if (!word)
            return NBODY_OK;
        NBG_CUDA(ctx, cudaMemsetAsync(ctx->dev_error, 0, sizeof(unsigned), ctx->stream), "error word reset");
        if (word & DEV_ERR_TIMEOUT)
            return fail(ctx, NBODY_ERR_TIMEOUT, "a bounded device wait timed out (device error word 0x%x)", word);
        return fail(ctx, NBODY_ERR_CUDA, "device-side check failed (device error word 0x%x)", word);
    }
}

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
extern "C" {

int nbody_cuda_probe(char* why, const size_t why_len)
{
    auto say = [&](const char* msg) {
        if (why && why_len)
        {
            std::strncpy(why, msg, why_len - 1);
            why[why_len - 1] = 0;
        }
    };
    if (fault_injected("nodevice"))
    {
        say("injected: no CUDA device (NBODY_CUDA_FAULT=nodevice)");
        return NBODY_ERR_NO_DEVICE;
    }
    int count = 0;
    const cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
    {
        char buf[256];
        std::snprintf(buf, sizeof buf, "no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "none found");
        cudaGetLastError();
        say(buf);
        return NBODY_ERR_NO_DEVICE;
    }
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3)
    {
        char buf[256];
        std::snprintf(buf, sizeof buf, "device %d is sm_%d%d; this build is for sm_103a (GB300) only", dev, major, minor);
        say(buf);
        return NBODY_ERR_UNSUPPORTED;
    }
    say("");
    return NBODY_OK;
}

int nbody_cuda_create(nbody_cuda** out, const int layout)
{
    if (!out)
        return fail(nullptr, NBODY_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (layout != NBODY_LAYOUT_SOA && layout != NBODY_LAYOUT_AOS)
        return fail(nullptr, NBODY_ERR_INVALID, "unknown layout %d", layout);
    char why[256];
    const int st = nbody_cuda_probe(why, sizeof why);
    if (st != NBODY_OK)
        return fail(nullptr, st, "%s", why);
    if (fault_injected("alloc"))
        return fail(nullptr, NBODY_ERR_ALLOC, "injected allocation failure (NBODY_CUDA_FAULT=alloc)");

    nbody_cuda* ctx = new (std::nothrow) nbody_cuda();
    if (!ctx)
        return fail(nullptr, NBODY_ERR_ALLOC, "host allocation failed");
    ctx->layout = layout;
    cudaGetDevice(&ctx->device);
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&ctx->dev_error, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaMemset(ctx->dev_error, 0, sizeof(unsigned));
    if (e != cudaSuccess)
    {
        const int s = cuda_fail(nullptr, e, "context creation");
        nbody_cuda_destroy(ctx);
        return s;
    }
    ctx->stream = ctx->own_stream;
    cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, ctx->device);
    cudaDeviceGetAttribute(&ctx->pageable_host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device);
    cudaGetLastError();
    // NBODY_CUDA_TRANSFER=staged|mapped|direct picks the initial transfer path (default auto),
    // so that a whole program can be run over each path unchanged.
    if (const char* t = std::getenv("NBODY_CUDA_TRANSFER"))
    {
        const int policy = !std::strcmp(t, "staged") ? NBODY_TRANSFER_STAGED
                           : !std::strcmp(t, "mapped") ? NBODY_TRANSFER_MAPPED
                           : (!std::strcmp(t, "direct") && ctx->pageable_access) ? NBODY_TRANSFER_DIRECT
                                                                                 : NBODY_TRANSFER_AUTO;
        ctx->transfer = policy;
    }
    *out = ctx;
    return NBODY_OK;
}

void nbody_cuda_destroy(nbody_cuda* ctx)
{
    if (!ctx)
        return;
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    release_bh(ctx);
    release_precise(ctx);
    release_batch(ctx);
    release_transfer(ctx);
    release_query(ctx);
    if (ctx->graph)
        cudaGraphExecDestroy(ctx->graph);
    cudaFree(ctx->pm);
    cudaFree(ctx->vr);
    cudaFree(ctx->acc);
    cudaFree(ctx->bodies);
    cudaFree(ctx->aos_stage);
    cudaFree(ctx->scratch);
    cudaFree(ctx->dev_error);
    cudaFreeHost(ctx->pinned);
    if (ctx->pinned_event)
        cudaEventDestroy(ctx->pinned_event);
    if (ctx->own_stream)
        cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int nbody_cuda_last_error(const nbody_cuda* ctx, char* buf, const size_t len)
{
    const std::string& msg = ctx ? ctx->last_error : g_create_error;
    if (buf && len)
    {
        std::strncpy(buf, msg.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return ctx ? ctx->last_status : g_create_status;
}

int nbody_cuda_set_stream(nbody_cuda* ctx, void* stream)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    if (s != ctx->stream)
    {
        // Order the new stream after everything queued so far.
        cudaEvent_t ev;
        NBG_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event create");
        cudaEventRecord(ev, ctx->stream);
        cudaStreamWaitEvent(s, ev, 0);
        cudaEventDestroy(ev);
        ctx->stream = s;
        ++ctx->generation;
    }
    return NBODY_OK;
}

void* nbody_cuda_stream(const nbody_cuda* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }
int nbody_cuda_layout(const nbody_cuda* ctx) { return ctx ? ctx->layout : -1; }
size_t nbody_cuda_count(const nbody_cuda* ctx) { return ctx ? ctx->count : 0; }
uint64_t nbody_cuda_launch_count(const nbody_cuda* ctx) { return ctx ? ctx->launches : 0; }

int nbody_cuda_last_direct_config(const nbody_cuda* ctx, int* T, int* block, int* tile, int* jsplit, int* grid)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    const DirectPlan& p = ctx->last_plan;
    if (T) *T = p.T;
    if (block) *block = p.block;
    if (tile) *tile = p.tile;
    if (jsplit) *jsplit = p.jsplit;
    if (grid) *grid = p.grid_x * p.jsplit;
    return NBODY_OK;
}

int nbody_cuda_reserve(nbody_cuda* ctx, const size_t n)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (n > static_cast<size_t>(INT32_MAX / 4))
        return fail(ctx, NBODY_ERR_INVALID, "body count %zu exceeds this build's limit", n);
    if (n <= ctx->cap)
        return NBODY_OK;
    if (const int st = before_allocation(ctx))
        return st;
    // Grow-only with headroom (Buffer::reserve, gpu.h:101-103); contents move with it.
    const size_t cap = std::max(n, ctx->cap + ctx->cap / 2);
    auto grow = [&](float4** p, const size_t per_body) -> int {
        float4* q = nullptr;
        NBG_CUDA(ctx, cudaMallocAsync(&q, cap * per_body, ctx->stream), "body storage allocation");
        if (*p && ctx->count)
            NBG_CUDA(ctx, cudaMemcpyAsync(q, *p, ctx->count * per_body, cudaMemcpyDeviceToDevice, ctx->stream), "body storage move");
        if (*p)
            cudaFreeAsync(*p, ctx->stream);
        *p = q;
        return NBODY_OK;
    };
    int st = NBODY_OK;
    if (ctx->layout == NBODY_LAYOUT_SOA)
    {
        if ((st = grow(&ctx->pm, 16)) || (st = grow(&ctx->vr, 16)) || (st = grow(&ctx->acc, 16)))
            return st;
    }
    else
    {
        float4* b = reinterpret_cast<float4*>(ctx->bodies);
        if ((st = grow(&b, 48)))
            return st;
        ctx->bodies = reinterpret_cast<float*>(b);
    }
    ctx->cap = cap;
    return NBODY_OK;
}

}   // extern "C"

namespace nbg
{
    // Pinned staging, reused across calls; waits for the previous transfer through it.
    int staging(nbody_cuda* ctx, const size_t bytes, void** out)
    {
        if (ctx->pinned_event)
            NBG_CUDA(ctx, cudaEventSynchronize(ctx->pinned_event), "staging wait");
        else
            NBG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->pinned_event, cudaEventDisableTiming), "event create");
        if (bytes > ctx->pinned_bytes)
        {
            cudaFreeHost(ctx->pinned);
            ctx->pinned = nullptr;
            ctx->pinned_bytes = 0;
            NBG_CUDA(ctx, cudaMallocHost(&ctx->pinned, bytes), "pinned staging allocation");
            ctx->pinned_bytes = bytes;
        }
        *out = ctx->pinned;
        return NBODY_OK;
    }

    // Host -> device copy of `bytes` from `src`: straight from page-locked memory
    // (waiting for it before returning, so the caller may reuse the buffer), or through
    // the pinned staging buffer.
    int h2d(nbody_cuda* ctx, void* dst, const void* src, const size_t bytes)
    {
        if (!bytes)
            return NBODY_OK;
        if (is_pinned(src))
        {
            NBG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "host to device copy");
            NBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "host to device copy");
            return NBODY_OK;
        }
        void* stage = nullptr;
        if (const int st = staging(ctx, bytes, &stage))
            return st;
        host_copy(stage, src, bytes);
        NBG_CUDA(ctx, cudaMemcpyAsync(dst, stage, bytes, cudaMemcpyHostToDevice, ctx->stream), "host to device copy");
        NBG_CUDA(ctx, cudaEventRecord(ctx->pinned_event, ctx->stream), "event record");
        return NBODY_OK;
    }

    // Device -> host, synchronous.
    int d2h(nbody_cuda* ctx, void* dst, const void* src, const size_t bytes)
    {
        if (!bytes)
            return NBODY_OK;
        if (is_pinned(dst))
        {
            NBG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "device to host copy");
            return check_device_error(ctx);
        }
        void* stage = nullptr;
        if (const int st = staging(ctx, bytes, &stage))
            return st;
        NBG_CUDA(ctx, cudaMemcpyAsync(stage, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "device to host copy");
        if (const int st = check_device_error(ctx))
            return st;
        host_copy(dst, stage, bytes);
        return NBODY_OK;
    }

    int ensure_aos_stage(nbody_cuda* ctx, const size_t n)
    {
        if (n <= ctx->aos_stage_cap)
            return NBODY_OK;
        if (const int st = before_allocation(ctx))
            return st;
        cudaFreeAsync(ctx->aos_stage, ctx->stream);
        ctx->aos_stage = nullptr;
        ctx->aos_stage_cap = 0;
        NBG_CUDA(ctx, cudaMallocAsync(&ctx->aos_stage, n * 48, ctx->stream), "body staging allocation");
        ctx->aos_stage_cap = n;
        return NBODY_OK;
    }
}

extern "C" {

int nbody_cuda_upload_bodies(nbody_cuda* ctx, const void* bodies, const size_t n)
{
    if (!ctx || (!bodies && n))
        return ctx ? fail(ctx, NBODY_ERR_INVALID, "null bodies") : NBODY_ERR_INVALID;
    if (const int st = nbody_cuda_reserve(ctx, n))
        return st;
    if (n != ctx->count)
        ++ctx->generation;      // the body count is an argument of captured launches
    ctx->count = n;
    ctx->origin_valid = false;
    ++ctx->body_version;
    if (!n)
        return NBODY_OK;
    return upload_records(ctx, bodies, n);
}

int nbody_cuda_download_bodies(nbody_cuda* ctx, void* bodies, const size_t n, const unsigned mask)
{
    if (!ctx || (!bodies && n))
        return ctx ? fail(ctx, NBODY_ERR_INVALID, "null bodies") : NBODY_ERR_INVALID;
    const size_t take = std::min(n, ctx->count);
    if (!take || !(mask & NBODY_READ_ALL))
        return check_device_error(ctx);
    if (const int st = sync_precise_positions(ctx))
        return st;
    return download_records(ctx, bodies, take, mask & NBODY_READ_ALL);
}

int nbody_cuda_upload_soa(nbody_cuda* ctx, const float* pos_mass, const float* vel_radius, const float* acc,
                          const size_t n)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (ctx->layout != NBODY_LAYOUT_SOA)
        return fail(ctx, NBODY_ERR_INVALID, "split-stream upload on an interleaved context");
    if (const int st = nbody_cuda_reserve(ctx, n))
        return st;
    if (n != ctx->count)
        ++ctx->generation;      // the body count is an argument of captured launches
    ctx->count = n;
    ctx->origin_valid = false;
    ++ctx->body_version;
    int st = NBODY_OK;
    if (pos_mass && (st = h2d(ctx, ctx->pm, pos_mass, n * 16)))
        return st;
    if (vel_radius && (st = h2d(ctx, ctx->vr, vel_radius, n * 16)))
        return st;
    if (acc && (st = h2d(ctx, ctx->acc, acc, n * 16)))
        return st;
    return NBODY_OK;
}

int nbody_cuda_download_soa(nbody_cuda* ctx, float* pos_mass, float* vel_radius, float* acc, const size_t n)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (ctx->layout != NBODY_LAYOUT_SOA)
        return fail(ctx, NBODY_ERR_INVALID, "split-stream download on an interleaved context");
    const size_t take = std::min(n, ctx->count);
    if (const int st = sync_precise_positions(ctx))
        return st;
    int st = NBODY_OK;
    if (pos_mass && (st = d2h(ctx, pos_mass, ctx->pm, take * 16)))
        return st;
    if (vel_radius && (st = d2h(ctx, vel_radius, ctx->vr, take * 16)))
        return st;
    if (acc && (st = d2h(ctx, acc, ctx->acc, take * 16)))
        return st;
    return check_device_error(ctx);
}

int nbody_cuda_synchronize(nbody_cuda* ctx)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    return check_device_error(ctx);
}

// --- stepping --------------------------------------------------------------------------

namespace
{
    int direct_accel(nbody_cuda* ctx, const nbody_step_params* p, const bool keep_partials)
    {
        const int n = static_cast<int>(ctx->count);
        const bool aos = ctx->layout == NBODY_LAYOUT_AOS;
        DirectPlan plan = plan_direct(ctx->count, p->law, aos, ctx->force_variant);
        ctx->last_plan = plan;
        if (plan.jsplit > 1)
            if (const int st = ensure_scratch(ctx, direct_scratch_bytes(plan, ctx->count)))
                return st;
        const float4* src = aos ? reinterpret_cast<const float4*>(ctx->bodies) : ctx->pm;
        float4* scratch = static_cast<float4*>(ctx->scratch);
        if (keep_partials && plan.jsplit > 1)
        {
            // The fused integrate sums the partials: launch the accelerate alone.
            const cudaError_t e = launch_direct(plan, src, ctx->vr, ctx->acc, ctx->bodies, scratch, n, p->G,
                                                p->eps2, ctx->dev_error, ctx->stream, &ctx->launches, false);
            if (e != cudaSuccess)
                return cuda_fail(ctx, e, "direct-sum launch");
            ctx->pending_partials = plan.jsplit;
            ctx->pending_G = p->G;
            return NBODY_OK;
        }
        ctx->pending_partials = 0;
        const cudaError_t e = launch_direct(plan, src, ctx->vr, ctx->acc, ctx->bodies, scratch, n, p->G, p->eps2,
                                            ctx->dev_error, ctx->stream, &ctx->launches);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "direct-sum launch");
        return NBODY_OK;
    }

    int do_integrate(nbody_cuda* ctx, const nbody_step_params* p)
    {
        const int n = static_cast<int>(ctx->count);
        const float4* part = ctx->pending_partials > 1 ? static_cast<const float4*>(ctx->scratch) : nullptr;
        const int js = ctx->pending_partials;
        ctx->pending_partials = 0;
        cudaError_t e;
        if (ctx->layout == NBODY_LAYOUT_SOA)
            e = launch_integrate_soa(ctx->pm, ctx->vr, ctx->acc, part, js, n, ctx->pending_G, p->dt, p->size, p->wrap,
                                     ctx->stream, &ctx->launches);
        else
            e = launch_integrate_aos(ctx->bodies, part, js, n, ctx->pending_G, p->dt, p->size, p->wrap, ctx->stream,
                                     &ctx->launches);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "integrate launch");
        return NBODY_OK;
    }

    int accelerate_impl(nbody_cuda* ctx, const nbody_step_params* p, const bool fuse_with_integrate)
    {
        if (p->mode == NBODY_MODE_BATCHED)
            return batch_accelerate(ctx, p);
        if (p->precision == NBODY_PREC_COMPENSATED || p->precision == NBODY_PREC_FP64)
            return precise_accelerate(ctx, p);
        if (p->mode == NBODY_MODE_NLOGN)
            return bh_accelerate(ctx, p);
        return direct_accel(ctx, p, fuse_with_integrate);
    }

    int integrate_impl(nbody_cuda* ctx, const nbody_step_params* p)
    {
        if (p->precision == NBODY_PREC_COMPENSATED)
            return precise_integrate(ctx, p);
        // an FP32 step moves the float positions past the split state: rebuild it later
        ctx->origin_valid = false;
        return do_integrate(ctx, p);
    }
}

int nbody_cuda_accelerate(nbody_cuda* ctx, const nbody_step_params* p)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!ctx->count)
        return NBODY_OK;
    ++ctx->body_version;
    return accelerate_impl(ctx, p, false);
}

int nbody_cuda_integrate(nbody_cuda* ctx, const nbody_step_params* p)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!ctx->count)
        return NBODY_OK;
    ctx->pending_partials = 0;
    ++ctx->body_version;
    return integrate_impl(ctx, p);
}

int nbody_cuda_update(nbody_cuda* ctx, const nbody_step_params* p, const int steps)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (steps < 0)
        return fail(ctx, NBODY_ERR_INVALID, "negative step count");
    if (!ctx->count)
        return NBODY_OK;
    ++ctx->body_version;
    for (int s = 0; s < steps; ++s)
    {
        if (const int st = accelerate_impl(ctx, p, true))
            return st;
        if (const int st = integrate_impl(ctx, p))
            return st;
    }
    return NBODY_OK;
}

// --- Barnes-Hut introspection ----------------------------------------------------------------

int nbody_cuda_bh_stats(nbody_cuda* ctx, uint64_t out[3])
{
    if (!ctx || !out)
        return NBODY_ERR_INVALID;
    unsigned long long v[3];
    const int st = bh_stats(ctx, v);
    for (int k = 0; k < 3; ++k)
        out[k] = v[k];
    return st;
}

int nbody_cuda_bh_stage_ms(nbody_cuda* ctx, float ms[2])
{
    if (!ctx || !ms)
        return NBODY_ERR_INVALID;
    return bh_stage_ms(ctx, ms);
}

int nbody_cuda_morton(nbody_cuda* ctx, const nbody_step_params* p, uint64_t* codes, uint32_t* order, double box[4])
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    return bh_morton(ctx, p, codes, order, box);
}

int nbody_cuda_direct_variant_count(void) { return direct_variant_count(); }

int nbody_cuda_direct_variant(const int index, int* T, int* block, int* packed)
{
    if (index < 0 || index >= direct_variant_count())
        return NBODY_ERR_INVALID;
    int a = 0, b = 0, c = 0;
    direct_variant_describe(index, &a, &b, &c);
    if (T) *T = a;
    if (block) *block = b;
    if (packed) *packed = c;
    return NBODY_OK;
}

int nbody_cuda_set_direct_variant(nbody_cuda* ctx, const int index)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (index >= direct_variant_count())
        return fail(ctx, NBODY_ERR_INVALID, "no direct-sum kernel shape %d", index);
    ctx->force_variant = index < 0 ? -1 : index;
    return NBODY_OK;
}

int nbody_cuda_direct_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms, size_t ntimes,
                               int* best)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!ctx->count)
        return fail(ctx, NBODY_ERR_INVALID, "no bodies to tune on");
    nbody_step_params q = *p;
    q.mode = NBODY_MODE_N2;
    q.precision = NBODY_PREC_FP32;
    EventPair ev;
    if (ev.status != cudaSuccess)
        return cuda_fail(ctx, ev.status, "event create");
    // one untimed launch first, so the clocks are up before the first shape is timed
    ctx->force_variant = -1;
    if (const int st = direct_accel(ctx, &q, false))
        return st;
    int best_i = 0;
    float best_ms = 1e30f;
    for (int i = 0; i < direct_variant_count(); ++i)
    {
        ctx->force_variant = i;
        float ms_best = 1e30f;
        for (int rep = 0; rep < 2; ++rep)
        {
            cudaEventRecord(ev.start, ctx->stream);
            const int st = direct_accel(ctx, &q, false);
            cudaEventRecord(ev.stop, ctx->stream);
            if (st != NBODY_OK)
            {
                ctx->force_variant = -1;
                return st;
            }
            ms_best = std::min(ms_best, ev.elapsed_ms());
        }
        if (times_ms && static_cast<size_t>(i) < ntimes)
            times_ms[i] = ms_best;
        if (ms_best < best_ms)
        {
            best_ms = ms_best;
            best_i = i;
        }
    }
    ctx->force_variant = best_i;
    if (best)
        *best = best_i;
    return check_device_error(ctx);
}

int nbody_cuda_set_systems(nbody_cuda* ctx, const int64_t* offsets, size_t nsys)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    return batch_set_systems(ctx, offsets, nsys);
}

int nbody_cuda_batch_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms, size_t ntimes, int* best)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    std::vector<double> t(static_cast<size_t>(batch_config_count()), 0.0);
    const int st = batch_autotune(ctx, p, t.data(), best);
    if (times_ms)
        for (size_t i = 0; i < ntimes && i < t.size(); ++i)
            times_ms[i] = t[i];
    return st;
}

int nbody_cuda_batch_config_count(void) { return batch_config_count(); }

int nbody_cuda_batch_config(const nbody_cuda* ctx, int index, int* tpt, int* t, int* unroll)
{
    if (index < 0)
        index = ctx ? batch_get_config(ctx) : 0;
    if (index >= batch_config_count())
        return NBODY_ERR_INVALID;
    int a = 0, b = 0, c = 0;
    batch_config_describe(index, &a, &b, &c);
    if (tpt) *tpt = a;
    if (t) *t = b;
    if (unroll) *unroll = c;
    return NBODY_OK;
}

int nbody_cuda_batch_set_config(nbody_cuda* ctx, int index)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    return batch_set_config(ctx, index);
}

int nbody_cuda_system_energy(nbody_cuda* ctx, const nbody_step_params* p, double* out, size_t nsys)
{
    if (!ctx || !out)
        return NBODY_ERR_INVALID;
    if (!p)
        return fail(ctx, NBODY_ERR_INVALID, "null step parameters");
    const size_t have = std::max<size_t>(1, batch_system_count(ctx));
    if (nsys < have)
        return fail(ctx, NBODY_ERR_INVALID, "output holds %zu systems, the table has %zu", nsys, have);
    nbody_step_params q = *p;
    if (q.law != NBODY_LAW_SOFTENED)
        q.eps2 = 0.f;
    return batch_energy(ctx, &q, out);
}

int nbody_cuda_energy(nbody_cuda* ctx, const nbody_step_params* p, double out[5])
{
    if (!ctx || !out)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (ctx->capturing)
        return fail(ctx, NBODY_ERR_UNSUPPORTED, "energy diagnostics are synchronous");
    if (const int st = energy_all(ctx, p, out))
        return st;
    return check_device_error(ctx);
}

int nbody_cuda_update_graph(nbody_cuda* ctx, const nbody_step_params* p, const int steps)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (steps < 0)
        return fail(ctx, NBODY_ERR_INVALID, "negative step count");
    if (!ctx->count || steps == 0)
        return NBODY_OK;
    ++ctx->body_version;
    // The first step runs eagerly: it grows every buffer the step needs, so nothing
    // allocates while the step is captured.
    if (const int st = nbody_cuda_update(ctx, p, 1))
        return st;
    if (steps == 1)
        return NBODY_OK;
    const bool stale = !ctx->graph || ctx->graph_generation != ctx->generation || ctx->graph_count != ctx->count
                       || ctx->graph_stream != ctx->stream
                       || std::memcmp(&ctx->graph_params, p, sizeof *p) != 0;
    if (stale)
    {
        if (ctx->graph)
            cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
        const uint64_t gen = ctx->generation;
        const uint64_t launches_before = ctx->launches;
        NBG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
        ctx->capturing = true;
        int st = accelerate_impl(ctx, p, true);
        if (st == NBODY_OK)
            st = integrate_impl(ctx, p);
        ctx->capturing = false;
        // captured, not run: count the kernels once per replay instead
        ctx->graph_launches = ctx->launches - launches_before;
        ctx->launches = launches_before;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (st != NBODY_OK || e != cudaSuccess || gen != ctx->generation)
        {
            if (g)
                cudaGraphDestroy(g);
            cudaGetLastError();
            if (st != NBODY_OK)
                return st;
            return e != cudaSuccess ? cuda_fail(ctx, e, "graph capture")
                                    : fail(ctx, NBODY_ERR_CUDA, "buffers changed during graph capture");
        }
        const cudaError_t ie = cudaGraphInstantiate(&ctx->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
        {
            ctx->graph = nullptr;
            return cuda_fail(ctx, ie, "graph instantiate");
        }
        ctx->graph_generation = ctx->generation;
        ctx->graph_count = ctx->count;
        ctx->graph_stream = ctx->stream;
        ctx->graph_params = *p;
    }
    for (int s = 1; s < steps; ++s)
    {
        NBG_CUDA(ctx, cudaGraphLaunch(ctx->graph, ctx->stream), "graph launch");
        ctx->launches += ctx->graph_launches;
    }
    ctx->tree_export_id = 0;    // replays rebuilt the tree without the host noticing
    return NBODY_OK;
}

int nbody_cuda_accel_sampled(nbody_cuda* ctx, const nbody_step_params* p, const int64_t* targets, size_t nt,
                             double* acc_out)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (nt && (!targets || !acc_out))
        return fail(ctx, NBODY_ERR_INVALID, "null target list or output");
    return precise_sampled(ctx, p, targets, nt, acc_out);
}

int nbody_cuda_split_origin(nbody_cuda* ctx, double out[4])
{
    if (!ctx || !out)
        return NBODY_ERR_INVALID;
    return precise_origin(ctx, out);
}

// --- caller-owned device buffers -----------------------------------------------------------

int nbody_cuda_dev_accel_soa(nbody_cuda* ctx, const void* pos_mass, const void* vel_radius, void* acc,
                             const size_t n, const nbody_step_params* p)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!n)
        return NBODY_OK;
    if (!pos_mass || !acc || (p->law == NBODY_LAW_CUTOFF && !vel_radius))
        return fail(ctx, NBODY_ERR_INVALID, "null device buffer");
    const uintptr_t vr = p->law == NBODY_LAW_CUTOFF ? reinterpret_cast<uintptr_t>(vel_radius) : 0;
    if ((reinterpret_cast<uintptr_t>(pos_mass) | reinterpret_cast<uintptr_t>(acc) | vr) & 15u)
        return fail(ctx, NBODY_ERR_INVALID, "device buffers must be 16-byte aligned");
    if (n > static_cast<size_t>(INT32_MAX / 4))
        return fail(ctx, NBODY_ERR_INVALID, "body count too large");
    if (p->mode != NBODY_MODE_N2 || p->precision != NBODY_PREC_FP32)
        return fail(ctx, NBODY_ERR_UNSUPPORTED, "caller-buffer accelerate is direct-sum FP32 only");
    const DirectPlan plan = plan_direct(n, p->law, false, ctx->force_variant);
    ctx->last_plan = plan;
    if (plan.jsplit > 1)
        if (const int st = ensure_scratch(ctx, direct_scratch_bytes(plan, n)))
            return st;
    const cudaError_t e = launch_direct(plan, static_cast<const float4*>(pos_mass), static_cast<const float4*>(vel_radius),
                                        static_cast<float4*>(acc), nullptr, static_cast<float4*>(ctx->scratch),
                                        static_cast<int>(n), p->G, p->eps2, ctx->dev_error, ctx->stream, &ctx->launches);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "direct-sum launch");
    return NBODY_OK;
}

int nbody_cuda_dev_accel_aos(nbody_cuda* ctx, void* bodies, const size_t n, const nbody_step_params* p)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!n)
        return NBODY_OK;
    if (!bodies || (reinterpret_cast<uintptr_t>(bodies) & 15u))
        return fail(ctx, NBODY_ERR_INVALID, "device body buffer must be non-null and 16-byte aligned");
    if (n > static_cast<size_t>(INT32_MAX / 4))
        return fail(ctx, NBODY_ERR_INVALID, "body count too large");
    if (p->mode != NBODY_MODE_N2 || p->precision != NBODY_PREC_FP32)
        return fail(ctx, NBODY_ERR_UNSUPPORTED, "caller-buffer accelerate is direct-sum FP32 only");
    const DirectPlan plan = plan_direct(n, p->law, true, ctx->force_variant);
    ctx->last_plan = plan;
    if (plan.jsplit > 1)
        if (const int st = ensure_scratch(ctx, direct_scratch_bytes(plan, n)))
            return st;
    const cudaError_t e = launch_direct(plan, static_cast<const float4*>(bodies), nullptr, nullptr,
                                        static_cast<float*>(bodies), static_cast<float4*>(ctx->scratch),
                                        static_cast<int>(n), p->G, p->eps2, ctx->dev_error, ctx->stream, &ctx->launches);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "direct-sum launch");
    return NBODY_OK;
}

int nbody_cuda_dev_integrate_soa(nbody_cuda* ctx, void* pos_mass, void* vel_radius, const void* acc,
                                 const size_t n, const nbody_step_params* p)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (const int st = check_params(ctx, p))
        return st;
    if (!n)
        return NBODY_OK;
    if (!pos_mass || !vel_radius || !acc)
        return fail(ctx, NBODY_ERR_INVALID, "null device buffer");
    if (n > static_cast<size_t>(INT32_MAX / 4))
        return fail(ctx, NBODY_ERR_INVALID, "body count too large");
    const cudaError_t e = launch_integrate_soa(static_cast<float4*>(pos_mass), static_cast<float4*>(vel_radius),
                                               const_cast<float4*>(static_cast<const float4*>(acc)), nullptr, 0,
                                               static_cast<int>(n), p->G, p->dt, p->size, p->wrap, ctx->stream,
                                               &ctx->launches);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "integrate launch");
    return NBODY_OK;
}

} // extern "C"
