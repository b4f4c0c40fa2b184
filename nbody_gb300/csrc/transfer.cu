// Host transfers of Body records, and the predicted readback.
//
// The reference moves bodies through mapped staging allocations and re-interleaves them on
// the host (GpuSolverSplit::upload_bodies / materialize, gpu_solver_split.h:155-177,
// 188-221), reading back after a step what GpuSolverSplit::wanted_readback predicts the
// next frame will need (gpu_solver_split.h:122-132). Here the (de)interleave always runs
// on the device, and the bytes take one of three paths:
//   STAGED  device Body staging -> copy engine -> pinned staging -> host copy;
//   MAPPED  a kernel writes (reads) the records in page-locked mapped host memory directly,
//           then one host copy to (from) the caller's array;
//   DIRECT  a kernel writes (reads) the caller's own array over the coherent host link
//           (NVLink-C2C on GB300: the device walks the host's page tables), no staging.
// A field-masked download writes only the selected fields of each record, on the device
// for DIRECT, in the host merge otherwise. Host copies of more than a few MiB are split
// across threads.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kBlock = 256;
        constexpr size_t kRecord = 48;      // sizeof(Body), source/body.h:6-19

        // Body record: pos xyz, radius, vel xyz, mass, acc xyz, pad (floats 0..11).
        // Split streams: pm = {pos, mass}, vr = {vel, radius}, acc = {acc, 0}.
        //
        // A CTA stages its 256 records (12 KiB) in shared memory, so that the host-side
        // array is written (read) in contiguous 16-byte chunks by consecutive threads:
        // whole lines cross the host link instead of three strided partial writes per
        // record. A field-masked write reads the caller's records first and writes them
        // back whole with the selected fields replaced.
        template <bool AOS>
        __global__ void __launch_bounds__(kBlock) records_out_kernel(
            const float4* __restrict__ pm, const float4* __restrict__ vr, const float4* __restrict__ acc,
            const float4* __restrict__ aos, float4* __restrict__ dst, const int n, const unsigned mask)
        {
            __shared__ float4 tile[3 * kBlock];
            const int base = blockIdx.x * kBlock;
            const int m = min(kBlock, n - base);
            const size_t off = 3 * static_cast<size_t>(base);
            const int t = threadIdx.x;
            const bool all = mask == NBODY_READ_ALL;
            if (AOS && all)
            {
                for (int k = t; k < 3 * m; k += kBlock)
                    dst[off + k] = aos[off + k];
                return;
            }
            if (!all)
                for (int k = t; k < 3 * m; k += kBlock)
                    tile[k] = dst[off + k];
            __syncthreads();
            if (t < m)
            {
                float4 r0, r1, r2;
                if (AOS)
                {
                    r0 = aos[off + 3 * t];
                    r1 = aos[off + 3 * t + 1];
                    r2 = aos[off + 3 * t + 2];
                }
                else
                {
                    const float4 p = pm[base + t], v = vr[base + t], a = acc[base + t];
                    r0 = make_float4(p.x, p.y, p.z, v.w);
                    r1 = make_float4(v.x, v.y, v.z, p.w);
                    r2 = make_float4(a.x, a.y, a.z, 0.f);
                }
                if (all)
                {
                    tile[3 * t] = r0;
                    tile[3 * t + 1] = r1;
                    tile[3 * t + 2] = r2;
                }
                else
                {
                    float* d = reinterpret_cast<float*>(&tile[3 * t]);
                    if (mask & NBODY_READ_POSITIONS)
                    {
                        d[0] = r0.x; d[1] = r0.y; d[2] = r0.z; d[7] = r1.w;
                    }
                    if (mask & NBODY_READ_VELOCITIES)
                    {
                        d[3] = r0.w; d[4] = r1.x; d[5] = r1.y; d[6] = r1.z;
                    }
                    if (mask & NBODY_READ_ACCELERATIONS)
                    {
                        d[8] = r2.x; d[9] = r2.y; d[10] = r2.z;
                    }
                }
            }
            __syncthreads();
            for (int k = t; k < 3 * m; k += kBlock)
                dst[off + k] = tile[k];
        }

        // Host records (mapped or pageable) -> device layout, read in contiguous chunks.
        template <bool AOS>
        __global__ void __launch_bounds__(kBlock) records_in_kernel(
            const float4* __restrict__ src, float4* __restrict__ pm, float4* __restrict__ vr,
            float4* __restrict__ acc, float4* __restrict__ aos, const int n)
        {
            __shared__ float4 tile[3 * kBlock];
            const int base = blockIdx.x * kBlock;
            const int m = min(kBlock, n - base);
            const size_t off = 3 * static_cast<size_t>(base);
            const int t = threadIdx.x;
            if (AOS)
            {
                for (int k = t; k < 3 * m; k += kBlock)
                    aos[off + k] = src[off + k];
                return;
            }
            for (int k = t; k < 3 * m; k += kBlock)
                tile[k] = src[off + k];
            __syncthreads();
            if (t < m)
            {
                const float4 r0 = tile[3 * t], r1 = tile[3 * t + 1], r2 = tile[3 * t + 2];
                pm[base + t] = make_float4(r0.x, r0.y, r0.z, r1.w);
                vr[base + t] = make_float4(r1.x, r1.y, r1.z, r0.w);
                acc[base + t] = make_float4(r2.x, r2.y, r2.z, 0.f);
            }
        }

        // Run body(begin, end) over [0, n) split across host threads when the work is large.
        template <class F>
        void host_parallel(const size_t n, const size_t bytes, F&& body)
        {
            constexpr size_t kPerThread = size_t(8) << 20;
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const size_t want = std::min<size_t>(std::min<size_t>(hw, 32), bytes / kPerThread);
            if (want <= 1 || n < 2 * want)
            {
                body(size_t(0), n);
                return;
            }
            std::vector<std::thread> pool;
            pool.reserve(want - 1);
            const size_t step = (n + want - 1) / want;
            for (size_t t = 1; t < want; ++t)
            {
                const size_t b = t * step, e = std::min(n, b + step);
                if (b < e)
                    pool.emplace_back([&body, b, e] { body(b, e); });
            }
            body(size_t(0), std::min(n, step));
            for (std::thread& th : pool)
                th.join();
        }

        // Copy the selected fields of `count` records from src to dst (host memory).
        void merge_records(float* dst, const float* src, const size_t count, const unsigned mask)
        {
            if ((mask & NBODY_READ_ALL) == NBODY_READ_ALL)
            {
                host_parallel(count, count * kRecord, [&](const size_t b, const size_t e) {
                    std::memcpy(dst + 12 * b, src + 12 * b, (e - b) * kRecord);
                });
                return;
            }
            host_parallel(count, count * kRecord, [&](const size_t b, const size_t e) {
                for (size_t i = b; i < e; ++i)
                {
                    const float* s = src + 12 * i;
                    float* d = dst + 12 * i;
                    if (mask & NBODY_READ_POSITIONS)
                    {
                        d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; d[7] = s[7];
                    }
                    if (mask & NBODY_READ_VELOCITIES)
                    {
                        d[3] = s[3]; d[4] = s[4]; d[5] = s[5]; d[6] = s[6];
                    }
                    if (mask & NBODY_READ_ACCELERATIONS)
                    {
                        d[8] = s[8]; d[9] = s[9]; d[10] = s[10];
                    }
                }
            });
        }

        int resolve(const nbody_cuda* ctx)
        {
            if (ctx->transfer != NBODY_TRANSFER_AUTO)
                return ctx->transfer;
            return (ctx->pageable_access && ctx->pageable_host_tables) ? NBODY_TRANSFER_DIRECT : NBODY_TRANSFER_MAPPED;
        }

        // Whether every page of [p, p + bytes) is resident. The device writing pages that
        // were never touched has each one faulted in and zeroed on its behalf, far slower
        // than the CPU doing the same while it copies (800 MB: 198 ms against 13 ms on the
        // test box), so a DIRECT download into such memory takes the MAPPED path instead.
        bool pages_resident(const void* p, const size_t bytes)
        {
            static const size_t page = static_cast<size_t>(sysconf(_SC_PAGESIZE));
            const uintptr_t lo = reinterpret_cast<uintptr_t>(p) & ~(page - 1);
            const uintptr_t hi = reinterpret_cast<uintptr_t>(p) + bytes;
            std::vector<unsigned char> vec((hi - lo + page - 1) / page);
            if (mincore(reinterpret_cast<void*>(lo), hi - lo, vec.data()) != 0)
                return true;    // not a mapping mincore can describe: let the device try
            for (const unsigned char v : vec)
                if (!(v & 1))
                    return false;
            return true;
        }

        // The device address a kernel may use for host memory `p`: page-locked memory's
        // mapped address, or `p` itself when the device reaches pageable memory; null when
        // neither, or when `p` is not 16-byte aligned (the caller's path is then MAPPED).
        void* device_view(const nbody_cuda* ctx, void* p)
        {
            if (reinterpret_cast<uintptr_t>(p) % 16)
                return nullptr;     // the record kernels move 16-byte chunks
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
            {
                cudaGetLastError();
                return ctx->pageable_access ? p : nullptr;
            }
            if (a.type == cudaMemoryTypeHost)
                return a.devicePointer;
            if (a.type == cudaMemoryTypeUnregistered)
                return ctx->pageable_access ? p : nullptr;
            return nullptr;     // device or managed memory is not a host array
        }

        // Mapped staging of at least `bytes`, once its last device access has finished.
        int mapped_staging(nbody_cuda* ctx, const size_t bytes)
        {
            if (ctx->mapped_event)
            {
                const cudaError_t e = cudaEventSynchronize(ctx->mapped_event);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "mapped staging wait");
            }
            else
            {
                const cudaError_t e = cudaEventCreateWithFlags(&ctx->mapped_event, cudaEventDisableTiming);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "event create");
            }
            if (bytes <= ctx->mapped_bytes)
                return NBODY_OK;
            if (ctx->capturing)
                return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "host staging would grow during graph capture");
            const size_t grow = std::max(bytes, ctx->mapped_bytes + ctx->mapped_bytes / 2);
            cudaFreeHost(ctx->mapped);
            ctx->mapped = ctx->mapped_dev = nullptr;
            ctx->mapped_bytes = 0;
            ctx->readback_valid = false;
            cudaError_t e = cudaHostAlloc(&ctx->mapped, grow, cudaHostAllocMapped | cudaHostAllocPortable);
            if (e == cudaSuccess)
                e = cudaHostGetDevicePointer(&ctx->mapped_dev, ctx->mapped, 0);
            if (e != cudaSuccess)
            {
                cudaFreeHost(ctx->mapped);
                ctx->mapped = ctx->mapped_dev = nullptr;
                return ctx_cuda_fail(ctx, e, "mapped staging allocation");
            }
            ctx->mapped_bytes = grow;
            return NBODY_OK;
        }

        cudaError_t launch_out(nbody_cuda* ctx, void* dst_dev, const size_t count, const unsigned mask)
        {
            if (!count)
                return cudaSuccess;
            const int n = static_cast<int>(count);
            const unsigned blocks = static_cast<unsigned>((count + kBlock - 1) / kBlock);
            if (ctx->layout == NBODY_LAYOUT_AOS)
                records_out_kernel<true><<<blocks, kBlock, 0, ctx->stream>>>(
                    nullptr, nullptr, nullptr, reinterpret_cast<const float4*>(ctx->bodies), static_cast<float4*>(dst_dev),
                    n, mask);
            else
                records_out_kernel<false><<<blocks, kBlock, 0, ctx->stream>>>(ctx->pm, ctx->vr, ctx->acc, nullptr,
                                                                               static_cast<float4*>(dst_dev), n, mask);
            ++ctx->launches;
            return cudaGetLastError();
        }

        cudaError_t launch_in(nbody_cuda* ctx, const void* src_dev, const size_t count)
        {
            if (!count)
                return cudaSuccess;
            const int n = static_cast<int>(count);
            const unsigned blocks = static_cast<unsigned>((count + kBlock - 1) / kBlock);
            const float4* src = static_cast<const float4*>(src_dev);
            if (ctx->layout == NBODY_LAYOUT_AOS)
                records_in_kernel<true><<<blocks, kBlock, 0, ctx->stream>>>(src, nullptr, nullptr, nullptr,
                                                                             reinterpret_cast<float4*>(ctx->bodies), n);
            else
                records_in_kernel<false><<<blocks, kBlock, 0, ctx->stream>>>(src, ctx->pm, ctx->vr, ctx->acc, nullptr, n);
            ++ctx->launches;
            return cudaGetLastError();
        }

        // STAGED download: device Body staging (split layout), copy engine, host merge.
        int download_staged(nbody_cuda* ctx, void* bodies, const size_t take, const unsigned mask)
        {
            const float* dev = ctx->bodies;
            if (ctx->layout == NBODY_LAYOUT_SOA)
            {
                if (const int st = ensure_aos_stage(ctx, take))
                    return st;
                const cudaError_t e = launch_join(ctx->pm, ctx->vr, ctx->acc, ctx->aos_stage, static_cast<int>(take),
                                                  ctx->stream, &ctx->launches);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "join launch");
                dev = ctx->aos_stage;
            }
            if ((mask & NBODY_READ_ALL) == NBODY_READ_ALL && is_pinned(bodies))
                return d2h(ctx, bodies, dev, take * kRecord);
            void* stage = nullptr;
            if (const int st = staging(ctx, take * kRecord, &stage))
                return st;
            const cudaError_t e = cudaMemcpyAsync(stage, dev, take * kRecord, cudaMemcpyDeviceToHost, ctx->stream);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "device to host copy");
            if (const int st = check_device_error(ctx))
                return st;
            merge_records(static_cast<float*>(bodies), static_cast<const float*>(stage), take, mask);
            return NBODY_OK;
        }
    }

    void host_copy(void* dst, const void* src, const size_t bytes)
    {
        unsigned char* d = static_cast<unsigned char*>(dst);
        const unsigned char* s = static_cast<const unsigned char*>(src);
        constexpr size_t kChunk = 4096;
        const size_t chunks = (bytes + kChunk - 1) / kChunk;
        host_parallel(chunks, bytes, [&](const size_t b, const size_t e) {
            const size_t lo = b * kChunk, hi = std::min(bytes, e * kChunk);
            std::memcpy(d + lo, s + lo, hi - lo);
        });
    }

    int download_records(nbody_cuda* ctx, void* bodies, const size_t take, const unsigned mask)
    {
        // DIRECT first: one device pass straight into the caller's records beats a host copy
        // out of staging, even one already holding the current bodies
        const int path = resolve(ctx);
        if (path == NBODY_TRANSFER_DIRECT)
        {
            void* view = device_view(ctx, bodies);
            if (view && view == bodies && !pages_resident(bodies, take * kRecord))
                view = nullptr;     // pageable memory not yet touched: stage it (see pages_resident)
            if (view)
            {
                const cudaError_t e = launch_out(ctx, view, take, mask);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "record write launch");
                return check_device_error(ctx);
            }
        }
        // a predicted readback that is still current and holds every field asked for
        if (ctx->readback_valid && ctx->readback_version == ctx->body_version && ctx->readback_count >= take
            && !(mask & ~ctx->readback_mask))
        {
            const cudaError_t e = cudaEventSynchronize(ctx->mapped_event);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "readback wait");
            if (const int st = check_device_error(ctx))
                return st;
            merge_records(static_cast<float*>(bodies), static_cast<const float*>(ctx->mapped), take, mask);
            ++ctx->readback_hits;
            return NBODY_OK;
        }
        if (path == NBODY_TRANSFER_MAPPED || path == NBODY_TRANSFER_DIRECT)
        {
            if (const int st = mapped_staging(ctx, take * kRecord))
                return st;
            const cudaError_t e = launch_out(ctx, ctx->mapped_dev, take, NBODY_READ_ALL);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "record write launch");
            cudaEventRecord(ctx->mapped_event, ctx->stream);
            if (const int st = check_device_error(ctx))
                return st;
            // the staging now holds every field of the current bodies
            ctx->readback_valid = true;
            ctx->readback_version = ctx->body_version;
            ctx->readback_count = take;
            ctx->readback_mask = NBODY_READ_ALL;
            merge_records(static_cast<float*>(bodies), static_cast<const float*>(ctx->mapped), take, mask);
            return NBODY_OK;
        }
        return download_staged(ctx, bodies, take, mask);
    }

    int upload_records(nbody_cuda* ctx, const void* bodies, const size_t n)
    {
        const int path = resolve(ctx);
        if (path == NBODY_TRANSFER_DIRECT)
        {
            if (void* view = device_view(ctx, const_cast<void*>(bodies)))
            {
                const cudaError_t e = launch_in(ctx, view, n);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "record read launch");
                // the kernel reads the caller's array: done before the caller may reuse it
                const cudaError_t s = cudaStreamSynchronize(ctx->stream);
                if (s != cudaSuccess)
                    return ctx_cuda_fail(ctx, s, "stream synchronize");
                return NBODY_OK;
            }
        }
        if (path == NBODY_TRANSFER_MAPPED || path == NBODY_TRANSFER_DIRECT)
        {
            if (const int st = mapped_staging(ctx, n * kRecord))
                return st;
            ctx->readback_valid = false;
            float* dst = static_cast<float*>(ctx->mapped);
            const float* src = static_cast<const float*>(bodies);
            host_parallel(n, n * kRecord, [&](const size_t b, const size_t e) {
                std::memcpy(dst + 12 * b, src + 12 * b, (e - b) * kRecord);
            });
            const cudaError_t e = launch_in(ctx, ctx->mapped_dev, n);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "record read launch");
            cudaEventRecord(ctx->mapped_event, ctx->stream);
            return NBODY_OK;
        }
        // STAGED: pinned staging, copy engine, split on the device
        if (ctx->layout == NBODY_LAYOUT_AOS)
            return h2d(ctx, ctx->bodies, bodies, n * kRecord);
        if (const int st = ensure_aos_stage(ctx, n))
            return st;
        if (const int st = h2d(ctx, ctx->aos_stage, bodies, n * kRecord))
            return st;
        const cudaError_t e = launch_split(ctx->aos_stage, ctx->pm, ctx->vr, ctx->acc, static_cast<int>(n), ctx->stream,
                                           &ctx->launches);
        return e == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, e, "split launch");
    }

    int prefetch_records(nbody_cuda* ctx, const unsigned mask)
    {
        const unsigned m = mask & NBODY_READ_ALL;
        if (!m || !ctx->count || resolve(ctx) == NBODY_TRANSFER_DIRECT)
            return NBODY_OK;
        if (ctx->readback_valid && ctx->readback_version == ctx->body_version && ctx->readback_count >= ctx->count
            && !(m & ~ctx->readback_mask))
            return NBODY_OK;
        if (const int st = mapped_staging(ctx, ctx->count * kRecord))
            return st;
        // Whole records: one pass writes whole lines whatever the mask, so a partial mask
        // would save nothing on the link and only narrow what the readback can serve.
        const cudaError_t e = launch_out(ctx, ctx->mapped_dev, ctx->count, NBODY_READ_ALL);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "record write launch");
        cudaEventRecord(ctx->mapped_event, ctx->stream);
        ctx->readback_valid = true;
        ctx->readback_version = ctx->body_version;
        ctx->readback_count = ctx->count;
        ctx->readback_mask = NBODY_READ_ALL;
        return NBODY_OK;
    }

    void release_transfer(nbody_cuda* ctx)
    {
        if (ctx->mapped_event)
            cudaEventSynchronize(ctx->mapped_event);
        cudaFreeHost(ctx->mapped);
        if (ctx->mapped_event)
            cudaEventDestroy(ctx->mapped_event);
        ctx->mapped = ctx->mapped_dev = nullptr;
        ctx->mapped_event = nullptr;
    }
}

extern "C" {

int nbody_cuda_set_transfer(nbody_cuda* ctx, const int policy)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (policy < NBODY_TRANSFER_AUTO || policy > NBODY_TRANSFER_DIRECT)
        return nbg::ctx_fail(ctx, NBODY_ERR_INVALID, "unknown transfer policy");
    if (policy == NBODY_TRANSFER_DIRECT && !ctx->pageable_access)
        return nbg::ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "this device does not access pageable host memory");
    ctx->transfer = policy;
    return NBODY_OK;
}

int nbody_cuda_transfer_info(const nbody_cuda* ctx, int* policy, int* resolved, int* pageable, uint64_t* readback_hits)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (policy)
        *policy = ctx->transfer;
    if (resolved)
        *resolved = nbg::resolve(ctx);
    if (pageable)
        *pageable = ctx->pageable_access ? (ctx->pageable_host_tables ? 2 : 1) : 0;
    if (readback_hits)
        *readback_hits = ctx->readback_hits;
    return NBODY_OK;
}

int nbody_cuda_prefetch(nbody_cuda* ctx, const unsigned mask)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    return nbg::prefetch_records(ctx, mask);
}

}
