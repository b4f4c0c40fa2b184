// Tree::query (source/bhtree.cpp:153-173) on the device: many rays at once, one thread per
// ray, over a tree in the reference's node layout (bh::Node, include/nbody/bhtree.h:13-22)
// -- the context's exported Barnes-Hut tree or any node array the caller passes.
//
// The walk is the reference's stackless pre-order over `children` / `next`. A node whose
// bounds the ray meets (Bounds::ray_intersect, include/nbody/bounds.h:64-133) is visited
// and the walk descends to its children, or moves to `next` at a leaf. At a node the ray
// misses, the reference's loop leaves its index where it is and so never ends; here the
// walk moves to that node's `next`, skipping its subtree, which is the only reading under
// which the walk ends. Wherever the reference's walk ends, the two visit the same nodes in
// the same order.
//
// ray_intersect is restated operation for operation, as rounded intrinsics: the box is
// centre +- size on every axis (the node's `size` is its edge, so this is twice the cell),
// a ray whose origin lies in it meets it, and otherwise the three face pairs are tried in
// order x, y, z with the line parameter t of either sign.
//
// Every walk is bounded: each node of a well-formed tree is entered at most once, so a walk
// that takes more steps than there are nodes, or reaches an index outside the array, stops
// and raises DEV_ERR_BOUNDS.
#include <cfloat>

#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kBlock = 128;

        struct Ray
        {
            float o[3], d[3];
        };

        // Bounds::ray_intersect_coord<i> with length = FLT_MAX: the reference only lowers
        // length on a hit, after which ray_intersect returns.
        __device__ __forceinline__ bool face(const Ray& r, const float c[3], const float s, const int i)
        {
            const int j = (i + 1) % 3, k = (i + 2) % 3;
            float t;
            if (r.d[i] < -FLT_EPSILON)
                t = __fdiv_rn(__fsub_rn(__fadd_rn(c[i], s), r.o[i]), r.d[i]);
            else if (r.d[i] > FLT_EPSILON)
                t = __fdiv_rn(__fsub_rn(__fsub_rn(c[i], s), r.o[i]), r.d[i]);
            else
                return false;
            if (!(t < FLT_MAX))
                return false;
            const float pj = __fadd_rn(r.o[j], __fmul_rn(r.d[j], t));
            const float pk = __fadd_rn(r.o[k], __fmul_rn(r.d[k], t));
            return pj > __fsub_rn(c[j], s) && pj < __fadd_rn(c[j], s) && pk > __fsub_rn(c[k], s)
                   && pk < __fadd_rn(c[k], s);
        }

        __device__ __forceinline__ bool ray_meets(const Ray& r, const float4 b)
        {
            const float c[3] = { b.x, b.y, b.z };
            const float s = b.w;
            bool inside = true;
            for (int i = 0; i < 3; ++i)
                if (r.o[i] < __fsub_rn(c[i], s) || r.o[i] > __fadd_rn(c[i], s))
                {
                    inside = false;
                    break;
                }
            if (inside)
                return true;
            return face(r, c, s, 0) || face(r, c, s, 1) || face(r, c, s, 2);
        }

        __global__ void __launch_bounds__(kBlock) query_kernel(const float4* __restrict__ nodes, const uint32_t count,
                                                               const float* __restrict__ rays, const uint32_t nrays,
                                                               const int stop, uint32_t* __restrict__ hits,
                                                               const uint32_t max_hits, uint32_t* __restrict__ counts,
                                                               unsigned* __restrict__ err)
        {
            const uint32_t q = blockIdx.x * kBlock + threadIdx.x;
            if (q >= nrays)
                return;
            Ray r;
            for (int i = 0; i < 3; ++i)
            {
                r.o[i] = rays[6 * static_cast<size_t>(q) + i];
                r.d[i] = rays[6 * static_cast<size_t>(q) + 3 + i];
            }
            uint32_t* out = hits + static_cast<size_t>(q) * max_hits;
            uint32_t idx = 0, visited = 0, steps = 0;
            do
            {
                if (idx >= count || ++steps > count)
                {
                    atomicOr(err, DEV_ERR_BOUNDS);
                    break;
                }
                const float4 bounds = __ldg(&nodes[3 * static_cast<size_t>(idx)]);
                const float4 com = __ldg(&nodes[3 * static_cast<size_t>(idx) + 1]);
                const uint4 links = __ldg(reinterpret_cast<const uint4*>(nodes) + 3 * static_cast<size_t>(idx) + 2);
                if (ray_meets(r, bounds))
                {
                    if (visited < max_hits)
                        out[visited] = idx;
                    ++visited;
                    if (stop == NBODY_QUERY_FIRST_BODY && links.y == 0 && com.w != 0.f)
                        break;      // the visitor returns false
                    idx = links.y ? links.y : links.x;
                }
                else
                    idx = links.x;
            } while (idx != 0);
            counts[q] = visited;
        }

        int grow(nbody_cuda* ctx, void** p, size_t* cap, const size_t bytes, const char* what)
        {
            if (bytes <= *cap)
                return NBODY_OK;
            if (const int st = before_allocation(ctx))
                return st;
            cudaFreeAsync(*p, ctx->stream);
            *p = nullptr;
            *cap = 0;
            const cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, what);
            *cap = bytes;
            return NBODY_OK;
        }
    }

    int tree_query(nbody_cuda* ctx, const void* nodes, size_t count, const float* rays, const size_t nrays,
                   const int stop, uint32_t* hits, const size_t max_hits, uint32_t* counts)
    {
        if (stop != NBODY_QUERY_ALL && stop != NBODY_QUERY_FIRST_BODY)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "unknown query stop rule");
        if (nrays && (!rays || !counts || (max_hits && !hits)))
            return ctx_fail(ctx, NBODY_ERR_INVALID, "null query buffers");
        if (nrays > UINT32_MAX || max_hits > UINT32_MAX || (max_hits && nrays > SIZE_MAX / 4 / max_hits))
            return ctx_fail(ctx, NBODY_ERR_INVALID, "query too large");
        const void* host_nodes = nodes;
        uint64_t id = 0;
        if (!nodes)
        {
            if (const int st = nbody_cuda_tree_export(ctx, nullptr, 0, &count))
                return st;
            host_nodes = ctx->tree_export.data();
            id = ctx->tree_export_id;
        }
        if (count > UINT32_MAX)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "tree too large");
        if (!nrays)
            return NBODY_OK;
        if (!count)
        {
            for (size_t q = 0; q < nrays; ++q)
                counts[q] = 0;
            return NBODY_OK;
        }
        // the exported tree stays on the device until the next build; a caller's array is
        // uploaded each call
        if (!id || id != ctx->query_nodes_id)
        {
            if (const int st = grow(ctx, &ctx->query_nodes, &ctx->query_nodes_cap, count * 48, "query tree allocation"))
                return st;
            if (const int st = h2d(ctx, ctx->query_nodes, host_nodes, count * 48))
                return st;
            ctx->query_nodes_id = id;
        }
        const size_t ray_bytes = nrays * 24, hit_bytes = nrays * max_hits * 4, count_bytes = nrays * 4;
        const size_t at_hits = (ray_bytes + 255) / 256 * 256, at_counts = at_hits + (hit_bytes + 255) / 256 * 256;
        if (const int st = grow(ctx, &ctx->query_buf, &ctx->query_buf_cap, at_counts + count_bytes, "query buffers"))
            return st;
        unsigned char* buf = static_cast<unsigned char*>(ctx->query_buf);
        if (const int st = h2d(ctx, buf, rays, ray_bytes))
            return st;
        query_kernel<<<static_cast<unsigned>((nrays + kBlock - 1) / kBlock), kBlock, 0, ctx->stream>>>(
            static_cast<const float4*>(ctx->query_nodes), static_cast<uint32_t>(count),
            reinterpret_cast<const float*>(buf), static_cast<uint32_t>(nrays), stop,
            reinterpret_cast<uint32_t*>(buf + at_hits), static_cast<uint32_t>(max_hits),
            reinterpret_cast<uint32_t*>(buf + at_counts), ctx->dev_error);
        ++ctx->launches;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "query launch");
        if (max_hits)
            if (const int st = d2h(ctx, hits, buf + at_hits, hit_bytes))
                return st;
        if (const int st = d2h(ctx, counts, buf + at_counts, count_bytes))
            return st;
        return check_device_error(ctx);
    }

    void release_query(nbody_cuda* ctx)
    {
        cudaFree(ctx->query_nodes);
        cudaFree(ctx->query_buf);
        ctx->query_nodes = ctx->query_buf = nullptr;
        ctx->query_nodes_cap = ctx->query_buf_cap = 0;
    }
}

extern "C" int nbody_cuda_tree_query(nbody_cuda* ctx, const void* nodes, const size_t count, const float* rays,
                                     const size_t nrays, const int stop, uint32_t* hits, const size_t max_hits,
                                     uint32_t* counts)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    return nbg::tree_query(ctx, nodes, count, rays, nrays, stop, hits, max_hits, counts);
}
