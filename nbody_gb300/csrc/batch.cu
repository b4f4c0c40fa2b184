// Batched direct sums: many independent systems of uneven size advanced by one persistent
// launch per accelerate (no reference counterpart; the reference runs one system per Sim).
//
// Work decomposition: the bodies of all systems are concatenated (system s owns
// [off[s], off[s+1])). A work item is (system, block of BLOCK x T targets, chunk of at most
// CHUNK sources): splitting the sources as well as the targets keeps every item short, so
// a largest-first list pulled by persistent CTAs from an atomic counter balances even when
// a few systems hold most of the pairs. Nothing ever waits on another CTA.
//
// Per item the chunk's sources stream through shared memory in 256-body TMA bulk copies
// (three stages, mbarrier completion, stage and parity carried across items), and every
// lane applies the same source to its own T targets, as the single-system kernel does: the
// source is warp-uniform. (Configurations marked DUP first expand each tile in shared memory
// into components already paired for the packed FP32x2 operands.)
// A target block of one chunk writes its accelerations directly. A block of several chunks
// writes each chunk's partial sums; the CTA that completes the block's last chunk (an
// atomic count, no waiting) sums the partials in chunk order and writes the result, so the
// sum does not depend on which CTA finished when.
#include <algorithm>
#include <vector>

#include "batch.cuh"
#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kTile = 256;
        constexpr int kStages = 3;
        constexpr int kEnergyBlock = 128;

        // One unit of work: system bodies [base, base + n); targets [t0, t0 + BLOCK*T) of it;
        // sources [chunk * CHUNK, ...) of it. A block of several chunks has a completion
        // counter `blk` and its chunk partials at slots [slot - chunk, slot - chunk + nchunk).
        struct Item
        {
            int base, n, t0, chunk;
            int nchunk, blk, slot, pad;
        };
        static_assert(sizeof(Item) == 32, "work item layout");
    }

    template <int LAW>
    __device__ __forceinline__ void bpair(const float2 sx, const float2 sy, const float2 sz, const float2 sm,
                                          const float2 nx, const float2 ny, const float2 nz, const float2 lim,
                                          float2& ax, float2& ay, float2& az)
    {
        const float2 dx = add2(sx, nx);
        const float2 dy = add2(sy, ny);
        const float2 dz = add2(sz, nz);
        float2 r2 = (LAW == NBODY_LAW_SOFTENED) ? fma2(dx, dx, lim) : mul2(dx, dx);
        r2 = fma2(dy, dy, r2);
        r2 = fma2(dz, dz, r2);
        float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
        if (LAW == NBODY_LAW_CUTOFF)
        {
            inv.x = r2.x > lim.x ? inv.x : 0.f;
            inv.y = r2.y > lim.y ? inv.y : 0.f;
        }
        const float2 inv2 = mul2(inv, inv);
        const float2 s = mul2(mul2(sm, inv), inv2);
        ax = fma2(dx, s, ax);
        ay = fma2(dy, s, ay);
        az = fma2(dz, s, az);
    }

    struct BatchShared
    {
        float4 tile[kStages][kTile];
        float4 dup[2 * kTile];      // (x, x, y, y), (z, z, m, m) per source, when DUP
        uint64_t bar[kStages];
        int item;
        int last;
    };

    // One work item, start to finish. Kept out of line: compiled on its own, the source loop
    // gets the same code as in a one-item-per-CTA launch; inlined into the persistent loop
    // it came out with a fifth of its instructions in extra integer work.
    template <int BLOCK, int T, int LAW, bool DUP>
    __device__ __noinline__ bool run_item(BatchShared& sh, const Item& w, unsigned& seq, const float4* __restrict__ pm,
                                          const float4* __restrict__ vr, const int csize, float4* __restrict__ acc,
                                          float4* __restrict__ partial, unsigned* __restrict__ block_done,
                                          const float G, const float eps2, unsigned* __restrict__ err)
    {
        constexpr int P = T / 2;
        constexpr int TB = BLOCK * T;           // targets per item
        const int tid = threadIdx.x;
        const int j0 = w.chunk * csize;
        const int jn = min(csize, w.n - j0);
        const int ntiles = (jn + kTile - 1) / kTile;
        auto issue = [&](const int k) {
            const int first = j0 + k * kTile;
            const int cnt = min(kTile, j0 + jn - first);
            const unsigned stage = (seq + k) % kStages;
            mbar_arrive_expect_tx(&sh.bar[stage], static_cast<unsigned>(cnt) * 16u);
            tma_load_1d(&sh.tile[stage][0], pm + w.base + first, static_cast<unsigned>(cnt) * 16u, &sh.bar[stage]);
        };
        if (tid == 0)
            for (int k = 0; k < kStages && k < ntiles; ++k)
                issue(k);

        float2 nx[P], ny[P], nz[P], lim[P], ax[P], ay[P], az[P];
#pragma unroll
        for (int p = 0; p < P; ++p)
        {
            float q[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int t = min(w.t0 + tid + (2 * p + h) * BLOCK, w.n - 1);
                const float4 x = pm[w.base + t];
                q[h][0] = -x.x;
                q[h][1] = -x.y;
                q[h][2] = -x.z;
                if (LAW == NBODY_LAW_CUTOFF)
                {
                    const float r = vr[w.base + t].w;
                    q[h][3] = r * r;
                }
                else
                    q[h][3] = eps2;
            }
            nx[p] = make_float2(q[0][0], q[1][0]);
            ny[p] = make_float2(q[0][1], q[1][1]);
            nz[p] = make_float2(q[0][2], q[1][2]);
            lim[p] = make_float2(q[0][3], q[1][3]);
            ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
        }

        for (int k = 0; k < ntiles; ++k)
        {
            const unsigned stage = (seq + k) % kStages;
            const bool ok = mbar_wait_bounded(&sh.bar[stage], ((seq + k) / kStages) & 1u, err);
            if (__syncthreads_or(!ok))
            {
                // a copy that never landed (the error word says so): let the ones still in
                // flight land, each with a bounded wait, before the CTA's shared memory goes
                if (tid == 0)
                    for (int q = k; q < ntiles && q < k + kStages; ++q)
                        mbar_wait_bounded(&sh.bar[(seq + q) % kStages], ((seq + q) / kStages) & 1u, err);
                return false;
            }
            const int cnt = min(kTile, jn - k * kTile);
            // pad to whole pairs with massless sources at the origin, which add exactly
            // zero under both laws (the copy wrote [0, cnt))
            const int padded = (cnt + 1) & ~1;
            if (DUP)
            {
                for (int j = tid; j < padded; j += BLOCK)
                {
                    const float4 v = j < cnt ? sh.tile[stage][j] : make_float4(0.f, 0.f, 0.f, 0.f);
                    sh.dup[2 * j] = make_float4(v.x, v.x, v.y, v.y);
                    sh.dup[2 * j + 1] = make_float4(v.z, v.z, v.w, v.w);
                }
                __syncthreads();
#pragma unroll 2
                for (int j = 0; j < padded; ++j)
                {
                    const float4 a = sh.dup[2 * j], b = sh.dup[2 * j + 1];
                    const float2 sx = make_float2(a.x, a.y), sy = make_float2(a.z, a.w);
                    const float2 sz = make_float2(b.x, b.y), sm = make_float2(b.z, b.w);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        bpair<LAW>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
            }
            else
            {
                if (padded > cnt)
                {
                    if (tid == 0)
                        sh.tile[stage][cnt] = make_float4(0.f, 0.f, 0.f, 0.f);
                    __syncthreads();
                }
                const float4* tl = sh.tile[stage];
#pragma unroll 2
                for (int j = 0; j < padded; ++j)
                {
                    const float4 v = tl[j];
                    const float2 sx = f2(v.x), sy = f2(v.y), sz = f2(v.z), sm = f2(v.w);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        bpair<LAW>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
            }
            __syncthreads();
            if (tid == 0 && k + kStages < ntiles)
                issue(k + kStages);
        }
        seq += static_cast<unsigned>(ntiles);

        if (w.nchunk == 1)
        {
#pragma unroll
            for (int p = 0; p < P; ++p)
#pragma unroll
                for (int h = 0; h < 2; ++h)
                {
                    const int t = w.t0 + tid + (2 * p + h) * BLOCK;
                    if (t < w.n)
                        acc[w.base + t] = make_float4(G * (h ? ax[p].y : ax[p].x), G * (h ? ay[p].y : ay[p].x),
                                                      G * (h ? az[p].y : az[p].x), 0.f);
                }
            return true;
        }
        // Several chunks: publish this chunk's partial sums, then count the chunk in; the CTA
        // that counts the last one sums all of them in chunk order.
        float4* mine = partial + static_cast<size_t>(w.slot - w.chunk) * TB;
#pragma unroll
        for (int p = 0; p < P; ++p)
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int q = tid + (2 * p + h) * BLOCK;
                __stcg(&mine[static_cast<size_t>(w.chunk) * TB + q],
                       make_float4(h ? ax[p].y : ax[p].x, h ? ay[p].y : ay[p].x, h ? az[p].y : az[p].x, 0.f));
            }
        __threadfence();
        __syncthreads();
        if (tid == 0)
            sh.last = atomicAdd(&block_done[w.blk], 1u) == static_cast<unsigned>(w.nchunk - 1);
        __syncthreads();
        if (!sh.last)
            return true;
        __threadfence();
#pragma unroll
        for (int p = 0; p < P; ++p)
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int q = tid + (2 * p + h) * BLOCK;
                float4 a = __ldcg(&mine[q]);
                for (int c = 1; c < w.nchunk; ++c)
                {
                    const float4 b = __ldcg(&mine[static_cast<size_t>(c) * TB + q]);
                    a.x += b.x;
                    a.y += b.y;
                    a.z += b.z;
                }
                const int t = w.t0 + q;
                if (t < w.n)
                    acc[w.base + t] = make_float4(G * a.x, G * a.y, G * a.z, 0.f);
            }
        return true;
    }

    // Persistent CTAs pull items from the counter until the list is exhausted.
    template <int BLOCK, int T, int LAW, bool DUP>
    __global__ void __launch_bounds__(BLOCK)
    batch_kernel(const float4* __restrict__ pm, const float4* __restrict__ vr, const Item* __restrict__ items,
                 const int nitems, const int csize, unsigned* __restrict__ counter, float4* __restrict__ acc,
                 float4* __restrict__ partial, unsigned* __restrict__ block_done, const float G, const float eps2,
                 unsigned* __restrict__ err)
    {
        __shared__ __align__(128) BatchShared sh;
        const int tid = threadIdx.x;
        if (tid == 0)
        {
            for (int s = 0; s < kStages; ++s)
                mbar_init(&sh.bar[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        unsigned seq = 0;   // tiles this CTA has consumed (stage = seq % kStages, parity = seq / kStages)
        for (;;)
        {
            if (tid == 0)
                sh.item = static_cast<int>(atomicAdd(counter, 1u));
            __syncthreads();
            const int it = sh.item;
            __syncthreads();
            if (it >= nitems)
                return;
            const Item w = items[it];
            if (!run_item<BLOCK, T, LAW, DUP>(sh, w, seq, pm, vr, csize, acc, partial, block_done, G, eps2, err))
                return;
        }
    }

    // FP64 energy and momentum per work item: kinetic, potential (half of each target's pair
    // sum, so pairs are counted once), momentum.
    __global__ void __launch_bounds__(kEnergyBlock)
    batch_energy_kernel(const float4* __restrict__ pm, const float4* __restrict__ vr, const int* __restrict__ off,
                        const int2* __restrict__ items, const double G, const double eps2,
                        double* __restrict__ out)
    {
        const int2 w = items[blockIdx.x];
        const int base = off[w.x];
        const int n = off[w.x + 1] - base;
        const int t = w.y + threadIdx.x;
        double ke = 0, pe = 0, px = 0, py = 0, pz = 0;
        if (t < n)
        {
            const float4 x = pm[base + t];
            const float4 v = vr[base + t];
            const double m = x.w;
            ke = 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
            px = m * v.x;
            py = m * v.y;
            pz = m * v.z;
            double sum = 0;
            for (int j = 0; j < n; ++j)
            {
                if (j == t)
                    continue;
                const float4 y = pm[base + j];
                const double dx = (double)y.x - x.x, dy = (double)y.y - x.y, dz = (double)y.z - x.z;
                sum += (double)y.w / sqrt(dx * dx + dy * dy + dz * dz + eps2);
            }
            pe = -0.5 * G * m * sum;
        }
        __shared__ double red[5][kEnergyBlock];
        red[0][threadIdx.x] = ke;
        red[1][threadIdx.x] = pe;
        red[2][threadIdx.x] = px;
        red[3][threadIdx.x] = py;
        red[4][threadIdx.x] = pz;
        __syncthreads();
        for (int s = kEnergyBlock / 2; s > 0; s >>= 1)
        {
            if (threadIdx.x < s)
                for (int k = 0; k < 5; ++k)
                    red[k][threadIdx.x] += red[k][threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x < 5)
            out[static_cast<size_t>(blockIdx.x) * 8 + threadIdx.x] = red[threadIdx.x][0];
    }

    // ------------------------------------------------------------------------------------
    // configuration table
    // ------------------------------------------------------------------------------------
    namespace
    {
        using BatchFn = void (*)(const float4*, const float4*, const Item*, int, int, unsigned*, float4*, float4*,
                                 unsigned*, float, float, unsigned*);

        struct Config
        {
            int block, t, chunk;
            BatchFn soft, cutoff;
        };

        template <int BLOCK, int T, bool DUP = false>
        Config cfg(const int chunk)
        {
            return { BLOCK, T, chunk, batch_kernel<BLOCK, T, NBODY_LAW_SOFTENED, DUP>,
                     batch_kernel<BLOCK, T, NBODY_LAW_CUTOFF, DUP> };
        }

        // Shapes the autotuner times: threads per CTA, targets per thread, sources per chunk.
        const std::vector<Config>& configs()
        {
            static const std::vector<Config> c = {
                cfg<64, 4>(1024), cfg<64, 4>(512),  cfg<64, 4>(2048), cfg<128, 4>(1024), cfg<64, 2>(1024),
                cfg<128, 2>(1024), cfg<64, 8>(1024), cfg<64, 2, true>(1024), cfg<64, 4, true>(1024),
                cfg<128, 4, true>(1024),
            };
            return c;
        }

        int targets_per_item(const Config& c) { return c.block * c.t; }
    }

    struct BatchState
    {
        std::vector<int> off;           // host copy of the system table
        int* d_off = nullptr;
        size_t off_cap = 0;
        Item* d_items = nullptr;        // work list of the active configuration
        size_t items_cap = 0;
        int nitems = 0;
        int items_config = -1;          // the configuration the list was built for
        int nblocks = 0;                // multi-chunk target blocks in the list
        unsigned* counter = nullptr;
        unsigned* block_done = nullptr;
        size_t block_cap = 0;
        float4* partial = nullptr;      // chunk partial sums, TB per item of a multi-chunk block
        size_t partial_cap = 0;
        int config = 0;                 // index into configs()
        bool tuned = false;
    };

    int batch_config_count() { return static_cast<int>(configs().size()); }

    void batch_config_describe(const int i, int* block, int* t, int* chunk)
    {
        const Config& c = configs()[i];
        *block = c.block;
        *t = c.t;
        *chunk = c.chunk;
    }

    namespace
    {
        // Items of the longest chunks first; the chunks of one target block are consecutive
        // in the list, so a block's partials are the item range [first, first + nchunk).
        std::vector<Item> make_items(const std::vector<int>& off, const Config& c, int* nblocks, size_t* nslots)
        {
            const int tb = targets_per_item(c);
            std::vector<int> order(off.size() - 1);
            for (size_t s = 0; s < order.size(); ++s)
                order[s] = static_cast<int>(s);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return off[a + 1] - off[a] > off[b + 1] - off[b];
            });
            std::vector<Item> items;
            int blk = 0, slot = 0;
            for (const int s : order)
            {
                const int n = off[s + 1] - off[s];
                if (n == 0)
                    continue;
                const int nchunk = (n + c.chunk - 1) / c.chunk;
                for (int t0 = 0; t0 < n; t0 += tb)
                {
                    for (int k = 0; k < nchunk; ++k)
                        items.push_back(Item{ off[s], n, t0, k, nchunk, nchunk > 1 ? blk : -1,
                                              nchunk > 1 ? slot + k : -1, 0 });
                    if (nchunk > 1)
                    {
                        ++blk;
                        slot += nchunk;
                    }
                }
            }
            *nblocks = blk;
            *nslots = static_cast<size_t>(slot);
            return items;
        }

        int ensure_items(nbody_cuda* ctx, const int config)
        {
            BatchState& b = *ctx->batch;
            if (b.items_config == config)
                return NBODY_OK;
            const Config& c = configs()[config];
            int nblocks = 0;
            size_t nslots = 0;
            const std::vector<Item> items = make_items(b.off, c, &nblocks, &nslots);
            const size_t partial_need = nslots * static_cast<size_t>(targets_per_item(c));
            if (items.size() > b.items_cap || static_cast<size_t>(nblocks) > b.block_cap || partial_need > b.partial_cap)
            {
                if (const int st = before_allocation(ctx))
                    return st;
                auto regrow = [&](auto** p, size_t* cap, const size_t need, const size_t elem) -> cudaError_t {
                    if (need <= *cap)
                        return cudaSuccess;
                    cudaFreeAsync(*p, ctx->stream);
                    *p = nullptr;
                    *cap = 0;
                    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), std::max<size_t>(1, need) * elem,
                                                          ctx->stream);
                    if (e == cudaSuccess)
                        *cap = need;
                    return e;
                };
                cudaError_t e = regrow(&b.d_items, &b.items_cap, items.size(), sizeof(Item));
                if (e == cudaSuccess)
                    e = regrow(&b.block_done, &b.block_cap, static_cast<size_t>(nblocks), sizeof(unsigned));
                if (e == cudaSuccess)
                    e = regrow(&b.partial, &b.partial_cap, partial_need, sizeof(float4));
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "batch work list allocation");
            }
            if (!items.empty())
            {
                cudaError_t e = cudaMemcpyAsync(b.d_items, items.data(), items.size() * sizeof(Item),
                                                cudaMemcpyHostToDevice, ctx->stream);
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(ctx->stream);     // the host vector goes out of scope
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "batch work list upload");
            }
            b.nitems = static_cast<int>(items.size());
            b.nblocks = nblocks;
            b.items_config = config;
            return NBODY_OK;
        }

        int occupancy_grid(nbody_cuda* ctx, BatchFn fn, const int block, const int nitems)
        {
            int sms = 0, per = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0) != cudaSuccess || per < 1)
                per = 1;
            return std::max(1, std::min(nitems, sms * per));
        }
    }

    int batch_set_systems(nbody_cuda* ctx, const int64_t* offsets, const size_t nsys)
    {
        if (!ctx->batch)
            ctx->batch = new BatchState();
        BatchState& b = *ctx->batch;
        if (nsys == 0 || !offsets)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "a system table needs at least one system");
        if (offsets[0] != 0 || static_cast<size_t>(offsets[nsys]) != ctx->count)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "system offsets must run from 0 to the body count");
        for (size_t s = 0; s < nsys; ++s)
            if (offsets[s + 1] < offsets[s])
                return ctx_fail(ctx, NBODY_ERR_INVALID, "system offsets must not decrease");
        b.off.assign(nsys + 1, 0);
        for (size_t s = 0; s <= nsys; ++s)
            b.off[s] = static_cast<int>(offsets[s]);
        if (b.off.size() > b.off_cap)
        {
            cudaFreeAsync(b.d_off, ctx->stream);
            b.d_off = nullptr;
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&b.d_off), b.off.size() * sizeof(int), ctx->stream);
            if (e == cudaSuccess && !b.counter)
                e = cudaMallocAsync(reinterpret_cast<void**>(&b.counter), 2 * sizeof(unsigned), ctx->stream);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "system table allocation");
            b.off_cap = b.off.size();
        }
        cudaError_t e = cudaMemcpyAsync(b.d_off, b.off.data(), b.off.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "system table upload");
        b.items_config = -1;
        ++ctx->generation;
        return NBODY_OK;
    }

    int batch_accelerate(nbody_cuda* ctx, const nbody_step_params* p)
    {
        if (!ctx->batch || ctx->batch->off.empty())
            return ctx_fail(ctx, NBODY_ERR_INVALID, "batched mode needs a system table (nbody_cuda_set_systems)");
        BatchState& b = *ctx->batch;
        if (static_cast<size_t>(b.off.back()) != ctx->count)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "the body count changed since the system table was set");
        if (ctx->layout != NBODY_LAYOUT_SOA)
            return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "batched mode runs on the split layout");
        if (p->precision != NBODY_PREC_FP32)
            return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "batched mode is FP32");
        const Config& c = configs()[b.config];
        if (const int st = ensure_items(ctx, b.config))
            return st;
        if (!b.nitems)
            return NBODY_OK;
        const BatchFn fn = p->law == NBODY_LAW_SOFTENED ? c.soft : c.cutoff;
        const int grid = occupancy_grid(ctx, fn, c.block, b.nitems);
        cudaError_t me = cudaMemsetAsync(b.counter, 0, sizeof(unsigned), ctx->stream);
        if (me == cudaSuccess && b.nblocks)
            me = cudaMemsetAsync(b.block_done, 0, static_cast<size_t>(b.nblocks) * sizeof(unsigned), ctx->stream);
        if (me != cudaSuccess)
            return ctx_cuda_fail(ctx, me, "batched counters");
        fn<<<grid, c.block, 0, ctx->stream>>>(ctx->pm, ctx->vr, b.d_items, b.nitems, c.chunk, b.counter, ctx->acc,
                                              b.partial, b.block_done, p->G, p->eps2, ctx->dev_error);
        ++ctx->launches;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "batched launch");
        ctx->pending_partials = 0;
        return NBODY_OK;
    }

    int batch_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms, int* best)
    {
        if (!ctx->batch || ctx->batch->off.empty())
            return ctx_fail(ctx, NBODY_ERR_INVALID, "batched mode needs a system table (nbody_cuda_set_systems)");
        BatchState& b = *ctx->batch;
        nbody_step_params q = *p;
        q.law = NBODY_LAW_SOFTENED;
        if (!(q.eps2 > 0.f))
            q.eps2 = 1e-4f;
        EventPair ev;
        if (ev.status != cudaSuccess)
            return ctx_cuda_fail(ctx, ev.status, "event create");
        int best_i = 0;
        float best_ms = 1e30f;
        for (int i = 0; i < batch_config_count(); ++i)
        {
            b.config = i;
            b.items_config = -1;
            float ms_best = 1e30f;
            for (int rep = 0; rep < 3; ++rep)
            {
                cudaEventRecord(ev.start, ctx->stream);
                if (const int st = batch_accelerate(ctx, &q))
                    return st;
                cudaEventRecord(ev.stop, ctx->stream);
                const float ms = ev.elapsed_ms();
                if (rep > 0)
                    ms_best = std::min(ms_best, ms);
            }
            if (times_ms)
                times_ms[i] = ms_best;
            if (ms_best < best_ms)
            {
                best_ms = ms_best;
                best_i = i;
            }
        }
        b.config = best_i;
        b.items_config = -1;
        b.tuned = true;
        if (best)
            *best = best_i;
        return check_device_error(ctx);
    }

    int batch_set_config(nbody_cuda* ctx, const int index)
    {
        if (!ctx->batch)
            ctx->batch = new BatchState();
        if (index < 0 || index >= batch_config_count())
            return ctx_fail(ctx, NBODY_ERR_INVALID, "no such batched configuration");
        ctx->batch->config = index;
        ctx->batch->items_config = -1;
        return NBODY_OK;
    }

    int batch_get_config(const nbody_cuda* ctx) { return ctx->batch ? ctx->batch->config : 0; }

    int batch_energy(nbody_cuda* ctx, const nbody_step_params* p, double* out)
    {
        std::vector<int> one;
        const std::vector<int>* off = nullptr;
        if (ctx->batch && !ctx->batch->off.empty() && static_cast<size_t>(ctx->batch->off.back()) == ctx->count)
            off = &ctx->batch->off;
        else
        {
            one = { 0, static_cast<int>(ctx->count) };
            off = &one;
        }
        if (ctx->layout != NBODY_LAYOUT_SOA)
            return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "energy diagnostics run on the split layout");
        const size_t nsys = off->size() - 1;
        std::vector<int2> items;
        std::vector<int> item_sys;
        for (size_t s = 0; s < nsys; ++s)
            for (int t = 0; t < (*off)[s + 1] - (*off)[s]; t += kEnergyBlock)
                items.push_back(make_int2(static_cast<int>(s), t));
        int* d_off = nullptr;
        int2* d_items = nullptr;
        double* d_out = nullptr;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_off), off->size() * sizeof(int), ctx->stream);
        if (e == cudaSuccess)
            e = cudaMallocAsync(reinterpret_cast<void**>(&d_items), std::max<size_t>(1, items.size()) * sizeof(int2), ctx->stream);
        if (e == cudaSuccess)
            e = cudaMallocAsync(reinterpret_cast<void**>(&d_out), std::max<size_t>(1, items.size()) * 8 * sizeof(double), ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_off, off->data(), off->size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && !items.empty())
            e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream);
        std::vector<double> part(items.size() * 8, 0.0);
        if (e == cudaSuccess && !items.empty())
        {
            batch_energy_kernel<<<static_cast<unsigned>(items.size()), kEnergyBlock, 0, ctx->stream>>>(
                ctx->pm, ctx->vr, d_off, d_items, p->G, p->eps2, d_out);
            ++ctx->launches;
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(part.data(), d_out, part.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        }
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        cudaFree(d_off);
        cudaFree(d_items);
        cudaFree(d_out);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "energy diagnostics");
        for (size_t s = 0; s < nsys; ++s)
            for (int k = 0; k < 5; ++k)
                out[5 * s + k] = 0.0;
        for (size_t i = 0; i < items.size(); ++i)
            for (int k = 0; k < 5; ++k)
                out[5 * items[i].x + k] += part[8 * i + k];
        return check_device_error(ctx);
    }

    size_t batch_system_count(const nbody_cuda* ctx)
    {
        return (ctx->batch && !ctx->batch->off.empty()) ? ctx->batch->off.size() - 1 : 0;
    }

    void release_batch(nbody_cuda* ctx)
    {
        if (!ctx->batch)
            return;
        BatchState& b = *ctx->batch;
        cudaFree(b.d_off);
        cudaFree(b.d_items);
        cudaFree(b.counter);
        cudaFree(b.block_done);
        cudaFree(b.partial);
        delete ctx->batch;
        ctx->batch = nullptr;
    }
}
