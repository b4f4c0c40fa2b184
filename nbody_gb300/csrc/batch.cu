// Batched direct sums: many independent systems of uneven size advanced by one persistent
// launch per accelerate (no reference counterpart; the reference runs one system per Sim).
//
// Work decomposition: the bodies of all systems are concatenated (system s owns
// [off[s], off[s+1])). A work item is (system, first target) covering the TB targets one
// CTA holds. Items are listed largest system first and a grid of (SMs x resident CTAs)
// persistent CTAs pulls them from an atomic counter -- each pull is one atomicAdd, nothing
// ever waits on another CTA, so there is no spin to bound.
//
// Per item: the system's bodies stream through shared memory in TILE-body TMA bulk copies
// (two stages, mbarrier completion, stage/parity carried across items); a group of TPT
// consecutive lanes shares each target, lane `sub` of the group taking sources sub,
// sub + TPT, ...; the group's partial sums are then combined with warp shuffles. Small
// systems want TPT > 1 (more parallelism per item, fewer idle threads), large ones TPT = 1
// (no reduction): the autotuner times every instantiated (TPT, T, UNROLL) and keeps the
// fastest for the batch at hand.
#include <algorithm>
#include <vector>

#include "batch.cuh"
#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kBlock = 256;
        constexpr int kTile = 256;
        constexpr int kStages = 2;
        constexpr int kEnergyBlock = 128;
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

    template <int TPT, int T, int UNROLL, int LAW>
    __global__ void __launch_bounds__(kBlock)
    batch_kernel(const float4* __restrict__ pm, const float4* __restrict__ vr, const int* __restrict__ off,
                 const int2* __restrict__ items, const int nitems, unsigned* __restrict__ counter,
                 float4* __restrict__ acc, const float G, const float eps2, unsigned* __restrict__ err)
    {
        constexpr int P = T / 2;
        constexpr int GROUPS = kBlock / TPT;
        __shared__ __align__(128) float4 tile[kStages][kTile];
        __shared__ __align__(8) uint64_t bar[kStages];
        __shared__ int item_s;
        const int tid = threadIdx.x;
        const int group = tid / TPT, sub = tid % TPT;
        if (tid == 0)
        {
            for (int s = 0; s < kStages; ++s)
                mbar_init(&bar[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        unsigned seq = 0;   // tiles this CTA has consumed so far (stage = seq % 2, parity = seq / 2)

        for (;;)
        {
            if (tid == 0)
                item_s = static_cast<int>(atomicAdd(counter, 1u));
            __syncthreads();
            const int it = item_s;
            __syncthreads();
            if (it >= nitems)
                break;
            const int2 w = items[it];
            const int base = off[w.x];
            const int n = off[w.x + 1] - base;
            const int ntiles = (n + kTile - 1) / kTile;
            auto issue = [&](const int k) {
                const int first = k * kTile;
                const int cnt = min(kTile, n - first);
                const unsigned stage = (seq + k) % kStages;
                mbar_arrive_expect_tx(&bar[stage], static_cast<unsigned>(cnt) * 16u);
                tma_load_1d(&tile[stage][0], pm + base + first, static_cast<unsigned>(cnt) * 16u, &bar[stage]);
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
                    const int t = min(w.y + group + (2 * p + h) * GROUPS, n - 1);
                    const float4 x = pm[base + t];
                    q[h][0] = -x.x;
                    q[h][1] = -x.y;
                    q[h][2] = -x.z;
                    if (LAW == NBODY_LAW_CUTOFF)
                    {
                        const float r = vr[base + t].w;
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

            int failed_at = -1;
            for (int k = 0; k < ntiles; ++k)
            {
                const unsigned stage = (seq + k) % kStages;
                const bool ok = mbar_wait_bounded(&bar[stage], ((seq + k) / kStages) & 1u, err);
                if (__syncthreads_or(!ok))
                {
                    failed_at = k;
                    break;
                }
                const int cnt = min(kTile, n - k * kTile);
                const float4* tl = tile[stage];
#pragma unroll UNROLL
                for (int j = sub; j < cnt; j += TPT)
                {
                    const float4 s = tl[j];
                    const float2 sx = f2(s.x), sy = f2(s.y), sz = f2(s.z), sm = f2(s.w);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        bpair<LAW>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
                __syncthreads();
                if (tid == 0 && k + kStages < ntiles)
                    issue(k + kStages);
            }
            if (failed_at >= 0)
            {
                // a copy that never landed (the error word says so): let the ones still in
                // flight land, each with a bounded wait, before the CTA's shared memory goes
                if (tid == 0)
                    for (int k = failed_at; k < ntiles && k < failed_at + kStages; ++k)
                        mbar_wait_bounded(&bar[(seq + k) % kStages], ((seq + k) / kStages) & 1u, err);
                return;
            }
            seq += static_cast<unsigned>(ntiles);

            // combine the TPT partial sums of each target (contiguous lanes of one warp)
#pragma unroll
            for (int p = 0; p < P; ++p)
            {
#pragma unroll
                for (int o = TPT / 2; o > 0; o >>= 1)
                {
                    ax[p].x += __shfl_xor_sync(0xffffffffu, ax[p].x, o);
                    ax[p].y += __shfl_xor_sync(0xffffffffu, ax[p].y, o);
                    ay[p].x += __shfl_xor_sync(0xffffffffu, ay[p].x, o);
                    ay[p].y += __shfl_xor_sync(0xffffffffu, ay[p].y, o);
                    az[p].x += __shfl_xor_sync(0xffffffffu, az[p].x, o);
                    az[p].y += __shfl_xor_sync(0xffffffffu, az[p].y, o);
                }
            }
            if (sub == 0)
            {
#pragma unroll
                for (int p = 0; p < P; ++p)
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                    {
                        const int t = w.y + group + (2 * p + h) * GROUPS;
                        if (t < n)
                            acc[base + t] = make_float4(G * (h ? ax[p].y : ax[p].x), G * (h ? ay[p].y : ay[p].x),
                                                        G * (h ? az[p].y : az[p].x), 0.f);
                    }
            }
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
        using BatchFn = void (*)(const float4*, const float4*, const int*, const int2*, int, unsigned*, float4*,
                                 float, float, unsigned*);

        struct Config
        {
            int tpt, t, unroll;
            BatchFn soft, cutoff;
        };

        template <int TPT, int T, int U>
        Config cfg()
        {
            return { TPT, T, U, batch_kernel<TPT, T, U, NBODY_LAW_SOFTENED>,
                     (TPT == 1 && T == 2 && U == 2) ? batch_kernel<1, 2, 2, NBODY_LAW_CUTOFF> : nullptr };
        }

        const std::vector<Config>& configs()
        {
            static const std::vector<Config> c = {
                cfg<1, 2, 2>(), cfg<1, 2, 4>(), cfg<1, 4, 2>(), cfg<1, 4, 4>(),
                cfg<2, 2, 2>(), cfg<2, 2, 4>(), cfg<2, 4, 2>(), cfg<2, 4, 4>(),
                cfg<4, 2, 2>(), cfg<4, 2, 4>(), cfg<4, 4, 2>(), cfg<4, 4, 4>(),
                cfg<8, 2, 2>(), cfg<8, 2, 4>(), cfg<8, 4, 2>(), cfg<8, 4, 4>(),
                cfg<2, 8, 2>(), cfg<4, 8, 2>(), cfg<8, 8, 2>(), cfg<8, 8, 4>(),
                cfg<16, 4, 4>(), cfg<16, 8, 2>(),
            };
            return c;
        }

        int targets_per_item(const Config& c) { return kBlock / c.tpt * c.t; }
    }

    struct BatchState
    {
        std::vector<int> off;           // host copy of the system table
        int* d_off = nullptr;
        size_t off_cap = 0;
        int2* d_items = nullptr;        // work list of the active configuration
        size_t items_cap = 0;
        int nitems = 0;
        int items_tb = 0;               // targets per item the list was built for
        unsigned* counter = nullptr;
        int config = 0;                 // index into configs()
        bool tuned = false;
    };

    int batch_config_count() { return static_cast<int>(configs().size()); }

    void batch_config_describe(const int i, int* tpt, int* t, int* unroll)
    {
        const Config& c = configs()[i];
        *tpt = c.tpt;
        *t = c.t;
        *unroll = c.unroll;
    }

    namespace
    {
        // Largest systems first: the longest items start first, the short ones fill the tail.
        std::vector<int2> make_items(const std::vector<int>& off, const int tb)
        {
            std::vector<int> order(off.size() - 1);
            for (size_t s = 0; s < order.size(); ++s)
                order[s] = static_cast<int>(s);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return off[a + 1] - off[a] > off[b + 1] - off[b];
            });
            std::vector<int2> items;
            for (const int s : order)
                for (int t = 0; t < off[s + 1] - off[s]; t += tb)
                    items.push_back(make_int2(s, t));
            return items;
        }

        int upload_items(nbody_cuda* ctx, const std::vector<int2>& items, int2** dst, size_t* cap)
        {
            if (items.size() > *cap)
            {
                cudaFreeAsync(*dst, ctx->stream);
                *dst = nullptr;
                *cap = 0;
                const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(dst), items.size() * sizeof(int2), ctx->stream);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "batch work list allocation");
                *cap = items.size();
                ++ctx->generation;
            }
            if (!items.empty())
            {
                const cudaError_t e = cudaMemcpyAsync(*dst, items.data(), items.size() * sizeof(int2),
                                                      cudaMemcpyHostToDevice, ctx->stream);
                if (e == cudaSuccess)
                    cudaStreamSynchronize(ctx->stream);     // the host vector goes out of scope
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "batch work list upload");
            }
            return NBODY_OK;
        }

        int ensure_items(nbody_cuda* ctx, const int config)
        {
            BatchState& b = *ctx->batch;
            const int tb = targets_per_item(configs()[config]);
            if (b.items_tb == tb)
                return NBODY_OK;
            const std::vector<int2> items = make_items(b.off, tb);
            if (const int st = upload_items(ctx, items, &b.d_items, &b.items_cap))
                return st;
            b.nitems = static_cast<int>(items.size());
            b.items_tb = tb;
            return NBODY_OK;
        }

        int occupancy_grid(nbody_cuda* ctx, BatchFn fn, const int nitems)
        {
            int sms = 0, per = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kBlock, 0) != cudaSuccess || per < 1)
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
        b.items_tb = 0;
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
        // the cutoff law is instantiated for the first configuration only
        const int ci = (p->law == NBODY_LAW_CUTOFF && !configs()[b.config].cutoff) ? 0 : b.config;
        const Config& c = configs()[ci];
        if (const int st = ensure_items(ctx, ci))
            return st;
        const BatchFn fn = p->law == NBODY_LAW_SOFTENED ? c.soft : c.cutoff;
        const int grid = occupancy_grid(ctx, fn, b.nitems);
        cudaMemsetAsync(b.counter, 0, sizeof(unsigned), ctx->stream);
        fn<<<grid, kBlock, 0, ctx->stream>>>(ctx->pm, ctx->vr, b.d_off, b.d_items, b.nitems, b.counter, ctx->acc, p->G,
                                             p->eps2, ctx->dev_error);
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
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        int best_i = 0;
        float best_ms = 1e30f;
        for (int i = 0; i < batch_config_count(); ++i)
        {
            b.config = i;
            b.items_tb = 0;
            float ms_best = 1e30f;
            for (int rep = 0; rep < 3; ++rep)
            {
                cudaEventRecord(e0, ctx->stream);
                if (const int st = batch_accelerate(ctx, &q))
                {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return st;
                }
                cudaEventRecord(e1, ctx->stream);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
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
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b.config = best_i;
        b.items_tb = 0;
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
        ctx->batch->items_tb = 0;
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
        delete ctx->batch;
        ctx->batch = nullptr;
    }
}
