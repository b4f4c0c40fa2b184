// Direct-sum accelerations (the reference's N^2 mode) for sm_103a.
//
// Reference behaviour restated: a_i = sum_j G*m_j*d_ij/|d_ij|^3 with the radius cutoff of
// source/detail/physics.h:21-42 (CUTOFF law), or softened by eps2 (SOFTENED law). The
// reference's GPU form is one invocation per target over plain SSBO loads
// (shaders/accelerate.comp:9-17, accelerate_split.comp:9-18); its CPU form skips j == i
// (source/solvers/cpu_brute_force.h:32-35). Here self-pairs contribute exactly zero under
// both laws (d = 0 is cut off, or multiplied out by d), so no index test is needed.
//
// Kernel shape (GB300):
//   - a CTA owns BLOCK*T targets: thread t holds targets base + t + k*BLOCK, k < T, in
//     registers as T/2 packed FP32x2 pairs, so every pair interaction issues as
//     3 FADD2 + 3 FFMA2 + 2 MUFU.RSQ + 3 FMUL2 + 3 FFMA2 for two targets.
//   - sources stream through shared memory in TILE-body tiles, STAGES deep, each tile
//     one TMA bulk copy (cp.async.bulk) completing on an mbarrier; every thread reads
//     the same source (a broadcast shared load) and applies it to its T targets. In the
//     pre-paired shapes (DUP) each landed tile is first rewritten once as operand pairs
//     {x,x,y,y}, {z,z,m,m}, which the inner loop reads with two 16-byte loads.
//   - the source range can be split into `jsplit` chunks (blockIdx.y) so that the grid
//     fills the 152 SMs evenly; chunk partials go to a scratch array and are summed in
//     a fixed order (deterministic) by reduce_partials or the fused integrate.
//   - summation: each run of 1024 sources (4 tiles; one 256-source tile when n < 65536)
//     is summed in FP32 from zero, and the run sums are folded into an (S, C) pair per
//     component by an error-free TwoSum, so S + C is the sum of the run sums to about
//     2^-44 of their magnitude. A chunk leaves (S, C); the
//     result is G * float(sum over chunks of S + C, as a double-float sum; direct.cuh
//     combine_partials). The runs are the same sources
//     for every kernel shape and split, so the result does not depend on the
//     launch shape (up to a rounding tie of the last fold), and it is more accurate than
//     one FP32 running sum over all N sources.
#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "direct.cuh"

namespace nbg
{
    // One source (sx, sy, sz, sm) applied to two targets held as negated positions, as
    // scalar FP32 instructions (the same arithmetic; for comparison with the packed form).
    template <int LAW>
    __device__ __forceinline__ void interact2_scalar(const float2 sx, const float2 sy, const float2 sz,
                                                     const float2 sm, const float2 nx, const float2 ny,
                                                     const float2 nz, const float2 lim, float2& ax,
                                                     float2& ay, float2& az)
    {
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            const float dx = (h ? sx.y : sx.x) + (h ? nx.y : nx.x);
            const float dy = (h ? sy.y : sy.x) + (h ? ny.y : ny.x);
            const float dz = (h ? sz.y : sz.x) + (h ? nz.y : nz.x);
            const float l = h ? lim.y : lim.x;
            float r2 = (LAW == NBODY_LAW_SOFTENED) ? fmaf(dx, dx, l) : dx * dx;
            r2 = fmaf(dy, dy, r2);
            r2 = fmaf(dz, dz, r2);
            float inv = rsqrt_sfu(r2);
            if (LAW == NBODY_LAW_CUTOFF)
                inv = r2 > l ? inv : 0.f;
            const float s = ((h ? sm.y : sm.x) * inv) * (inv * inv);
            float& x = h ? ax.y : ax.x;
            float& y = h ? ay.y : ay.x;
            float& z = h ? az.y : az.x;
            x = fmaf(dx, s, x);
            y = fmaf(dy, s, y);
            z = fmaf(dz, s, z);
        }
    }

    // One source (sx, sy, sz, sm) applied to two targets held as negated positions.
    template <int LAW, bool PACKED = true>
    __device__ __forceinline__ void interact2(const float2 sx, const float2 sy, const float2 sz,
                                              const float2 sm, const float2 nx, const float2 ny,
                                              const float2 nz, const float2 lim, float2& ax,
                                              float2& ay, float2& az)
    {
        if (!PACKED)
        {
            interact2_scalar<LAW>(sx, sy, sz, sm, nx, ny, nz, lim, ax, ay, az);
            return;
        }
        const float2 dx = add2(sx, nx);
        const float2 dy = add2(sy, ny);
        const float2 dz = add2(sz, nz);
        float2 r2 = (LAW == NBODY_LAW_SOFTENED) ? fma2(dx, dx, lim) : mul2(dx, dx);
        r2 = fma2(dy, dy, r2);
        r2 = fma2(dz, dz, r2);
        float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
        if (LAW == NBODY_LAW_CUTOFF)
        {
            // physics.h:38-39: nothing when |d|^2 <= radius^2 (lim holds radius^2)
            inv.x = r2.x > lim.x ? inv.x : 0.f;
            inv.y = r2.y > lim.y ? inv.y : 0.f;
        }
        const float2 inv2 = mul2(inv, inv);
        const float2 mi = mul2(sm, inv);
        const float2 s = mul2(mi, inv2);
        ax = fma2(dx, s, ax);
        ay = fma2(dy, s, ay);
        az = fma2(dz, s, az);
    }

    // Fold one tile's FP32 sums t (two targets) into the thread's (S, C) pair, kept at
    // sc[0] and sc[3 * stride] in shared memory: S + t = s + e exactly, S = s, C = C + e.
    __device__ __forceinline__ void fold_tile(float2* sc, const int stride, const float2 t)
    {
        float2 s, e;
        two_sum2(sc[0], t, s, e);
        sc[0] = s;
        sc[3 * stride] = add2(sc[3 * stride], e);
    }

    // Source records: SoA streams one float4 {x,y,z,m} per body; AoS streams the whole
    // 48-byte Body (3 float4: {pos, radius}, {vel, mass}, {acc, pad}).
    template <bool AOS>
    struct Layout
    {
        static constexpr int kRec = AOS ? 3 : 1;
    };

    // DUP: each landed tile is first rewritten in shared memory as source pairs {x,x,y,y},
    // {z,z,m,m}, so the inner loop reads the packed operands ready-made (two 16-byte loads)
    // instead of broadcasting each scalar into a register pair.
    template <int T, int BLOCK, int TILE, int STAGES, int LAW, bool AOS, bool PACKED = true, bool DUP = false>
    __global__ void __launch_bounds__(BLOCK, (T >= 8 ? 2 : 3))
    direct_fp32_kernel(const float4* __restrict__ src,        // pos_mass (SoA) or Body (AoS)
                       const float4* __restrict__ vel_radius, // SoA radius source (CUTOFF)
                       float4* __restrict__ out,              // acc (SoA) / partials
                       float* __restrict__ body_out,          // AoS Body array to write acc
                       const int n, const int chunk, const int fold, const float G, const float eps2,
                       unsigned* __restrict__ err)
    {
        constexpr int P = T / 2;
        constexpr int REC = Layout<AOS>::kRec;
        __shared__ __align__(128) float4 tile[STAGES][TILE * REC];
        __shared__ __align__(16) float4 pairs[DUP ? 2 * TILE : 1];
        __shared__ __align__(8) uint64_t bar[STAGES];
        // Each thread's fold of its tile sums (dynamic shared memory, fold_bytes(T, BLOCK)):
        // row 6p + c holds S of component c (x, y, z) of pair p, row 6p + 3 + c its
        // compensation C; one column per thread, so a warp's accesses are conflict-free.
        // Shared memory rather than registers: the 4 x 256 shape runs three CTAs per SM
        // only within 85 registers.
        extern __shared__ __align__(16) float2 fold_sc[];

        const int tid = threadIdx.x;
        const int base = blockIdx.x * (BLOCK * T);
        const int j0 = blockIdx.y * chunk;
        const int j1 = min(n, j0 + chunk);
        const int ntiles = (j1 > j0) ? (j1 - j0 + TILE - 1) / TILE : 0;

        if (tid == 0)
        {
            for (int s = 0; s < STAGES; ++s)
                mbar_init(&bar[s], 1);
            fence_mbar_init();
        }
        __syncthreads();

        auto issue = [&](const int stage, const int t) {
            const int first = j0 + t * TILE;
            const int cnt = min(TILE, j1 - first);
            const unsigned bytes = static_cast<unsigned>(cnt) * 16u * REC;
            mbar_arrive_expect_tx(&bar[stage], bytes);
            tma_load_1d(&tile[stage][0], src + static_cast<size_t>(first) * REC, bytes, &bar[stage]);
        };
        if (tid == 0)
            for (int s = 0; s < STAGES && s < ntiles; ++s)
                issue(s, s);

        // Targets: negated positions (so d = s + (-x)) and the cutoff radius^2 or eps^2.
        float2 nx[P], ny[P], nz[P], lim[P], ax[P], ay[P], az[P];
#pragma unroll
        for (int p = 0; p < P; ++p)
        {
            float q[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int i = min(base + tid + (2 * p + h) * BLOCK, n - 1);
                const float4 x = src[static_cast<size_t>(i) * REC];
                q[h][0] = -x.x;
                q[h][1] = -x.y;
                q[h][2] = -x.z;
                if (LAW == NBODY_LAW_CUTOFF)
                {
                    const float r = AOS ? x.w : vel_radius[i].w;
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
#pragma unroll
            for (int r = 0; r < 6; ++r)
                fold_sc[(6 * p + r) * BLOCK + tid] = make_float2(0.f, 0.f);
        }

        int failed_at = -1;
        for (int t = 0; t < ntiles; ++t)
        {
            const int stage = t % STAGES;
            const bool ok = mbar_wait_bounded(&bar[stage], (t / STAGES) & 1u, err);
            if (__syncthreads_or(!ok))
            {
                failed_at = t;
                break;
            }
            const int cnt = min(TILE, j1 - (j0 + t * TILE));
            if (cnt < TILE)
            {
                // Last, partial tile: pad with massless sources at the origin, which
                // contribute exactly zero under both laws. The copy only wrote [0, cnt).
                for (int k = cnt * REC + tid; k < TILE * REC; k += BLOCK)
                    tile[stage][k] = make_float4(0.f, 0.f, 0.f, 0.f);
                __syncthreads();
            }
            const float4* tl = tile[stage];
            if (DUP)
            {
                for (int j = tid; j < TILE; j += BLOCK)
                {
                    const float4 s = tl[j * REC];
                    const float m = AOS ? tl[j * REC + 1].w : s.w;
                    pairs[2 * j] = make_float4(s.x, s.x, s.y, s.y);
                    pairs[2 * j + 1] = make_float4(s.z, s.z, m, m);
                }
                __syncthreads();
#pragma unroll 2
                for (int j = 0; j < TILE; ++j)
                {
                    const float4 a = pairs[2 * j], b = pairs[2 * j + 1];
                    const float2 sx = make_float2(a.x, a.y), sy = make_float2(a.z, a.w);
                    const float2 sz = make_float2(b.x, b.y), sm = make_float2(b.z, b.w);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        interact2<LAW, PACKED>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
            }
            else
            {
#pragma unroll 2
                for (int j = 0; j < TILE; ++j)
                {
                    const float4 s = tl[j * REC];
                    const float m = AOS ? tl[j * REC + 1].w : s.w;
                    const float2 sx = f2(s.x), sy = f2(s.y), sz = f2(s.z), sm = f2(m);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        interact2<LAW, PACKED>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
            }
            // every `fold` tiles (and after the chunk's last), fold the running sums into
            // (S, C) and start again from zero; chunks start on fold boundaries
            if ((t + 1) % fold == 0 || t + 1 == ntiles)
#pragma unroll
            for (int p = 0; p < P; ++p)
            {
                fold_tile(&fold_sc[(6 * p) * BLOCK + tid], BLOCK, ax[p]);
                fold_tile(&fold_sc[(6 * p + 1) * BLOCK + tid], BLOCK, ay[p]);
                fold_tile(&fold_sc[(6 * p + 2) * BLOCK + tid], BLOCK, az[p]);
                ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (tid == 0 && t + STAGES < ntiles)
                issue(stage, t + STAGES);
        }
        if (failed_at >= 0)
        {
            // Let the copies still in flight (tiles failed_at .. failed_at+STAGES-1) land,
            // each with a bounded wait, before the CTA's shared memory goes away.
            if (tid == 0)
                for (int t = failed_at; t < ntiles && t < failed_at + STAGES; ++t)
                    mbar_wait_bounded(&bar[t % STAGES], (t / STAGES) & 1u, err);
            return;
        }

        const bool partial = gridDim.y > 1;
#pragma unroll
        for (int p = 0; p < P; ++p)
        {
            float2 S[3], Cc[3];
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
                S[c] = fold_sc[(6 * p + c) * BLOCK + tid];
                Cc[c] = fold_sc[(6 * p + 3 + c) * BLOCK + tid];
            }
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int i = base + tid + (2 * p + h) * BLOCK;
                if (i >= n)
                    continue;
                const float4 s4 = make_float4(h ? S[0].y : S[0].x, h ? S[1].y : S[1].x, h ? S[2].y : S[2].x, 0.f);
                const float4 c4 = make_float4(h ? Cc[0].y : Cc[0].x, h ? Cc[1].y : Cc[1].x, h ? Cc[2].y : Cc[2].x, 0.f);
                if (partial)
                {
                    // the chunk's unscaled (S, C); reduce_partials or the fused integrate sums
                    // them over chunks in FP64 and applies G once
                    out[(2 * static_cast<size_t>(blockIdx.y)) * n + i] = s4;
                    out[(2 * static_cast<size_t>(blockIdx.y) + 1) * n + i] = c4;
                    continue;
                }
                const float3 a = combine_partials(&s4, &c4, 1, 0, 0, G);
                const float a0 = a.x, a1 = a.y, a2 = a.z;
                if (AOS)
                {
                    float* b = body_out + static_cast<size_t>(i) * 12 + 8;
                    b[0] = a0;
                    b[1] = a1;
                    b[2] = a2;
                }
                else
                    out[i] = make_float4(a0, a1, a2, 0.f);
            }
        }
    }

    // Sum jsplit chunk partials in chunk order into acc (SoA float4) or Body::acc (AoS).
    template <int W>
    __global__ void reduce_partials_kernel(const float4* __restrict__ part, const int jsplit,
                                           const int n, const float G, float4* __restrict__ acc,
                                           float* __restrict__ body_out)
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        const int i = t / W, g = t % W;
        if (W == 1 && i >= n)
            return;
        const float3 a = combine_partials_w<W>(part, part + n, jsplit, n, min(i, n - 1), g, G);
        if (i >= n || g != 0)
            return;
        if (body_out)
        {
            float* b = body_out + static_cast<size_t>(i) * 12 + 8;
            b[0] = a.x;
            b[1] = a.y;
            b[2] = a.z;
        }
        else
            acc[i] = make_float4(a.x, a.y, a.z, 0.f);
    }

    // ------------------------------------------------------------------------------
    // Launch planning
    // ------------------------------------------------------------------------------
    namespace
    {
        constexpr int kTile = 256;
        constexpr int kStages = 3;

        using KernelFn = void (*)(const float4*, const float4*, float4*, float*, int, int, int, float,
                                  float, unsigned*);
        // Sources per exact fold of the running sums: 4 tiles (1024) from n = 65536 up, where
        // folding after every tile cost 3 % of the FMA pipe's time at n = 2^20; 1 tile below,
        // where the split gives small systems chunks of a single tile. A function of n only,
        // so every shape at a given n folds at the same sources.
        constexpr int kFoldTiles = 4;
        constexpr size_t kFoldMinN = 65536;

        struct Variant
        {
            int T, block;
            bool packed, dup;
            KernelFn fn[2][2];  // [law][aos]
            int fold_bytes;     // dynamic shared memory: the (S, C) fold, 6 float2 per target pair
        };

        // Dynamic shared memory of a shape's fold array (6 float2 rows per target pair and
        // one column per thread).
        constexpr int fold_bytes_of(const int T, const int block) { return 6 * (T / 2) * block * 8; }

        // Let fn take `bytes` of dynamic shared memory (beyond the 48 KB default where its
        // static tiles and the fold need it). Cheap, and legal while a stream is captured.
        void allow_dynamic_smem(const KernelFn fn, const int bytes)
        {
            cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        }

        constexpr int kPlanned = 3;

        template <int T, int B, bool PACKED = true, bool DUP = false>
        Variant make_variant()
        {
            Variant v;
            v.T = T;
            v.block = B;
            v.packed = PACKED;
            v.dup = DUP;
            v.fn[0][0] = direct_fp32_kernel<T, B, kTile, kStages, NBODY_LAW_CUTOFF, false, PACKED, DUP>;
            v.fn[0][1] = direct_fp32_kernel<T, B, kTile, kStages, NBODY_LAW_CUTOFF, true, PACKED, DUP>;
            v.fn[1][0] = direct_fp32_kernel<T, B, kTile, kStages, NBODY_LAW_SOFTENED, false, PACKED, DUP>;
            v.fn[1][1] = direct_fp32_kernel<T, B, kTile, kStages, NBODY_LAW_SOFTENED, true, PACKED, DUP>;
            v.fold_bytes = fold_bytes_of(T, B);
            return v;
        }

        const Variant* variants(int* count)
        {
            // The first kPlanned entries are what plan_direct chooses between by size; the
            // rest are further shapes the direct-sum autotuner can time and pin.
            static const Variant v[] = {
                make_variant<4, 256, true, true>(),     // the fastest at N >= 65536 (timed)
                make_variant<4, 128>(),
                make_variant<2, 64>(),                  // the fastest at N = 16384
                make_variant<8, 256>(),
                make_variant<4, 256>(),
                make_variant<8, 256, false>(),
                make_variant<8, 128>(),
                make_variant<6, 128>(),
                make_variant<12, 128>(),
                make_variant<8, 256, true, true>(),
            };
            *count = static_cast<int>(sizeof(v) / sizeof(v[0]));
            return v;
        }

        int sm_count()
        {
            static int sms = [] {
                int dev = 0, s = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
                return s > 0 ? s : 1;
            }();
            return sms;
        }

        int occupancy(KernelFn fn, const int block, const int dyn_bytes)
        {
            int blocks = 0;
            allow_dynamic_smem(fn, dyn_bytes);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, block, dyn_bytes) != cudaSuccess)
            {
                cudaGetLastError();
                return 1;
            }
            return blocks > 0 ? blocks : 1;
        }
    }

    DirectPlan plan_direct(const size_t n, const int law, const bool aos, const int force_variant)
    {
        DirectPlan plan{};
        int nv = 0;
        const Variant* vs = variants(&nv);
        const int li = law == NBODY_LAW_SOFTENED ? 1 : 0;
        const int ai = aos ? 1 : 0;
        const int sms = sm_count();

        int chosen = -1;
        if (force_variant >= 0 && force_variant < nv)
            chosen = force_variant;
        else
        {
            // Largest register block whose (target blocks x max chunks) fills the GPU.
            for (int k = 0; k < kPlanned; ++k)
            {
                const size_t per = static_cast<size_t>(vs[k].T) * vs[k].block;
                const size_t tb = (n + per - 1) / per;
                const size_t max_js = std::max<size_t>(1, n / (kTile * 4));
                const size_t slots =
                    static_cast<size_t>(occupancy(vs[k].fn[li][ai], vs[k].block, vs[k].fold_bytes)) * sms;
                if (tb * max_js >= slots)
                {
                    chosen = k;
                    break;
                }
            }
            if (chosen < 0)
                chosen = kPlanned - 1;
        }
        const Variant& v = vs[chosen];
        const size_t per = static_cast<size_t>(v.T) * v.block;
        const size_t tb = std::max<size_t>(1, (n + per - 1) / per);
        const size_t slots = static_cast<size_t>(occupancy(v.fn[li][ai], v.block, v.fold_bytes)) * sms;
        // Split the sources so tb*js CTAs pack into whole waves: minimise the padded
        // work ceil(tb*js/slots)*slots/(tb*js) per unit, preferring fewer chunks. Chunks may
        // be a single tile: at small n the target blocks alone would leave most SMs idle
        // (N = 4096 has 32 target blocks of 128).
        const size_t max_js = std::max<size_t>(1, std::min<size_t>(64, n / kTile));
        size_t best_js = 1;
        double best_cost = 1e300;
        for (size_t js = 1; js <= max_js; ++js)
        {
            const size_t ctas = tb * js;
            const size_t waves = (ctas + slots - 1) / slots;
            // time ~ waves * (work per CTA) = waves / js (work per CTA shrinks with js)
            const double cost = static_cast<double>(waves) / static_cast<double>(js)
                                * (1.0 + 0.002 * static_cast<double>(js));
            if (cost < best_cost - 1e-12)
            {
                best_cost = cost;
                best_js = js;
            }
        }
        // Chunks hold whole fold units, so the last chunk is the only ragged one.
        const int fold = n >= kFoldMinN ? kFoldTiles : 1;
        const size_t unit = static_cast<size_t>(kTile) * fold;
        size_t chunk = (n + best_js - 1) / best_js;
        chunk = (chunk + unit - 1) / unit * unit;
        const size_t js = std::max<size_t>(1, (n + chunk - 1) / chunk);

        plan.variant = chosen;
        plan.T = v.T;
        plan.block = v.block;
        plan.tile = kTile;
        plan.fold = fold;
        plan.jsplit = static_cast<int>(js);
        plan.chunk = static_cast<int>(chunk);
        plan.grid_x = static_cast<int>(tb);
        plan.law = law;
        plan.aos = aos;
        return plan;
    }

    cudaError_t launch_direct(const DirectPlan& plan, const float4* src, const float4* vel_radius,
                              float4* acc, float* body_out, float4* scratch, const int n,
                              const float G, const float eps2, unsigned* err, cudaStream_t stream,
                              uint64_t* launches, const bool reduce)
    {
        if (n <= 0)
            return cudaSuccess;
        int nv = 0;
        const Variant* vs = variants(&nv);
        const Variant& v = vs[plan.variant];
        const KernelFn fn = v.fn[plan.law == NBODY_LAW_SOFTENED ? 1 : 0][plan.aos ? 1 : 0];
        const dim3 grid(plan.grid_x, plan.jsplit);
        float4* out = plan.jsplit > 1 ? scratch : acc;
        allow_dynamic_smem(fn, v.fold_bytes);
        fn<<<grid, v.block, v.fold_bytes, stream>>>(src, vel_radius, out, plan.aos ? body_out : nullptr, n,
                                                    plan.chunk, plan.fold, G, eps2, err);
        ++*launches;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess || plan.jsplit <= 1 || !reduce)
            return e;
        return launch_reduce(scratch, plan.jsplit, n, G, acc, plan.aos ? body_out : nullptr, stream, launches);
    }

    int direct_variant_count()
    {
        int nv = 0;
        variants(&nv);
        return nv;
    }

    void direct_variant_describe(const int i, int* T, int* block, int* packed)
    {
        int nv = 0;
        const Variant* vs = variants(&nv);
        *T = vs[i].T;
        *block = vs[i].block;
        *packed = vs[i].dup ? 2 : (vs[i].packed ? 1 : 0);
    }

    cudaError_t launch_reduce(const float4* scratch, const int jsplit, const int n, const float G, float4* acc,
                              float* body_out, cudaStream_t stream, uint64_t* launches)
    {
        if (combine_width(n, jsplit) == 8)
            reduce_partials_kernel<8><<<ceil_div(static_cast<size_t>(n) * 8, 256), 256, 0, stream>>>(
                scratch, jsplit, n, G, acc, body_out);
        else
            reduce_partials_kernel<1><<<ceil_div(n, 256), 256, 0, stream>>>(scratch, jsplit, n, G, acc, body_out);
        ++*launches;
        return cudaGetLastError();
    }
}
