// Split-precision ("compensated") and FP64 direct sums, and the compensated integrator.
//
// Compensated form (no reference counterpart; the reference is FP32 throughout):
//   - positions are an FP64 origin per context plus FP32 offsets. The origin is a corner
//     of the power-of-two grid that holds the bodies (a multiple of the box edge), which
//     makes x - origin exact in FP32 for every body when the state is set up, and keeps
//     the offsets small wherever the system sits in space;
//   - pair forces are the FP32 ones of the plain kernel (same 12 lane-ops per pair),
//     summed in FP32 over 64-source sub-tiles; the sub-tile sums are Kahan-added into a
//     running (sum, compensation) pair per target, and the chunk partials are summed in
//     FP64 -- so the summation error no longer grows with N;
//   - the integrator keeps Kahan compensation terms for the velocity and the offset, and
//     writes the rounded float positions back to the body streams every step.
// FP64 form: the whole pair sum in FP64 (positions promoted exactly from the FP32 offsets
// plus the FP64 origin, or from the float positions when no split state exists).
#include <algorithm>

#include "common.cuh"
#include "context.cuh"
#include "direct.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kSub = 64;        // sources per FP32 sub-tile sum
        constexpr int kTileC = 256;     // sources per TMA tile (compensated)
        constexpr int kTile64 = 128;    // sources per TMA tile (FP64)
        constexpr int kStages = 3;
        constexpr int kBboxBlocks = 512;
    }

    struct PreciseState
    {
        size_t cap = 0;
        float4* off = nullptr;      // offset xyz from the origin, mass
        float4* cx = nullptr;       // Kahan compensation of the offset
        float4* cv = nullptr;       // Kahan compensation of the velocity
        double4* pos64 = nullptr;   // FP64 positions + mass (FP64 form)
        double* origin = nullptr;   // device: origin xyz, edge
        double* part = nullptr;     // bounding-box partials
        int* tlist = nullptr;       // sampled targets
        size_t tlist_cap = 0;
        double4* out64 = nullptr;   // sampled results
    };

    // --------------------------------------------------------------------------------------
    // set-up of the split state
    // --------------------------------------------------------------------------------------
    __global__ void minmax_kernel(const float4* __restrict__ src, const int stride, const int n,
                                  double* __restrict__ part)
    {
        double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const float4 p = src[static_cast<size_t>(i) * stride];
            lo[0] = fmin(lo[0], (double)p.x); hi[0] = fmax(hi[0], (double)p.x);
            lo[1] = fmin(lo[1], (double)p.y); hi[1] = fmax(hi[1], (double)p.y);
            lo[2] = fmin(lo[2], (double)p.z); hi[2] = fmax(hi[2], (double)p.z);
        }
        __shared__ double red[6][256];
        for (int a = 0; a < 3; ++a)
        {
            red[a][threadIdx.x] = lo[a];
            red[3 + a][threadIdx.x] = hi[a];
        }
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1)
        {
            if (threadIdx.x < s)
                for (int a = 0; a < 3; ++a)
                {
                    red[a][threadIdx.x] = fmin(red[a][threadIdx.x], red[a][threadIdx.x + s]);
                    red[3 + a][threadIdx.x] = fmax(red[3 + a][threadIdx.x], red[3 + a][threadIdx.x + s]);
                }
            __syncthreads();
        }
        if (threadIdx.x < 6)
            part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
    }

    // Per axis: origin 0 when the bodies straddle 0 (then offset == x, exactly); otherwise
    // the multiple of e nearest the box centre, e the power of two >= the largest extent,
    // so that the origin lies within e/2 of the centre and x - origin is exact by Sterbenz's
    // lemma for a system far from 0 (its whole point). Whatever rounding remains at set-up
    // goes into the compensation term, so origin + offset - compensation == x exactly.
    __global__ void origin_kernel(const double* __restrict__ part, const int nparts, double* __restrict__ origin)
    {
        if (threadIdx.x || blockIdx.x)
            return;
        double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
        for (int k = 0; k < nparts; ++k)
            for (int a = 0; a < 3; ++a)
            {
                lo[a] = fmin(lo[a], part[k * 6 + a]);
                hi[a] = fmax(hi[a], part[k * 6 + 3 + a]);
            }
        double ext = 0.0;
        for (int a = 0; a < 3; ++a)
            ext = fmax(ext, hi[a] - lo[a]);
        const double e = (ext > 0.0 && isfinite(ext)) ? exp2(ceil(log2(ext))) : 1.0;
        for (int a = 0; a < 3; ++a)
        {
            double o = 0.0;
            if (isfinite(lo[a]) && (lo[a] > 0.0 || hi[a] < 0.0))
                o = rint(0.5 * (lo[a] + hi[a]) / e) * e;
            origin[a] = o;
        }
        origin[3] = e;
    }

    __global__ void to_offsets_kernel(const float4* __restrict__ src, const int stride, const int n,
                                      const double* __restrict__ origin, float4* __restrict__ off,
                                      float4* __restrict__ cx, float4* __restrict__ cv)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        const float4 p = src[static_cast<size_t>(i) * stride];
        const float m = stride == 3 ? src[static_cast<size_t>(i) * 3 + 1].w : p.w;
        const double r[3] = { p.x - origin[0], p.y - origin[1], p.z - origin[2] };   // exact in FP64
        const float o[3] = { static_cast<float>(r[0]), static_cast<float>(r[1]), static_cast<float>(r[2]) };
        off[i] = make_float4(o[0], o[1], o[2], m);
        // Kahan convention: true = offset - compensation
        cx[i] = make_float4(static_cast<float>(o[0] - r[0]), static_cast<float>(o[1] - r[1]),
                            static_cast<float>(o[2] - r[2]), 0.f);
        cv[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    // FP64 positions: origin + (offset - compensation), or the float positions promoted.
    __global__ void pos64_kernel(const float4* __restrict__ src, const int stride, const float4* __restrict__ off,
                                 const float4* __restrict__ cx, const double* __restrict__ origin, const int n,
                                 double4* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        if (off)
        {
            const float4 o = off[i], c = cx[i];
            out[i] = make_double4(origin[0] + ((double)o.x - (double)c.x), origin[1] + ((double)o.y - (double)c.y),
                                  origin[2] + ((double)o.z - (double)c.z), (double)o.w);
        }
        else
        {
            const float4 p = src[static_cast<size_t>(i) * stride];
            const float m = stride == 3 ? src[static_cast<size_t>(i) * 3 + 1].w : p.w;
            out[i] = make_double4(p.x, p.y, p.z, m);
        }
    }

    // --------------------------------------------------------------------------------------
    // compensated direct sum
    // --------------------------------------------------------------------------------------
    __device__ __forceinline__ void kahan(float& s, float& c, const float v)
    {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }

    template <int LAW>
    __device__ __forceinline__ void interact2c(const float2 sx, const float2 sy, const float2 sz, const float2 sm,
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
        const float2 mi = mul2(sm, inv);
        const float2 s = mul2(mi, inv2);
        ax = fma2(dx, s, ax);
        ay = fma2(dy, s, ay);
        az = fma2(dz, s, az);
    }

    // Targets: all n (tlist == nullptr) or tlist[0 .. nt). Output: FP64 partials
    // part[blockIdx.y * nt + t] = G * (sum - compensation).
    template <int T, int BLOCK, int LAW>
    __global__ void __launch_bounds__(BLOCK, 2)
    direct_comp_kernel(const float4* __restrict__ src, const float* __restrict__ radius2, const int* __restrict__ tlist,
                       const int nt, const int n, const int chunk, const float G, const float eps2,
                       double4* __restrict__ part, unsigned* __restrict__ err)
    {
        constexpr int P = T / 2;
        __shared__ __align__(128) float4 tile[kStages][kTileC];
        // each landed tile rewritten as operand pairs {x,x,y,y}, {z,z,m,m} (see direct.cu)
        __shared__ __align__(16) float4 pairs[2 * kTileC];
        __shared__ __align__(8) uint64_t bar[kStages];
        const int tid = threadIdx.x;
        const int base = blockIdx.x * (BLOCK * T);
        const int j0 = blockIdx.y * chunk;
        const int j1 = min(n, j0 + chunk);
        const int ntiles = (j1 > j0) ? (j1 - j0 + kTileC - 1) / kTileC : 0;
        if (tid == 0)
        {
            for (int s = 0; s < kStages; ++s)
                mbar_init(&bar[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        auto issue = [&](const int stage, const int t) {
            const int first = j0 + t * kTileC;
            const int cnt = min(kTileC, j1 - first);
            const unsigned bytes = static_cast<unsigned>(cnt) * 16u;
            mbar_arrive_expect_tx(&bar[stage], bytes);
            tma_load_1d(&tile[stage][0], src + first, bytes, &bar[stage]);
        };
        if (tid == 0)
            for (int s = 0; s < kStages && s < ntiles; ++s)
                issue(s, s);

        float2 nx[P], ny[P], nz[P], lim[P], ax[P], ay[P], az[P];
        float2 sx_[P], sy_[P], sz_[P], cx_[P], cy_[P], cz_[P];
#pragma unroll
        for (int p = 0; p < P; ++p)
        {
            float q[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int t = min(base + tid + (2 * p + h) * BLOCK, nt - 1);
                const int i = tlist ? tlist[t] : t;
                const float4 x = src[i];
                q[h][0] = -x.x;
                q[h][1] = -x.y;
                q[h][2] = -x.z;
                q[h][3] = (LAW == NBODY_LAW_CUTOFF) ? radius2[i] : eps2;
            }
            nx[p] = make_float2(q[0][0], q[1][0]);
            ny[p] = make_float2(q[0][1], q[1][1]);
            nz[p] = make_float2(q[0][2], q[1][2]);
            lim[p] = make_float2(q[0][3], q[1][3]);
            ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
            sx_[p] = sy_[p] = sz_[p] = cx_[p] = cy_[p] = cz_[p] = make_float2(0.f, 0.f);
        }

        int failed_at = -1;
        for (int t = 0; t < ntiles; ++t)
        {
            const int stage = t % kStages;
            const bool ok = mbar_wait_bounded(&bar[stage], (t / kStages) & 1u, err);
            if (__syncthreads_or(!ok))
            {
                failed_at = t;
                break;
            }
            const int cnt = min(kTileC, j1 - (j0 + t * kTileC));
            if (cnt < kTileC)
            {
                for (int k = cnt + tid; k < kTileC; k += BLOCK)
                    tile[stage][k] = make_float4(0.f, 0.f, 0.f, 0.f);
                __syncthreads();
            }
            const float4* tl = tile[stage];
            for (int j = tid; j < kTileC; j += BLOCK)
            {
                const float4 s = tl[j];
                pairs[2 * j] = make_float4(s.x, s.x, s.y, s.y);
                pairs[2 * j + 1] = make_float4(s.z, s.z, s.w, s.w);
            }
            __syncthreads();
            for (int sb = 0; sb < kTileC; sb += kSub)
            {
#pragma unroll 2
                for (int j = sb; j < sb + kSub; ++j)
                {
                    const float4 a = pairs[2 * j], b = pairs[2 * j + 1];
                    const float2 sx = make_float2(a.x, a.y), sy = make_float2(a.z, a.w);
                    const float2 sz = make_float2(b.x, b.y), sm = make_float2(b.z, b.w);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        interact2c<LAW>(sx, sy, sz, sm, nx[p], ny[p], nz[p], lim[p], ax[p], ay[p], az[p]);
                }
#pragma unroll
                for (int p = 0; p < P; ++p)
                {
                    kahan(sx_[p].x, cx_[p].x, ax[p].x);
                    kahan(sx_[p].y, cx_[p].y, ax[p].y);
                    kahan(sy_[p].x, cy_[p].x, ay[p].x);
                    kahan(sy_[p].y, cy_[p].y, ay[p].y);
                    kahan(sz_[p].x, cz_[p].x, az[p].x);
                    kahan(sz_[p].y, cz_[p].y, az[p].y);
                    ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
                }
            }
            __syncthreads();
            if (tid == 0 && t + kStages < ntiles)
                issue(stage, t + kStages);
        }
        if (failed_at >= 0)
        {
            if (tid == 0)
                for (int t = failed_at; t < ntiles && t < failed_at + kStages; ++t)
                    mbar_wait_bounded(&bar[t % kStages], (t / kStages) & 1u, err);
            return;
        }
#pragma unroll
        for (int p = 0; p < P; ++p)
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int t = base + tid + (2 * p + h) * BLOCK;
                if (t >= nt)
                    continue;
                const double g = G;
                const double rx = h ? (double)sx_[p].y - (double)cx_[p].y : (double)sx_[p].x - (double)cx_[p].x;
                const double ry = h ? (double)sy_[p].y - (double)cy_[p].y : (double)sy_[p].x - (double)cy_[p].x;
                const double rz = h ? (double)sz_[p].y - (double)cz_[p].y : (double)sz_[p].x - (double)cz_[p].x;
                part[static_cast<size_t>(blockIdx.y) * nt + t] = make_double4(g * rx, g * ry, g * rz, 0.0);
            }
    }

    // --------------------------------------------------------------------------------------
    // FP64 direct sum (sources staged as double4 tiles)
    // --------------------------------------------------------------------------------------
    template <int BLOCK, int LAW>
    __global__ void __launch_bounds__(BLOCK)
    direct_fp64_kernel(const double4* __restrict__ src, const float* __restrict__ radius2, const int* __restrict__ tlist,
                       const int nt, const int n, const int chunk, const double G, const double eps2,
                       double4* __restrict__ part, unsigned* __restrict__ err)
    {
        constexpr int T = 2;
        __shared__ __align__(128) double4 tile[kStages][kTile64];
        __shared__ __align__(8) uint64_t bar[kStages];
        const int tid = threadIdx.x;
        const int base = blockIdx.x * (BLOCK * T);
        const int j0 = blockIdx.y * chunk;
        const int j1 = min(n, j0 + chunk);
        const int ntiles = (j1 > j0) ? (j1 - j0 + kTile64 - 1) / kTile64 : 0;
        if (tid == 0)
        {
            for (int s = 0; s < kStages; ++s)
                mbar_init(&bar[s], 1);
            fence_mbar_init();
        }
        __syncthreads();
        auto issue = [&](const int stage, const int t) {
            const int first = j0 + t * kTile64;
            const int cnt = min(kTile64, j1 - first);
            const unsigned bytes = static_cast<unsigned>(cnt) * 32u;
            mbar_arrive_expect_tx(&bar[stage], bytes);
            tma_load_1d(&tile[stage][0], src + first, bytes, &bar[stage]);
        };
        if (tid == 0)
            for (int s = 0; s < kStages && s < ntiles; ++s)
                issue(s, s);
        double px[T], py[T], pz[T], lim[T], ax[T], ay[T], az[T];
#pragma unroll
        for (int k = 0; k < T; ++k)
        {
            const int t = min(base + tid + k * BLOCK, nt - 1);
            const int i = tlist ? tlist[t] : t;
            const double4 x = src[i];
            px[k] = x.x;
            py[k] = x.y;
            pz[k] = x.z;
            lim[k] = (LAW == NBODY_LAW_CUTOFF) ? (double)radius2[i] : eps2;
            ax[k] = ay[k] = az[k] = 0.0;
        }
        int failed_at = -1;
        for (int t = 0; t < ntiles; ++t)
        {
            const int stage = t % kStages;
            const bool ok = mbar_wait_bounded(&bar[stage], (t / kStages) & 1u, err);
            if (__syncthreads_or(!ok))
            {
                failed_at = t;
                break;
            }
            const int cnt = min(kTile64, j1 - (j0 + t * kTile64));
            if (cnt < kTile64)
            {
                for (int k = cnt + tid; k < kTile64; k += BLOCK)
                    tile[stage][k] = make_double4(0, 0, 0, 0);
                __syncthreads();
            }
            const double4* tl = tile[stage];
            for (int j = 0; j < kTile64; ++j)
            {
                const double4 s = tl[j];
#pragma unroll
                for (int k = 0; k < T; ++k)
                {
                    const double dx = s.x - px[k], dy = s.y - py[k], dz = s.z - pz[k];
                    double r2 = (LAW == NBODY_LAW_SOFTENED) ? fma(dx, dx, lim[k]) : dx * dx;
                    r2 = fma(dy, dy, r2);
                    r2 = fma(dz, dz, r2);
                    double inv = rsqrt(r2);
                    if (LAW == NBODY_LAW_CUTOFF)
                        inv = r2 > lim[k] ? inv : 0.0;
                    if (!(r2 > 0.0))
                        inv = 0.0;      // massless padding at the origin / self at d = 0
                    const double f = s.w * inv * inv * inv;
                    ax[k] = fma(dx, f, ax[k]);
                    ay[k] = fma(dy, f, ay[k]);
                    az[k] = fma(dz, f, az[k]);
                }
            }
            __syncthreads();
            if (tid == 0 && t + kStages < ntiles)
                issue(stage, t + kStages);
        }
        if (failed_at >= 0)
        {
            if (tid == 0)
                for (int t = failed_at; t < ntiles && t < failed_at + kStages; ++t)
                    mbar_wait_bounded(&bar[t % kStages], (t / kStages) & 1u, err);
            return;
        }
#pragma unroll
        for (int k = 0; k < T; ++k)
        {
            const int t = base + tid + k * BLOCK;
            if (t < nt)
                part[static_cast<size_t>(blockIdx.y) * nt + t] = make_double4(G * ax[k], G * ay[k], G * az[k], 0.0);
        }
    }

    // Fixed-order FP64 sum of chunk partials -> float acc (SoA/AoS, indexed through tlist
    // when sampling) and/or double results.
    __global__ void reduce64_kernel(const double4* __restrict__ part, const int js, const int nt,
                                    const int* __restrict__ tlist, float4* __restrict__ acc, float* __restrict__ body_out,
                                    double4* __restrict__ out64)
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= nt)
            return;
        double4 a = part[t];
        for (int s = 1; s < js; ++s)
        {
            const double4 b = part[static_cast<size_t>(s) * nt + t];
            a.x += b.x;
            a.y += b.y;
            a.z += b.z;
        }
        if (out64)
            out64[t] = a;
        const int i = tlist ? tlist[t] : t;
        if (acc)
            acc[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
        if (body_out)
        {
            float* o = body_out + static_cast<size_t>(i) * 12 + 8;
            o[0] = (float)a.x;
            o[1] = (float)a.y;
            o[2] = (float)a.z;
        }
    }

    __global__ void radius2_kernel(const float4* __restrict__ src, const int stride, const float4* __restrict__ vr,
                                   const int n, float* __restrict__ out)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        const float r = stride == 3 ? src[static_cast<size_t>(i) * 3].w : (vr ? vr[i].w : 0.f);
        out[i] = r * r;
    }

    // --------------------------------------------------------------------------------------
    // compensated integrator
    // --------------------------------------------------------------------------------------
    __global__ void integrate_comp_kernel(float4* __restrict__ off, float4* __restrict__ cx, float4* __restrict__ cv,
                                          float4* __restrict__ pm, float4* __restrict__ vr, float* __restrict__ bodies,
                                          const float4* __restrict__ acc, const double* __restrict__ origin,
                                          const int n, const float dt, const float size, const int wrap)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        float4 o = off[i], c = cx[i], w = cv[i];
        float4 v, a;
        if (bodies)
        {
            const float4* b = reinterpret_cast<const float4*>(bodies) + static_cast<size_t>(i) * 3;
            v = b[1];
            a = b[2];
        }
        else
        {
            v = vr[i];
            a = acc[i];
        }
        // v += a*dt and x += v*dt, each as a Kahan-compensated sum
        kahan(v.x, w.x, __fmul_rn(a.x, dt));
        kahan(v.y, w.y, __fmul_rn(a.y, dt));
        kahan(v.z, w.z, __fmul_rn(a.z, dt));
        kahan(o.x, c.x, __fmul_rn(v.x, dt));
        kahan(o.y, c.y, __fmul_rn(v.y, dt));
        kahan(o.z, c.z, __fmul_rn(v.z, dt));
        double pos[3] = { origin[0] + ((double)o.x - (double)c.x), origin[1] + ((double)o.y - (double)c.y),
                          origin[2] + ((double)o.z - (double)c.z) };
        if (wrap && size > 0.f)
        {
            // the 3-torus of physics.h:50-58, applied to the compensated position in FP64;
            // a wrapped body's offset and compensation are re-derived from the new position
            const double s = size, half = 0.5 * s;
            float* oo[3] = { &o.x, &o.y, &o.z };
            float* cc[3] = { &c.x, &c.y, &c.z };
            for (int a = 0; a < 3; ++a)
                if (pos[a] < -half || pos[a] > half)
                {
                    pos[a] = fmod(fmod(pos[a] + half, s) + s, s) - half;
                    const double r = pos[a] - origin[a];
                    *oo[a] = (float)r;
                    *cc[a] = (float)((double)*oo[a] - r);
                }
        }
        off[i] = o;
        cx[i] = c;
        cv[i] = w;
        const float x = (float)pos[0];
        const float y = (float)pos[1];
        const float z = (float)pos[2];
        if (bodies)
        {
            float4* b = reinterpret_cast<float4*>(bodies) + static_cast<size_t>(i) * 3;
            b[0] = make_float4(x, y, z, b[0].w);
            b[1] = make_float4(v.x, v.y, v.z, v.w);
        }
        else
        {
            pm[i] = make_float4(x, y, z, o.w);
            vr[i] = v;
        }
    }

    // --------------------------------------------------------------------------------------
    // host side
    // --------------------------------------------------------------------------------------
    namespace
    {
        template <typename T>
        cudaError_t regrow(T** p, size_t count, cudaStream_t s)
        {
            if (*p)
                cudaFreeAsync(*p, s);
            *p = nullptr;
            return cudaMallocAsync(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T), s);
        }

        const float4* body_src(const nbody_cuda* ctx, int* stride)
        {
            if (ctx->layout == NBODY_LAYOUT_AOS)
            {
                *stride = 3;
                return reinterpret_cast<const float4*>(ctx->bodies);
            }
            *stride = 1;
            return ctx->pm;
        }

        int reserve_precise(nbody_cuda* ctx, const size_t n)
        {
            if (!ctx->precise)
                ctx->precise = new PreciseState();
            PreciseState& s = *ctx->precise;
            cudaStream_t st = ctx->stream;
            if (!s.origin)
            {
                cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&s.origin), 4 * sizeof(double), st);
                if (e == cudaSuccess)
                    e = cudaMallocAsync(reinterpret_cast<void**>(&s.part), kBboxBlocks * 6 * sizeof(double), st);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "precision state allocation");
            }
            if (n <= s.cap)
                return NBODY_OK;
            if (const int st = before_allocation(ctx))
                return st;
            const size_t cap = std::max(n, s.cap + s.cap / 2);
            cudaError_t e = regrow(&s.off, cap, st);
            if (e == cudaSuccess) e = regrow(&s.cx, cap, st);
            if (e == cudaSuccess) e = regrow(&s.cv, cap, st);
            if (e == cudaSuccess) e = regrow(&s.pos64, cap, st);
            if (e != cudaSuccess)
            {
                s.cap = 0;
                return ctx_cuda_fail(ctx, e, "precision state allocation");
            }
            s.cap = cap;
            return NBODY_OK;
        }

        // Set up origin + offsets from the float positions (after any upload or FP32 step).
        int ensure_split_state(nbody_cuda* ctx)
        {
            const size_t n = ctx->count;
            if (const int st = reserve_precise(ctx, n))
                return st;
            if (ctx->origin_valid)
                return NBODY_OK;
            PreciseState& s = *ctx->precise;
            int stride = 1;
            const float4* src = body_src(ctx, &stride);
            minmax_kernel<<<kBboxBlocks, 256, 0, ctx->stream>>>(src, stride, static_cast<int>(n), s.part);
            origin_kernel<<<1, 32, 0, ctx->stream>>>(s.part, kBboxBlocks, s.origin);
            to_offsets_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(src, stride, static_cast<int>(n), s.origin,
                                                                         s.off, s.cx, s.cv);
            ctx->launches += 3;
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "precision state set-up");
            ctx->origin_valid = true;
            return NBODY_OK;
        }

        struct Split
        {
            int tb, js, chunk;
        };

        Split plan_split(const size_t nt, const size_t n, const int per_cta, const int tile, const int slots)
        {
            Split p;
            p.tb = static_cast<int>(std::max<size_t>(1, (nt + per_cta - 1) / per_cta));
            const size_t max_js = std::max<size_t>(1, std::min<size_t>(64, n / (static_cast<size_t>(tile) * 4)));
            size_t best = 1;
            double best_cost = 1e300;
            for (size_t js = 1; js <= max_js; ++js)
            {
                const size_t waves = (p.tb * js + slots - 1) / slots;
                const double cost = static_cast<double>(waves) / static_cast<double>(js) * (1.0 + 0.002 * js);
                if (cost < best_cost - 1e-12)
                {
                    best_cost = cost;
                    best = js;
                }
            }
            size_t chunk = (n + best - 1) / best;
            chunk = (chunk + tile - 1) / tile * tile;
            p.chunk = static_cast<int>(chunk);
            p.js = static_cast<int>((n + chunk - 1) / chunk);
            return p;
        }

        int sms_of(const nbody_cuda* ctx)
        {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            return sms > 0 ? sms : 1;
        }

        // Queue the compensated or FP64 sum for targets tlist (or all) into FP64 partials,
        // then their fixed-order sum into acc / out64.
        int precise_sum(nbody_cuda* ctx, const nbody_step_params* p, const int* tlist, const size_t nt,
                        double4* out64, const bool write_acc)
        {
            const size_t n = ctx->count;
            PreciseState& s = *ctx->precise;
            int stride = 1;
            const float4* src = body_src(ctx, &stride);
            const int ni = static_cast<int>(n), nti = static_cast<int>(nt);
            const bool fp64 = p->precision == NBODY_PREC_FP64;
            const int sms = sms_of(ctx);
            constexpr int kT = 4, kB = 256, kB64 = 128;
            const Split sp = fp64 ? plan_split(nt, n, kB64 * 2, kTile64, sms * 4)
                                  : plan_split(nt, n, kB * kT, kTileC, sms * 2);
            // scratch: partials (js * nt double4) + radius^2 (n floats)
            const size_t part_bytes = static_cast<size_t>(sp.js) * nt * sizeof(double4);
            const size_t rad_bytes = (p->law == NBODY_LAW_CUTOFF) ? n * sizeof(float) : 0;
            if (const int st = ensure_scratch(ctx, part_bytes + rad_bytes + 256))
                return st;
            double4* part = static_cast<double4*>(ctx->scratch);
            float* rad2 = reinterpret_cast<float*>(static_cast<char*>(ctx->scratch) + ((part_bytes + 255) / 256) * 256);
            cudaStream_t st = ctx->stream;
            if (p->law == NBODY_LAW_CUTOFF)
            {
                radius2_kernel<<<ceil_div(n, 256), 256, 0, st>>>(src, stride, ctx->vr, ni, rad2);
                ++ctx->launches;
            }
            const dim3 grid(sp.tb, sp.js);
            if (fp64)
            {
                pos64_kernel<<<ceil_div(n, 256), 256, 0, st>>>(src, stride, ctx->origin_valid ? s.off : nullptr, s.cx,
                                                              s.origin, ni, s.pos64);
                if (p->law == NBODY_LAW_SOFTENED)
                    direct_fp64_kernel<kB64, NBODY_LAW_SOFTENED><<<grid, kB64, 0, st>>>(
                        s.pos64, rad2, tlist, nti, ni, sp.chunk, p->G, p->eps2, part, ctx->dev_error);
                else
                    direct_fp64_kernel<kB64, NBODY_LAW_CUTOFF><<<grid, kB64, 0, st>>>(
                        s.pos64, rad2, tlist, nti, ni, sp.chunk, p->G, p->eps2, part, ctx->dev_error);
                ctx->launches += 2;
            }
            else
            {
                if (p->law == NBODY_LAW_SOFTENED)
                    direct_comp_kernel<kT, kB, NBODY_LAW_SOFTENED><<<grid, kB, 0, st>>>(
                        s.off, rad2, tlist, nti, ni, sp.chunk, p->G, p->eps2, part, ctx->dev_error);
                else
                    direct_comp_kernel<kT, kB, NBODY_LAW_CUTOFF><<<grid, kB, 0, st>>>(
                        s.off, rad2, tlist, nti, ni, sp.chunk, p->G, p->eps2, part, ctx->dev_error);
                ++ctx->launches;
            }
            float4* acc = (write_acc && ctx->layout == NBODY_LAYOUT_SOA) ? ctx->acc : nullptr;
            float* body_out = (write_acc && ctx->layout == NBODY_LAYOUT_AOS) ? ctx->bodies : nullptr;
            reduce64_kernel<<<ceil_div(nt, 256), 256, 0, st>>>(part, sp.js, nti, tlist, acc, body_out, out64);
            ++ctx->launches;
            DirectPlan& lp = ctx->last_plan;
            lp = DirectPlan{};
            lp.T = fp64 ? 2 : kT;
            lp.block = fp64 ? kB64 : kB;
            lp.tile = fp64 ? kTile64 : kTileC;
            lp.jsplit = sp.js;
            lp.chunk = sp.chunk;
            lp.grid_x = sp.tb;
            lp.law = p->law;
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "precise direct-sum launch");
            return NBODY_OK;
        }
    }

    int precise_accelerate(nbody_cuda* ctx, const nbody_step_params* p)
    {
        if (p->mode == NBODY_MODE_NLOGN)
        {
            if (p->precision == NBODY_PREC_FP64)
                return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "FP64 precision is provided for direct summation only");
            // FP32 tree forces; the compensation lives in the integrator
            return bh_accelerate(ctx, p);
        }
        if (ctx->count > static_cast<size_t>(INT32_MAX / 64))
            return ctx_fail(ctx, NBODY_ERR_INVALID, "body count too large for the precise forms");
        if (const int st = ensure_split_state(ctx))
            return st;
        ctx->pending_partials = 0;
        return precise_sum(ctx, p, nullptr, ctx->count, nullptr, true);
    }

    int precise_integrate(nbody_cuda* ctx, const nbody_step_params* p)
    {
        if (const int st = ensure_split_state(ctx))
            return st;
        if (ctx->pending_partials > 1)
        {
            // an FP32 accelerate left partials for the fused FP32 integrate: sum them first
            const cudaError_t e = launch_reduce(static_cast<const float4*>(ctx->scratch), ctx->pending_partials,
                                                static_cast<int>(ctx->count), ctx->pending_G,
                                                ctx->layout == NBODY_LAYOUT_SOA ? ctx->acc : nullptr,
                                                ctx->layout == NBODY_LAYOUT_AOS ? ctx->bodies : nullptr, ctx->stream,
                                                &ctx->launches);
            ctx->pending_partials = 0;
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "partial sum launch");
        }
        PreciseState& s = *ctx->precise;
        integrate_comp_kernel<<<ceil_div(ctx->count, 256), 256, 0, ctx->stream>>>(
            s.off, s.cx, s.cv, ctx->pm, ctx->vr, ctx->layout == NBODY_LAYOUT_AOS ? ctx->bodies : nullptr, ctx->acc,
            s.origin, static_cast<int>(ctx->count), p->dt, p->size, p->wrap);
        ++ctx->launches;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "compensated integrate launch");
        return NBODY_OK;
    }

    // Float positions are rewritten by every compensated step, so nothing is pending; an
    // FP32 step invalidates the split state instead (context.cu).
    int sync_precise_positions(nbody_cuda*) { return NBODY_OK; }

    int precise_sampled(nbody_cuda* ctx, const nbody_step_params* p, const int64_t* targets, const size_t nt,
                        double* out)
    {
        if (p->precision != NBODY_PREC_COMPENSATED && p->precision != NBODY_PREC_FP64)
            return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "sampled accelerations need COMPENSATED or FP64 precision");
        if (p->mode != NBODY_MODE_N2)
            return ctx_fail(ctx, NBODY_ERR_UNSUPPORTED, "sampled accelerations are direct-sum only");
        const size_t n = ctx->count;
        if (nt == 0 || n == 0)
            return NBODY_OK;
        for (size_t k = 0; k < nt; ++k)
            if (targets[k] < 0 || static_cast<size_t>(targets[k]) >= n)
                return ctx_fail(ctx, NBODY_ERR_INVALID, "sampled target index out of range");
        if (p->precision == NBODY_PREC_COMPENSATED || ctx->origin_valid)
        {
            if (const int st = ensure_split_state(ctx))
                return st;
        }
        else if (const int st = reserve_precise(ctx, n))
            return st;
        PreciseState& s = *ctx->precise;
        if (nt > s.tlist_cap)
        {
            cudaFreeAsync(s.tlist, ctx->stream);
            cudaFreeAsync(s.out64, ctx->stream);
            s.tlist = nullptr;
            s.out64 = nullptr;
            s.tlist_cap = 0;
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&s.tlist), nt * sizeof(int), ctx->stream);
            if (e == cudaSuccess)
                e = cudaMallocAsync(reinterpret_cast<void**>(&s.out64), nt * sizeof(double4), ctx->stream);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "sample buffers");
            s.tlist_cap = nt;
        }
        int* host_list = new int[nt];
        for (size_t k = 0; k < nt; ++k)
            host_list[k] = static_cast<int>(targets[k]);
        cudaError_t e = cudaMemcpyAsync(s.tlist, host_list, nt * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        delete[] host_list;
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "sample upload");
        if (const int st = precise_sum(ctx, p, s.tlist, nt, s.out64, false))
            return st;
        double4* h = new double4[nt];
        e = cudaMemcpyAsync(h, s.out64, nt * sizeof(double4), cudaMemcpyDeviceToHost, ctx->stream);
        const int st = (e == cudaSuccess) ? check_device_error(ctx) : ctx_cuda_fail(ctx, e, "sample readback");
        if (st == NBODY_OK)
            for (size_t k = 0; k < nt; ++k)
            {
                out[3 * k] = h[k].x;
                out[3 * k + 1] = h[k].y;
                out[3 * k + 2] = h[k].z;
            }
        delete[] h;
        return st;
    }

    int precise_origin(nbody_cuda* ctx, double out[4])
    {
        if (!ctx->precise || !ctx->origin_valid)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "no split-precision state (run a compensated step first)");
        const cudaError_t e = cudaMemcpyAsync(out, ctx->precise->origin, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                                              ctx->stream);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "origin readback");
        return check_device_error(ctx);
    }

    void release_precise(nbody_cuda* ctx)
    {
        if (!ctx->precise)
            return;
        PreciseState& s = *ctx->precise;
        void* ptrs[] = { s.off, s.cx, s.cv, s.pos64, s.origin, s.part, s.tlist, s.out64 };
        for (void* q : ptrs)
            cudaFree(q);
        delete ctx->precise;
        ctx->precise = nullptr;
    }
}
