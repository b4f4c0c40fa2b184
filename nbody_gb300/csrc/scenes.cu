// Device scene generators: util::disk and util::cube (source/util.cpp:14-126), for sm_103a.
//
// The reference draws from a local std::default_random_engine (libstdc++ of GCC 13:
// minstd_rand0, x <- 16807 x mod (2^31 - 1), seed 1) through
// std::uniform_real_distribution<float> and std::normal_distribution<float>. The draws are
// a fixed sequence, so every value is reachable by jump-ahead: the j-th value the engine
// returns is 16807^(j+1) mod (2^31 - 1). The algorithms restated here (the C++ standard's
// [rand.eng.lcong], [rand.util.canonical] as libstdc++ implements it, and the Marsaglia
// polar method libstdc++'s normal_distribution uses) are:
//   canonical(x)  = float(x - 1) / 2^31, clamped below 1 (generate_canonical<float, 24>
//                   with one engine call: the engine's range is 2^31 - 2);
//   uniform(a, b) = canonical * (b - a) + a;
//   normal        = pairs (2u - 1, 2v - 1) until 0 < r2 = x^2 + y^2 <= 1, then
//                   m = sqrt(-2 log(r2) / r2), returning y*m and saving x*m for the next
//                   call; scaled by stddev and shifted by mean.
//
// util::cube draws x, y, z for body i at stream positions 3i, 3i+1, 3i+2: one thread per
// body.
//
// util::disk draws, for star i (i = 1 .. num-1), one uniform then one normal. Odd stars
// consume a fresh polar pair (with rejections), even stars the saved half. Number the
// pairs the stream could start at after the first draw: slot j holds draws (2j+1, 2j+2).
// The first odd star's pair search starts at slot 0. After slot a is accepted, slot a+1
// holds the next even star's uniform and the next odd star's uniform, and the search
// resumes at slot a+2. Hence slot j is used as a pair exactly when
//     chosen_j = accepted_j && !chosen_{j-1},        chosen_{-1} = false,
// a one-bit recurrence that any rejected slot resets. The k-th chosen slot a_k (k from 0)
// serves stars 2k+1 (uniform at draw 2 a_{k-1} + 4, with a_{-1} = -2; the normal y*m) and
// 2k+2 (uniform at draw 2 a_k + 3; the normal x*m). The device evaluates the accept test
// for all slots (64 per thread, a bit word each), resolves the recurrence per word (a word
// without a rejection passes its carry through unchanged, being 64 slots long), counts and
// scans the chosen slots, lists them, and then builds every star independently.
//
// The circular speeds (util.cpp:81-95): the reference walks its own octree (theta 0.5)
// from every body and folds the applied nodes into a running centre of mass and mass.
// The nodes such a walk applies partition the bodies, so the result is the centre of
// mass and total mass of all the generated bodies for every body, up to the rounding of
// the running mean. Here it is one FP64 reduction, and the speed sqrt(G M / |com - x|).
//
// Every float operation is written as the rounded intrinsic of the reference's operation,
// in the reference's order, so nothing is contracted. sin, cos and log are evaluated in
// double and rounded to float (the reference calls sinf, cosf, logf).
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "context.cuh"
#include "scan.cuh"

namespace nbg
{
    namespace
    {
        constexpr uint32_t kModulus = 2147483647u;     // 2^31 - 1
        constexpr uint32_t kMultiplier = 16807u;
        constexpr float kPi = 3.14159265358979323846f;  // nbody::pi (constants.h:6)
        constexpr float kStarDensity = 1e2f;            // nbody::star_density (constants.h:10)
        constexpr int kBlock = 256;
        constexpr int kReduceBlocks = 304;              // 2 per SM; fixed, so the sums are deterministic

        struct Powers
        {
            uint32_t p[31];     // 16807^(2^b) mod (2^31 - 1)
        };

        __host__ __device__ __forceinline__ uint32_t mulmod(const uint32_t a, const uint32_t b)
        {
            const uint64_t p = static_cast<uint64_t>(a) * b;
            uint64_t r = (p & kModulus) + (p >> 31);
            r = (r & kModulus) + (r >> 31);
            return static_cast<uint32_t>(r >= kModulus ? r - kModulus : r);
        }

        Powers make_powers()
        {
            Powers w{};
            w.p[0] = kMultiplier;
            for (int b = 1; b < 31; ++b)
                w.p[b] = mulmod(w.p[b - 1], w.p[b - 1]);
            return w;
        }

        // The j-th value (from 0) the seed-1 engine returns.
        __device__ __forceinline__ uint32_t draw_at(const uint64_t j, const Powers& w)
        {
            uint64_t e = (j + 1) % (kModulus - 1);
            uint32_t r = 1;
            for (int b = 0; e; ++b, e >>= 1)
                if (e & 1)
                    r = mulmod(r, w.p[b]);
            return r;
        }

        __device__ __forceinline__ uint32_t next(const uint32_t x) { return mulmod(x, kMultiplier); }

        __device__ __forceinline__ float canonical(const uint32_t x)
        {
            const float f = __fmul_rn(__uint2float_rn(x - 1u), 0x1p-31f);
            return f >= 1.f ? 0x1.fffffep-1f : f;
        }

        // One polar attempt from two engine values; true when the pair is accepted.
        __device__ __forceinline__ bool polar(const uint32_t xa, const uint32_t xb, float& x, float& y, float& r2)
        {
            x = __fsub_rn(__fmul_rn(2.f, canonical(xa)), 1.f);
            y = __fsub_rn(__fmul_rn(2.f, canonical(xb)), 1.f);
            r2 = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
            return !(r2 > 1.f || r2 == 0.f);
        }

        struct Records
        {
            float4* pm;         // split layout
            float4* vr;
            float4* acc;
            float4* aos;        // interleaved layout (3 float4 per body)
        };

        __device__ __forceinline__ void put_body(const Records& r, const size_t i, const float px, const float py,
                                                 const float pz, const float radius, const float vx, const float vy,
                                                 const float vz, const float mass)
        {
            if (r.aos)
            {
                r.aos[3 * i] = make_float4(px, py, pz, radius);
                r.aos[3 * i + 1] = make_float4(vx, vy, vz, mass);
                r.aos[3 * i + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            else
            {
                r.pm[i] = make_float4(px, py, pz, mass);
                r.vr[i] = make_float4(vx, vy, vz, radius);
                r.acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }

        // --- util::cube ---------------------------------------------------------------------

        struct CubeParams
        {
            float lo, span;     // uniform(lo, hi): span = hi - lo
            float vx, vy, vz, radius, mass;
        };

        __global__ void __launch_bounds__(kBlock) cube_kernel(const Powers w, const CubeParams c, const size_t begin,
                                                              const size_t num, const Records r)
        {
            const size_t i = static_cast<size_t>(blockIdx.x) * kBlock + threadIdx.x;
            if (i >= num)
                return;
            uint32_t x = draw_at(3 * static_cast<uint64_t>(i), w);
            const float ux = canonical(x);
            x = next(x);
            const float uy = canonical(x);
            x = next(x);
            const float uz = canonical(x);
            const float px = __fadd_rn(__fmul_rn(ux, c.span), c.lo);
            const float py = __fadd_rn(__fmul_rn(uy, c.span), c.lo);
            const float pz = __fadd_rn(__fmul_rn(uz, c.span), c.lo);
            put_body(r, begin + i, px, py, pz, c.radius, c.vx, c.vy, c.vz, c.mass);
        }

        // --- util::disk ---------------------------------------------------------------------

        struct DiskParams
        {
            float cx, cy, cz;           // DiskArgs::center
            float ax, ay, az;           // DiskArgs::axis
            float vx, vy, vz;           // DiskArgs::vel
            float inner, outer;         // radii after the clamp to the central body's radius
            float thick_crad;           // thickness * center_radius
            float star_radius, star_mass;
            float center_radius, central_mass;
            uint64_t num;
        };

        // Accept bits for slots [64 w, 64 w + 64).
        __global__ void __launch_bounds__(kBlock) disk_accept_kernel(const Powers w, const int words,
                                                                     uint64_t* __restrict__ accept)
        {
            const int k = blockIdx.x * kBlock + threadIdx.x;
            if (k >= words)
                return;
            uint32_t x = draw_at(128 * static_cast<uint64_t>(k) + 1, w);
            uint64_t bits = 0;
            for (int b = 0; b < 64; ++b)
            {
                const uint32_t xa = x;
                x = next(x);
                const uint32_t xb = x;
                x = next(x);
                float fx, fy, r2;
                if (polar(xa, xb, fx, fy, r2))
                    bits |= 1ull << b;
            }
            accept[k] = bits;
        }

        __device__ __forceinline__ uint64_t choose(const uint64_t acc, bool prev, bool* last)
        {
            uint64_t ch = 0;
            for (int b = 0; b < 64; ++b)
            {
                const bool c = ((acc >> b) & 1) && !prev;
                ch |= static_cast<uint64_t>(c) << b;
                prev = c;
            }
            *last = prev;
            return ch;
        }

        __global__ void __launch_bounds__(kBlock) disk_choose_kernel(const uint64_t* __restrict__ accept, const int words,
                                                                     uint64_t* __restrict__ chosen,
                                                                     uint32_t* __restrict__ counts)
        {
            const int k = blockIdx.x * kBlock + threadIdx.x;
            if (k >= words)
                return;
            // The carry into word k: the last chosen bit of the nearest earlier word with a
            // rejection (its carry out does not depend on its carry in); the all-accepted
            // words in between pass it through.
            int j = k - 1;
            while (j >= 0 && accept[j] == ~0ull)
                --j;
            bool carry = false;
            if (j >= 0)
                choose(accept[j], false, &carry);
            bool last;
            const uint64_t ch = choose(accept[k], carry, &last);
            chosen[k] = ch;
            counts[k] = static_cast<uint32_t>(__popcll(ch));
        }

        __global__ void __launch_bounds__(kBlock) disk_list_kernel(const uint64_t* __restrict__ chosen,
                                                                   const uint32_t* __restrict__ offsets, const int words,
                                                                   const uint32_t need, uint32_t* __restrict__ list)
        {
            const int k = blockIdx.x * kBlock + threadIdx.x;
            if (k >= words)
                return;
            uint64_t ch = chosen[k];
            uint32_t at = offsets[k];
            while (ch && at < need)
            {
                const int b = __ffsll(static_cast<long long>(ch)) - 1;
                ch &= ch - 1;
                list[at++] = 64u * static_cast<uint32_t>(k) + static_cast<uint32_t>(b);
            }
        }

        __device__ __forceinline__ float sin_f(const float a) { return __double2float_rn(sin(static_cast<double>(a))); }
        __device__ __forceinline__ float cos_f(const float a) { return __double2float_rn(cos(static_cast<double>(a))); }
        __device__ __forceinline__ float log_f(const float a) { return __double2float_rn(log(static_cast<double>(a))); }

        // Star i of the disk loop (util.cpp:54-79) from its uniform u and its normal value g.
        __device__ void disk_star(const DiskParams& d, const Records& r, const size_t begin, const uint64_t i,
                                  const float u, const float g)
        {
            // perpendicular frame of the axis (util.cpp:44-50)
            const float c0x = copysignf(d.az, d.ax);
            const float c0y = copysignf(d.az, d.ay);
            const float c0z = __fsub_rn(-copysignf(d.ax, d.az), copysignf(d.ay, d.az));
            const float c1x = __fsub_rn(__fmul_rn(d.ay, c0z), __fmul_rn(d.az, c0y));
            const float c1y = __fsub_rn(__fmul_rn(d.az, c0x), __fmul_rn(d.ax, c0z));
            const float c1z = __fsub_rn(__fmul_rn(d.ax, c0y), __fmul_rn(d.ay, c0x));

            const float t = __fdiv_rn(__ull2float_rn(i), __ull2float_rn(d.num - 1));
            const float angle = __fmul_rn(__fmul_rn(t, 2.f), kPi);
            // inner + sqrt(u) * (outer - inner): the unqualified sqrt is ::sqrt(double)
            const float dist = __double2float_rn(__dadd_rn(
                static_cast<double>(d.inner),
                __dmul_rn(__dsqrt_rn(static_cast<double>(u)), static_cast<double>(__fsub_rn(d.outer, d.inner)))));
            const float disp = __fmul_rn(__fmul_rn(__fdiv_rn(__fsub_rn(d.outer, dist), d.outer), d.thick_crad), g);

            const float s = sin_f(angle), c = cos_f(angle);
            float vx = __fadd_rn(__fmul_rn(s, c0x), __fmul_rn(c, c1x));
            float vy = __fadd_rn(__fmul_rn(s, c0y), __fmul_rn(c, c1y));
            float vz = __fadd_rn(__fmul_rn(s, c0z), __fmul_rn(c, c1z));
            float n = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz)));
            const float s0x = __fdiv_rn(vx, n), s0y = __fdiv_rn(vy, n), s0z = __fdiv_rn(vz, n);
            vx = __fsub_rn(__fmul_rn(d.ay, s0z), __fmul_rn(d.az, s0y));
            vy = __fsub_rn(__fmul_rn(d.az, s0x), __fmul_rn(d.ax, s0z));
            vz = __fsub_rn(__fmul_rn(d.ax, s0y), __fmul_rn(d.ay, s0x));
            n = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz)));
            const float s1x = __fdiv_rn(vx, n), s1y = __fdiv_rn(vy, n), s1z = __fdiv_rn(vz, n);

            const float px = __fadd_rn(__fadd_rn(d.cx, __fmul_rn(s0x, dist)), __fmul_rn(d.ax, disp));
            const float py = __fadd_rn(__fadd_rn(d.cy, __fmul_rn(s0y, dist)), __fmul_rn(d.ay, disp));
            const float pz = __fadd_rn(__fadd_rn(d.cz, __fmul_rn(s0z, dist)), __fmul_rn(d.az, disp));
            put_body(r, begin + i, px, py, pz, d.star_radius, s1x, s1y, s1z, d.star_mass);
        }

        // Chosen slot k serves stars 2k+1 and 2k+2; thread 0 also writes the central body.
        __global__ void __launch_bounds__(kBlock) disk_star_kernel(const Powers w, const DiskParams d,
                                                                   const uint32_t* __restrict__ list, const uint32_t pairs,
                                                                   const size_t begin, const Records r)
        {
            const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
            if (k == 0)
                put_body(r, begin, d.cx, d.cy, d.cz, d.center_radius, 0.f, 0.f, 0.f, d.central_mass);
            if (k >= pairs)
                return;
            const int64_t a = list[k];
            const int64_t prev = k ? static_cast<int64_t>(list[k - 1]) : -2;
            const uint32_t xa = draw_at(static_cast<uint64_t>(2 * a + 1), w);
            float fx, fy, r2;
            polar(xa, next(xa), fx, fy, r2);
            const float mult = __fsqrt_rn(__fdiv_rn(__fmul_rn(-2.f, log_f(r2)), r2));
            // normal(0, .5): value * stddev + mean
            const float g_odd = __fadd_rn(__fmul_rn(__fmul_rn(fy, mult), 0.5f), 0.f);
            const float g_even = __fadd_rn(__fmul_rn(__fmul_rn(fx, mult), 0.5f), 0.f);
            // uniform(0, 1): canonical * (1 - 0) + 0
            const uint64_t i_odd = 2 * static_cast<uint64_t>(k) + 1;
            const float u_odd = __fadd_rn(__fmul_rn(canonical(draw_at(static_cast<uint64_t>(2 * prev + 4), w)), 1.f), 0.f);
            disk_star(d, r, begin, i_odd, u_odd, g_odd);
            if (i_odd + 1 <= d.num - 1)
            {
                const float u_even = __fadd_rn(__fmul_rn(canonical(draw_at(static_cast<uint64_t>(2 * a + 3), w)), 1.f), 0.f);
                disk_star(d, r, begin, i_odd + 1, u_even, g_even);
            }
        }

        // FP64 (mass, mass * position) over the generated bodies, fixed grid and order.
        __global__ void __launch_bounds__(kBlock) mass_moment_kernel(const Records r, const size_t begin,
                                                                     const size_t num, double4* __restrict__ partial)
        {
            double m = 0, mx = 0, my = 0, mz = 0;
            for (size_t i = static_cast<size_t>(blockIdx.x) * kBlock + threadIdx.x; i < num;
                 i += static_cast<size_t>(gridDim.x) * kBlock)
            {
                float4 p;
                if (r.aos)
                {
                    const float4 a = r.aos[3 * (begin + i)], b = r.aos[3 * (begin + i) + 1];
                    p = make_float4(a.x, a.y, a.z, b.w);
                }
                else
                    p = r.pm[begin + i];
                const double w = p.w;
                m += w;
                mx += w * p.x;
                my += w * p.y;
                mz += w * p.z;
            }
            __shared__ double4 sh[kBlock];
            sh[threadIdx.x] = make_double4(m, mx, my, mz);
            __syncthreads();
            for (int s = kBlock / 2; s > 0; s >>= 1)
            {
                if (threadIdx.x < s)
                {
                    double4& a = sh[threadIdx.x];
                    const double4 b = sh[threadIdx.x + s];
                    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
                partial[blockIdx.x] = sh[0];
        }

        __global__ void __launch_bounds__(kBlock) mass_moment_final_kernel(const double4* __restrict__ partial, const int n,
                                                                           double4* __restrict__ out)
        {
            __shared__ double4 sh[kBlock];
            double4 acc = make_double4(0, 0, 0, 0);
            for (int i = threadIdx.x; i < n; i += kBlock)
            {
                const double4 b = partial[i];
                acc.x += b.x; acc.y += b.y; acc.z += b.z; acc.w += b.w;
            }
            sh[threadIdx.x] = acc;
            __syncthreads();
            for (int s = kBlock / 2; s > 0; s >>= 1)
            {
                if (threadIdx.x < s)
                {
                    double4& a = sh[threadIdx.x];
                    const double4 b = sh[threadIdx.x + s];
                    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
                *out = sh[0];
        }

        // vel = args.vel + vel * sqrt(G M / |com - x|), G = 1 (util.cpp:84-96).
        __global__ void __launch_bounds__(kBlock) disk_speed_kernel(const DiskParams d, const double4* __restrict__ moment,
                                                                    const size_t begin, const size_t num, const Records r)
        {
            const size_t i = static_cast<size_t>(blockIdx.x) * kBlock + threadIdx.x;
            if (i >= num)
                return;
            const double4 s = *moment;
            const float mass = __double2float_rn(s.x);
            const float comx = __double2float_rn(s.y / s.x);
            const float comy = __double2float_rn(s.z / s.x);
            const float comz = __double2float_rn(s.w / s.x);
            const size_t b = begin + i;
            float4 p, v;
            if (r.aos)
            {
                p = r.aos[3 * b];
                v = r.aos[3 * b + 1];
            }
            else
            {
                p = r.pm[b];
                v = r.vr[b];
            }
            const float dx = __fsub_rn(comx, p.x), dy = __fsub_rn(comy, p.y), dz = __fsub_rn(comz, p.z);
            const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
            const float speed = __fsqrt_rn(__fdiv_rn(__fmul_rn(1.f, mass), dist));
            v.x = __fadd_rn(d.vx, __fmul_rn(v.x, speed));
            v.y = __fadd_rn(d.vy, __fmul_rn(v.y, speed));
            v.z = __fadd_rn(d.vz, __fmul_rn(v.z, speed));
            if (r.aos)
                r.aos[3 * b + 1] = v;
            else
                r.vr[b] = v;
        }

        // util::compute_radius (util.cpp:9-12).
        float compute_radius(const float mass, const float density)
        {
            return std::pow((3.f * kPi * mass) / (4.f * density), 1.f / 3.f);
        }

        unsigned blocks_for(const size_t n) { return static_cast<unsigned>((n + kBlock - 1) / kBlock); }

        // Make room for bodies [begin, begin + num) and account for the change of the body set.
        int prepare_range(nbody_cuda* ctx, const size_t begin, const size_t num, Records* r)
        {
            if (begin > ctx->count)
                return ctx_fail(ctx, NBODY_ERR_INVALID, "a generated range must start at or before the body count");
            const size_t end = begin + num;
            if (const int st = nbody_cuda_reserve(ctx, end))
                return st;
            if (end > ctx->count)
            {
                ctx->count = end;
                ++ctx->generation;      // the body count is an argument of captured launches
            }
            ctx->origin_valid = false;
            ctx->pending_partials = 0;
            ++ctx->body_version;
            if (ctx->layout == NBODY_LAYOUT_AOS)
                *r = Records{ nullptr, nullptr, nullptr, reinterpret_cast<float4*>(ctx->bodies) };
            else
                *r = Records{ ctx->pm, ctx->vr, ctx->acc, nullptr };
            return NBODY_OK;
        }

        size_t align_up(const size_t v, const size_t a) { return (v + a - 1) / a * a; }
    }

    int scene_cube(nbody_cuda* ctx, const nbody_cube_args* a, const size_t begin, const size_t num)
    {
        if (!num)
            return NBODY_OK;
        Records r;
        if (const int st = prepare_range(ctx, begin, num, &r))
            return st;
        CubeParams c{};
        c.lo = static_cast<float>(-.5 * static_cast<double>(a->size));
        const float hi = static_cast<float>(.5 * static_cast<double>(a->size));
        c.span = hi - c.lo;
        c.vx = a->vel[0];
        c.vy = a->vel[1];
        c.vz = a->vel[2];
        c.radius = compute_radius(a->star_mass, kStarDensity);
        c.mass = a->star_mass;
        cube_kernel<<<blocks_for(num), kBlock, 0, ctx->stream>>>(make_powers(), c, begin, num, r);
        ++ctx->launches;
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, e, "cube launch");
    }

    int scene_disk(nbody_cuda* ctx, const nbody_disk_args* a, const size_t begin, const size_t num)
    {
        if (!num)
            return NBODY_OK;
        if (num - 1 > (size_t(1) << 30))
            return ctx_fail(ctx, NBODY_ERR_INVALID, "disk larger than this generator's stream bound (2^30 stars)");
        Records r;
        if (const int st = prepare_range(ctx, begin, num, &r))
            return st;
        DiskParams d{};
        d.cx = a->center[0]; d.cy = a->center[1]; d.cz = a->center[2];
        d.ax = a->axis[0]; d.ay = a->axis[1]; d.az = a->axis[2];
        d.vx = a->vel[0]; d.vy = a->vel[1]; d.vz = a->vel[2];
        d.center_radius = compute_radius(a->central_mass, kStarDensity);
        d.central_mass = a->central_mass;
        d.outer = std::max(a->outer_radius, d.center_radius);
        d.inner = std::max(a->inner_radius, d.center_radius);
        d.thick_crad = a->thickness * d.center_radius;
        d.star_radius = compute_radius(a->star_mass, kStarDensity);
        d.star_mass = a->star_mass;
        d.num = num;
        const Powers w = make_powers();
        const uint32_t pairs = static_cast<uint32_t>(num / 2);  // ceil((num - 1) / 2) pairs for num - 1 stars

        uint32_t* list = nullptr;
        double4* moment = nullptr;
        double4* partial = nullptr;
        if (pairs)
        {
            // About 2.27 slots per chosen slot (one accept in pi/4, plus the skipped slot);
            // 1.2 slots per star leaves a margin of several thousand standard deviations.
            size_t slots = align_up(static_cast<size_t>(1.2 * static_cast<double>(num - 1)) + 4096, 64);
            for (int attempt = 0;; ++attempt)
            {
                const size_t words = slots / 64;
                const size_t scan_elems = scan_temp_elems(words);
                const size_t bytes = align_up(words * 8, 256) * 2 + align_up(words * 4, 256) * 2
                                     + align_up(scan_elems * 4, 256) + align_up(static_cast<size_t>(pairs) * 4, 256)
                                     + align_up(sizeof(double4) * (kReduceBlocks + 1), 256);
                if (const int st = ensure_scratch(ctx, bytes))
                    return st;
                unsigned char* s = static_cast<unsigned char*>(ctx->scratch);
                uint64_t* accept = reinterpret_cast<uint64_t*>(s);
                s += align_up(words * 8, 256);
                uint64_t* chosen = reinterpret_cast<uint64_t*>(s);
                s += align_up(words * 8, 256);
                uint32_t* counts = reinterpret_cast<uint32_t*>(s);
                s += align_up(words * 4, 256);
                uint32_t* offsets = reinterpret_cast<uint32_t*>(s);
                s += align_up(words * 4, 256);
                uint32_t* scan_tmp = reinterpret_cast<uint32_t*>(s);
                s += align_up(scan_elems * 4, 256);
                list = reinterpret_cast<uint32_t*>(s);
                s += align_up(static_cast<size_t>(pairs) * 4, 256);
                moment = reinterpret_cast<double4*>(s);
                partial = moment + 1;

                const int nw = static_cast<int>(words);
                disk_accept_kernel<<<blocks_for(words), kBlock, 0, ctx->stream>>>(w, nw, accept);
                disk_choose_kernel<<<blocks_for(words), kBlock, 0, ctx->stream>>>(accept, nw, chosen, counts);
                ctx->launches += 2;
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "disk slot launch");
                e = exclusive_scan<uint32_t>(counts, offsets, words, scan_tmp, ctx->stream, &ctx->launches);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "disk slot scan");
                uint32_t tail[2] = { 0, 0 };
                e = cudaMemcpyAsync(&tail[0], offsets + words - 1, 4, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(&tail[1], counts + words - 1, 4, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(ctx->stream);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "disk slot count");
                if (static_cast<uint64_t>(tail[0]) + tail[1] >= pairs)
                {
                    disk_list_kernel<<<blocks_for(words), kBlock, 0, ctx->stream>>>(chosen, offsets, nw, pairs, list);
                    ++ctx->launches;
                    break;
                }
                if (attempt >= 4)
                    return ctx_fail(ctx, NBODY_ERR_CUDA, "disk generator: too few accepted pairs in the slot window");
                slots = align_up(slots + slots / 2, 64);
            }
        }
        else
        {
            if (const int st = ensure_scratch(ctx, sizeof(double4) * (kReduceBlocks + 1)))
                return st;
            moment = static_cast<double4*>(ctx->scratch);
            partial = moment + 1;
        }
        disk_star_kernel<<<std::max(1u, blocks_for(pairs)), kBlock, 0, ctx->stream>>>(w, d, list, pairs, begin, r);
        mass_moment_kernel<<<kReduceBlocks, kBlock, 0, ctx->stream>>>(r, begin, num, partial);
        mass_moment_final_kernel<<<1, kBlock, 0, ctx->stream>>>(partial, kReduceBlocks, moment);
        disk_speed_kernel<<<blocks_for(num), kBlock, 0, ctx->stream>>>(d, moment, begin, num, r);
        ctx->launches += 4;
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, e, "disk launch");
    }
}

extern "C" {

int nbody_cuda_scene_disk(nbody_cuda* ctx, const nbody_disk_args* args, const size_t begin, const size_t num)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (!args)
        return nbg::ctx_fail(ctx, NBODY_ERR_INVALID, "null disk arguments");
    return nbg::scene_disk(ctx, args, begin, num);
}

int nbody_cuda_scene_cube(nbody_cuda* ctx, const nbody_cube_args* args, const size_t begin, const size_t num)
{
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (!args)
        return nbg::ctx_fail(ctx, NBODY_ERR_INVALID, "null cube arguments");
    return nbg::scene_cube(ctx, args, begin, num);
}

}
