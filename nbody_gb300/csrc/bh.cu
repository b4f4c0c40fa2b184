// Barnes-Hut on the device: the reference's octree (source/bhtree.cpp:14-138) rebuilt from
// sorted 63-bit Morton codes, traversed with the reference's opening criterion.
//
// Pipeline per accelerate (all on the context's stream, no host round trip):
//   1. root box: the reference's fixed box centred at the origin with edge State::size
//      (source/detail/tree.h:20), or the smallest power-of-two cube around the bodies'
//      bounding box (tree_box = 1; an exact FP32 min/max); the same pass finds the
//      largest |m| and |x|, which fix the fixed-point scale of step 4;
//   2. morton_kernel: 21 bits per axis, q = floor((x - lo) * 2^21 / edge), clamped and
//      interleaved x -> bit 0: in integers for power-of-two cells on a cell-aligned corner
//      (always for the fitted box), else with both double operations rounded toward
//      -inf. Either way every body lands in exactly the octant the reference's float
//      centre comparisons choose (bounds.h:31-38), whose octant bit is set when the
//      coordinate is below the centre: reference octant = digit ^ 7;
//   3. radix_sort_pairs over (code, index): stable, so ties keep index order;
//   4. gather_sum_kernel: bodies into Morton order, and exact fixed-point (int64) prefix
//      sums of m and m*x within tiles of sorted bodies, plus a scan of the tile totals:
//      differences of their sums give each cell's mass and COM;
//   5. adjacent_prefix_kernel, radix_near_kernel, radix_far_kernel: binary radix tree over
//      the sorted codes (Karras 2012), duplicates separated by index; each internal node's
//      common-prefix length fixes its octree level floor(prefix / 3) (capped at 21, the
//      last Morton level), and the node is flagged as an octree node here;
//   6. octree nodes = binary nodes whose level exceeds their parent's (plus the root).
//      A reference cell whose bodies all sit in one octant (a chain of single-child
//      cells) has the same centre of mass and mass at every level of the chain, and the
//      smallest cell of the chain is the easiest to accept, so the chain behaves exactly
//      as its deepest cell: that is the node kept. Each node lists its <= 8 children
//      (cells or single bodies); cells at the Morton limit (identical codes) are buckets
//      whose bodies are applied one by one when opened;
//   7. traverse_pairs_kernel (the default; traverse_kernel is its one-target-per-lane
//      form): a warp walks the tree for 128 Morton-consecutive targets, four per lane as
//      two packed pairs, with one shared stack of (node, lane mask per target slot)
//      entries. Every target evaluates the reference test itself -- accept when
//      |com - x|^2 > size^2 * theta^2 (bhtree.cpp:117-125), leaves always applied,
//      massless nodes skipped -- and a node is opened only for the targets that rejected
//      it, so each target sums exactly the nodes the reference's traversal would, in a
//      different order (the same order in every walk width, so the sums agree bit for
//      bit).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "bh.cuh"
#include "common.cuh"
#include "context.cuh"
#include "scan.cuh"
#include "sort.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kMortonBits = 21;
        constexpr int kMaxLevel = 21;
        constexpr int kTravWarps = 8;
        // warps per CTA of the walk with Q packed pairs per lane: its stack entries carry 2Q
        // lane masks, and the stacks of one CTA stay within 48 KB of static shared memory
        __host__ __device__ constexpr int pair_warps(const int q) { return q > 2 ? 4 : kTravWarps; }
        constexpr int kStack = 192;
        // group walk: warps per CTA, list entries and stacked parent cells per warp (the
        // stack grows by at most 28 parents per tree level, 22 levels: 616 < 768)
        constexpr int kListWarps = 4;
        // interaction-list entries per warp: the long list (8 KB; five CTAs per SM) drains half
        // as often, the short one (4 KB; six CTAs) keeps more warps resident when the groups
        // are too few to fill them
        constexpr int kListLong = 512;
        constexpr int kListShort = 256;
        constexpr int kGroupStack = 768;
        constexpr int kRuns = 4;            // runs (own acceptance boxes) per group
        constexpr int kBboxBlocks = 1024;
        constexpr int kBboxVals = 8;    // min x y z, max x y z, max |m|, max |x|
        constexpr int kStatsWords = 8;
        // The Morton sort: radix passes over the top 45 code bits (octree levels 1-15), then
        // each run of codes that agree on them (a level-15 cell) is put in order by the low 18
        // bits. A run longer than kMaxRun (not met by a workload of 16.8M disk and halo
        // bodies, whose longest is 10) instead makes the build finish with a full sort.
        constexpr int kRunShift = 18;
        constexpr int kMaxRun = 32;
        constexpr int kMomThreads = 512;
        constexpr int kMomItems = 4;
        constexpr int kMomTile = kMomThreads * kMomItems;   // bodies per cell-sum tile
    }

    struct BhState
    {
        size_t cap = 0;                 // bodies the buffers hold
        uint64_t* keys[2] = { nullptr, nullptr };
        uint32_t* vals[2] = { nullptr, nullptr };
        float4* spm = nullptr;          // pos_mass in Morton order
        float* srad = nullptr;          // target radius in Morton order
        int2* child = nullptr;          // binary children: >= 0 internal, < 0 ~leaf
        int2* range = nullptr;          // [first, last] of each internal node
        int* prefix = nullptr;          // common-prefix bits of each internal node
        uint32_t* octflag = nullptr;
        uint32_t* octidx = nullptr;
        Int64x4* psum = nullptr;        // N + 1 fixed-point sums of {m x, m y, m z, m} over the
                                        // sorted bodies before x within x's cell-sum tile
        OctNode* nodes = nullptr;
        void* temp = nullptr;           // sort and scan temporaries
        size_t temp_bytes = 0;
        BoxParams* box = nullptr;
        float* bbox_part = nullptr;
        unsigned long long* stats = nullptr;   // [0] interactions, [1] node visits, [2] octree nodes,
                                               // [3] the traversal's tile counter, [4] the Morton
                                               // sort's full-sort flag (as unsigned)
        const uint32_t* order = nullptr;       // sorted indices of the last build (keys/vals ping-pong)
        const uint64_t* codes = nullptr;
        bool built = false;                    // a tree for built_n bodies is on the device
        cudaEvent_t ev[3] = { nullptr, nullptr, nullptr };  // build start, traversal start, end
        bool timed = false;                    // ev[] bracket the last accelerate
        size_t built_n = 0;
        uint64_t build_id = 0;
    };

    // ------------------------------------------------------------------------------------
    // 1. root box
    // ------------------------------------------------------------------------------------
    // Per block: the box's min and max per axis, and the largest finite |m| and |x| (over
    // all axes), which fix the fixed-point scale of the cell sums. Min and max are exact,
    // so the float fold equals a double one; the partials are widened at the end.
    __global__ void __launch_bounds__(256) bbox_partial_kernel(const float4* __restrict__ src, const int stride,
                                                               const int n, float* __restrict__ part)
    {
        float v[kBboxVals] = { INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.f, 0.f };
        auto fold = [&](const float4 p, const float m) {
            const float x[3] = { p.x, p.y, p.z };
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                v[a] = fminf(v[a], x[a]);
                v[3 + a] = fmaxf(v[3 + a], x[a]);
                if (isfinite(x[a]))
                    v[7] = fmaxf(v[7], fabsf(x[a]));
            }
            if (isfinite(m))
                v[6] = fmaxf(v[6], fabsf(m));
        };
        const int step = gridDim.x * blockDim.x;
        int i = blockIdx.x * blockDim.x + threadIdx.x;
        // four bodies in flight per thread
        for (; static_cast<long long>(i) + 3 * step < n; i += 4 * step)
        {
            float4 p[4];
            float m[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const size_t k = static_cast<size_t>(i + u * step);
                p[u] = src[k * stride];
                m[u] = stride == 3 ? src[k * 3 + 1].w : p[u].w;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                fold(p[u], m[u]);
        }
        for (; i < n; i += step)
        {
            const float4 p = src[static_cast<size_t>(i) * stride];
            fold(p, stride == 3 ? src[static_cast<size_t>(i) * 3 + 1].w : p.w);
        }
        __shared__ float red[kBboxVals][256];
#pragma unroll
        for (int a = 0; a < kBboxVals; ++a)
            red[a][threadIdx.x] = v[a];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1)
        {
            if (threadIdx.x < s)
            {
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    red[a][threadIdx.x] = fminf(red[a][threadIdx.x], red[a][threadIdx.x + s]);
#pragma unroll
                for (int a = 3; a < kBboxVals; ++a)
                    red[a][threadIdx.x] = fmaxf(red[a][threadIdx.x], red[a][threadIdx.x + s]);
            }
            __syncthreads();
        }
        if (threadIdx.x < kBboxVals)
            part[blockIdx.x * kBboxVals + threadIdx.x] = red[threadIdx.x][0];
    }

    // The exponent e with 0 <= v < 2^e for a finite float v >= 0 (v = M 2^(E - 150) with
    // M < 2^24, so v < 2^(E - 126); subnormals and zero lie below 2^-126).
    __device__ __forceinline__ int bound_exp(const float v)
    {
        const uint32_t E = (__float_as_uint(v) >> 23) & 0xffu;
        return (E ? static_cast<int>(E) : 1) - 126;
    }

    __global__ void __launch_bounds__(256) box_final_kernel(const float* __restrict__ part, const int nparts,
                                                            const int n, const int mode, const float size,
                                                            BoxParams* __restrict__ box)
    {
        // one block folds the per-block partials (a strided pass, then a tree), in float:
        // min and max are exact
        __shared__ float red[kBboxVals][256];
        float v[kBboxVals] = { INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.f, 0.f };
        for (int k = threadIdx.x; k < nparts; k += blockDim.x)
        {
            for (int a = 0; a < 3; ++a)
                v[a] = fminf(v[a], part[k * kBboxVals + a]);
            for (int a = 3; a < kBboxVals; ++a)
                v[a] = fmaxf(v[a], part[k * kBboxVals + a]);
        }
        for (int a = 0; a < kBboxVals; ++a)
            red[a][threadIdx.x] = v[a];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1)
        {
            if (threadIdx.x < s)
            {
                for (int a = 0; a < 3; ++a)
                    red[a][threadIdx.x] = fminf(red[a][threadIdx.x], red[a][threadIdx.x + s]);
                for (int a = 3; a < kBboxVals; ++a)
                    red[a][threadIdx.x] = fmaxf(red[a][threadIdx.x], red[a][threadIdx.x + s]);
            }
            __syncthreads();
        }
        if (threadIdx.x != 0)
            return;
        BoxParams b;
        // |m| < 2^em and |x| < 2^ex for every finite value, and n <= 2^cn, so
        // n |m| 2^mass_shift and n |m x| 2^mom_shift stay below 2^61
        const int cn = n > 1 ? 32 - __clz(n - 1) : 0;
        const int m_exp = bound_exp(red[6][0]), x_exp = bound_exp(red[7][0]);
        b.mass_shift = 61 - cn - m_exp;
        b.mom_shift = 61 - cn - m_exp - x_exp;
        if (mode == 0)
        {
            // tree.h:20 / bhtree.h:29: centred at the origin, edge State::size
            const double e = static_cast<double>(size);
            for (int a = 0; a < 3; ++a)
            {
                b.lo[a] = -0.5 * e;
                b.center[a] = 0.0;
            }
            b.edge = e;
        }
        else
        {
            const double lo[3] = { red[0][0], red[1][0], red[2][0] };
            const double hi[3] = { red[3][0], red[4][0], red[5][0] };
            double ext = 0.0;
            for (int a = 0; a < 3; ++a)
                ext = fmax(ext, hi[a] - lo[a]);
            // the smallest power of two above ext (ext = f 2^k with f in [0.5, 1), so 2^k),
            // which keeps the maximum strictly inside the top cell; 1 for a zero or
            // non-finite extent
            double e = 1.0;
            if (ext > 0.0 && isfinite(ext))
            {
                int k = 0;
                frexp(ext, &k);
                e = ldexp(1.0, k);
            }
            // centre the cube on the bodies, then move its corner down onto the cell grid
            // (a shift of less than one cell); double the edge if that would uncover the
            // maximum. Cells are powers of two, so dividing by one is an exact multiply.
            for (int pass = 0; pass < 2; ++pass)
            {
                const double cell = ldexp(e, -kMortonBits), per_cell = ldexp(1.0 / e, kMortonBits);
                bool fits = true;
                for (int a = 0; a < 3; ++a)
                {
                    const double c = isfinite(lo[a]) ? 0.5 * (lo[a] + hi[a]) : 0.0;
                    b.lo[a] = floor((c - 0.5 * e) * per_cell) * cell;
                    b.center[a] = b.lo[a] + 0.5 * e;
                    fits = fits && (!isfinite(hi[a]) || hi[a] < b.lo[a] + e);
                }
                if (fits)
                    break;
                e *= 2.0;
            }
            b.edge = e;
        }
        b.inv_cell = static_cast<double>(1u << kMortonBits) / b.edge;
        // the integer quantisation applies when the cells are powers of two and the corner
        // sits on their grid (always for the fitted cube)
        int ex = 0;
        const double mant = frexp(b.edge, &ex);
        b.cell_exp = ex - 1 - kMortonBits;
        bool exact = mant == 0.5 && isfinite(b.edge) && b.cell_exp >= -149;
        for (int a = 0; a < 3; ++a)
        {
            const double lc = ldexp(b.lo[a], -b.cell_exp);
            exact = exact && lc == floor(lc) && fabs(lc) < 4.0e15;
            b.lo_cells[a] = exact ? static_cast<long long>(lc) : 0;
        }
        b.exact = exact ? 1 : 0;
        b.edge_f = static_cast<float>(b.edge);
        *box = b;
    }

    // ------------------------------------------------------------------------------------
    // 2. Morton codes
    // ------------------------------------------------------------------------------------
    __device__ __forceinline__ uint64_t spread3(uint64_t v)
    {
        v &= 0x1fffffull;
        v = (v | (v << 32)) & 0x001f00000000ffffull;
        v = (v | (v << 16)) & 0x001f0000ff0000ffull;
        v = (v | (v << 8)) & 0x100f00f00f00f00full;
        v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
        v = (v | (v << 2)) & 0x1249249249249249ull;
        return v;
    }

    __device__ __forceinline__ uint64_t quantise(const float x, const double lo, const double inv_cell)
    {
        const double t = __dmul_rd(__dsub_rd(static_cast<double>(x), lo), inv_cell);
        const double f = floor(t);
        if (!(f >= 0.0))
            return 0;
        if (f > 2097151.0)
            return 2097151;
        return static_cast<uint64_t>(f);
    }

    // The same cell index with integer operations only, for a box whose cells are 2^cell_exp
    // and whose corner is lo_cells cells from the origin: x = M 2^E exactly (M the 24-bit
    // significand), so floor(x / cell) = floor(M 2^(E - cell_exp)) is a shift (rounding
    // toward -inf for negative x), and the index is that minus lo_cells, clamped. It equals
    // quantise() there: the directed roundings make floor(rd(rd(x - lo) * inv_cell)) the
    // exact floor((x - lo) / cell) when every cell boundary is a double.
    __device__ __forceinline__ uint64_t quantise_exact(const float x, const int cell_exp, const long long lo_cells)
    {
        const uint32_t bits = __float_as_uint(x);
        const uint32_t e = (bits >> 23) & 0xffu;
        const uint32_t frac = bits & 0x7fffffu;
        const bool neg = bits >> 31;
        if (e == 0xffu)
            return (frac == 0 && !neg) ? 2097151u : 0u;     // +inf clamps high; -inf and NaN to 0
        const long long m = e ? static_cast<long long>(frac | 0x800000u) : static_cast<long long>(frac);
        const int s = (e ? static_cast<int>(e) - 150 : -149) - cell_exp;     // x / cell = m 2^s
        long long cells;
        if (s >= 0)
        {
            if (s > 38)     // |x| / cell >= 2^61: far outside the box
                return neg ? 0u : 2097151u;
            cells = neg ? -(m << s) : (m << s);
        }
        else
        {
            const int r = -s;
            if (r >= 62)
                cells = (neg && m) ? -1 : 0;
            else
                cells = neg ? -((m + (1ll << r) - 1) >> r) : (m >> r);
        }
        const long long q = cells - lo_cells;
        return q < 0 ? 0u : (q > 2097151 ? 2097151u : static_cast<uint64_t>(q));
    }

    constexpr int kMortonItems = 4;     // bodies per thread, all loads issued first

    __global__ void __launch_bounds__(256) morton_kernel(const float4* __restrict__ src, const int stride,
                                                         const int n, const BoxParams* __restrict__ box,
                                                         uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
    {
        const int base = blockIdx.x * (256 * kMortonItems) + threadIdx.x;
        float4 p[kMortonItems];
#pragma unroll
        for (int j = 0; j < kMortonItems; ++j)
        {
            const int i = base + j * 256;
            p[j] = i < n ? src[static_cast<size_t>(i) * stride] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const BoxParams& b = *box;
#pragma unroll
        for (int j = 0; j < kMortonItems; ++j)
        {
            const int i = base + j * 256;
            if (i >= n)
                break;
            uint64_t qx, qy, qz;
            if (b.exact)
            {
                qx = quantise_exact(p[j].x, b.cell_exp, b.lo_cells[0]);
                qy = quantise_exact(p[j].y, b.cell_exp, b.lo_cells[1]);
                qz = quantise_exact(p[j].z, b.cell_exp, b.lo_cells[2]);
            }
            else
            {
                qx = quantise(p[j].x, b.lo[0], b.inv_cell);
                qy = quantise(p[j].y, b.lo[1], b.inv_cell);
                qz = quantise(p[j].z, b.lo[2], b.inv_cell);
            }
            keys[i] = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
            vals[i] = static_cast<uint32_t>(i);
        }
    }

    // After the radix passes over bits [kRunShift, 63), the codes are in order of their top
    // bits, and the codes of one run (equal top bits) keep index order. The thread at the
    // start of a run of 2 .. kMaxRun codes puts it in order of the whole code by a stable
    // insertion sort, so ties keep index order: the result is the order by (code, index).
    // A longer run sets *full, and the build sorts everything again by all 63 bits. Other
    // threads read their neighbours' top bits while a run is being reordered: those bits are
    // the same for every code of the run, so what they see does not depend on the moment.
    __global__ void __launch_bounds__(256) run_sort_kernel(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                           const int n, unsigned* __restrict__ full)
    {
        const int i = blockIdx.x * 256 + threadIdx.x;
        if (i >= n)
            return;
        const uint64_t top = keys[i] >> kRunShift;
        if (i > 0 && (keys[i - 1] >> kRunShift) == top)
            return;     // not the first code of its run
        int len = 1;
        while (i + len < n && len <= kMaxRun && (keys[i + len] >> kRunShift) == top)
            ++len;
        if (len == 1)
            return;
        if (len > kMaxRun)
        {
            atomicOr(full, 1u);
            return;
        }
        for (int a = i + 1; a < i + len; ++a)
        {
            const uint64_t k = keys[a];
            const uint32_t v = vals[a];
            int b = a - 1;
            while (b >= i && keys[b] > k)
            {
                keys[b + 1] = keys[b];
                vals[b + 1] = vals[b];
                --b;
            }
            keys[b + 1] = k;
            vals[b + 1] = v;
        }
    }

    // Copies a full sort's result back into the buffers the build reads, when *run_if is set.
    __global__ void __launch_bounds__(256) copy_back_kernel(const uint64_t* __restrict__ ks,
                                                            const uint32_t* __restrict__ vs, uint64_t* __restrict__ kd,
                                                            uint32_t* __restrict__ vd, const int n,
                                                            const unsigned* __restrict__ run_if)
    {
        if (!*run_if)
            return;
        for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256)
        {
            kd[i] = ks[i];
            vd[i] = vs[i];
        }
    }

    // ------------------------------------------------------------------------------------
    // 4. Morton-ordered copies and the fixed-point cell sums
    // ------------------------------------------------------------------------------------
    // A cell's mass and centre of mass come from differences of prefix sums over the sorted
    // bodies. The sums are integers -- each body's m 2^mass_shift and m x 2^mom_shift,
    // rounded once -- so a difference is the exact sum of the cell's rounded terms: no
    // cancellation against the large prefixes before it, and the same bits whatever order
    // the additions run in. A body's term is formed from the float significands with
    // integer multiplies (m x is an exact 48-bit product), without FP64 arithmetic.

    // v = M 2^e with M < 2^24 (the significand, implicit bit included); false for inf/NaN
    __device__ __forceinline__ bool split_float(const float v, uint32_t& M, int& e, bool& neg)
    {
        const uint32_t bits = __float_as_uint(v);
        const uint32_t E = (bits >> 23) & 0xffu;
        neg = (bits >> 31) != 0;
        M = E ? ((bits & 0x7fffffu) | 0x800000u) : (bits & 0x7fffffu);
        e = (E ? static_cast<int>(E) : 1) - 150;
        return E != 0xffu;
    }

    // round(P 2^s), halves away from zero, with the sign applied. P < 2^48; the box's shifts
    // keep P 2^s below 2^61, so a left shift never overflows (and s >= 64 only when P = 0).
    __device__ __forceinline__ long long fixed_round(const uint64_t P, const int s, const bool neg)
    {
        uint64_t q;
        if (s >= 0)
            q = s < 64 ? P << s : 0;
        else if (s > -50)
            q = (P + (1ull << (-s - 1))) >> -s;
        else
            q = 0;      // P 2^s < 2^-2
        return neg ? -static_cast<long long>(q) : static_cast<long long>(q);
    }

    // {m x, m y, m z, m} of one body in the box's fixed-point units. A non-finite mass
    // contributes nothing; a non-finite coordinate contributes no moment on its axis.
    __device__ __forceinline__ Int64x4 body_terms(const float4 pm, const int mass_shift, const int mom_shift)
    {
        uint32_t Mm;
        int em;
        bool nm;
        if (!split_float(pm.w, Mm, em, nm))
            return Int64x4{ 0, 0, 0, 0 };
        const float x[3] = { pm.x, pm.y, pm.z };
        long long q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            uint32_t Mx;
            int ex;
            bool nx;
            q[a] = split_float(x[a], Mx, ex, nx)
                       ? fixed_round(static_cast<uint64_t>(Mm) * Mx, em + ex + mom_shift, nm != nx) : 0;
        }
        return Int64x4{ q[0], q[1], q[2], fixed_round(Mm, em + mass_shift, nm) };
    }

    __device__ __forceinline__ Int64x4 add4(const Int64x4 a, const Int64x4 b)
    {
        return Int64x4{ a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w };
    }

    // Bodies into Morton order (pos_mass, and the radius when srad is given: only the cutoff
    // law reads it), and the fixed-point prefix sums within each tile of kMomTile sorted
    // bodies: part[x] = the sum of the terms of the bodies of x's tile before x, for
    // x = 0 .. n (x = n belongs to tile n / kMomTile, which is past the last tile, and has
    // sum 0, when n is a multiple of the tile). Each tile's total goes to tile_sum; the sum
    // of all bodies before x is then tile_prefix[x / kMomTile] + part[x], with tile_prefix
    // the exclusive scan of the totals (a tile past the last has total 0). Tiles need not
    // wait for one another. Four consecutive bodies per thread; every random read is issued
    // before any is used (indices past the end read the last body and are not stored).
    __global__ void __launch_bounds__(kMomThreads) gather_sum_kernel(
        const float4* __restrict__ src, const int stride, const float4* __restrict__ vel_radius,
        const uint32_t* __restrict__ order, const int n, const BoxParams* __restrict__ box,
        float4* __restrict__ spm, float* __restrict__ srad, Int64x4* __restrict__ part,
        Int64x4* __restrict__ tile_sum)
    {
        using Op = ScanOps<Int64x4>;
        if (n <= 0)
            return;
        __shared__ Int64x4 warp_tot[kMomThreads / 32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int tile = blockIdx.x;
        const int mass_shift = box->mass_shift, mom_shift = box->mom_shift;
        const int base = tile * kMomTile + threadIdx.x * kMomItems;

        uint32_t idx[kMomItems];
        if (base + kMomItems <= n)
        {
            const uint4 o = *reinterpret_cast<const uint4*>(order + base);
            idx[0] = o.x;
            idx[1] = o.y;
            idx[2] = o.z;
            idx[3] = o.w;
        }
        else
        {
#pragma unroll
            for (int k = 0; k < kMomItems; ++k)
                idx[k] = order[min(base + k, n - 1)];
        }
        float4 p[kMomItems];
        float m[kMomItems], r[kMomItems];
#pragma unroll
        for (int k = 0; k < kMomItems; ++k)
        {
            const uint32_t i = idx[k];
            p[k] = src[static_cast<size_t>(i) * stride];
            if (stride == 3)
            {
                m[k] = src[static_cast<size_t>(i) * 3 + 1].w;     // Body: {pos, radius}, {vel, mass}
                r[k] = p[k].w;
            }
            else
            {
                m[k] = p[k].w;
                r[k] = vel_radius ? vel_radius[i].w : 0.f;
            }
        }
        // the thread's total here; its bodies' terms are formed again for the prefixes below
        // (cheaper than holding four more Int64x4 through the scan)
        Int64x4 run{ 0, 0, 0, 0 };
#pragma unroll
        for (int k = 0; k < kMomItems; ++k)
        {
            const int i = base + k;
            p[k].w = m[k];
            if (i < n)
            {
                spm[i] = p[k];
                if (srad)
                    srad[i] = r[k];
                run = add4(run, body_terms(p[k], mass_shift, mom_shift));
            }
        }

        // the tile's scan: within warps, then over the warps' totals
        Int64x4 incl = run;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
        {
            const Int64x4 o = Op::shfl_up(incl, d);
            if (lane >= d)
                incl = add4(incl, o);
        }
        if (lane == 31)
            warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0)
        {
            constexpr int kWarpsPerTile = kMomThreads / 32;
            Int64x4 wi = lane < kWarpsPerTile ? warp_tot[lane] : Int64x4{ 0, 0, 0, 0 };
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const Int64x4 o = Op::shfl_up(wi, d);
                if (lane >= d)
                    wi = add4(wi, o);
            }
            if (lane < kWarpsPerTile)
                warp_tot[lane] = wi;    // inclusive over warps
            if (lane == 31)
                tile_sum[tile] = wi;    // the tile's total
        }
        __syncthreads();
        Int64x4 off = Op::shfl_up(incl, 1);
        if (lane == 0)
            off = Int64x4{ 0, 0, 0, 0 };
        if (warp > 0)
            off = add4(off, warp_tot[warp - 1]);
#pragma unroll
        for (int k = 0; k < kMomItems; ++k)
        {
            const int i = base + k;
            if (i < n)
            {
                part[i] = off;
                off = add4(off, body_terms(p[k], mass_shift, mom_shift));
            }
        }
        if (base <= n - 1 && n - 1 < base + kMomItems)
        {
            const int past = (n % kMomTile) == 0 ? 1 : 0;    // x = n opens the tile past the last
            part[n] = past ? Int64x4{ 0, 0, 0, 0 } : off;
            tile_sum[tile + 1] = Int64x4{ 0, 0, 0, 0 };      // past the last tile: total 0
        }
    }

    // ------------------------------------------------------------------------------------
    // 5. binary radix tree (Karras 2012)
    // ------------------------------------------------------------------------------------
    // common-prefix length of sorted keys i and j (0 <= i < n), duplicates separated by
    // index (64 + the index bits they share); -1 for j outside [0, n)
    __device__ __forceinline__ int delta(const uint64_t* __restrict__ keys, const int n, const int i, const int j)
    {
        if (j < 0 || j >= n)
            return -1;
        const uint64_t a = keys[i], b = keys[j];
        if (a != b)
            return __clzll(static_cast<long long>(a ^ b));
        return 64 + __clz(static_cast<int>(static_cast<unsigned>(i) ^ static_cast<unsigned>(j)));
    }

    __device__ __forceinline__ int level_of(const int prefix) { return min(kMaxLevel, prefix / 3); }

    // dl[k] = delta(k, k + 1) for k < n - 1: 1 .. 95, one byte, and smp[k] = the key at 64 k
    // for 64 k < n - 1. Four per thread. For sorted keys the common prefix of keys i < j is
    // the least of dl[i .. j - 1].
    __global__ void __launch_bounds__(256) adjacent_prefix_kernel(const uint64_t* __restrict__ keys, const int n,
                                                                  uint8_t* __restrict__ dl, uint64_t* __restrict__ smp)
    {
        const int k0 = (blockIdx.x * 256 + threadIdx.x) * 4;
        if (k0 >= n - 1)
            return;
        uint64_t a[5];
#pragma unroll
        for (int u = 0; u < 5; ++u)
            a[u] = keys[min(k0 + u, n - 1)];
        if ((k0 & 63) == 0)
            smp[k0 >> 6] = a[0];        // every 64th key, for the far nodes' coarse searches
        uint32_t packed = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const int k = k0 + u;
            const uint32_t v = a[u] != a[u + 1]
                                   ? static_cast<uint32_t>(__clzll(static_cast<long long>(a[u] ^ a[u + 1])))
                                   : 64u + static_cast<uint32_t>(__clz(k ^ (k + 1)));
            packed |= (k < n - 1 ? v : 0u) << (8 * u);
        }
        if (k0 + 4 <= n - 1)
            *reinterpret_cast<uint32_t*>(dl + k0) = packed;
        else
            for (int u = 0; k0 + u < n - 1; ++u)
                dl[k0 + u] = static_cast<uint8_t>(packed >> (8 * u));
    }

    // one bit per byte of four 0x00 / 0xff bytes, byte 0 to bit 0
    __device__ __forceinline__ uint32_t movemask4(const uint32_t m) { return ((m & 0x80808080u) * 0x00204081u) >> 28; }

    // One bit for each of four bytes of x below the matching byte of lim (each <= 128),
    // without SIMD instructions, exact for bytes below 128 (every dl byte is at most 95):
    // with bit 7 set in each byte of x first, subtracting a byte of at most 128 borrows from
    // no other byte, and leaves bit 7 clear exactly where x's byte was the smaller.
    __device__ __forceinline__ uint32_t lt_mask4(const uint32_t x, const uint32_t lim)
    {
        return movemask4(~((x | 0x80808080u) - lim));
    }

    // 16 bytes: bit t set where byte t is below each byte of lim / equal to each byte of q
    __device__ __forceinline__ uint32_t lt_mask16(const uint4 w, const uint32_t lim)
    {
        return lt_mask4(w.x, lim) | (lt_mask4(w.y, lim) << 4) | (lt_mask4(w.z, lim) << 8) | (lt_mask4(w.w, lim) << 12);
    }

    __device__ __forceinline__ uint32_t eq_mask16(const uint4 w, const uint32_t q)
    {
        return lt_mask4(w.x ^ q, 0x01010101u) | (lt_mask4(w.y ^ q, 0x01010101u) << 4)
               | (lt_mask4(w.z ^ q, 0x01010101u) << 8) | (lt_mask4(w.w ^ q, 0x01010101u) << 12);
    }

    // The record of binary node i (Karras 2012) with range [lo, hi], split after gamma and
    // common prefix dnode bits, and whether it is an octree node. The range is bounded by
    // two splits, dmin at i's end and dfar at the other (-1 past either end of the array),
    // both below its own; its parent splits at the larger of the two (the smallest range
    // that strictly contains [lo, hi] ends where the shared prefix first shortens), so the
    // parent's prefix is known without a parent array. A node is an octree node when its
    // level exceeds its parent's, or it is the root.
    __device__ __forceinline__ void write_radix_node(const int i, const int lo, const int hi, const int gamma,
                                                     const int dnode, const int dmin, const int dfar,
                                                     int2* __restrict__ child, int2* __restrict__ range,
                                                     int* __restrict__ prefix, uint32_t* __restrict__ flag)
    {
        child[i] = make_int2(lo == gamma ? ~gamma : gamma, hi == gamma + 1 ? ~(gamma + 1) : gamma + 1);
        range[i] = make_int2(lo, hi);
        const int pre = dnode - 1;      // codes are 63-bit: the top key bit is always shared
        prefix[i] = pre;
        const int up = max(dmin, dfar) - 1;
        flag[i] = (i == 0 || level_of(pre) > level_of(up)) ? 1u : 0u;
    }

    // Radix-tree nodes whose ranges end within about kNearScan keys (97.5 % of them at 16.8M
    // disk + halo bodies), found without searches. Node i extends in direction d while the
    // adjacent prefixes stay above dmin = delta(i, i - d), so its far end is the first byte
    // of dl beyond i (in that direction) that is <= dmin: 16 bytes are compared at a time.
    // Its split is the one position of its range's least prefix, dnode = delta(i, j): the
    // first byte equal to dnode from the range's low end. A node whose end lies farther goes
    // to far_list for radix_far_kernel, so that no warp waits on one lane's long search
    // (Karras's searches for every node took 0.47 ms at 16.8M bodies; these kernels and the
    // prefix bytes take about 0.37).
    constexpr int kNearScan = 64;
    constexpr int kNearChunks = kNearScan / 16 + 1;

    // Node i by the byte scans: false when its record is written, true when its range ends
    // too far for them
    __device__ __forceinline__ bool near_node(const uint64_t* __restrict__ keys, const uint8_t* __restrict__ dl,
                                              const int n, const int i, int2* __restrict__ child,
                                              int2* __restrict__ range, int* __restrict__ prefix,
                                              uint32_t* __restrict__ flag, unsigned* __restrict__ err)
    {
        const int dr = dl[i];
        const int dlf = i > 0 ? static_cast<int>(dl[i - 1]) : -1;
        const int d = dr - dlf >= 0 ? 1 : -1;
        const int dmin = d > 0 ? dlf : dr;
        int j = -1;
        if (dmin >= 0)
        {
            const uint32_t rep = static_cast<uint32_t>(dmin + 1) * 0x01010101u;     // bytes <= dmin
            if (d > 0)
            {
                // the first p >= i with dl[p] <= dmin, or n - 1 (past the last pair)
                for (int c = 0; c < kNearChunks; ++c)
                {
                    const int base = (i & ~15) + 16 * c;
                    uint32_t mk = base < n - 1 ? lt_mask16(*reinterpret_cast<const uint4*>(dl + base), rep) : 0u;
                    if (c == 0)
                        mk &= ~((1u << (i & 15)) - 1u);
                    const int past = n - 1 - base;      // bytes from here on are past the last pair
                    if (past < 16)
                        mk |= past <= 0 ? 0xffffu : (0xffffu << past) & 0xffffu;
                    if (mk)
                    {
                        j = base + __ffs(mk) - 1;
                        break;
                    }
                }
            }
            else
            {
                // the last p <= i - 1 with dl[p] <= dmin, plus one; or 0 (before the first)
                for (int c = 0; c < kNearChunks; ++c)
                {
                    const int base = ((i - 1) & ~15) - 16 * c;
                    if (base < 0)
                    {
                        j = 0;
                        break;
                    }
                    uint32_t mk = lt_mask16(*reinterpret_cast<const uint4*>(dl + base), rep);
                    if (c == 0)
                        mk &= (2u << ((i - 1) & 15)) - 1u;
                    if (mk)
                    {
                        j = base + (31 - __clz(mk)) + 1;
                        break;
                    }
                    if (base == 0)
                    {
                        j = 0;
                        break;
                    }
                }
            }
        }
        if (j < 0)
            return true;
        const int lo = min(i, j), hi = max(i, j);
        const int dnode = delta(keys, n, i, j);
        const uint32_t rq = static_cast<uint32_t>(dnode) * 0x01010101u;
        int gamma = -1;
        for (int c = 0; c < kNearChunks + 1; ++c)
        {
            const int base = (lo & ~15) + 16 * c;
            if (base > n - 2)
                break;      // past the last pair: the split was not found
            uint32_t mk = eq_mask16(*reinterpret_cast<const uint4*>(dl + base), rq);
            if (c == 0)
                mk &= ~((1u << (lo & 15)) - 1u);
            if (mk)
            {
                gamma = base + __ffs(mk) - 1;
                break;
            }
        }
        if (gamma < lo || gamma >= hi)
        {
            atomicOr(err, DEV_ERR_BOUNDS);      // a range without its split: not sorted keys
            return false;
        }
        const int dfar = d > 0 ? (j < n - 1 ? static_cast<int>(dl[j]) : -1) : (j > 0 ? static_cast<int>(dl[j - 1]) : -1);
        write_radix_node(i, lo, hi, gamma, dnode, dmin, dfar, child, range, prefix, flag);
        return false;
    }

    __global__ void __launch_bounds__(256) radix_near_kernel(
        const uint64_t* __restrict__ keys, const uint8_t* __restrict__ dl, const int n, int2* __restrict__ child,
        int2* __restrict__ range, int* __restrict__ prefix, uint32_t* __restrict__ flag, int* __restrict__ far_list,
        unsigned* __restrict__ far_count, unsigned* __restrict__ err)
    {
        const int i = blockIdx.x * 256 + threadIdx.x;
        const bool far = i < n - 1 && near_node(keys, dl, n, i, child, range, prefix, flag, err);
        // a warp's far nodes take consecutive slots of far_list: one global atomic a warp
        const unsigned fm = __ballot_sync(0xffffffffu, far);
        if (!fm)
            return;
        const int lane = threadIdx.x & 31, leader = __ffs(fm) - 1;
        unsigned base = 0;
        if (lane == leader)
            base = atomicAdd(far_count, static_cast<unsigned>(__popc(fm)));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (far)
            far_list[base + __popc(fm & ((1u << lane) - 1u))] = i;
    }

    __device__ __forceinline__ int delta_of(const uint64_t a, const int i, const uint64_t b, const int j)
    {
        return a != b ? __clzll(static_cast<long long>(a ^ b))
                      : 64 + __clz(static_cast<int>(static_cast<unsigned>(i) ^ static_cast<unsigned>(j)));
    }

    // The first p >= start with dl[p] <= D (n - 1 when none: past the last pair), given
    // dl[ref .. start - 1] > D and kref = key ref. A coarse search over every 64th key finds
    // the last sampled position P with delta(ref, P) > D, that is dl[ref .. P - 1] > D
    // (exponential, then binary); the answer lies in the 64 bytes after it, found by the
    // byte scan. The samples are 1/64 of the keys and stay in the caches.
    __device__ int first_le_up(const uint64_t* __restrict__ smp, const uint8_t* __restrict__ dl, const int n,
                               const uint64_t kref, const int ref, const int start, const int D,
                               unsigned* __restrict__ err)
    {
        auto f = [&](const int k) {
            const int P = 64 * k;
            return P < n - 1 && delta_of(kref, ref, smp[k], P) > D;
        };
        int q0 = start;
        const int ka = (start >> 6) + 1;
        if (f(ka))
        {
            int lo = ka, step = 1;
            while (f(lo + step))
            {
                lo += step;
                step <<= 1;
            }
            int hi = lo + step;
            while (hi - lo > 1)
            {
                const int mid = (lo + hi) >> 1;
                if (f(mid))
                    lo = mid;
                else
                    hi = mid;
            }
            q0 = 64 * lo;
        }
        const uint32_t lim = static_cast<uint32_t>(D + 1) * 0x01010101u;      // bytes <= D
        for (int c = 0; c < 8; ++c)
        {
            const int base = (q0 & ~15) + 16 * c;
            uint32_t mk = base < n - 1 ? lt_mask16(*reinterpret_cast<const uint4*>(dl + base), lim) : 0u;
            if (c == 0)
                mk &= ~((1u << (q0 & 15)) - 1u);
            const int past = n - 1 - base;
            if (past < 16)
                mk |= past <= 0 ? 0xffffu : (0xffffu << past) & 0xffffu;
            if (mk)
                return base + __ffs(mk) - 1;
        }
        atomicOr(err, DEV_ERR_BOUNDS);      // not sorted keys
        return n - 1;
    }

    // The last p <= start with dl[p] <= D (-1 when none), given dl[start + 1 .. ref - 1] > D;
    // the same coarse search downward (delta(ref, P) > D means dl[P .. ref - 1] > D).
    __device__ int last_le_down(const uint64_t* __restrict__ smp, const uint8_t* __restrict__ dl, const uint64_t kref,
                                const int ref, const int start, const int D, unsigned* __restrict__ err)
    {
        auto f = [&](const int k) { return k >= 0 && delta_of(kref, ref, smp[k], 64 * k) > D; };
        int q0 = start;
        const int ka = start >> 6;
        if (f(ka))
        {
            int hi = ka, step = 1;
            while (f(hi - step))
            {
                hi -= step;
                step <<= 1;
            }
            int lo = hi - step;
            while (hi - lo > 1)
            {
                const int mid = (lo + hi) >> 1;
                if (f(mid))
                    hi = mid;
                else
                    lo = mid;
            }
            q0 = 64 * hi - 1;
        }
        const uint32_t lim = static_cast<uint32_t>(D + 1) * 0x01010101u;
        for (int c = 0; c < 8; ++c)
        {
            const int base = (q0 & ~15) - 16 * c;
            if (q0 < 0 || base < 0)
                return -1;
            uint32_t mk = lt_mask16(*reinterpret_cast<const uint4*>(dl + base), lim);
            if (c == 0)
                mk &= (2u << (q0 & 15)) - 1u;
            if (mk)
                return base + 31 - __clz(mk);
        }
        atomicOr(err, DEV_ERR_BOUNDS);
        return -1;
    }

    // The nodes radix_near_kernel passed on, one per thread: the range's far end and the
    // split by the coarse-then-fine searches above (the top levels' nodes span millions of
    // keys; their searches over the samples stay in the caches).
    __global__ void __launch_bounds__(256) radix_far_kernel(const uint64_t* __restrict__ keys,
                                                            const uint8_t* __restrict__ dl,
                                                            const uint64_t* __restrict__ smp, const int n,
                                                            const int* __restrict__ far_list,
                                                            const unsigned* __restrict__ far_count,
                                                            int2* __restrict__ child, int2* __restrict__ range,
                                                            int* __restrict__ prefix, uint32_t* __restrict__ flag,
                                                            unsigned* __restrict__ err)
    {
        const int count = static_cast<int>(*far_count);
        for (int q = blockIdx.x * 256 + threadIdx.x; q < count; q += gridDim.x * 256)
        {
            const int i = far_list[q];
            const uint64_t ki = keys[i];
            const int dr = dl[i];
            const int dlf = i > 0 ? static_cast<int>(dl[i - 1]) : -1;
            const int d = dr - dlf >= 0 ? 1 : -1;
            const int dmin = d > 0 ? dlf : dr;
            const int j = d > 0 ? first_le_up(smp, dl, n, ki, i, i, dmin, err)
                                : last_le_down(smp, dl, ki, i, i - 1, dmin, err) + 1;
            const int lo = min(i, j), hi = max(i, j);
            const int dnode = delta(keys, n, i, j);
            const int gamma = first_le_up(smp, dl, n, keys[lo], lo, lo, dnode, err);
            if (gamma < lo || gamma >= hi)
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                continue;
            }
            const int dfar = d > 0 ? (j < n - 1 ? static_cast<int>(dl[j]) : -1) : (j > 0 ? static_cast<int>(dl[j - 1]) : -1);
            write_radix_node(i, lo, hi, gamma, dnode, dmin, dfar, child, range, prefix, flag);
        }
    }

    // ------------------------------------------------------------------------------------
    // 6. octree records
    // ------------------------------------------------------------------------------------
    // The children of a cell: walking down through the binary nodes of the cell's own level
    // (at most three splits below it), every leaf body and every node of a deeper level is
    // one child. Right subtrees first, which is the order the traversal has always used.
    // Children are kept in registers (kid[k] selected by a static index) and stored at once.
    __device__ __forceinline__ void emit_child(int (&kid)[8], int& nc, const int v, unsigned* __restrict__ err)
    {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            kid[k] = k == nc ? v : kid[k];
        if (nc >= 8)
            atomicOr(err, DEV_ERR_BOUNDS);
        ++nc;
    }

    template <int DEPTH>
    __device__ __forceinline__ void collect_children(const int c, const int2* __restrict__ child,
                                                     const uint32_t* __restrict__ flag,
                                                     const uint32_t* __restrict__ octidx, int (&kid)[8],
                                                     int& nc, unsigned* __restrict__ err)
    {
        if (c < 0 || flag[c])
        {
            emit_child(kid, nc, c < 0 ? c : static_cast<int>(octidx[c]), err);
            return;
        }
        if (DEPTH == 0)
        {
            atomicOr(err, DEV_ERR_BOUNDS);      // more than three splits inside one octal level
            return;
        }
        const int2 ch = child[c];
        collect_children<DEPTH ? DEPTH - 1 : 0>(ch.y, child, flag, octidx, kid, nc, err);
        collect_children<DEPTH ? DEPTH - 1 : 0>(ch.x, child, flag, octidx, kid, nc, err);
    }

    // position of the r-th set bit (from 0) of v, for r < popc(v)
    __device__ __forceinline__ int select_bit(unsigned v, int r)
    {
        int pos = 0;
#pragma unroll
        for (int w = 16; w > 0; w >>= 1)
        {
            const int c = __popc(v & ((1u << w) - 1u));
            if (r >= c)
            {
                r -= c;
                v >>= w;
                pos += w;
            }
        }
        return pos;
    }

    // An int64 as float: |v| split into two 32-bit halves, each converted exactly or with one
    // rounding, joined by one FMA (within about an ulp). No FP64 operation: GB300's FP64
    // pipe is its slowest.
    __device__ __forceinline__ float i64_to_float(const long long v)
    {
        const unsigned long long u = v < 0 ? 0ull - static_cast<unsigned long long>(v) : static_cast<unsigned long long>(v);
        const float f = fmaf(static_cast<float>(static_cast<uint32_t>(u >> 32)), 4294967296.0f,
                             static_cast<float>(static_cast<uint32_t>(u)));
        return v < 0 ? -f : f;
    }

    constexpr int kOctSpan = 4;     // binary nodes per lane that one warp scans for octree nodes

    // One octree record per flagged binary node. Latency bound (chains of dependent loads),
    // so a warp first gathers the flagged nodes among 32 * kOctSpan consecutive binary nodes
    // (ballots; about 40 % are flagged) and its lanes then take them in turn, instead of
    // idling on unflagged ones; and full occupancy (32 registers) beats fewer spills.
    __global__ void __launch_bounds__(256, 8) octnode_kernel(const int2* __restrict__ child, const int2* __restrict__ range,
                                   const int* __restrict__ prefix, const uint32_t* __restrict__ flag,
                                   const uint32_t* __restrict__ octidx, const Int64x4* __restrict__ part,
                                   const Int64x4* __restrict__ tile_prefix, const int m,
                                   const BoxParams* __restrict__ box, const float theta,
                                   OctNode* __restrict__ nodes, unsigned* __restrict__ err,
                                   unsigned long long* __restrict__ stats)
    {
        const int gt = blockIdx.x * blockDim.x + threadIdx.x;
        if (gt == 0)
            atomicAdd(&stats[2], static_cast<unsigned long long>(octidx[m - 1] + flag[m - 1]));
        const int lane = threadIdx.x & 31;
        const int first = (gt >> 5) * (32 * kOctSpan);
        if (first >= m)
            return;     // the whole warp
        unsigned mask[kOctSpan];
        int total = 0;
#pragma unroll
        for (int u = 0; u < kOctSpan; ++u)
        {
            const int i = first + u * 32 + lane;
            mask[u] = __ballot_sync(0xffffffffu, i < m && flag[i] != 0u);
            total += __popc(mask[u]);
        }
        const int shift = box->mass_shift - box->mom_shift;
        for (int q = lane; q < total; q += 32)
        {
            int u = 0, r = q;
#pragma unroll
            for (int k = 0; k < kOctSpan - 1; ++k)
                if (u == k && r >= __popc(mask[k]))
                {
                    r -= __popc(mask[k]);
                    u = k + 1;
                }
            unsigned mu = mask[0];
#pragma unroll
            for (int k = 1; k < kOctSpan; ++k)
                mu = u == k ? mask[k] : mu;
            const int i = first + u * 32 + select_bit(mu, r);
            const int2 rg = range[i];
            const int pre = prefix[i];
            const int lvl = level_of(pre);
            // the sums before the cell's first body and after its last: exact integers
            const Int64x4 hi = add4(tile_prefix[(rg.y + 1) / kMomTile], part[rg.y + 1]);
            const Int64x4 lo = add4(tile_prefix[rg.x / kMomTile], part[rg.x]);
            const long long ms = hi.w - lo.w;   // exact: the cell's own terms
            OctNode* out = nodes + octidx[i];
            float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ms > 0)
            {
                // com = (sum of m x 2^mom_shift) / (sum of m 2^mass_shift) * 2^(mass_shift - mom_shift),
                // in float: the quotient lies in [-1, 1] before the exact power-of-two scaling
                const float fm = i64_to_float(ms);
                const float rm = __frcp_rn(fm);
                cm = make_float4(ldexpf(i64_to_float(hi.x - lo.x) * rm, shift),
                                 ldexpf(i64_to_float(hi.y - lo.y) * rm, shift),
                                 ldexpf(i64_to_float(hi.z - lo.z) * rm, shift), ldexpf(fm, -box->mass_shift));
            }
            // the reference's node size is the root size halved per level, in float
            const float sz = ldexpf(box->edge_f, -lvl);
            const float open_r2 = __fmul_rn(__fmul_rn(sz, sz), __fmul_rn(theta, theta));
            int kid[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
            int nc = 0;
            if (pre >= 3 * kMaxLevel)
                nc = -1;     // bucket: identical codes, bodies applied one by one
            else
            {
                const int2 ch = child[i];
                collect_children<2>(ch.y, child, flag, octidx, kid, nc, err);
                collect_children<2>(ch.x, child, flag, octidx, kid, nc, err);
                nc = min(nc, 8);
            }
            out->com_mass = cm;
            *reinterpret_cast<int4*>(&out->open_r2) = make_int4(__float_as_int(open_r2), nc, rg.x, rg.y);
            int4* kids = reinterpret_cast<int4*>(out->child);
            kids[0] = make_int4(kid[0], kid[1], kid[2], kid[3]);
            kids[1] = make_int4(kid[4], kid[5], kid[6], kid[7]);
        }
    }

    // ------------------------------------------------------------------------------------
    // 7. traversal
    // ------------------------------------------------------------------------------------
    template <int LAW>
    __device__ __forceinline__ void apply(const float px, const float py, const float pz, const float lim,
                                          const float sx, const float sy, const float sz, const float m,
                                          float& ax, float& ay, float& az)
    {
        const float dx = sx - px, dy = sy - py, dz = sz - pz;
        float r2 = (LAW == NBODY_LAW_SOFTENED) ? fmaf(dx, dx, lim) : dx * dx;
        r2 = fmaf(dy, dy, r2);
        r2 = fmaf(dz, dz, r2);
        float inv = rsqrt_sfu(r2);
        if (LAW == NBODY_LAW_CUTOFF)
            inv = r2 > lim ? inv : 0.f;     // physics.h:38-39
        const float s = m * inv * inv * inv;
        ax = fmaf(dx, s, ax);
        ay = fmaf(dy, s, ay);
        az = fmaf(dz, s, az);
    }

    template <int LAW>
    __global__ void __launch_bounds__(kTravWarps * 32, 4) traverse_kernel(
        const OctNode* __restrict__ nodes, const float4* __restrict__ spm, const float* __restrict__ srad,
        const uint32_t* __restrict__ order, const int n, const float G, const float eps2,
        float4* __restrict__ acc, float* __restrict__ body_out, unsigned* __restrict__ err,
        unsigned long long* __restrict__ stats)
    {
        // one 8-byte entry per stacked cell: {cell index, mask of the lanes that opened it}
        __shared__ int2 stk[kTravWarps][kStack];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1u;
        unsigned inter = 0, visits = 0;

        // 32-target tiles are handed out in order by a counter (stats[3], zeroed with the
        // statistics at every build), so warps that drew cheap tiles take more of them
        auto next_tile = [&]() {
            unsigned long long t = 0;
            if (lane == 0)
                t = atomicAdd(&stats[3], 1ull);
            return static_cast<int>(__shfl_sync(0xffffffffu, t, 0));
        };
        for (int tile = next_tile(); static_cast<long long>(tile) * 32 < n; tile = next_tile())
        {
            const int k = tile * 32 + lane;
            const bool valid = k < n;
            const float4 me = spm[valid ? k : n - 1];
            const float rad = srad[valid ? k : n - 1];
            const float lim = (LAW == NBODY_LAW_CUTOFF) ? rad * rad : eps2;
            float ax = 0.f, ay = 0.f, az = 0.f;
            const unsigned valid_mask = __ballot_sync(0xffffffffu, valid);
            if (lane == 0)
                stk[warp][0] = make_int2(0, static_cast<int>(valid_mask));
            int sp = 1;
            __syncwarp();
            // Each cell is reached from its one parent, so a warp pops at most one entry
            // per cell (< n). The bound only trips on a malformed tree: it records the
            // error and stops this warp instead of spinning.
            int guard = 0;
            const int guard_limit = n + 64;
            while (sp > 0)
            {
                if (++guard > guard_limit)
                {
                    if (lane == 0)
                        atomicOr(err, DEV_ERR_BOUNDS);
                    break;
                }
                --sp;
                const int2 top = stk[warp][sp];
                __syncwarp();
                const int nd = top.x;
                const unsigned mask = static_cast<unsigned>(top.y);
                ++visits;
                const OctNode* cell = nodes + nd;
                // the three loads of a visit issue together: centre of mass + mass;
                // open_r2, nchild, first, last; this lane's child slot
                const float4 cm = cell->com_mass;
                const int4 meta = *reinterpret_cast<const int4*>(&cell->open_r2);
                const int cslot = cell->child[lane & 7];
                if (cm.w == 0.f)
                    continue;       // bhtree.cpp:109-113: empty nodes are skipped
                const bool in = (mask >> lane) & 1u;
                // bhtree.cpp:117-125, evaluated in the reference's operation order
                const float dx = __fsub_rn(cm.x, me.x), dy = __fsub_rn(cm.y, me.y), dz = __fsub_rn(cm.z, me.z);
                const float dist_sq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                const bool accept = in && dist_sq > __int_as_float(meta.x);
                if (accept)
                {
                    apply<LAW>(me.x, me.y, me.z, lim, cm.x, cm.y, cm.z, cm.w, ax, ay, az);
                    ++inter;
                }
                const unsigned open = mask & ~__ballot_sync(0xffffffffu, accept);
                if (!open)
                    continue;
                const bool mine = (open >> lane) & 1u;
                const int nchild = meta.y;
                if (nchild < 0)
                {
                    for (int b = meta.z; b <= meta.w; ++b)
                    {
                        const float4 s = spm[b];
                        if (mine)
                        {
                            apply<LAW>(me.x, me.y, me.z, lim, s.x, s.y, s.z, s.w, ax, ay, az);
                            ++inter;
                        }
                    }
                    continue;
                }
                const int c = lane < nchild ? cslot : 0;
                const bool is_cell = lane < nchild && c >= 0;
                const bool is_leaf = lane < nchild && c < 0;
                // each child lane fetches its own leaf body, so the leaf loop below only
                // broadcasts registers
                const float4 leaf = is_leaf ? spm[~c] : make_float4(0.f, 0.f, 0.f, 0.f);
                const unsigned cells = __ballot_sync(0xffffffffu, is_cell);
                unsigned leaves = __ballot_sync(0xffffffffu, is_leaf && leaf.w != 0.f);
                if (is_cell)
                {
                    const int at = sp + __popc(cells & lt);
                    if (at < kStack)
                        stk[warp][at] = make_int2(c, static_cast<int>(open));
                    else
                        atomicOr(err, DEV_ERR_BOUNDS);
                }
                sp = min(kStack, sp + __popc(cells));
                __syncwarp();
                while (leaves)
                {
                    const int l = __ffs(leaves) - 1;
                    leaves &= leaves - 1;
                    const float sx = __shfl_sync(0xffffffffu, leaf.x, l);
                    const float sy = __shfl_sync(0xffffffffu, leaf.y, l);
                    const float sz = __shfl_sync(0xffffffffu, leaf.z, l);
                    const float sw = __shfl_sync(0xffffffffu, leaf.w, l);
                    if (mine)
                    {
                        apply<LAW>(me.x, me.y, me.z, lim, sx, sy, sz, sw, ax, ay, az);
                        ++inter;
                    }
                }
            }
            if (valid)
            {
                const uint32_t i = order[k];
                if (body_out)
                {
                    float* o = body_out + static_cast<size_t>(i) * 12 + 8;
                    o[0] = G * ax;
                    o[1] = G * ay;
                    o[2] = G * az;
                }
                else
                    acc[i] = make_float4(G * ax, G * ay, G * az, 0.f);
            }
        }
        // per-warp totals
        unsigned long long total = inter;
        for (int o = 16; o > 0; o >>= 1)
            total += __shfl_down_sync(0xffffffffu, total, o);
        if (lane == 0)
        {
            atomicAdd(&stats[0], total);
            atomicAdd(&stats[1], static_cast<unsigned long long>(visits));
        }
    }

    // Two targets per lane: the packed form of apply(). Both halves run the scalar
    // operations of apply() in the same order (an FP32x2 operation is two correctly rounded
    // FP32 operations), and a half whose target does not take the node gets s = 0, which
    // adds exactly zero. Targets are held as negated positions (d = s + (-x)).
    template <int LAW>
    __device__ __forceinline__ void apply2(const float2 npx, const float2 npy, const float2 npz, const float2 lim,
                                           const float sx, const float sy, const float sz, const float m,
                                           const bool take_a, const bool take_b, float2& ax, float2& ay, float2& az)
    {
        const float2 dx = add2(f2(sx), npx), dy = add2(f2(sy), npy), dz = add2(f2(sz), npz);
        float2 r2 = (LAW == NBODY_LAW_SOFTENED) ? fma2(dx, dx, lim) : mul2(dx, dx);
        r2 = fma2(dy, dy, r2);
        r2 = fma2(dz, dz, r2);
        float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
        if (LAW == NBODY_LAW_CUTOFF)
        {
            inv.x = r2.x > lim.x ? inv.x : 0.f;     // physics.h:38-39
            inv.y = r2.y > lim.y ? inv.y : 0.f;
        }
        float2 sc = mul2(mul2(mul2(f2(m), inv), inv), inv);
        sc.x = take_a ? sc.x : 0.f;
        sc.y = take_b ? sc.y : 0.f;
        ax = fma2(dx, sc, ax);
        ay = fma2(dy, sc, ay);
        az = fma2(dz, sc, az);
    }

    // The walk of traverse_kernel for 64 Q Morton-consecutive targets per warp: lane l holds
    // targets 64 Q t + 32 h + l for h < 2Q, as Q packed pairs (halves 2p and 2p + 1), and a
    // stack entry carries one lane mask per target slot h. Each target still decides every
    // node itself with the reference test, and its accepted nodes come in the same
    // depth-first order, so its sum is the one traverse_kernel forms; one walk now serves
    // 2Q times the targets and every interaction is a packed pair.
    template <int LAW, int Q>
    __global__ void __launch_bounds__(pair_warps(Q) * 32, 2 * kTravWarps / pair_warps(Q)) traverse_pairs_kernel(
        const OctNode* __restrict__ nodes, const float4* __restrict__ spm, const float* __restrict__ srad,
        const uint32_t* __restrict__ order, const int n, const float G, const float eps2,
        float4* __restrict__ acc, float* __restrict__ body_out, unsigned* __restrict__ err,
        unsigned long long* __restrict__ stats)
    {
        constexpr int H = 2 * Q;                    // target slots per lane
        constexpr int TW = 32 * H;                  // targets per warp walk
        constexpr int W = pair_warps(Q);
        __shared__ int stk_cell[W][kStack];
        __shared__ unsigned stk_mask[W][kStack][H];     // lanes of each slot that opened it
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1u;
        unsigned inter = 0, visits = 0;

        // tiles are handed out in order by a counter (stats[3], zeroed with the statistics at
        // every build), so warps that drew cheap tiles take more of them: a tile from the
        // dense centre of a disk costs many times one from its edge
        auto next_tile = [&]() {
            unsigned long long t = 0;
            if (lane == 0)
                t = atomicAdd(&stats[3], 1ull);
            return static_cast<int>(__shfl_sync(0xffffffffu, t, 0));
        };
        for (int tile = next_tile(); static_cast<long long>(tile) * TW < n; tile = next_tile())
        {
            float2 npx[Q], npy[Q], npz[Q], lim[Q], ax[Q], ay[Q], az[Q];
            unsigned m0[H];
#pragma unroll
            for (int q = 0; q < Q; ++q)
            {
                float v[2][4];
#pragma unroll
                for (int e = 0; e < 2; ++e)
                {
                    const int k = tile * TW + (2 * q + e) * 32 + lane;
                    const bool valid = k < n;
                    m0[2 * q + e] = __ballot_sync(0xffffffffu, valid);
                    const float4 pk = spm[valid ? k : n - 1];
                    v[e][0] = -pk.x;
                    v[e][1] = -pk.y;
                    v[e][2] = -pk.z;
                    if (LAW == NBODY_LAW_CUTOFF)
                    {
                        const float r = srad[valid ? k : n - 1];
                        v[e][3] = r * r;
                    }
                    else
                        v[e][3] = eps2;
                }
                npx[q] = make_float2(v[0][0], v[1][0]);
                npy[q] = make_float2(v[0][1], v[1][1]);
                npz[q] = make_float2(v[0][2], v[1][2]);
                lim[q] = make_float2(v[0][3], v[1][3]);
                ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
            }
            if (lane == 0)
            {
                stk_cell[warp][0] = 0;
#pragma unroll
                for (int h = 0; h < H; ++h)
                    stk_mask[warp][0][h] = m0[h];
            }
            int sp = 1;
            __syncwarp();
            // Each cell is reached from its one parent, so a warp pops at most one entry
            // per cell (< n). The bound only trips on a malformed tree: it records the
            // error and stops this warp instead of spinning.
            int guard = 0;
            const int guard_limit = n + 64;
            while (sp > 0)
            {
                if (++guard > guard_limit)
                {
                    if (lane == 0)
                        atomicOr(err, DEV_ERR_BOUNDS);
                    break;
                }
                --sp;
                const int nd = stk_cell[warp][sp];
                unsigned mask[H];
#pragma unroll
                for (int h = 0; h < H; ++h)
                    mask[h] = stk_mask[warp][sp][h];
                __syncwarp();
                ++visits;
                const OctNode* cell = nodes + nd;
                const float4 cm = cell->com_mass;
                const int4 meta = *reinterpret_cast<const int4*>(&cell->open_r2);
                const int cslot = cell->child[lane & 7];
                if (cm.w == 0.f)
                    continue;       // bhtree.cpp:109-113: empty nodes are skipped
                const float open_r2 = __int_as_float(meta.x);
                bool take[H];
                unsigned open_any = 0;
                unsigned open[H];
#pragma unroll
                for (int q = 0; q < Q; ++q)
                {
                    // bhtree.cpp:117-125, evaluated in the reference's operation order with
                    // every operation rounded on its own (packed, two targets at a time). A
                    // contracted multiply-add has one rounding less, which flips borderline
                    // acceptances; sq2 forms the squares so that none can be contracted.
                    const float2 dx = add2(f2(cm.x), npx[q]), dy = add2(f2(cm.y), npy[q]), dz = add2(f2(cm.z), npz[q]);
                    const float2 ds = add2(add2(sq2(dx), sq2(dy)), sq2(dz));
                    const float ds0 = ds.x, ds1 = ds.y;
                    take[2 * q] = ((mask[2 * q] >> lane) & 1u) && ds0 > open_r2;
                    take[2 * q + 1] = ((mask[2 * q + 1] >> lane) & 1u) && ds1 > open_r2;
                    if (take[2 * q] || take[2 * q + 1])
                    {
                        apply2<LAW>(npx[q], npy[q], npz[q], lim[q], cm.x, cm.y, cm.z, cm.w, take[2 * q],
                                    take[2 * q + 1], ax[q], ay[q], az[q]);
                        inter += static_cast<unsigned>(take[2 * q]) + static_cast<unsigned>(take[2 * q + 1]);
                    }
                }
#pragma unroll
                for (int h = 0; h < H; ++h)
                {
                    open[h] = mask[h] & ~__ballot_sync(0xffffffffu, take[h]);
                    open_any |= open[h];
                }
                if (!open_any)
                    continue;
                bool mine[H], mine_any = false;
#pragma unroll
                for (int h = 0; h < H; ++h)
                {
                    mine[h] = (open[h] >> lane) & 1u;
                    mine_any |= mine[h];
                }
                const int nchild = meta.y;
                if (nchild < 0)
                {
                    for (int b = meta.z; b <= meta.w; ++b)
                    {
                        const float4 sb = spm[b];
                        if (mine_any)
                        {
#pragma unroll
                            for (int q = 0; q < Q; ++q)
                                if (mine[2 * q] || mine[2 * q + 1])
                                {
                                    apply2<LAW>(npx[q], npy[q], npz[q], lim[q], sb.x, sb.y, sb.z, sb.w, mine[2 * q],
                                                mine[2 * q + 1], ax[q], ay[q], az[q]);
                                    inter += static_cast<unsigned>(mine[2 * q]) + static_cast<unsigned>(mine[2 * q + 1]);
                                }
                        }
                    }
                    continue;
                }
                const int c = lane < nchild ? cslot : 0;
                const bool is_cell = lane < nchild && c >= 0;
                const bool is_leaf = lane < nchild && c < 0;
                // each child lane fetches its own leaf body, so the leaf loop below only
                // broadcasts registers
                const float4 leaf = is_leaf ? spm[~c] : make_float4(0.f, 0.f, 0.f, 0.f);
                const unsigned cells = __ballot_sync(0xffffffffu, is_cell);
                unsigned leaves = __ballot_sync(0xffffffffu, is_leaf && leaf.w != 0.f);
                if (is_cell)
                {
                    const int at = sp + __popc(cells & lt);
                    if (at < kStack)
                    {
                        stk_cell[warp][at] = c;
#pragma unroll
                        for (int h = 0; h < H; ++h)
                            stk_mask[warp][at][h] = open[h];
                    }
                    else
                        atomicOr(err, DEV_ERR_BOUNDS);
                }
                sp = min(kStack, sp + __popc(cells));
                __syncwarp();
                while (leaves)
                {
                    const int l = __ffs(leaves) - 1;
                    leaves &= leaves - 1;
                    const float sx = __shfl_sync(0xffffffffu, leaf.x, l);
                    const float sy = __shfl_sync(0xffffffffu, leaf.y, l);
                    const float sz = __shfl_sync(0xffffffffu, leaf.z, l);
                    const float sw = __shfl_sync(0xffffffffu, leaf.w, l);
                    if (mine_any)
                    {
#pragma unroll
                        for (int q = 0; q < Q; ++q)
                            if (mine[2 * q] || mine[2 * q + 1])
                            {
                                apply2<LAW>(npx[q], npy[q], npz[q], lim[q], sx, sy, sz, sw, mine[2 * q], mine[2 * q + 1],
                                            ax[q], ay[q], az[q]);
                                inter += static_cast<unsigned>(mine[2 * q]) + static_cast<unsigned>(mine[2 * q + 1]);
                            }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < Q; ++q)
#pragma unroll
                for (int e = 0; e < 2; ++e)
                {
                    const int k = tile * TW + (2 * q + e) * 32 + lane;
                    if (k >= n)
                        continue;
                    const uint32_t i = order[k];
                    const float gx = G * (e ? ax[q].y : ax[q].x), gy = G * (e ? ay[q].y : ay[q].x);
                    const float gz = G * (e ? az[q].y : az[q].x);
                    if (body_out)
                    {
                        float* o = body_out + static_cast<size_t>(i) * 12 + 8;
                        o[0] = gx;
                        o[1] = gy;
                        o[2] = gz;
                    }
                    else
                        acc[i] = make_float4(gx, gy, gz, 0.f);
                }
        }
        // per-warp totals
        unsigned long long total = inter;
        for (int o = 16; o > 0; o >>= 1)
            total += __shfl_down_sync(0xffffffffu, total, o);
        if (lane == 0)
        {
            atomicAdd(&stats[0], total);
            atomicAdd(&stats[1], static_cast<unsigned long long>(visits));
        }
    }

    // ------------------------------------------------------------------------------------
    // 7b. group walk with interaction lists (walk = NBODY_WALK_GROUP)
    // ------------------------------------------------------------------------------------
    // One list source applied to two targets (negated positions), both taking it: the direct
    // sum's packed interaction, 3 FADD2 + 3 FFMA2 + 2 MUFU.RSQ + 3 FMUL2 + 3 FFMA2.
    template <int LAW>
    __device__ __forceinline__ void apply_list2(const float2 npx, const float2 npy, const float2 npz, const float2 lim,
                                                const float4 s, float2& ax, float2& ay, float2& az)
    {
        const float2 dx = add2(f2(s.x), npx), dy = add2(f2(s.y), npy), dz = add2(f2(s.z), npz);
        float2 r2 = (LAW == NBODY_LAW_SOFTENED) ? fma2(dx, dx, lim) : mul2(dx, dx);
        r2 = fma2(dy, dy, r2);
        r2 = fma2(dz, dz, r2);
        float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
        if (LAW == NBODY_LAW_CUTOFF)
        {
            inv.x = r2.x > lim.x ? inv.x : 0.f;     // physics.h:38-39
            inv.y = r2.y > lim.y ? inv.y : 0.f;
        }
        const float2 inv2 = mul2(inv, inv);
        const float2 mi = mul2(f2(s.w), inv);
        const float2 sc = mul2(mi, inv2);
        ax = fma2(dx, sc, ax);
        ay = fma2(dy, sc, ay);
        az = fma2(dz, sc, az);
    }

    // The reference's opening test (bhtree.cpp:117-125) for a box of targets: the cell is
    // accepted when the nearest point of the box lies beyond its opening distance,
    // |com - p|^2 > size^2 * theta^2. Every target in the box is at least that far from the
    // centre of mass, so each would accept the cell itself.
    __device__ __forceinline__ bool box_accepts(const float4 cm, const float open_r2, const float4 lo, const float4 hi)
    {
        const float dx = fmaxf(fmaxf(lo.x - cm.x, cm.x - hi.x), 0.f);
        const float dy = fmaxf(fmaxf(lo.y - cm.y, cm.y - hi.y), 0.f);
        const float dz = fmaxf(fmaxf(lo.z - cm.z, cm.z - hi.z), 0.f);
        return fmaf(dz, dz, fmaf(dy, dy, dx * dx)) > open_r2;
    }

    // A warp serves 64 Q Morton-consecutive targets (lane l holds targets 64 Q t + 32 h + l,
    // h < 2Q, as Q packed pairs) with one walk of the tree, the interaction-list walk of GPU
    // tree codes (Barnes 1990's grouping; Bonsai, Bedorf et al. 2012): the walk decides each
    // cell once for the whole group and appends the sources it yields -- accepted cells as
    // (com, mass), leaves and the bodies of opened buckets as (x, m) -- to an interaction list
    // in shared memory, which every CAP entries is applied to every target of the group
    // with the direct sum's packed loop: no selection and no per-target test.
    //
    // The acceptance box. The group is split at the NSG - 1 largest jumps of its Morton codes
    // (the smallest common prefixes of neighbours) into runs, each with its own bounding box,
    // and a cell is accepted only when every run's box lies beyond its opening distance;
    // otherwise it is opened for the whole group. One box over the group would be wrong in
    // shape: a run that crosses from one cell of the tree into a distant one (at the end of a
    // top-level octant the curve jumps across the whole system) has a box spanning everything
    // between, which opens every cell there down to its leaves. Accepting per run instead
    // (some runs taking a cell, the others its children) was measured too: half the list then
    // applies to only some targets, and the walk took 54 against 45 ms at 16.8M bodies.
    //
    // The walk tests up to 32 cells at a time: it pops up to four opened parent cells from a
    // stack, and lane l tests child l % 8 of parent l / 8. The stack grows by at most 28
    // parents per tree level (22 levels: 616 < kGroupStack).
    //
    // Each target's sources refine the cells the reference's walk accepts for it alone (a
    // cell opened for the group may be one the target would have accepted), so each target
    // is summed at least as finely as in the reference, over more interactions.
    template <int LAW, int Q, int NSG, int CAP>
    __global__ void __launch_bounds__(kListWarps * 32) traverse_list_kernel(
        const OctNode* __restrict__ nodes, const float4* __restrict__ spm, const float* __restrict__ srad,
        const uint64_t* __restrict__ codes, const uint32_t* __restrict__ order, const int n, const float G,
        const float eps2, float4* __restrict__ acc, float* __restrict__ body_out, unsigned* __restrict__ err,
        unsigned long long* __restrict__ stats)
    {
        constexpr int H = 2 * Q;                    // target slots per lane
        constexpr int TW = 32 * H;                  // targets per group
        static_assert(NSG >= 1 && NSG <= 32, "runs per group");
        __shared__ __align__(16) float4 list_mem[kListWarps][CAP];
        __shared__ int stack_mem[kListWarps][kGroupStack];
        __shared__ __align__(16) float4 box_mem[kListWarps][2 * NSG];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1u;
        float4* list = list_mem[warp];
        int* stk = stack_mem[warp];
        const float4* box = box_mem[warp];
        unsigned long long inter = 0;               // interactions summed by this warp (uniform)
        unsigned iters = 0;

        auto next_tile = [&]() {
            unsigned long long t = 0;
            if (lane == 0)
                t = atomicAdd(&stats[3], 1ull);
            return static_cast<int>(__shfl_sync(0xffffffffu, t, 0));
        };
        for (int tile = next_tile(); static_cast<long long>(tile) * TW < n; tile = next_tile())
        {
            const int t0 = tile * TW;
            const int nvalid = static_cast<int>(min(static_cast<long long>(TW), static_cast<long long>(n) - t0));
            // --- runs: split at the NSG - 1 largest Morton jumps between neighbours ---
            unsigned key[H];    // (common prefix bits << 8 | position); 0xffffffff: no boundary
#pragma unroll
            for (int h = 0; h < H; ++h)
            {
                const int b = 32 * h + lane;        // boundary between positions b - 1 and b
                key[h] = 0xffffffffu;
                if (b > 0 && b < nvalid)
                    key[h] = (static_cast<unsigned>(__clzll(static_cast<long long>(codes[t0 + b - 1] ^ codes[t0 + b])))
                              << 8) | static_cast<unsigned>(b);
            }
            int split[NSG > 1 ? NSG - 1 : 1];
            split[0] = TW;
#pragma unroll
            for (int sidx = 0; sidx < NSG - 1; ++sidx)
            {
                unsigned m = key[0];
#pragma unroll
                for (int h = 1; h < H; ++h)
                    m = min(m, key[h]);
                for (int o = 16; o > 0; o >>= 1)
                    m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
                split[sidx] = m == 0xffffffffu ? TW : static_cast<int>(m & 0xffu);
#pragma unroll
                for (int h = 0; h < H; ++h)
                    if (key[h] == m)
                        key[h] = 0xffffffffu;
            }
            // --- targets and the run boxes ---
            float2 npx[Q], npy[Q], npz[Q], lim[Q], ax[Q], ay[Q], az[Q];
            float4 blo[NSG], bhi[NSG];
#pragma unroll
            for (int g = 0; g < NSG; ++g)
            {
                blo[g] = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
                bhi[g] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
            }
#pragma unroll
            for (int q = 0; q < Q; ++q)
            {
                float v[2][4];
#pragma unroll
                for (int e = 0; e < 2; ++e)
                {
                    const int pos = 32 * (2 * q + e) + lane;
                    const int k = t0 + pos;
                    const bool valid = k < n;
                    int run = 0;
#pragma unroll
                    for (int sidx = 0; sidx < NSG - 1; ++sidx)
                        run += pos >= split[sidx] ? 1 : 0;
                    const float4 pk = spm[valid ? k : n - 1];
#pragma unroll
                    for (int g = 0; g < NSG; ++g)
                        if (valid && run == g)
                        {
                            blo[g] = make_float4(fminf(blo[g].x, pk.x), fminf(blo[g].y, pk.y), fminf(blo[g].z, pk.z), 0.f);
                            bhi[g] = make_float4(fmaxf(bhi[g].x, pk.x), fmaxf(bhi[g].y, pk.y), fmaxf(bhi[g].z, pk.z), 0.f);
                        }
                    v[e][0] = -pk.x;
                    v[e][1] = -pk.y;
                    v[e][2] = -pk.z;
                    if (LAW == NBODY_LAW_CUTOFF)
                    {
                        const float r = srad[valid ? k : n - 1];
                        v[e][3] = r * r;
                    }
                    else
                        v[e][3] = eps2;
                }
                npx[q] = make_float2(v[0][0], v[1][0]);
                npy[q] = make_float2(v[0][1], v[1][1]);
                npz[q] = make_float2(v[0][2], v[1][2]);
                lim[q] = make_float2(v[0][3], v[1][3]);
                ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int g = 0; g < NSG; ++g)
                for (int o = 16; o > 0; o >>= 1)
                {
                    blo[g].x = fminf(blo[g].x, __shfl_xor_sync(0xffffffffu, blo[g].x, o));
                    blo[g].y = fminf(blo[g].y, __shfl_xor_sync(0xffffffffu, blo[g].y, o));
                    blo[g].z = fminf(blo[g].z, __shfl_xor_sync(0xffffffffu, blo[g].z, o));
                    bhi[g].x = fmaxf(bhi[g].x, __shfl_xor_sync(0xffffffffu, bhi[g].x, o));
                    bhi[g].y = fmaxf(bhi[g].y, __shfl_xor_sync(0xffffffffu, bhi[g].y, o));
                    bhi[g].z = fmaxf(bhi[g].z, __shfl_xor_sync(0xffffffffu, bhi[g].z, o));
                }
            __syncwarp();       // the previous group's readers of the boxes are done
            if (lane < 2 * NSG)
            {
                const int g = lane >> 1;
                float4 bv = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int gg = 0; gg < NSG; ++gg)
                    if (gg == g)
                        bv = (lane & 1) ? bhi[gg] : blo[gg];
                box_mem[warp][lane] = bv;
            }
            __syncwarp();

            int ln = 0;     // list entries (warp-uniform)
            // apply the whole list to every target of the group, then empty it
            auto drain = [&]() {
                __syncwarp();
#pragma unroll 2
                for (int e = 0; e < ln; ++e)
                {
                    const float4 s = list[e];
#pragma unroll
                    for (int q = 0; q < Q; ++q)
                        apply_list2<LAW>(npx[q], npy[q], npz[q], lim[q], s, ax[q], ay[q], az[q]);
                }
                inter += static_cast<unsigned long long>(ln) * nvalid;
                ln = 0;
                __syncwarp();
            };
            // append one source per flagged lane, draining first when the list would overflow
            auto append = [&](const bool take, const float4 src) {
                const unsigned m = __ballot_sync(0xffffffffu, take);
                if (ln + __popc(m) > CAP)
                    drain();
                if (take)
                    list[ln + __popc(m & lt)] = src;
                ln += __popc(m);
            };
            // the bodies of an opened bucket (identical codes), 32 at a time
            auto append_range = [&](const int first, const int last) {
                for (int b0 = first; b0 <= last; b0 += 32)
                {
                    const int bi = b0 + lane;
                    float4 sb = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (bi <= last)
                        sb = spm[bi];
                    append(bi <= last && sb.w != 0.f, sb);
                }
            };
            // every run's box lies beyond the cell's opening distance (an empty run's box is
            // inverted, +inf to -inf, and accepts everything)
            auto accepts = [&](const float4 cm, const float open_r2) {
                bool a = true;
#pragma unroll
                for (int g = 0; g < NSG; ++g)
                    a = a && box_accepts(cm, open_r2, box[2 * g], box[2 * g + 1]);
                return a;
            };

            // the root: accepted, a bucket, or the first parent on the stack
            int sp = 0;
            {
                const float4 cm = nodes[0].com_mass;
                const int4 meta = *reinterpret_cast<const int4*>(&nodes[0].open_r2);
                if (cm.w != 0.f)
                {
                    if (accepts(cm, __int_as_float(meta.x)))
                        append(lane == 0, cm);
                    else if (meta.y < 0)
                        append_range(meta.z, meta.w);
                    else
                    {
                        if (lane == 0)
                            stk[0] = 0;
                        sp = 1;
                    }
                }
            }
            __syncwarp();
            // Each cell is pushed at most once per group, so the walk takes at most one
            // round per cell (< n); the bound only trips on a malformed tree.
            int guard = 0;
            const int guard_limit = n + 64;
            while (sp > 0)
            {
                if (++guard > guard_limit)
                {
                    if (lane == 0)
                        atomicOr(err, DEV_ERR_BOUNDS);
                    break;
                }
                ++iters;
                const int k = min(sp, 4);
                const int slot = lane >> 3;
                int c = 0;              // 0: no child (cell 0 is the root, never a child)
                if (slot < k)
                    c = nodes[stk[sp - 1 - slot]].child[lane & 7];
                __syncwarp();           // every parent read before pushes overwrite its slot
                sp -= k;
                bool take = false, push = false, bucket = false;
                float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
                int4 meta = make_int4(0, 0, 0, 0);
                if (c < 0)
                {
                    src = spm[~c];      // a leaf: always applied (bhtree.cpp:115-116)
                    take = src.w != 0.f;
                }
                else if (c > 0)
                {
                    const float4 cm = nodes[c].com_mass;
                    meta = *reinterpret_cast<const int4*>(&nodes[c].open_r2);
                    if (cm.w != 0.f)    // empty cells are skipped (bhtree.cpp:109-113)
                    {
                        if (accepts(cm, __int_as_float(meta.x)))
                        {
                            src = cm;
                            take = true;
                        }
                        else if (meta.y < 0)
                            bucket = true;
                        else
                            push = true;
                    }
                }
                append(take, src);
                const unsigned pm = __ballot_sync(0xffffffffu, push);
                if (push)
                {
                    const int at = sp + __popc(pm & lt);
                    if (at < kGroupStack)
                        stk[at] = c;
                    else
                        atomicOr(err, DEV_ERR_BOUNDS);
                }
                sp = min(kGroupStack, sp + __popc(pm));
                unsigned bm = __ballot_sync(0xffffffffu, bucket);
                while (bm)
                {
                    const int bl = __ffs(bm) - 1;
                    bm &= bm - 1;
                    append_range(__shfl_sync(0xffffffffu, meta.z, bl), __shfl_sync(0xffffffffu, meta.w, bl));
                }
                __syncwarp();
            }
            drain();
#pragma unroll
            for (int q = 0; q < Q; ++q)
#pragma unroll
                for (int e = 0; e < 2; ++e)
                {
                    const int k = t0 + (2 * q + e) * 32 + lane;
                    if (k >= n)
                        continue;
                    const uint32_t i = order[k];
                    const float gx = G * (e ? ax[q].y : ax[q].x), gy = G * (e ? ay[q].y : ay[q].x);
                    const float gz = G * (e ? az[q].y : az[q].x);
                    if (body_out)
                    {
                        float* o = body_out + static_cast<size_t>(i) * 12 + 8;
                        o[0] = gx;
                        o[1] = gy;
                        o[2] = gz;
                    }
                    else
                        acc[i] = make_float4(gx, gy, gz, 0.f);
                }
        }
        if (lane == 0)
        {
            atomicAdd(&stats[0], inter);
            atomicAdd(&stats[1], static_cast<unsigned long long>(iters));
        }
    }

    // ------------------------------------------------------------------------------------
    // host side
    // ------------------------------------------------------------------------------------
    namespace
    {
        template <typename T>
        cudaError_t grow(T** p, const size_t count, cudaStream_t s)
        {
            if (*p)
                cudaFreeAsync(*p, s);
            *p = nullptr;
            return cudaMallocAsync(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T), s);
        }

        int reserve_bh(nbody_cuda* ctx, const size_t n)
        {
            if (!ctx->bh)
                ctx->bh = new BhState();
            BhState& b = *ctx->bh;
            if (!b.box)
            {
                cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&b.box), sizeof(BoxParams), ctx->stream);
                if (e == cudaSuccess)
                    e = cudaMallocAsync(reinterpret_cast<void**>(&b.bbox_part), kBboxBlocks * kBboxVals * sizeof(float),
                                        ctx->stream);
                if (e == cudaSuccess)
                    e = cudaMallocAsync(reinterpret_cast<void**>(&b.stats), kStatsWords * sizeof(unsigned long long), ctx->stream);
                if (e != cudaSuccess)
                    return ctx_cuda_fail(ctx, e, "tree allocation");
            }
            if (n <= b.cap)
                return NBODY_OK;
            if (const int st = before_allocation(ctx))
                return st;
            const size_t cap = std::max(n, b.cap + b.cap / 2);
            const size_t tiles = (cap + kMomTile - 1) / kMomTile;
            // the sort's temporaries; later the cell sums' tile totals and tile prefixes, and
            // after them the scans' temporaries (the tile totals' and the octree compaction's)
            const size_t tb = std::max(sort_temp_bytes(cap),
                                       2 * (tiles + 1) * sizeof(Int64x4)
                                           + std::max(scan_temp_elems(tiles + 1) * sizeof(Int64x4),
                                                      scan_temp_elems(cap) * sizeof(uint32_t)));
            cudaError_t e = cudaSuccess;
            cudaStream_t s = ctx->stream;
            for (int k = 0; k < 2 && e == cudaSuccess; ++k)
            {
                e = grow(&b.keys[k], cap, s);
                if (e == cudaSuccess)
                    e = grow(&b.vals[k], cap, s);
            }
            if (e == cudaSuccess) e = grow(&b.spm, cap, s);
            if (e == cudaSuccess) e = grow(&b.srad, cap, s);
            if (e == cudaSuccess) e = grow(&b.child, cap, s);
            if (e == cudaSuccess) e = grow(&b.range, cap, s);
            if (e == cudaSuccess) e = grow(&b.prefix, cap, s);
            if (e == cudaSuccess) e = grow(&b.octflag, cap, s);
            if (e == cudaSuccess) e = grow(&b.octidx, cap, s);
            if (e == cudaSuccess) e = grow(&b.psum, cap + 1, s);
            if (e == cudaSuccess) e = grow(&b.nodes, cap, s);
            if (e == cudaSuccess)
            {
                if (b.temp)
                    cudaFreeAsync(b.temp, s);
                b.temp = nullptr;
                e = cudaMallocAsync(&b.temp, tb, s);
                b.temp_bytes = tb;
            }
            if (e != cudaSuccess)
            {
                b.cap = 0;
                return ctx_cuda_fail(ctx, e, "tree allocation");
            }
            b.cap = cap;
            return NBODY_OK;
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
    }

    int bh_build(nbody_cuda* ctx, const nbody_step_params* p)
    {
        const size_t n = ctx->count;
        if (const int st = reserve_bh(ctx, n))
            return st;
        BhState& b = *ctx->bh;
        cudaStream_t s = ctx->stream;
        int stride = 1;
        const float4* src = body_src(ctx, &stride);
        const int ni = static_cast<int>(n);
        uint64_t& L = ctx->launches;

        if (const cudaError_t me = cudaMemsetAsync(b.stats, 0, kStatsWords * sizeof(unsigned long long), s))
            return ctx_cuda_fail(ctx, me, "tree statistics");
        // tree_box = 0 is the reference's fixed root box; it needs a positive size
        const bool auto_box = p->tree_box != 0 || !(p->size > 0.f);
        // the bounds pass runs for the fixed box too: the cell sums' scale comes from it
        bbox_partial_kernel<<<kBboxBlocks, 256, 0, s>>>(src, stride, ni, b.bbox_part);
        ++L;
        box_final_kernel<<<1, 256, 0, s>>>(b.bbox_part, kBboxBlocks, ni, auto_box ? 1 : 0, p->size, b.box);
        ++L;
        morton_kernel<<<ceil_div(n, 256 * kMortonItems), 256, 0, s>>>(src, stride, ni, b.box, b.keys[0], b.vals[0]);
        ++L;
        bool in_alt = false;
        cudaError_t e = radix_sort_pairs(b.keys[0], b.vals[0], b.keys[1], b.vals[1], n, kRunShift, 63, b.temp, s, &L,
                                         &in_alt, ctx->dev_error);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "radix sort");
        if (n > 1)
        {
            // runs of equal top bits into order; a run too long for that sorts everything
            // again by all bits, from the current order (its ties are in index order too), and
            // copies the result back, so that the sorted pairs are where the passes left them
            const int cur = in_alt ? 1 : 0;
            unsigned* full = reinterpret_cast<unsigned*>(b.stats + 4);
            run_sort_kernel<<<ceil_div(n, 256), 256, 0, s>>>(b.keys[cur], b.vals[cur], ni, full);
            ++L;
            bool alt2 = false;
            e = radix_sort_pairs(b.keys[cur], b.vals[cur], b.keys[1 - cur], b.vals[1 - cur], n, 0, 63, b.temp, s, &L,
                                 &alt2, ctx->dev_error, full, (63 - kRunShift + 8) / 9);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "radix sort");
            if (alt2)
            {
                copy_back_kernel<<<1024, 256, 0, s>>>(b.keys[1 - cur], b.vals[1 - cur], b.keys[cur], b.vals[cur], ni,
                                                         full);
                ++L;
            }
        }
        const uint64_t* keys = b.keys[in_alt ? 1 : 0];
        const uint32_t* order = b.vals[in_alt ? 1 : 0];
        b.order = order;
        b.codes = keys;
        const unsigned tiles = std::max(1u, ceil_div(n, kMomTile));
        // temporaries: tile totals and their exclusive scan (tiles + 1 each: the entry past
        // the last tile gives the sum of all bodies), then the scans' own
        Int64x4* tile_sum = static_cast<Int64x4*>(b.temp);
        Int64x4* tile_prefix = tile_sum + tiles + 1;
        void* scan_temp = tile_prefix + tiles + 1;
        const bool radius = p->law == NBODY_LAW_CUTOFF;
        gather_sum_kernel<<<tiles, kMomThreads, 0, s>>>(src, stride,
                                                        radius && ctx->layout != NBODY_LAYOUT_AOS ? ctx->vr : nullptr,
                                                        order, ni, b.box, b.spm, radius ? b.srad : nullptr, b.psum,
                                                        tile_sum);
        ++L;
        e = exclusive_scan<Int64x4>(tile_sum, tile_prefix, tiles + 1, static_cast<Int64x4*>(scan_temp), s, &L);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "cell sums");
        if (n < 2)
        {
            b.built = true;
            b.built_n = n;
            ++b.build_id;
            return NBODY_OK;
        }
        const int m = ni - 1;
        {
            // adjacent prefix lengths, key samples and the far nodes' list live in the sort's
            // other key and value buffers, free until the next build
            const int other = in_alt ? 0 : 1;
            uint8_t* dl = reinterpret_cast<uint8_t*>(b.keys[other]);
            // (n rounded up to 8 bytes, then n / 64 + 1 keys: within the buffer's 8 n bytes for n >= 2)
            uint64_t* smp = reinterpret_cast<uint64_t*>(dl + ((n + 7) & ~size_t(7)));
            int* far_list = reinterpret_cast<int*>(b.vals[other]);
            unsigned* far_count = reinterpret_cast<unsigned*>(b.stats + 5);
            adjacent_prefix_kernel<<<ceil_div(m, 256 * 4), 256, 0, s>>>(keys, ni, dl, smp);
            ++L;
            radix_near_kernel<<<ceil_div(m, 256), 256, 0, s>>>(keys, dl, ni, b.child, b.range, b.prefix, b.octflag,
                                                               far_list, far_count, ctx->dev_error);
            ++L;
            radix_far_kernel<<<std::min(ceil_div(m, 256), 2048u), 256, 0, s>>>(keys, dl, smp, ni, far_list, far_count,
                                                                                  b.child, b.range, b.prefix,
                                                                                  b.octflag, ctx->dev_error);
            ++L;
        }
        e = exclusive_scan<uint32_t>(b.octflag, b.octidx, m, static_cast<uint32_t*>(scan_temp), s, &L);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "octree compaction");
        octnode_kernel<<<ceil_div(m, 256 * kOctSpan), 256, 0, s>>>(b.child, b.range, b.prefix, b.octflag, b.octidx,
                                                                    b.psum, tile_prefix, m, b.box, p->theta, b.nodes,
                                                                    ctx->dev_error, b.stats);
        ++L;
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "tree build");
        b.built = true;
        b.built_n = n;
        ++b.build_id;
        return NBODY_OK;
    }

    int bh_accelerate(nbody_cuda* ctx, const nbody_step_params* p)
    {
        const size_t n = ctx->count;
        if (!ctx->bh)
            ctx->bh = new BhState();
        // stage timing: three events on the stream, except while it is captured into a graph
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        bool timed = cudaStreamIsCapturing(ctx->stream, &capture) == cudaSuccess && capture == cudaStreamCaptureStatusNone;
        for (int k = 0; k < 3 && timed; ++k)
            timed = ctx->bh->ev[k] || cudaEventCreate(&ctx->bh->ev[k]) == cudaSuccess;
        ctx->bh->timed = false;
        if (timed)
            cudaEventRecord(ctx->bh->ev[0], ctx->stream);
        if (const int st = bh_build(ctx, p))
            return st;
        BhState& b = *ctx->bh;
        cudaStream_t s = ctx->stream;
        if (timed)
            cudaEventRecord(b.ev[1], s);
        const int ni = static_cast<int>(n);
        float4* acc = ctx->layout == NBODY_LAYOUT_AOS ? nullptr : ctx->acc;
        float* body_out = ctx->layout == NBODY_LAYOUT_AOS ? ctx->bodies : nullptr;
        if (n < 2)
        {
            // a lone body feels nothing (its own leaf is cut off / multiplied by d = 0)
            cudaError_t me = cudaSuccess;
            if (acc)
                me = cudaMemsetAsync(acc, 0, n * sizeof(float4), s);
            else
                for (size_t i = 0; i < n && me == cudaSuccess; ++i)
                    me = cudaMemsetAsync(body_out + i * 12 + 8, 0, 3 * sizeof(float), s);
            return me == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, me, "lone-body acceleration");
        }
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        if (p->walk == NBODY_WALK_GROUP)
        {
            // Group walk: 128 targets per group (4 per lane) while the groups outnumber the
            // resident warps, else 64. NBODY_CUDA_BH_GROUP (64, 128 or 256) overrides; the
            // group size changes which cells each target applies, not the bar they meet.
            const bool soft = p->law == NBODY_LAW_SOFTENED;
            using Walk = void (*)(const OctNode*, const float4*, const float*, const uint64_t*, const uint32_t*, int,
                                  float, float, float4*, float*, unsigned*, unsigned long long*);
            // [group 64, 128, 256][short, long list]
            const Walk fns[3][2] = {
                { soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 1, kRuns, kListShort>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 1, kRuns, kListShort>,
                  soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 1, kRuns, kListLong>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 1, kRuns, kListLong> },
                { soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 2, kRuns, kListShort>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 2, kRuns, kListShort>,
                  soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 2, kRuns, kListLong>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 2, kRuns, kListLong> },
                { soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 4, kRuns, kListShort>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 4, kRuns, kListShort>,
                  soft ? traverse_list_kernel<NBODY_LAW_SOFTENED, 4, kRuns, kListLong>
                       : traverse_list_kernel<NBODY_LAW_CUTOFF, 4, kRuns, kListLong> } };
            auto per_sm = [&](Walk fn) {
                int per = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kListWarps * 32, 0) != cudaSuccess || per < 1)
                    per = 1;
                return per;
            };
            const char* gsel = std::getenv("NBODY_CUDA_BH_GROUP");
            int group = gsel ? std::atoi(gsel) : 0;
            if (group != 64 && group != 128 && group != 256)
                group = static_cast<long long>(ni) >= 128LL * per_sm(fns[1][0]) * sms * kListWarps ? 128 : 64;
            const int gi = group == 256 ? 2 : (group == 128 ? 1 : 0);
            const int groups = (ni + group - 1) / group;
            // the long list once the groups are at least twice the warps it leaves resident
            const bool long_list = groups >= 2LL * per_sm(fns[gi][1]) * sms * kListWarps;
            const Walk fn = fns[gi][long_list ? 1 : 0];
            const int per = per_sm(fn);
            const int grid = std::min((groups + kListWarps - 1) / kListWarps, sms * per);
            fn<<<grid, kListWarps * 32, 0, s>>>(b.nodes, b.spm, b.srad, b.codes, b.order, ni, p->G, p->eps2, acc,
                                                body_out, ctx->dev_error, b.stats);
            ++ctx->launches;
            if (timed)
                b.timed = cudaEventRecord(b.ev[2], s) == cudaSuccess;
            const cudaError_t eg = cudaGetLastError();
            return eg == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, eg, "group tree walk");
        }
        // Targets per warp walk: 128 (traverse_pairs_kernel, 4 per lane) while the tiles
        // outnumber the resident warps, then 64 (2 per lane) while they are at least half of
        // them, then 32 (traverse_kernel): a narrower walk visits more cells but keeps more
        // warps busy. At 262,144 bodies the 64-target walk is 9 % faster than the 128 one.
        // NBODY_CUDA_BH_TARGETS (32, 64, 128 or 256) overrides; all give the same sums.
        const char* tsel = std::getenv("NBODY_CUDA_BH_TARGETS");
        int per_warp = tsel ? std::atoi(tsel) : 0;
        if (!per_warp)
        {
            auto resident_warps = [&](auto fn) {
                int per = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kTravWarps * 32, 0) != cudaSuccess || per < 1)
                    per = 1;
                return static_cast<long long>(per) * sms * kTravWarps;
            };
            const bool soft = p->law == NBODY_LAW_SOFTENED;
            const long long w128 = resident_warps(soft ? traverse_pairs_kernel<NBODY_LAW_SOFTENED, 2>
                                                       : traverse_pairs_kernel<NBODY_LAW_CUTOFF, 2>);
            const long long w64 = resident_warps(soft ? traverse_pairs_kernel<NBODY_LAW_SOFTENED, 1>
                                                      : traverse_pairs_kernel<NBODY_LAW_CUTOFF, 1>);
            const long long nn = static_cast<long long>(ni);
            per_warp = nn >= 128 * w128 ? 128 : (2 * nn >= 64 * w64 ? 64 : 32);
        }
        if (per_warp == 64 || per_warp == 128 || per_warp == 256)
        {
            const bool soft = p->law == NBODY_LAW_SOFTENED;
            using Walk = void (*)(const OctNode*, const float4*, const float*, const uint32_t*, int, float, float,
                                  float4*, float*, unsigned*, unsigned long long*);
            Walk fn;
            int warps = kTravWarps;
            if (per_warp == 256)
            {
                fn = soft ? traverse_pairs_kernel<NBODY_LAW_SOFTENED, 4> : traverse_pairs_kernel<NBODY_LAW_CUTOFF, 4>;
                warps = pair_warps(4);
            }
            else if (per_warp == 128)
                fn = soft ? traverse_pairs_kernel<NBODY_LAW_SOFTENED, 2> : traverse_pairs_kernel<NBODY_LAW_CUTOFF, 2>;
            else
                fn = soft ? traverse_pairs_kernel<NBODY_LAW_SOFTENED, 1> : traverse_pairs_kernel<NBODY_LAW_CUTOFF, 1>;
            // one resident wave of CTAs, each warp drawing tiles until none are left
            int per = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, warps * 32, 0) != cudaSuccess || per < 1)
                per = 1;
            const int tiles2 = (ni + per_warp - 1) / per_warp;
            const int grid2 = std::min((tiles2 + warps - 1) / warps, sms * per);
            fn<<<grid2, warps * 32, 0, s>>>(b.nodes, b.spm, b.srad, b.order, ni, p->G, p->eps2, acc, body_out,
                                             ctx->dev_error, b.stats);
            ++ctx->launches;
            if (timed)
                b.timed = cudaEventRecord(b.ev[2], s) == cudaSuccess;
            const cudaError_t e2 = cudaGetLastError();
            return e2 == cudaSuccess ? NBODY_OK : ctx_cuda_fail(ctx, e2, "tree traversal");
        }
        const int tiles = (ni + 31) / 32;
        const int grid = std::min((tiles + kTravWarps - 1) / kTravWarps, sms * 8);
        if (p->law == NBODY_LAW_SOFTENED)
            traverse_kernel<NBODY_LAW_SOFTENED><<<grid, kTravWarps * 32, 0, s>>>(
                b.nodes, b.spm, b.srad, b.order, ni, p->G, p->eps2, acc, body_out, ctx->dev_error, b.stats);
        else
            traverse_kernel<NBODY_LAW_CUTOFF><<<grid, kTravWarps * 32, 0, s>>>(
                b.nodes, b.spm, b.srad, b.order, ni, p->G, p->eps2, acc, body_out, ctx->dev_error, b.stats);
        ++ctx->launches;
        if (timed)
            b.timed = cudaEventRecord(b.ev[2], s) == cudaSuccess;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "tree traversal");
        return NBODY_OK;
    }

    int bh_stage_ms(nbody_cuda* ctx, float ms[2])
    {
        if (!ctx->bh || !ctx->bh->timed)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "no timed Barnes-Hut accelerate");
        BhState& b = *ctx->bh;
        cudaError_t e = cudaEventSynchronize(b.ev[2]);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms[0], b.ev[0], b.ev[1]);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms[1], b.ev[1], b.ev[2]);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "stage timing");
        return check_device_error(ctx);
    }

    void release_bh(nbody_cuda* ctx)
    {
        if (!ctx->bh)
            return;
        BhState& b = *ctx->bh;
        for (int k = 0; k < 2; ++k)
        {
            cudaFree(b.keys[k]);
            cudaFree(b.vals[k]);
        }
        void* ptrs[] = { b.spm, b.srad, b.child, b.range, b.prefix, b.octflag, b.octidx, b.psum,
                         b.nodes, b.temp, b.box, b.bbox_part, b.stats };
        for (void* q : ptrs)
            cudaFree(q);
        for (cudaEvent_t ev : b.ev)
            if (ev)
                cudaEventDestroy(ev);
        delete ctx->bh;
        ctx->bh = nullptr;
    }

    int bh_stats(nbody_cuda* ctx, unsigned long long out[3])
    {
        if (!ctx->bh || !ctx->bh->stats)
        {
            out[0] = out[1] = out[2] = 0;
            return NBODY_OK;
        }
        const cudaError_t e = cudaMemcpyAsync(out, ctx->bh->stats, 3 * sizeof(unsigned long long),
                                              cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "tree statistics readback");
        return check_device_error(ctx);
    }

    uint64_t bh_build_id(const nbody_cuda* ctx)
    {
        return (ctx->bh && ctx->bh->built) ? ctx->bh->build_id : 0;
    }

    int bh_download(nbody_cuda* ctx, TreeSnapshot* out)
    {
        out->n = 0;
        out->cells.clear();
        out->codes.clear();
        out->bodies.clear();
        if (!ctx->bh || !ctx->bh->built)
            return ctx_fail(ctx, NBODY_ERR_INVALID, "no Barnes-Hut tree has been built");
        BhState& b = *ctx->bh;
        const size_t n = b.built_n;
        out->n = n;
        out->build_id = b.build_id;
        cudaStream_t s = ctx->stream;
        out->codes.resize(n);
        out->bodies.resize(n);
        unsigned long long st[3] = { 0, 0, 0 };
        cudaError_t e = cudaMemcpyAsync(out->codes.data(), b.codes, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out->bodies.data(), b.spm, n * sizeof(float4), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&out->box, b.box, sizeof(BoxParams), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(st, b.stats, sizeof st, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "tree readback");
        const size_t cells = n >= 2 ? static_cast<size_t>(st[2]) : 0;
        out->cells.resize(cells);
        if (cells)
        {
            e = cudaMemcpyAsync(out->cells.data(), b.nodes, cells * sizeof(OctNode), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess)
                return ctx_cuda_fail(ctx, e, "tree readback");
        }
        return check_device_error(ctx);
    }

    int bh_morton(nbody_cuda* ctx, const nbody_step_params* p, uint64_t* codes, uint32_t* order, double box[4])
    {
        if (!ctx->count)
            return NBODY_OK;
        if (const int st = bh_build(ctx, p))
            return st;
        BhState& b = *ctx->bh;
        const size_t n = ctx->count;
        cudaError_t e = cudaSuccess;
        if (codes)
            e = cudaMemcpyAsync(codes, b.codes, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess && order)
            e = cudaMemcpyAsync(order, b.order, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
        BoxParams hb;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&hb, b.box, sizeof hb, cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "Morton readback");
        if (const int st = check_device_error(ctx))
            return st;
        if (box)
        {
            box[0] = hb.lo[0];
            box[1] = hb.lo[1];
            box[2] = hb.lo[2];
            box[3] = hb.edge;
        }
        return NBODY_OK;
    }
}
