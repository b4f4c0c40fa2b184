// LSD radix sort of (uint64 key, uint32 value) pairs, 9-bit digits, stable.
//
// Seven passes cover a 63-bit Morton code exactly. One pass, three steps:
//   1. digit_count: each CTA histograms the digits of its 4096-key tile into
//      counts[digit * tiles + tile] (digit-major, so one exclusive scan of the whole
//      array gives every (digit, tile) its global output offset);
//   2. exclusive scan of counts (scan.cu);
//   3. digit_scatter: each CTA re-reads its tile, ranks every key stably among the tile's
//      equal digits, stages the tile in shared memory in digit order, and writes it out
//      so that each digit's run of keys lands contiguously (coalesced stores).
// Stability: warp w of a CTA owns the contiguous slice [w*512, (w+1)*512) of the tile and
// walks it in 16 rounds of 32 consecutive keys; a key's rank is (equal digits in earlier
// warps) + (equal digits in earlier rounds of its warp) + (equal digits on lower lanes of
// its round, from __match_any_sync). Equal keys therefore keep their input order, and a
// sort of (code, index) pairs starting from index order yields the order by (code, index).
#include "common.cuh"
#include "scan.cuh"
#include "sort.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kThreads = 256;
        constexpr int kWarps = kThreads / 32;
        constexpr int kRounds = 16;
        constexpr int kTile = kThreads * kRounds;     // 4096 keys per CTA
        constexpr int kBits = 9;
        constexpr int kDigits = 1 << kBits;
        constexpr unsigned kMask = kDigits - 1;

        // dynamic shared memory of the scatter: per-warp counters, digit starts within the
        // tile, global offsets, and the staged keys and values
        constexpr size_t kScatterSmem = sizeof(uint32_t) * (kWarps * kDigits + 2 * kDigits)
                                        + sizeof(uint64_t) * kTile + sizeof(uint32_t) * kTile;
    }

    __global__ void __launch_bounds__(kThreads) digit_count_kernel(const uint64_t* __restrict__ keys, const int n,
                                                                   const int shift, const int tiles,
                                                                   uint32_t* __restrict__ counts)
    {
        __shared__ uint32_t hist[kDigits];
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
            hist[d] = 0;
        __syncthreads();
        // Warp-aggregated: one shared atomic per distinct digit per 32 keys (the top digits
        // of Morton codes are often all equal, which would serialise per-key atomics).
        const int base = blockIdx.x * kTile;
        const int lane = threadIdx.x & 31;
        for (int k = threadIdx.x; k < kTile; k += kThreads)
        {
            const int i = base + k;
            const bool ok = i < n;
            const unsigned d = ok ? static_cast<unsigned>((keys[i] >> shift) & kMask) : static_cast<unsigned>(kDigits);
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            if (ok && lane == __ffs(peers) - 1)
                atomicAdd(&hist[d], static_cast<uint32_t>(__popc(peers)));
        }
        __syncthreads();
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
            counts[static_cast<size_t>(d) * tiles + blockIdx.x] = hist[d];
    }

    __global__ void __launch_bounds__(kThreads, 2) digit_scatter_kernel(
        const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint64_t* __restrict__ keys_out,
        uint32_t* __restrict__ vals_out, const int n, const int shift, const int tiles,
        const uint32_t* __restrict__ offsets)
    {
        extern __shared__ __align__(16) unsigned char smem[];
        uint64_t* stage_k = reinterpret_cast<uint64_t*>(smem);                     // kTile
        uint32_t* stage_v = reinterpret_cast<uint32_t*>(stage_k + kTile);          // kTile
        uint32_t* warp_cnt = stage_v + kTile;                                      // kWarps * kDigits
        uint32_t* digit_start = warp_cnt + kWarps * kDigits;                       // kDigits
        uint32_t* tile_off = digit_start + kDigits;                                // kDigits

        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int d = threadIdx.x; d < kWarps * kDigits; d += kThreads)
            warp_cnt[d] = 0;
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
            tile_off[d] = offsets[static_cast<size_t>(d) * tiles + blockIdx.x];
        __syncthreads();

        const int tile_base = blockIdx.x * kTile;
        const int tile_n = min(kTile, n - tile_base);
        const int base = tile_base + warp * (kTile / kWarps);
        const unsigned lt = (1u << lane) - 1u;
        // only the ranks stay in registers; keys and values are read again (from L1/L2)
        // when the tile is staged, which keeps the kernel at two CTAs per SM
        uint32_t rank[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; ++r)
        {
            const int i = base + r * 32 + lane;
            const bool ok = i < n;
            // out-of-range lanes take a digit value no real key has; they are matched among
            // themselves, counted nowhere and never written
            const unsigned d = ok ? static_cast<unsigned>((keys[i] >> shift) & kMask) : static_cast<unsigned>(kDigits);
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const int leader = __ffs(peers) - 1;
            uint32_t before = 0;
            if (lane == leader && ok)
            {
                before = warp_cnt[warp * kDigits + d];
                warp_cnt[warp * kDigits + d] = before + __popc(peers);
            }
            before = __shfl_sync(0xffffffffu, before, leader);
            rank[r] = before + __popc(peers & lt);
        }
        __syncthreads();
        // Thread t owns the consecutive digits kPer*t ..: exclusive scan over warps per digit
        // (warp_cnt becomes the count in earlier warps) and the digit's total in the tile.
        constexpr int kPer = kDigits / kThreads;
        uint32_t total[kPer];
        uint32_t mine = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q)
        {
            const int d = threadIdx.x * kPer + q;
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w)
            {
                const uint32_t c = warp_cnt[w * kDigits + d];
                warp_cnt[w * kDigits + d] = run;
                run += c;
            }
            total[q] = run;
            mine += run;
        }
        // block-wide exclusive scan of the per-thread totals -> where each digit's run starts
        {
            __shared__ uint32_t warp_sum[kWarps];
            uint32_t incl = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += v;
            }
            if (lane == 31)
                warp_sum[warp] = incl;
            __syncthreads();
            uint32_t before = 0;
            for (int w = 0; w < warp; ++w)
                before += warp_sum[w];
            uint32_t start = before + incl - mine;
#pragma unroll
            for (int q = 0; q < kPer; ++q)
            {
                digit_start[threadIdx.x * kPer + q] = start;
                start += total[q];
            }
        }
        __syncthreads();
        // stage the tile in digit order
#pragma unroll
        for (int r = 0; r < kRounds; ++r)
        {
            const int i = base + r * 32 + lane;
            if (i >= n)
                continue;
            const uint64_t key = keys[i];
            const unsigned d = static_cast<unsigned>((key >> shift) & kMask);
            const uint32_t pos = digit_start[d] + warp_cnt[warp * kDigits + d] + rank[r];
            stage_k[pos] = key;
            stage_v[pos] = vals[i];
        }
        __syncthreads();
        // write out in staged order: consecutive threads take consecutive staged keys, which
        // within a digit go to consecutive global positions
        for (int s = threadIdx.x; s < tile_n; s += kThreads)
        {
            const uint64_t key = stage_k[s];
            const unsigned d = static_cast<unsigned>((key >> shift) & kMask);
            const uint32_t pos = tile_off[d] + (static_cast<uint32_t>(s) - digit_start[d]);
            keys_out[pos] = key;
            vals_out[pos] = stage_v[s];
        }
    }

    size_t sort_temp_bytes(const size_t n)
    {
        const size_t tiles = (n + kTile - 1) / kTile;
        const size_t cnt = tiles * kDigits;
        return 2 * cnt * sizeof(uint32_t) + scan_temp_elems(cnt) * sizeof(uint32_t) + 256;
    }

    cudaError_t radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt,
                                 const size_t n, const int begin_bit, const int end_bit, void* temp,
                                 cudaStream_t stream, uint64_t* launches, bool* in_alt)
    {
        *in_alt = false;
        if (n <= 1)
            return cudaSuccess;
        static const cudaError_t attr = cudaFuncSetAttribute(
            digit_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kScatterSmem));
        if (attr != cudaSuccess)
            return attr;
        const int tiles = static_cast<int>((n + kTile - 1) / kTile);
        const size_t cnt = static_cast<size_t>(tiles) * kDigits;
        uint32_t* counts = static_cast<uint32_t*>(temp);
        uint32_t* offsets = counts + cnt;
        uint32_t* scan_tmp = offsets + cnt;
        uint64_t* kin = keys;
        uint32_t* vin = vals;
        uint64_t* kout = keys_alt;
        uint32_t* vout = vals_alt;
        for (int shift = begin_bit; shift < end_bit; shift += kBits)
        {
            digit_count_kernel<<<tiles, kThreads, 0, stream>>>(kin, static_cast<int>(n), shift, tiles, counts);
            ++*launches;
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess)
                return e;
            e = exclusive_scan<uint32_t>(counts, offsets, cnt, scan_tmp, stream, launches);
            if (e != cudaSuccess)
                return e;
            digit_scatter_kernel<<<tiles, kThreads, kScatterSmem, stream>>>(kin, vin, kout, vout, static_cast<int>(n),
                                                                             shift, tiles, offsets);
            ++*launches;
            e = cudaGetLastError();
            if (e != cudaSuccess)
                return e;
            std::swap(kin, kout);
            std::swap(vin, vout);
            *in_alt = !*in_alt;
        }
        return cudaSuccess;
    }
}
