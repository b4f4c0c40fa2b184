// LSD radix sort of (uint64 key, uint32 value) pairs, 8-bit digits, stable.
//
// One pass per digit, three steps:
//   1. digit_count: each CTA histograms the digits of its 4096-key tile into
//      counts[digit * tiles + tile] (digit-major, so one exclusive scan of the whole
//      array gives every (digit, tile) its global output offset);
//   2. exclusive scan of counts (scan.cu);
//   3. digit_scatter: each CTA re-reads its tile and writes every pair to
//      offset[digit][tile] + its stable rank among equal digits in the tile.
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
        constexpr int kDigits = 256;
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
            const unsigned d = ok ? static_cast<unsigned>((keys[i] >> shift) & 0xffu) : 0x100u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            if (ok && lane == __ffs(peers) - 1)
                atomicAdd(&hist[d], static_cast<uint32_t>(__popc(peers)));
        }
        __syncthreads();
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
            counts[static_cast<size_t>(d) * tiles + blockIdx.x] = hist[d];
    }

    __global__ void __launch_bounds__(kThreads) digit_scatter_kernel(
        const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint64_t* __restrict__ keys_out,
        uint32_t* __restrict__ vals_out, const int n, const int shift, const int tiles,
        const uint32_t* __restrict__ offsets)
    {
        __shared__ uint32_t warp_cnt[kWarps][kDigits];
        __shared__ uint32_t tile_off[kDigits];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int d = threadIdx.x; d < kWarps * kDigits; d += kThreads)
            (&warp_cnt[0][0])[d] = 0;
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
            tile_off[d] = offsets[static_cast<size_t>(d) * tiles + blockIdx.x];
        __syncthreads();

        const int base = blockIdx.x * kTile + warp * (kTile / kWarps);
        const unsigned lt = (1u << lane) - 1u;
        uint64_t k_reg[kRounds];
        uint32_t v_reg[kRounds];
        uint32_t rank[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; ++r)
        {
            const int i = base + r * 32 + lane;
            const bool ok = i < n;
            k_reg[r] = ok ? keys[i] : ~0ull;
            v_reg[r] = ok ? vals[i] : 0u;
            // out-of-range lanes take a digit value no real key shares in this warp's
            // counters: they are matched among themselves and never written
            const unsigned d = ok ? static_cast<unsigned>((k_reg[r] >> shift) & 0xffu) : 0x100u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const int leader = __ffs(peers) - 1;
            uint32_t before = 0;
            if (lane == leader && ok)
            {
                before = warp_cnt[warp][d];
                warp_cnt[warp][d] = before + __popc(peers);
            }
            before = __shfl_sync(0xffffffffu, before, leader);
            rank[r] = before + __popc(peers & lt);
        }
        __syncthreads();
        // exclusive scan over warps, per digit: warp_cnt[w][d] becomes the count of digit d
        // in warps before w
        for (int d = threadIdx.x; d < kDigits; d += kThreads)
        {
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w)
            {
                const uint32_t c = warp_cnt[w][d];
                warp_cnt[w][d] = run;
                run += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kRounds; ++r)
        {
            const int i = base + r * 32 + lane;
            if (i >= n)
                continue;
            const unsigned d = static_cast<unsigned>((k_reg[r] >> shift) & 0xffu);
            const uint32_t pos = tile_off[d] + warp_cnt[warp][d] + rank[r];
            keys_out[pos] = k_reg[r];
            vals_out[pos] = v_reg[r];
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
        const int tiles = static_cast<int>((n + kTile - 1) / kTile);
        const size_t cnt = static_cast<size_t>(tiles) * kDigits;
        uint32_t* counts = static_cast<uint32_t*>(temp);
        uint32_t* offsets = counts + cnt;
        uint32_t* scan_tmp = offsets + cnt;
        uint64_t* kin = keys;
        uint32_t* vin = vals;
        uint64_t* kout = keys_alt;
        uint32_t* vout = vals_alt;
        for (int shift = begin_bit; shift < end_bit; shift += 8)
        {
            digit_count_kernel<<<tiles, kThreads, 0, stream>>>(kin, static_cast<int>(n), shift, tiles, counts);
            ++*launches;
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess)
                return e;
            e = exclusive_scan<uint32_t>(counts, offsets, cnt, scan_tmp, stream, launches);
            if (e != cudaSuccess)
                return e;
            digit_scatter_kernel<<<tiles, kThreads, 0, stream>>>(kin, vin, kout, vout, static_cast<int>(n), shift,
                                                                  tiles, offsets);
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
