// LSD radix sort of (uint64 key, uint32 value) pairs, 9-bit digits, stable, one kernel per
// digit pass (a onesweep-style sort: Adinets & Merrill 2022).
//
// Seven passes cover a 63-bit Morton code exactly.
//   0. digit_hist: one read of the keys histograms the digits of every pass at once (a
//      key's digits do not depend on the order of the keys), into ghist[pass][digit].
//   1. digit_pass (once per pass): a CTA takes the next 4096-key tile in launch order (an
//      atomic ticket), ranks its keys stably, publishes its per-digit counts, stages the
//      tile in shared memory in digit order, and then finds how many keys of each digit
//      the earlier tiles hold by decoupled look-back over their published counts (staging
//      first gives those tiles time to publish). The tile is written out so that each
//      digit's run lands contiguously (coalesced stores).
// The look-back only waits on tiles whose tickets were taken earlier, by CTAs that are
// already running and that publish their counts before they wait themselves, so the wait
// always ends; it is still bounded in time, and a wait that gives up records
// DEV_ERR_TIMEOUT. Counts are exact integers, so the result does not depend on timing.
// Stability: warp w of a CTA owns the contiguous slice [w*256, (w+1)*256) of the tile and
// walks it in 8 rounds of 32 consecutive keys; a key's rank is (equal digits in earlier
// warps) + (equal digits in earlier rounds of its warp) + (equal digits on lower lanes of
// its round, from __match_any_sync). A round's per-warp count (16 bits, two to a word) is
// taken and advanced by one shared-memory atomic of the round's leader lane; a warp's
// atomics complete in program order, so rounds count in order. Equal keys therefore keep their input order, and a
// sort of (code, index) pairs starting from index order yields the order by (code, index).
#include <algorithm>

#include "common.cuh"
#include "sort.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kThreads = 512;
        constexpr int kWarps = kThreads / 32;
        constexpr int kRounds = 8;
        constexpr int kTile = kThreads * kRounds;     // 4096 keys per CTA
        constexpr int kBits = 9;
        constexpr int kDigits = 1 << kBits;
        constexpr unsigned kMask = kDigits - 1;
        constexpr int kPer = kDigits / kThreads;      // digits per thread in the per-digit steps
        constexpr int kMaxPasses = 16;      // over the calls that share one set of temporaries
        constexpr int kHistThreads = 1024;

        // A tile's published count for one digit: flag in bits 62-63, the pass's epoch
        // (pass + 1) in bits 32-61, the count in bits 0-31. A word from an earlier pass (or
        // the zeroed array) has another epoch and reads as not yet published.
        constexpr uint64_t kFlagAggregate = 1ull << 62;    // this tile's own count
        constexpr uint64_t kFlagInclusive = 2ull << 62;    // count of this and all earlier tiles

        // dynamic shared memory of a pass: staged keys and values, per-warp 16-bit counters,
        // digit starts within the tile and global digit bases (68 KB: three CTAs per SM)
        constexpr size_t kPassSmem = sizeof(uint64_t) * kTile + sizeof(uint32_t) * kTile
                                     + sizeof(uint16_t) * kWarps * kDigits + sizeof(uint32_t) * 2 * kDigits;

        struct TempLayout
        {
            uint32_t* tickets;      // kMaxPasses tile tickets
            uint32_t* ghist;        // kMaxPasses x kDigits global digit counts
            uint64_t* status;       // tiles x kDigits published counts
            size_t zero_bytes;      // everything above is zeroed before a sort
        };

        constexpr size_t kGhistOffset = 256;
        constexpr size_t kStatusOffset = kGhistOffset + sizeof(uint32_t) * kMaxPasses * kDigits;

        size_t zero_bytes(const size_t tiles) { return kStatusOffset + sizeof(uint64_t) * tiles * kDigits; }

        TempLayout layout(void* temp, const size_t tiles)
        {
            TempLayout t;
            unsigned char* p = static_cast<unsigned char*>(temp);
            t.tickets = reinterpret_cast<uint32_t*>(p);
            t.ghist = reinterpret_cast<uint32_t*>(p + kGhistOffset);
            t.status = reinterpret_cast<uint64_t*>(p + kStatusOffset);
            t.zero_bytes = zero_bytes(tiles);
            return t;
        }
    }

    // Histograms of the digits of all passes, in one read of the keys.
    __global__ void __launch_bounds__(kHistThreads) digit_hist_kernel(const uint64_t* __restrict__ keys, const int n,
                                                                      const int shift0, const int passes,
                                                                      uint32_t* __restrict__ ghist,
                                                                      const unsigned* __restrict__ run_if)
    {
        if (run_if && !*run_if)
            return;
        __shared__ uint32_t hist[kMaxPasses * kDigits];
        for (int d = threadIdx.x; d < passes * kDigits; d += kHistThreads)
            hist[d] = 0;
        __syncthreads();
        const int stride = gridDim.x * kHistThreads;
        int i = blockIdx.x * kHistThreads + threadIdx.x;
        // four keys in flight per thread
        for (; static_cast<long long>(i) + 3 * stride < n; i += 4 * stride)
        {
            uint64_t k[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                k[u] = keys[i + u * stride];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                for (int p = 0; p < passes; ++p)
                    atomicAdd(&hist[p * kDigits + static_cast<int>((k[u] >> (shift0 + p * kBits)) & kMask)], 1u);
        }
        for (; i < n; i += stride)
        {
            const uint64_t k = keys[i];
            for (int p = 0; p < passes; ++p)
                atomicAdd(&hist[p * kDigits + static_cast<int>((k >> (shift0 + p * kBits)) & kMask)], 1u);
        }
        __syncthreads();
        for (int d = threadIdx.x; d < passes * kDigits; d += kHistThreads)
            if (hist[d])
                atomicAdd(&ghist[d], hist[d]);
    }

    __device__ __forceinline__ uint64_t load_relaxed(const uint64_t* p)
    {
        uint64_t v;
        asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
        return v;
    }

    __device__ __forceinline__ void store_relaxed(uint64_t* p, const uint64_t v)
    {
        asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
    }

    // Exclusive block-wide scan of kPer consecutive values per thread (the thread's digits).
    __device__ __forceinline__ void block_exclusive(const uint32_t (&v)[kPer], uint32_t (&out)[kPer],
                                                    uint32_t* __restrict__ warp_sum)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t mine = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q)
            mine += v[q];
        uint32_t incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        if (lane == 31)
            warp_sum[warp] = incl;
        __syncthreads();
        uint32_t start = incl - mine;
        for (int w = 0; w < warp; ++w)
            start += warp_sum[w];
#pragma unroll
        for (int q = 0; q < kPer; ++q)
        {
            out[q] = start;
            start += v[q];
        }
    }

    // PERSIST: a CTA takes tiles until none is left (launched with one CTA per resident slot);
    // otherwise one tile per CTA (launched with one CTA per tile)
    template <bool PERSIST>
    __global__ void __launch_bounds__(kThreads, 3) digit_pass_kernel(
        const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint64_t* __restrict__ keys_out,
        uint32_t* __restrict__ vals_out, const int n, const int shift, const int pass,
        const uint32_t* __restrict__ ghist, uint64_t* __restrict__ status, uint32_t* __restrict__ ticket,
        unsigned* __restrict__ err, const unsigned* __restrict__ run_if)
    {
        if (run_if && !*run_if)
            return;
        extern __shared__ __align__(16) unsigned char smem[];
        uint64_t* stage_k = reinterpret_cast<uint64_t*>(smem);                     // kTile
        uint32_t* stage_v = reinterpret_cast<uint32_t*>(stage_k + kTile);          // kTile
        uint32_t* warp_cnt2 = stage_v + kTile;                                     // kWarps * kDigits / 2
        uint16_t* warp_cnt = reinterpret_cast<uint16_t*>(warp_cnt2);               // kWarps * kDigits
        uint32_t* digit_start = warp_cnt2 + kWarps * kDigits / 2;                  // kDigits
        uint32_t* gbase = digit_start + kDigits;                                   // kDigits
        __shared__ uint32_t warp_sum[2][kWarps];
        __shared__ int tile_s;

        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int tiles = (n + kTile - 1) / kTile;
        for (;;)
        {
            if (threadIdx.x == 0)
                tile_s = static_cast<int>(atomicAdd(ticket, 1u));
            for (int d = threadIdx.x; d < kWarps * kDigits / 2; d += kThreads)
                warp_cnt2[d] = 0;
            __syncthreads();
            const int tile = tile_s;
            if (tile >= tiles)
                break;
            const int tile_base = tile * kTile;
            const int tile_n = min(kTile, n - tile_base);
            const int base = tile_base + warp * (kTile / kWarps);
            const unsigned lt = (1u << lane) - 1u;

            // load and rank (out-of-range lanes take digit kDigits, which no key has: they are
            // matched among themselves, counted nowhere and never written)
            uint64_t key[kRounds];
            uint32_t rank[kRounds];
#pragma unroll
            for (int r = 0; r < kRounds; ++r)
            {
                const int i = base + r * 32 + lane;
                key[r] = i < n ? keys[i] : 0ull;
            }
#pragma unroll
            for (int r = 0; r < kRounds; ++r)
            {
                const bool ok = base + r * 32 + lane < n;
                const unsigned d = ok ? static_cast<unsigned>((key[r] >> shift) & kMask) : static_cast<unsigned>(kDigits);
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                const int leader = __ffs(peers) - 1;
                uint32_t before = 0;
                if (lane == leader && ok)
                {
                    // counter warp * kDigits + d is the (d & 1) half of word (warp * kDigits + d) / 2
                    const unsigned half = (d & 1u) * 16u;
                    const uint32_t old = atomicAdd(&warp_cnt2[(warp * kDigits + static_cast<int>(d)) >> 1],
                                                   static_cast<uint32_t>(__popc(peers)) << half);
                    before = (old >> half) & 0xffffu;
                }
                rank[r] = __shfl_sync(0xffffffffu, before, leader) + __popc(peers & lt);
            }
            __syncthreads();

            // per digit: the count in earlier warps (warp_cnt becomes exclusive over warps) and
            // the tile's total
            uint32_t total[kPer];
#pragma unroll
            for (int q = 0; q < kPer; ++q)
            {
                const int d = threadIdx.x * kPer + q;
                uint32_t run = 0;
#pragma unroll
                for (int w = 0; w < kWarps; ++w)
                {
                    const uint32_t c = warp_cnt[w * kDigits + d];
                    warp_cnt[w * kDigits + d] = static_cast<uint16_t>(run);    // < kTile
                    run += c;
                }
                total[q] = run;
            }
            // publish this tile's counts at once: later tiles may already be waiting for them
            const uint64_t epoch = static_cast<uint64_t>(pass + 1) << 32;
#pragma unroll
            for (int q = 0; q < kPer; ++q)
            {
                const int d = threadIdx.x * kPer + q;
                store_relaxed(&status[static_cast<size_t>(tile) * kDigits + d],
                              (tile == 0 ? kFlagInclusive : kFlagAggregate) | epoch | total[q]);
            }
            // where each digit starts within the tile, and where it starts in the output
            {
                uint32_t start[kPer], gcount[kPer], gstart[kPer];
                block_exclusive(total, start, warp_sum[0]);
#pragma unroll
                for (int q = 0; q < kPer; ++q)
                    gcount[q] = ghist[threadIdx.x * kPer + q];
                block_exclusive(gcount, gstart, warp_sum[1]);
#pragma unroll
                for (int q = 0; q < kPer; ++q)
                {
                    digit_start[threadIdx.x * kPer + q] = start[q];
                    gbase[threadIdx.x * kPer + q] = gstart[q];
                }
            }
            // stage the tile in digit order: it needs only the tile's own counts, and done
            // before the look-back it gives the earlier tiles time to publish theirs
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kRounds; ++r)
            {
                const int i = base + r * 32 + lane;
                if (i >= n)
                    continue;
                const unsigned d = static_cast<unsigned>((key[r] >> shift) & kMask);
                const uint32_t pos = digit_start[d] + warp_cnt[warp * kDigits + d] + rank[r];
                stage_k[pos] = key[r];
                stage_v[pos] = vals[i];
            }
            // decoupled look-back: sum the earlier tiles' counts of each digit, four tiles per
            // step, back to the nearest tile that has published an inclusive count
            if (tile > 0)
            {
#pragma unroll
                for (int q = 0; q < kPer; ++q)
                {
                    const int d = threadIdx.x * kPer + q;
                    uint32_t before = 0;
                    int j = tile - 1;
                    uint64_t t0 = 0;
                    while (j >= 0)
                    {
                        uint64_t w[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u)
                            w[u] = j - u >= 0 ? load_relaxed(&status[static_cast<size_t>(j - u) * kDigits + d]) : 0ull;
                        // take the words in order while they are published aggregates; stop at
                        // an inclusive one, or wait where one is not published yet
                        int u = 0;
                        bool done = false;
                        for (; u < 4 && j - u >= 0; ++u)
                        {
                            if ((w[u] & ~(3ull << 62)) >> 32 != static_cast<uint64_t>(pass + 1) || !(w[u] >> 62))
                                break;
                            before += static_cast<uint32_t>(w[u]);
                            if ((w[u] >> 62) == 2)
                            {
                                done = true;
                                break;
                            }
                        }
                        if (done)
                            break;
                        j -= u;
                        if (j >= 0 && u == 0)
                        {
                            // tile j has not published yet: it is running and will
                            if (!t0)
                                t0 = globaltimer();
                            else if (globaltimer() - t0 > kWaitLimitNs)
                            {
                                atomicOr(err, DEV_ERR_TIMEOUT);
                                break;
                            }
                            __nanosleep(100);
                        }
                    }
                    store_relaxed(&status[static_cast<size_t>(tile) * kDigits + d],
                                  kFlagInclusive | epoch | (before + total[q]));
                    gbase[d] += before;
                }
            }
            __syncthreads();

            // write out in staged order: consecutive threads take consecutive staged keys, which
            // within a digit go to consecutive output positions
            for (int s = threadIdx.x; s < tile_n; s += kThreads)
            {
                const uint64_t k = stage_k[s];
                const unsigned d = static_cast<unsigned>((k >> shift) & kMask);
                const uint32_t pos = gbase[d] + (static_cast<uint32_t>(s) - digit_start[d]);
                if (pos < static_cast<uint32_t>(n))     // always, unless a look-back wait gave up
                {
                    keys_out[pos] = k;
                    vals_out[pos] = stage_v[s];
                }
                else
                    atomicOr(err, DEV_ERR_BOUNDS);
            }
            if (!PERSIST)
                break;
            __syncthreads();        // shared memory is the next tile's
        }
    }

    size_t sort_temp_bytes(const size_t n)
    {
        const size_t tiles = (n + kTile - 1) / kTile;
        return zero_bytes(tiles) + 256;
    }

    cudaError_t radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt,
                                 const size_t n, const int begin_bit, const int end_bit, void* temp,
                                 cudaStream_t stream, uint64_t* launches, bool* in_alt, unsigned* err,
                                 const unsigned* run_if, const int pass_base)
    {
        *in_alt = false;
        if (n <= 1)
            return cudaSuccess;
        if (n > 0x7fffffffu)
            return cudaErrorInvalidValue;
        const int passes = (end_bit - begin_bit + kBits - 1) / kBits;
        if (passes < 1 || pass_base < 0 || pass_base + passes > kMaxPasses)
            return cudaErrorInvalidValue;
        static const cudaError_t attr = [] {
            const cudaError_t a = cudaFuncSetAttribute(digit_pass_kernel<false>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(kPassSmem));
            return a != cudaSuccess ? a
                                    : cudaFuncSetAttribute(digit_pass_kernel<true>,
                                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                           static_cast<int>(kPassSmem));
        }();
        if (attr != cudaSuccess)
            return attr;
        const int tiles = static_cast<int>((n + kTile - 1) / kTile);
        const TempLayout t = layout(temp, static_cast<size_t>(tiles));
        // a call that may do nothing (run_if) launches persistent passes, one CTA per
        // resident slot, so that a pass with nothing to do costs few CTAs; otherwise one CTA
        // per tile
        static const int per_sm = [] {
            int b = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, digit_pass_kernel<true>, kThreads, kPassSmem);
            return std::max(1, b);
        }();
        // the first call zeroes the tickets, histograms and published counts of every pass;
        // a later call's passes have their own tickets and histograms, and their counts carry
        // other epochs
        cudaError_t e = pass_base == 0 ? cudaMemsetAsync(temp, 0, t.zero_bytes, stream) : cudaSuccess;
        if (e != cudaSuccess)
            return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int hist_grid = std::max(1, std::min((static_cast<int>(n) + kHistThreads - 1) / kHistThreads, 2 * sms));
        const int pass_grid = std::min(tiles, per_sm * sms);
        digit_hist_kernel<<<hist_grid, kHistThreads, 0, stream>>>(keys, static_cast<int>(n), begin_bit, passes,
                                                                  t.ghist + pass_base * kDigits, run_if);
        ++*launches;
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        uint64_t* kin = keys;
        uint32_t* vin = vals;
        uint64_t* kout = keys_alt;
        uint32_t* vout = vals_alt;
        for (int p = 0; p < passes; ++p)
        {
            const int q = pass_base + p;
            if (run_if)
                digit_pass_kernel<true><<<pass_grid, kThreads, kPassSmem, stream>>>(
                    kin, vin, kout, vout, static_cast<int>(n), begin_bit + p * kBits, q, t.ghist + q * kDigits,
                    t.status, t.tickets + q, err, run_if);
            else
                digit_pass_kernel<false><<<tiles, kThreads, kPassSmem, stream>>>(
                    kin, vin, kout, vout, static_cast<int>(n), begin_bit + p * kBits, q, t.ghist + q * kDigits,
                    t.status, t.tickets + q, err, run_if);
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
