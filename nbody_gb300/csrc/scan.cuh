// Device-wide exclusive prefix sums (uint32 and four int64 lanes), used by the radix sort,
// the octree compaction and the fixed-point centre-of-mass sums. Three-phase: each CTA scans a 4096-item
// tile and records its total; the totals are scanned (recursively); each tile then adds
// its offset. All temporaries come from a caller-provided buffer.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace nbg
{
    constexpr int kScanThreads = 1024;
    constexpr int kScanItems = 4;
    constexpr int kScanTile = kScanThreads * kScanItems;

    // Four int64 lanes: a cell sum {m x, m y, m z, m} in fixed point. Integer sums are exact,
    // so any association of the additions gives the same bits.
    struct __align__(32) Int64x4
    {
        long long x, y, z, w;
    };

    template <typename T> struct ScanOps;

    template <> struct ScanOps<uint32_t>
    {
        static __device__ __forceinline__ uint32_t zero() { return 0u; }
        static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) { return a + b; }
        static __device__ __forceinline__ uint32_t shfl_up(uint32_t v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
    };

    template <> struct ScanOps<Int64x4>
    {
        static __device__ __forceinline__ Int64x4 zero() { return Int64x4{ 0, 0, 0, 0 }; }
        static __device__ __forceinline__ Int64x4 add(Int64x4 a, Int64x4 b)
        {
            return Int64x4{ a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w };
        }
        static __device__ __forceinline__ Int64x4 shfl_up(Int64x4 v, int d)
        {
            return Int64x4{ __shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                            __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d) };
        }
        static __device__ __forceinline__ Int64x4 shfl_down(Int64x4 v, int d)
        {
            return Int64x4{ __shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
                            __shfl_down_sync(0xffffffffu, v.z, d), __shfl_down_sync(0xffffffffu, v.w, d) };
        }
    };

    // Number of T elements of temporary storage exclusive_scan needs for n items.
    inline size_t scan_temp_elems(size_t n)
    {
        size_t total = 0;
        while (n > 1)
        {
            n = (n + kScanTile - 1) / kScanTile;
            total += n + 1;
        }
        return total + 1;
    }

    template <typename T>
    cudaError_t exclusive_scan(const T* in, T* out, size_t n, T* temp, cudaStream_t stream, uint64_t* launches);

    extern template cudaError_t exclusive_scan<uint32_t>(const uint32_t*, uint32_t*, size_t, uint32_t*, cudaStream_t, uint64_t*);
    extern template cudaError_t exclusive_scan<Int64x4>(const Int64x4*, Int64x4*, size_t, Int64x4*, cudaStream_t, uint64_t*);
}
