// Device-wide exclusive scan (see scan.cuh).
#include "common.cuh"
#include "scan.cuh"

namespace nbg
{
    // Exclusive scan of one tile of kScanTile items; writes the tile total to sums[blockIdx.x]
    // (when sums != nullptr). Items beyond n read as zero and are not written.
    template <typename T>
    __global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const T* in, T* out, T* __restrict__ sums,
                                                                     const size_t n)
    {
        using Op = ScanOps<T>;
        __shared__ T warp_tot[kScanThreads / 32];
        const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile + static_cast<size_t>(threadIdx.x) * kScanItems;
        T v[kScanItems];
        T run = Op::zero();
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const size_t i = base + k;
            v[k] = i < n ? in[i] : Op::zero();
            const T t = v[k];
            v[k] = run;             // exclusive within the thread
            run = Op::add(run, t);
        }
        // inclusive warp scan of the thread totals
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        T incl = run;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
        {
            const T o = Op::shfl_up(incl, d);
            if (lane >= d)
                incl = Op::add(incl, o);
        }
        if (lane == 31)
            warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0)
        {
            T w = lane < kScanThreads / 32 ? warp_tot[lane] : Op::zero();
            T wi = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const T o = Op::shfl_up(wi, d);
                if (lane >= d)
                    wi = Op::add(wi, o);
            }
            if (lane < kScanThreads / 32)
                warp_tot[lane] = wi;    // inclusive over warps
        }
        __syncthreads();
        // exclusive prefix of this thread = (all earlier warps) + (earlier lanes of this warp)
        T excl_in_warp = Op::shfl_up(incl, 1);
        if (lane == 0)
            excl_in_warp = Op::zero();
        const T offset = Op::add(warp > 0 ? warp_tot[warp - 1] : Op::zero(), excl_in_warp);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const size_t i = base + k;
            if (i < n)
                out[i] = Op::add(offset, v[k]);
        }
        if (sums && threadIdx.x == kScanThreads - 1)
            sums[blockIdx.x] = Op::add(offset, run);
    }

    template <typename T>
    __global__ void add_offsets_kernel(T* __restrict__ out, const T* __restrict__ offsets, const size_t n)
    {
        using Op = ScanOps<T>;
        const T off = offsets[blockIdx.x];
        const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile;
        for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        {
            const size_t i = base + k;
            if (i < n)
                out[i] = Op::add(out[i], off);
        }
    }

    template <typename T>
    cudaError_t exclusive_scan(const T* in, T* out, const size_t n, T* temp, cudaStream_t stream, uint64_t* launches)
    {
        if (n == 0)
            return cudaSuccess;
        const size_t tiles = (n + kScanTile - 1) / kScanTile;
        if (tiles == 1)
        {
            scan_tile_kernel<T><<<1, kScanThreads, 0, stream>>>(in, out, nullptr, n);
            ++*launches;
            return cudaGetLastError();
        }
        T* sums = temp;                 // tiles elements
        T* rest = temp + tiles + 1;     // deeper levels
        scan_tile_kernel<T><<<static_cast<unsigned>(tiles), kScanThreads, 0, stream>>>(in, out, sums, n);
        ++*launches;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        // scan the tile totals in place (each item is read, then written, by the same thread)
        e = exclusive_scan<T>(sums, sums, tiles, rest, stream, launches);
        if (e != cudaSuccess)
            return e;
        add_offsets_kernel<T><<<static_cast<unsigned>(tiles), 256, 0, stream>>>(out, sums, n);
        ++*launches;
        return cudaGetLastError();
    }

    template cudaError_t exclusive_scan<uint32_t>(const uint32_t*, uint32_t*, size_t, uint32_t*, cudaStream_t, uint64_t*);
    template cudaError_t exclusive_scan<Int64x4>(const Int64x4*, Int64x4*, size_t, Int64x4*, cudaStream_t, uint64_t*);
}
