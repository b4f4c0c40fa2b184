// Stable LSD radix sort of (uint64 key, uint32 value) pairs (sort.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <utility>
#include <cuda_runtime.h>

namespace nbg
{
    // Temporary bytes radix_sort_pairs needs for n pairs.
    size_t sort_temp_bytes(size_t n);

    // Sort by bits [begin_bit, end_bit) of the key, 9 bits per pass, ping-ponging between
    // (keys, vals) and (keys_alt, vals_alt). *in_alt tells which pair holds the result.
    // n < 2^31. A look-back wait that gives up (it cannot, unless the device is broken) ORs
    // DEV_ERR_TIMEOUT into *err.
    // run_if: when given, every kernel of the call first reads *run_if on the device and
    // does nothing if it is 0 (the launches are made either way, so the host need not know).
    // pass_base: a call with pass_base 0 zeroes temp for 16 passes in all; a later call on
    // the same temp and n gives its passes the indices pass_base, pass_base + 1, ... (< 16),
    // so their tickets, histograms and published counts are their own.
    cudaError_t radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt,
                                 size_t n, int begin_bit, int end_bit, void* temp, cudaStream_t stream,
                                 uint64_t* launches, bool* in_alt, unsigned* err,
                                 const unsigned* run_if = nullptr, int pass_base = 0);
}
