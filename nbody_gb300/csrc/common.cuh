// Shared device helpers for the sm_103a kernels: bounded mbarrier waits, TMA bulk
// copies, the packed FP32x2 arithmetic and the SFU reciprocal square root.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nbody_cuda.h"

namespace nbg
{
    // Device error word bits (ctx->dev_error). Kernels OR these in and return; the host
    // reads the word at the next synchronisation point and maps it to a status.
    enum : unsigned
    {
        DEV_ERR_TIMEOUT = 1u,   // a bounded mbarrier / flag wait gave up
        DEV_ERR_BOUNDS = 2u,    // an index failed a bounds check and the access was skipped
    };

    // Limit on any spin-wait, in nanoseconds of %globaltimer. A tile copy completes in
    // microseconds; a wait this long only ends when something is broken, and then the
    // kernel reports DEV_ERR_TIMEOUT instead of hanging the device.
    constexpr uint64_t kWaitLimitNs = 2000000000ull;

    __device__ __forceinline__ uint64_t globaltimer()
    {
        uint64_t t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        return t;
    }

    __device__ __forceinline__ uint32_t smem_addr(const void* p)
    {
        return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    __device__ __forceinline__ void mbar_init(uint64_t* bar, const unsigned count)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
    }

    // Make mbarrier initialisation visible to the async (TMA) proxy.
    __device__ __forceinline__ void fence_mbar_init()
    {
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    __device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, const unsigned bytes)
    {
        asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;"
                     :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
    }

    __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, const unsigned parity)
    {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        return ok != 0;
    }

    // As mbar_try_wait, but the thread may be suspended for up to hint_ns while the phase is
    // incomplete instead of returning at once, so a waiting warp takes no issue slots from
    // the warps that are computing.
    __device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, const unsigned parity, const unsigned hint_ns)
    {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns) : "memory");
        return ok != 0;
    }

    // Wait for phase `parity` of `bar` to complete, giving up after limit_ns.
    // Returns false on timeout (and records it in *err).
    __device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, const unsigned parity,
                                                      unsigned* err, const uint64_t limit_ns = kWaitLimitNs)
    {
        if (mbar_try_wait(bar, parity))
            return true;
        const uint64_t start = globaltimer();
        for (;;)
        {
            if (mbar_try_wait_suspend(bar, parity, 20000u))
                return true;
            if (globaltimer() - start > limit_ns)
            {
                atomicOr(err, DEV_ERR_TIMEOUT);
                return false;
            }
        }
    }

    // One-dimensional TMA bulk copy global -> shared, completing on `bar` with a byte
    // count. dst, src and bytes must all be multiples of 16.
    __device__ __forceinline__ void tma_load_1d(void* dst, const void* src, const unsigned bytes,
                                                uint64_t* bar)
    {
        asm volatile(
            "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
    }

    // MUFU reciprocal square root (approximate, flush-to-zero): one SFU instruction.
    __device__ __forceinline__ float rsqrt_sfu(const float x)
    {
        float y;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }

    __device__ __forceinline__ float2 f2(const float a) { return make_float2(a, a); }
    __device__ __forceinline__ float2 add2(const float2 a, const float2 b) { return __fadd2_rn(a, b); }
    __device__ __forceinline__ float2 mul2(const float2 a, const float2 b) { return __fmul2_rn(a, b); }
    __device__ __forceinline__ float2 fma2(const float2 a, const float2 b, const float2 c) { return __ffma2_rn(a, b, c); }

    // The exactly rounded packed square a*a of each half, as a*a + 0 in one FMA. The code
    // generator fuses a packed multiply into a dependent packed add (one rounding less),
    // even when both are written as PTX with an explicit .rn; an FMA result cannot be fused
    // again, and fma(a, a, +0) rounds exactly as the product a*a (a*a is never -0).
    __device__ __forceinline__ float2 sq2(const float2 a) { return __ffma2_rn(a, a, make_float2(0.f, 0.f)); }

    // a - b per half (the negation is exact, so this is the correctly rounded difference).
    __device__ __forceinline__ float2 sub2(const float2 a, const float2 b)
    {
        return __fadd2_rn(a, make_float2(-b.x, -b.y));
    }

    // Error-free transformation of a sum (Knuth's TwoSum): s = fl(a + b) and
    // e = (a + b) - s exactly, for any a and b. Six additions, none reassociated (the
    // intrinsics are never contracted or reordered).
    __device__ __forceinline__ void two_sum(const float a, const float b, float& s, float& e)
    {
        s = __fadd_rn(a, b);
        const float bb = __fsub_rn(s, a);
        e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    }

    // Error-free transformation of a sum (Knuth's TwoSum), per half: s = fl(a + b) and
    // e = (a + b) - s exactly, for any a and b (no ordering of magnitudes needed). Six
    // additions, none of which may be reassociated; packed adds are never contracted.
    __device__ __forceinline__ void two_sum2(const float2 a, const float2 b, float2& s, float2& e)
    {
        s = add2(a, b);
        const float2 bb = sub2(s, a);
        e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
    }

    inline unsigned ceil_div(const size_t a, const size_t b) { return static_cast<unsigned>((a + b - 1) / b); }
}
