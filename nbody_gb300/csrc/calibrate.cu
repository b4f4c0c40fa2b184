// FP32 pipe calibration: the measured FFMA throughput the direct-sum roofline is stated
// against (the measured peaks cover only HBM copy and BF16 tensor throughput).
//
// Each thread runs 8 independent multiply-add chains (scalar FFMA or packed FFMA2) for
// `iters` iterations; the grid is 4 CTAs of 256 threads per SM. The chains' final values
// are stored so nothing is dead code.
#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    template <bool PACKED>
    __global__ void __launch_bounds__(256) ffma_peak_kernel(float* out, const int iters, const float a, const float b)
    {
        float2 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            v[k] = make_float2(threadIdx.x * 1e-3f + k, blockIdx.x * 1e-3f - k);
        const float2 A = make_float2(a, a), B = make_float2(b, b);
        for (int i = 0; i < iters; ++i)
        {
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
                if (PACKED)
                    v[k] = __ffma2_rn(v[k], A, B);
                else
                {
                    v[k].x = fmaf(v[k].x, a, b);
                    v[k].y = fmaf(v[k].y, a, b);
                }
            }
        }
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            s += v[k].x + v[k].y;
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

extern "C" int nbody_cuda_calibrate_fp32(nbody_cuda* ctx, double* tflops_scalar, double* tflops_packed)
{
    using namespace nbg;
    if (!ctx)
        return NBODY_ERR_INVALID;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int blocks = sms * 4, threads = 256, iters = 1 << 14;
    if (const int st = ensure_scratch(ctx, static_cast<size_t>(blocks) * threads * sizeof(float)))
        return st;
    float* out = static_cast<float*>(ctx->scratch);
    EventPair ev;
    if (ev.status != cudaSuccess)
        return ctx_cuda_fail(ctx, ev.status, "event create");
    double res[2] = { 0, 0 };
    for (int packed = 0; packed < 2; ++packed)
    {
        float best = 1e30f;
        for (int rep = 0; rep < 4; ++rep)
        {
            cudaEventRecord(ev.start, ctx->stream);
            if (packed)
                ffma_peak_kernel<true><<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999f, 1e-3f);
            else
                ffma_peak_kernel<false><<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999f, 1e-3f);
            ++ctx->launches;
            cudaEventRecord(ev.stop, ctx->stream);
            const float ms = ev.elapsed_ms();
            if (rep > 0 && ms < best)
                best = ms;
        }
        // 8 chains x 2 lanes x 2 flop per iteration per thread
        const double flop = static_cast<double>(blocks) * threads * iters * 8.0 * 2.0 * 2.0;
        res[packed] = flop / (best * 1e-3) / 1e12;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return ctx_cuda_fail(ctx, e, "calibration kernel");
    if (tflops_scalar)
        *tflops_scalar = res[0];
    if (tflops_packed)
        *tflops_packed = res[1];
    return NBODY_OK;
}

namespace nbg
{
    __global__ void __launch_bounds__(256) dfma_peak_kernel(double* out, const int iters, const double a, const double b)
    {
        double v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            v[k] = threadIdx.x * 1e-3 + k;
        for (int i = 0; i < iters; ++i)
        {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                v[k] = fma(v[k], a, b);
        }
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            s += v[k];
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

extern "C" int nbody_cuda_calibrate_fp64(nbody_cuda* ctx, double* tflops)
{
    using namespace nbg;
    if (!ctx || !tflops)
        return NBODY_ERR_INVALID;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int blocks = sms * 4, threads = 256, iters = 1 << 10;
    if (const int st = ensure_scratch(ctx, static_cast<size_t>(blocks) * threads * sizeof(double)))
        return st;
    EventPair ev;
    if (ev.status != cudaSuccess)
        return ctx_cuda_fail(ctx, ev.status, "event create");
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep)
    {
        cudaEventRecord(ev.start, ctx->stream);
        dfma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(static_cast<double*>(ctx->scratch), iters, 0.999, 1e-3);
        ++ctx->launches;
        cudaEventRecord(ev.stop, ctx->stream);
        const float ms = ev.elapsed_ms();
        if (rep > 0 && ms < best)
            best = ms;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return ctx_cuda_fail(ctx, e, "calibration kernel");
    *tflops = static_cast<double>(blocks) * threads * iters * 8.0 * 2.0 / (best * 1e-3) / 1e12;
    return NBODY_OK;
}

namespace nbg
{
    // Waits on an mbarrier phase that nothing completes (one arrival expected, none made,
    // no copy issued), with the bounded wait every pipeline uses, so the give-up path runs:
    // the wait returns after limit_ns, sets DEV_ERR_TIMEOUT and the kernel exits normally.
    __global__ void selftest_wait_kernel(unsigned* err, const unsigned long long limit_ns)
    {
        __shared__ __align__(8) uint64_t bar;
        if (threadIdx.x == 0)
        {
            mbar_init(&bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        mbar_wait_bounded(&bar, 0, err, limit_ns);
    }
}

extern "C" int nbody_cuda_selftest_wait(nbody_cuda* ctx, const uint64_t limit_ns)
{
    using namespace nbg;
    if (!ctx)
        return NBODY_ERR_INVALID;
    if (limit_ns == 0 || limit_ns > 100000000ull)
        return ctx_fail(ctx, NBODY_ERR_INVALID, "self-test wait limit must be in (0, 0.1 s]");
    selftest_wait_kernel<<<1, 32, 0, ctx->stream>>>(ctx->dev_error, limit_ns);
    ++ctx->launches;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return ctx_cuda_fail(ctx, e, "self-test launch");
    return check_device_error(ctx);
}
