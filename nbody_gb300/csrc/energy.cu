// Energy and momentum of every body of a context at the direct sum's rate (sm_103a).
//
// No reference counterpart: the reference keeps no diagnostics. The FP64 per-system
// diagnostics (nbody_cuda_system_energy) take O(N^2) FP64 work, which GB300's FP64 pipe
// cannot carry at millions of bodies; this form keeps every pair term in FP32 and every
// sum exact enough that the energy drift of a run can be read to a few 1e-9:
//   - the potential is E_pot = -G sum_{i<j} m_i m_j / sqrt(|d_ij|^2 + eps2), over the
//     upper triangle of 1024-body blocks: one CTA per block row I sums blocks J >= I, the
//     diagonal block at half weight (it holds every pair of the block twice);
//   - per target, packed FP32 pair terms m_j / r_ij (rsqrt on the SFU) are summed in FP32
//     per 256-source tile and the tile sums folded into an (S, C) pair by an error-free
//     TwoSum, as the direct sum folds its accelerations; m_i (S + C) is added in FP64;
//   - pairs at zero separation are left out: the self-pair, and coincident bodies
//     (with eps2 > 0, also pairs whose |d|^2 is below half an ulp of eps2);
//   - E_kin = 1/2 sum_i m_i |v_i|^2 and P = sum_i m_i v_i in FP64;
//   - every total is summed per block in a fixed tree order and the block partials in
//     order on the host, so the result is deterministic.
#include <vector>

#include "common.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        constexpr int kEBlock = 256;            // threads per CTA; also sources per tile
        constexpr int kET = 4;                  // targets per thread (two packed pairs)
        constexpr int kRedBlock = 256;
    }

    // Row I of the block triangle: part[I] = sum over blocks J >= I of
    // sum_{i in I, j in J} m_i m_j / r_ij, the diagonal block at half weight (unscaled by
    // G). src is pos_mass (stride 1) or the Body array as float4 (stride 3: mass in the
    // second record's w). The longest rows (small I) are the first CTAs, so the short ones
    // fill in at the end.
    __global__ void __launch_bounds__(kEBlock, 3) potential_rows_kernel(const float4* __restrict__ src, const int stride,
                                                                        const int n, const float eps2,
                                                                        double* __restrict__ part)
    {
        constexpr int P = kET / 2;
        constexpr int kRows = kEBlock * kET;        // bodies per block
        __shared__ float4 tile[kEBlock];
        __shared__ double red[kEBlock];
        const int tid = threadIdx.x;
        const int row = blockIdx.x;
        const int base = row * kRows;
        float2 nx[P], ny[P], nz[P], mt[P], acc[P], S[P], C[P];
#pragma unroll
        for (int p = 0; p < P; ++p)
        {
            float q[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                const int i = base + tid + (2 * p + h) * kEBlock;
                const size_t ic = static_cast<size_t>(min(i, n - 1));
                const float4 x = src[ic * stride];
                const float m = stride == 3 ? src[ic * 3 + 1].w : x.w;
                q[h][0] = -x.x;
                q[h][1] = -x.y;
                q[h][2] = -x.z;
                q[h][3] = i < n ? m : 0.f;          // a padding target adds nothing
            }
            nx[p] = make_float2(q[0][0], q[1][0]);
            ny[p] = make_float2(q[0][1], q[1][1]);
            nz[p] = make_float2(q[0][2], q[1][2]);
            mt[p] = make_float2(q[0][3], q[1][3]);
            acc[p] = S[p] = C[p] = make_float2(0.f, 0.f);
        }
        const float2 e2 = f2(eps2);
        double diag = 0.0, off = 0.0;
        // m_i (S + C) per target into an FP64 total, and (S, C) back to zero
        auto settle = [&](double& total) {
#pragma unroll
            for (int p = 0; p < P; ++p)
            {
                total += static_cast<double>(mt[p].x) * (static_cast<double>(S[p].x) + static_cast<double>(C[p].x));
                total += static_cast<double>(mt[p].y) * (static_cast<double>(S[p].y) + static_cast<double>(C[p].y));
                S[p] = C[p] = make_float2(0.f, 0.f);
            }
        };
        for (int j0 = base; j0 < n; j0 += kEBlock)
        {
            const int j = j0 + tid;
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);     // padding: massless, adds 0
            if (j < n)
            {
                s = src[static_cast<size_t>(j) * stride];
                if (stride == 3)
                    s.w = src[static_cast<size_t>(j) * 3 + 1].w;
            }
            tile[tid] = s;
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kEBlock; ++k)
            {
                const float4 t = tile[k];
#pragma unroll
                for (int p = 0; p < P; ++p)
                {
                    const float2 dx = add2(f2(t.x), nx[p]), dy = add2(f2(t.y), ny[p]), dz = add2(f2(t.z), nz[p]);
                    float2 r2 = fma2(dx, dx, e2);
                    r2 = fma2(dy, dy, r2);
                    r2 = fma2(dz, dz, r2);
                    float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
                    inv.x = r2.x > eps2 ? inv.x : 0.f;      // zero separation: left out
                    inv.y = r2.y > eps2 ? inv.y : 0.f;
                    acc[p] = fma2(f2(t.w), inv, acc[p]);
                }
            }
            __syncthreads();
#pragma unroll
            for (int p = 0; p < P; ++p)
            {
                float2 sum, err;
                two_sum2(S[p], acc[p], sum, err);
                S[p] = sum;
                C[p] = add2(C[p], err);
                acc[p] = make_float2(0.f, 0.f);
            }
            // the diagonal block is complete after its last tile (a short one in the last row)
            if (j0 < base + kRows && j0 + kEBlock >= min(n, base + kRows))
                settle(diag);
        }
        settle(off);
        red[tid] = 0.5 * diag + off;
        __syncthreads();
        for (int k = kEBlock / 2; k > 0; k >>= 1)
        {
            if (tid < k)
                red[tid] += red[tid + k];
            __syncthreads();
        }
        if (tid == 0)
            part[row] = red[0];
    }

    // Per block: {sum m |v|^2, sum m v} in FP64, by a fixed-order tree.
    __global__ void __launch_bounds__(kRedBlock) kinetic_kernel(const float4* __restrict__ src,
                                                                const float4* __restrict__ vel, const int stride,
                                                                const int n, double* __restrict__ part)
    {
        __shared__ double red[4][kRedBlock];
        const int i = blockIdx.x * kRedBlock + threadIdx.x;
        double v[4] = { 0.0, 0.0, 0.0, 0.0 };
        if (i < n)
        {
            float m;
            float3 u;
            if (stride == 3)
            {
                const float4 b1 = src[static_cast<size_t>(i) * 3 + 1];     // vel, mass
                m = b1.w;
                u = make_float3(b1.x, b1.y, b1.z);
            }
            else
            {
                m = src[i].w;
                const float4 w = vel[i];
                u = make_float3(w.x, w.y, w.z);
            }
            const double md = m;
            v[0] = md * (static_cast<double>(u.x) * u.x + static_cast<double>(u.y) * u.y + static_cast<double>(u.z) * u.z);
            v[1] = md * u.x;
            v[2] = md * u.y;
            v[3] = md * u.z;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            red[c][threadIdx.x] = v[c];
        __syncthreads();
        for (int s = kRedBlock / 2; s > 0; s >>= 1)
        {
            if (threadIdx.x < s)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    red[c][threadIdx.x] += red[c][threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x < 4)
            part[static_cast<size_t>(blockIdx.x) * 4 + threadIdx.x] = red[threadIdx.x][0];
    }

    int energy_all(nbody_cuda* ctx, const nbody_step_params* p, double out[5])
    {
        const size_t n = ctx->count;
        for (int c = 0; c < 5; ++c)
            out[c] = 0.0;
        if (n == 0)
            return NBODY_OK;
        const int ni = static_cast<int>(n);
        const bool aos = ctx->layout == NBODY_LAYOUT_AOS;
        const float4* src = aos ? reinterpret_cast<const float4*>(ctx->bodies) : ctx->pm;
        const int stride = aos ? 3 : 1;
        const float eps2 = p->law == NBODY_LAW_SOFTENED ? p->eps2 : 0.f;
        const unsigned rows = ceil_div(n, kEBlock * kET);
        const unsigned red_blocks = ceil_div(n, kRedBlock);
        const size_t words = static_cast<size_t>(rows) + 4 * static_cast<size_t>(red_blocks);
        if (const int st = ensure_scratch(ctx, words * sizeof(double)))
            return st;
        ctx->pending_partials = 0;      // the scratch is reused here
        double* rowsum = static_cast<double*>(ctx->scratch);
        double* kin = rowsum + rows;
        potential_rows_kernel<<<rows, kEBlock, 0, ctx->stream>>>(src, stride, ni, eps2, rowsum);
        kinetic_kernel<<<red_blocks, kRedBlock, 0, ctx->stream>>>(src, aos ? nullptr : ctx->vr, stride, ni, kin);
        ctx->launches += 2;
        cudaError_t e = cudaGetLastError();
        std::vector<double> h(words);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h.data(), rowsum, words * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess)
            return ctx_cuda_fail(ctx, e, "energy diagnostics");
        double pot = 0.0, sum[4] = { 0.0, 0.0, 0.0, 0.0 };
        for (unsigned r = 0; r < rows; ++r)
            pot += h[r];
        for (unsigned b = 0; b < red_blocks; ++b)
            for (int c = 0; c < 4; ++c)
                sum[c] += h[rows + static_cast<size_t>(b) * 4 + c];
        out[0] = 0.5 * sum[0];
        out[1] = -static_cast<double>(p->G) * pot;
        out[2] = sum[1];
        out[3] = sum[2];
        out[4] = sum[3];
        return NBODY_OK;
    }
}
