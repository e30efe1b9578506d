// Shared body of the Lagrange-multiplier preparation kernels, included by mese.cu (FP32: compiled without
// FMA contraction, the reference's roundings) and by mese_f64.cu (FP64: compiled with contraction, the
// precision form needs no particular rounding order and GB300's FP64 rate makes every fused operation count).
// Everything here has internal linkage: each translation unit holds its own copy of the constant tables.
#pragma once

#include "internal.h"
#include "mese_device.cuh"

namespace mraygb
{
namespace
{

__constant__ float c_two_pi_over_l_f[256];
__constant__ double c_two_pi_over_l_d[256];

template <typename T> __device__ __forceinline__ const T *two_pi_over_l();
template <> __device__ __forceinline__ const float *two_pi_over_l<float>() { return c_two_pi_over_l_f; }
template <> __device__ __forceinline__ const double *two_pi_over_l<double>() { return c_two_pi_over_l_d; }

__device__ __forceinline__ void pixel_span(const uint32_t *index, int m, int p, size_t &idx, int &n)
{
    if (index)
    {
        idx = index[p];
        n = (int)(index[p + 1] - index[p]);
    }
    else
    {
        idx = (size_t)p * (size_t)m;
        n = m;
    }
}

// Shared-memory budget of one block: NC complex and NR real arrays of MAXM elements per thread.
template <typename T, int MAXM, int NC, int NR> constexpr int smem_per_thread()
{
    return MAXM * (NC * (int)sizeof(cx<T>) + NR * (int)sizeof(T));
}

// Lagrange multipliers (prepare_moments_from_std_coding / prepare_moments_from_pred_coding).  Arrays live in
// thread-strided shared memory: e (exponential moments), poly (Levinson solution) and the real accumulators of the
// correlation; prediction codes are dequantized one at a time as the decode reads them.
template <typename T, int MAXM, int BLOCK, bool PC, typename CArr, typename RArr>
__device__ __forceinline__ void prepare_pixel(int n, const float *in, const CArr &e, const CArr &poly,
                                              const RArr &acc, int coding_warp, const float *params, float bias,
                                              float *out)
{
    if (PC)
    {
        // the codes are dequantized as the decode asks for them (transform_dequantization_real, then decode)
        pc_decode_from<T>(n, PcDequant<T>(in, coding_warp, params), e, poly);
    }
    else
    {
        // cut::lerp(m, target, bias) = (1 - bias) m + bias target (cuda_math.h:72-75), into the accumulators
        const T b = T(bias);
        acc[0] = (T(1) - b) * T(in[0]) + b * T(0.5f);
        for (int i = 1; i < n; ++i)
            acc[i] = (T(1) - b) * T(in[i]) + b * T(0.0f);
        trig_to_exp<T>(n, e, acc, two_pi_over_l<T>());
        levinson<T>(n, poly, e);
    }
    lagrange_from_poly<T>(n, poly, e, acc);
    const T norm = T(1) / (MeseConst<T>::pi * ((cx<T>)poly[0]).x);
    for (int i = 0; i < n; ++i)
        out[i] = float(norm * T(acc[i]));
}

// Lagrange multipliers (prepare_moments_from_std_coding / prepare_moments_from_pred_coding).  SMEM: the arrays
// live in thread-strided shared memory (the FP32 form); otherwise in per-thread local arrays (the FP64 form,
// whose arrays are twice as large and whose throughput is set by GB300's FP64 rate, not by memory).
template <typename T, int MAXM, int BLOCK, bool PC, bool SMEM>
__global__ void __launch_bounds__(BLOCK) prepare_kernel(int num_pixels, int m, const uint32_t *__restrict__ index,
                                                        const float *__restrict__ data, int prediction_code,
                                                        int coding_warp, const uint16_t *__restrict__ coding_params,
                                                        float bias, float *__restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float s_params[2 * MAXM];
    if (prediction_code && coding_warp == 0 && coding_params)
        for (int i = threadIdx.x; i < 2 * (m - 1); i += blockDim.x)
            s_params[i] = coding_params[i] / 65535.f; // CodingParamType::get_param1/2 (coding_params.h:52-54)
    __syncthreads();

    const int p = blockIdx.x * BLOCK + threadIdx.x;
    if (p >= num_pixels)
        return;
    size_t idx;
    int n;
    pixel_span(index, m, p, idx, n);
    if (n <= 0)
        return;
    if (n > MAXM)
        n = MAXM;

    if (SMEM)
    {
        cx<T> *base = reinterpret_cast<cx<T> *>(smem);
        const Strided<cx<T>, BLOCK> e{base + threadIdx.x};
        const Strided<cx<T>, BLOCK> poly{base + MAXM * BLOCK + threadIdx.x};
        const Strided<T, BLOCK> acc{reinterpret_cast<T *>(base + 2 * MAXM * BLOCK) + threadIdx.x};
        prepare_pixel<T, MAXM, BLOCK, PC>(n, data + idx, e, poly, acc, coding_warp, s_params, bias, out + idx);
    }
    else
    {
        cx<T> ae[MAXM], apoly[MAXM];
        T aacc[MAXM];
        const Strided<cx<T>, 1> e{ae}, poly{apoly};
        const Strided<T, 1> acc{aacc};
        prepare_pixel<T, MAXM, BLOCK, PC>(n, data + idx, e, poly, acc, coding_warp, s_params, bias, out + idx);
    }
}


// threads per block for a per-thread shared-memory need: the largest of 128, 64, 32, 16, 8 threads whose arrays
// fit in 60 KiB, so that three blocks share an SM's 228 KiB (large moment counts in FP64 get sub-warp blocks
// rather than local-memory arrays)
template <int PER_THREAD> constexpr int block_for()
{
    constexpr int budget = 60 * 1024;
    return budget / PER_THREAD >= 128 ? 128
         : budget / PER_THREAD >= 64  ? 64
         : budget / PER_THREAD >= 32  ? 32
         : budget / PER_THREAD >= 16  ? 16
                                      : 8;
}

template <typename T, int MAXM, bool PC>
cudaError_t launch_prepare_pc(int num_pixels, int m, const uint32_t *index, const float *data, int warp,
                              const uint16_t *cp, float bias, float *out, cudaStream_t stream)
{
    constexpr bool smem = sizeof(T) == 4;
    constexpr int per = smem_per_thread<T, MAXM, 2, 1>();
    constexpr int block = smem ? block_for<per>() : 128;
    constexpr int bytes = smem ? per * block : 0;
    if (smem)
    {
        cudaError_t e = cudaFuncSetAttribute(prepare_kernel<T, MAXM, block, PC, smem>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess)
            return e;
        // the whole shared-memory carveout: resident pixels are what this latency-bound kernel lives on
        if ((e = cudaFuncSetAttribute(prepare_kernel<T, MAXM, block, PC, smem>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout, 100)) != cudaSuccess)
            return e;
    }
    const int grid = (num_pixels + block - 1) / block;
    prepare_kernel<T, MAXM, block, PC, smem><<<grid, block, bytes, stream>>>(num_pixels, m, index, data, PC ? 1 : 0,
                                                                              warp, cp, bias, out);
    return cudaGetLastError();
}

template <typename T, int MAXM>
cudaError_t launch_prepare_t(int num_pixels, int m, const uint32_t *index, const float *data, int pc, int warp,
                             const uint16_t *cp, float bias, float *out, cudaStream_t stream)
{
    if (pc)
        return launch_prepare_pc<T, MAXM, true>(num_pixels, m, index, data, warp, cp, bias, out, stream);
    return launch_prepare_pc<T, MAXM, false>(num_pixels, m, index, data, warp, cp, bias, out, stream);
}

template <typename T>
cudaError_t launch_prepare_m(int num_pixels, int m, const uint32_t *index, const float *data, int pc, int warp,
                             const uint16_t *cp, float bias, float *out, cudaStream_t stream)
{
    if (m <= 32)
        return launch_prepare_t<T, 32>(num_pixels, m, index, data, pc, warp, cp, bias, out, stream);
    if (m <= 64)
        return launch_prepare_t<T, 64>(num_pixels, m, index, data, pc, warp, cp, bias, out, stream);
    if (m <= 128)
        return launch_prepare_t<T, 128>(num_pixels, m, index, data, pc, warp, cp, bias, out, stream);
    return launch_prepare_t<T, 256>(num_pixels, m, index, data, pc, warp, cp, bias, out, stream);
}

// the constant tables of this translation unit
inline cudaError_t init_tables()
{
    float f[256];
    double d[256];
    f[0] = 0.f;
    d[0] = 0.0;
    for (int l = 1; l < 256; ++l)
    {
        f[l] = (float)(2.0f * 3.141592653589793 / (double)(float)l); // 2.0f * M_PI / static_cast<float>(l)
        d[l] = 2.0 * 3.141592653589793 / (double)l;
    }
    cudaError_t e = cudaMemcpyToSymbol(c_two_pi_over_l_f, f, sizeof(f));
    if (e != cudaSuccess)
        return e;
    return cudaMemcpyToSymbol(c_two_pi_over_l_d, d, sizeof(d));
}

} // namespace
} // namespace mraygb
