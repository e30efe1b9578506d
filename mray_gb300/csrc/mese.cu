// Per-pixel MESE kernels: Lagrange-multiplier preparation (standard and prediction-coded moments, FP32 or
// FP64) and the error-threshold moment count of compaction.  Built without FMA contraction so that the FP32
// form performs the reference's roundings (see mese_device.cuh).
//
//   prepare_moments_from_std_coding   src/moment_preparation.h:55-64 (bias lerp + prepareMESELagrange)
//   prepare_moments_from_pred_coding  src/moment_preparation.h:32-53
//   determine_best_number_moments     src/moment_compaction.h:113-142 (with :35-111)
//
// One thread per pixel; the O(m^2) recursions work on per-thread arrays of m complex values.

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

template <typename T, int MAXM>
__global__ void __launch_bounds__(128) prepare_kernel(int num_pixels, int m, const uint32_t *__restrict__ index,
                                                      const float *__restrict__ data, int prediction_code,
                                                      int coding_warp, const uint16_t *__restrict__ coding_params,
                                                      float bias, float *__restrict__ out)
{
    __shared__ float s_params[2 * MAXM];
    if (prediction_code && coding_warp == 0 && coding_params)
        for (int i = threadIdx.x; i < 2 * (m - 1); i += blockDim.x)
            s_params[i] = coding_params[i] / 65535.f; // CodingParamType::get_param1/2 (coding_params.h:52-54)
    __syncthreads();

    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= num_pixels)
        return;
    size_t idx;
    int n;
    pixel_span(index, m, p, idx, n);
    if (n <= 0)
        return;
    if (n > MAXM)
        n = MAXM;

    cx<T> a0[MAXM], a1[MAXM], a2[MAXM];
    if (prediction_code)
    {
        cx<T> code[MAXM];
        pc_dequant_real<T>(n, data + idx, code, coding_warp, s_params);
        pc_decode<T>(n, code, a0, a1, a2);          // a0 = exp moments, a1 = evaluation polynomial
        lagrange_from_poly<T, float>(n, a1, a0, a2, out + idx);
    }
    else
    {
        T mom[MAXM];
        const T b = T(bias);
        mom[0] = (T(1) - b) * T(data[idx]) + b * T(0.5f); // cut::lerp (cuda_math.h:72-75)
        for (int i = 1; i < n; ++i)
            mom[i] = (T(1) - b) * T(data[idx + i]) + b * T(0.0f);
        trig_to_exp<T>(n, a0, mom, two_pi_over_l<T>());
        levinson<T>(n, a1, a0, a2);
        lagrange_from_poly<T, float>(n, a1, a0, a2, out + idx);
    }
}

// ---- error-threshold compaction (float, the reference's arithmetic) ---------------------------------------

template <int MAXM>
__device__ void eval_unknown(int num, const cx<float> *e, int max_moments, cx<float> *new_e, cx<float> *lev)
{
    const int mm = max_moments - 1;
    const int n = num - 1;
    levinson<float>(num, lev, e, new_e);
    for (int i = 0; i < n + 1; ++i)
        lev[i] = cscale(MeseConst<float>::two_pi, lev[i]);
    for (int l = 0; l < n + 1; ++l)
        new_e[l] = e[l];
    const cx<float> inv_lev0 = cdiv(mk<float>(-1.f, 0.f), lev[0]);
    for (int k = 0; k < mm - n; ++k)
    {
        cx<float> acc = mk<float>(0, 0);
        for (int j = 1; j < n + 1; ++j)
            acc = cadd(acc, cmulc(new_e[j + k], lev[n + 1 - j]));
        new_e[n + k + 1] = cmulc(acc, inv_lev0);
    }
}

// exponential_to_bounded_moments: the reference multiplies by exp_moments[l] inside the sum (kept as is)
__device__ void exp_to_bounded(int num, const cx<float> *e, cx<float> *b, int n)
{
    const cx<float> gamma_0 = cdivr(e[0], 2.f);
    // float_complex(0, 2) * M_PI * gamma_0: M_PI converts to float_complex((float)M_PI)
    const cx<float> i2pi = cmulc(mk<float>(0.f, 2.f), mk<float>(MeseConst<float>::pi_l, 0.f));
    for (int l = n; l < num; ++l)
    {
        b[l] = mk<float>(0, 0);
        for (int j = 0; j < l; ++j)
        {
            const cx<float> dq = cdiv(mk<float>((float)(l - j), 0.f), cscale((float)l, gamma_0));
            b[l] = cadd(b[l], cmulc(cmulc(dq, e[l]), b[l - j]));
        }
        b[l] = csub(cdiv(e[l], cmulc(i2pi, gamma_0)), b[l]);
    }
}

template <int MAXM>
__global__ void __launch_bounds__(128) count_moments_kernel(int num_pixels, int m, float thr,
                                                            const float *__restrict__ moments,
                                                            uint32_t *__restrict__ counts)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= num_pixels || counts[p] == 0)
        return;
    const float *mo = moments + (size_t)p * (size_t)m;
    cx<float> te[MAXM], text[MAXM], tlev[MAXM];
    const float norm = 1.0f / mo[0];
    trig_to_exp<float>(m, te, mo, two_pi_over_l<float>());
    int n = m / 2;
    int s = m / 4;
    while (s > 0)
    {
        eval_unknown<MAXM>(n, te, m, text, tlev);
        cx<float> *ext = tlev;
        for (int l = 0; l < n; ++l)
            ext[l] = mk<float>(mo[l], 0.f);
        exp_to_bounded(m, text, ext, n);
        float sum = 0.f;
        for (int k = n; k < m; ++k)
        {
            const float diff = ext[k].x - mo[k];
            sum += diff * diff;
        }
        const float rrmse = sqrtf(sum) * norm;
        if (tmax(rrmse - thr, thr - rrmse) < MeseConst<float>::rrmse_tie) // cut::abs(rrmse - thr) < 1e-8f
            break;
        else if (rrmse > thr)
            n += s;
        else
            n -= s;
        s = s / 2;
    }
    counts[p] = (uint32_t)n;
}

// MomentImageHost::prediction_encode, per-pixel part (moment_image.cpp:103-126): bias lerp, trigonometric ->
// exponential moments, encode, projection of the residuals to the real line; in place
template <int MAXM>
__global__ void __launch_bounds__(128) prediction_encode_kernel(int num_pixels, int m,
                                                                const uint32_t *__restrict__ index,
                                                                float *__restrict__ data, float bias)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= num_pixels)
        return;
    size_t idx;
    int n;
    pixel_span(index, m, p, idx, n);
    if (n <= 0)
        return;
    if (n > MAXM)
        n = MAXM;
    float *d = data + idx;
    d[0] = (1 - bias) * d[0] + bias * 0.5f; // cut::lerp(data[idx], 0.5f, bias)
    for (int i = 1; i < n; ++i)
        d[i] = (1 - bias) * d[i] + bias * 0.0f;
    cx<float> e[MAXM], code[MAXM], poly[MAXM], tmp[MAXM];
    trig_to_exp<float>(n, e, d, two_pi_over_l<float>());
    pc_encode<float>(n, e, code, poly, tmp);
    // transform_quantization_real (moment_prediction_coding.h:81-92): out[0] = c_0 stays d[0]
    const cx<float> axis = mk(-code[0].y, code[0].x);
    const float len = sqrtf(cabs2(axis));
    const cx<float> inv_axis = cdiv(mk(len, 0.f), axis);
    for (int l = 1; l < n; ++l)
        d[l] = cmulc(code[l], inv_axis).x;
}

template <typename T, int MAXM>
cudaError_t launch_prepare_t(int num_pixels, int m, const uint32_t *index, const float *data, int pc, int warp,
                             const uint16_t *cp, float bias, float *out, cudaStream_t stream)
{
    const int block = 128;
    const int grid = (num_pixels + block - 1) / block;
    prepare_kernel<T, MAXM><<<grid, block, 0, stream>>>(num_pixels, m, index, data, pc, warp, cp, bias, out);
    return cudaGetLastError();
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

} // namespace

cudaError_t mese_init_constants()
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

cudaError_t launch_count_moments(int num_pixels, int m, float thr, const float *moments, uint32_t *counts,
                                 cudaStream_t stream)
{
    const int block = 128;
    const int grid = (num_pixels + block - 1) / block;
    if (m <= 32)
        count_moments_kernel<32><<<grid, block, 0, stream>>>(num_pixels, m, thr, moments, counts);
    else if (m <= 64)
        count_moments_kernel<64><<<grid, block, 0, stream>>>(num_pixels, m, thr, moments, counts);
    else if (m <= 128)
        count_moments_kernel<128><<<grid, block, 0, stream>>>(num_pixels, m, thr, moments, counts);
    else
        count_moments_kernel<256><<<grid, block, 0, stream>>>(num_pixels, m, thr, moments, counts);
    return cudaGetLastError();
}

cudaError_t launch_prediction_encode(int num_pixels, int m, const uint32_t *index, float *data, float bias,
                                     cudaStream_t stream)
{
    const int block = 128;
    const int grid = (num_pixels + block - 1) / block;
    if (m <= 32)
        prediction_encode_kernel<32><<<grid, block, 0, stream>>>(num_pixels, m, index, data, bias);
    else if (m <= 64)
        prediction_encode_kernel<64><<<grid, block, 0, stream>>>(num_pixels, m, index, data, bias);
    else if (m <= 128)
        prediction_encode_kernel<128><<<grid, block, 0, stream>>>(num_pixels, m, index, data, bias);
    else
        prediction_encode_kernel<256><<<grid, block, 0, stream>>>(num_pixels, m, index, data, bias);
    return cudaGetLastError();
}

cudaError_t launch_prepare(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                           int coding_warp, const uint16_t *coding_params, float bias, bool fp64, float *pmoments,
                           cudaStream_t stream)
{
    if (fp64)
        return launch_prepare_m<double>(num_pixels, m, index, data, prediction_code, coding_warp, coding_params, bias,
                                        pmoments, stream);
    return launch_prepare_m<float>(num_pixels, m, index, data, prediction_code, coding_warp, coding_params, bias,
                                   pmoments, stream);
}

} // namespace mraygb
