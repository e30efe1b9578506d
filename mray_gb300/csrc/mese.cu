// Per-pixel MESE kernels: Lagrange-multiplier preparation (standard and prediction-coded moments, FP32 or
// FP64) and the error-threshold moment count of compaction.  Built without FMA contraction so that the FP32
// form performs the reference's roundings (see mese_device.cuh).
//
//   prepare_moments_from_std_coding   src/moment_preparation.h:55-64 (bias lerp + prepareMESELagrange)
//   prepare_moments_from_pred_coding  src/moment_preparation.h:32-53
//   determine_best_number_moments     src/moment_compaction.h:113-142 (with :35-111)
//
// One thread per pixel; the O(m^2) recursions work on per-thread arrays of m complex values held in
// thread-strided shared memory (element k of thread t at k * BLOCK + t: conflict-free, no local-memory spills).

#include "mese_kernels.cuh"

namespace mraygb
{

namespace
{

// ---- error-threshold compaction (float, the reference's arithmetic) ---------------------------------------

template <typename A> __device__ void eval_unknown(int num, const A &e, int max_moments, const A &new_e, const A &lev)
{
    const int mm = max_moments - 1;
    const int n = num - 1;
    levinson<float>(num, lev, e);
    for (int i = 0; i < n + 1; ++i)
        lev[i] = cscale(MeseConst<float>::two_pi, (cx<float>)lev[i]);
    for (int l = 0; l < n + 1; ++l)
        new_e[l] = (cx<float>)e[l];
    const cx<float> inv_lev0 = cdiv(mk<float>(-1.f, 0.f), (cx<float>)lev[0]);
    for (int k = 0; k < mm - n; ++k)
    {
        cx<float> a = mk<float>(0, 0);
        for (int j = 1; j < n + 1; ++j)
            a = cadd(a, cmulc((cx<float>)new_e[j + k], (cx<float>)lev[n + 1 - j]));
        new_e[n + k + 1] = cmulc(a, inv_lev0);
    }
}

// exponential_to_bounded_moments: the reference multiplies by exp_moments[l] inside the sum (kept as is)
template <typename A> __device__ void exp_to_bounded(int num, const A &e, const A &b, int n)
{
    const cx<float> gamma_0 = cdivr((cx<float>)e[0], 2.f);
    // float_complex(0, 2) * M_PI * gamma_0: M_PI converts to float_complex((float)M_PI)
    const cx<float> i2pi = cmulc(mk<float>(0.f, 2.f), mk<float>(MeseConst<float>::pi_l, 0.f));
    for (int l = n; l < num; ++l)
    {
        b[l] = mk<float>(0, 0);
        for (int j = 0; j < l; ++j)
        {
            const cx<float> dq = cdiv(mk<float>((float)(l - j), 0.f), cscale((float)l, gamma_0));
            b[l] = cadd((cx<float>)b[l], cmulc(cmulc(dq, (cx<float>)e[l]), (cx<float>)b[l - j]));
        }
        b[l] = csub(cdiv((cx<float>)e[l], cmulc(i2pi, gamma_0)), (cx<float>)b[l]);
    }
}

// determine_best_number_moments for the pixels whose count is non-zero
template <int MAXM, int BLOCK>
__global__ void __launch_bounds__(BLOCK) count_moments_kernel(int num_pixels, int m, float thr,
                                                              const float *__restrict__ moments,
                                                              uint32_t *__restrict__ counts)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int p = blockIdx.x * BLOCK + threadIdx.x;
    if (p >= num_pixels || counts[p] == 0)
        return;
    const float *mo = moments + (size_t)p * (size_t)m;
    cx<float> *base = reinterpret_cast<cx<float> *>(smem);
    const Strided<cx<float>, BLOCK> te{base + threadIdx.x};
    const Strided<cx<float>, BLOCK> text{base + MAXM * BLOCK + threadIdx.x};
    const Strided<cx<float>, BLOCK> tlev{base + 2 * MAXM * BLOCK + threadIdx.x};
    const float norm = 1.0f / mo[0];
    trig_to_exp<float>(m, te, mo, two_pi_over_l<float>());
    int n = m / 2;
    int s = m / 4;
    while (s > 0)
    {
        eval_unknown(n, te, m, text, tlev);
        const Strided<cx<float>, BLOCK> &ext = tlev;
        for (int l = 0; l < n; ++l)
            ext[l] = mk<float>(mo[l], 0.f);
        exp_to_bounded(m, text, ext, n);
        float sum = 0.f;
        for (int k = n; k < m; ++k)
        {
            const float diff = ((cx<float>)ext[k]).x - mo[k];
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
template <int MAXM, int BLOCK>
__global__ void __launch_bounds__(BLOCK) prediction_encode_kernel(int num_pixels, int m,
                                                                  const uint32_t *__restrict__ index,
                                                                  float *__restrict__ data, float bias)
{
    extern __shared__ __align__(16) unsigned char smem[];
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
    float *d = data + idx;
    d[0] = (1 - bias) * d[0] + bias * 0.5f; // cut::lerp(data[idx], 0.5f, bias)
    for (int i = 1; i < n; ++i)
        d[i] = (1 - bias) * d[i] + bias * 0.0f;
    cx<float> *base = reinterpret_cast<cx<float> *>(smem);
    const Strided<cx<float>, BLOCK> e{base + threadIdx.x};
    const Strided<cx<float>, BLOCK> poly{base + MAXM * BLOCK + threadIdx.x};
    trig_to_exp<float>(n, e, d, two_pi_over_l<float>());
    // transform_quantization_real (moment_prediction_coding.h:81-92) on the code as encode produces it: out[0] =
    // c_0 stays d[0]; the axis comes from code_0 = e_0.  The trigonometric moments in d are no longer read once
    // the exponential moments exist, so each residual can overwrite its moment at once (no code array).
    const cx<float> c0 = e[0];
    const cx<float> axis = mk(-c0.y, c0.x);
    const float len = sqrtf(cabs2(axis));
    const cx<float> inv_axis = cdiv(mk(len, 0.f), axis);
    pc_encode<float>(n, e, poly, [&](int l, cx<float> code_l) { d[l] = cmulc(code_l, inv_axis).x; });
}

__global__ void libm_sincosf_kernel(uint64_t n, const float *__restrict__ x, float *__restrict__ s,
                                    float *__restrict__ c)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        float sv, cv;
        libm_sincosf(x[i], &sv, &cv);
        s[i] = sv;
        c[i] = cv;
    }
}

template <int MAXM>
cudaError_t launch_count_t(int num_pixels, int m, float thr, const float *moments, uint32_t *counts,
                           cudaStream_t stream)
{
    constexpr int per = smem_per_thread<float, MAXM, 3, 0>();
    constexpr int block = block_for<per>();
    constexpr int bytes = per * block;
    cudaError_t e = cudaFuncSetAttribute(count_moments_kernel<MAXM, block>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess)
        return e;
    count_moments_kernel<MAXM, block><<<(num_pixels + block - 1) / block, block, bytes, stream>>>(num_pixels, m, thr,
                                                                                              moments, counts);
    return cudaGetLastError();
}

template <int MAXM>
cudaError_t launch_encode_t(int num_pixels, int m, const uint32_t *index, float *data, float bias, cudaStream_t stream)
{
    constexpr int per = smem_per_thread<float, MAXM, 2, 0>();
    constexpr int block = block_for<per>();
    constexpr int bytes = per * block;
    cudaError_t e = cudaFuncSetAttribute(prediction_encode_kernel<MAXM, block>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess)
        return e;
    // the whole shared-memory carveout: the resident pixels are what this latency-bound kernel lives on
    if ((e = cudaFuncSetAttribute(prediction_encode_kernel<MAXM, block>,
                                  cudaFuncAttributePreferredSharedMemoryCarveout, 100)) != cudaSuccess)
        return e;
    prediction_encode_kernel<MAXM, block><<<(num_pixels + block - 1) / block, block, bytes, stream>>>(
        num_pixels, m, index, data, bias);
    return cudaGetLastError();
}

// The differentiation form's preparation: the FP32 kernel's arithmetic on the uncompacted W*H*m image (so the same
// multipliers), and in `keep` the two arrays of each pixel that the preparation adjoint reads, as 2m float2: P = 2 pi
// x with x the Levinson solution (exactly zero from a latched step on, where the Herglotz check failed), then the
// exponential moments with the zeroth halved.  Both are what lagrange_from_poly leaves in the pixel's arrays.  The
// arrays' stride is BLOCK + 1 elements, so that the block's copy-out (one pixel's elements in a row, then the next
// pixel's: the block's kept arrays are one contiguous run) reads shared memory with at most two-way conflicts and
// writes global memory coalesced.
template <int MAXM, int BLOCK> constexpr int keep_smem_bytes()
{
    return MAXM * (BLOCK + 1) * (2 * (int)sizeof(cx<float>) + (int)sizeof(float));
}

template <int MAXM, int BLOCK>
__global__ void __launch_bounds__(BLOCK) prepare_keep_kernel(int num_pixels, int m, const float *__restrict__ data,
                                                             float bias, float *__restrict__ out,
                                                             float2 *__restrict__ keep)
{
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int S = BLOCK + 1;
    const int p = blockIdx.x * BLOCK + threadIdx.x;
    const int n = m < MAXM ? m : MAXM;
    cx<float> *base = reinterpret_cast<cx<float> *>(smem);
    const Strided<cx<float>, S> e{base + threadIdx.x};
    const Strided<cx<float>, S> poly{base + MAXM * S + threadIdx.x};
    const Strided<float, S> acc{reinterpret_cast<float *>(base + 2 * MAXM * S) + threadIdx.x};
    if (p < num_pixels)
        prepare_pixel<float, MAXM, BLOCK, false>(n, data + (size_t)p * (size_t)m, e, poly, acc, 0, nullptr, bias,
                                                 out + (size_t)p * (size_t)m);
    __syncthreads();
    const int p0 = blockIdx.x * BLOCK;
    const int np = min(BLOCK, num_pixels - p0);
    const int per = 2 * n;
    float2 *dst = keep + (size_t)p0 * (size_t)per;
    for (int i = threadIdx.x; i < np * per; i += BLOCK)
    {
        const int t = i / per, k = i - t * per;
        const cx<float> v = k < n ? base[MAXM * S + k * S + t] : base[(k - n) * S + t];
        dst[i] = make_float2(v.x, v.y);
    }
}

template <int MAXM>
cudaError_t launch_keep_t(int num_pixels, int m, const float *data, float bias, float *out, float2 *keep,
                          cudaStream_t stream)
{
    constexpr int block = block_for<smem_per_thread<float, MAXM, 2, 1>()>();
    constexpr int bytes = keep_smem_bytes<MAXM, block>();
    cudaError_t e = cudaFuncSetAttribute(prepare_keep_kernel<MAXM, block>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         bytes);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(prepare_keep_kernel<MAXM, block>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  100)) != cudaSuccess)
        return e;
    prepare_keep_kernel<MAXM, block><<<(num_pixels + block - 1) / block, block, bytes, stream>>>(num_pixels, m, data,
                                                                                              bias, out, keep);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_prepare_keep(int num_pixels, int m, const float *data, float bias, float *pmoments, float2 *keep,
                                cudaStream_t stream)
{
    if (m <= 32)
        return launch_keep_t<32>(num_pixels, m, data, bias, pmoments, keep, stream);
    return launch_keep_t<64>(num_pixels, m, data, bias, pmoments, keep, stream);
}

cudaError_t mese_init_constants()
{
    LibmTrigTable trig;
    cudaError_t e = libm_trig_device_table(&trig);
    if (e != cudaSuccess)
        return e;
    if ((e = init_tables()) != cudaSuccess)
        return e;
    if ((e = set_libm_trig_constants(trig)) != cudaSuccess)
        return e;
    if ((e = mese_ff_init_constants(trig)) != cudaSuccess)
        return e;
    if ((e = quant_curve_init_constants(trig)) != cudaSuccess)
        return e;
    return mese_f64_init_constants(trig);
}

cudaError_t launch_libm_sincosf(uint64_t n, const float *x, float *s, float *c, cudaStream_t stream)
{
    if (n == 0)
        return cudaSuccess;
    const uint64_t blocks = (n + 255) / 256;
    libm_sincosf_kernel<<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, stream>>>(n, x, s, c);
    return cudaGetLastError();
}

cudaError_t launch_count_moments(int num_pixels, int m, float thr, const float *moments, uint32_t *counts,
                                 cudaStream_t stream)
{
    if (m <= 32)
        return launch_count_t<32>(num_pixels, m, thr, moments, counts, stream);
    if (m <= 64)
        return launch_count_t<64>(num_pixels, m, thr, moments, counts, stream);
    if (m <= 128)
        return launch_count_t<128>(num_pixels, m, thr, moments, counts, stream);
    return launch_count_t<256>(num_pixels, m, thr, moments, counts, stream);
}

cudaError_t launch_prediction_encode(int num_pixels, int m, const uint32_t *index, float *data, float bias,
                                     cudaStream_t stream)
{
    if (m <= 32)
        return launch_encode_t<32>(num_pixels, m, index, data, bias, stream);
    if (m <= 64)
        return launch_encode_t<64>(num_pixels, m, index, data, bias, stream);
    if (m <= 128)
        return launch_encode_t<128>(num_pixels, m, index, data, bias, stream);
    return launch_encode_t<256>(num_pixels, m, index, data, bias, stream);
}

cudaError_t launch_prepare(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                           int coding_warp, const uint16_t *coding_params, float bias, bool fp64, float *pmoments,
                           cudaStream_t stream)
{
    if (fp64)
        return launch_prepare_f64(num_pixels, m, index, data, prediction_code, coding_warp, coding_params, bias,
                                  pmoments, stream);
    return launch_prepare_m<float>(num_pixels, m, index, data, prediction_code, coding_warp, coding_params, bias,
                                   pmoments, stream);
}

} // namespace mraygb
