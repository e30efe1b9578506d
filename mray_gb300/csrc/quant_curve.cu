// Data-dependent quantization curve: create_quantization_table (src/measure_coding_error.cpp:374-438; GPU form
// :280-346 with src/measure_coding_error.cu:33-262) on the sample of a compact prediction-coded moment image
// (sample_moment_image, src/moment_image_sample.h:33-62, taken by main.cpp:318-327).
//
// The reference searches the table one (index, bits) pair at a time: quantize moment idx of every sampled pixel
// to b bits, decode, convert back to trigonometric moments, average the per-pixel rRMSE, compare with the error
// threshold, and only then pick the next pair.  Each step is a few thousand pixels of sequential O(m^2) work,
// far too little to fill 152 SMs, and the chain of decisions serialises the steps.
//
// Here every pair the search can ever reach (idx in [1, m), b in [min(2, start_bits), start_bits]) is
// evaluated at once, one thread per (sampled pixel, idx) with a loop over b:
//   * qc_reference_kernel: per sampled pixel, the unquantized exponential and trigonometric moments
//     (compute_reference, src/measure_coding_error.cpp:92-141), kept as complex values;
//   * qc_error_kernel: quantizing moment idx changes nothing below idx, so the decode and the conversion restart
//     at idx from the Levinson polynomial after the first idx codes (rebuilt from the codes alone) and the stored
//     moments below idx;
//   * qc_mean_kernel: get_mean (src/measure_coding_error.cpp:184-192), the sequential float sum in the
//     reference's pixel order, one thread per pair.
// The search itself (a few hundred comparisons) then runs on the host over the table of means.
//
// The per-pixel arithmetic is the reference CPU build's, operation for operation (this file is compiled without
// FMA contraction; divisions and square roots are IEEE-rounded, cosf / sinf return the C library's results
// (libm_trig_core.h), atan2 is the double function rounded to float).  The reference's CUDA build sums the errors with
// thrust::reduce (a different order) over a count that leaves out the last pixel when it is non-empty
// (exclusive scan, measure_coding_error.cu:190-197); the CPU build's sequential mean over every non-empty pixel
// is the one followed here.

#include "internal.h"
#include "mese_device.cuh"

#include <cmath>

namespace mraygb
{
namespace
{

constexpr int kBlock = 128;
// float_complex(0.0f, 2.0f * M_PI) (MESE_dynamic.h:96): the double 2 pi rounded to float
constexpr float kTwoPiF = 6.28318530717958647692f;

struct QcArgs
{
    int sx, sy; // the sample is sx x sy pixels
    int width;  // of the image
    int fx, fy; // width / sx, height / sy
    int m;
    const uint32_t *index;
    const float *data;
    int warp;
    const uint16_t *coding_params; // 2(m-1) u16 (default warp) or null
    uint32_t *s_off;               // per sampled pixel: offset in data
    int *s_n;                      // per sampled pixel: moment count
    float2 *ref_e, *ref_t;         // [l * P + s]: exponential / trigonometric moments (complex)
    float *errors;                 // [(row * nb + bi) * P + s]
    float *means;                  // [(idx - 1) * nb + bi]
    int idx_begin;                 // first index of this pass
    int bmin, nb;                  // bits bmin .. bmin + nb - 1
};

template <int MAXM> __device__ __forceinline__ void load_params(const QcArgs &a, float *s_params)
{
    if (a.warp == 0 && a.coding_params)
        for (int i = threadIdx.x; i < 2 * (a.m - 1); i += blockDim.x)
            s_params[i] = a.coding_params[i] / 65535.f; // CodingParamType::get_param1/2 (coding_params.h:52-54)
    __syncthreads();
}

// transform_dequantization_real (moment_prediction_coding.h:97-118) for code 0: the first code and the factor
// that maps every later real residual onto the axis perpendicular to it (the operations of pc_dequant_real).
// The rRMSE is a difference of nearly equal moments, so one ulp in the first code moves a pixel's error by up to
// ~1e-2 relative at 16 bits: cosf / sinf must return the C library's results (libm_sincosf).
__device__ __forceinline__ void dequant_head(float c0, cx<float> &code0, cx<float> &factor)
{
    using K = MeseConst<float>;
    const float phase = K::pi * c0 - K::half_pi;
    float s, c;
    libm_sincosf(phase, &s, &c);
    code0 = cscale(2.f * K::inv_4pi, mk(c, s));
    const cx<float> axis = mk(-code0.y, code0.x);
    const float len = dsqrt(cabs2(axis));
    factor = cdivr(axis, len);
}

__device__ __forceinline__ cx<float> dequant_code(int l, float v, int warp, const float *params, cx<float> factor)
{
    return cscale(pc_inv_warp<float>(l, v, warp, params), factor);
}

// exponentialToTrigonometricMoments (MESE_dynamic.h:77-98), out may not alias e
template <typename A> __device__ void exp_to_trig(int n, const A &out, const A &e)
{
    using K = MeseConst<float>;
    const cx<float> g0 = cdivr((cx<float>)e[0], 2.f);
    const cx<float> t0 = cdivr(g0, K::inv_4pi);
    // atan2 on floats resolves to the C library's double function in the reference's CPU build
    const float phase = (float)atan2((double)t0.y, (double)t0.x);
    out[0] = mk((phase + K::half_pi) / K::pi, 0.f);
    const cx<float> i2pi_g0 = cmulc(mk(0.f, kTwoPiF), g0);
    for (int l = 1; l < n; ++l)
    {
        const cx<float> lg = cscale((float)l, g0);
        cx<float> acc = mk(0.f, 0.f);
        for (int j = 1; j < l; ++j)
        {
            const cx<float> d = cdiv(mk((float)(l - j), 0.f), lg);
            acc = cadd(acc, cmulc(cmulc(d, (cx<float>)e[j]), (cx<float>)out[l - j]));
        }
        out[l] = csub(cdiv((cx<float>)e[l], i2pi_g0), acc);
    }
}

__device__ __forceinline__ float2 f2(cx<float> c) { return make_float2(c.x, c.y); }
__device__ __forceinline__ cx<float> c2(float2 v) { return mk(v.x, v.y); }

// sample_moment_image's pixel (x, y) -> (x * fx, y * fy) of the image, and compute_reference's moments
template <int MAXM> __global__ void __launch_bounds__(kBlock) qc_reference_kernel(QcArgs a)
{
    __shared__ float s_params[2 * MAXM];
    load_params<MAXM>(a, s_params);
    const int P = a.sx * a.sy;
    const int s = blockIdx.x * kBlock + threadIdx.x;
    if (s >= P)
        return;
    const int x = s % a.sx, y = s / a.sx;
    const size_t src = (size_t)(y * a.fy) * (size_t)a.width + (size_t)(x * a.fx);
    const uint32_t off = a.index[src];
    int n = (int)(a.index[src + 1] - off);
    if (n > MAXM)
        n = MAXM;
    a.s_off[s] = off;
    a.s_n[s] = n;
    if (n <= 0)
        return;
    const float *in = a.data + off;
    cx<float> acode[MAXM], ae[MAXM], apoly[MAXM];
    cx<float> *code = acode, *e = ae, *poly = apoly; // the array helpers take pointers to mutable elements
    cx<float> factor;
    dequant_head(in[0], code[0], factor);
    for (int l = 1; l < n; ++l)
        code[l] = dequant_code(l, in[l], a.warp, s_params, factor);
    pc_decode<float>(n, code, e, poly);
    exp_to_trig(n, code, e);
    for (int l = 0; l < n; ++l)
    {
        a.ref_e[(size_t)l * P + s] = f2(e[l]);
        a.ref_t[(size_t)l * P + s] = f2(code[l]);
    }
}

// compute_coding_error (measure_coding_error.cpp:143-182) with moment idx quantized by apply_quantization
// (:41-47), for every b of the pass
template <int MAXM> __global__ void __launch_bounds__(kBlock) qc_error_kernel(QcArgs a)
{
    using K = MeseConst<float>;
    __shared__ float s_params[2 * MAXM];
    load_params<MAXM>(a, s_params);
    const int P = a.sx * a.sy;
    const int s = blockIdx.x * kBlock + threadIdx.x;
    const int idx = a.idx_begin + (int)blockIdx.y;
    if (s >= P)
        return;
    const int n = a.s_n[s];
    if (n <= 0)
        return;
    const float2 *re = a.ref_e + s, *rt = a.ref_t + s;
    const float ref0 = rt[0].x;
    float *err = a.errors + (size_t)blockIdx.y * a.nb * P + s;
    if (n <= idx)
    {
        // nothing quantized: every moment equals the reference's, the sum of squares is 0
        for (int bi = 0; bi < a.nb; ++bi)
            err[(size_t)bi * P] = sqrtf(0.f) / ref0;
        return;
    }
    const float *in = a.data + a.s_off[s];
    cx<float> code0, factor;
    dequant_head(in[0], code0, factor);
    const cx<float> g0 = cdivr(c2(re[0]), 2.f); // gamma_0 = exp_moments[0] / 2.f
    const cx<float> i2pi_g0 = cmulc(mk(0.f, kTwoPiF), g0);

    // decode's Levinson polynomial after codes 0 .. idx-1 (it depends on the codes only)
    cx<float> apre[MAXM], apoly[MAXM], en[MAXM], tn[MAXM];
    cx<float> *pre = apre, *poly = apoly;
    pre[0] = mk(1.f / code0.x, 0.f);
    bool invalid0 = false;
    for (int l = 1; l < idx; ++l)
    {
        cx<float> u = dequant_code(l, in[l], a.warp, s_params, factor);
        float a2 = cabs2(u);
        if (invalid0 || a2 >= (1.f - K::eps_decode))
        {
            u = mk(0.f, 0.f);
            a2 = 0.f;
            invalid0 = true;
        }
        levinson_update<float>(l, pre, u, 1.f / (1.f - a2));
    }
    const float qv = in[idx];

    for (int bi = 0; bi < a.nb; ++bi)
    {
        const int b = a.bmin + bi;
        const float p = ldexpf(1.f, b);
        for (int k = 0; k < idx; ++k)
            poly[k] = pre[k];
        bool invalid = invalid0;
        // decode (moment_prediction_coding.h:163-208) from step idx on; en[l - idx] = exponential moment l
        for (int l = idx; l < n; ++l)
        {
            const float v = (l == idx) ? floorf(qv * p) / p : in[l];
            cx<float> u = dequant_code(l, v, a.warp, s_params, factor);
            float a2 = cabs2(u);
            if (invalid || a2 >= (1.f - K::eps_decode))
            {
                u = mk(0.f, 0.f);
                a2 = 0.f;
                invalid = true;
            }
            cx<float> gamma = mk(0.f, 0.f);
            const int ksplit = l - idx; // k <= ksplit: e[l - k] is a new moment
            for (int k = 1; k < l; ++k)
            {
                const cx<float> ek = (k <= ksplit) ? en[l - k - idx] : c2(re[(size_t)(l - k) * P]);
                gamma = cadd(gamma, cmulc(poly[k], ek));
            }
            en[l - idx] = cmulc(cdiv(mk(1.f, 0.f), poly[0]), csub(u, gamma));
            levinson_update<float>(l, poly, u, 1.f / (1.f - a2));
        }
        // exponentialToTrigonometricMoments from moment idx on; tn[l - idx] = trigonometric moment l
        float sum = 0.f;
        for (int l = idx; l < n; ++l)
        {
            const cx<float> lg = cscale((float)l, g0);
            cx<float> acc = mk(0.f, 0.f);
            const int jsplit = l - idx; // j <= jsplit: out[l - j] is a new moment
            for (int j = 1; j < l; ++j)
            {
                const cx<float> d = cdiv(mk((float)(l - j), 0.f), lg);
                const cx<float> ej = (j >= idx) ? en[j - idx] : c2(re[(size_t)j * P]);
                const cx<float> tj = (j <= jsplit) ? tn[l - j - idx] : c2(rt[(size_t)(l - j) * P]);
                acc = cadd(acc, cmulc(cmulc(d, ej), tj));
            }
            const cx<float> t = csub(cdiv(en[l - idx], i2pi_g0), acc);
            tn[l - idx] = t;
            const float diff = rt[(size_t)l * P].x - t.x;
            sum = sum + diff * diff;
        }
        err[(size_t)bi * P] = sqrtf(sum) / ref0;
    }
}

// get_mean (measure_coding_error.cpp:184-192): the sequential sum over the non-empty pixels in row-major order
__global__ void qc_mean_kernel(QcArgs a, int pairs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pairs)
        return;
    const int P = a.sx * a.sy;
    const float *err = a.errors + (size_t)t * P;
    float sum = 0.f;
    uint32_t count = 0;
    for (int s = 0; s < P; ++s)
        if (a.s_n[s] > 0)
        {
            sum = sum + err[s];
            ++count;
        }
    a.means[(size_t)(a.idx_begin - 1) * a.nb + t] = sum / (float)count;
}

template <int MAXM>
cudaError_t run_curve(const QcArgs &base, size_t rows_per_pass, cudaStream_t stream, int *launches)
{
    const int P = base.sx * base.sy;
    const unsigned blocks = (unsigned)((P + kBlock - 1) / kBlock);
    qc_reference_kernel<MAXM><<<blocks, kBlock, 0, stream>>>(base);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    *launches += 1;
    for (int begin = 1; begin < base.m; begin += (int)rows_per_pass)
    {
        const int rows = (int)std::min<size_t>(rows_per_pass, (size_t)(base.m - begin));
        QcArgs a = base;
        a.idx_begin = begin;
        qc_error_kernel<MAXM><<<dim3(blocks, (unsigned)rows), kBlock, 0, stream>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        const int pairs = rows * a.nb;
        qc_mean_kernel<<<(pairs + 63) / 64, 64, 0, stream>>>(a, pairs);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        *launches += 2;
    }
    return cudaSuccess;
}

} // namespace

cudaError_t quant_curve_init_constants(const LibmTrigTable &trig) { return set_libm_trig_constants(trig); }

size_t quant_curve_scratch_bytes(int sx, int sy, int m, int nb, size_t rows_per_pass)
{
    const size_t P = (size_t)sx * (size_t)sy;
    return P * (sizeof(uint32_t) + sizeof(int)) + 2 * P * (size_t)m * sizeof(float2) +
           rows_per_pass * (size_t)nb * P * sizeof(float) + (size_t)m * (size_t)nb * sizeof(float) + 256 * 6;
}

cudaError_t launch_quant_curve(int width, int height, int m, const uint32_t *index, const float *data, int warp,
                               const uint16_t *coding_params, int sx, int sy, int bmin, int nb,
                               size_t rows_per_pass, void *scratch, float *d_means, cudaStream_t stream, int *launches)
{
    const size_t P = (size_t)sx * (size_t)sy;
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    char *p = static_cast<char *>(scratch);
    QcArgs a{};
    a.sx = sx;
    a.sy = sy;
    a.width = width;
    a.fx = width / sx;
    a.fy = height / sy;
    a.m = m;
    a.index = index;
    a.data = data;
    a.warp = warp;
    a.coding_params = coding_params;
    a.s_off = reinterpret_cast<uint32_t *>(p);
    p += align(P * sizeof(uint32_t));
    a.s_n = reinterpret_cast<int *>(p);
    p += align(P * sizeof(int));
    a.ref_e = reinterpret_cast<float2 *>(p);
    p += align(P * (size_t)m * sizeof(float2));
    a.ref_t = reinterpret_cast<float2 *>(p);
    p += align(P * (size_t)m * sizeof(float2));
    a.errors = reinterpret_cast<float *>(p);
    a.means = d_means;
    a.idx_begin = 1;
    a.bmin = bmin;
    a.nb = nb;
    if (m <= 32)
        return run_curve<32>(a, rows_per_pass, stream, launches);
    if (m <= 64)
        return run_curve<64>(a, rows_per_pass, stream, launches);
    if (m <= 128)
        return run_curve<128>(a, rows_per_pass, stream, launches);
    return run_curve<256>(a, rows_per_pass, stream, launches);
}

} // namespace mraygb
