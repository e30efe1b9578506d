// Per-pixel bounded-MESE algebra on the device, generic over float / double.
//
// The float instantiation performs the reference's operations in the reference's order (these kernels are
// compiled without FMA contraction), so its results differ from the reference's CPU build only where CUDA's
// cosf / sinf round differently from the C library's.  The double instantiation is the same method in FP64
// with exact constants (the precision form).
//
//   trigonometricToExponentialMoments  src/mese/MESE_dynamic.h:35-54
//   levinsonsAlgorithm                 src/mese/MESE_dynamic.h:100-135
//   computeAutocorrelation             src/mese/MESE_dynamic.h:137-147
//   computeImaginaryCorrelation        src/mese/MESE_dynamic.h:161-171
//   prepareMESELagrange                src/mese/MESE_dynamic.h:194-211
//   encode / decode                    src/moment_prediction_coding.h:123-208
//   transform_(de)quantization_real    src/moment_prediction_coding.h:81-118
//   prediction_coding_(inv_)warp       src/moment_prediction_coding.h:47-67
//   evaluate_unknown_moments, exponential_to_bounded_moments, rmse, determine_best_number_moments
//                                      src/moment_compaction.h:35-142
#pragma once

#include <cuda_runtime.h>

namespace mraygb
{

template <typename T> struct cx
{
    T x, y;
};

template <typename T> struct MeseConst;
template <> struct MeseConst<float>
{
    static constexpr float pi = 3.14159265f;
    static constexpr float half_pi = 1.57079633f;
    static constexpr float inv_4pi = 0.0795774715f;
    static constexpr float two_pi = 6.28318531f;
    static constexpr float pi_l = 3.14159274101257324f; // (float)M_PI
    static constexpr float eps_decode = 1e-6f;
    static constexpr float rrmse_tie = 1e-8f;
};
template <> struct MeseConst<double>
{
    static constexpr double pi = 3.14159265358979323846;
    static constexpr double half_pi = 1.57079632679489661923;
    static constexpr double inv_4pi = 0.07957747154594766788;
    static constexpr double two_pi = 6.28318530717958647692;
    static constexpr double pi_l = 3.14159265358979323846;
    static constexpr double eps_decode = 1e-6;
    static constexpr double rrmse_tie = 1e-8;
};

__device__ __forceinline__ void dsincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void dsincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }

template <typename T> __device__ __forceinline__ cx<T> mk(T x, T y) { return {x, y}; }
template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T> __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T> __device__ __forceinline__ cx<T> cconj(cx<T> a) { return {a.x, -a.y}; }
template <typename T> __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// real * complex
template <typename T> __device__ __forceinline__ cx<T> cscale(T s, cx<T> z) { return {s * z.x, s * z.y}; }
// complex * real through float_complex(real) (a full complex product, as the reference computes it)
template <typename T> __device__ __forceinline__ cx<T> cmulr(cx<T> a, T b) { return cmulc(a, mk<T>(b, T(0))); }
template <typename T> __device__ __forceinline__ T cabs2(cx<T> z) { return z.x * z.x + z.y * z.y; }
template <typename T> __device__ __forceinline__ cx<T> cdiv(cx<T> n, cx<T> d)
{
    T f = T(1) / cabs2(d);
    return {(n.x * d.x + n.y * d.y) * f, (-n.x * d.y + n.y * d.x) * f};
}
template <typename T> __device__ __forceinline__ cx<T> cdivr(cx<T> n, T d)
{
    T f = T(1) / d;
    return {n.x * f, n.y * f};
}
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return (a < b) ? a : b; }
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return (a > b) ? a : b; }
template <typename T> __device__ __forceinline__ T tclamp(T v, T lo, T hi) { return tmin(tmax(v, lo), hi); }

// trigonometricToExponentialMoments (float* trig overload)
// two_pi_over_l[l] = float_complex(0, 2.0f * M_PI / float(l)).y: the reference's double quotient rounded to T
template <typename T, typename TrigArr>
__device__ void trig_to_exp(int n, cx<T> *e, const TrigArr &trig, const T *two_pi_over_l)
{
    using K = MeseConst<T>;
    T phase = K::pi * T(trig[0]) - K::half_pi;
    T s, c;
    dsincos(phase, &s, &c);
    e[0] = cscale(K::inv_4pi, mk(c, s));
    for (int l = 1; l < n; ++l)
    {
        cx<T> acc = mk<T>(0, 0);
        for (int j = 0; j < l; ++j)
            acc = cadd(acc, cmulr(cscale(T(l - j), e[j]), T(trig[l - j])));
        e[l] = cmulc(acc, mk<T>(0, two_pi_over_l[l]));
    }
    e[0] = cscale(T(2), e[0]);
}

template <typename T> __device__ void levinson(int n, cx<T> *sol, const cx<T> *col, cx<T> *tmp)
{
    sol[0] = mk<T>(T(1) / col[0].x, 0);
    bool invalid = false;
    for (int j = 1; j < n; ++j)
    {
        cx<T> u = mk<T>(0, 0);
        if (!invalid)
            for (int k = 0; k < j; ++k)
                u = cadd(u, cmulc(sol[k], col[j - k]));
        T a2 = cabs2(u);
        if (a2 >= T(1))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        const T factor = T(1) / (T(1) - a2);
        for (int k = 1; k < j; ++k)
            tmp[k] = cconj(sol[j - k]);
        tmp[j] = mk<T>(sol[0].x, 0);
        sol[0] = mk<T>(factor * sol[0].x, 0);
        for (int k = 1; k < j; ++k)
            sol[k] = cscale(factor, csub(sol[k], cmulc(tmp[k], u)));
        sol[j] = cscale(factor, cscale(-tmp[j].x, u));
    }
}

template <typename T> __device__ void autocorr(int n, cx<T> *out, const cx<T> *s)
{
    for (int k = 0; k < n; ++k)
    {
        cx<T> acc = mk<T>(0, 0);
        for (int j = 0; j < n - k; ++j)
            acc = cadd(acc, cmulc(s[j], cconj(s[j + k])));
        out[k] = acc;
    }
}

// computeImaginaryCorrelation, written straight to an output of type O
template <typename T, typename O> __device__ void imag_corr_scaled(int n, O *out, const cx<T> *lhs, const cx<T> *rhs,
                                                                   T norm)
{
    for (int k = 0; k < n; ++k)
    {
        T acc = 0;
        for (int j = 0; j < n - k; ++j)
            acc += lhs[k + j].x * rhs[j].y + lhs[k + j].y * rhs[j].x;
        out[k] = O(norm * acc);
    }
}

// the shared tail of prepareMESELagrange / prepare_moments_from_pred_coding: poly (Levinson solution) and
// exp (exponential moments) in, Lagrange multipliers out
template <typename T, typename O>
__device__ void lagrange_from_poly(int n, cx<T> *poly, cx<T> *e, cx<T> *tmp, O *out)
{
    using K = MeseConst<T>;
    for (int i = 0; i < n; ++i)
        poly[i] = cscale(K::two_pi, poly[i]);
    autocorr(n, tmp, poly);
    e[0] = cscale(T(0.5), e[0]);
    const T norm = T(1) / (K::pi * poly[0].x);
    imag_corr_scaled(n, out, tmp, e, norm);
}

// encode (moment_prediction_coding.h:123-158)
template <typename T> __device__ void pc_encode(int n, const cx<T> *e, cx<T> *code, cx<T> *poly, cx<T> *tmp)
{
    code[0] = e[0];
    poly[0] = mk<T>(T(1) / e[0].x, 0);
    bool invalid = false;
    for (int l = 1; l < n; ++l)
    {
        cx<T> u = mk<T>(0, 0);
        for (int k = 0; k < l; ++k)
            u = cadd(u, cmulc(poly[k], e[l - k]));
        code[l] = u;
        T a2 = cabs2(u);
        if (invalid || a2 >= T(1))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        const T factor = T(1) / (T(1) - a2);
        for (int k = 1; k < l; ++k)
            tmp[k] = cconj(poly[l - k]);
        tmp[l] = mk<T>(poly[0].x, 0);
        poly[0] = mk<T>(factor * poly[0].x, 0);
        for (int k = 1; k < l; ++k)
            poly[k] = cscale(factor, csub(poly[k], cmulc(tmp[k], u)));
        poly[l] = cscale(factor, cscale(-tmp[l].x, u));
    }
}

// decode (moment_prediction_coding.h:163-208)
template <typename T> __device__ void pc_decode(int n, const cx<T> *code, cx<T> *e, cx<T> *poly, cx<T> *tmp)
{
    using K = MeseConst<T>;
    e[0] = code[0];
    poly[0] = mk<T>(T(1) / e[0].x, 0);
    bool invalid = false;
    for (int l = 1; l < n; ++l)
    {
        cx<T> u = code[l];
        T a2 = cabs2(u);
        if (invalid || a2 >= (T(1) - K::eps_decode))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        cx<T> gamma = mk<T>(0, 0);
        for (int k = 1; k < l; ++k)
            gamma = cadd(gamma, cmulc(poly[k], e[l - k]));
        e[l] = cmulc(cdiv(mk<T>(1, 0), poly[0]), csub(u, gamma));
        const T factor = T(1) / (T(1) - a2);
        for (int k = 1; k < l; ++k)
            tmp[k] = cconj(poly[l - k]);
        tmp[l] = mk<T>(poly[0].x, 0);
        poly[0] = mk<T>(factor * poly[0].x, 0);
        for (int k = 1; k < l; ++k)
            poly[k] = cscale(factor, csub(poly[k], cmulc(tmp[k], u)));
        poly[l] = cscale(factor, cscale(-tmp[l].x, u));
    }
}

// prediction_coding_warp / prediction_coding_inv_warp; params are the dequantized u16 coding parameters
__device__ __forceinline__ float pc_warp(int l, float x, int warp, const float *p)
{
    float w;
    if (warp == 0)
        w = (x + p[(l - 1) * 2]) / (p[(l - 1) * 2 + 1] * 2.f);
    else
        w = x * 0.5f + 0.5f;
    return tclamp(w, 0.f, 1.f);
}
template <typename T> __device__ __forceinline__ T pc_inv_warp(int l, T x, int warp, const float *p)
{
    if (warp == 0)
        return (x * T(p[(l - 1) * 2 + 1]) * T(2)) - T(p[(l - 1) * 2]);
    return x * T(2) - T(1);
}

// transform_dequantization_real
template <typename T>
__device__ void pc_dequant_real(int n, const float *in, cx<T> *out, int warp, const float *params)
{
    using K = MeseConst<T>;
    const T c0 = T(in[0]);
    const T phase = K::pi * c0 - K::half_pi;
    T s, c;
    dsincos(phase, &s, &c);
    out[0] = cscale(T(2) * K::inv_4pi, mk(c, s));
    const cx<T> axis = mk(-out[0].y, out[0].x);
    const T len = dsqrt(cabs2(axis));
    const cx<T> factor = cdivr(axis, len);
    for (int l = 1; l < n; ++l)
        out[l] = cscale(pc_inv_warp<T>(l, T(in[l]), warp, params), factor);
}

} // namespace mraygb
