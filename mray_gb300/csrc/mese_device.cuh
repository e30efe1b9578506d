// Per-pixel bounded-MESE algebra on the device, generic over float / double and over the array type.
//
// The float instantiation performs the reference's operations in the reference's order (these kernels are
// compiled without FMA contraction), and its cosf / sinf return the host C library's results
// (libm_trig_core.h), so its results equal the reference's CPU build bit for bit.  The double instantiation is
// the same method in FP64 with exact constants (the precision form).
//
// Arrays are accessed through an index operator only: the kernels pass thread-strided views of shared memory
// (element k of thread t at k * BLOCK + t, so a warp reading element k touches 32 consecutive words).
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

#include "libm_trig.cuh"

namespace mraygb
{

template <typename T> struct cx
{
    T x, y;
};

// element k of a thread's array in thread-strided shared memory
template <typename E, int STRIDE> struct Strided
{
    E *p;
    __device__ __forceinline__ E &operator[](int k) const { return p[k * STRIDE]; }
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

__device__ __forceinline__ void dsincos(float x, float *s, float *c) { libm_sincosf(x, s, c); }
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
template <typename T, typename A, typename TrigArr>
__device__ void trig_to_exp(int n, const A &e, const TrigArr &trig, const T *two_pi_over_l)
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
            acc = cadd(acc, cmulr(cscale(T(l - j), (cx<T>)e[j]), T(trig[l - j])));
        e[l] = cmulc(acc, mk<T>(0, two_pi_over_l[l]));
    }
    e[0] = cscale(T(2), (cx<T>)e[0]);
}

// One Levinson-style update of the solution / evaluation polynomial in place: with the old values o,
//   new[0] = f o[0].x,  new[k] = f (o[k] - conj(o[j-k]) u) (0 < k < j),  new[j] = f (-o[0].x u).
// The reference copies the flipped solution to a temporary first; updating the pairs (k, j-k) together needs
// no copy and performs the same operations on the same values.
template <typename T, typename A> __device__ __forceinline__ void levinson_update(int j, const A &sol, cx<T> u, T f)
{
    const T s0 = ((cx<T>)sol[0]).x;
    int k = 1, kk = j - 1;
    for (; k < kk; ++k, --kk)
    {
        const cx<T> a = sol[k], b = sol[kk];
        sol[k] = cscale(f, csub(a, cmulc(cconj(b), u)));
        sol[kk] = cscale(f, csub(b, cmulc(cconj(a), u)));
    }
    if (k == kk)
    {
        const cx<T> a = sol[k];
        sol[k] = cscale(f, csub(a, cmulc(cconj(a), u)));
    }
    sol[j] = cscale(f, cscale(-s0, u));
    sol[0] = mk<T>(f * s0, 0);
}

template <typename T, typename A, typename C> __device__ void levinson(int n, const A &sol, const C &col)
{
    sol[0] = mk<T>(T(1) / ((cx<T>)col[0]).x, 0);
    bool invalid = false;
    for (int j = 1; j < n; ++j)
    {
        cx<T> u = mk<T>(0, 0);
        if (!invalid)
            for (int k = 0; k < j; ++k)
                u = cadd(u, cmulc((cx<T>)sol[k], (cx<T>)col[j - k]));
        T a2 = cabs2(u);
        if (a2 >= T(1))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        levinson_update<T>(j, sol, u, T(1) / (T(1) - a2));
    }
}

// the tail of prepareMESELagrange / prepare_moments_from_pred_coding: poly (the Levinson solution, scaled by
// 2 pi here) and e (the exponential moments, e[0] halved here) in, Lagrange multipliers out.  The autocorrelation
// of poly (computeAutocorrelation) is formed one lag q at a time and scattered straight into the imaginary
// correlation with e (computeImaginaryCorrelation): out[k] accumulates its terms in the order of q = k + j,
// the reference's order, so no autocorrelation array is needed.
template <typename T, typename A, typename O>
__device__ void lagrange_from_poly(int n, const A &poly, const A &e, const O &acc)
{
    using K = MeseConst<T>;
    for (int i = 0; i < n; ++i)
        poly[i] = cscale(K::two_pi, (cx<T>)poly[i]);
    e[0] = cscale(T(0.5), (cx<T>)e[0]);
    for (int k = 0; k < n; ++k)
        acc[k] = T(0);
    for (int q = 0; q < n; ++q)
    {
        cx<T> a = mk<T>(0, 0);
        for (int j = 0; j < n - q; ++j)
            a = cadd(a, cmulc((cx<T>)poly[j], cconj((cx<T>)poly[j + q])));
        for (int k = 0; k <= q; ++k)
        {
            const cx<T> ej = e[q - k];
            acc[k] = T(acc[k]) + (a.x * ej.y + a.y * ej.x);
        }
    }
}

// encode (moment_prediction_coding.h:123-158).  code[0] = e[0]; code[l] for l >= 1 goes to sink(l, code_l) as
// soon as it is known (the caller stores or transforms it; nothing later reads it back).
template <typename T, typename A, typename Sink> __device__ void pc_encode(int n, const A &e, const A &poly, Sink &&sink)
{
    poly[0] = mk<T>(T(1) / ((cx<T>)e[0]).x, 0);
    bool invalid = false;
    for (int l = 1; l < n; ++l)
    {
        cx<T> u = mk<T>(0, 0);
        for (int k = 0; k < l; ++k)
            u = cadd(u, cmulc((cx<T>)poly[k], (cx<T>)e[l - k]));
        sink(l, u);
        T a2 = cabs2(u);
        if (invalid || a2 >= T(1))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        levinson_update<T>(l, poly, u, T(1) / (T(1) - a2));
    }
}

// decode (moment_prediction_coding.h:163-208); code(l) yields code l (each is asked for once, in order)
template <typename T, typename A, typename Code>
__device__ void pc_decode_from(int n, Code &&code, const A &e, const A &poly)
{
    using K = MeseConst<T>;
    e[0] = code(0);
    poly[0] = mk<T>(T(1) / ((cx<T>)e[0]).x, 0);
    bool invalid = false;
    for (int l = 1; l < n; ++l)
    {
        cx<T> u = code(l);
        T a2 = cabs2(u);
        if (invalid || a2 >= (T(1) - K::eps_decode))
        {
            u = mk<T>(0, 0);
            a2 = 0;
            invalid = true;
        }
        cx<T> gamma = mk<T>(0, 0);
        for (int k = 1; k < l; ++k)
            gamma = cadd(gamma, cmulc((cx<T>)poly[k], (cx<T>)e[l - k]));
        e[l] = cmulc(cdiv(mk<T>(1, 0), (cx<T>)poly[0]), csub(u, gamma));
        levinson_update<T>(l, poly, u, T(1) / (T(1) - a2));
    }
}

template <typename T, typename A> __device__ void pc_decode(int n, const A &code, const A &e, const A &poly)
{
    pc_decode_from<T>(n, [&](int l) { return (cx<T>)code[l]; }, e, poly);
}

// prediction_coding_inv_warp; params are the dequantized u16 coding parameters
template <typename T> __device__ __forceinline__ T pc_inv_warp(int l, T x, int warp, const float *p)
{
    if (warp == 0)
        return (x * T(p[(l - 1) * 2 + 1]) * T(2)) - T(p[(l - 1) * 2]);
    return x * T(2) - T(1);
}

// transform_dequantization_real, one code at a time: code 0 and the factor that maps every later real residual
// onto the axis perpendicular to it
template <typename T> struct PcDequant
{
    const float *in;
    int warp;
    const float *params;
    cx<T> o0, factor;
    __device__ PcDequant(const float *in_, int warp_, const float *params_) : in(in_), warp(warp_), params(params_)
    {
        using K = MeseConst<T>;
        const T c0 = T(in[0]);
        const T phase = K::pi * c0 - K::half_pi;
        T s, c;
        dsincos(phase, &s, &c);
        o0 = cscale(T(2) * K::inv_4pi, mk(c, s));
        const cx<T> axis = mk(-o0.y, o0.x);
        const T len = dsqrt(cabs2(axis));
        factor = cdivr(axis, len);
    }
    __device__ cx<T> operator()(int l) const
    {
        return l == 0 ? o0 : cscale(pc_inv_warp<T>(l, T(in[l]), warp, params), factor);
    }
};

} // namespace mraygb
