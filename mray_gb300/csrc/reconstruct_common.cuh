// Device functions shared by the MESE re-march (reconstruct.cu) and its adjoint (adjoint.cu): fast_atan, the
// transfer-function samples and the MESE density by Reinsch's modified Clenshaw recurrence.
#pragma once

#include "device_common.cuh"

namespace mraygb
{

// fast_atan (src/mese/complex_algebra.h:133-152)
__device__ __forceinline__ float fast_atan(float tan)
{
    const bool negative = tan < 0.0f;
    const float abs_tan = negative ? -tan : tan;
    const bool greater_one = abs_tan > 1.0f;
    float x = greater_one ? abs_tan : 1.0f;
    x = 1.0f / x;
    float y = greater_one ? 1.0f : abs_tan;
    x = x * y;
    y = x * x;
    float z = y * 0.020835f - 0.085133f;
    z = y * z + 0.180141f;
    z = y * z - 0.330299f;
    y = y * z + 0.999866f;
    z = y * x;
    z = z * -2.0f + 1.570796f;
    z = greater_one ? z : 0.0f;
    x = x * y + z;
    return negative ? -x : x;
}

__device__ __forceinline__ float4 tf_sample(const float4 *T, float fs, float bs)
{
    const float ipx = fs * 256.f, ipy = bs * 256.f;
    const float flx = floorf(ipx);
    const float ax = ipx - flx, ay = ipy - floorf(ipy);
    const int xl = (int)flx;
    const int x0 = min(max(xl, 0), 255);
    const int x1 = min(max(xl + 1, 0), 255);
    const float4 a = T[x0], b = T[x1];
    const float wll = (1.f - ax) * (1.f - ay), wlr = ax * (1.f - ay), wrl = (1.f - ax) * ay, wrr = ax * ay;
    float4 r;
    r.x = wll * a.x + wlr * a.x + wrl * b.x + wrr * b.x;
    r.y = wll * a.y + wlr * a.y + wrl * b.y + wrr * b.y;
    r.z = wll * a.z + wlr * a.z + wrl * b.z + wrr * b.z;
    r.w = wll * a.w + wlr * a.w + wrl * b.w + wrr * b.w;
    return r;
}

// The differentiation form's transfer function: the row as a uniform cubic B-spline in the front density (C2, so an
// image-space loss stays smooth where a density crosses a table entry; the rows being equal, the back density
// drops out).  Knots at the texel centres of the reference's GPU texture (TransferFunctionDevice::sample,
// src/transfer_function_device.cuh:30-65: u = 256 fs - 1/2), entries clamped at the ends.  Base entry i - 1 and
// the four weights in *base / w when asked for.
struct BSplineTap
{
    int i; // entries i - 1 .. i + 2 (clamped)
    float t;
    float w[4];
};

__device__ __forceinline__ BSplineTap bspline_tap(float fs)
{
    BSplineTap k;
    const float u = fs * 256.f - 0.5f;
    const float fl = floorf(u);
    k.t = u - fl;
    k.i = (int)fl;
    const float t = k.t, s = 1.f - t, t2 = t * t, t3 = t2 * t;
    k.w[0] = s * s * s * (1.f / 6.f);
    k.w[1] = (3.f * t3 - 6.f * t2 + 4.f) * (1.f / 6.f);
    k.w[2] = (-3.f * t3 + 3.f * t2 + 3.f * t + 1.f) * (1.f / 6.f);
    k.w[3] = t3 * (1.f / 6.f);
    return k;
}

__device__ __forceinline__ int bspline_entry(const BSplineTap &k, int j) { return min(max(k.i - 1 + j, 0), 255); }

// The same row sampled linearly in the front density with the texel convention of the reference's GPU texture
// (TransferFunctionDevice::sample, src/transfer_function_device.cuh:30-65: u = 256 fs - 1/2, clamp to edge) as a tap
// of the same four-entry window: entries i and i + 1 with weights 1 - t and t (the outer two weigh 0).  Exact float
// weights, not the texture unit's 8-bit fractions.
__device__ __forceinline__ BSplineTap linear_tap(float fs)
{
    BSplineTap k;
    const float u = fs * 256.f - 0.5f;
    const float fl = floorf(u);
    k.t = u - fl;
    k.i = (int)fl;
    k.w[0] = 0.f;
    k.w[1] = 1.f - k.t;
    k.w[2] = k.t;
    k.w[3] = 0.f;
    return k;
}

// the differentiation form's tap of either transfer-function row
__device__ __forceinline__ BSplineTap diff_tf_tap(float fs, bool linear) { return linear ? linear_tap(fs) : bspline_tap(fs); }

__device__ __forceinline__ float4 tf_sample_bspline(const float4 *T, const BSplineTap &k)
{
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        const float4 e = T[bspline_entry(k, j)];
        r.x = fmaf(k.w[j], e.x, r.x);
        r.y = fmaf(k.w[j], e.y, r.y);
        r.z = fmaf(k.w[j], e.z, r.z);
        r.w = fmaf(k.w[j], e.w, r.w);
    }
    return r;
}

// the sample and its derivative in fs from one read of the four entries
__device__ __forceinline__ void tf_bspline_value_derivative(const float4 *T, const BSplineTap &k, float4 &val,
                                                            float4 &dval)
{
    const float t = k.t, s = 1.f - t;
    const float d[4] = {-128.f * s * s, 128.f * (3.f * t * t - 4.f * t), 128.f * (-3.f * t * t + 2.f * t + 1.f),
                        128.f * t * t};
    val = make_float4(0.f, 0.f, 0.f, 0.f);
    dval = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        const float4 e = T[bspline_entry(k, j)];
        val.x = fmaf(k.w[j], e.x, val.x);
        val.y = fmaf(k.w[j], e.y, val.y);
        val.z = fmaf(k.w[j], e.z, val.z);
        val.w = fmaf(k.w[j], e.w, val.w);
        dval.x = fmaf(d[j], e.x, dval.x);
        dval.y = fmaf(d[j], e.y, dval.y);
        dval.z = fmaf(d[j], e.z, dval.z);
        dval.w = fmaf(d[j], e.w, dval.w);
    }
}

// the same from one float table per channel (channel c of entry i at c * 256 + i): the same operations; with
// `linear` the tap is linear_tap's and the derivative d / d fs = 256 (T[i + 1] - T[i])
__device__ __forceinline__ void tf_bspline_value_derivative_soa(const float *T, const BSplineTap &k, float4 &val,
                                                                float4 &dval, bool linear = false)
{
    const float t = k.t, s = 1.f - t;
    float d[4] = {-128.f * s * s, 128.f * (3.f * t * t - 4.f * t), 128.f * (-3.f * t * t + 2.f * t + 1.f),
                  128.f * t * t};
    if (linear)
    {
        d[0] = 0.f;
        d[1] = -256.f;
        d[2] = 256.f;
        d[3] = 0.f;
    }
    val = make_float4(0.f, 0.f, 0.f, 0.f);
    dval = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        const int i = bspline_entry(k, j);
        const float4 e = make_float4(T[i], T[256 + i], T[512 + i], T[768 + i]);
        val.x = fmaf(k.w[j], e.x, val.x);
        val.y = fmaf(k.w[j], e.y, val.y);
        val.z = fmaf(k.w[j], e.z, val.z);
        val.w = fmaf(k.w[j], e.w, val.w);
        dval.x = fmaf(d[j], e.x, dval.x);
        dval.y = fmaf(d[j], e.y, dval.y);
        dval.z = fmaf(d[j], e.z, dval.z);
        dval.w = fmaf(d[j], e.w, dval.w);
    }
}

// d tf_sample_bspline / d fs (256 d / d u)
__device__ __forceinline__ float4 tf_bspline_derivative(const float4 *T, const BSplineTap &k)
{
    const float t = k.t, s = 1.f - t;
    const float d[4] = {-0.5f * s * s, 0.5f * (3.f * t * t - 4.f * t), 0.5f * (-3.f * t * t + 2.f * t + 1.f),
                        0.5f * t * t};
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 4; ++j)
    {
        const float4 e = T[bspline_entry(k, j)];
        r.x = fmaf(d[j], e.x, r.x);
        r.y = fmaf(d[j], e.y, r.y);
        r.z = fmaf(d[j], e.z, r.z);
        r.w = fmaf(d[j], e.w, r.w);
    }
    return make_float4(256.f * r.x, 256.f * r.y, 256.f * r.z, 256.f * r.w);
}

// S(theta) = sum_{k=0}^{n-1} a_k cos(k theta), a_0 = l_0, a_k = 2 l_k, by Reinsch's recurrence:
//   cos(theta) > 0 : lam = -4 sin^2(theta/2),  u <- u + d,  d <- a_k + lam u + d
//   cos(theta) <= 0: lam =  4 cos^2(theta/2),  u <- d - u,  d <- a_k + lam u - d
//   S = d - (lam / 2) u
// (reinsch_lambda gives lam and the branch; a caller that runs a second recurrence at the same theta takes them
// once)
__device__ __forceinline__ float reinsch_lambda(float pc, bool &pos)
{
    float sh, ch;
    sincosf(0.5f * pc, &sh, &ch);
    pos = fabsf(pc) < 1.5707963267948966f; // cos(pc) > 0
    return pos ? -4.f * sh * sh : 4.f * ch * ch;
}

template <int MAXM>
__device__ __forceinline__ float mese_series_reinsch(const float (&lam2)[MAXM], float lam0, bool pos, float lam)
{
    const float sg = pos ? 1.f : -1.f;
    float u = 0.f, d = 0.f;
#pragma unroll
    for (int l = MAXM - 1; l >= 1; --l)
    {
        u = fmaf(sg, u, d);
        d = fmaf(lam, u, fmaf(sg, d, lam2[l]));
    }
    u = fmaf(sg, u, d);
    d = fmaf(lam, u, fmaf(sg, d, lam0));
    return fmaf(-0.5f * lam, u, d);
}

template <int MAXM> __device__ __forceinline__ float mese_series(const float (&lam2)[MAXM], float lam0, float pc)
{
    bool pos;
    const float lam = reinsch_lambda(pc, pos);
    return mese_series_reinsch<MAXM>(lam2, lam0, pos, lam);
}

// the bounded density at phase p: lo + span (atan(S) / pi + 1/2) (MESEReconstruction::reconstruct,
// src/reconstruction_techniques.h:72-96), p clamped to [-pi, 0]
template <int MAXM>
__device__ __forceinline__ float mese_density(const float (&lam2)[MAXM], float lam0, float p, float lo, float span)
{
    const float pc = rclamp(p, -kPiF, 0.0f);
    const float s = mese_series<MAXM>(lam2, lam0, pc);
    return (fast_atan(s) * 0.318309886f + 0.5f) * span + lo;
}

// the differentiation form's density: exact atan (fast_atan jumps by 2.4e-5 at |t| = 1)
template <int MAXM>
__device__ __forceinline__ float mese_density_exact(const float (&lam2)[MAXM], float lam0, float p, float lo,
                                                    float span)
{
    const float pc = rclamp(p, -kPiF, 0.0f);
    const float s = mese_series<MAXM>(lam2, lam0, pc);
    return (atanf(s) * 0.318309886f + 0.5f) * span + lo;
}

// henyey_greenstein (src/cut/phase_functions.h:33-36) at cos_theta = dot(-ray.dir, light_dir); the reference's CPU
// build divides by pow of the float arguments promoted to double, so the division is in double
__device__ __forceinline__ float henyey_greenstein_ray(const float d[3], const float light[3], float g)
{
    const float cos_theta =
        __fadd_rn(__fadd_rn(__fmul_rn(-d[0], light[0]), __fmul_rn(-d[1], light[1])), __fmul_rn(-d[2], light[2]));
    const float num = __fmul_rn(__fsub_rn(1.f, __fmul_rn(g, g)), 0.07957747154594766788f);
    const float base = __fsub_rn(__fadd_rn(1.f, __fmul_rn(g, g)), __fmul_rn(__fmul_rn(2.f, g), cos_theta));
    return (float)((double)num / pow((double)base, 1.5));
}

// d fast_atan / dt: fast_atan is t P(t^2) for |t| <= 1 and pi/2 - P(1/t^2) / |t| (odd) beyond, with P the
// polynomial above; the derivative is Q(y) = P(y) + 2 y P'(y) at y = t^2, or Q(1/t^2) / t^2.
__device__ __forceinline__ float fast_atan_derivative(float t)
{
    const float a = fabsf(t);
    const bool greater_one = a > 1.0f;
    const float r = greater_one ? 1.0f / a : a;
    const float y = r * r;
    // P(y) = (((0.020835 y - 0.085133) y + 0.180141) y - 0.330299) y + 0.999866
    // Q(y) = P + 2 y P' = ((9 * 0.020835 y - 7 * 0.085133) y + 5 * 0.180141) y - 3 * 0.330299) y + 0.999866
    float q = fmaf(9.0f * 0.020835f, y, -7.0f * 0.085133f);
    q = fmaf(q, y, 5.0f * 0.180141f);
    q = fmaf(q, y, -3.0f * 0.330299f);
    q = fmaf(q, y, 0.999866f);
    return greater_one ? q * y : q;
}

} // namespace mraygb
