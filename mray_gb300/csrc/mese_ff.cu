// The float-float form of the Lagrange-multiplier preparation (MRAYGB_PRECISION_COMPENSATED_FF_MESE): the same
// method as the FP64 form with FP64 arithmetic replaced by pairs of floats, for a GPU whose FP32 rate is 64 times
// its FP64 rate.
//
// Which steps need the extra precision was measured against the FP64 oracle on 64-moment mixing-layer pixels:
// the exponential moments (trigonometricToExponentialMoments, src/mese/MESE_dynamic.h:35-54) and Levinson's
// recursion (:100-135) lose about 1e-4 of the multipliers in FP32, and rounding their results to float between the
// steps loses as much again; the autocorrelation / imaginary correlation tail (:137-211) run in FP32 on the rounded
// Levinson solution and exponential moments adds about 1e-7.  So the values of the first two steps are float pairs
// (hi + lo, about 48 significant bits) and the tail is FP32.
//
// Arithmetic: error-free transformations (two-sum, two-product by FMA) written with explicit round-to-nearest
// intrinsics, so no contraction can change them.  Sums of products use the compensated dot-product scheme of
// Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005): the running sum in
// one float, every rounding error (of the products and of the additions) in a second float, which gives the
// result as if accumulated in twice the working precision.

#include "internal.h"
#include "mese_device.cuh"

namespace mraygb
{

namespace
{

struct ff
{
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_div(ff a, ff b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const ff r = ff_add(a, ff_neg(ff_mul_f(b, q1)));
    return fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}

__device__ __forceinline__ ff ff_from_double(double v)
{
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

__device__ __forceinline__ float ff_round(ff a) { return __fadd_rn(a.hi, a.lo); }

// compensated accumulation of products of pairs
struct Dot
{
    float s = 0.f, c = 0.f;

    __device__ __forceinline__ void init(ff a)
    {
        s = a.hi;
        c = a.lo;
    }
    __device__ __forceinline__ void add(ff a, ff b)
    {
        const float p = __fmul_rn(a.hi, b.hi);
        float e = fmaf(a.hi, b.hi, -p);
        e = fmaf(a.hi, b.lo, e);
        e = fmaf(a.lo, b.hi, e);
        const ff t = two_sum(s, p);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    __device__ __forceinline__ void sub(ff a, ff b) { add(ff_neg(a), b); }
    __device__ __forceinline__ ff result() const { return two_sum(s, c); }
};

struct cff
{
    ff re, im;
};

__constant__ float2 c_two_pi_over_l_ff[256]; // 2 pi / l as a float pair

__device__ __forceinline__ void pixel_span_ff(const uint32_t *index, int m, int p, size_t &idx, int &n)
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

// Lagrange multipliers of one pixel (prepare_moments_from_std_coding, src/moment_preparation.h:55-64)
template <int MAXM>
__global__ void __launch_bounds__(128) prepare_ff_kernel(int num_pixels, int m, const uint32_t *__restrict__ index,
                                                         const float *__restrict__ data, float bias,
                                                         float *__restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= num_pixels)
        return;
    size_t idx;
    int n;
    pixel_span_ff(index, m, p, idx, n);
    if (n <= 0)
        return;
    if (n > MAXM)
        n = MAXM;
    const float *in = data + idx;

    // cut::lerp(m, target, bias) in pairs: (1 - b) m_i (+ b / 2 for i = 0)
    ff x[MAXM];
    const ff omb = two_sum(1.f, -bias);
    for (int i = 0; i < n; ++i)
        x[i] = ff_mul_f(omb, in[i]);
    x[0] = ff_add(x[0], {__fmul_rn(bias, 0.5f), 0.f});

    // exponential moments: E_0 = e^{i (pi x_0 - pi / 2)} / (4 pi) (in FP64: one sincos per pixel),
    // E_l = (2 pi i / l) sum_{j<l} (l - j) x_{l-j} E_j, E_0 doubled at the end
    cff E[MAXM];
    {
        const double phi = 3.141592653589793 * ((double)x[0].hi + (double)x[0].lo) - 1.5707963267948966;
        double sp, cp;
        sincos(phi, &sp, &cp);
        E[0].re = ff_from_double(0.07957747154594767 * cp);
        E[0].im = ff_from_double(0.07957747154594767 * sp);
    }
    for (int l = 1; l < n; ++l)
    {
        Dot ar, ai;
        for (int j = 0; j < l; ++j)
        {
            const ff s = ff_mul_f(x[l - j], (float)(l - j));
            ar.add(s, E[j].re);
            ai.add(s, E[j].im);
        }
        const float2 w2 = c_two_pi_over_l_ff[l];
        const ff w = {w2.x, w2.y};
        // (i w)(re + i im) = (-w im, w re)
        E[l].re = ff_neg(ff_mul(w, ai.result()));
        E[l].im = ff_mul(w, ar.result());
    }
    E[0].re = {2.f * E[0].re.hi, 2.f * E[0].re.lo};
    E[0].im = {2.f * E[0].im.hi, 2.f * E[0].im.lo};

    // Levinson's recursion with the invalid latch
    cff sol[MAXM];
    sol[0].re = ff_div({1.f, 0.f}, E[0].re);
    sol[0].im = {0.f, 0.f};
    bool invalid = false;
    for (int j = 1; j < n; ++j)
    {
        cff u = {{0.f, 0.f}, {0.f, 0.f}};
        if (!invalid)
        {
            Dot ur, ui;
            for (int k = 0; k < j; ++k)
            {
                const cff a = sol[k], b = E[j - k];
                ur.add(a.re, b.re);
                ur.sub(a.im, b.im);
                ui.add(a.re, b.im);
                ui.add(a.im, b.re);
            }
            u.re = ur.result();
            u.im = ui.result();
        }
        Dot a2d;
        a2d.add(u.re, u.re);
        a2d.add(u.im, u.im);
        ff a2 = a2d.result();
        if (invalid || a2.hi >= 1.f)
        {
            u = {{0.f, 0.f}, {0.f, 0.f}};
            a2 = {0.f, 0.f};
            invalid = true;
        }
        const ff f = ff_div({1.f, 0.f}, ff_add({1.f, 0.f}, ff_neg(a2)));
        // new_k = f (o_k - conj(o_{j-k}) u), pairs (k, j - k) in place
        const ff s0 = sol[0].re;
        int k = 1, kk = j - 1;
        for (; k <= kk; ++k, --kk)
        {
            const cff a = sol[k], b = sol[kk];
            // conj(b) u = (b.re u.re + b.im u.im, b.re u.im - b.im u.re)
            Dot vr, vi;
            vr.init(a.re);
            vr.sub(b.re, u.re);
            vr.sub(b.im, u.im);
            vi.init(a.im);
            vi.sub(b.re, u.im);
            vi.add(b.im, u.re);
            sol[k].re = ff_mul(f, vr.result());
            sol[k].im = ff_mul(f, vi.result());
            if (k != kk)
            {
                Dot wr, wi;
                wr.init(b.re);
                wr.sub(a.re, u.re);
                wr.sub(a.im, u.im);
                wi.init(b.im);
                wi.sub(a.re, u.im);
                wi.add(a.im, u.re);
                sol[kk].re = ff_mul(f, wr.result());
                sol[kk].im = ff_mul(f, wi.result());
            }
        }
        sol[j].re = ff_neg(ff_mul(ff_mul(f, s0), u.re));
        sol[j].im = ff_neg(ff_mul(ff_mul(f, s0), u.im));
        sol[0].re = ff_mul(f, s0);
    }

    // the tail in FP32 on the rounded values: P = 2 pi sol, E_0 halved, autocorrelation scattered into the
    // imaginary correlation (lagrange_from_poly)
    cx<float> P[MAXM], Ef[MAXM];
    float acc[MAXM];
    for (int i = 0; i < n; ++i)
    {
        P[i] = {6.28318531f * ff_round(sol[i].re), 6.28318531f * ff_round(sol[i].im)};
        Ef[i] = {ff_round(E[i].re), ff_round(E[i].im)};
        acc[i] = 0.f;
    }
    Ef[0] = {0.5f * Ef[0].x, 0.5f * Ef[0].y};
    for (int q = 0; q < n; ++q)
    {
        float ar = 0.f, ai = 0.f;
        for (int j = 0; j < n - q; ++j)
        {
            // P_j conj(P_{j+q})
            ar = fmaf(P[j].x, P[j + q].x, fmaf(P[j].y, P[j + q].y, ar));
            ai = fmaf(P[j].y, P[j + q].x, fmaf(-P[j].x, P[j + q].y, ai));
        }
        for (int k = 0; k <= q; ++k)
        {
            const cx<float> e = Ef[q - k];
            acc[k] = fmaf(ar, e.y, fmaf(ai, e.x, acc[k]));
        }
    }
    const float norm = 1.f / (3.14159265f * P[0].x);
    float *o = out + idx;
    for (int i = 0; i < n; ++i)
        o[i] = norm * acc[i];
}

template <int MAXM>
cudaError_t launch_ff_m(int num_pixels, int m, const uint32_t *index, const float *data, float bias, float *out,
                        cudaStream_t stream)
{
    prepare_ff_kernel<MAXM><<<(num_pixels + 127) / 128, 128, 0, stream>>>(num_pixels, m, index, data, bias, out);
    return cudaGetLastError();
}

} // namespace

cudaError_t mese_ff_init_constants()
{
    float2 t[256];
    t[0] = make_float2(0.f, 0.f);
    for (int l = 1; l < 256; ++l)
    {
        const double w = 6.283185307179586476925 / (double)l;
        const float hi = (float)w;
        t[l] = make_float2(hi, (float)(w - (double)hi));
    }
    return cudaMemcpyToSymbol(c_two_pi_over_l_ff, t, sizeof(t));
}

cudaError_t launch_prepare_ff(int num_pixels, int m, const uint32_t *index, const float *data, float bias,
                              float *pmoments, cudaStream_t stream)
{
    if (m <= 16)
        return launch_ff_m<16>(num_pixels, m, index, data, bias, pmoments, stream);
    if (m <= 32)
        return launch_ff_m<32>(num_pixels, m, index, data, bias, pmoments, stream);
    if (m <= 64)
        return launch_ff_m<64>(num_pixels, m, index, data, bias, pmoments, stream);
    if (m <= 128)
        return launch_ff_m<128>(num_pixels, m, index, data, bias, pmoments, stream);
    return launch_ff_m<256>(num_pixels, m, index, data, bias, pmoments, stream);
}

} // namespace mraygb
