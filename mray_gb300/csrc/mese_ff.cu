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
// Layout: a pixel per group of 8 lanes, its arrays in shared memory (see prepare_ff_kernel).
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
    // where the compensation is far below the sum (or both are tiny): the pair normalised in three operations
    __device__ __forceinline__ ff fast_result() const { return fast_two_sum(s, c); }
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

// ---- one pixel per group of G lanes -----------------------------------------------------------------------
// The arrays of a pixel (E and the solution as float pairs; x in the solution's space while it is not yet used)
// live in shared memory; the G lanes of its group split every sum (lane r takes the indices = r mod G, each with
// its own compensated accumulator) and combine the partial sums with butterfly shuffles, and split the Levinson
// update by index pairs.  Per pixel 8 floats per moment of shared memory.

// G = 8 lanes per pixel (measured at 64 moments: 3.36 ms per 512^2 launch; 4 lanes, with one shuffle level less
// per sum but half the warps per SM for the same shared memory, 4.60 ms)
template <int MAXM> struct FfGroup
{
    static constexpr int G = 8;
    static constexpr int pixels = MAXM <= 128 ? 16 : 8;
};

// (s, c) compensated partial sums of the group combined: two-sum of the running sums, compensations added
template <int G> __device__ __forceinline__ void group_reduce(Dot &d)
{
#pragma unroll
    for (int o = 1; o < G; o <<= 1)
    {
        const float s2 = __shfl_xor_sync(0xffffffffu, d.s, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, d.c, o);
        const ff t = two_sum(d.s, s2);
        d.s = t.hi;
        d.c = __fadd_rn(__fadd_rn(d.c, c2), t.lo);
    }
}

// two compensated partial sums of the group combined with about half the shuffles of two group_reduce calls: at the
// first level the even lane of each pair keeps `a` and takes its partner's `a`, the odd lane does the same with `b`;
// the remaining levels reduce within each parity; a last exchange between the lanes of each pair gives every lane
// both sums.  The combination tree of each sum, and so its result, is group_reduce's.
template <int G> __device__ __forceinline__ void group_reduce2(Dot &a, Dot &b, int r)
{
    const bool even = (r & 1) == 0;
    float ks = even ? a.s : b.s, kc = even ? a.c : b.c;
    const float ss = even ? b.s : a.s, sc = even ? b.c : a.c;
#pragma unroll
    for (int o = 1; o < G; o <<= 1)
    {
        const float s2 = __shfl_xor_sync(0xffffffffu, o == 1 ? ss : ks, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, o == 1 ? sc : kc, o);
        const ff t = two_sum(ks, s2);
        ks = t.hi;
        kc = __fadd_rn(__fadd_rn(kc, c2), t.lo);
    }
    const float os = __shfl_xor_sync(0xffffffffu, ks, 1);
    const float oc = __shfl_xor_sync(0xffffffffu, kc, 1);
    a.s = even ? ks : os;
    a.c = even ? kc : oc;
    b.s = even ? os : ks;
    b.c = even ? oc : kc;
}

// per pixel: E (4 floats per moment), then one region of 4 floats per moment that holds x (2) during the
// exponential moments, the solution (4) during Levinson's recursion and in the tail the rounded polynomial (2) and
// the autocorrelation (2)
template <int MAXM> struct FfLayout
{
    static constexpr int floats_per_pixel = MAXM * 8;
};

// the pair update of Levinson's recursion on the solution divided by prod_j f_j (see the kernel): for the pairs
// (k, j - k), 1 <= k <= j / 2, shat_k - conj(shat_{j-k}) u and shat_{j-k} - conj(shat_k) u, split over the group
template <int G> __device__ __forceinline__ void scaled_levinson_update(cff *sol, int j, int r, const cff &u)
{
    for (int k = 1 + r; k <= j - k; k += G)
    {
        const int kk = j - k;
        const cff a = sol[k], b = sol[kk];
        Dot vr, vi;
        vr.init(a.re);
        vr.sub(b.re, u.re);
        vr.sub(b.im, u.im);
        vi.init(a.im);
        vi.sub(b.re, u.im);
        vi.add(b.im, u.re);
        const cff na = {vr.fast_result(), vi.fast_result()};
        if (k != kk)
        {
            Dot wr, wi;
            wr.init(b.re);
            wr.sub(a.re, u.re);
            wr.sub(a.im, u.im);
            wi.init(b.im);
            wi.sub(a.re, u.im);
            wi.add(a.im, u.re);
            sol[kk] = {wr.fast_result(), wi.fast_result()};
        }
        sol[k] = na;
    }
}

// PC: prediction-coded input (prepare_moments_from_pred_coding, src/moment_preparation.h:32-53): the codes are
// turned into reflection coefficients (transform_dequantization_real, src/moment_prediction_coding.h:97-118) and
// decoded (decode, :163-208) into the exponential moments and the evaluation polynomial; otherwise standard
// coding (prepare_moments_from_std_coding, :55-64).
template <int MAXM, bool PC>
__global__ void __launch_bounds__(128) prepare_ff_kernel(int num_pixels, int m, const uint32_t *__restrict__ index,
                                                         const float *__restrict__ data, float bias, int coding_warp,
                                                         const uint16_t *__restrict__ coding_params,
                                                         float *__restrict__ out)
{
    extern __shared__ __align__(16) float smem_ff[];
    __shared__ float s_params[PC ? 2 * MAXM : 1];
    if (PC && coding_warp == 0 && coding_params)
        for (int i = threadIdx.x; i < 2 * (m - 1); i += blockDim.x)
            s_params[i] = coding_params[i] / 65535.f; // CodingParamType::get_param1/2 (coding_params.h:52-54)
    __syncthreads();
    const int lane = threadIdx.x & 31;
    constexpr int kGroup = FfGroup<MAXM>::G;
    const int r = lane & (kGroup - 1);
    const int slot = threadIdx.x / kGroup;
    const int p = blockIdx.x * FfGroup<MAXM>::pixels + slot;
    float *base = smem_ff + (size_t)slot * FfLayout<MAXM>::floats_per_pixel;
    cff *E = reinterpret_cast<cff *>(base);
    cff *sol = E + MAXM;
    ff *x = reinterpret_cast<ff *>(sol); // standard coding: dead once the exponential moments are done

    size_t idx = 0;
    int n = 0;
    if (p < num_pixels)
    {
        pixel_span_ff(index, m, p, idx, n);
        n = n < MAXM ? n : MAXM;
    }
    // every group of the warp runs the same number of steps (the shuffles span the warp)
    const int nw = __reduce_max_sync(0xffffffffu, n);
    if (nw == 0)
        return;
    const float *in = data + idx;

    bool invalid = false;
    ff F = {1.f, 0.f};
    if (!PC)
    {
        // cut::lerp(m, target, bias) in pairs; x holds y_i = i x_i, the factors of the recurrence below
        const ff omb = two_sum(1.f, -bias);
        for (int i = r; i < nw; i += kGroup)
            x[i] = ff_mul_f(ff_mul_f(omb, i < n ? in[i] : 0.f), (float)i);
        if (r == 0)
        {
            const ff x0 = ff_add(ff_mul_f(omb, n > 0 ? in[0] : 0.f), {__fmul_rn(bias, 0.5f), 0.f});
            const double phi = 3.141592653589793 * ((double)x0.hi + (double)x0.lo) - 1.5707963267948966;
            double sp, cp;
            sincos(phi, &sp, &cp);
            E[0].re = ff_from_double(0.07957747154594767 * cp);
            E[0].im = ff_from_double(0.07957747154594767 * sp);
        }
        __syncwarp();

        // exponential moments: E_l = (2 pi i / l) sum_{j<l} y_{l-j} E_j
        for (int l = 1; l < nw; ++l)
        {
            Dot ar, ai;
            for (int j = r; j < l; j += kGroup)
            {
                const ff sc = x[l - j];
                const cff e = E[j];
                ar.add(sc, e.re);
                ai.add(sc, e.im);
            }
            group_reduce2<kGroup>(ar, ai, r);
            if (r == 0)
            {
                const float2 w2 = c_two_pi_over_l_ff[l];
                const ff w = {w2.x, w2.y};
                E[l].re = ff_neg(ff_mul(w, ai.result()));
                E[l].im = ff_mul(w, ar.result());
            }
            __syncwarp();
        }
        __syncwarp(); // every lane is done with x before the solution takes its space
        if (r == 0)
        {
            E[0].re = {2.f * E[0].re.hi, 2.f * E[0].re.lo};
            E[0].im = {2.f * E[0].im.hi, 2.f * E[0].im.lo};
            sol[0].re = ff_div({1.f, 0.f}, E[0].re);
            sol[0].im = {0.f, 0.f};
        }
        __syncwarp();

        // Levinson's recursion with the invalid latch, on the solution divided by F = prod_j f_j: with
        // sol = F shat the update new_k = f (o_k - conj(o_{j-k}) u) becomes shat_k - conj(shat_{j-k}) u, and
        // shat_0 stays 1 / E_0 (only F changes), u = F sum_k shat_k E_{j-k}
        for (int j = 1; j < nw; ++j)
        {
            Dot ur, ui;
            if (!invalid)
                for (int k = r; k < j; k += kGroup)
                {
                    const cff a = sol[k], b = E[j - k];
                    ur.add(a.re, b.re);
                    ur.sub(a.im, b.im);
                    ui.add(a.re, b.im);
                    ui.add(a.im, b.re);
                }
            group_reduce2<kGroup>(ur, ui, r);
            cff u = {ff_mul(F, ur.result()), ff_mul(F, ui.result())};
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
            scaled_levinson_update<kGroup>(sol, j, r, u);
            if (r == 0)
            {
                const ff s0 = sol[0].re;
                sol[j] = {ff_neg(ff_mul(s0, u.re)), ff_neg(ff_mul(s0, u.im))};
            }
            F = ff_div(F, ff_add({1.f, 0.f}, ff_neg(a2)));
            __syncwarp();
        }
    }
    else
    {
        // transform_dequantization_real: code_0 = 2 e^{i (pi c_0 - pi/2)} / (4 pi), code_l = w_l axis / |axis| with
        // axis = i code_0 and w_l the inverse warp of the input (formed per step, below)
        double cp, sp;
        sincos(3.141592653589793 * (double)(n > 0 ? in[0] : 0.f) - 1.5707963267948966, &sp, &cp);
        const ff fre = ff_from_double(-sp), fim = ff_from_double(cp); // axis / |axis| = i e^{i phi}
        if (r == 0)
        {
            E[0].re = ff_from_double(0.15915494309189535 * cp);
            E[0].im = ff_from_double(0.15915494309189535 * sp);
            sol[0].re = ff_div({1.f, 0.f}, E[0].re);
            sol[0].im = {0.f, 0.f};
        }
        __syncwarp();
        // decode: u_l = code_l (latched once |u|^2 >= 1 - 1e-6), E_l = (u_l - sum_{k=1}^{l-1} poly_k E_{l-k}) / poly_0,
        // then the Levinson update with u_l; poly = F shat as above
        const ff p0 = sol[0].re;
        for (int l = 1; l < nw; ++l)
        {
            Dot gr, gi;
            for (int k = 1 + r; k < l; k += kGroup)
            {
                const cff a = sol[k], b = E[l - k];
                gr.add(a.re, b.re);
                gr.sub(a.im, b.im);
                gi.add(a.re, b.im);
                gi.add(a.im, b.re);
            }
            group_reduce2<kGroup>(gr, gi, r);
            const float c = l < n ? in[l] : 0.f;
            ff w;
            if (coding_warp == 0)
            {
                // prediction_coding_inv_warp: c p1 2 - p0
                const ff cp1 = ff_mul_f({c, 0.f}, s_params[(l - 1) * 2 + 1]);
                w = ff_add({2.f * cp1.hi, 2.f * cp1.lo}, {-s_params[(l - 1) * 2], 0.f});
            }
            else
            {
                w = two_sum(2.f * c, -1.f);
            }
            cff u = {ff_mul(w, fre), ff_mul(w, fim)};
            Dot a2d;
            a2d.add(u.re, u.re);
            a2d.add(u.im, u.im);
            ff a2 = a2d.result();
            if (invalid || a2.hi >= 1.f - 1e-6f)
            {
                u = {{0.f, 0.f}, {0.f, 0.f}};
                a2 = {0.f, 0.f};
                invalid = true;
            }
            if (r == 0)
            {
                // (u - F gamma_hat) / (F p0)
                const ff fp0 = ff_mul(F, p0);
                const ff er = ff_add(u.re, ff_neg(ff_mul(F, gr.result())));
                const ff ei = ff_add(u.im, ff_neg(ff_mul(F, gi.result())));
                E[l] = {ff_div(er, fp0), ff_div(ei, fp0)};
            }
            scaled_levinson_update<kGroup>(sol, l, r, u);
            if (r == 0)
                sol[l] = {ff_neg(ff_mul(p0, u.re)), ff_neg(ff_mul(p0, u.im))};
            F = ff_div(F, ff_add({1.f, 0.f}, ff_neg(a2)));
            __syncwarp();
        }
    }
    // the tail in FP32 on the rounded values (lagrange_from_poly): P = 2 pi sol with sol = F shat, and the
    // exponential moments with E_0 halved; then the autocorrelation a_q and the correlation.  P is formed in
    // registers, then stored over the solution (the first half of its region), a_q in the second half.
    constexpr int kPer = (MAXM + kGroup - 1) / kGroup;
    float pre[kPer], pim[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k)
    {
        const int i = r + k * kGroup;
        if (i < nw)
        {
            pre[k] = 6.28318531f * ff_round(ff_mul(F, sol[i].re));
            pim[k] = 6.28318531f * ff_round(ff_mul(F, sol[i].im));
        }
    }
    __syncwarp();
    cx<float> *Pf = reinterpret_cast<cx<float> *>(sol);
#pragma unroll
    for (int k = 0; k < kPer; ++k)
    {
        const int i = r + k * kGroup;
        if (i < nw)
            Pf[i] = {pre[k], pim[k]};
    }
    __syncwarp();
    cx<float> *A = Pf + MAXM;
    for (int q = r; q < nw; q += kGroup)
    {
        float ar = 0.f, ai = 0.f;
        for (int j = 0; j < nw - q; ++j)
        {
            const cx<float> a = Pf[j], b = Pf[j + q];
            ar = fmaf(a.x, b.x, fmaf(a.y, b.y, ar));
            ai = fmaf(a.y, b.x, fmaf(-a.x, b.y, ai));
        }
        A[q] = {ar, ai};
    }
    __syncwarp();
    const float norm = 1.f / (3.14159265f * Pf[0].x);
    for (int k = r; k < nw; k += kGroup)
    {
        float acc = 0.f;
        for (int q = k; q < nw; ++q)
        {
            const cff e = E[q - k];
            float ex = ff_round(e.re), ey = ff_round(e.im);
            if (q == k)
            {
                ex *= 0.5f;
                ey *= 0.5f;
            }
            acc = fmaf(A[q].x, ey, fmaf(A[q].y, ex, acc));
        }
        if (k < n)
            out[idx + k] = norm * acc;
    }
}

template <int MAXM, bool PC>
cudaError_t launch_ff_pc(int num_pixels, int m, const uint32_t *index, const float *data, float bias, int warp,
                         const uint16_t *cp, float *out, cudaStream_t stream)
{
    constexpr int ppb = FfGroup<MAXM>::pixels;
    const int bytes = ppb * FfLayout<MAXM>::floats_per_pixel * (int)sizeof(float);
    cudaError_t e =
        cudaFuncSetAttribute(prepare_ff_kernel<MAXM, PC>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess)
        return e;
    prepare_ff_kernel<MAXM, PC><<<(num_pixels + ppb - 1) / ppb, ppb * FfGroup<MAXM>::G, bytes, stream>>>(
        num_pixels, m, index, data, bias, warp, cp, out);
    return cudaGetLastError();
}

template <int MAXM>
cudaError_t launch_ff_m(int num_pixels, int m, const uint32_t *index, const float *data, int pc, int warp,
                        const uint16_t *cp, float bias, float *out, cudaStream_t stream)
{
    if (pc)
        return launch_ff_pc<MAXM, true>(num_pixels, m, index, data, bias, warp, cp, out, stream);
    return launch_ff_pc<MAXM, false>(num_pixels, m, index, data, bias, warp, cp, out, stream);
}

} // namespace

cudaError_t mese_ff_init_constants(const LibmTrigTable &trig)
{
    cudaError_t e = set_libm_trig_constants(trig);
    if (e != cudaSuccess)
        return e;
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

cudaError_t launch_prepare_ff(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                              int coding_warp, const uint16_t *coding_params, float bias, float *pmoments,
                              cudaStream_t stream)
{
    const int pc = prediction_code ? 1 : 0;
    if (m <= 16)
        return launch_ff_m<16>(num_pixels, m, index, data, pc, coding_warp, coding_params, bias, pmoments, stream);
    if (m <= 32)
        return launch_ff_m<32>(num_pixels, m, index, data, pc, coding_warp, coding_params, bias, pmoments, stream);
    if (m <= 64)
        return launch_ff_m<64>(num_pixels, m, index, data, pc, coding_warp, coding_params, bias, pmoments, stream);
    if (m <= 128)
        return launch_ff_m<128>(num_pixels, m, index, data, pc, coding_warp, coding_params, bias, pmoments, stream);
    return launch_ff_m<256>(num_pixels, m, index, data, pc, coding_warp, coding_params, bias, pmoments, stream);
}

} // namespace mraygb
