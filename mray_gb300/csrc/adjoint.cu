// The differentiation form: hand-written adjoints of the MESE re-march, of the Lagrange-multiplier preparation
// and of moment generation, which back-propagate an image-space loss to the transfer-function row and to the
// voxel densities.
//
// The differentiated method is the moment-image path with four changes that make the loss smooth almost everywhere
// in its inputs: the image is not compacted (every pixel keeps m moments), reconstruction reads the unquantized
// per-pixel density bounds (lo, hi) that generation computed, the MESE density uses the exact arctangent (the
// reference's fast_atan jumps by 2.4e-5 at |t| = 1), and the transfer-function row is a uniform cubic B-spline in
// the front density with knots at the texel centres of the reference's GPU texture (transfer_function_device.cuh).
// A piecewise-linear row has a kink at every entry, dense enough that a 1e-3 change of one voxel crosses several
// along a ray; it is still offered (tf_linear: the GPU texture's own interpolation, exact weights), as the same
// four-entry tap with the outer two weights zero.
//
// Memory: none of the three adjoints keeps a per-sample tape.  The re-march adjoint replays the forward march
// and uses the final radiance of the forward pass for the suffix sums of front-to-back compositing (d L / d tau_k
// needs the radiance gathered behind sample k, which is the final radiance minus the radiance so far); the
// generation adjoint replays the sample positions; the preparation adjoint reads two arrays per pixel that the
// forward preparation kept (the Levinson solution and the exponential moments, 2m complex values) and needs no
// recursion run backwards (see prepare_adjoint_kernel).

#include "device_common.cuh"
#include "internal.h"
#include "reconstruct_common.cuh"

namespace mraygb
{

namespace
{

constexpr unsigned kFull = 0xffffffffu;

// ------------------------------------------------------------------------------------------------------------
// re-march adjoint
// ------------------------------------------------------------------------------------------------------------

struct ReconAdjDev
{
    DeviceCamera cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const float *pmoments;  // W*H*m Lagrange multipliers
    const float4 *bounds4;  // (lo, hi, ., .)
    const float4 *tf;       // 256 entries
    float step, emission, ert;
    const float4 *rgba;     // forward result
    const float4 *grad_rgba;
    float *grad_lambda;     // W*H*m
    float2 *grad_bounds;    // W*H (d/d lo, d/d hi)
    float4 *grad_tf;        // 256, accumulated
    int tf_linear;          // the row linear in the front density instead of the cubic B-spline
    int *error_flag;
};

// The transfer-function gradient of a block is accumulated in kTfCopies copies of the 256-entry row in shared
// memory, lane l adding to copy l mod kTfCopies: neighbouring rays sample similar densities at the same step, and
// shared-memory atomics on one address from many lanes of a warp serialize.  Row and gradient are held as one float
// table per channel (scalar loads and atomics: lanes whose entries differ by less than 32 never share a bank; the
// float4 entries of a gather conflicted whenever two entries of a quarter-warp were 8 apart), the tables of the
// copies kTfCopyStride = 257 floats apart (copy c's channel ch at (4 c + ch) * 257), so the lanes that add to the same
// entry in their own copies fall into different banks.
constexpr int kTfCopies = 8;
constexpr int kTfCopyStride = 257;

// accumulates the B-spline weights times g into the shared transfer-function gradient through a cache of the
// last four entries: consecutive samples of a ray mostly fall between the same knots
struct TfGradCache
{
    int base = -1000;
    float4 acc[4];

    // s_g: this lane's copy, channel c at c * kTfCopyStride
    __device__ __forceinline__ void flush(float *s_g)
    {
        if (base <= -1000)
            return;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int x = min(max(base - 1 + j, 0), 255);
            atomicAdd(&s_g[x], acc[j].x);
            atomicAdd(&s_g[kTfCopyStride + x], acc[j].y);
            atomicAdd(&s_g[2 * kTfCopyStride + x], acc[j].z);
            atomicAdd(&s_g[3 * kTfCopyStride + x], acc[j].w);
        }
    }
    __device__ __forceinline__ void add(float *s_g, const BSplineTap &k, float4 g)
    {
        if (k.i != base)
        {
            flush(s_g);
            base = k.i;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            acc[j].x = fmaf(k.w[j], g.x, acc[j].x);
            acc[j].y = fmaf(k.w[j], g.y, acc[j].y);
            acc[j].z = fmaf(k.w[j], g.z, acc[j].z);
            acc[j].w = fmaf(k.w[j], g.w, acc[j].w);
        }
    }
};


template <int MAXM> __global__ void __launch_bounds__(128, 4) reconstruct_adjoint_kernel(const ReconAdjDev a)
{
    __shared__ float s_tf[4 * 256]; // channel c of entry i at c * 256 + i
    extern __shared__ float s_gall[]; // kTfCopies * 4 * kTfCopyStride (dynamic: above the 48 KiB of static memory)
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    for (int i = tid; i < 256; i += blockDim.x * blockDim.y)
    {
        const float4 v = a.tf[i];
        s_tf[i] = v.x;
        s_tf[256 + i] = v.y;
        s_tf[512 + i] = v.z;
        s_tf[768 + i] = v.w;
    }
    for (int i = tid; i < kTfCopies * 4 * kTfCopyStride; i += blockDim.x * blockDim.y)
        s_gall[i] = 0.f;
    __syncthreads();
    float *s_g = s_gall + (tid % kTfCopies) * 4 * kTfCopyStride;

    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    TfGradCache cache;
    if (x < a.width && y < a.height)
    {
        const size_t pix = (size_t)y * (size_t)a.width + (size_t)x;
        const size_t idx = pix * (size_t)a.m;
        const int n = a.m < MAXM ? a.m : MAXM;
        float lam2[MAXM], glam[MAXM];
        const float lam0 = a.pmoments[idx];
#pragma unroll
        for (int l = 0; l < MAXM; ++l)
        {
            lam2[l] = (l < n && l > 0) ? 2.f * a.pmoments[idx + l] : 0.f;
            glam[l] = 0.f;
        }
        const float4 b4 = a.bounds4[pix];
        const float lo = b4.x, span = b4.y - b4.x;
        const float4 out = a.rgba[pix];
        const float4 g = a.grad_rgba[pix];
        float glo = 0.f, ghi = 0.f;

        float nx, ny, o[3], d[3];
        pixel_ndc(x, y, a.width, a.height, nx, ny);
        eye_ray(a.cam, nx, ny, o, d);
        float t_near, t_far;
        const bool hit = intersect_aabb(o, d, a.dmin, a.dmax, t_near, t_far);
        t_near = rmax(t_near, a.cam.znear);
        if (hit && t_far > 0.f)
        {
            const float range = __fsub_rn(t_far, t_near);
            float t = t_near;
            float p = (float)((double)__fdiv_rn(__fsub_rn(t, t_near), range) * 3.141592653589793 -
                              3.141592653589793);
            const float phase_step = (float)(3.141592653589793 * (double)__fdiv_rn(a.step, range));
            const float est = range / a.step;
            const int cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
            // alpha == 1 marks a terminated march (then alpha no longer depends on the samples)
            const float galpha_T = out.w == 1.f ? 0.f : g.w * (1.f - out.w);
            float L0 = 0.f, L1 = 0.f, L2 = 0.f, T = 1.f, tau = 0.f;
            // each step takes its front sample at phase p: the series value S by the forward's own recurrence
            // (mese_series), and d S / d lambda_l = 2 cos(l p) from the modified three-term recurrence below
            float pc = rclamp(p, -kPiF, 0.0f);
            int it = 0;
            while (t <= t_far)
            {
                if (++it > cap)
                {
                    atomicExch(a.error_flag, 1);
                    break;
                }
                bool pos;
                const float dl = reinsch_lambda(pc, pos);
                const float S = mese_series_reinsch<MAXM>(lam2, lam0, pos, dl);
                const float r = atanf(S) * 0.318309886f + 0.5f;
                const float fs = r * span + lo;
                const BSplineTap k = diff_tf_tap(fs, a.tf_linear);
                float4 s, dt;
                tf_bspline_value_derivative_soa(s_tf, k, s, dt, a.tf_linear);
                // d loss / d sample: emission terms see T before this step, extinction the radiance behind it
                float4 gs;
                gs.x = g.x * a.emission * T;
                gs.y = g.y * a.emission * T;
                gs.z = g.z * a.emission * T;
                L0 += (a.emission * s.x) * T;
                L1 += (a.emission * s.y) * T;
                L2 += (a.emission * s.z) * T;
                gs.w = galpha_T - (g.x * (out.x - L0) + g.y * (out.y - L1) + g.z * (out.z - L2));
                tau += s.w;
                T = expf(-tau);
                const float alpha = 1.f - T;
                // transfer-function entries
                cache.add(s_g, k, gs);
                // front density -> series value -> multipliers and bounds
                const float gfs = dt.x * gs.x + dt.y * gs.y + dt.z * gs.z + dt.w * gs.w;
                glo = fmaf(gfs, 1.f - r, glo);
                ghi = fmaf(gfs, r, ghi);
                const float gS = __fdividef(gfs * span * 0.318309886f, fmaf(S, S, 1.f));
                glam[0] += gS;
                // cos(l pc) for l >= 1 by Reinsch's modification of the three-term recurrence (stable where pc
                // nears 0 or -pi, the two ends of every ray), with the series' own d: with d = -4 sin^2(pc / 2)
                // while cos pc > 0,
                //   e_{l+1} = e_l + d c_l,  c_{l+1} = c_l + e_{l+1}      (e_l = c_l - c_{l-1}),
                // and with d = 4 cos^2(pc / 2) otherwise,
                //   e_{l+1} = d c_l - e_l,  c_{l+1} = e_{l+1} - c_l      (e_l = c_l + c_{l-1});
                // one loop per branch, so each step is one FMA and one add besides the accumulation
                {
                    float e = 0.5f * dl;
                    const float g2 = 2.f * gS;
                    if (pos)
                    {
                        float c = e + 1.f; // cos pc = 1 + d/2
#pragma unroll
                        for (int l = 1; l < MAXM; ++l)
                        {
                            glam[l] = fmaf(g2, c, glam[l]);
                            e = fmaf(dl, c, e);
                            c = c + e;
                        }
                    }
                    else
                    {
                        float c = e - 1.f; // cos pc = d/2 - 1
#pragma unroll
                        for (int l = 1; l < MAXM; ++l)
                        {
                            glam[l] = fmaf(g2, c, glam[l]);
                            e = fmaf(dl, c, -e);
                            c = e - c;
                        }
                    }
                }
                t = __fadd_rn(t, a.step);
                p = __fadd_rn(p, phase_step);
                pc = rclamp(p, -kPiF, 0.0f);
                if (alpha >= a.ert)
                    break;
            }
        }
#pragma unroll
        for (int l = 0; l < MAXM; ++l)
            if (l < n)
                a.grad_lambda[idx + l] = glam[l];
        a.grad_bounds[pix] = make_float2(glo, ghi);
    }
    cache.flush(s_g);
    __syncthreads();
    for (int i = tid; i < 4 * 256; i += blockDim.x * blockDim.y)
    {
        const int ch = i >> 8, e = i & 255;
        float v = 0.f;
#pragma unroll
        for (int c = 0; c < kTfCopies; ++c)
            v += s_gall[(4 * c + ch) * kTfCopyStride + e];
        if (v != 0.f)
            atomicAdd(reinterpret_cast<float *>(a.grad_tf + e) + ch, v);
    }
}

// ------------------------------------------------------------------------------------------------------------
// preparation adjoint (prepare_moments_from_std_coding -> prepareMESELagrange, src/moment_preparation.h:55-64,
// src/mese/MESE_dynamic.h:35-211)
// ------------------------------------------------------------------------------------------------------------
//
// The forward per pixel, with x the Levinson solution, P = 2 pi x, E the exponential moments and Eh = E with its
// zeroth halved (the arrays the forward kept):
//   A_q = sum_j P_j conj(P_{j+q}),  acc_k = sum_{q>=k} Im(A_q Eh_{q-k}),  lambda_k = acc_k / (pi P_0)
// and x = T^-1 e_0 for the Hermitian Toeplitz matrix T of E (diagonal Re E_0), restricted to its leading nn x nn
// block when Levinson's Herglotz check latched at step nn (x is then zero from nn on and independent of E_d,
// d >= nn).  The reverse sweep needs no recursion run backwards:
// * Levinson: with gsol the adjoint of x, y = T^-1 gsol and dT = -y x^H, which sums along the diagonals to
//   E_d: -sum_c (y_{c+d} conj(x_c) + conj(y_c) x_{c+d}) (d >= 1) and -sum_c Re(y_c conj(x_c)) (d = 0, real).
//   T^-1 comes from x itself (Gohberg-Semencul): T^-1 = (L(x) L(x)^H - L(v) L(v)^H) / x_0 with L(.) the lower
//   triangular Toeplitz matrix of a vector and v = (0, conj(x_{nn-1}), ..., conj(x_1)), four triangular products.
// * Exponential moments: E = E_0 exp(2 pi i X(z)) as power series with X(z) = sum_{k>=1} x'_k z^k (x' the biased
//   moments; E_l = (2 pi i / l) sum_{j<l} (l - j) x'_{l-j} E_j is its recurrence), so dE_l / dx'_k = 2 pi i E_{l-k}
//   (k >= 1) and dE_l / dphi = i E_l, phi = pi x'_0 - pi / 2 (with E_0 undoubled).
// Every step is then a correlation or a triangular product: lane r of a warp forms output r (and r + 32) by a
// loop over the pixel's arrays in shared memory, padded with zeros so every lane runs the same loop.
//
// Complex adjoints are carried as d L / d re + i d L / d im.

__device__ __forceinline__ float2 cmul2(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a conj(b)
__device__ __forceinline__ float2 cmulcj(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
__device__ __forceinline__ void cacc(float2 &s, float2 v)
{
    s.x += v.x;
    s.y += v.y;
}

// two consecutive complex values (an even index of a 16-byte aligned array) in one shared-memory load: the operand
// every lane reads at the same index comes in pairs, halving those loads
__device__ __forceinline__ float4 ld_pair(const float2 *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// per warp in shared memory (complex values as float2), M = MAXM (even: the loops below step over index pairs and read
// one entry past an odd bound, which every array holds as zero)
template <int M> struct PrepAdjSmem
{
    float2 xp[3 * M]; // P at offset M, zeros on both sides
    float2 eh[2 * M]; // Eh at offset M, zeros below
    float2 ww[2 * M]; // v (in P's scale) at offset M, zeros below
    float2 a[2 * M];  // A, then y; zeros above
    float2 ga[M];     // adjoint of A
    float2 gp[M];     // adjoint of P
    float2 ge[M];     // adjoint of Eh, then of the undoubled E
    float4 t[M];      // L(P)^H gP and L(v)^H gP
    float gc[M];      // d loss / d lambda, then d loss / d acc
};

constexpr int kPrepAdjWarps = 4;

template <int MAXM>
__global__ void __launch_bounds__(32 * kPrepAdjWarps) prepare_adjoint_kernel(int num_pixels, int m,
                                                                             const float2 *__restrict__ keep,
                                                                             float bias, const float *grad_lambda,
                                                                             float *grad_moments)
{
    __shared__ PrepAdjSmem<MAXM> s_all[kPrepAdjWarps];
    PrepAdjSmem<MAXM> &s = s_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int pix = blockIdx.x * kPrepAdjWarps + (threadIdx.x >> 5);
    if (pix >= num_pixels)
        return; // whole warps
    constexpr float kPi = 3.14159265358979f;
    constexpr float kTwoPi = 6.283185307179586f;
    constexpr int M = MAXM;
    const int n = m < MAXM ? m : MAXM;
    const size_t idx = (size_t)pix * (size_t)m;
    const float2 *kp = keep + 2 * idx;
    const float2 z2 = make_float2(0.f, 0.f);

    bool any = false;
    int last = -1;
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int k = lane + 32 * i;
        const float g = k < n ? grad_lambda[idx + k] : 0.f;
        any |= g != 0.f;
        const float2 pk = k < n ? kp[k] : z2;
        if (pk.x != 0.f || pk.y != 0.f)
            last = k;
        s.xp[k] = z2;
        s.xp[M + k] = pk;
        s.xp[2 * M + k] = z2;
        s.eh[k] = z2;
        s.eh[M + k] = k < n ? kp[m + k] : z2;
        s.ww[k] = z2;
        s.a[M + k] = z2;
        s.gc[k] = g;
    }
    if (!__any_sync(kFull, any))
    {
        for (int k = lane; k < n; k += 32)
            grad_moments[idx + k] = 0.f;
        return;
    }
    // the leading block Levinson solved: past the last non-zero entry of x every step latched
    const int nn = __reduce_max_sync(kFull, last) + 1;
    __syncwarp();

    // A_q
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int q = lane + 32 * i;
        float2 acc = z2;
        for (int j = 0; j < n; j += 2)
        {
            const float4 pj = ld_pair(&s.xp[M + j]);
            cacc(acc, cmulcj(lo2(pj), s.xp[M + j + q]));
            cacc(acc, cmulcj(hi2(pj), s.xp[M + j + 1 + q]));
        }
        s.a[q] = q < n ? acc : z2;
    }
    __syncwarp();
    // d loss / d norm = sum_k glambda_k acc_k
    float gn = 0.f;
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int k = lane + 32 * i;
        float acc = 0.f;
        for (int d = 0; d < n; d += 2)
        {
            const float4 e = ld_pair(&s.eh[M + d]);
            const float2 a0 = s.a[k + d], a1 = s.a[k + d + 1];
            acc += a0.x * e.y + a0.y * e.x;
            acc += a1.x * e.w + a1.y * e.z;
        }
        gn += s.gc[k] * acc;
    }
    gn = warp_sum(gn);
    const float P0 = s.xp[M].x;
    const float norm = 1.f / (kPi * P0);
    __syncwarp();
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
        s.gc[lane + 32 * i] *= norm;
    __syncwarp();
    // acc_k = sum_q Im(A_q Eh_{q-k}): gA_q += gacc_k (Eh_{q-k}.y, Eh_{q-k}.x), gEh_d += gacc_k (A_{k+d}.y, A_{k+d}.x)
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int q = lane + 32 * i;
        float2 gA = z2, gE = z2;
        for (int k = 0; k < n; k += 2)
        {
            const float2 g = *reinterpret_cast<const float2 *>(&s.gc[k]);
            const float2 e0 = s.eh[M + q - k], e1 = s.eh[M + q - k - 1];
            const float2 a0 = s.a[k + q], a1 = s.a[k + q + 1];
            gA.x += g.x * e0.y + g.y * e1.y;
            gA.y += g.x * e0.x + g.y * e1.x;
            gE.x += g.x * a0.y + g.y * a1.y;
            gE.y += g.x * a0.x + g.y * a1.x;
        }
        s.ga[q] = q < n ? gA : z2;
        s.ge[q] = q < n ? gE : z2;
    }
    __syncwarp();
    // A_q = sum_j P_j conj(P_{j+q}): gP_j += gA_q P_{j+q} + conj(gA_q) P_{j-q}; P_0 also through the norm
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int j = lane + 32 * i;
        float2 g = z2;
        for (int q = 0; q < n; q += 2)
        {
            const float4 gA = ld_pair(&s.ga[q]);
            cacc(g, cmul2(lo2(gA), s.xp[M + j + q]));
            cacc(g, cmulcj(s.xp[M + j - q], lo2(gA)));
            cacc(g, cmul2(hi2(gA), s.xp[M + j + q + 1]));
            cacc(g, cmulcj(s.xp[M + j - q - 1], hi2(gA)));
        }
        if (j == 0)
            g.x -= gn * norm / P0;
        s.gp[j] = j < nn ? g : z2;
        // v_i = conj(x_{nn-i}), 1 <= i < nn (in P's scale)
        if (j >= 1 && j < nn)
        {
            const float2 p = s.xp[M + nn - j];
            s.ww[M + j] = make_float2(p.x, -p.y);
        }
        else
            s.ww[M + j] = z2;
    }
    __syncwarp();
    // Levinson: gsol = 2 pi gP, y = T^-1 gsol = (L(P) L(P)^H gP - L(v) L(v)^H gP) / P_0
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int r = lane + 32 * i;
        float2 t1 = z2, t2 = z2;
        for (int c = 0; c < nn; c += 2)
        {
            const float4 g = ld_pair(&s.gp[c]);
            cacc(t1, cmulcj(lo2(g), s.xp[M + c - r]));
            cacc(t2, cmulcj(lo2(g), s.ww[M + c - r]));
            cacc(t1, cmulcj(hi2(g), s.xp[M + c + 1 - r]));
            cacc(t2, cmulcj(hi2(g), s.ww[M + c + 1 - r]));
        }
        s.t[r] = r < nn ? make_float4(t1.x, t1.y, t2.x, t2.y) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    const float inv_p0 = 1.f / P0;
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int r = lane + 32 * i;
        float2 y = z2;
        for (int c = 0; c < nn; ++c)
        {
            const float4 tc = s.t[c];
            const float2 p = s.xp[M + r - c], v = s.ww[M + r - c];
            cacc(y, cmul2(p, make_float2(tc.x, tc.y)));
            const float2 vt = cmul2(v, make_float2(tc.z, tc.w));
            y.x -= vt.x;
            y.y -= vt.y;
        }
        s.a[r] = r < nn ? make_float2(y.x * inv_p0, y.y * inv_p0) : z2; // A is no longer read
    }
    __syncwarp();
    // dT = -y x^H onto E (x = P / 2 pi); the total adjoint of the undoubled E: gE'_0 = gEh_0 + 2 gE_0(T), gE'_d = gEh_d
    // + gE_d(T)
    constexpr float kInv2Pi = 0.15915494309189535f;
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int d = lane + 32 * i;
        float2 lev = z2;
        for (int c = 0; c < nn; c += 2)
        {
            const float4 pc = ld_pair(&s.xp[M + c]), yc = ld_pair(&s.a[c]);
            cacc(lev, cmulcj(s.a[c + d], lo2(pc)));
            cacc(lev, cmulcj(s.xp[M + c + d], lo2(yc)));
            cacc(lev, cmulcj(s.a[c + d + 1], hi2(pc)));
            cacc(lev, cmulcj(s.xp[M + c + d + 1], hi2(yc)));
        }
        float2 g = s.ge[d];
        if (d == 0)
            g.x -= kInv2Pi * lev.x; // 2 * (-(1/2pi) Re sum y_c conj(x_c)) / 2: lev.x counts the sum twice
        else if (d < nn)
        {
            g.x -= kInv2Pi * lev.x;
            g.y -= kInv2Pi * lev.y;
        }
        s.ge[d] = g;
    }
    __syncwarp();
    // moments: gx_k = -2 pi sum_{l>=k} Im(conj(gE'_l) E'_{l-k}) (k >= 1), gx_0 = pi dphi = -pi sum_l Im(conj(gE'_l) E'_l)
    const float omb = 1.f - bias;
#pragma unroll
    for (int i = 0; i < MAXM / 32; ++i)
    {
        const int k = lane + 32 * i;
        float acc = 0.f;
        for (int l = 0; l < n; l += 2)
        {
            const float4 g = ld_pair(&s.ge[l]);
            const float2 e0 = s.eh[M + l - k], e1 = s.eh[M + l + 1 - k];
            acc += g.x * e0.y - g.y * e0.x;
            acc += g.z * e1.y - g.w * e1.x;
        }
        if (k < n)
            grad_moments[idx + k] = omb * (k == 0 ? -kPi * acc : -kTwoPi * acc);
    }
}

// ------------------------------------------------------------------------------------------------------------
// generation adjoint (a regular grid)
// ------------------------------------------------------------------------------------------------------------

struct GenAdjArgs
{
    GridView grid;
    float *grad_volume; // nx*ny*nz, accumulated
    DeviceCamera cam;
    int width, height, m;
    float step, data_min, data_max, bound_eps;
    const float *moments;      // W*H*m (normalized, as generated)
    const float4 *bounds4;     // (lo, hi, min, max)
    const float *grad_moments; // W*H*m
    const float2 *grad_bounds; // W*H, from the re-march adjoint
    int *error_flag;
};

// d loss / d sample scattered to the eight corners of the trilinear sample at q (the sample's own corners and
// weights, with the clamp to the grid)
__device__ __forceinline__ void scatter_sample(const GridView &g, float *grad, const GridPoint &q, float gs)
{
    const int x0 = min(max((int)q.fl[0], 0), g.nx - 1), x1 = min(max((int)q.fl[0] + 1, 0), g.nx - 1);
    const float wx[2] = {(1.f - q.a[0]) * gs, q.a[0] * gs};
#pragma unroll
    for (int c = 0; c < 4; ++c)
    {
        const int dy = c & 1, dz = c >> 1;
        const float wyz = (dy ? q.a[1] : 1.f - q.a[1]) * (dz ? q.a[2] : 1.f - q.a[2]);
        const int y = min(max((int)q.fl[1] + dy, 0), g.ny - 1), z = min(max((int)q.fl[2] + dz, 0), g.nz - 1);
        float *row = grad + (size_t)(z * g.ny + y) * (size_t)g.nx;
        const float w0 = wx[0] * wyz, w1 = wx[1] * wyz;
        if (w0 != 0.f)
            atomicAdd(row + x0, w0);
        if (w1 != 0.f)
            atomicAdd(row + x1, w1);
    }
}

// d map_density / d sample: 1 / (dmax - dmin) inside (0, 1), 0 where clamped
__device__ __forceinline__ float map_density_derivative(float s, float dmin, float dmax)
{
    const float v = __fdiv_rn(__fsub_rn(s, dmin), __fsub_rn(dmax, dmin));
    return (v > 0.f && v < 1.f) ? 1.f / (dmax - dmin) : 0.f;
}

// Quad per ray as in the forward kernel: per round the four lanes take four consecutive samples; each lane sums
// over the moments it owns (j = q + 4i) the two per-segment series
//     A_k = sum_j rbar_j alpha_j(h) cos(j p_k),   B_k = sum_j rbar_j beta_j(h) sin(j p_k)
// (rbar = d loss / d raw moment), a butterfly over the quad completes them, and the sample between segments k and
// k + 1 receives (A_k - B_k) + (A_{k+1} + B_{k+1}).  The last sample of a round waits for the next round's first
// segment (or the final segment to t_far).
template <int NJ> __global__ void __launch_bounds__(128) generate_adjoint_kernel(const GenAdjArgs a)
{
    const int lane = threadIdx.x & 31;
    const int q = lane & 3;
    const int qbase = lane & ~3;
    const int px = blockIdx.x * 8 + (lane >> 2);
    const int py = blockIdx.y * 4 + (threadIdx.x >> 5);
    const bool in_image = (px < a.width) && (py < a.height);
    const size_t pix = in_image ? (size_t)py * (size_t)a.width + (size_t)px : 0;

    float o[3], d[3];
    float t_near = 0.f, t_far = 0.f;
    bool hit = false;
    float4 b4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 gb = make_float2(0.f, 0.f);
    if (in_image)
    {
        float nx, ny;
        pixel_ndc(px, py, a.width, a.height, nx, ny);
        eye_ray(a.cam, nx, ny, o, d);
        hit = intersect_aabb(o, d, a.grid.dmin, a.grid.dmax, t_near, t_far);
        t_near = rmax(t_near, a.cam.znear);
        hit = hit && (t_far > 0.f);
        b4 = a.bounds4[pix];
        gb = a.grad_bounds[pix];
    }

    // rbar: d loss / d trig_j, the moment integral before the 1/pi scale and the bounds transform
    // m_0 = (trig_0 / pi - lo) / (hi - lo), m_j = trig_j / pi / (hi - lo) (raymarch_generate.h:115-131)
    const float lo = b4.x, hi = b4.y, span = hi - lo;
    float rbar[NJ];
    float glo = q == 0 ? gb.x : 0.f, ghi = q == 0 ? gb.y : 0.f;
#pragma unroll
    for (int i = 0; i < NJ; ++i)
    {
        const int j = q + 4 * i;
        rbar[i] = 0.f;
        if (hit && j < a.m)
        {
            const float mj = a.moments[pix * (size_t)a.m + j];
            const float gm = a.grad_moments[pix * (size_t)a.m + j];
            rbar[i] = gm / span * kMInvPi;
            glo += gm * (j == 0 ? mj - 1.f : mj) / span;
            ghi -= gm * mj / span;
        }
    }
    // every lane needs the quad's totals of the bound adjoints
    glo += __shfl_xor_sync(kFull, glo, 1);
    ghi += __shfl_xor_sync(kFull, ghi, 1);
    glo += __shfl_xor_sync(kFull, glo, 2);
    ghi += __shfl_xor_sync(kFull, ghi, 2);
    // the bounds transform: lo = max(min - eps, 0), hi = min(max + eps, 1)
    const float g_min = (__fsub_rn(b4.z, a.bound_eps) > 0.f) ? glo : 0.f;
    const float g_max = (__fadd_rn(b4.w, a.bound_eps) < 1.f) ? ghi : 0.f;

    float pti = 0.f, pss = 0.f;
    float t = t_near;
    const float step = a.step;
    if (hit)
    {
        pti = (float)(3.141592653589793 / (double)__fsub_rn(t_far, t_near));
        pss = (float)(3.141592653589793 * (double)__fdiv_rn(step, __fsub_rn(t_far, t_near)));
    }
    const float h = 0.5f * pss;
    // per-lane series coefficients for the regular segments
    float ca[NJ], cb[NJ];
#pragma unroll
    for (int i = 0; i < NJ; ++i)
    {
        float al, be;
        seg_coeffs(q + 4 * i, h, al, be);
        ca[i] = rbar[i] * al;
        cb[i] = rbar[i] * be;
    }

    // the sample waiting for its left-end weight: lane 0 holds the first sample (at t_near)
    bool min_done = false, max_done = false;
    GridPoint pend_q = {};
    float pend_g = 0.f, pend_f = 0.f;
    bool pend = false;
    float p_tail = -kPiF;
    if (hit)
    {
        const GridPoint q0 = grid_point(a.grid, __fadd_rn(o[0], __fmul_rn(t, d[0])),
                                        __fadd_rn(o[1], __fmul_rn(t, d[1])), __fadd_rn(o[2], __fmul_rn(t, d[2])));
        const float s0 = grid_blend(a.grid, q0);
        const float f0 = map_density(s0, a.data_min, a.data_max);
        float g0 = 0.f;
        if (f0 == b4.z && !min_done)
        {
            g0 += g_min;
            min_done = true;
        }
        if (f0 == b4.w && !max_done)
        {
            g0 += g_max;
            max_done = true;
        }
        pend = (q == 0);
        pend_g = g0;
        pend_f = s0;
        pend_q = q0;
    }
    int cap = 0;
    if (hit)
    {
        const float est = __fsub_rn(t_far, t_near) / step;
        cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
    }
    int marched = 0;
    bool active = hit;
    while (__any_sync(kFull, active))
    {
        float tt = t, my_t = 0.f;
        int nv = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            const float tn = __fadd_rn(tt, step);
            if (active && nv == i && tn < t_far)
            {
                nv = i + 1;
                tt = tn;
                if (q == i)
                    my_t = tn;
            }
        }
        const bool my_valid = q < nv;
        float p_my = 0.f, s_my = 0.f, f_my = 0.f;
        GridPoint q_my = {};
        cf z = {1.f, 0.f};
        if (my_valid)
        {
            p_my = sub_pi(__fmul_rn(__fsub_rn(my_t, t_near), pti));
            q_my = grid_point(a.grid, __fadd_rn(o[0], __fmul_rn(my_t, d[0])), __fadd_rn(o[1], __fmul_rn(my_t, d[1])),
                              __fadd_rn(o[2], __fmul_rn(my_t, d[2])));
            s_my = grid_blend(a.grid, q_my);
            f_my = map_density(s_my, a.data_min, a.data_max);
            // the segment's phase factor only weighs the gradient (no forward value is replayed from it): the
            // hardware sine and cosine (absolute error about 4e-7 on [-pi - h, 0]) are accurate enough for it
            float sn, cs;
            __sincosf(p_my - h, &sn, &cs);
            z = {cs, -sn};
        }
        // partial A, B of the four segments over this lane's moments j = q + 4i: both parts of z^j follow the
        // three-term recurrence x_{j+4} = 2 cos(4 theta) x_j - x_{j-4} from z^q and z^(q+4), one FMA per part and
        // moment (the forward's scheme) instead of a complex rotation's four operations
        float As[4], Bs[4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            cf zs;
            zs.x = __shfl_sync(kFull, z.x, qbase + s);
            zs.y = __shfl_sync(kFull, z.y, qbase + s);
            const cf z2 = csq(zs);
            const cf v = csq(z2);
            cf w = {1.f, 0.f};
            w = (q == 1) ? zs : w;
            w = (q == 2) ? z2 : w;
            w = (q == 3) ? cmul(z2, zs) : w;
            cf wn = cmul(w, v);
            const float c4 = 2.f * v.x;
            float A = 0.f, B = 0.f;
#pragma unroll
            for (int i = 0; i < NJ; ++i)
            {
                // Re(z^j) = cos(j p), Im(z^j) = -sin(j p)
                A = fmaf(ca[i], w.x, A);
                B = fmaf(-cb[i], w.y, B);
                if (i + 1 < NJ)
                {
                    const cf next = {fmaf(c4, wn.x, -w.x), fmaf(c4, wn.y, -w.y)};
                    w = wn;
                    wn = next;
                }
            }
            As[s] = A;
            Bs[s] = B;
        }
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            As[s] += __shfl_xor_sync(kFull, As[s], 1);
            Bs[s] += __shfl_xor_sync(kFull, Bs[s], 1);
            As[s] += __shfl_xor_sync(kFull, As[s], 2);
            Bs[s] += __shfl_xor_sync(kFull, Bs[s], 2);
        }
        // warp-wide exchanges first (every lane of the warp takes part), then the per-quad work
        const unsigned qmask = 0xfu << qbase;
        const unsigned is_min = __ballot_sync(kFull, my_valid && f_my == b4.z) & qmask;
        const unsigned is_max = __ballot_sync(kFull, my_valid && f_my == b4.w) & qmask;
        const float p_last = __shfl_sync(kFull, p_my, qbase + (nv > 0 ? nv - 1 : 0));
        if (nv > 0)
        {
            // the pending sample (the previous round's last, or the first sample) is the left end of segment 0
            if (pend)
            {
                const float gsamp = (pend_g + As[0] + Bs[0]) * map_density_derivative(pend_f, a.data_min, a.data_max);
                if (gsamp != 0.f)
                    scatter_sample(a.grid, a.grad_volume, pend_q, gsamp);
                pend = false;
            }
            // the bound adjoints go to the first sample equal to the minimum / maximum
            float gmy = 0.f;
            if (!min_done && is_min)
            {
                if (lane == __ffs(is_min) - 1)
                    gmy += g_min;
                min_done = true;
            }
            if (!max_done && is_max)
            {
                if (lane == __ffs(is_max) - 1)
                    gmy += g_max;
                max_done = true;
            }
            // own segment (right end) and the next segment (left end)
            float a_own = As[0], b_own = Bs[0], a_next = As[1], b_next = Bs[1];
#pragma unroll
            for (int s = 1; s < 4; ++s)
                if (q == s)
                {
                    a_own = As[s];
                    b_own = Bs[s];
                    a_next = s + 1 < 4 ? As[(s + 1) & 3] : 0.f;
                    b_next = s + 1 < 4 ? Bs[(s + 1) & 3] : 0.f;
                }
            if (my_valid)
            {
                gmy += a_own - b_own;
                if (q + 1 < nv)
                {
                    const float gsamp = (gmy + a_next + b_next) * map_density_derivative(s_my, a.data_min, a.data_max);
                    if (gsamp != 0.f)
                        scatter_sample(a.grid, a.grad_volume, q_my, gsamp);
                }
                else
                {
                    pend = true;
                    pend_g = gmy;
                    pend_f = s_my;
                    pend_q = q_my;
                }
            }
            p_tail = p_last;
            t = tt;
        }
        if (nv < 4)
            active = false;
        marched += nv;
        if (active && marched > cap)
        {
            active = false;
            if (q == 0)
                atomicExch(a.error_flag, 1);
        }
    }

    // the final segment [p_tail, 0] between the pending sample and the sample at t_far
    float AL = 0.f, BL = 0.f;
    if (hit)
    {
        const float hL = -0.5f * p_tail;
        float snL, csL;
        sincosf(0.5f * p_tail, &snL, &csL);
        const cf zL = {csL, -snL};
        const cf zL2 = csq(zL);
        const cf vL = csq(zL2);
        cf w = {1.f, 0.f};
        w = (q == 1) ? zL : w;
        w = (q == 2) ? zL2 : w;
        w = (q == 3) ? cmul(zL2, zL) : w;
#pragma unroll
        for (int i = 0; i < NJ; ++i)
        {
            float al, be;
            seg_coeffs(q + 4 * i, hL, al, be);
            AL = fmaf(rbar[i] * al, w.x, AL);
            BL = fmaf(-rbar[i] * be, w.y, BL);
            w = cmul(w, vL);
        }
    }
    AL += __shfl_xor_sync(kFull, AL, 1);
    BL += __shfl_xor_sync(kFull, BL, 1);
    AL += __shfl_xor_sync(kFull, AL, 2);
    BL += __shfl_xor_sync(kFull, BL, 2);
    if (!hit)
        return;
    if (pend)
    {
        const float gsamp = (pend_g + AL + BL) * map_density_derivative(pend_f, a.data_min, a.data_max);
        if (gsamp != 0.f)
            scatter_sample(a.grid, a.grad_volume, pend_q, gsamp);
    }
    if (q == 0)
    {
        const GridPoint qf = grid_point(a.grid, __fadd_rn(o[0], __fmul_rn(t_far, d[0])),
                                        __fadd_rn(o[1], __fmul_rn(t_far, d[1])), __fadd_rn(o[2], __fmul_rn(t_far, d[2])));
        const float s_far = grid_blend(a.grid, qf);
        const float f_far = map_density(s_far, a.data_min, a.data_max);
        float g = AL - BL;
        if (!min_done && f_far == b4.z)
            g += g_min;
        if (!max_done && f_far == b4.w)
            g += g_max;
        const float gsamp = g * map_density_derivative(s_far, a.data_min, a.data_max);
        if (gsamp != 0.f)
            scatter_sample(a.grid, a.grad_volume, qf, gsamp);
    }
}

template <int MAXM> cudaError_t launch_recon_adj(const ReconAdjDev &a, cudaStream_t stream)
{
    const int bytes = kTfCopies * 4 * kTfCopyStride * (int)sizeof(float);
    cudaError_t e =
        cudaFuncSetAttribute(reconstruct_adjoint_kernel<MAXM>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess)
        return e;
    dim3 block(16, 8);
    dim3 grid((a.width + 15) / 16, (a.height + 7) / 8);
    reconstruct_adjoint_kernel<MAXM><<<grid, block, bytes, stream>>>(a);
    return cudaGetLastError();
}

template <int MAXM>
cudaError_t launch_prep_adj(int P, int m, const float2 *keep, float bias, const float *gl, float *gm,
                            cudaStream_t stream)
{
    prepare_adjoint_kernel<MAXM><<<(P + kPrepAdjWarps - 1) / kPrepAdjWarps, 32 * kPrepAdjWarps, 0, stream>>>(
        P, m, keep, bias, gl, gm);
    return cudaGetLastError();
}

template <int NJ> void launch_gen_adj(const GenAdjArgs &a, cudaStream_t stream)
{
    dim3 grid((a.width + 7) / 8, (a.height + 3) / 4);
    generate_adjoint_kernel<NJ><<<grid, 128, 0, stream>>>(a);
}

} // namespace

cudaError_t launch_reconstruct_adjoint(const ReconAdjArgs &r, int *error_flag, cudaStream_t stream)
{
    ReconAdjDev a;
    a.cam = *r.cam;
    a.width = r.width;
    a.height = r.height;
    a.m = r.m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = r.dmin[i];
        a.dmax[i] = r.dmax[i];
    }
    a.pmoments = r.pmoments;
    a.bounds4 = r.bounds4;
    a.tf = r.tf;
    a.step = r.step;
    a.emission = r.emission;
    a.ert = r.ert;
    a.rgba = r.rgba;
    a.grad_rgba = r.grad_rgba;
    a.grad_lambda = r.grad_lambda;
    a.grad_bounds = r.grad_bounds;
    a.grad_tf = r.grad_tf;
    a.tf_linear = r.tf_linear;
    a.error_flag = error_flag;
    if (r.m <= 8)
        return launch_recon_adj<8>(a, stream);
    if (r.m <= 16)
        return launch_recon_adj<16>(a, stream);
    if (r.m <= 32)
        return launch_recon_adj<32>(a, stream);
    return launch_recon_adj<64>(a, stream);
}

cudaError_t launch_prepare_adjoint(int num_pixels, int m, const float2 *keep, float bias, const float *grad_lambda,
                                   float *grad_moments, cudaStream_t stream)
{
    if (m <= 32)
        return launch_prep_adj<32>(num_pixels, m, keep, bias, grad_lambda, grad_moments, stream);
    return launch_prep_adj<64>(num_pixels, m, keep, bias, grad_lambda, grad_moments, stream);
}

cudaError_t launch_generate_adjoint(const GridView &grid, float *grad_volume, const DeviceCamera &cam,
                                    const mraygb_generation_params &gp, int width, int height, int m,
                                    const float *moments, const float4 *bounds4, const float *grad_moments,
                                    const float2 *grad_bounds, int *error_flag, cudaStream_t stream)
{
    GenAdjArgs a;
    a.grid = grid;
    a.grad_volume = grad_volume;
    a.cam = cam;
    a.width = width;
    a.height = height;
    a.m = m;
    a.step = gp.step_size;
    a.data_min = gp.data_min;
    a.data_max = gp.data_max;
    a.bound_eps = gp.transform_bound_eps;
    a.moments = moments;
    a.bounds4 = bounds4;
    a.grad_moments = grad_moments;
    a.grad_bounds = grad_bounds;
    a.error_flag = error_flag;
    const int nj = (m + 3) / 4;
    if (nj <= 2)
        launch_gen_adj<2>(a, stream);
    else if (nj <= 4)
        launch_gen_adj<4>(a, stream);
    else if (nj <= 8)
        launch_gen_adj<8>(a, stream);
    else
        launch_gen_adj<16>(a, stream);
    return cudaGetLastError();
}

} // namespace mraygb
