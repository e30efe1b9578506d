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
// along a ray.
//
// Memory: none of the three adjoints keeps a per-sample tape.  The re-march adjoint replays the forward march
// and uses the final radiance of the forward pass for the suffix sums of front-to-back compositing (d L / d tau_k
// needs the radiance gathered behind sample k, which is the final radiance minus the radiance so far); the
// generation adjoint replays the sample positions; the preparation adjoint runs Levinson's recursion backwards by
// inverting each update (old_k = new_k + u conj(new_{j-k})), so it stores only the reflection coefficients.

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
    int *error_flag;
};

// accumulates the B-spline weights times g into the shared transfer-function gradient through a cache of the
// last four entries: consecutive samples of a ray mostly fall between the same knots
struct TfGradCache
{
    int base = -1000;
    float4 acc[4];

    __device__ __forceinline__ void flush(float4 *s_g)
    {
        if (base <= -1000)
            return;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int x = min(max(base - 1 + j, 0), 255);
            atomicAdd(&s_g[x].x, acc[j].x);
            atomicAdd(&s_g[x].y, acc[j].y);
            atomicAdd(&s_g[x].z, acc[j].z);
            atomicAdd(&s_g[x].w, acc[j].w);
        }
    }
    __device__ __forceinline__ void add(float4 *s_g, const BSplineTap &k, float4 g)
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

// The transfer-function gradient of a block is accumulated in kTfCopies copies of the 256-entry table in shared
// memory, lane l adding to copy l mod kTfCopies: neighbouring rays sample similar densities at the same step, and
// shared-memory atomics on one address from many lanes of a warp serialize.
constexpr int kTfCopies = 8;

template <int MAXM> __global__ void __launch_bounds__(128, 4) reconstruct_adjoint_kernel(const ReconAdjDev a)
{
    __shared__ float4 s_tf[256];
    extern __shared__ float4 s_gall[]; // kTfCopies * 256 (dynamic: above the 48 KiB of static shared memory)
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    for (int i = tid; i < 256; i += blockDim.x * blockDim.y)
        s_tf[i] = a.tf[i];
    for (int i = tid; i < kTfCopies * 256; i += blockDim.x * blockDim.y)
        s_gall[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    float4 *s_g = s_gall + (tid % kTfCopies) * 256;

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
                const float S = mese_series<MAXM>(lam2, lam0, pc);
                const float r = atanf(S) * 0.318309886f + 0.5f;
                const float fs = r * span + lo;
                const BSplineTap k = bspline_tap(fs);
                float4 s, dt;
                tf_bspline_value_derivative(s_tf, k, s, dt);
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
                const float gS = gfs * span * 0.318309886f / fmaf(S, S, 1.f);
                glam[0] += gS;
                // cos(l pc) for l >= 1 by Reinsch's modification of the three-term recurrence (stable where pc
                // nears 0 or -pi, the two ends of every ray): with d = -4 sin^2(pc / 2) while cos pc > 0,
                //   e_{l+1} = e_l + d c_l,  c_{l+1} = c_l + e_{l+1}      (e_l = c_l - c_{l-1}),
                // and with d = 4 cos^2(pc / 2) otherwise,
                //   e_{l+1} = d c_l - e_l,  c_{l+1} = e_{l+1} - c_l      (e_l = c_l + c_{l-1})
                {
                    float sh, ch;
                    sincosf(0.5f * pc, &sh, &ch);
                    const bool pos = fabsf(pc) < 1.5707963267948966f;
                    const float sg = pos ? 1.f : -1.f;
                    const float d = pos ? -4.f * sh * sh : 4.f * ch * ch;
                    float e = 0.5f * d;
                    float c = e + sg; // cos pc: 1 + d/2, or d/2 - 1
                    const float g2 = 2.f * gS;
#pragma unroll
                    for (int l = 1; l < MAXM; ++l)
                    {
                        glam[l] = fmaf(g2, c, glam[l]);
                        e = fmaf(d, c, sg * e);
                        c = fmaf(sg, c, e);
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
    for (int i = tid; i < 256; i += blockDim.x * blockDim.y)
    {
        float4 v = s_gall[i];
#pragma unroll
        for (int c = 1; c < kTfCopies; ++c)
        {
            const float4 w = s_gall[c * 256 + i];
            v.x += w.x;
            v.y += w.y;
            v.z += w.z;
            v.w += w.w;
        }
        if (v.x != 0.f)
            atomicAdd(&a.grad_tf[i].x, v.x);
        if (v.y != 0.f)
            atomicAdd(&a.grad_tf[i].y, v.y);
        if (v.z != 0.f)
            atomicAdd(&a.grad_tf[i].z, v.z);
        if (v.w != 0.f)
            atomicAdd(&a.grad_tf[i].w, v.w);
    }
}

// ------------------------------------------------------------------------------------------------------------
// preparation adjoint (prepare_moments_from_std_coding -> prepareMESELagrange, src/moment_preparation.h:55-64,
// src/mese/MESE_dynamic.h:35-211)
// ------------------------------------------------------------------------------------------------------------

struct C2
{
    float x, y;
};
__device__ __forceinline__ C2 c2(float x, float y) { return {x, y}; }
__device__ __forceinline__ C2 operator+(C2 a, C2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ C2 operator-(C2 a, C2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ C2 operator*(C2 a, C2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ C2 operator*(float s, C2 a) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ C2 conj(C2 a) { return {a.x, -a.y}; }
__device__ __forceinline__ float abs2(C2 a) { return a.x * a.x + a.y * a.y; }

// Complex adjoints are carried as d L / d re + i d L / d im.  For w = a b: a_bar += w_bar conj(b); for w = conj(c) u:
// c_bar += conj(w_bar) u, u_bar += w_bar c.
//
// One thread per pixel, the arrays (2 KiB at 32 moments) in local memory: measured faster (1.44 ms per 512^2 launch
// at m = 31) than the same kernel with its arrays in shared memory, one lane per pixel (1.80 ms: fewer resident
// threads) or one pixel per group of 8 lanes (1.93 ms: the per-step reductions and syncs of the sequential
// recursions cost more than the split of their O(n) bodies saves).
template <int MAXM>
__global__ void __launch_bounds__(64) prepare_adjoint_kernel(int num_pixels, int m, const float *__restrict__ moments,
                                                             float bias, const float *grad_lambda,
                                                             float *grad_moments)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= num_pixels)
        return;
    const int n = m < MAXM ? m : MAXM;
    const size_t idx = (size_t)pix * (size_t)m;
    float gl[MAXM];
    bool any = false;
    for (int k = 0; k < n; ++k)
    {
        gl[k] = grad_lambda[idx + k];
        any |= gl[k] != 0.f;
    }
    if (!any)
    {
        for (int k = 0; k < n; ++k)
            grad_moments[idx + k] = 0.f;
        return;
    }
    constexpr float kPi = 3.14159265358979f;
    constexpr float kInv4Pi = 0.0795774715459477f;

    // ---- forward, keeping what the reverse sweep needs ----
    float xm[MAXM];
    C2 E[MAXM], sol[MAXM], uu[MAXM];
    uint32_t latched[(MAXM + 31) / 32];
    for (int i = 0; i < (MAXM + 31) / 32; ++i)
        latched[i] = 0u;
    xm[0] = (1.f - bias) * moments[idx] + bias * 0.5f;
    for (int i = 1; i < n; ++i)
        xm[i] = (1.f - bias) * moments[idx + i];
    // trigonometricToExponentialMoments (E[0] un-doubled inside the recurrence)
    const float phi = kPi * xm[0] - 0.5f * kPi;
    float sphi, cphi;
    sincosf(phi, &sphi, &cphi);
    E[0] = c2(kInv4Pi * cphi, kInv4Pi * sphi);
    for (int l = 1; l < n; ++l)
    {
        C2 acc = c2(0.f, 0.f);
        for (int j = 0; j < l; ++j)
            acc = acc + (float(l - j) * xm[l - j]) * E[j];
        const float w = (float)(6.283185307179586 / (double)l);
        E[l] = c2(-w * acc.y, w * acc.x);
    }
    E[0] = 2.f * E[0];
    // levinsonsAlgorithm with the invalid latch
    sol[0] = c2(1.f / E[0].x, 0.f);
    bool invalid = false;
    for (int j = 1; j < n; ++j)
    {
        C2 u = c2(0.f, 0.f);
        if (!invalid)
            for (int k = 0; k < j; ++k)
                u = u + sol[k] * E[j - k];
        float a2 = abs2(u);
        if (invalid || a2 >= 1.f)
        {
            u = c2(0.f, 0.f);
            a2 = 0.f;
            invalid = true;
            latched[j >> 5] |= 1u << (j & 31);
        }
        uu[j] = u;
        const float f = 1.f / (1.f - a2);
        const float s0 = sol[0].x;
        int k = 1, kk = j - 1;
        for (; k < kk; ++k, --kk)
        {
            const C2 p = sol[k], q = sol[kk];
            sol[k] = f * (p - conj(q) * u);
            sol[kk] = f * (q - conj(p) * u);
        }
        if (k == kk)
        {
            const C2 p = sol[k];
            sol[k] = f * (p - conj(p) * u);
        }
        sol[j] = f * ((-s0) * u);
        sol[0] = c2(f * s0, 0.f);
    }
    // P = 2 pi sol; Eh = E with Eh[0] = E[0] / 2; a_q = sum_j P_j conj(P_{j+q}); acc_k = sum_{q>=k} Im(a_q Eh_{q-k})
    constexpr float kTwoPi = 6.283185307179586f;
    C2 A[MAXM];
    float accv[MAXM];
    for (int q = 0; q < n; ++q)
    {
        C2 s = c2(0.f, 0.f);
        for (int j = 0; j + q < n; ++j)
            s = s + (kTwoPi * sol[j]) * conj(kTwoPi * sol[j + q]);
        A[q] = s;
    }
    for (int k = 0; k < n; ++k)
    {
        float s = 0.f;
        for (int q = k; q < n; ++q)
        {
            const C2 e = (q - k == 0) ? 0.5f * E[0] : E[q - k];
            s += A[q].x * e.y + A[q].y * e.x;
        }
        accv[k] = s;
    }
    const float P0 = kTwoPi * sol[0].x;
    const float norm = 1.f / (kPi * P0);

    // ---- reverse ----
    // lambda_k = norm acc_k
    float gnorm = 0.f;
    for (int k = 0; k < n; ++k)
    {
        gnorm += gl[k] * accv[k];
        gl[k] *= norm; // now d / d acc_k
    }
    // acc_k = sum_{q>=k} Im(A_q Eh_{q-k}): A_bar_q += acc_bar_k (Eh.y, Eh.x); Eh_bar_{q-k} += acc_bar_k (A.y, A.x)
    C2 gE[MAXM], gP[MAXM];
    for (int i = 0; i < n; ++i)
    {
        gE[i] = c2(0.f, 0.f);
        gP[i] = c2(0.f, 0.f);
    }
    for (int q = 0; q < n; ++q)
    {
        C2 gA = c2(0.f, 0.f);
        for (int k = 0; k <= q; ++k)
        {
            const C2 e = (q - k == 0) ? 0.5f * E[0] : E[q - k];
            gA = gA + gl[k] * c2(e.y, e.x);
            gE[q - k] = gE[q - k] + gl[k] * c2(A[q].y, A[q].x);
        }
        // A_q = sum_j P_j conj(P_{j+q})
        for (int j = 0; j + q < n; ++j)
        {
            const C2 pj = kTwoPi * sol[j], pq = kTwoPi * sol[j + q];
            gP[j] = gP[j] + gA * pq;
            gP[j + q] = gP[j + q] + conj(gA) * pj;
        }
    }
    gP[0].x += gnorm * (-norm / P0);
    gE[0] = 0.5f * gE[0]; // Eh[0] = E[0] / 2
    // sol_bar = 2 pi P_bar (reuse gP)
    for (int i = 0; i < n; ++i)
        gP[i] = kTwoPi * gP[i];

    // Levinson backwards: sol holds the state after step j, gP its adjoint
    for (int j = n - 1; j >= 1; --j)
    {
        const C2 u = uu[j];
        const float a2 = abs2(u);
        const float f = 1.f / (1.f - a2);
        // f_bar = sum_k Re(conj(s_bar_k) new_k) / f
        float gf = 0.f;
        for (int k = 0; k <= j; ++k)
            gf += gP[k].x * sol[k].x + gP[k].y * sol[k].y;
        gf /= f;
        // old_k = new_k + u conj(new_{j-k}), k = 0..j-1 (pairs in place)
        {
            int k = 0, kk = j;
            for (; k < kk; ++k, --kk)
            {
                const C2 p = sol[k], q = sol[kk];
                sol[k] = p + u * conj(q);
                sol[kk] = q + u * conj(p);
            }
            if (k == kk)
            {
                const C2 p = sol[k];
                sol[k] = p + u * conj(p);
            }
            sol[j] = c2(0.f, 0.f);
        }
        // v_bar = f s_bar; u_bar = -f sum_{k=1..j} s_bar_k old_{j-k}; old_bar_i = f s_bar_i - conj(f s_bar_{j-i}) u
        C2 gu = c2(0.f, 0.f);
        for (int k = 1; k <= j; ++k)
            gu = gu - (f * gP[k]) * sol[j - k];
        {
            int i = 0, ii = j;
            for (; i < ii; ++i, --ii)
            {
                const C2 vi = f * gP[i], vii = f * gP[ii];
                gP[i] = vi - conj(vii) * u;
                gP[ii] = vii - conj(vi) * u; // ii = j: old_j is the constant 0, its adjoint is dropped below
            }
            if (i == ii)
            {
                const C2 vi = f * gP[i];
                gP[i] = vi - conj(vi) * u;
            }
            gP[j] = c2(0.f, 0.f);
        }
        if (!((latched[j >> 5] >> (j & 31)) & 1u))
        {
            // f = 1 / (1 - |u|^2): d f / d u = 2 f^2 u
            gu = gu + (2.f * gf * f * f) * u;
            // u = sum_{k<j} old_k E_{j-k}
            for (int k = 0; k < j; ++k)
            {
                const C2 ok = sol[k];
                gP[k] = gP[k] + gu * conj(E[j - k]);
                gE[j - k] = gE[j - k] + gu * conj(ok);
            }
        }
    }
    // sol_0 = 1 / E_0.x (real)
    gE[0].x += -gP[0].x / (E[0].x * E[0].x);

    // trigonometricToExponentialMoments backwards: E[0] = 2 e_0
    float gx[MAXM];
    for (int i = 0; i < n; ++i)
        gx[i] = 0.f;
    E[0] = 0.5f * E[0];
    gE[0] = 2.f * gE[0];
    for (int l = n - 1; l >= 1; --l)
    {
        const float w = (float)(6.283185307179586 / (double)l);
        // E_l = (i w) acc: acc_bar = E_bar_l (-i w)
        const C2 gacc = c2(gE[l].y * w, -gE[l].x * w);
        for (int j = 0; j < l; ++j)
        {
            const float sc = float(l - j) * xm[l - j];
            gE[j] = gE[j] + sc * gacc;
            gx[l - j] += float(l - j) * (gacc.x * E[j].x + gacc.y * E[j].y);
        }
    }
    // e_0 = (cos phi, sin phi) / (4 pi), phi = pi x_0 - pi / 2
    gx[0] += kPi * kInv4Pi * (-gE[0].x * sphi + gE[0].y * cphi);
    for (int i = 0; i < n; ++i)
        grad_moments[idx + i] = (1.f - bias) * gx[i];
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
            float sn, cs;
            sincosf(p_my - h, &sn, &cs);
            z = {cs, -sn};
        }
        // partial A, B of the four segments over this lane's moments
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
            float A = 0.f, B = 0.f;
#pragma unroll
            for (int i = 0; i < NJ; ++i)
            {
                // Re(z^j) = cos(j p), Im(z^j) = -sin(j p)
                A = fmaf(ca[i], w.x, A);
                B = fmaf(-cb[i], w.y, B);
                if (i + 1 < NJ)
                    w = cmul(w, v);
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
    const int bytes = kTfCopies * 256 * (int)sizeof(float4);
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
cudaError_t launch_prep_adj(int P, int m, const float *moments, float bias, const float *gl, float *gm,
                            cudaStream_t stream)
{
    prepare_adjoint_kernel<MAXM><<<(P + 63) / 64, 64, 0, stream>>>(P, m, moments, bias, gl, gm);
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
    a.error_flag = error_flag;
    if (r.m <= 8)
        return launch_recon_adj<8>(a, stream);
    if (r.m <= 16)
        return launch_recon_adj<16>(a, stream);
    if (r.m <= 32)
        return launch_recon_adj<32>(a, stream);
    return launch_recon_adj<64>(a, stream);
}

cudaError_t launch_prepare_adjoint(int num_pixels, int m, const float *moments, float bias, const float *grad_lambda,
                                   float *grad_moments, cudaStream_t stream)
{
    if (m <= 8)
        return launch_prep_adj<8>(num_pixels, m, moments, bias, grad_lambda, grad_moments, stream);
    if (m <= 16)
        return launch_prep_adj<16>(num_pixels, m, moments, bias, grad_lambda, grad_moments, stream);
    if (m <= 32)
        return launch_prep_adj<32>(num_pixels, m, moments, bias, grad_lambda, grad_moments, stream);
    return launch_prep_adj<64>(num_pixels, m, moments, bias, grad_lambda, grad_moments, stream);
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
