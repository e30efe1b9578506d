// Bounded-MESE re-march: one thread per pixel (reconstruct_ray with MESEReconstruction, without single
// scattering or with the transmittance cache, src/raymarch_reconstruct.h:127-200 and src/reconstruction_techniques.h:72-96; driven per pixel
// as reconstruct_host / reconstruct_moments_kernel, src/moment_raymarcher.cpp:283-327, .cu:339-384).
//
// Per sample the density is rho(p) = lo + (hi - lo) (fast_atan(S(p)) / pi + 1/2) with the Lagrange series
// S(p) = l_0 + 2 sum_{l>=1} l_l cos(l p) (evaluateMESELagrange, src/mese/MESE_dynamic.h:242-250).  The series is
// summed by Reinsch's modification of Clenshaw's recurrence (three operations per term, multipliers held in
// registers) instead of the reference's complex power recurrence (five per term).  Plain Clenshaw loses
// accuracy as p approaches 0 or -pi - the two ends of every ray - and the multipliers of high-order moment
// sets are large and cancel, so the modified form is used: measured on 64-moment mixing-layer images it
// leaves fewer than half as many pixels off by more than 1e-3 in density as the reference's own FP32
// evaluation does.
//
// The transfer-function row lives in shared memory and is sampled exactly as TransferFunction::sample does on
// a table whose rows are all equal (src/transfer_function.h:44-59): the column comes from floor(256 fs), the
// blend weight from frac(256 bs).

#include "device_common.cuh"
#include "internal.h"
#include "reconstruct_common.cuh"

namespace mraygb
{

namespace
{

struct ReconDev
{
    DeviceCamera cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const float4 *tf;
    float step, emission, ert;
    float *rgba;
    uint8_t *rgba8;
    const float4 *bounds4;
    int diff_tf_linear;
    int *error_flag;
    // single scattering: the transmittance cache, the light direction, intensity, phase asymmetry and the medium's
    // scattering coefficient
    GridView cache;
    float light[3], intensity[3], hg_g, scattering;
};

// DIFF: the differentiation form (float bounds read by the caller's choice, exact atan, the transfer-function row
// as a cubic B-spline or, with a.diff_tf_linear, linear in the front density)
// SS: in-scattered light from the transmittance cache (inscattering with SingleScatteringCache,
// src/raymarch_reconstruct.h:36-46 and 112-125)
template <int MAXM, bool DIFF, bool SS>
__global__ void __launch_bounds__(128) reconstruct_kernel(const ReconDev a)
{
    __shared__ float4 s_tf[256];
    for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y)
        s_tf[i] = a.tf[i];
    __syncthreads();

    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.width || y >= a.height)
        return;
    const size_t pix = (size_t)y * (size_t)a.width + (size_t)x;
    size_t idx;
    int n;
    if (a.index)
    {
        idx = a.index[pix];
        n = (int)(a.index[pix + 1] - a.index[pix]);
    }
    else
    {
        idx = pix * (size_t)a.m;
        n = a.m;
    }

    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (n == 0)
    {
        // reconstruct_zero_ray (src/raymarch_reconstruct.h:127-131)
        const float4 z = DIFF ? tf_sample_bspline(s_tf, diff_tf_tap(0.f, a.diff_tf_linear)) : tf_sample(s_tf, 0.f, 0.f);
        out = make_float4(z.x, z.y, z.z, 0.f);
    }
    else
    {
        if (n > MAXM)
            n = MAXM;
        float lam2[MAXM];
        const float lam0 = a.pmoments[idx];
#pragma unroll
        for (int l = 0; l < MAXM; ++l)
            lam2[l] = (l < n && l > 0) ? 2.f * a.pmoments[idx + l] : 0.f;
        float lo = 0.f, hi = 1.f;
        if (a.bounds4)
        {
            const float4 b4 = a.bounds4[pix];
            lo = b4.x;
            hi = b4.y;
        }
        else if (a.bounds)
        {
            lo = a.bounds[2 * pix] / 65535.f;
            hi = a.bounds[2 * pix + 1] / 65535.f;
        }
        const float span = hi - lo;

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
            // the march ends by itself after about range / step samples; the cap only guards a step that is too
            // small to advance t in float
            const float est = range / a.step;
            const int cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
            float L0 = 0.f, L1 = 0.f, L2 = 0.f, alpha = 0.f, T = 1.f, tau = 0.f;
            const float pf = SS ? henyey_greenstein_ray(d, a.light, a.hg_g) : 0.f;
            float fs = DIFF ? mese_density_exact<MAXM>(lam2, lam0, p, lo, span)
                            : mese_density<MAXM>(lam2, lam0, p, lo, span);
            int it = 0;
            while (t <= t_far)
            {
                if (++it > cap)
                {
                    atomicExch(a.error_flag, 1);
                    break;
                }
                t = __fadd_rn(t, a.step);
                p = __fadd_rn(p, phase_step);
                const float bs = DIFF ? mese_density_exact<MAXM>(lam2, lam0, p, lo, span)
                                      : mese_density<MAXM>(lam2, lam0, p, lo, span);
                const float4 s = DIFF ? tf_sample_bspline(s_tf, diff_tf_tap(fs, a.diff_tf_linear)) : tf_sample(s_tf, fs, bs);
                if (SS)
                {
                    // L += (Le + Ls sigma_s) T with Ls = T_ss pf intensity, T_ss the cache at ray.origin + t ray.dir
                    const float T_ss = grid_sample(a.cache, __fadd_rn(o[0], __fmul_rn(t, d[0])),
                                                   __fadd_rn(o[1], __fmul_rn(t, d[1])),
                                                   __fadd_rn(o[2], __fmul_rn(t, d[2])));
                    const float tp = __fmul_rn(T_ss, pf);
                    L0 = __fadd_rn(L0, __fmul_rn(__fadd_rn(__fmul_rn(a.emission, s.x),
                                                           __fmul_rn(__fmul_rn(tp, a.intensity[0]), a.scattering)),
                                                 T));
                    L1 = __fadd_rn(L1, __fmul_rn(__fadd_rn(__fmul_rn(a.emission, s.y),
                                                           __fmul_rn(__fmul_rn(tp, a.intensity[1]), a.scattering)),
                                                 T));
                    L2 = __fadd_rn(L2, __fmul_rn(__fadd_rn(__fmul_rn(a.emission, s.z),
                                                           __fmul_rn(__fmul_rn(tp, a.intensity[2]), a.scattering)),
                                                 T));
                }
                else
                {
                    L0 += (a.emission * s.x) * T;
                    L1 += (a.emission * s.y) * T;
                    L2 += (a.emission * s.z) * T;
                }
                tau += s.w;
                T = expf(-tau);
                alpha = 1.f - T;
                fs = bs;
                if (alpha >= a.ert)
                {
                    alpha = 1.f;
                    break;
                }
            }
            out = make_float4(L0, L1, L2, alpha);
        }
    }
    if (a.rgba)
        reinterpret_cast<float4 *>(a.rgba)[pix] = out;
    if (a.rgba8)
    {
        // ColorImageHost::rgba8_t (src/color_image.h:41-47) after clamp to [0, 1]
        uchar4 c;
        c.x = (unsigned char)(rclamp(out.x, 0.f, 1.f) * 255.f);
        c.y = (unsigned char)(rclamp(out.y, 0.f, 1.f) * 255.f);
        c.z = (unsigned char)(rclamp(out.z, 0.f, 1.f) * 255.f);
        c.w = (unsigned char)(rclamp(out.w, 0.f, 1.f) * 255.f);
        reinterpret_cast<uchar4 *>(a.rgba8)[pix] = c;
    }
}

template <int MAXM> void launch_m(const ReconDev &a, bool diff, bool ss, cudaStream_t stream)
{
    dim3 block(16, 8);
    dim3 grid((a.width + 15) / 16, (a.height + 7) / 8);
    if (diff)
        reconstruct_kernel<MAXM, true, false><<<grid, block, 0, stream>>>(a);
    else if (ss)
        reconstruct_kernel<MAXM, false, true><<<grid, block, 0, stream>>>(a);
    else
        reconstruct_kernel<MAXM, false, false><<<grid, block, 0, stream>>>(a);
}

} // namespace

cudaError_t launch_reconstruct(const ReconArgs &r, int *error_flag, cudaStream_t stream)
{
    ReconDev a;
    a.cam = *r.cam;
    a.width = r.width;
    a.height = r.height;
    a.m = r.m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = r.dmin[i];
        a.dmax[i] = r.dmax[i];
    }
    a.index = r.index;
    a.pmoments = r.pmoments;
    a.bounds = r.bounds;
    a.tf = r.tf;
    a.step = r.step;
    a.emission = r.emission;
    a.ert = r.ert;
    a.rgba = r.rgba;
    a.rgba8 = r.rgba8;
    a.bounds4 = r.bounds4;
    a.diff_tf_linear = r.diff_tf_linear;
    a.error_flag = error_flag;
    // inscattering only where the medium scatters (raymarch_reconstruct.h:176-179)
    const bool ss = r.ss_cache && r.ss && r.scattering > 0.0f && r.diff_form == 0;
    a.cache = ss ? *r.ss_cache : GridView{};
    a.scattering = r.scattering;
    a.light[0] = ss ? r.ss->direction_x : 0.f;
    a.light[1] = ss ? r.ss->direction_y : 0.f;
    a.light[2] = ss ? r.ss->direction_z : 0.f;
    a.intensity[0] = ss ? r.ss->intensity_r : 0.f;
    a.intensity[1] = ss ? r.ss->intensity_g : 0.f;
    a.intensity[2] = ss ? r.ss->intensity_b : 0.f;
    a.hg_g = ss ? r.ss->henyey_greenstein_g : 0.f;
    const bool lin = r.diff_form != 0;
    if (r.m <= 8)
        launch_m<8>(a, lin, ss, stream);
    else if (r.m <= 16)
        launch_m<16>(a, lin, ss, stream);
    else if (r.m <= 32)
        launch_m<32>(a, lin, ss, stream);
    else if (r.m <= 64)
        launch_m<64>(a, lin, ss, stream);
    else if (r.m <= 128)
        launch_m<128>(a, lin, ss, stream);
    else
        launch_m<256>(a, lin, ss, stream);
    return cudaGetLastError();
}

} // namespace mraygb
