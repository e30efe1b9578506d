// Reference direct volume rendering: generate_reference (src/moment_raymarcher.cpp:45-80, GPU
// src/moment_raymarcher.cu:65-114) with reference_ray (src/raymarch_reference.h:93-160): the ground-truth image the
// moment path approximates, marched through the volume itself with the preintegrated transfer function.  With
// single scattering enabled every sample marches a secondary ray towards the light (the brute-force transmittance
// of raymarch_reference.h:40-75), or samples the transmittance cache of a light moment image
// (generate_reference_reconstructed_ss, src/moment_raymarcher.cpp:259-281); the Henyey-Greenstein phase function
// depends on the eye ray only and is evaluated once per ray.
//
// One thread per pixel in 16 x 8 tiles over the resident volume (grid texture or SPH particles); the transfer
// function row in shared memory, sampled as TransferFunction::sample does (src/transfer_function.h:44-59).  Sample
// positions, densities and the compositing order are the reference's; exp is CUDA's expf where the reference's
// CPU build rounds the double function.

#include "device_common.cuh"
#include "internal.h"
#include "reconstruct_common.cuh"

namespace mraygb
{
namespace
{

struct ReferenceDev
{
    DeviceCamera cam;
    int width, height;
    mraygb_reference_params rp;
    const float4 *tf;
    float *rgba;
    uint8_t *rgba8;
    int *error_flag;
    bool has_cache;
    GridView cache;
};

__device__ __forceinline__ int march_cap(float range, float step)
{
    const float est = range / step;
    return (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
}

// compute_transmittance with SingleScatteringBruteForce (src/raymarch_reference.h:40-75)
template <class V>
__device__ float transmittance(const V &vol, const float o[3], const float d[3], const float4 *s_tf,
                               const mraygb_reference_params &rp, int *error_flag)
{
    float t_near, t_far;
    const bool hit = intersect_aabb(o, d, vol.dmin, vol.dmax, t_near, t_far);
    if (!hit || t_far <= 0.0f || t_near >= t_far)
        return 0.0f;
    t_near = rmax(t_near, 0.0f);
    float t = t_near;
    float fs = map_density(volume_sample(vol, __fadd_rn(o[0], __fmul_rn(t, d[0])), __fadd_rn(o[1], __fmul_rn(t, d[1])),
                                         __fadd_rn(o[2], __fmul_rn(t, d[2]))),
                           rp.data_min, rp.data_max);
    const float ss_step = __fmul_rn(rp.step_size, rp.ss.step_size_factor);
    const int cap = march_cap(__fsub_rn(t_far, t_near), ss_step);
    float tau = 0.0f;
    int it = 0;
    while (t <= t_far)
    {
        if (++it > cap)
        {
            atomicExch(error_flag, 1);
            break;
        }
        t = __fadd_rn(t, ss_step);
        const float bs =
            map_density(volume_sample(vol, __fadd_rn(o[0], __fmul_rn(t, d[0])), __fadd_rn(o[1], __fmul_rn(t, d[1])),
                                      __fadd_rn(o[2], __fmul_rn(t, d[2]))),
                        rp.data_min, rp.data_max);
        tau = __fadd_rn(tau, tf_sample(s_tf, fs, bs).w);
        fs = bs;
    }
    return expf(-__fmul_rn(tau, rp.ss.step_size_factor));
}

// SS: 0 no single scattering, 1 brute-force transmittance, 2 the transmittance cache
template <class V, int SS> __global__ void __launch_bounds__(128) reference_kernel(const ReferenceDev a, const V vol)
{
    __shared__ float4 s_tf[256];
    for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y)
        s_tf[i] = a.tf[i];
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.width || y >= a.height)
        return;
    const mraygb_reference_params &rp = a.rp;
    float nx, ny, o[3], d[3];
    pixel_ndc(x, y, a.width, a.height, nx, ny);
    eye_ray(a.cam, nx, ny, o, d);
    float t_near, t_far;
    const bool hit = intersect_aabb(o, d, vol.dmin, vol.dmax, t_near, t_far);
    t_near = rmax(t_near, a.cam.znear);
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (hit && t_far > 0.f)
    {
        const float light[3] = {rp.ss.direction_x, rp.ss.direction_y, rp.ss.direction_z};
        const float to_light[3] = {-light[0], -light[1], -light[2]};
        const float pf = SS != 0 ? henyey_greenstein_ray(d, light, rp.ss.henyey_greenstein_g) : 0.f;
        const float step = rp.step_size;
        const int cap = march_cap(__fsub_rn(t_far, t_near), step);
        float L0 = 0.f, L1 = 0.f, L2 = 0.f, alpha = 0.f, T = 1.f, tau = 0.f;
        float t = t_near;
        float fs = map_density(volume_sample(vol, __fadd_rn(o[0], __fmul_rn(t, d[0])),
                                             __fadd_rn(o[1], __fmul_rn(t, d[1])), __fadd_rn(o[2], __fmul_rn(t, d[2]))),
                               rp.data_min, rp.data_max);
        int it = 0;
        while (t < t_far)
        {
            if (++it > cap)
            {
                atomicExch(a.error_flag, 1);
                break;
            }
            t = __fadd_rn(t, step);
            float p[3];
            p[0] = __fadd_rn(o[0], __fmul_rn(t, d[0]));
            p[1] = __fadd_rn(o[1], __fmul_rn(t, d[1]));
            p[2] = __fadd_rn(o[2], __fmul_rn(t, d[2]));
            const float sv = volume_sample(vol, p[0], p[1], p[2]);
            const float bs = map_density(sv, rp.data_min, rp.data_max);
            float4 s = tf_sample(s_tf, fs, bs);
            if (sv >= 1e10f) // an invalid sample
                s = make_float4(0.f, 1.f, 0.f, 0.05f);
            float ls0 = 0.f, ls1 = 0.f, ls2 = 0.f;
            const float sigma_s = rp.medium_scattering;
            if (SS != 0)
            {
                // compute_transmittance: the brute-force march, or the cache sampled at the sample position
                // (raymarch_reference.h:77-86)
                const float T_ss = SS == 1 ? transmittance(vol, p, to_light, s_tf, rp, a.error_flag)
                                           : grid_sample(a.cache, p[0], p[1], p[2]);
                const float tp = __fmul_rn(T_ss, pf);
                ls0 = __fmul_rn(tp, rp.ss.intensity_r);
                ls1 = __fmul_rn(tp, rp.ss.intensity_g);
                ls2 = __fmul_rn(tp, rp.ss.intensity_b);
            }
            L0 = __fadd_rn(L0, __fmul_rn(__fadd_rn(__fmul_rn(rp.medium_emission, s.x), __fmul_rn(ls0, sigma_s)), T));
            L1 = __fadd_rn(L1, __fmul_rn(__fadd_rn(__fmul_rn(rp.medium_emission, s.y), __fmul_rn(ls1, sigma_s)), T));
            L2 = __fadd_rn(L2, __fmul_rn(__fadd_rn(__fmul_rn(rp.medium_emission, s.z), __fmul_rn(ls2, sigma_s)), T));
            tau = __fadd_rn(tau, s.w);
            T = expf(-tau);
            alpha = __fsub_rn(1.f, T);
            fs = bs;
            if (alpha >= rp.early_ray_termination)
            {
                alpha = 1.f;
                break;
            }
        }
        out = make_float4(L0, L1, L2, alpha);
    }
    if (a.rgba)
        reinterpret_cast<float4 *>(a.rgba)[(size_t)y * a.width + x] = out;
    if (a.rgba8)
    {
        // ColorImageHost::rgba8_t (src/color_image.h:41-47) after clamp to [0, 1]
        uchar4 c;
        c.x = (unsigned char)(rclamp(out.x, 0.f, 1.f) * 255.f);
        c.y = (unsigned char)(rclamp(out.y, 0.f, 1.f) * 255.f);
        c.z = (unsigned char)(rclamp(out.z, 0.f, 1.f) * 255.f);
        c.w = (unsigned char)(rclamp(out.w, 0.f, 1.f) * 255.f);
        reinterpret_cast<uchar4 *>(a.rgba8)[(size_t)y * a.width + x] = c;
    }
}

template <class V> cudaError_t launch_reference_v(const ReferenceDev &a, const V &vol, cudaStream_t stream)
{
    const dim3 block(16, 8), grid((a.width + 15) / 16, (a.height + 7) / 8);
    const bool ss = a.rp.ss.enable && a.rp.medium_scattering > 0.0f;
    if (ss && a.has_cache)
        reference_kernel<V, 2><<<grid, block, 0, stream>>>(a, vol);
    else if (ss)
        reference_kernel<V, 1><<<grid, block, 0, stream>>>(a, vol);
    else
        reference_kernel<V, 0><<<grid, block, 0, stream>>>(a, vol);
    return cudaGetLastError();
}

ReferenceDev reference_args(const ReferenceArgs &r, int *error_flag)
{
    ReferenceDev a;
    a.cam = *r.cam;
    a.width = r.width;
    a.height = r.height;
    a.rp = *r.rp;
    a.tf = r.tf;
    a.rgba = r.rgba;
    a.rgba8 = r.rgba8;
    a.error_flag = error_flag;
    a.has_cache = r.ss_cache != nullptr;
    a.cache = r.ss_cache ? *r.ss_cache : GridView{};
    return a;
}

} // namespace

cudaError_t launch_reference_grid(const GridView &grid, const ReferenceArgs &r, int *error_flag, cudaStream_t stream)
{
    return launch_reference_v(reference_args(r, error_flag), grid, stream);
}

cudaError_t launch_reference_particles(const ParticleView &parts, const ReferenceArgs &r, int *error_flag,
                                       cudaStream_t stream)
{
    return launch_reference_v(reference_args(r, error_flag), parts, stream);
}

} // namespace mraygb
