// The single-scattering transmittance cache: reconstruct_single_scattering_cache (src/moment_raymarcher.cpp:217-258)
// with reconstruct_single_scattering_ray (src/raymarch_single_scattering_cache.h:33-70) and ScatterGrid::scatter
// (src/scatter_grid.h:54-66).  Every pixel of a moment image rendered from the light re-marches its bounded-MESE
// density along its eye ray, accumulates the optical depth tau and writes exp(-tau) into the voxel of a regular
// grid (domain = the moment image's domain) that holds the sample position.  Voxels no sample reaches keep 0.
//
// Several samples land in one voxel, from one ray and from many.  The reference's writes race (an OpenMP loop
// over rows on the CPU, surface stores on the GPU); the result here is the one of a sequential run of its loop:
// the write of the last pixel in row-major order, and of that pixel's last sample in the voxel, wins.  Each
// voxel keeps a 64-bit key
//     (pixel + 1) << 32  |  (0xffffffff - bits(T))
// raised by atomicMax.  The pixel field orders the rays.  Within one ray T = exp(-tau) does not increase (the
// transfer function's extinction is not negative, so tau does not decrease), so its last write in a voxel is its
// smallest T, which has the largest low field.  A thread also keeps its current voxel and writes it only when
// the ray moves on: one atomic per voxel crossed instead of one per sample.
//
// One thread per light pixel in 16 x 8 tiles; the transfer-function row in shared memory.  Sample positions,
// phases and voxel indices are the reference's float operations, so every sample lands in the reference's voxel;
// T differs from the reference's by the rounding of the MESE density (as in the re-march) and of exp.

#include "device_common.cuh"
#include "internal.h"
#include "reconstruct_common.cuh"

namespace mraygb
{
namespace
{

struct CacheDev
{
    DeviceCamera cam;
    int width, height, m;
    float dmin[3], dmax[3], ext[3];
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const float4 *tf;
    float step;
    int cx, cy, cz;
    unsigned long long *keys;
    int *error_flag;
};

__device__ __forceinline__ void flush(unsigned long long *keys, long long voxel, unsigned long long pixkey, float T)
{
    if (voxel >= 0)
        atomicMax(keys + voxel, pixkey | (unsigned long long)(0xffffffffu - __float_as_uint(T)));
}

template <int MAXM> __global__ void __launch_bounds__(128) cache_march_kernel(const CacheDev a)
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
    if (n == 0)
        return; // empty pixels scatter nothing
    if (n > MAXM)
        n = MAXM;
    float lam2[MAXM];
    const float lam0 = a.pmoments[idx];
#pragma unroll
    for (int l = 0; l < MAXM; ++l)
        lam2[l] = (l < n && l > 0) ? 2.f * a.pmoments[idx + l] : 0.f;
    float lo = 0.f, hi = 1.f;
    if (a.bounds)
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
    if (!(hit && t_far > 0.f))
        return;
    const float range = __fsub_rn(t_far, t_near);
    float t = t_near;
    float p = (float)((double)__fdiv_rn(__fsub_rn(t, t_near), range) * 3.141592653589793 - 3.141592653589793);
    const float phase_step = (float)(3.141592653589793 * (double)__fdiv_rn(a.step, range));
    const float est = range / a.step;
    const int cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
    const unsigned long long pixkey = (unsigned long long)(pix + 1) << 32;
    const float fcx = (float)a.cx, fcy = (float)a.cy, fcz = (float)a.cz;

    float tau = 0.f;
    float fs = mese_density<MAXM>(lam2, lam0, p, lo, span);
    long long voxel = -1;
    float voxel_T = 0.f;
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
        const float bs = mese_density<MAXM>(lam2, lam0, p, lo, span);
        tau = __fadd_rn(tau, tf_sample(s_tf, fs, bs).w);
        fs = bs;
        const float T = expf(-tau);
        // ScatterGrid::scatter at ray.origin + t * ray.dir: the voxel int(((q - min) / (max - min)) * size)
        const int ix = (int)__fmul_rn(__fdiv_rn(__fsub_rn(__fadd_rn(o[0], __fmul_rn(t, d[0])), a.dmin[0]), a.ext[0]), fcx);
        const int iy = (int)__fmul_rn(__fdiv_rn(__fsub_rn(__fadd_rn(o[1], __fmul_rn(t, d[1])), a.dmin[1]), a.ext[1]), fcy);
        const int iz = (int)__fmul_rn(__fdiv_rn(__fsub_rn(__fadd_rn(o[2], __fmul_rn(t, d[2])), a.dmin[2]), a.ext[2]), fcz);
        if (ix >= 0 && ix < a.cx && iy >= 0 && iy < a.cy && iz >= 0 && iz < a.cz)
        {
            const long long v = ((long long)iz * a.cy + iy) * a.cx + ix;
            if (v != voxel)
            {
                flush(a.keys, voxel, pixkey, voxel_T);
                voxel = v;
            }
            voxel_T = T;
        }
    }
    flush(a.keys, voxel, pixkey, voxel_T);
}

__global__ void cache_decode_kernel(const unsigned long long *keys, size_t n, float *cache)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        const unsigned long long k = keys[i];
        cache[i] = k ? __uint_as_float(0xffffffffu - (unsigned)(k & 0xffffffffull)) : 0.f;
    }
}

template <int MAXM> void launch_m(const CacheDev &a, cudaStream_t stream)
{
    const dim3 block(16, 8), grid((a.width + 15) / 16, (a.height + 7) / 8);
    cache_march_kernel<MAXM><<<grid, block, 0, stream>>>(a);
}

} // namespace

cudaError_t launch_ss_cache(const SsCacheArgs &r, int *error_flag, cudaStream_t stream)
{
    const size_t nvox = (size_t)r.cx * r.cy * r.cz;
    cudaError_t e = cudaMemsetAsync(r.keys, 0, nvox * sizeof(unsigned long long), stream);
    if (e != cudaSuccess)
        return e;
    CacheDev a;
    a.cam = *r.cam;
    a.width = r.width;
    a.height = r.height;
    a.m = r.m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = r.dmin[i];
        a.dmax[i] = r.dmax[i];
        a.ext[i] = r.dmax[i] - r.dmin[i];
    }
    a.index = r.index;
    a.pmoments = r.pmoments;
    a.bounds = r.bounds;
    a.tf = r.tf;
    a.step = r.step;
    a.cx = r.cx;
    a.cy = r.cy;
    a.cz = r.cz;
    a.keys = r.keys;
    a.error_flag = error_flag;
    if (r.m <= 8)
        launch_m<8>(a, stream);
    else if (r.m <= 16)
        launch_m<16>(a, stream);
    else if (r.m <= 32)
        launch_m<32>(a, stream);
    else if (r.m <= 64)
        launch_m<64>(a, stream);
    else if (r.m <= 128)
        launch_m<128>(a, stream);
    else
        launch_m<256>(a, stream);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    const int threads = 256;
    const size_t want = (nvox + threads - 1) / threads;
    const int blocks = (int)(want < 152 * 8 ? want : 152 * 8);
    cache_decode_kernel<<<blocks, threads, 0, stream>>>(r.keys, nvox, r.cache);
    return cudaGetLastError();
}

} // namespace mraygb
