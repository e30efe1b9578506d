// Device-side building blocks shared by the kernels: camera rays, ray/box test, corner-aligned trilinear
// grid sampling, density mapping and small complex helpers.
//
// The ray set-up and the volume sample reproduce the reference's float operations one by one (explicit
// round-to-nearest intrinsics, no contraction), so that the sample positions and sampled densities - and
// with them the u16 density bounds and the compaction decisions - are the reference's own:
//   get_eye_ray / _ortho / _persp  src/cut/raytracing.h:39-65
//   intersect_AABB                 src/cut/raytracing.h:67-86
//   RegularGrid::get / sample      src/volume.h:89-123
//   map_density                    src/parameters.h:31-34
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mraygb_types.h"

namespace mraygb
{

constexpr float kPiF = 3.14159274101257324f;        // float(M_PI)
constexpr float kPiLoF = -8.74227765734758577e-08f;  // M_PI - float(M_PI)
constexpr float kMInvPi = 0.3183098861837907f;       // M_INV_PI, src/raymarch_generate.h:30

struct DeviceCamera
{
    float m[4][4];
    float pos[3], right[3], up[3], dir[3];
    float scale, aspect, znear;
    int orthographic;
};

inline DeviceCamera to_device_camera(const mraygb_camera &c)
{
    DeviceCamera d;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            d.m[i][j] = c.transform[i][j];
    for (int i = 0; i < 3; ++i)
    {
        d.pos[i] = c.position[i];
        d.right[i] = c.right[i];
        d.up[i] = c.up[i];
        d.dir[i] = c.dir[i];
    }
    d.scale = c.scale;
    d.aspect = c.aspect;
    d.znear = c.znear;
    d.orthographic = c.orthographic;
    return d;
}

struct GridView
{
    const float *data;
    int nx, ny, nz;
    float dmin[3];
    float ext[3]; // dmax - dmin, rounded as the reference rounds it
    float dmax[3];
};

// cut::min / cut::max (src/cut/cuda_math.h:77-85): ternaries, so NaN handling matches the reference
__device__ __forceinline__ float rmin(float a, float b) { return (a < b) ? a : b; }
__device__ __forceinline__ float rmax(float a, float b) { return (a > b) ? a : b; }
__device__ __forceinline__ float rclamp(float v, float lo, float hi) { return rmin(rmax(v, lo), hi); }

// ndc of pixel (x, y): x / W * 2 - 1 (src/moment_raymarcher.cpp:133, no half-pixel offset)
__device__ __forceinline__ void pixel_ndc(int x, int y, int w, int h, float &nx, float &ny)
{
    nx = __fsub_rn(__fmul_rn(__fdiv_rn((float)x, (float)w), 2.f), 1.f);
    ny = __fsub_rn(__fmul_rn(__fdiv_rn((float)y, (float)h), 2.f), 1.f);
}

__device__ __forceinline__ void eye_ray(const DeviceCamera &c, float ndcx, float ndcy, float o[3], float d[3])
{
    if (c.orthographic)
    {
#pragma unroll
        for (int i = 0; i < 3; ++i)
        {
            o[i] = __fadd_rn(__fadd_rn(c.pos[i], __fmul_rn(ndcx, c.right[i])), __fmul_rn(ndcy, c.up[i]));
            d[i] = c.dir[i];
        }
    }
    else
    {
        float x = __fmul_rn(__fmul_rn(ndcx, c.aspect), c.scale);
        float y = __fmul_rn(ndcy, c.scale);
        float v[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
        {
            o[i] = c.pos[i];
            v[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.m[i][0], x), __fmul_rn(c.m[i][1], y)),
                                       __fmul_rn(c.m[i][2], -1.0f)),
                             __fmul_rn(c.m[i][3], 0.0f));
        }
        float len2 = __fadd_rn(__fadd_rn(__fmul_rn(v[0], v[0]), __fmul_rn(v[1], v[1])), __fmul_rn(v[2], v[2]));
        float inv = __fdiv_rn(1.0f, __fsqrt_rn(len2));
#pragma unroll
        for (int i = 0; i < 3; ++i)
            d[i] = __fmul_rn(v[i], inv);
    }
}

// slab test; returns hit and writes t_near / t_far
__device__ __forceinline__ bool intersect_aabb(const float o[3], const float d[3], const float bmin[3],
                                               const float bmax[3], float &tn, float &tf)
{
    float tmin[3], tmax[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float inv = __fdiv_rn(1.0f, d[i]);
        float tbot = __fmul_rn(inv, __fsub_rn(bmin[i], o[i]));
        float ttop = __fmul_rn(inv, __fsub_rn(bmax[i], o[i]));
        tmin[i] = rmin(ttop, tbot);
        tmax[i] = rmax(ttop, tbot);
    }
    float largest_tmin = rmax(rmax(tmin[0], tmin[1]), rmax(tmin[0], tmin[2]));
    float smallest_tmax = rmin(rmin(tmax[0], tmax[1]), rmin(tmax[0], tmax[2]));
    tn = largest_tmin;
    tf = smallest_tmax;
    return smallest_tmax > largest_tmin;
}

__device__ __forceinline__ float grid_get(const GridView &g, int x, int y, int z)
{
    x = x < 0 ? 0 : (x > g.nx - 1 ? g.nx - 1 : x);
    y = y < 0 ? 0 : (y > g.ny - 1 ? g.ny - 1 : y);
    z = z < 0 ? 0 : (z > g.nz - 1 ? g.nz - 1 : z);
    return __ldg(g.data + ((size_t)z * (size_t)(g.ny * g.nx) + (size_t)(y * g.nx) + (size_t)x));
}

// Corner-aligned trilinear sample with clamp-to-edge, summed in the reference's order.
__device__ __forceinline__ float grid_sample(const GridView &g, float px, float py, float pz)
{
    const float p[3] = {px, py, pz};
    const int sz[3] = {g.nx, g.ny, g.nz};
    float a[3];
    int il[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float np = __fdiv_rn(__fsub_rn(p[i], g.dmin[i]), g.ext[i]);
        float ip = __fmul_rn(np, (float)sz[i]);
        float fl = floorf(ip);
        a[i] = __fsub_rn(ip, fl);
        il[i] = (int)fl;
    }
    const int xl = il[0], yl = il[1], zl = il[2];
    const float lll = grid_get(g, xl, yl, zl);
    const float lrl = grid_get(g, xl, yl + 1, zl);
    const float rrl = grid_get(g, xl + 1, yl + 1, zl);
    const float rll = grid_get(g, xl + 1, yl, zl);
    const float llr = grid_get(g, xl, yl, zl + 1);
    const float lrr = grid_get(g, xl, yl + 1, zl + 1);
    const float rrr = grid_get(g, xl + 1, yl + 1, zl + 1);
    const float rlr = grid_get(g, xl + 1, yl, zl + 1);
    const float ax = a[0], ay = a[1], az = a[2];
    const float bx = __fsub_rn(1.f, ax), by = __fsub_rn(1.f, ay), bz = __fsub_rn(1.f, az);
    float s = __fmul_rn(__fmul_rn(__fmul_rn(bx, by), bz), lll);
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(ax, by), bz), rll));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(bx, ay), bz), lrl));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(ax, ay), bz), rrl));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(bx, by), az), llr));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(ax, by), az), rlr));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(bx, ay), az), lrr));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(__fmul_rn(ax, ay), az), rrr));
    return s;
}

__device__ __forceinline__ float map_density(float s, float dmin, float dmax)
{
    return rclamp(__fdiv_rn(__fsub_rn(s, dmin), __fsub_rn(dmax, dmin)), 0.f, 1.f);
}

// float((double)x - M_PI) without double arithmetic: x - pi with pi split into two floats (exact two-sum of
// x and -pi_hi, then the low part), the same value the reference's double expression rounds to.
__device__ __forceinline__ float sub_pi(float x)
{
    float s = __fadd_rn(x, -kPiF);
    float bp = __fsub_rn(s, x);
    float err = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bp)), __fsub_rn(-kPiF, bp));
    return __fadd_rn(s, __fsub_rn(err, kPiLoF));
}

// ---- complex helpers ------------------------------------------------------------------------------------
struct cf
{
    float x, y;
};
__device__ __forceinline__ cf cmul(cf a, cf b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cf csq(cf a) { return {a.x * a.x - a.y * a.y, 2.f * a.x * a.y}; }

// Kahan-compensated accumulation of `v` into (sum, comp)
__device__ __forceinline__ void kahan_add(float &sum, float &comp, float v)
{
    float y = __fsub_rn(v, comp);
    float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

} // namespace mraygb
