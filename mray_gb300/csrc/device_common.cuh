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

#include <cmath>
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
    cudaTextureObject_t tex; // the voxels in a 3D array: point sampling, unnormalized coordinates, clamp to edge
    int nx, ny, nz;
    float dmin[3];
    float ext[3]; // dmax - dmin, rounded as the reference rounds it
    float dmax[3];
    // where ext is a power of two, x / ext is x * (1 / ext) exactly (both are the correctly rounded x 2^-k)
    float inv_ext[3];
    int ext_pow2[3];
};

// exactly x / d: a multiply by the exact reciprocal where d is a power of two (`pow2` uniform across the launch)
__device__ __forceinline__ float div_exact(float x, float d, float inv, int pow2)
{
    return pow2 ? __fmul_rn(x, inv) : __fdiv_rn(x, d);
}

// host side: whether d is +-2^k with a normal reciprocal
inline bool is_pow2_divisor(float d)
{
    if (!(d != 0.f) || d != d || d - d != 0.f)
        return false;
    int e = 0;
    const float mant = std::frexp(d < 0.f ? -d : d, &e);
    return mant == 0.5f && e > -125 && e < 127;
}

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

// voxel (floor(x), floor(y), floor(z)) of the 3D texture, clamped to the grid (RegularGrid::get's clamp,
// src/volume.h:89-95): the coordinates passed are integer + 1/2
__device__ __forceinline__ float grid_get(const GridView &g, float x, float y, float z)
{
    return tex3D<float>(g.tex, x, y, z);
}

// The position of a sample in voxel units: the lower corner floor(ip) and the fractions ip - floor(ip), in the
// reference's float operations (RegularGrid::sample, src/volume.h:97-123).
struct GridPoint
{
    float fl[3], a[3];
};

__device__ __forceinline__ GridPoint grid_point(const GridView &g, float px, float py, float pz)
{
    const float p[3] = {px, py, pz};
    const int sz[3] = {g.nx, g.ny, g.nz};
    GridPoint q;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float np = div_exact(__fsub_rn(p[i], g.dmin[i]), g.ext[i], g.inv_ext[i], g.ext_pow2[i]);
        float ip = __fmul_rn(np, (float)sz[i]);
        q.fl[i] = floorf(ip);
        q.a[i] = __fsub_rn(ip, q.fl[i]);
    }
    return q;
}

// Corner-aligned trilinear blend with clamp-to-edge, summed in the reference's order.
__device__ __forceinline__ float grid_blend(const GridView &g, const GridPoint &q)
{
    // texel centres of the lower and upper corners (the clamp is the texture's address mode)
    const float xl = __fadd_rn(q.fl[0], 0.5f), yl = __fadd_rn(q.fl[1], 0.5f), zl = __fadd_rn(q.fl[2], 0.5f);
    const float xr = __fadd_rn(q.fl[0], 1.5f), yr = __fadd_rn(q.fl[1], 1.5f), zr = __fadd_rn(q.fl[2], 1.5f);
    const float lll = grid_get(g, xl, yl, zl);
    const float lrl = grid_get(g, xl, yr, zl);
    const float rrl = grid_get(g, xr, yr, zl);
    const float rll = grid_get(g, xr, yl, zl);
    const float llr = grid_get(g, xl, yl, zr);
    const float lrr = grid_get(g, xl, yr, zr);
    const float rrr = grid_get(g, xr, yr, zr);
    const float rlr = grid_get(g, xr, yl, zr);
    const float ax = q.a[0], ay = q.a[1], az = q.a[2];
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

__device__ __forceinline__ float grid_sample(const GridView &g, float px, float py, float pz)
{
    return grid_blend(g, grid_point(g, px, py, pz));
}

// ---- SPH particles ----------------------------------------------------------------------------------------
// The reference's uniform grid (src/particle_grid.cuh:284-306, createGridFromDomain :392-403): cell size = the
// smoothing length h, origin at the particles' minimum, sx and sy padded to multiples of 4 (sz too unless the
// grid is flat), cells in 4x4x4 tiles (4x4x1 when flat).
struct ParticleGridParams
{
    float gmin[3];
    float inv_cell; // (float)(1.0 / h)
    float r2;       // h * h
    float inv_h;    // 1.f / h
    int sx, sy, sz, tz;
    uint32_t total;
};

struct ParticleView
{
    ParticleGridParams g;
    const float4 *pts;          // (x, y, z, value) sorted by cell, input order inside a cell
    const uint32_t *cell_start; // CSR: the particles of cell c are [cell_start[c], cell_start[c + 1])
    float dmin[3], dmax[3];     // the ray box (Particles::domain)
};

// getIndexFromCell (src/particle_grid.cuh:64-83)
__host__ __device__ __forceinline__ uint32_t particle_cell_index(const ParticleGridParams &g, int cx, int cy, int cz)
{
    const int width_tiles = (g.sx + 3) / 4, height_tiles = (g.sy + 3) / 4;
    const int tile = (cz / g.tz) * height_tiles * width_tiles + (cy / 4) * width_tiles + cx / 4;
    return (uint32_t)(tile * (16 * g.tz) + (cz % g.tz) * 16 + (cy % 4) * 4 + cx % 4);
}

// the cell of a particle during the grid build (getCellIndex, clamped: the reference indexes past its grid when
// rounding lands a particle on the padded edge)
__device__ __forceinline__ uint32_t particle_cell(const ParticleGridParams &g, float x, float y, float z)
{
    const float p[3] = {x, y, z};
    const int s[3] = {g.sx, g.sy, g.sz};
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        c[k] = (int)__fmul_rn(__fsub_rn(p[k], g.gmin[k]), g.inv_cell);
        c[k] = c[k] < 0 ? 0 : (c[k] > s[k] - 1 ? s[k] - 1 : c[k]);
    }
    return particle_cell_index(g, c[0], c[1], c[2]);
}

// cubicSpline (src/cut/kernels.h:55-64)
__device__ __forceinline__ float cubic_spline(float x)
{
    constexpr float sigma = 0.5641895835477563f;
    if (x < 1.f)
        return __fmul_rn(sigma, __fsub_rn(1.f, __fmul_rn(__fmul_rn(__fmul_rn(1.5f, x), x),
                                                        __fsub_rn(1.f, __fmul_rn(x, 0.5f)))));
    if (x < 2.f)
    {
        const float u = __fsub_rn(2.f, x);
        return __fmul_rn(__fmul_rn(__fmul_rn(sigma / 4.f, u), u), u);
    }
    return 0.f;
}

// Particles::sample (src/volume.cpp:83-94): the 27 cells around p in z, y, x order (forEachNeighbor,
// src/particle_grid.cuh:156-211), weights W(|p - x_i| / h) for |p - x_i|^2 < h^2, normalised by their sum
// (InterpolateParticlesOp, src/particle_interpolate.h:35-58).  Cells come from the CSR array instead of the
// reference's EMPTY_CELL scan; the particles visited and their order are the same.
__device__ __forceinline__ float particle_sample(const ParticleView &v, float px, float py, float pz)
{
    const float p[3] = {px, py, pz};
    const int s[3] = {v.g.sx, v.g.sy, v.g.sz};
    int lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int c = (int)__fmul_rn(__fsub_rn(p[k], v.g.gmin[k]), v.g.inv_cell);
        c = c < -2 ? -2 : (c > s[k] + 1 ? s[k] + 1 : c); // no effect on the loop ranges below
        lo[k] = c - 1 > 0 ? c - 1 : 0;
        hi[k] = c + 2 < s[k] ? c + 2 : s[k];
    }
    float value = 0.f, wsum = 0.f;
    for (int z = lo[2]; z < hi[2]; ++z)
        for (int y = lo[1]; y < hi[1]; ++y)
            for (int x = lo[0]; x < hi[0]; ++x)
            {
                const uint32_t cell = particle_cell_index(v.g, x, y, z);
                const uint32_t b = __ldg(v.cell_start + cell), e = __ldg(v.cell_start + cell + 1);
                for (uint32_t i = b; i < e; ++i)
                {
                    const float4 q = __ldg(v.pts + i);
                    const float dx = __fsub_rn(px, q.x), dy = __fsub_rn(py, q.y), dz = __fsub_rn(pz, q.z);
                    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    if (d2 < v.g.r2)
                    {
                        const float w = cubic_spline(__fmul_rn(__fsqrt_rn(d2), v.g.inv_h));
                        wsum = __fadd_rn(wsum, w);
                        value = __fadd_rn(value, __fmul_rn(w, q.w));
                    }
                }
            }
    if (wsum != 0.f)
        value = __fdiv_rn(value, wsum);
    return value;
}

// SPH particles with a smoothing length per particle and the Wendland C2 kernel (this build's variant: the
// reference's particles carry one smoothing length and the cubic spline).  The grid is the reference's grid with
// the largest smoothing length as its cell size, so the 27 cells around a point hold every particle whose support
// (radius h_i, as the reference's radius test uses h) contains it.  Per record (1 / h_i, 1 / h_i^3).
struct ParticleHView : ParticleView
{
    const float2 *inv_h;
};

// W(q) h^3 up to the constant 21 / (2 pi), which the normalised sum cancels: (1 - q)^4 (1 + 4 q) for q < 1
__device__ __forceinline__ float wendland_c2(float q)
{
    const float u = __fsub_rn(1.f, q);
    const float u2 = __fmul_rn(u, u);
    return __fmul_rn(__fmul_rn(u2, u2), __fadd_rn(__fmul_rn(4.f, q), 1.f));
}

// sum_i W(|p - x_i|, h_i) v_i / sum_i W(|p - x_i|, h_i) over the 27 cells in z, y, x order and the cells' order
__device__ __forceinline__ float particle_sample_h(const ParticleHView &v, float px, float py, float pz)
{
    const float p[3] = {px, py, pz};
    const int s[3] = {v.g.sx, v.g.sy, v.g.sz};
    int lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int c = (int)__fmul_rn(__fsub_rn(p[k], v.g.gmin[k]), v.g.inv_cell);
        c = c < -2 ? -2 : (c > s[k] + 1 ? s[k] + 1 : c);
        lo[k] = c - 1 > 0 ? c - 1 : 0;
        hi[k] = c + 2 < s[k] ? c + 2 : s[k];
    }
    float value = 0.f, wsum = 0.f;
    for (int z = lo[2]; z < hi[2]; ++z)
        for (int y = lo[1]; y < hi[1]; ++y)
            for (int x = lo[0]; x < hi[0]; ++x)
            {
                const uint32_t cell = particle_cell_index(v.g, x, y, z);
                const uint32_t b = __ldg(v.cell_start + cell), e = __ldg(v.cell_start + cell + 1);
                for (uint32_t i = b; i < e; ++i)
                {
                    const float4 q = __ldg(v.pts + i);
                    const float dx = __fsub_rn(px, q.x), dy = __fsub_rn(py, q.y), dz = __fsub_rn(pz, q.z);
                    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    if (d2 < v.g.r2)
                    {
                        const float2 ih = __ldg(v.inv_h + i);
                        const float r = __fmul_rn(__fsqrt_rn(d2), ih.x);
                        if (r < 1.f)
                        {
                            const float w = __fmul_rn(wendland_c2(r), ih.y);
                            wsum = __fadd_rn(wsum, w);
                            value = __fadd_rn(value, __fmul_rn(w, q.w));
                        }
                    }
                }
            }
    if (wsum != 0.f)
        value = __fdiv_rn(value, wsum);
    return value;
}

// the two volumes behind one generate kernel: the ray box and one sample
__device__ __forceinline__ float volume_sample(const GridView &g, float x, float y, float z)
{
    return grid_sample(g, x, y, z);
}
__device__ __forceinline__ float volume_sample(const ParticleView &v, float x, float y, float z)
{
    return particle_sample(v, x, y, z);
}
__device__ __forceinline__ float volume_sample(const ParticleHView &v, float x, float y, float z)
{
    return particle_sample_h(v, x, y, z);
}

__device__ __forceinline__ float map_density(float s, float dmin, float dmax)
{
    return rclamp(__fdiv_rn(__fsub_rn(s, dmin), __fsub_rn(dmax, dmin)), 0.f, 1.f);
}

// map_density with the span dmax - dmin, its reciprocal and whether it is a power of two precomputed
__device__ __forceinline__ float map_density(float s, float dmin, float span, float inv_span, int span_pow2)
{
    return rclamp(div_exact(__fsub_rn(s, dmin), span, inv_span, span_pow2), 0.f, 1.f);
}

// Every float t of [0, t_far] plus step is exact when step is a multiple of the float spacing at t_far (the largest
// spacing a sample t < t_far has): the lowest set bit of step's significand at or above t_far's last place.
__device__ __forceinline__ bool exact_steps(float step, float t_far)
{
    const uint32_t sb = __float_as_uint(step), fb = __float_as_uint(t_far);
    const int es = (int)((sb >> 23) & 0xffu), ef = (int)((fb >> 23) & 0xffu);
    if (es == 0 || es == 0xff || ef == 0xff)
        return false; // subnormal, infinite or NaN step; infinite t_far
    const uint32_t sig = (sb & 0x7fffffu) | 0x800000u;
    return es + (__ffs(sig) - 1) >= ef;
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

// alpha_j(h) = sin(jh)/j and beta_j(h) = (sin(jh) - jh cos(jh)) / (j^2 h); beta by its series for small jh
__device__ __forceinline__ void seg_coeffs(int j, float h, float &alpha, float &beta)
{
    if (j == 0)
    {
        alpha = h;
        beta = 0.f;
        return;
    }
    const float x = (float)j * h;
    float s, c;
    sincosf(x, &s, &c);
    alpha = s / (float)j;
    float num;
    if (fabsf(x) < 0.5f)
    {
        // sin x - x cos x = x^3/3 - x^5/30 + x^7/840 - x^9/45360 + x^11/3991680 - ...
        const float x2 = x * x;
        float poly = 1.f / 3991680.f;
        poly = fmaf(poly, -x2, 1.f / 45360.f);
        poly = fmaf(poly, -x2, 1.f / 840.f);
        poly = fmaf(poly, -x2, 1.f / 30.f);
        poly = fmaf(poly, -x2, 1.f / 3.f);
        num = poly * x2 * x;
    }
    else
    {
        num = s - x * c;
    }
    beta = num / ((float)j * x);
}

// Kahan-compensated accumulation into (sum, comp) of a term y that already has the compensation taken off
// (y = v - comp, formed by the caller, e.g. as the first FMA of a partial sum)
__device__ __forceinline__ void kahan_add_corrected(float &sum, float &comp, float y)
{
    float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

} // namespace mraygb
