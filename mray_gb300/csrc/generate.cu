// Moment generation over a regular grid or SPH particles: one ray per 4-lane quad, moments split across the
// quad's lanes.  The two volumes share the kernel body (generate_quads); they differ only in the sample
// (corner-aligned trilinear grid sample, or the SPH sum over the 27 neighbour cells) and the ray box.
//
// Method (src/raymarch_generate.h:35-148).  A ray is marched from t_near in steps of `step` while
// t + step < t_far (t accumulated in float exactly as the reference does), with one last sample at t_far.
// Between consecutive samples the density is linear in the phase p in [-pi, 0], and the reference adds the
// closed-form integral of that linear piece times e^{-ijp} to moment j (update_moments).  Over a segment
// [p_m - h, p_m + h] with end values f0, f1 that integral is, exactly,
//
//     (f0 + f1) * alpha_j(h) * cos(j p_m)  -  (f1 - f0) * beta_j(h) * sin(j p_m)
//     alpha_j(h) = sin(j h) / j,   beta_j(h) = (sin(j h) - j h cos(j h)) / (j^2 h)   (alpha_0 = h, beta_0 = 0)
//
// All regular segments share h = phase_step / 2, so a ray needs only the two sums
//     C_j = sum_k (f_{k-1} + f_k) Re(z_k^j),   D_j = sum_k (f_k - f_{k-1}) Im(z_k^j),   z_k = e^{-i p_m,k}
// and m_j = alpha_j C_j + beta_j D_j + (last segment, computed directly).  This is the reference's integral
// regrouped; it avoids the reference's difference of two O(S/j^2) terms per step and needs one sincos per
// segment instead of 2(m-1).
//
// Layout: a warp holds 8 rays (quads).  Per round the 4 lanes of a quad each march one sample (the four
// consecutive t values are computed by every lane with the reference's sequential float adds), exchange
// (f_{k-1}+f_k, f_k-f_{k-1}, z_k) with shuffles, and each lane accumulates the moments j = q + 4i it owns:
// z_k^j by the three-term recurrence in j (steps of four) from z_k^q and z_k^(q+4), so no moment is more than
// 15 steps from a fresh sincos (largest error of the trigonometric values 6e-5, where sin(4 p_m) is near 0).
//
// Two arithmetic forms: plain FP32 sums, or per-round partial sums of C added with Kahan compensation
// (MRAYGB_PRECISION_COMPENSATED_FP64_MESE; the partial starts from minus the compensation, which saves Kahan's
// separate correction step).

#include "device_common.cuh"
#include "internal.h"

namespace mraygb
{

namespace
{

constexpr unsigned kFull = 0xffffffffu;

template <class V> struct GenArgs
{
    V vol; // GridView or ParticleView
    DeviceCamera cam;
    int width, height, m;
    float step;
    float data_min, data_max;
    float data_span, data_inv_span; // data_max - data_min and its reciprocal
    int data_span_pow2;             // the span is a power of two: the mapping's division is a multiply
    float bound_eps;
    int transform_to_bounds;
    int compact_image;
    int error_threshold_zero;
    float *moments;
    uint16_t *bounds;
    uint32_t *counts;
    float4 *bounds4; // the differentiation form: (lo, hi, min, max) of the samples, unquantized, or NULL
    int *error_flag;
};

template <class V, int NJ, bool KAHAN> __device__ __forceinline__ void generate_quads(const GenArgs<V> &a)
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
    if (in_image)
    {
        float nx, ny;
        pixel_ndc(px, py, a.width, a.height, nx, ny);
        eye_ray(a.cam, nx, ny, o, d);
        const float bmin[3] = {a.vol.dmin[0], a.vol.dmin[1], a.vol.dmin[2]};
        const float bmax[3] = {a.vol.dmax[0], a.vol.dmax[1], a.vol.dmax[2]};
        hit = intersect_aabb(o, d, bmin, bmax, t_near, t_far);
        t_near = rmax(t_near, a.cam.znear);
        hit = hit && (t_far > 0.f);
    }

    float C[NJ], Dc[NJ], Ck[NJ];
#pragma unroll
    for (int i = 0; i < NJ; ++i)
    {
        C[i] = 0.f;
        Dc[i] = 0.f;
        Ck[i] = 0.f;
    }

    float blo = 1.f, bhi = 0.f;
    float pti = 0.f, pss = 0.f;
    float f_tail = 0.f;
    // The sums run over the density minus a baseline c, and c's share is added back in closed form: over the phase
    // interval [-pi, 0] a constant contributes exactly c to the zeroth moment and nothing to the others.  The sums
    // then scale with the ray's density range instead of its level, and so do their rounding errors, which the
    // bounds transform divides by that range.  The closed form holds only where the segments [p - pss, p] tile
    // [-pi, 0], i.e. where every t += step is exact: step a multiple of the float spacing at t_far.  Elsewhere (a
    // step such as 1/192) t drifts by a constant amount per step, a constant density covers slightly more or less
    // than pi, and the ray runs with c = 0.  c is the midrange of the first sample and 16 coarse samples spread
    // over the ray (four per lane of the quad); it only chooses the split, not the integrals.
    float base = 0.f;
    float p_tail = -kPiF;
    float t = t_near;
    const float step = a.step;
    if (hit)
    {
        pti = (float)(3.141592653589793 / (double)__fsub_rn(t_far, t_near));
        pss = (float)(3.141592653589793 * (double)__fdiv_rn(step, __fsub_rn(t_far, t_near)));
        const float f0 = map_density(volume_sample(a.vol, __fadd_rn(o[0], __fmul_rn(t, d[0])),
                                                 __fadd_rn(o[1], __fmul_rn(t, d[1])),
                                                 __fadd_rn(o[2], __fmul_rn(t, d[2]))),
                                     a.data_min, a.data_span, a.data_inv_span, a.data_span_pow2);
        blo = rmin(blo, f0);
        bhi = rmax(bhi, f0);
        f_tail = f0;
        if (exact_steps(step, t_far))
        {
            float cmin = f0, cmax = f0;
            const float len = __fsub_rn(t_far, t_near);
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                const float tc = t_near + len * ((float)(4 * i + q) + 0.5f) * (1.f / 16.f);
                const float fc = map_density(volume_sample(a.vol, o[0] + tc * d[0], o[1] + tc * d[1], o[2] + tc * d[2]),
                                             a.data_min, a.data_span, a.data_inv_span, a.data_span_pow2);
                cmin = rmin(cmin, fc);
                cmax = rmax(cmax, fc);
            }
            cmin = rmin(cmin, __shfl_xor_sync(0xfu << qbase, cmin, 1));
            cmax = rmax(cmax, __shfl_xor_sync(0xfu << qbase, cmax, 1));
            cmin = rmin(cmin, __shfl_xor_sync(0xfu << qbase, cmin, 2));
            cmax = rmax(cmax, __shfl_xor_sync(0xfu << qbase, cmax, 2));
            base = 0.5f * (cmin + cmax);
        }
    }
    const float half_pss = 0.5f * pss;
    // A ray ends by itself after about (t_far - t_near) / step samples; the cap only guards a step too small to
    // advance t in float (the reference would loop forever there).
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
        // the next four t values, each taken only while t + step < t_far (raymarch_generate.h:90-95)
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
        float f_my = 0.f, p_my = 0.f;
        if (my_valid)
        {
            p_my = sub_pi(__fmul_rn(__fsub_rn(my_t, t_near), pti));
            f_my = map_density(volume_sample(a.vol, __fadd_rn(o[0], __fmul_rn(my_t, d[0])),
                                           __fadd_rn(o[1], __fmul_rn(my_t, d[1])),
                                           __fadd_rn(o[2], __fmul_rn(my_t, d[2]))),
                               a.data_min, a.data_span, a.data_inv_span, a.data_span_pow2);
            blo = rmin(blo, f_my);
            bhi = rmax(bhi, f_my);
        }
        float f_left = __shfl_up_sync(kFull, f_my, 1);
        if (q == 0)
            f_left = f_tail;
        float S = 0.f, D = 0.f;
        cf z = {1.f, 0.f};
        if (my_valid)
        {
            S = __fsub_rn(f_left, base) + __fsub_rn(f_my, base);
            D = f_my - f_left;
            float sn, cs;
            sincosf(p_my - half_pss, &sn, &cs);
            z = {cs, -sn};
        }

        // Per sample s the lane needs z_s^j for its moments j = q + 4i.  Both parts of z^j satisfy the three-term
        // recurrence x_{j+4} = 2 cos(4 theta) x_j - x_{j-4} (Chebyshev in steps of four), one FMA per part and
        // moment instead of a complex rotation's four operations; the recurrence starts from z^q and z^(q+4).
        float Ss[4], Ds[4], c4[4];
        cf wa[4], wb[4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            Ss[s] = __shfl_sync(kFull, S, qbase + s);
            Ds[s] = __shfl_sync(kFull, D, qbase + s);
            cf zs;
            zs.x = __shfl_sync(kFull, z.x, qbase + s);
            zs.y = __shfl_sync(kFull, z.y, qbase + s);
            const cf z2 = csq(zs);
            const cf z3 = cmul(z2, zs);
            const cf z4 = csq(z2);
            cf u = {1.f, 0.f};
            u = (q == 1) ? zs : u;
            u = (q == 2) ? z2 : u;
            u = (q == 3) ? z3 : u;
            wa[s] = u;
            wb[s] = cmul(u, z4);
            c4[s] = 2.f * z4.x;
        }

#pragma unroll
        for (int i = 0; i < NJ; ++i)
        {
            if (KAHAN)
            {
                // the partial sum starts from minus the compensation, so it is already Kahan's corrected term.
                // Only C is compensated: D enters moment j through beta_j(h) ~ j h^2 / 3, at most a few percent of
                // alpha_j(h) ~ h, so its rounding is that much smaller in the moment.
                float pc = fmaf(Ss[0], wa[0].x, -Ck[i]);
#pragma unroll
                for (int s = 1; s < 4; ++s)
                    pc = fmaf(Ss[s], wa[s].x, pc);
                kahan_add_corrected(C[i], Ck[i], pc);
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    Dc[i] = fmaf(Ds[s], wa[s].y, Dc[i]);
            }
            else
            {
#pragma unroll
                for (int s = 0; s < 4; ++s)
                {
                    C[i] = fmaf(Ss[s], wa[s].x, C[i]);
                    Dc[i] = fmaf(Ds[s], wa[s].y, Dc[i]);
                }
            }
            if (i + 1 < NJ)
            {
#pragma unroll
                for (int s = 0; s < 4; ++s)
                {
                    const cf next = {fmaf(c4[s], wb[s].x, -wa[s].x), fmaf(c4[s], wb[s].y, -wa[s].y)};
                    wa[s] = wb[s];
                    wb[s] = next;
                }
            }
        }

        // the last valid sample of this round becomes the left end of the next segment
        const int src = qbase + (nv > 0 ? nv - 1 : 0);
        const float f_last = __shfl_sync(kFull, f_my, src);
        const float p_last = __shfl_sync(kFull, p_my, src);
        if (nv > 0)
        {
            f_tail = f_last;
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

    // last sample exactly at t_far (raymarch_generate.h:107-113)
    float f_far = 0.f;
    if (hit)
    {
        f_far = map_density(volume_sample(a.vol, __fadd_rn(o[0], __fmul_rn(t_far, d[0])),
                                        __fadd_rn(o[1], __fmul_rn(t_far, d[1])),
                                        __fadd_rn(o[2], __fmul_rn(t_far, d[2]))),
                            a.data_min, a.data_span, a.data_inv_span, a.data_span_pow2);
        blo = rmin(blo, f_far);
        bhi = rmax(bhi, f_far);
    }
    // bounds over the quad (every lane of the warp takes part in the shuffles)
    blo = rmin(blo, __shfl_xor_sync(kFull, blo, 1));
    bhi = rmax(bhi, __shfl_xor_sync(kFull, bhi, 1));
    blo = rmin(blo, __shfl_xor_sync(kFull, blo, 2));
    bhi = rmax(bhi, __shfl_xor_sync(kFull, bhi, 2));

    if (!in_image)
        return;

    float *out = a.moments + pix * (size_t)a.m;
    if (!hit)
    {
        // missed ray: zero moments, bound (0, 0), no moments kept by compaction
        for (int j = q; j < a.m; j += 4)
            out[j] = 0.f;
        if (q == 0)
        {
            if (a.bounds && a.transform_to_bounds)
            {
                a.bounds[2 * pix] = 0;
                a.bounds[2 * pix + 1] = 0;
            }
            if (a.counts && a.compact_image)
                a.counts[pix] = 0;
            if (a.bounds4)
                a.bounds4[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }

    const float sL = __fsub_rn(f_tail, base) + __fsub_rn(f_far, base);
    const float dL = f_far - f_tail;
    const float hL = -0.5f * p_tail;
    float snL, csL;
    sincosf(0.5f * p_tail, &snL, &csL);
    const cf zL = {csL, -snL};
    const cf zL2 = csq(zL);
    const cf vL = csq(zL2);
    cf wL = {1.f, 0.f};
    wL = (q == 1) ? zL : wL;
    wL = (q == 2) ? zL2 : wL;
    wL = (q == 3) ? cmul(zL2, zL) : wL;

    float lo = blo, hi = bhi;
    double inv = 1.0;
    if (a.transform_to_bounds)
    {
        lo = rmax(__fsub_rn(blo, a.bound_eps), 0.f);
        hi = rmin(__fadd_rn(bhi, a.bound_eps), 1.f);
        inv = 1.0 / (double)__fsub_rn(hi, lo);
    }

    const float h = half_pss;
    float m0 = 0.f;
#pragma unroll
    for (int i = 0; i < NJ; ++i)
    {
        const int j = q + 4 * i;
        if (j < a.m)
        {
            float al, be, alL, beL;
            seg_coeffs(j, h, al, be);
            seg_coeffs(j, hL, alL, beL);
            const float trig = al * C[i] + be * Dc[i] + (alL * sL * wL.x + beL * dL * wL.y);
            // the baseline's share: c for the zeroth moment, nothing for the others
            const float rel = __fmul_rn(trig, kMInvPi);
            float val;
            if (a.transform_to_bounds)
                val = (j == 0) ? (float)(((double)base - (double)lo + (double)rel) * inv) : (float)((double)rel * inv);
            else
                val = (j == 0) ? __fadd_rn(base, rel) : rel;
            out[j] = val;
            if (j == 0)
                m0 = val;
        }
        wL = cmul(wL, vL);
    }

    if (q == 0)
    {
        if (a.bounds4)
            a.bounds4[pix] = make_float4(lo, hi, blo, bhi);
        const uint16_t lo16 = (uint16_t)__fmul_rn(lo, 65535.f);
        const uint16_t hi16 = (uint16_t)__fmul_rn(hi, 65535.f);
        if (a.bounds && a.transform_to_bounds)
        {
            a.bounds[2 * pix] = lo16;
            a.bounds[2 * pix + 1] = hi16;
        }
        if (a.counts && a.compact_image)
        {
            // compute_num_moments (moment_compaction.h:147-174): an empty ray keeps no moments; with a zero
            // error threshold every other ray keeps all m (otherwise count_moments_kernel refines this).
            const bool is_zero = a.transform_to_bounds ? (lo16 == hi16) : (m0 == 0.f);
            a.counts[pix] = is_zero ? 0u : (uint32_t)a.m;
        }
    }
}

template <int NJ, bool KAHAN>
__global__ void __launch_bounds__(128) generate_grid_kernel(const GenArgs<GridView> a)
{
    generate_quads<GridView, NJ, KAHAN>(a);
}

template <int NJ, bool KAHAN>
__global__ void __launch_bounds__(128) generate_particles_kernel(const GenArgs<ParticleView> a)
{
    generate_quads<ParticleView, NJ, KAHAN>(a);
}

template <int NJ, bool KAHAN>
__global__ void __launch_bounds__(128) generate_particles_h_kernel(const GenArgs<ParticleHView> a)
{
    generate_quads<ParticleHView, NJ, KAHAN>(a);
}

// The compensated instantiations at five blocks per SM: 96 registers, the Kahan terms kept with a few bytes of
// spill (9.84 ms against 10.6 at the four blocks of their unbounded 120-128 registers, 512^3 / 1024^2 / m = 64).
// The plain ones keep the unbounded allocation (96 registers for the grid, 72 with some spill for particles, seven
// blocks): a stated minimum gives them 110-128 registers, or spills, and measured slower.
#define MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, NJ)                                                                       \
    template <> __global__ void __launch_bounds__(128, 5) NAME<NJ, true>(const GenArgs<VIEW> a)                      \
    {                                                                                                              \
        generate_quads<VIEW, NJ, true>(a);                                                                         \
    }
#define MRAYGB_KAHAN_5_BLOCKS_ALL(NAME, VIEW)                                                                       \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 1)                                                                           \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 2)                                                                           \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 4)                                                                           \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 8)                                                                           \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 16)                                                                          \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 32)                                                                          \
    MRAYGB_KAHAN_5_BLOCKS(NAME, VIEW, 64)
MRAYGB_KAHAN_5_BLOCKS_ALL(generate_grid_kernel, GridView)
MRAYGB_KAHAN_5_BLOCKS_ALL(generate_particles_kernel, ParticleView)
MRAYGB_KAHAN_5_BLOCKS_ALL(generate_particles_h_kernel, ParticleHView)
#undef MRAYGB_KAHAN_5_BLOCKS_ALL
#undef MRAYGB_KAHAN_5_BLOCKS

template <int NJ, bool KAHAN> void launch_kernel(const GenArgs<GridView> &a, dim3 grid, cudaStream_t stream)
{
    generate_grid_kernel<NJ, KAHAN><<<grid, 128, 0, stream>>>(a);
}
template <int NJ, bool KAHAN> void launch_kernel(const GenArgs<ParticleView> &a, dim3 grid, cudaStream_t stream)
{
    generate_particles_kernel<NJ, KAHAN><<<grid, 128, 0, stream>>>(a);
}
template <int NJ, bool KAHAN> void launch_kernel(const GenArgs<ParticleHView> &a, dim3 grid, cudaStream_t stream)
{
    generate_particles_h_kernel<NJ, KAHAN><<<grid, 128, 0, stream>>>(a);
}

template <int NJ, class V> void launch_nj(const GenArgs<V> &a, bool kahan, cudaStream_t stream)
{
    const dim3 grid((a.width + 7) / 8, (a.height + 3) / 4);
    if (kahan)
        launch_kernel<NJ, true>(a, grid, stream);
    else
        launch_kernel<NJ, false>(a, grid, stream);
}

template <class V>
cudaError_t launch_generate(const V &vol, const DeviceCamera &cam, const mraygb_generation_params &gp, int width,
                            int height, int m, bool kahan, float *moments, uint16_t *bounds, uint32_t *counts,
                            float4 *bounds4, int *error_flag, cudaStream_t stream)
{
    GenArgs<V> a;
    a.vol = vol;
    a.cam = cam;
    a.width = width;
    a.height = height;
    a.m = m;
    a.step = gp.step_size;
    a.data_min = gp.data_min;
    a.data_max = gp.data_max;
    a.data_span = gp.data_max - gp.data_min;
    a.data_span_pow2 = is_pow2_divisor(a.data_span) ? 1 : 0;
    a.data_inv_span = a.data_span_pow2 ? 1.0f / a.data_span : 0.f;
    a.bound_eps = gp.transform_bound_eps;
    a.transform_to_bounds = gp.transform_to_bounds ? 1 : 0;
    a.compact_image = gp.compact_image ? 1 : 0;
    a.error_threshold_zero = gp.error_threshold == 0.f ? 1 : 0;
    a.moments = moments;
    a.bounds = bounds;
    a.counts = counts;
    a.bounds4 = bounds4;
    a.error_flag = error_flag;
    const int nj = (m + 3) / 4;
    if (nj <= 1)
        launch_nj<1>(a, kahan, stream);
    else if (nj <= 2)
        launch_nj<2>(a, kahan, stream);
    else if (nj <= 4)
        launch_nj<4>(a, kahan, stream);
    else if (nj <= 8)
        launch_nj<8>(a, kahan, stream);
    else if (nj <= 16)
        launch_nj<16>(a, kahan, stream);
    else if (nj <= 32)
        launch_nj<32>(a, kahan, stream);
    else
        launch_nj<64>(a, kahan, stream);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_generate_grid(const GridView &grid, const DeviceCamera &cam, const mraygb_generation_params &gp,
                                 int width, int height, int m, bool kahan, float *moments, uint16_t *bounds,
                                 uint32_t *counts, float4 *bounds4, int *error_flag, cudaStream_t stream)
{
    return launch_generate(grid, cam, gp, width, height, m, kahan, moments, bounds, counts, bounds4, error_flag,
                           stream);
}

cudaError_t launch_generate_particles(const ParticleView &parts, const DeviceCamera &cam,
                                      const mraygb_generation_params &gp, int width, int height, int m, bool kahan,
                                      float *moments, uint16_t *bounds, uint32_t *counts, float4 *bounds4,
                                      int *error_flag, cudaStream_t stream)
{
    return launch_generate(parts, cam, gp, width, height, m, kahan, moments, bounds, counts, bounds4, error_flag,
                           stream);
}

cudaError_t launch_generate_particles_h(const ParticleHView &parts, const DeviceCamera &cam,
                                        const mraygb_generation_params &gp, int width, int height, int m, bool kahan,
                                        float *moments, uint16_t *bounds, uint32_t *counts, float4 *bounds4,
                                        int *error_flag, cudaStream_t stream)
{
    return launch_generate(parts, cam, gp, width, height, m, kahan, moments, bounds, counts, bounds4, error_flag,
                           stream);
}

} // namespace mraygb
