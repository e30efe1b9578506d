// Error bounds and uncertainty rendering.
//
// * error_bound_kernel: reconstruct_error (src/raymarch_reconstruct.h:322-378, driven per pixel by
//   reconstruct_error_host / reconstruct_error_kernel, src/moment_raymarcher.cpp:516-560, .cu:693-752): one
//   thread per pixel marches its eye ray through the resident volume (grid texture or SPH particles) at the error
//   step, evaluates the bounded-MESE density at the sample's phase and updates one error measure against the
//   volume's mapped density: the maximum, the RMSE, or the P^2 estimate of a percentile (src/error_measures.h:
//   30-229, its five markers in registers).  The result is stored as MomentImageHost::set_error_bound does.
// * uncertainty_tf_kernel: the 256 x 256 tables of read_from_disk_uncertainty (src/transfer_function.cpp:151-248),
//   one thread per entry, the reference's float operations in its order (this file is compiled without FMA
//   contraction).
// * uncertainty_kernel: reconstruct_uncertainty_interpolation (mode 0: reconstruct_ray with the density
//   lerp(clamp(rho - e), clamp(rho + e), t) and the preintegrated row) and reconstruct_uncertainty_convolution
//   (mode 1: reconstruct_ray_uncertainty_tf with the (lower, upper) or (mean, deviation) pair looked up in the
//   uncertainty table), src/moment_raymarcher.cpp:562-717, src/raymarch_reconstruct.h:137-259,
//   src/reconstruction_techniques.h:99-155.
//
// The MESE density is the re-march's (Reinsch's series, fast_atan); the sample positions, phases and volume
// samples are the reference's.

#include "device_common.cuh"
#include "internal.h"
#include "reconstruct_common.cuh"

namespace mraygb
{
namespace
{

constexpr double kPiD = 3.141592653589793;

// to_phase (src/raymarch_common.h:41-44): (t - t_near) / (t_far - t_near) * M_PI - M_PI
__device__ __forceinline__ float to_phase(float t, float t_near, float range)
{
    return (float)((double)__fdiv_rn(__fsub_rn(t, t_near), range) * kPiD - kPiD);
}

// The same phase without FP64 (GB300 runs FP64 at 1/64 of the FP32 rate and this is evaluated per sample):
// M_PI * q - M_PI = M_PI (q - 1) with q - 1 split exactly into s + e (two-sum) and the double M_PI split exactly
// into three floats, the leading product exact by FMA; the float result equals the reference's except where the
// exact value lies within about 2^-48 of a float rounding boundary.
constexpr float kPi1 = (float)kPiD;
constexpr float kPi2 = (float)(kPiD - (double)kPi1);
constexpr float kPi3 = (float)((kPiD - (double)kPi1) - (double)kPi2);
__device__ __forceinline__ float to_phase_ff(float t, float t_near, float range)
{
    const float q = __fdiv_rn(__fsub_rn(t, t_near), range);
    const float s = __fadd_rn(q, -1.f);
    const float bb = __fsub_rn(s, q);
    const float e = __fadd_rn(__fsub_rn(q, __fsub_rn(s, bb)), __fsub_rn(-1.f, bb));
    const float h = __fmul_rn(s, kPi1);
    const float l = __fmaf_rn(s, kPi1, -h);
    const float small = __fmaf_rn(s, kPi2, __fmaf_rn(e, kPi1, __fmaf_rn(s, kPi3, __fmaf_rn(e, kPi2, l))));
    return __fadd_rn(h, small);
}

// ---- error measures (src/error_measures.h:30-229) -------------------------------------------------------------

struct ErrMax
{
    float e = 0.f;
    __device__ __forceinline__ void update(float ref, float pred) { e = rmax(e, fabsf(__fsub_rn(pred, ref))); }
    __device__ __forceinline__ float value() const { return e; }
};

struct ErrRmse
{
    float squares = 0.f;
    int count = 0;
    __device__ __forceinline__ void update(float ref, float pred)
    {
        count += 1;
        const float diff = __fsub_rn(pred, ref);
        squares = __fadd_rn(squares, __fmul_rn(diff, diff));
    }
    __device__ __forceinline__ float value() const { return sqrtf(__fdiv_rn(squares, (float)count)); }
};

// The P^2 estimator of Jain and Chlamtac with the reference's steps.  Markers start at 0 (the reference leaves
// them uninitialised, read by rays of fewer than three samples).  The reference's adjust loop also visits the last
// marker, whose desired and actual positions both grow by exactly 1 per update, so its test always fails there;
// only the three middle markers move.  All indices are compile-time constants, so the state stays in registers.
struct ErrPercentile
{
    float q, q_half, q_mid; // q, q / 2 and (1 + q) / 2: the constant marker increments of update
    int init_num = 0;
    float h[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    int pos[5] = {0, 0, 0, 0, 0};
    float des[5] = {0.f, 0.f, 0.f, 0.f, 0.f};

    // ErrorPercentile(float p) : q(p / 100.f); built on the host and passed to the kernel as the initial state
    __host__ __device__ explicit ErrPercentile(int percentile)
        : q((float)percentile / 100.f), q_half(q / 2.0f), q_mid((1.0f + q) / 2.f)
    {
    }

    __device__ __forceinline__ static void swap(float &a, float &b)
    {
        const float t = a;
        a = b;
        b = t;
    }

    // sort_five_numbers (error_measures.h:55-101)
    __device__ __forceinline__ void sort5()
    {
        if (h[1] < h[0])
            swap(h[0], h[1]);
        if (h[2] < h[1])
        {
            swap(h[2], h[1]);
            if (h[1] < h[0])
                swap(h[1], h[0]);
        }
        if (h[3] < h[2])
        {
            swap(h[3], h[2]);
            if (h[1] < h[0])
                swap(h[1], h[0]);
            if (h[2] < h[1])
            {
                swap(h[2], h[1]);
                if (h[1] < h[0])
                    swap(h[1], h[0]);
            }
        }
        if (h[4] < h[3])
        {
            swap(h[4], h[3]);
            if (h[3] < h[2])
            {
                swap(h[3], h[2]);
                if (h[1] < h[0])
                    swap(h[1], h[0]);
                if (h[2] < h[1])
                {
                    swap(h[2], h[1]);
                    if (h[1] < h[0])
                        swap(h[1], h[0]);
                }
            }
        }
    }

    template <int I> __device__ __forceinline__ void adjust_one()
    {
        const float di = __fsub_rn(des[I], (float)pos[I]);
        if ((di >= 1.f && (pos[I + 1] - pos[I] > 1)) || (di <= -1.f && (pos[I - 1] - pos[I] < -1)))
        {
            const int sdi = (di > 0.f) ? 1 : -1;
            // parabolic (error_measures.h:121-132)
            const float t1 = __fdiv_rn((float)sdi, (float)(pos[I + 1] - pos[I - 1]));
            const float t2 = __fdiv_rn(__fmul_rn((float)(pos[I] - pos[I - 1] + sdi), __fsub_rn(h[I + 1], h[I])),
                                       (float)(pos[I + 1] - pos[I]));
            const float t3 = __fdiv_rn(__fmul_rn((float)(pos[I + 1] - pos[I] - sdi), __fsub_rn(h[I], h[I - 1])),
                                       (float)(pos[I] - pos[I - 1]));
            const float qprime = __fadd_rn(h[I], __fmul_rn(t1, __fadd_rn(t2, t3)));
            if ((h[I - 1] < qprime) && (qprime < h[I + 1]))
                h[I] = qprime;
            else
            {
                // linear (error_measures.h:134-138)
                const float hn = sdi > 0 ? h[I + 1] : h[I - 1];
                const int pn = sdi > 0 ? pos[I + 1] : pos[I - 1];
                h[I] = __fadd_rn(h[I], __fdiv_rn(__fmul_rn((float)sdi, __fsub_rn(hn, h[I])), (float)(pn - pos[I])));
            }
            pos[I] += sdi;
        }
    }

    __device__ __forceinline__ void update(float ref, float pred)
    {
        const float value = fabsf(__fsub_rn(pred, ref));
        if (init_num < 5)
        {
#pragma unroll
            for (int k = 0; k < 5; ++k)
                if (init_num == k)
                    h[k] = value;
            ++init_num;
            if (init_num == 5)
            {
                sort5();
#pragma unroll
                for (int i = 0; i < 5; ++i)
                    pos[i] = 1 + i;
                des[0] = 1.0f;
                des[1] = __fadd_rn(1.0f, __fmul_rn(2.0f, q));
                des[2] = __fadd_rn(1.0f, __fmul_rn(4.0f, q));
                des[3] = __fadd_rn(3.0f, __fmul_rn(2.0f, q));
                des[4] = 5.0f;
            }
            return;
        }
        int move_idx = 0;
        if (value < h[0])
        {
            h[0] = value;
            move_idx = 1;
        }
        else if (value < h[1])
            move_idx = 1;
        else if (value < h[2])
            move_idx = 2;
        else if (value < h[3])
            move_idx = 3;
        else if (value < h[4])
            move_idx = 4;
        else if (value > h[4])
        {
            h[4] = value;
            move_idx = 4;
        }
#pragma unroll
        for (int k = 0; k < 5; ++k)
            if (k >= move_idx)
                pos[k] += 1;
        des[1] = __fadd_rn(des[1], q_half);
        des[2] = __fadd_rn(des[2], q);
        des[3] = __fadd_rn(des[3], q_mid);
        des[4] = __fadd_rn(des[4], 1.0f);
        adjust_one<1>();
        adjust_one<2>();
        adjust_one<3>();
    }

    __device__ __forceinline__ float value() const { return h[2]; }
};

struct ErrorDev
{
    DeviceCamera cam;
    int width, height, m;
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    float step, data_min, data_max;
    int percentile;
    uint16_t *error_bounds;
    float *errors;
    int *error_flag;
};

template <int MAXM>
__device__ __forceinline__ int load_multipliers(const uint32_t *index, const float *pmoments, int m, size_t pix,
                                                float (&lam2)[MAXM], float &lam0)
{
    size_t idx;
    int n;
    if (index)
    {
        idx = index[pix];
        n = (int)(index[pix + 1] - index[pix]);
    }
    else
    {
        idx = pix * (size_t)m;
        n = m;
    }
    if (n > MAXM)
        n = MAXM;
    lam0 = n > 0 ? pmoments[idx] : 0.f;
#pragma unroll
    for (int l = 0; l < MAXM; ++l)
        lam2[l] = (l < n && l > 0) ? 2.f * pmoments[idx + l] : 0.f;
    return n;
}

template <class V, int MAXM, class E>
__global__ void __launch_bounds__(128) error_bound_kernel(const ErrorDev a, const V vol, E proto)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.width || y >= a.height)
        return;
    const size_t pix = (size_t)y * (size_t)a.width + (size_t)x;
    float lam2[MAXM], lam0;
    const int n = load_multipliers<MAXM>(a.index, a.pmoments, a.m, pix, lam2, lam0);
    float e = 0.f;
    if (n > 0)
    {
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
        const bool hit = intersect_aabb(o, d, vol.dmin, vol.dmax, t_near, t_far);
        t_near = rmax(t_near, a.cam.znear);
        if (hit && t_far > 0.f)
        {
            E acc = proto;
            const float range = __fsub_rn(t_far, t_near);
            // the march ends by itself after about range / step samples; the cap only guards a step too small to
            // advance t in float
            const float est = range / a.step;
            const int cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
            int it = 0;
            float t = t_near;
            while (t <= t_far)
            {
                if (++it > cap)
                {
                    atomicExch(a.error_flag, 1);
                    break;
                }
                const float fs = mese_density<MAXM>(lam2, lam0, to_phase_ff(t, t_near, range), lo, span);
                const float ref = map_density(volume_sample(vol, __fadd_rn(o[0], __fmul_rn(t, d[0])),
                                                            __fadd_rn(o[1], __fmul_rn(t, d[1])),
                                                            __fadd_rn(o[2], __fmul_rn(t, d[2]))),
                                              a.data_min, a.data_max);
                acc.update(ref, fs);
                t = __fadd_rn(t, a.step);
            }
            e = acc.value();
        }
    }
    if (a.errors)
        a.errors[pix] = e;
    // MomentImageHost::set_error_bound (src/moment_image.h:102-106): static_cast<uint16_t>(e * 65535)
    a.error_bounds[pix] = (uint16_t)(int)__fmul_rn(e, 65535.f);
}

// ---- the uncertainty table (transfer_function.cpp:151-248) ----------------------------------------------------

// cut::normal_cdf (src/cut/gaussian.h:33-59) with its double intermediates; exp of the float argument correctly
// rounded (the double function rounded to float)
__device__ __forceinline__ float normal_cdf(float x)
{
    const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f, a4 = -1.453152027f, a5 = 1.061405429f,
                p = 0.3275911f;
    const int sign = (x < 0.f) ? -1 : 1;
    x = (float)((double)fabsf(x) / 1.41421356237);
    const float t = (float)(1.0 / (1.0 + (double)(p * x)));
    const float ex = (float)exp((double)(-x * x));
    const float y = (float)(1.0 - (double)((((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * ex));
    return (float)(0.5 * (1.0 + (double)sign * (double)y));
}

__global__ void uncertainty_tf_kernel(const float4 *__restrict__ tf1d, float step, int error_type,
                                      float4 *__restrict__ table)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= 256)
        return;
    float4 rgba = make_float4(0.f, 0.f, 0.f, 0.f);
    if (error_type == MRAYGB_ERROR_RMSE)
    {
        // gaussian_filter (transfer_function.cpp:188-231)
        const float mean = x / 256.f, sd = y / 256.f;
        if (sd != 0.f)
        {
            const float delta = 1.0f / 256.f;
            for (int i = 0; i < 256; ++i)
            {
                const float xi = i * delta;
                const float weight = normal_cdf((xi + delta - mean) / sd) - normal_cdf((xi - mean) / sd);
                const float4 v = tf1d[i];
                const float a = weight * v.w * step;
                rgba.x += v.x * a;
                rgba.y += v.y * a;
                rgba.z += v.z * a;
                rgba.w += a;
            }
        }
        else
        {
            rgba = tf1d[x];
            rgba.w *= step;
            rgba.x = rgba.x * rgba.w;
            rgba.y = rgba.y * rgba.w;
            rgba.z = rgba.z * rgba.w;
        }
    }
    else
    {
        // box_filter (transfer_function.cpp:151-186) with sample1D (:37-43)
        const float sf = x / 256.f, sb = y / 256.f;
        const int num_steps = abs(y - x) + 2;
        const float dw = 1.0f / (float)num_steps;
        for (int i = 0; i < num_steps; ++i)
        {
            const float w = (float)i / (float)(num_steps - 1);
            const float s = w * sb + (1.f - w) * sf;
            const float ip = s * 256.f;
            const float af = ip - floorf(ip);
            const int xl = (int)floorf(ip);
            const float4 v0 = tf1d[min(max(xl, 0), 255)], v1 = tf1d[min(max(xl + 1, 0), 255)];
            float4 v;
            v.x = (1.f - af) * v0.x + af * v1.x;
            v.y = (1.f - af) * v0.y + af * v1.y;
            v.z = (1.f - af) * v0.z + af * v1.z;
            v.w = (1.f - af) * v0.w + af * v1.w;
            const float a = dw * v.w * step;
            rgba.x += v.x * a;
            rgba.y += v.y * a;
            rgba.z += v.z * a;
            rgba.w += a;
        }
    }
    table[y * 256 + x] = rgba;
}

// ---- uncertainty rendering --------------------------------------------------------------------------------------

// TransferFunction::sample on a whole 256 x 256 table (src/transfer_function.h:36-59) with the reference's
// weights: the (x, y + 1) texel takes a.x (1 - a.y) and the (x + 1, y) texel (1 - a.x) a.y
__device__ __forceinline__ float4 tf2d_sample(const float4 *__restrict__ T, float fs, float bs)
{
    const float ipx = fs * 256.f, ipy = bs * 256.f;
    const float flx = floorf(ipx), fly = floorf(ipy);
    const float ax = ipx - flx, ay = ipy - fly;
    const int xl = (int)flx, yl = (int)fly;
    const int x0 = min(max(xl, 0), 255), x1 = min(max(xl + 1, 0), 255);
    const int y0 = min(max(yl, 0), 255), y1 = min(max(yl + 1, 0), 255);
    const float4 ll = __ldg(T + y0 * 256 + x0), lr = __ldg(T + y1 * 256 + x0), rr = __ldg(T + y1 * 256 + x1),
                 rl = __ldg(T + y0 * 256 + x1);
    const float wll = (1.f - ax) * (1.f - ay), wlr = ax * (1.f - ay), wrl = (1.f - ax) * ay, wrr = ax * ay;
    float4 r;
    r.x = wll * ll.x + wlr * lr.x + wrl * rl.x + wrr * rr.x;
    r.y = wll * ll.y + wlr * lr.y + wrl * rl.y + wrr * rr.y;
    r.z = wll * ll.z + wlr * lr.z + wrl * rl.z + wrr * rr.z;
    r.w = wll * ll.w + wlr * lr.w + wrl * rl.w + wrr * rr.w;
    return r;
}

struct UncertaintyDev
{
    DeviceCamera cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const uint16_t *error_bounds;
    const float4 *tf;    // mode 0: the preintegrated row (256)
    const float4 *table; // mode 1: the uncertainty table (256 x 256)
    float step, emission, ert, interp;
    int pair_bounds; // mode 1: (lower, upper) for MAX_ERROR, (mean, deviation) otherwise
    float *rgba;
    uint8_t *rgba8;
    int *error_flag;
};

// ErrorBoundInterpolator::reconstruct over ErrorBoundMESEReconstruction: lerp of the clamped bounds
// (cut::lerp = (1 - t) a + t b)
template <int MAXM>
__device__ __forceinline__ float interp_density(const float (&lam2)[MAXM], float lam0, float p, float lo, float hi,
                                                float span, float e, float t)
{
    const float rho = mese_density<MAXM>(lam2, lam0, p, lo, span);
    const float b0 = rclamp(rho - e, lo, hi), b1 = rclamp(rho + e, lo, hi);
    return (1.f - t) * b0 + t * b1;
}

template <int MAXM, int MODE> __global__ void __launch_bounds__(128) uncertainty_kernel(const UncertaintyDev a)
{
    __shared__ float4 s_tf[256];
    if (MODE == 0)
    {
        for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y)
            s_tf[i] = a.tf[i];
        __syncthreads();
    }
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.width || y >= a.height)
        return;
    const size_t pix = (size_t)y * (size_t)a.width + (size_t)x;
    float lam2[MAXM], lam0;
    const int n = load_multipliers<MAXM>(a.index, a.pmoments, a.m, pix, lam2, lam0);
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (n == 0)
    {
        // reconstruct_zero_ray (src/raymarch_reconstruct.h:127-131)
        const float4 z = MODE == 0 ? tf_sample(s_tf, 0.f, 0.f) : tf2d_sample(a.table, 0.f, 0.f);
        out = make_float4(z.x, z.y, z.z, 0.f);
    }
    else
    {
        float lo = 0.f, hi = 1.f;
        if (a.bounds)
        {
            lo = a.bounds[2 * pix] / 65535.f;
            hi = a.bounds[2 * pix + 1] / 65535.f;
        }
        const float span = hi - lo;
        const float e = a.error_bounds[pix] / 65535.f; // MomentImageHost::get_error_bound
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
            float p = to_phase(t, t_near, range);
            const float phase_step = (float)(kPiD * (double)__fdiv_rn(a.step, range));
            const float est = range / a.step;
            const int cap = (est < 1.6e9f ? (int)(1.25f * est) : 2000000000) + 64;
            float L0 = 0.f, L1 = 0.f, L2 = 0.f, alpha = 0.f, T = 1.f, tau = 0.f;
            float fs = MODE == 0 ? interp_density<MAXM>(lam2, lam0, p, lo, hi, span, e, a.interp) : 0.f;
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
                float4 s;
                if (MODE == 0)
                {
                    const float bs = interp_density<MAXM>(lam2, lam0, p, lo, hi, span, e, a.interp);
                    s = tf_sample(s_tf, fs, bs);
                    fs = bs;
                }
                else
                {
                    const float rho = mese_density<MAXM>(lam2, lam0, p, lo, span);
                    const float dx = a.pair_bounds ? rclamp(rho - e, lo, hi) : rho;
                    const float dy = a.pair_bounds ? rclamp(rho + e, lo, hi) : e;
                    s = tf2d_sample(a.table, dx, dy);
                }
                L0 += (a.emission * s.x) * T;
                L1 += (a.emission * s.y) * T;
                L2 += (a.emission * s.z) * T;
                tau += s.w;
                T = expf(-tau);
                alpha = 1.f - T;
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

template <class V, int MAXM>
cudaError_t launch_error_m(const ErrorDev &a, const V &vol, int error_type, cudaStream_t stream)
{
    const dim3 block(16, 8), grid((a.width + 15) / 16, (a.height + 7) / 8);
    if (error_type == MRAYGB_ERROR_MAX)
        error_bound_kernel<V, MAXM, ErrMax><<<grid, block, 0, stream>>>(a, vol, ErrMax{});
    else if (error_type == MRAYGB_ERROR_RMSE)
        error_bound_kernel<V, MAXM, ErrRmse><<<grid, block, 0, stream>>>(a, vol, ErrRmse{});
    else
        error_bound_kernel<V, MAXM, ErrPercentile><<<grid, block, 0, stream>>>(a, vol, ErrPercentile(a.percentile));
    return cudaGetLastError();
}

template <class V>
cudaError_t launch_error_v(const ErrorDev &a, const V &vol, int error_type, cudaStream_t stream)
{
    if (a.m <= 8)
        return launch_error_m<V, 8>(a, vol, error_type, stream);
    if (a.m <= 16)
        return launch_error_m<V, 16>(a, vol, error_type, stream);
    if (a.m <= 32)
        return launch_error_m<V, 32>(a, vol, error_type, stream);
    if (a.m <= 64)
        return launch_error_m<V, 64>(a, vol, error_type, stream);
    if (a.m <= 128)
        return launch_error_m<V, 128>(a, vol, error_type, stream);
    return launch_error_m<V, 256>(a, vol, error_type, stream);
}

ErrorDev error_args(const ErrorArgs &r, int *error_flag)
{
    ErrorDev a;
    a.cam = *r.cam;
    a.width = r.width;
    a.height = r.height;
    a.m = r.m;
    a.index = r.index;
    a.pmoments = r.pmoments;
    a.bounds = r.bounds;
    a.step = r.step;
    a.data_min = r.data_min;
    a.data_max = r.data_max;
    a.percentile = r.percentile;
    a.error_bounds = r.error_bounds;
    a.errors = r.errors;
    a.error_flag = error_flag;
    return a;
}

template <int MAXM> cudaError_t launch_uncertainty_m(const UncertaintyDev &a, int mode, cudaStream_t stream)
{
    const dim3 block(16, 8), grid((a.width + 15) / 16, (a.height + 7) / 8);
    if (mode == 0)
        uncertainty_kernel<MAXM, 0><<<grid, block, 0, stream>>>(a);
    else
        uncertainty_kernel<MAXM, 1><<<grid, block, 0, stream>>>(a);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_error_bounds_grid(const GridView &grid, const ErrorArgs &r, int error_type, int *error_flag,
                                     cudaStream_t stream)
{
    return launch_error_v(error_args(r, error_flag), grid, error_type, stream);
}

cudaError_t launch_error_bounds_particles(const ParticleView &parts, const ErrorArgs &r, int error_type,
                                          int *error_flag, cudaStream_t stream)
{
    return launch_error_v(error_args(r, error_flag), parts, error_type, stream);
}

cudaError_t launch_uncertainty_tf(const float4 *tf1d, float step, int error_type, float4 *table, cudaStream_t stream)
{
    uncertainty_tf_kernel<<<dim3(2, 256), 128, 0, stream>>>(tf1d, step, error_type, table);
    return cudaGetLastError();
}

cudaError_t launch_uncertainty(const UncertaintyArgs &r, int *error_flag, cudaStream_t stream)
{
    UncertaintyDev a;
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
    a.error_bounds = r.error_bounds;
    a.tf = r.tf;
    a.table = r.table;
    a.step = r.step;
    a.emission = r.emission;
    a.ert = r.ert;
    a.interp = r.interp;
    a.pair_bounds = r.error_type == MRAYGB_ERROR_MAX;
    a.rgba = r.rgba;
    a.rgba8 = r.rgba8;
    a.error_flag = error_flag;
    if (r.m <= 8)
        return launch_uncertainty_m<8>(a, r.mode, stream);
    if (r.m <= 16)
        return launch_uncertainty_m<16>(a, r.mode, stream);
    if (r.m <= 32)
        return launch_uncertainty_m<32>(a, r.mode, stream);
    if (r.m <= 64)
        return launch_uncertainty_m<64>(a, r.mode, stream);
    if (r.m <= 128)
        return launch_uncertainty_m<128>(a, r.mode, stream);
    return launch_uncertainty_m<256>(a, r.mode, stream);
}

} // namespace mraygb
