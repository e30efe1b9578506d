// The C ABI (include/mraygb.h): contexts, resident inputs, the stage API and the drop-in host API.
//
// Host code only: argument checks, device buffers owned by the context, launches in stream order and the
// copies of the drop-in calls.  Every failure is reported through the return code and mraygb_last_error;
// nothing here aborts.

#include "../../include/mraygb.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "device_common.cuh"
#include "internal.h"
#include "lz4_block.h"
#include "moment_file.h"

using namespace mraygb;

namespace
{

struct DeviceBuffer
{
    void *ptr = nullptr;
    size_t bytes = 0;

    cudaError_t reserve(size_t n)
    {
        if (n <= bytes)
            return cudaSuccess;
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess)
            bytes = n;
        return e;
    }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

} // namespace

struct mraygb_context
{
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int precision = MRAYGB_PRECISION_FP32;
    // the differentiation form's transfer-function row: MRAYGB_DIFF_TF_BSPLINE or MRAYGB_DIFF_TF_LINEAR
    int diff_tf_sampling = MRAYGB_DIFF_TF_BSPLINE;
    std::string error;
    uint64_t launches = 0;

    // resident inputs: the volume uploaded last (a grid or particles) and the transfer function
    enum Volume
    {
        NONE,
        GRID,
        PARTICLES
    } volume = NONE;
    // the grid as a 3D array behind a point-sampled texture (hardware clamp to edge, 3D-blocked layout)
    cudaArray_t grid_array = nullptr;
    cudaTextureObject_t grid_tex = 0;
    int nx = 0, ny = 0, nz = 0;
    float dmin[3] = {0, 0, 0}, dmax[3] = {0, 0, 0};
    DeviceBuffer particle_pts, particle_cells;
    ParticleGridParams particle_grid{};
    uint64_t num_particles = 0;
    // per-particle smoothing lengths with the Wendland C2 kernel (mraygb_upload_particles_h): (1/h, 1/h^3) per record
    DeviceBuffer particle_inv_h;
    bool particle_wendland = false;
    DeviceBuffer tf;
    bool has_tf = false;

    // work buffers of the drop-in calls and of the scan
    DeviceBuffer moments, counts, index, compact, bounds, coding_params, pmoments, rgba, rgba8, scan_scratch;
    DeviceBuffer error_flag;
    // prediction coding and quantization
    DeviceBuffer coding_partial, coding_params_f, table, bits, bit_offset, scan_scratch64, packed;
    // adjoint work buffers of the differentiation form; diff_keep: the preparation's Levinson solution and
    // exponential moments (2m float2 per pixel) for the buffers and sizes in diff_key, valid while diff_key.valid
    DeviceBuffer adj_lambda, adj_bounds, diff_keep;
    struct
    {
        bool valid = false;
        const float *moments = nullptr, *pmoments = nullptr;
        int width = 0, height = 0, m = 0;
        float bias = 0.f;
    } diff_key;
    // the quantization curve: per-sample moments and errors, the means, the uploaded sample of the host call
    DeviceBuffer qc_scratch, qc_means, qc_index, qc_data;
    // error bounds and uncertainty rendering: the bounds and errors of the host calls, the 256 x 256 uncertainty
    // table (resident) and the 1D table it is built from
    DeviceBuffer error_bounds, errors, unc_table, unc_tf1d;
    bool has_unc_table = false;
    // the single-scattering transmittance cache as a float grid behind a point-sampled texture (as the volume), the
    // per-voxel keys of its build and its linear copy
    cudaArray_t ss_array = nullptr;
    cudaTextureObject_t ss_tex = 0;
    int ss_size[3] = {0, 0, 0};
    float ss_dmin[3] = {0, 0, 0}, ss_dmax[3] = {0, 0, 0};
    bool has_ss_cache = false;
    DeviceBuffer ss_keys, ss_linear;
    // the moment-image file format: the last encoded file and the codes of the entropy coder
    std::vector<uint8_t> encoded;
    DeviceBuffer file_codes;
};

namespace
{

int fail(mraygb_context *ctx, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->error = buf;
    return code;
}

int cuda_fail(mraygb_context *ctx, cudaError_t e, const char *what)
{
    cudaGetLastError(); // clear a sticky launch error where possible
    return fail(ctx, e == cudaErrorMemoryAllocation ? MRAYGB_OUT_OF_MEMORY : MRAYGB_CUDA_ERROR, "%s: %s (%s)", what,
                cudaGetErrorString(e), cudaGetErrorName(e));
}

#define CK(expr, what)                                                                                              \
    do                                                                                                              \
    {                                                                                                               \
        cudaError_t e_ = (expr);                                                                                    \
        if (e_ != cudaSuccess)                                                                                      \
            return cuda_fail(ctx, e_, what);                                                                        \
    } while (0)

#define CHECK_CTX()                                                                                                 \
    do                                                                                                              \
    {                                                                                                               \
        if (!ctx)                                                                                                   \
            return MRAYGB_INVALID_ARGUMENT;                                                                         \
        ctx->error.clear();                                                                                         \
        cudaError_t e_ = cudaSetDevice(ctx->device);                                                                \
        if (e_ != cudaSuccess)                                                                                      \
            return cuda_fail(ctx, e_, "cudaSetDevice");                                                             \
    } while (0)

int check_image(mraygb_context *ctx, int width, int height, int m)
{
    if (width <= 0 || height <= 0 || width > 65535 || height > 65535)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "image size %dx%d outside 1..65535", width, height);
    if (m < 1 || m > MRAYGB_MAX_MOMENTS)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "num_moments %d outside 1..%d", m, MRAYGB_MAX_MOMENTS);
    if ((uint64_t)width * (uint64_t)height * (uint64_t)m >= (1ull << 32))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "W*H*m = %llu exceeds the u32 moment index",
                    (unsigned long long)width * height * m);
    return MRAYGB_OK;
}

void set_extent(GridView &g, const float dmin[3], const float dmax[3])
{
    for (int i = 0; i < 3; ++i)
    {
        g.dmin[i] = dmin[i];
        g.dmax[i] = dmax[i];
        g.ext[i] = dmax[i] - dmin[i];
        g.ext_pow2[i] = is_pow2_divisor(g.ext[i]) ? 1 : 0;
        g.inv_ext[i] = g.ext_pow2[i] ? 1.0f / g.ext[i] : 0.f;
    }
}

GridView grid_view(const mraygb_context *ctx)
{
    GridView g;
    g.tex = ctx->grid_tex;
    g.nx = ctx->nx;
    g.ny = ctx->ny;
    g.nz = ctx->nz;
    set_extent(g, ctx->dmin, ctx->dmax);
    return g;
}

ParticleHView particle_h_view(const mraygb_context *ctx);

ParticleView particle_view(const mraygb_context *ctx)
{
    ParticleView v;
    v.g = ctx->particle_grid;
    v.pts = ctx->particle_pts.as<float4>();
    v.cell_start = ctx->particle_cells.as<uint32_t>();
    for (int i = 0; i < 3; ++i)
    {
        v.dmin[i] = ctx->dmin[i];
        v.dmax[i] = ctx->dmax[i];
    }
    return v;
}

ParticleHView particle_h_view(const mraygb_context *ctx)
{
    ParticleHView v;
    static_cast<ParticleView &>(v) = particle_view(ctx);
    v.inv_h = ctx->particle_inv_h.as<float2>();
    return v;
}

void release_grid(mraygb_context *ctx)
{
    if (ctx->grid_tex)
        cudaDestroyTextureObject(ctx->grid_tex);
    if (ctx->grid_array)
        cudaFreeArray(ctx->grid_array);
    ctx->grid_tex = 0;
    ctx->grid_array = nullptr;
    ctx->nx = ctx->ny = ctx->nz = 0;
}

void release_ss_cache(mraygb_context *ctx)
{
    if (ctx->ss_tex)
        cudaDestroyTextureObject(ctx->ss_tex);
    if (ctx->ss_array)
        cudaFreeArray(ctx->ss_array);
    ctx->ss_tex = 0;
    ctx->ss_array = nullptr;
    ctx->ss_size[0] = ctx->ss_size[1] = ctx->ss_size[2] = 0;
    ctx->has_ss_cache = false;
}

GridView ss_cache_view(const mraygb_context *ctx)
{
    GridView g;
    g.tex = ctx->ss_tex;
    g.nx = ctx->ss_size[0];
    g.ny = ctx->ss_size[1];
    g.nz = ctx->ss_size[2];
    set_extent(g, ctx->ss_dmin, ctx->ss_dmax);
    return g;
}

int check_device_error_flag(mraygb_context *ctx)
{
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, ctx->error_flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
       "reading the device error flag");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    if (flag)
    {
        CK(cudaMemsetAsync(ctx->error_flag.ptr, 0, sizeof(int), ctx->stream), "clearing the device error flag");
        return fail(ctx, MRAYGB_NUMERICAL,
                    "a ray exceeded its step bound: the step size is too small to advance t in float");
    }
    return MRAYGB_OK;
}

int validate_gen(mraygb_context *ctx, const mraygb_generation_params *gp)
{
    if (!gp)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "generation parameters are NULL");
    if (!(gp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)gp->step_size);
    if (gp->prediction_coding && !gp->compact_image)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction_coding requires compact_image");
    if (gp->coding_warp != MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && gp->coding_warp != MRAYGB_CODING_WARP_NONE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown coding_warp %d", gp->coding_warp);
    return MRAYGB_OK;
}

int run_generate_moments(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                         int width, int height, int m, float *d_moments, uint16_t *d_bounds, uint32_t *d_counts,
                         float4 *d_bounds4 = nullptr)
{
    const DeviceCamera dc = to_device_camera(*cam);
    const bool kahan = ctx->precision != MRAYGB_PRECISION_FP32;
    if (ctx->volume == mraygb_context::PARTICLES && ctx->particle_wendland)
        CK(launch_generate_particles_h(particle_h_view(ctx), dc, *gp, width, height, m, kahan, d_moments, d_bounds,
                                       d_counts, d_bounds4, ctx->error_flag.as<int>(), ctx->stream),
           "generate kernel launch");
    else if (ctx->volume == mraygb_context::PARTICLES)
        CK(launch_generate_particles(particle_view(ctx), dc, *gp, width, height, m, kahan, d_moments, d_bounds,
                                     d_counts, d_bounds4, ctx->error_flag.as<int>(), ctx->stream),
           "generate kernel launch");
    else
        CK(launch_generate_grid(grid_view(ctx), dc, *gp, width, height, m, kahan, d_moments, d_bounds, d_counts,
                                d_bounds4, ctx->error_flag.as<int>(), ctx->stream),
           "generate kernel launch");
    ctx->launches += 1;
    if (gp->compact_image && d_counts && gp->error_threshold != 0.f)
    {
        CK(launch_count_moments(width * height, m, gp->error_threshold, d_moments, d_counts, ctx->stream),
           "moment count kernel launch");
        ctx->launches += 1;
    }
    return MRAYGB_OK;
}

int run_compact(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_counts, const float *d_moments,
                uint32_t *d_index, float *d_compact, uint64_t capacity, uint64_t *h_total)
{
    const size_t P = (size_t)width * (size_t)height;
    const size_t words = scan_scratch_words(P);
    CK(ctx->scan_scratch.reserve((words + 1) * sizeof(uint32_t)), "scan scratch allocation");
    int launches = 0;
    CK(launch_exclusive_scan(d_counts, d_index, P, ctx->scan_scratch.as<uint32_t>(), ctx->stream, &launches),
       "scan launch");
    ctx->launches += (uint64_t)launches;
    uint32_t total = 0;
    CK(cudaMemcpyAsync(&total, d_index + P, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream),
       "reading the compact size");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    if ((uint64_t)total > capacity)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "compact buffer holds %llu floats, %u needed",
                    (unsigned long long)capacity, total);
    CK(launch_compact_copy(width * height, m, d_counts, d_index, d_moments, d_compact, ctx->stream),
       "compaction copy launch");
    ctx->launches += 1;
    if (h_total)
        *h_total = total;
    return MRAYGB_OK;
}

int run_prepare(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index, const float *d_data,
                int prediction_code, int coding_warp, const uint16_t *d_coding_params, float bias, float *d_out)
{
    if (ctx->precision == MRAYGB_PRECISION_COMPENSATED_FF_MESE)
        CK(launch_prepare_ff(width * height, m, d_index, d_data, prediction_code, coding_warp, d_coding_params, bias,
                             d_out, ctx->stream),
           "prepare kernel launch");
    else
        CK(launch_prepare(width * height, m, d_index, d_data, prediction_code, coding_warp, d_coding_params, bias,
                          ctx->precision != MRAYGB_PRECISION_FP32, d_out, ctx->stream),
           "prepare kernel launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

// the differentiation form's FP32 preparation of W*H*m moments, keeping its arrays in ctx->diff_keep
int run_prepare_keep(mraygb_context *ctx, int width, int height, int m, const float *d_moments, float bias,
                     float *d_out)
{
    const size_t P = (size_t)width * (size_t)height;
    CK(ctx->diff_keep.reserve(P * 2 * (size_t)m * sizeof(float2)), "preparation buffer allocation");
    CK(launch_prepare_keep((int)P, m, d_moments, bias, d_out, ctx->diff_keep.as<float2>(), ctx->stream),
       "prepare kernel launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

int run_reconstruct(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp, int width,
                    int height, int m, const float dmin[3], const float dmax[3], const uint32_t *d_index,
                    const float *d_pm, const uint16_t *d_bounds, float *d_rgba, uint8_t *d_rgba8,
                    const float4 *d_bounds4 = nullptr, const float4 *d_tf = nullptr, int diff_form = 0)
{
    const DeviceCamera dc = to_device_camera(*cam);
    ReconArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.m = m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = dmin[i];
        a.dmax[i] = dmax[i];
    }
    a.index = d_index;
    a.pmoments = d_pm;
    a.bounds = d_bounds;
    a.tf = d_tf ? d_tf : ctx->tf.as<float4>();
    a.bounds4 = d_bounds4;
    a.diff_form = diff_form;
    a.diff_tf_linear = diff_form && ctx->diff_tf_sampling == MRAYGB_DIFF_TF_LINEAR;
    a.step = rp->step_size;
    a.emission = rp->medium_emission;
    a.ert = rp->early_ray_termination;
    a.rgba = d_rgba;
    a.rgba8 = d_rgba8;
    GridView cache;
    if (!diff_form && rp->ss.enable && rp->medium_scattering > 0.0f && ctx->has_ss_cache)
    {
        cache = ss_cache_view(ctx);
        a.ss_cache = &cache;
        a.ss = &rp->ss;
        a.scattering = rp->medium_scattering;
    }
    CK(launch_reconstruct(a, ctx->error_flag.as<int>(), ctx->stream), "reconstruct kernel launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

int run_prediction_encode(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index, float *d_data,
                          uint64_t data_size, int coding_warp, float bias, uint16_t *d_coding_params)
{
    const int P = width * height;
    CK(launch_prediction_encode(P, m, d_index, d_data, bias, ctx->stream), "prediction encode launch");
    ctx->launches += 1;
    CK(ctx->coding_params_f.reserve(2 * (size_t)m * sizeof(float)), "coding parameter allocation");
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
    {
        if (m > 1)
        {
            const int blocks = coding_minmax_blocks(P);
            CK(ctx->coding_partial.reserve((size_t)blocks * (size_t)(m - 1) * sizeof(float2)), "partial allocation");
            CK(launch_coding_params(P, m, d_index, d_data, data_size, ctx->coding_partial.as<float2>(),
                                    d_coding_params, ctx->coding_params_f.as<float>(), ctx->stream),
               "coding parameter launch");
            ctx->launches += 2;
        }
    }
    if (m > 1)
    {
        CK(launch_coding_warp(P, d_index, d_data, coding_warp, ctx->coding_params_f.as<float>(), ctx->stream),
           "coding warp launch");
        ctx->launches += 1;
    }
    return MRAYGB_OK;
}

// bit counts per index (table) and their prefix sums, uploaded to the context; returns the table pointers
int upload_table(mraygb_context *ctx, int m, const uint8_t *h_table, const uint8_t **d_table,
                 const uint32_t **d_prefix)
{
    if (!h_table)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "quantization table is NULL");
    uint8_t host[256 + 4 * 257];
    std::memset(host, 0, sizeof(host));
    uint32_t prefix[257];
    prefix[0] = 0;
    for (int l = 0; l < m; ++l)
    {
        if (h_table[l] < 1 || h_table[l] > 32)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "quantization table entry %d is %d bits (1..32)", l,
                        (int)h_table[l]);
        host[l] = h_table[l];
        prefix[l + 1] = prefix[l] + h_table[l];
    }
    std::memcpy(host + 256, prefix, sizeof(uint32_t) * (size_t)(m + 1));
    CK(ctx->table.reserve(sizeof(host)), "table allocation");
    CK(cudaMemcpyAsync(ctx->table.ptr, host, sizeof(host), cudaMemcpyHostToDevice, ctx->stream), "table upload");
    *d_table = ctx->table.as<uint8_t>();
    *d_prefix = reinterpret_cast<const uint32_t *>(ctx->table.as<uint8_t>() + 256);
    return MRAYGB_OK;
}

// per-pixel bit offsets of the packed stream; *total_bits is read back to the host
int run_bit_offsets(mraygb_context *ctx, int P, const uint32_t *d_index, const uint32_t *d_prefix,
                    uint64_t *total_bits)
{
    CK(ctx->bits.reserve((size_t)P * sizeof(unsigned long long)), "bit count allocation");
    CK(ctx->bit_offset.reserve(((size_t)P + 1) * sizeof(unsigned long long)), "bit offset allocation");
    const size_t words = scan_scratch_words((size_t)P);
    CK(ctx->scan_scratch64.reserve((words + 1) * sizeof(unsigned long long)), "scan scratch allocation");
    CK(launch_pixel_bits(P, d_index, d_prefix, ctx->bits.as<unsigned long long>(), ctx->stream), "bit count launch");
    ctx->launches += 1;
    int launches = 0;
    CK(launch_exclusive_scan_u64(ctx->bits.as<unsigned long long>(), ctx->bit_offset.as<unsigned long long>(),
                                 (size_t)P, ctx->scan_scratch64.as<unsigned long long>(), ctx->stream, &launches),
       "bit offset scan");
    ctx->launches += (uint64_t)launches;
    unsigned long long tb = 0;
    CK(cudaMemcpyAsync(&tb, ctx->bit_offset.as<unsigned long long>() + P, sizeof(tb), cudaMemcpyDeviceToHost,
                       ctx->stream),
       "reading the bit count");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    *total_bits = tb;
    return MRAYGB_OK;
}

int run_quantize(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index, const float *d_data,
                 const uint8_t *h_table, uint8_t *d_out, uint64_t capacity, uint64_t *h_nbytes)
{
    const int P = width * height;
    const uint8_t *d_table;
    const uint32_t *d_prefix;
    int rc = upload_table(ctx, m, h_table, &d_table, &d_prefix);
    if (rc)
        return rc;
    uint64_t total_bits = 0;
    if ((rc = run_bit_offsets(ctx, P, d_index, d_prefix, &total_bits)))
        return rc;
    const uint64_t nbytes = total_bits / 8; // pack_bits emits whole bytes only
    const uint64_t word_bytes = ((total_bits + 31) / 32) * 4;
    if (capacity < word_bytes)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "packed buffer holds %llu bytes, %llu needed",
                    (unsigned long long)capacity, (unsigned long long)word_bytes);
    if (word_bytes)
        CK(cudaMemsetAsync(d_out, 0, word_bytes, ctx->stream), "clearing the packed buffer");
    CK(launch_pack(P, d_index, d_data, d_table, d_prefix, ctx->bit_offset.as<unsigned long long>(),
                   reinterpret_cast<uint32_t *>(d_out), ctx->stream),
       "pack launch");
    ctx->launches += 1;
    *h_nbytes = nbytes;
    return MRAYGB_OK;
}

// the moment image of a drop-in call on the device: data into ctx->compact, index / bounds / coding parameters when
// given; pointers to the device copies (null where the image has none)
int upload_moment_image(mraygb_context *ctx, int width, int height, int m, const uint32_t *h_index,
                        const float *h_data, uint64_t data_size, const uint16_t *h_bounds, int prediction_code,
                        int coding_warp, const uint16_t *h_coding_params, const uint32_t **d_index,
                        const uint16_t **d_bounds, const uint16_t **d_cp)
{
    const size_t P = (size_t)width * (size_t)height;
    if (!h_data)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL moment data");
    if (!h_index && data_size < P * (size_t)m)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "a non-compact image needs W*H*m floats");
    if (prediction_code && coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && !h_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction-coded moments need their coding parameters");
    const size_t nd = data_size ? data_size : 1;
    CK(ctx->compact.reserve(nd * sizeof(float)), "moment buffer allocation");
    CK(ctx->pmoments.reserve(nd * sizeof(float)), "multiplier buffer allocation");
    if (data_size)
        CK(cudaMemcpyAsync(ctx->compact.ptr, h_data, data_size * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
           "moment upload");
    *d_index = nullptr;
    if (h_index)
    {
        CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
        CK(cudaMemcpyAsync(ctx->index.ptr, h_index, (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
           "index upload");
        *d_index = ctx->index.as<uint32_t>();
    }
    *d_bounds = nullptr;
    if (h_bounds)
    {
        CK(ctx->bounds.reserve(2 * P * sizeof(uint16_t)), "bounds buffer allocation");
        CK(cudaMemcpyAsync(ctx->bounds.ptr, h_bounds, 2 * P * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->stream),
           "bounds upload");
        *d_bounds = ctx->bounds.as<uint16_t>();
    }
    *d_cp = nullptr;
    if (prediction_code && coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
    {
        CK(ctx->coding_params.reserve(2 * (size_t)m * sizeof(uint16_t)), "coding parameter allocation");
        CK(cudaMemcpyAsync(ctx->coding_params.ptr, h_coding_params, 2 * (size_t)(m - 1) * sizeof(uint16_t),
                           cudaMemcpyHostToDevice, ctx->stream),
           "coding parameter upload");
        *d_cp = ctx->coding_params.as<uint16_t>();
    }
    return MRAYGB_OK;
}

int validate_error_params(mraygb_context *ctx, const mraygb_error_params *ep)
{
    if (!ep)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "error parameters are NULL");
    if (!(ep->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)ep->step_size);
    if (ep->error_type < MRAYGB_ERROR_MAX || ep->error_type > MRAYGB_ERROR_PERCENTILE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown error type %d", ep->error_type);
    if (ep->error_type == MRAYGB_ERROR_PERCENTILE && (ep->error_percentile < 1 || ep->error_percentile > 99))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "error_percentile %d outside 1..99", ep->error_percentile);
    if (ctx->volume == mraygb_context::NONE)
        return fail(ctx, MRAYGB_NO_VOLUME, "no volume uploaded");
    return MRAYGB_OK;
}

// the error measure per pixel over the resident volume
int run_error_bounds(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_error_params *ep, int width,
                     int height, int m, const uint32_t *d_index, const float *d_pm, const uint16_t *d_bounds,
                     uint16_t *d_error_bounds, float *d_errors)
{
    const DeviceCamera dc = to_device_camera(*cam);
    ErrorArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.m = m;
    a.index = d_index;
    a.pmoments = d_pm;
    a.bounds = d_bounds;
    a.step = ep->step_size;
    a.data_min = ep->data_min;
    a.data_max = ep->data_max;
    a.percentile = ep->error_percentile;
    a.error_bounds = d_error_bounds;
    a.errors = d_errors;
    if (ctx->volume == mraygb_context::PARTICLES && ctx->particle_wendland)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "error bounds over particles with per-particle smoothing lengths");
    if (ctx->volume == mraygb_context::PARTICLES)
        CK(launch_error_bounds_particles(particle_view(ctx), a, ep->error_type, ctx->error_flag.as<int>(), ctx->stream),
           "error bound launch");
    else
        CK(launch_error_bounds_grid(grid_view(ctx), a, ep->error_type, ctx->error_flag.as<int>(), ctx->stream),
           "error bound launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

int validate_uncertainty(mraygb_context *ctx, const mraygb_uncertainty_params *up, int mode)
{
    if (!up)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "uncertainty parameters are NULL");
    const mraygb_reconstruction_params *rp = &up->rec;
    if (!(rp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)rp->step_size);
    if (rp->use_truncated_fourier)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "truncated Fourier reconstruction is not part of this path");
    if (rp->ss.enable && rp->medium_scattering > 0.0f)
        return fail(ctx, MRAYGB_NOT_SUPPORTED,
                    "uncertainty rendering with single scattering (the reference marches the light's moment image, "
                    "not the cache) is not supported");
    if (mode != 0 && mode != 1)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "mode %d: 0 = interpolation, 1 = convolution", mode);
    if (mode == 0 && !ctx->has_tf)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no transfer function uploaded");
    if (mode == 1 && !ctx->has_unc_table)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no uncertainty transfer function uploaded");
    return MRAYGB_OK;
}

int run_uncertainty(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_uncertainty_params *up, int mode,
                    int width, int height, int m, const float dmin[3], const float dmax[3], const uint32_t *d_index,
                    const float *d_pm, const uint16_t *d_bounds, const uint16_t *d_error_bounds, float *d_rgba,
                    uint8_t *d_rgba8)
{
    const DeviceCamera dc = to_device_camera(*cam);
    UncertaintyArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.m = m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = dmin[i];
        a.dmax[i] = dmax[i];
    }
    a.index = d_index;
    a.pmoments = d_pm;
    a.bounds = d_bounds;
    a.error_bounds = d_error_bounds;
    a.tf = ctx->tf.as<float4>();
    a.table = ctx->unc_table.as<float4>();
    a.step = up->rec.step_size;
    a.emission = up->rec.medium_emission;
    a.ert = up->rec.early_ray_termination;
    a.interp = up->bound_interpolation;
    a.mode = mode;
    a.error_type = up->error_type;
    a.rgba = d_rgba;
    a.rgba8 = d_rgba8;
    CK(launch_uncertainty(a, ctx->error_flag.as<int>(), ctx->stream), "uncertainty launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

int validate_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp)
{
    if (!cam || !rp)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL camera or parameters");
    if (!(rp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)rp->step_size);
    if (rp->ss.enable && !(rp->ss.step_size_factor > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "single-scattering step_size_factor must be > 0 (got %g)",
                    (double)rp->ss.step_size_factor);
    if (ctx->volume == mraygb_context::NONE)
        return fail(ctx, MRAYGB_NO_VOLUME, "no volume uploaded");
    if (!ctx->has_tf)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no transfer function uploaded");
    return MRAYGB_OK;
}

int run_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp, int width,
                  int height, float *d_rgba, uint8_t *d_rgba8, bool use_cache = false)
{
    const DeviceCamera dc = to_device_camera(*cam);
    ReferenceArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.rp = rp;
    a.tf = ctx->tf.as<float4>();
    a.rgba = d_rgba;
    a.rgba8 = d_rgba8;
    const GridView cache = ss_cache_view(ctx);
    if (use_cache)
        a.ss_cache = &cache;
    if (ctx->volume == mraygb_context::PARTICLES && ctx->particle_wendland)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "the reference renderer over particles with per-particle smoothing lengths");
    if (ctx->volume == mraygb_context::PARTICLES)
        CK(launch_reference_particles(particle_view(ctx), a, ctx->error_flag.as<int>(), ctx->stream),
           "reference launch");
    else
        CK(launch_reference_grid(grid_view(ctx), a, ctx->error_flag.as<int>(), ctx->stream), "reference launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

// the single-scattering block of a reconstruction: only the cached form, and only with a cache built or uploaded
int validate_rec_ss(mraygb_context *ctx, const mraygb_reconstruction_params *rp)
{
    if (!rp->ss.enable || !(rp->medium_scattering > 0.0f))
        return MRAYGB_OK;
    if (!rp->ss.use_cache)
        return fail(ctx, MRAYGB_NOT_SUPPORTED,
                    "single scattering marched through the light's moment image (ss.use_cache = 0) is not supported; "
                    "use the transmittance cache");
    if (!ctx->has_ss_cache)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT,
                    "single scattering needs a transmittance cache (mraygb_reconstruct_single_scattering_cache or "
                    "mraygb_upload_single_scattering_cache)");
    return MRAYGB_OK;
}

int validate_rec(mraygb_context *ctx, const mraygb_reconstruction_params *rp)
{
    if (!rp)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "reconstruction parameters are NULL");
    if (!(rp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)rp->step_size);
    if (rp->use_truncated_fourier)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "truncated Fourier reconstruction is not part of this path");
    if (!ctx->has_tf)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no transfer function uploaded");
    return validate_rec_ss(ctx, rp);
}

} // namespace

extern "C" {

int mraygb_create(int device, mraygb_context **out)
{
    if (!out)
        return MRAYGB_INVALID_ARGUMENT;
    *out = nullptr;
    mraygb_context *ctx = new (std::nothrow) mraygb_context();
    if (!ctx)
        return MRAYGB_OUT_OF_MEMORY;
    ctx->device = device;
    int rc = MRAYGB_OK;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = mese_init_constants();
    if (e == cudaSuccess)
        e = ctx->error_flag.reserve(sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemset(ctx->error_flag.ptr, 0, sizeof(int));
    if (e != cudaSuccess)
    {
        rc = e == cudaErrorMemoryAllocation ? MRAYGB_OUT_OF_MEMORY : MRAYGB_CUDA_ERROR;
        mraygb_destroy(ctx);
        return rc;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return MRAYGB_OK;
}

void mraygb_destroy(mraygb_context *ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    release_grid(ctx);
    release_ss_cache(ctx);
    DeviceBuffer *bufs[] = {&ctx->particle_pts, &ctx->particle_cells,
                            &ctx->tf,       &ctx->moments,       &ctx->counts,
                            &ctx->index,   &ctx->compact,  &ctx->bounds,        &ctx->coding_params,
                            &ctx->pmoments, &ctx->rgba,    &ctx->rgba8,         &ctx->scan_scratch,
                            &ctx->error_flag, &ctx->coding_partial, &ctx->coding_params_f, &ctx->table,
                            &ctx->bits,    &ctx->bit_offset, &ctx->scan_scratch64, &ctx->packed,
                            &ctx->adj_lambda, &ctx->adj_bounds, &ctx->diff_keep, &ctx->qc_scratch, &ctx->qc_means,
                            &ctx->qc_index, &ctx->qc_data, &ctx->error_bounds, &ctx->errors, &ctx->unc_table,
                            &ctx->unc_tf1d, &ctx->ss_keys, &ctx->ss_linear, &ctx->file_codes};
    for (DeviceBuffer *b : bufs)
        b->release();
    if (ctx->own_stream)
        cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char *mraygb_last_error(const mraygb_context *ctx) { return ctx ? ctx->error.c_str() : "null context"; }

int mraygb_set_stream(mraygb_context *ctx, void *stream)
{
    CHECK_CTX();
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return MRAYGB_OK;
}

void *mraygb_get_stream(const mraygb_context *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

int mraygb_synchronize(mraygb_context *ctx)
{
    CHECK_CTX();
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

int mraygb_set_precision(mraygb_context *ctx, int precision)
{
    CHECK_CTX();
    if (precision != MRAYGB_PRECISION_FP32 && precision != MRAYGB_PRECISION_COMPENSATED_FP64_MESE &&
        precision != MRAYGB_PRECISION_COMPENSATED_FF_MESE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown precision form %d", precision);
    ctx->precision = precision;
    return MRAYGB_OK;
}

int mraygb_set_diff_tf_sampling(mraygb_context *ctx, int sampling)
{
    CHECK_CTX();
    if (sampling != MRAYGB_DIFF_TF_BSPLINE && sampling != MRAYGB_DIFF_TF_LINEAR)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown transfer-function sampling %d", sampling);
    ctx->diff_tf_sampling = sampling;
    return MRAYGB_OK;
}

uint64_t mraygb_kernel_launches(const mraygb_context *ctx) { return ctx ? ctx->launches : 0; }

int mraygb_upload_grid(mraygb_context *ctx, const float *data, int nx, int ny, int nz, const float dmin[3],
                       const float dmax[3], int data_on_device)
{
    CHECK_CTX();
    if (!data || !dmin || !dmax || nx <= 0 || ny <= 0 || nz <= 0)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "invalid grid (%p, %d x %d x %d)", (const void *)data, nx, ny, nz);
    if ((uint64_t)nx * (uint64_t)ny >= (1ull << 31))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "grid slices of %d x %d exceed the reference's int indexing", nx, ny);
    for (int i = 0; i < 3; ++i)
        if (!(dmax[i] > dmin[i]))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "empty domain along axis %d", i);
    int max3d[3] = {0, 0, 0};
    cudaDeviceGetAttribute(&max3d[0], cudaDevAttrMaxTexture3DWidth, ctx->device);
    cudaDeviceGetAttribute(&max3d[1], cudaDevAttrMaxTexture3DHeight, ctx->device);
    cudaDeviceGetAttribute(&max3d[2], cudaDevAttrMaxTexture3DDepth, ctx->device);
    if (nx > max3d[0] || ny > max3d[1] || nz > max3d[2])
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "grid %d x %d x %d exceeds the 3D texture limits %d x %d x %d", nx, ny,
                    nz, max3d[0], max3d[1], max3d[2]);
    // same dimensions: the array is reused
    if (!(ctx->grid_array && ctx->nx == nx && ctx->ny == ny && ctx->nz == nz))
    {
        release_grid(ctx);
        const cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
        CK(cudaMalloc3DArray(&ctx->grid_array, &desc, make_cudaExtent(nx, ny, nz)), "grid allocation");
        cudaResourceDesc res;
        std::memset(&res, 0, sizeof(res));
        res.resType = cudaResourceTypeArray;
        res.res.array.array = ctx->grid_array;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        CK(cudaCreateTextureObject(&ctx->grid_tex, &res, &td, nullptr), "grid texture");
    }
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<float *>(data), (size_t)nx * sizeof(float), nx, ny);
    cp.dstArray = ctx->grid_array;
    cp.extent = make_cudaExtent(nx, ny, nz);
    cp.kind = data_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(cudaMemcpy3DAsync(&cp, ctx->stream), "grid upload");
    ctx->nx = nx;
    ctx->ny = ny;
    ctx->nz = nz;
    for (int i = 0; i < 3; ++i)
    {
        ctx->dmin[i] = dmin[i];
        ctx->dmax[i] = dmax[i];
    }
    ctx->volume = mraygb_context::GRID;
    ctx->particle_pts.release();
    ctx->particle_cells.release();
    if (!data_on_device)
        CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

namespace
{

// the particle upload of both forms: one smoothing length h (hs == NULL, the reference's), or one per particle
// (hs, Wendland C2; the grid's cell size is then the largest of them)
int upload_particles(mraygb_context *ctx, const float *x, const float *y, const float *z, const float *v,
                     const float *hs, uint64_t n, float h, const float dmin[3], const float dmax[3],
                     int data_on_device)
{
    CHECK_CTX();
    if (!x || !y || !z || !v || !dmin || !dmax)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL particle array or domain");
    if (n == 0 || n > (1ull << 31))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "particle count %llu outside 1..2^31", (unsigned long long)n);
    if (!hs && (!(h > 0.f) || !std::isfinite(h)))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "smoothing length must be finite and > 0 (got %g)", (double)h);
    for (int i = 0; i < 3; ++i)
        if (!(dmax[i] > dmin[i]))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "empty domain along axis %d", i);

    // the buffers of a previous volume may be overwritten from here on; on failure no volume is resident
    ctx->volume = mraygb_context::NONE;

    // temporaries of the build, released at the end
    DeviceBuffer stage, keys, keys_alt, vals, vals_alt, counts, hist, hist_scan, minmax;
    struct Release
    {
        DeviceBuffer *b[9];
        ~Release()
        {
            for (DeviceBuffer *p : b)
                p->release();
        }
    } release{{&stage, &keys, &keys_alt, &vals, &vals_alt, &counts, &hist, &hist_scan, &minmax}};

    const int arrays = hs ? 5 : 4;
    const float *dx = x, *dy = y, *dz = z, *dv = v, *dh = hs;
    if (!data_on_device)
    {
        CK(stage.reserve(arrays * n * sizeof(float)), "particle staging allocation");
        float *s = stage.as<float>();
        const float *src[5] = {x, y, z, v, hs};
        for (int k = 0; k < arrays; ++k)
            CK(cudaMemcpyAsync(s + k * n, src[k], n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
               "particle upload");
        dx = s;
        dy = s + n;
        dz = s + 2 * n;
        dv = s + 3 * n;
        dh = hs ? s + 4 * n : nullptr;
    }
    if (dh)
    {
        // the largest smoothing length sets the cell size; every one must be finite and > 0
        CK(minmax.reserve(2 * sizeof(unsigned int)), "particle scratch allocation");
        CK(launch_particle_h_range(n, dh, minmax.as<unsigned int>(), ctx->stream), "smoothing length kernel");
        unsigned int hr[2];
        CK(cudaMemcpyAsync(hr, minmax.ptr, sizeof(hr), cudaMemcpyDeviceToHost, ctx->stream),
           "reading the smoothing lengths");
        CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        ctx->launches += 1;
        if (hr[1])
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "%u smoothing lengths are not finite and > 0", hr[1]);
        std::memcpy(&h, &hr[0], sizeof(float));
    }

    // 1. bounding box of the particles -> grid parameters (createGridFromDomain)
    const size_t mm_floats = particle_minmax_scratch_floats(n);
    CK(minmax.reserve((mm_floats + 6) * sizeof(float)), "particle scratch allocation");
    float *box_d = minmax.as<float>() + mm_floats;
    CK(launch_particle_minmax(dx, dy, dz, n, minmax.as<float>(), box_d, ctx->stream), "particle bounds kernel");
    float box[6];
    CK(cudaMemcpyAsync(box, box_d, sizeof(box), cudaMemcpyDeviceToHost, ctx->stream), "reading particle bounds");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    ctx->launches += 2;
    uint64_t cells = 1;
    for (int k = 0; k < 3; ++k)
    {
        const float c = (box[3 + k] - box[k]) / h + 1.0f;
        if (!std::isfinite(c) || c >= 16777216.f)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "particle extent / h = %g cells along axis %d", (double)c, k);
        cells *= (uint64_t)c + 4;
    }
    if (cells > (1ull << 30))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the particle grid needs about %llu cells (limit 2^30): h too small",
                    (unsigned long long)cells);
    const ParticleGridParams g = particle_grid_params(box, box + 3, h);
    const uint32_t total = g.total;

    // 2. cell of every particle, per-cell counts, CSR starts
    CK(keys.reserve(n * sizeof(uint32_t)), "particle key allocation");
    CK(counts.reserve((size_t)total * sizeof(uint32_t)), "particle cell count allocation");
    CK(ctx->particle_cells.reserve(((size_t)total + 1) * sizeof(uint32_t)), "particle cell allocation");
    CK(cudaMemsetAsync(counts.ptr, 0, (size_t)total * sizeof(uint32_t), ctx->stream), "clearing cell counts");
    CK(launch_particle_cells(dx, dy, dz, n, g, keys.as<uint32_t>(), counts.as<uint32_t>(), ctx->stream),
       "particle cell kernel");
    const size_t hw = particle_radix_hist_words((uint32_t)n);
    const size_t words = std::max(scan_scratch_words(total), scan_scratch_words(hw)) + 1;
    CK(ctx->scan_scratch.reserve(words * sizeof(uint32_t)), "scan scratch allocation");
    int launches = 1;
    CK(launch_exclusive_scan(counts.as<uint32_t>(), ctx->particle_cells.as<uint32_t>(), total,
                             ctx->scan_scratch.as<uint32_t>(), ctx->stream, &launches),
       "cell scan");

    // 3. stable sort by cell, 4. gather into (x, y, z, v) records
    CK(keys_alt.reserve(n * sizeof(uint32_t)), "particle key allocation");
    CK(vals.reserve(n * sizeof(uint32_t)), "particle index allocation");
    CK(vals_alt.reserve(n * sizeof(uint32_t)), "particle index allocation");
    CK(hist.reserve(hw * sizeof(uint32_t)), "radix histogram allocation");
    CK(hist_scan.reserve((hw + 1) * sizeof(uint32_t)), "radix histogram allocation");
    uint32_t *order = nullptr;
    CK(launch_particle_sort((uint32_t)n, total, keys.as<uint32_t>(), keys_alt.as<uint32_t>(), vals.as<uint32_t>(),
                            vals_alt.as<uint32_t>(), hist.as<uint32_t>(), hist_scan.as<uint32_t>(),
                            ctx->scan_scratch.as<uint32_t>(), &order, ctx->stream, &launches),
       "particle sort");
    CK(ctx->particle_pts.reserve(n * sizeof(float4)), "particle allocation");
    CK(launch_particle_gather(n, order, dx, dy, dz, dv, ctx->particle_pts.as<float4>(), ctx->stream),
       "particle gather kernel");
    launches += 1;
    if (dh)
    {
        CK(ctx->particle_inv_h.reserve(n * sizeof(float2)), "smoothing length allocation");
        CK(launch_particle_gather_h(n, order, dh, ctx->particle_inv_h.as<float2>(), ctx->stream),
           "smoothing length gather kernel");
        launches += 1;
    }
    else
    {
        ctx->particle_inv_h.release();
    }
    ctx->particle_wendland = dh != nullptr;
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    ctx->launches += (uint64_t)launches;

    ctx->particle_grid = g;
    ctx->num_particles = n;
    for (int i = 0; i < 3; ++i)
    {
        ctx->dmin[i] = dmin[i];
        ctx->dmax[i] = dmax[i];
    }
    ctx->volume = mraygb_context::PARTICLES;
    release_grid(ctx);
    return MRAYGB_OK;
}

} // namespace

int mraygb_upload_particles(mraygb_context *ctx, const float *x, const float *y, const float *z, const float *v,
                            uint64_t n, float h, const float dmin[3], const float dmax[3], int data_on_device)
{
    return upload_particles(ctx, x, y, z, v, nullptr, n, h, dmin, dmax, data_on_device);
}

int mraygb_upload_particles_h(mraygb_context *ctx, const float *x, const float *y, const float *z, const float *v,
                              const float *h, uint64_t n, const float dmin[3], const float dmax[3], int data_on_device)
{
    if (ctx && !h)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL smoothing length array");
    return upload_particles(ctx, x, y, z, v, h, n, 0.f, dmin, dmax, data_on_device);
}

int mraygb_upload_tf(mraygb_context *ctx, const float *table)
{
    CHECK_CTX();
    if (!table)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "transfer function table is NULL");
    CK(ctx->tf.reserve(256 * 4 * sizeof(float)), "transfer function allocation");
    CK(cudaMemcpyAsync(ctx->tf.ptr, table, 256 * 4 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
       "transfer function upload");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    ctx->has_tf = true;
    return MRAYGB_OK;
}

// ---- stage API ------------------------------------------------------------------------------------------------

int mraygb_stage_generate_moments(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                                  int width, int height, int m, float *d_moments, uint16_t *d_bounds,
                                  uint32_t *d_counts)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_gen(ctx, gp)))
        return rc;
    if (!cam || !d_moments)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "camera or moment buffer is NULL");
    if (ctx->volume == mraygb_context::NONE)
        return fail(ctx, MRAYGB_NO_VOLUME, "no volume uploaded");
    if (gp->compact_image && !d_counts)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "compact_image needs a count buffer");
    if (gp->transform_to_bounds && !d_bounds)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "transform_to_bounds needs a bounds buffer");
    return run_generate_moments(ctx, cam, gp, width, height, m, d_moments, d_bounds, d_counts);
}

int mraygb_stage_compact(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_counts,
                         const float *d_moments, uint32_t *d_index, float *d_compact, uint64_t capacity,
                         uint64_t *h_total)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!d_counts || !d_moments || !d_index || !d_compact)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL buffer");
    return run_compact(ctx, width, height, m, d_counts, d_moments, d_index, d_compact, capacity, h_total);
}

int mraygb_stage_prepare_moments(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index,
                                 const float *d_data, int prediction_code, int coding_warp,
                                 const uint16_t *d_coding_params, float bias, float *d_pmoments)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!d_data || !d_pmoments)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL buffer");
    if (prediction_code && coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && !d_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction-coded moments need their coding parameters");
    return run_prepare(ctx, width, height, m, d_index, d_data, prediction_code, coding_warp, d_coding_params, bias,
                       d_pmoments);
}

int mraygb_stage_reconstruct(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp,
                             int width, int height, int m, const float domain_min[3], const float domain_max[3],
                             const uint32_t *d_index, const float *d_pmoments, const uint16_t *d_bounds, float *d_rgba,
                             uint8_t *d_rgba8)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_rec(ctx, rp)))
        return rc;
    if (!cam || !d_pmoments || !domain_min || !domain_max || (!d_rgba && !d_rgba8))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    return run_reconstruct(ctx, cam, rp, width, height, m, domain_min, domain_max, d_index, d_pmoments, d_bounds,
                           d_rgba, d_rgba8);
}

int mraygb_measure_fp32_rate(mraygb_context *ctx, double *h_tflops)
{
    CHECK_CTX();
    if (!h_tflops)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "cudaDeviceGetAttribute");
    CK(ctx->pmoments.reserve(fp32_rate_scratch_floats(sms) * sizeof(float)), "scratch allocation");
    CK(measure_fp32_rate(sms, ctx->stream, ctx->pmoments.as<float>(), h_tflops), "FP32 rate kernel");
    ctx->launches += 2;
    return MRAYGB_OK;
}

int mraygb_stage_libm_sincosf(mraygb_context *ctx, const float *d_x, float *d_sin, float *d_cos, uint64_t n)
{
    CHECK_CTX();
    if (n > 0 && (!d_x || !d_sin || !d_cos))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    CK(launch_libm_sincosf(n, d_x, d_sin, d_cos, ctx->stream), "libm_sincosf");
    ctx->launches += n > 0 ? 1 : 0;
    return MRAYGB_OK;
}

int mraygb_stage_prediction_encode(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index,
                                   float *d_data, uint64_t data_size, int coding_warp, float bias,
                                   uint16_t *d_coding_params)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!d_index || !d_data)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction coding needs a compact image (index and data)");
    if (coding_warp != MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && coding_warp != MRAYGB_CODING_WARP_NONE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown coding_warp %d", coding_warp);
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && m > 1 && !d_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the default warp needs a coding parameter buffer");
    return run_prediction_encode(ctx, width, height, m, d_index, d_data, data_size, coding_warp, bias,
                                 d_coding_params);
}

int mraygb_stage_quantize_prediction_coding(mraygb_context *ctx, int width, int height, int m,
                                            const uint32_t *d_index, const float *d_data, const uint8_t *h_table,
                                            uint8_t *d_out, uint64_t capacity, uint64_t *h_nbytes)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!d_index || !d_data || !d_out || !h_nbytes)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    return run_quantize(ctx, width, height, m, d_index, d_data, h_table, d_out, capacity, h_nbytes);
}

int mraygb_stage_dequantize_prediction_coding(mraygb_context *ctx, int width, int height, int m,
                                              const uint32_t *d_index, const uint8_t *h_table,
                                              const uint8_t *d_bytes, uint64_t num_bytes, float *d_data)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!d_index || !d_data || (!d_bytes && num_bytes))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const int P = width * height;
    const uint8_t *d_table;
    const uint32_t *d_prefix;
    if ((rc = upload_table(ctx, m, h_table, &d_table, &d_prefix)))
        return rc;
    uint64_t total_bits = 0;
    if ((rc = run_bit_offsets(ctx, P, d_index, d_prefix, &total_bits)))
        return rc;
    CK(launch_unpack(P, d_index, d_table, d_prefix, ctx->bit_offset.as<unsigned long long>(), d_bytes, num_bytes,
                     d_data, ctx->stream),
       "unpack launch");
    ctx->launches += 1;
    return MRAYGB_OK;
}

// ---- quantization curve ---------------------------------------------------------------------------------------

namespace
{

int check_quant_table_args(mraygb_context *ctx, int width, int height, int m, int coding_warp, int start_bits,
                           uint8_t *h_table)
{
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (m < 2)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the quantization table needs num_moments >= 2 (got %d)", m);
    if (start_bits < 1 || start_bits > 31)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "start_bits %d outside 1..31", start_bits);
    if (coding_warp != MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && coding_warp != MRAYGB_CODING_WARP_NONE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown coding warp %d", coding_warp);
    if (!h_table)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL table");
    return MRAYGB_OK;
}

// sample_moment_image's size as main.cpp:320-322 chooses it
int sample_shape(mraygb_context *ctx, int width, int height, int sampling, int *sx, int *sy)
{
    if (sampling <= 0)
    {
        *sx = width;
        *sy = height;
        return MRAYGB_OK;
    }
    const int w = std::min(width, sampling), h = std::min(height, sampling);
    if (w != h)
        return fail(ctx, MRAYGB_NOT_SUPPORTED,
                    "sample_moment_image of a %dx%d image at %d gives a %dx%d sample, which the reference indexes "
                    "as %dx%d; only square samples are defined",
                    width, height, sampling, w, h, h, w);
    *sx = w;
    *sy = h;
    return MRAYGB_OK;
}

// the error means of every reachable (index, bits) pair on the device, then create_quantization_table's search
// (measure_coding_error.cpp:400-435) over them
int run_quant_table(mraygb_context *ctx, int width, int height, int m, const uint32_t *d_index, const float *d_data,
                    int coding_warp, const uint16_t *d_coding_params, int sx, int sy, int start_bits,
                    uint8_t *h_table, float *h_means)
{
    const int bmin = std::min(2, start_bits), nb = start_bits - bmin + 1;
    const size_t P = (size_t)sx * (size_t)sy;
    // the per-pixel errors of one pass stay within 1 GiB
    const size_t row_bytes = (size_t)nb * P * sizeof(float);
    const size_t rows = std::max<size_t>(1, std::min<size_t>((size_t)(m - 1), (size_t(1) << 30) / row_bytes));
    CK(ctx->qc_scratch.reserve(quant_curve_scratch_bytes(sx, sy, m, nb, rows)), "quantization curve scratch");
    CK(ctx->qc_means.reserve((size_t)(m - 1) * nb * sizeof(float)), "quantization curve means");
    int launches = 0;
    CK(launch_quant_curve(width, height, m, d_index, d_data, coding_warp,
                          coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED ? d_coding_params : nullptr, sx, sy,
                          bmin, nb, rows, ctx->qc_scratch.ptr, ctx->qc_means.as<float>(), ctx->stream, &launches),
       "quantization curve launch");
    ctx->launches += launches;
    std::vector<float> means((size_t)(m - 1) * nb);
    CK(cudaMemcpyAsync(means.data(), ctx->qc_means.ptr, means.size() * sizeof(float), cudaMemcpyDeviceToHost,
                       ctx->stream),
       "means download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    auto mean = [&](int idx, int b) { return means[(size_t)(idx - 1) * nb + (b - bmin)]; };
    h_table[0] = 16;
    h_table[1] = (uint8_t)start_bits;
    const int minimum_bits = 2;
    const float threshold = mean(1, start_bits);
    for (int idx = 2; idx < m; ++idx)
    {
        h_table[idx] = h_table[idx - 1];
        for (int b = h_table[idx - 1]; b >= minimum_bits; --b)
        {
            if (mean(idx, b) >= threshold)
                break;
            h_table[idx] = (uint8_t)b;
        }
    }
    if (h_means)
    {
        std::fill(h_means, h_means + (size_t)m * 32, NAN);
        for (int idx = 1; idx < m; ++idx)
            for (int b = bmin; b <= start_bits; ++b)
                h_means[idx * 32 + b] = mean(idx, b);
    }
    return MRAYGB_OK;
}

} // namespace

int mraygb_stage_create_quantization_table(mraygb_context *ctx, int width, int height, int m,
                                           const uint32_t *d_index, const float *d_data, int coding_warp,
                                           const uint16_t *d_coding_params, int start_bits, int sampling,
                                           uint8_t *h_table, float *h_means)
{
    CHECK_CTX();
    int rc = check_quant_table_args(ctx, width, height, m, coding_warp, start_bits, h_table);
    if (rc)
        return rc;
    if (!d_index || !d_data)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the quantization curve needs a compact image (index and data)");
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && !d_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the default coding warp needs the coding parameters");
    int sx, sy;
    if ((rc = sample_shape(ctx, width, height, sampling, &sx, &sy)))
        return rc;
    return run_quant_table(ctx, width, height, m, d_index, d_data, coding_warp, d_coding_params, sx, sy, start_bits,
                           h_table, h_means);
}

// ---- drop-in host API -------------------------------------------------------------------------------------------

int mraygb_create_quantization_table(mraygb_context *ctx, int width, int height, int m, const uint32_t *h_index,
                                     const float *h_data, uint64_t data_size, int coding_warp,
                                     const uint16_t *h_coding_params, int start_bits, int sampling, uint8_t *h_table,
                                     float *h_means)
{
    CHECK_CTX();
    int rc = check_quant_table_args(ctx, width, height, m, coding_warp, start_bits, h_table);
    if (rc)
        return rc;
    if (!h_index || (!h_data && data_size))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the quantization curve needs a compact image (index and data)");
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && !h_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the default coding warp needs the coding parameters");
    int sx, sy;
    if ((rc = sample_shape(ctx, width, height, sampling, &sx, &sy)))
        return rc;
    // sample on the host (moment_image_sample.h:33-62 and MomentImageHost::compact) and move only the sample
    const int fx = width / sx, fy = height / sy;
    const size_t P = (size_t)sx * (size_t)sy;
    std::vector<uint32_t> s_index(P + 1);
    uint64_t total = 0;
    for (int y = 0; y < sy; ++y)
        for (int x = 0; x < sx; ++x)
        {
            const size_t src = (size_t)(y * fy) * (size_t)width + (size_t)(x * fx);
            const uint32_t off = h_index[src], n = h_index[src + 1] - off;
            if (h_index[src + 1] < off || n > (uint32_t)m || (uint64_t)off + n > data_size)
                return fail(ctx, MRAYGB_INVALID_ARGUMENT, "pixel (%d, %d): moments [%u, %u) outside the %llu values",
                            x * fx, y * fy, off, off + n, (unsigned long long)data_size);
            s_index[(size_t)y * sx + x] = (uint32_t)total;
            total += n;
        }
    s_index[P] = (uint32_t)total;
    std::vector<float> s_data(total ? total : 1);
    for (size_t s = 0; s < P; ++s)
    {
        const int x = (int)(s % sx), y = (int)(s / sx);
        const size_t src = (size_t)(y * fy) * (size_t)width + (size_t)(x * fx);
        std::memcpy(s_data.data() + s_index[s], h_data + h_index[src], (s_index[s + 1] - s_index[s]) * sizeof(float));
    }
    CK(ctx->qc_index.reserve((P + 1) * sizeof(uint32_t)), "sample index buffer");
    CK(ctx->qc_data.reserve(s_data.size() * sizeof(float)), "sample data buffer");
    CK(cudaMemcpyAsync(ctx->qc_index.ptr, s_index.data(), (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       ctx->stream),
       "sample index upload");
    CK(cudaMemcpyAsync(ctx->qc_data.ptr, s_data.data(), s_data.size() * sizeof(float), cudaMemcpyHostToDevice,
                       ctx->stream),
       "sample data upload");
    const uint16_t *d_cp = nullptr;
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
    {
        CK(ctx->coding_params.reserve(2 * (size_t)(m - 1) * sizeof(uint16_t)), "coding parameter buffer");
        CK(cudaMemcpyAsync(ctx->coding_params.ptr, h_coding_params, 2 * (size_t)(m - 1) * sizeof(uint16_t),
                           cudaMemcpyHostToDevice, ctx->stream),
           "coding parameter upload");
        d_cp = ctx->coding_params.as<uint16_t>();
    }
    return run_quant_table(ctx, sx, sy, m, ctx->qc_index.as<uint32_t>(), ctx->qc_data.as<float>(), coding_warp, d_cp,
                           sx, sy, start_bits, h_table, h_means);
}


int mraygb_quantize_prediction_coding(mraygb_context *ctx, int width, int height, int m, const uint32_t *h_index,
                                      const float *h_data, uint64_t data_size, const uint8_t *h_table,
                                      uint8_t *h_out, uint64_t capacity, uint64_t *h_nbytes)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!h_index || (!h_data && data_size) || !h_nbytes)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const size_t P = (size_t)width * (size_t)height;
    const size_t nd = data_size ? data_size : 1;
    CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
    CK(ctx->compact.reserve(nd * sizeof(float)), "moment buffer allocation");
    CK(cudaMemcpyAsync(ctx->index.ptr, h_index, (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
       "index upload");
    if (data_size)
        CK(cudaMemcpyAsync(ctx->compact.ptr, h_data, data_size * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
           "moment upload");
    // upper bound of the packed size: 32 bits per value
    const uint64_t cap = (uint64_t)nd * 4 + 8;
    CK(ctx->packed.reserve(cap), "packed buffer allocation");
    uint64_t nbytes = 0;
    rc = run_quantize(ctx, width, height, m, ctx->index.as<uint32_t>(), ctx->compact.as<float>(), h_table,
                      ctx->packed.as<uint8_t>(), cap, &nbytes);
    if (rc)
        return rc;
    *h_nbytes = nbytes;
    if (h_out)
    {
        if (capacity < nbytes)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "output holds %llu bytes, %llu needed",
                        (unsigned long long)capacity, (unsigned long long)nbytes);
        if (nbytes)
            CK(cudaMemcpyAsync(h_out, ctx->packed.ptr, nbytes, cudaMemcpyDeviceToHost, ctx->stream), "packed download");
    }
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

int mraygb_dequantize_prediction_coding(mraygb_context *ctx, int width, int height, int m, const uint32_t *h_index,
                                        const uint8_t *h_table, const uint8_t *h_bytes, uint64_t num_bytes,
                                        float *h_data, uint64_t data_size)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if (!h_index || !h_table || (!h_bytes && num_bytes) || (!h_data && data_size))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const size_t P = (size_t)width * (size_t)height;
    if ((uint64_t)h_index[P] != data_size)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "data_size %llu differs from the index's total %u",
                    (unsigned long long)data_size, h_index[P]);
    CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
    CK(ctx->compact.reserve((data_size ? data_size : 1) * sizeof(float)), "moment buffer allocation");
    CK(ctx->packed.reserve(num_bytes ? num_bytes : 1), "packed buffer allocation");
    CK(cudaMemcpyAsync(ctx->index.ptr, h_index, (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
       "index upload");
    if (num_bytes)
        CK(cudaMemcpyAsync(ctx->packed.ptr, h_bytes, num_bytes, cudaMemcpyHostToDevice, ctx->stream),
           "packed upload");
    if ((rc = mraygb_stage_dequantize_prediction_coding(ctx, width, height, m, ctx->index.as<uint32_t>(), h_table,
                                                        ctx->packed.as<uint8_t>(), num_bytes,
                                                        ctx->compact.as<float>())))
        return rc;
    if (data_size)
        CK(cudaMemcpyAsync(h_data, ctx->compact.ptr, data_size * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "moment download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

int mraygb_generate(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp, int width,
                    int height, int m, float *h_data, uint32_t *h_index, uint16_t *h_bounds, uint16_t *h_coding_params,
                    uint64_t *h_data_size)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_gen(ctx, gp)))
        return rc;
    if (!cam || !h_data || !h_data_size)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "camera, data or size pointer is NULL");
    if (gp->compact_image && !h_index)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "compact_image needs an index buffer");
    if (gp->transform_to_bounds && !h_bounds)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "transform_to_bounds needs a bounds buffer");
    if (ctx->volume == mraygb_context::NONE)
        return fail(ctx, MRAYGB_NO_VOLUME, "no volume uploaded");
    if (gp->prediction_coding && gp->coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && m > 1 &&
        !h_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction coding with the default warp needs a coding "
                                                  "parameter buffer");

    const size_t P = (size_t)width * (size_t)height;
    const size_t N = P * (size_t)m;
    CK(ctx->moments.reserve(N * sizeof(float)), "moment buffer allocation");
    CK(ctx->counts.reserve(P * sizeof(uint32_t)), "count buffer allocation");
    CK(ctx->bounds.reserve(2 * P * sizeof(uint16_t)), "bounds buffer allocation");
    rc = run_generate_moments(ctx, cam, gp, width, height, m, ctx->moments.as<float>(), ctx->bounds.as<uint16_t>(),
                              ctx->counts.as<uint32_t>());
    if (rc)
        return rc;
    const float *d_out = ctx->moments.as<float>();
    uint64_t size = N;
    if (gp->compact_image)
    {
        CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
        CK(ctx->compact.reserve(N * sizeof(float)), "compact buffer allocation");
        rc = run_compact(ctx, width, height, m, ctx->counts.as<uint32_t>(), ctx->moments.as<float>(),
                         ctx->index.as<uint32_t>(), ctx->compact.as<float>(), N, &size);
        if (rc)
            return rc;
        d_out = ctx->compact.as<float>();
        if (gp->prediction_coding)
        {
            CK(ctx->coding_params.reserve(2 * (size_t)m * sizeof(uint16_t)), "coding parameter allocation");
            rc = run_prediction_encode(ctx, width, height, m, ctx->index.as<uint32_t>(), ctx->compact.as<float>(),
                                       size, gp->coding_warp, gp->bias, ctx->coding_params.as<uint16_t>());
            if (rc)
                return rc;
            if (gp->coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && m > 1)
                CK(cudaMemcpyAsync(h_coding_params, ctx->coding_params.ptr, 2 * (size_t)(m - 1) * sizeof(uint16_t),
                                   cudaMemcpyDeviceToHost, ctx->stream),
                   "coding parameter download");
        }
        CK(cudaMemcpyAsync(h_index, ctx->index.ptr, (P + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream),
           "index download");
    }
    if (size)
        CK(cudaMemcpyAsync(h_data, d_out, size * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "moment download");
    if (gp->transform_to_bounds)
        CK(cudaMemcpyAsync(h_bounds, ctx->bounds.ptr, 2 * P * sizeof(uint16_t), cudaMemcpyDeviceToHost, ctx->stream),
           "bounds download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    *h_data_size = size;
    return check_device_error_flag(ctx);
}

int mraygb_reconstruct(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp,
                       int width, int height, int m, const float domain_min[3], const float domain_max[3],
                       const uint32_t *h_index, const float *h_data, uint64_t data_size, const uint16_t *h_bounds,
                       int prediction_code, int coding_warp, const uint16_t *h_coding_params, float *h_rgba,
                       uint8_t *h_rgba8)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_rec(ctx, rp)))
        return rc;
    if (!cam || !h_data || !domain_min || !domain_max || (!h_rgba && !h_rgba8))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const size_t P = (size_t)width * (size_t)height;
    if (!h_index && data_size < P * (size_t)m)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "a non-compact image needs W*H*m floats");
    if (prediction_code && coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED && !h_coding_params)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction-coded moments need their coding parameters");

    const size_t nd = data_size ? data_size : 1;
    CK(ctx->compact.reserve(nd * sizeof(float)), "moment buffer allocation");
    CK(ctx->pmoments.reserve(nd * sizeof(float)), "multiplier buffer allocation");
    CK(ctx->rgba.reserve(P * 4 * sizeof(float)), "colour buffer allocation");
    if (h_rgba8)
        CK(ctx->rgba8.reserve(P * 4), "u8 colour buffer allocation");
    if (data_size)
        CK(cudaMemcpyAsync(ctx->compact.ptr, h_data, data_size * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
           "moment upload");
    const uint32_t *d_index = nullptr;
    if (h_index)
    {
        CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
        CK(cudaMemcpyAsync(ctx->index.ptr, h_index, (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
           "index upload");
        d_index = ctx->index.as<uint32_t>();
    }
    const uint16_t *d_bounds = nullptr;
    if (h_bounds)
    {
        CK(ctx->bounds.reserve(2 * P * sizeof(uint16_t)), "bounds buffer allocation");
        CK(cudaMemcpyAsync(ctx->bounds.ptr, h_bounds, 2 * P * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->stream),
           "bounds upload");
        d_bounds = ctx->bounds.as<uint16_t>();
    }
    const uint16_t *d_cp = nullptr;
    if (prediction_code && coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
    {
        CK(ctx->coding_params.reserve(2 * (size_t)m * sizeof(uint16_t)), "coding parameter allocation");
        CK(cudaMemcpyAsync(ctx->coding_params.ptr, h_coding_params, 2 * (size_t)(m - 1) * sizeof(uint16_t),
                           cudaMemcpyHostToDevice, ctx->stream),
           "coding parameter upload");
        d_cp = ctx->coding_params.as<uint16_t>();
    }
    rc = run_prepare(ctx, width, height, m, d_index, ctx->compact.as<float>(), prediction_code, coding_warp, d_cp,
                     rp->bias, ctx->pmoments.as<float>());
    if (rc)
        return rc;
    rc = run_reconstruct(ctx, cam, rp, width, height, m, domain_min, domain_max, d_index, ctx->pmoments.as<float>(),
                         d_bounds, ctx->rgba.as<float>(), h_rgba8 ? ctx->rgba8.as<uint8_t>() : nullptr);
    if (rc)
        return rc;
    if (h_rgba)
        CK(cudaMemcpyAsync(h_rgba, ctx->rgba.ptr, P * 4 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "colour download");
    if (h_rgba8)
        CK(cudaMemcpyAsync(h_rgba8, ctx->rgba8.ptr, P * 4, cudaMemcpyDeviceToHost, ctx->stream), "u8 colour download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

// ---- error bounds and uncertainty rendering ----------------------------------------------------------------------

int mraygb_stage_reconstruct_error(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_error_params *ep,
                                   int width, int height, int m, const uint32_t *d_index, const float *d_pmoments,
                                   const uint16_t *d_bounds, uint16_t *d_error_bounds, float *d_errors)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_error_params(ctx, ep)))
        return rc;
    if (!cam || !d_pmoments || !d_error_bounds)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    return run_error_bounds(ctx, cam, ep, width, height, m, d_index, d_pmoments, d_bounds, d_error_bounds, d_errors);
}

int mraygb_reconstruct_error(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_error_params *ep, int width,
                             int height, int m, const uint32_t *h_index, const float *h_data, uint64_t data_size,
                             const uint16_t *h_bounds, int prediction_code, int coding_warp,
                             const uint16_t *h_coding_params, uint16_t *h_error_bounds, float *h_errors)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_error_params(ctx, ep)))
        return rc;
    if (!cam || !h_error_bounds)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const size_t P = (size_t)width * (size_t)height;
    const uint32_t *d_index;
    const uint16_t *d_bounds, *d_cp;
    if ((rc = upload_moment_image(ctx, width, height, m, h_index, h_data, data_size, h_bounds, prediction_code,
                                  coding_warp, h_coding_params, &d_index, &d_bounds, &d_cp)))
        return rc;
    CK(ctx->error_bounds.reserve(P * sizeof(uint16_t)), "error bound buffer allocation");
    if (h_errors)
        CK(ctx->errors.reserve(P * sizeof(float)), "error buffer allocation");
    rc = run_prepare(ctx, width, height, m, d_index, ctx->compact.as<float>(), prediction_code, coding_warp, d_cp,
                     ep->bias, ctx->pmoments.as<float>());
    if (rc)
        return rc;
    rc = run_error_bounds(ctx, cam, ep, width, height, m, d_index, ctx->pmoments.as<float>(), d_bounds,
                          ctx->error_bounds.as<uint16_t>(), h_errors ? ctx->errors.as<float>() : nullptr);
    if (rc)
        return rc;
    CK(cudaMemcpyAsync(h_error_bounds, ctx->error_bounds.ptr, P * sizeof(uint16_t), cudaMemcpyDeviceToHost,
                       ctx->stream),
       "error bound download");
    if (h_errors)
        CK(cudaMemcpyAsync(h_errors, ctx->errors.ptr, P * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "error download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

int mraygb_upload_uncertainty_tf(mraygb_context *ctx, const float *tf1d_rgba256, float step_size, int error_type,
                                 float *h_table)
{
    CHECK_CTX();
    if (!tf1d_rgba256)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL transfer function");
    if (error_type < MRAYGB_ERROR_MAX || error_type > MRAYGB_ERROR_PERCENTILE)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "unknown error type %d", error_type);
    CK(ctx->unc_tf1d.reserve(256 * sizeof(float4)), "transfer function allocation");
    CK(ctx->unc_table.reserve(256 * 256 * sizeof(float4)), "uncertainty table allocation");
    CK(cudaMemcpyAsync(ctx->unc_tf1d.ptr, tf1d_rgba256, 256 * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream),
       "transfer function upload");
    CK(launch_uncertainty_tf(ctx->unc_tf1d.as<float4>(), step_size, error_type, ctx->unc_table.as<float4>(),
                             ctx->stream),
       "uncertainty table launch");
    ctx->launches += 1;
    if (h_table)
        CK(cudaMemcpyAsync(h_table, ctx->unc_table.ptr, 256 * 256 * sizeof(float4), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "uncertainty table download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    ctx->has_unc_table = true;
    return MRAYGB_OK;
}

// ---- reference direct volume rendering ------------------------------------------------------------------------

int mraygb_stage_generate_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp,
                                    int width, int height, float *d_rgba)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, 1);
    if (rc)
        return rc;
    if ((rc = validate_reference(ctx, cam, rp)))
        return rc;
    if (!d_rgba)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL colour buffer");
    return run_reference(ctx, cam, rp, width, height, d_rgba, nullptr);
}

int mraygb_generate_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp,
                              int width, int height, float *h_rgba, uint8_t *h_rgba8)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, 1);
    if (rc)
        return rc;
    if ((rc = validate_reference(ctx, cam, rp)))
        return rc;
    if (!h_rgba && !h_rgba8)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no output");
    const size_t P = (size_t)width * (size_t)height;
    CK(ctx->rgba.reserve(P * 4 * sizeof(float)), "colour buffer allocation");
    if (h_rgba8)
        CK(ctx->rgba8.reserve(P * 4), "u8 colour buffer allocation");
    if ((rc = run_reference(ctx, cam, rp, width, height, ctx->rgba.as<float>(),
                            h_rgba8 ? ctx->rgba8.as<uint8_t>() : nullptr)))
        return rc;
    if (h_rgba)
        CK(cudaMemcpyAsync(h_rgba, ctx->rgba.ptr, P * 4 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "colour download");
    if (h_rgba8)
        CK(cudaMemcpyAsync(h_rgba8, ctx->rgba8.ptr, P * 4, cudaMemcpyDeviceToHost, ctx->stream), "u8 colour download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

// ---- single scattering: the transmittance cache ---------------------------------------------------------------

namespace
{

int check_texture3d(mraygb_context *ctx, int nx, int ny, int nz, const char *what)
{
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "%s of %d x %d x %d voxels", what, nx, ny, nz);
    int max3d[3] = {0, 0, 0};
    cudaDeviceGetAttribute(&max3d[0], cudaDevAttrMaxTexture3DWidth, ctx->device);
    cudaDeviceGetAttribute(&max3d[1], cudaDevAttrMaxTexture3DHeight, ctx->device);
    cudaDeviceGetAttribute(&max3d[2], cudaDevAttrMaxTexture3DDepth, ctx->device);
    if (nx > max3d[0] || ny > max3d[1] || nz > max3d[2])
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "%s %d x %d x %d exceeds the 3D texture limits %d x %d x %d", what, nx,
                    ny, nz, max3d[0], max3d[1], max3d[2]);
    return MRAYGB_OK;
}

// the cache's array and texture for nx x ny x nz voxels (kept while the size stays), filled from `src`
int store_ss_cache(mraygb_context *ctx, const float *src, int nx, int ny, int nz, const float dmin[3],
                   const float dmax[3], cudaMemcpyKind kind)
{
    if (!(ctx->ss_array && ctx->ss_size[0] == nx && ctx->ss_size[1] == ny && ctx->ss_size[2] == nz))
    {
        release_ss_cache(ctx);
        const cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
        CK(cudaMalloc3DArray(&ctx->ss_array, &desc, make_cudaExtent(nx, ny, nz)), "cache allocation");
        cudaResourceDesc res;
        std::memset(&res, 0, sizeof(res));
        res.resType = cudaResourceTypeArray;
        res.res.array.array = ctx->ss_array;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        CK(cudaCreateTextureObject(&ctx->ss_tex, &res, &td, nullptr), "cache texture");
        ctx->ss_size[0] = nx;
        ctx->ss_size[1] = ny;
        ctx->ss_size[2] = nz;
    }
    ctx->has_ss_cache = false;
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<float *>(src), (size_t)nx * sizeof(float), nx, ny);
    cp.dstArray = ctx->ss_array;
    cp.extent = make_cudaExtent(nx, ny, nz);
    cp.kind = kind;
    CK(cudaMemcpy3DAsync(&cp, ctx->stream), "cache copy");
    for (int i = 0; i < 3; ++i)
    {
        ctx->ss_dmin[i] = dmin[i];
        ctx->ss_dmax[i] = dmax[i];
    }
    ctx->has_ss_cache = true;
    return MRAYGB_OK;
}

int validate_ss_cache(mraygb_context *ctx, const mraygb_camera *light_cam, const mraygb_reconstruction_params *rp,
                      const float dmin[3], const float dmax[3])
{
    if (!light_cam || !rp || !dmin || !dmax)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    if (!(rp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "step_size must be > 0 (got %g)", (double)rp->step_size);
    if (rp->use_truncated_fourier)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "truncated Fourier reconstruction is not part of this path");
    for (int i = 0; i < 3; ++i)
        if (!(dmax[i] > dmin[i]))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "empty domain along axis %d", i);
    if (!ctx->has_tf)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no transfer function uploaded");
    return check_texture3d(ctx, rp->ss.cache_size_x, rp->ss.cache_size_y, rp->ss.cache_size_z,
                           "single-scattering cache");
}

int run_ss_cache(mraygb_context *ctx, const mraygb_camera *light_cam, const mraygb_reconstruction_params *rp,
                 int width, int height, int m, const float dmin[3], const float dmax[3], const uint32_t *d_index,
                 const float *d_pm, const uint16_t *d_bounds, float *d_cache)
{
    const int cx = rp->ss.cache_size_x, cy = rp->ss.cache_size_y, cz = rp->ss.cache_size_z;
    const size_t nvox = (size_t)cx * (size_t)cy * (size_t)cz;
    CK(ctx->ss_keys.reserve(nvox * sizeof(unsigned long long)), "cache key allocation");
    if (!d_cache)
    {
        CK(ctx->ss_linear.reserve(nvox * sizeof(float)), "cache allocation");
        d_cache = ctx->ss_linear.as<float>();
    }
    const DeviceCamera dc = to_device_camera(*light_cam);
    SsCacheArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.m = m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = dmin[i];
        a.dmax[i] = dmax[i];
    }
    a.index = d_index;
    a.pmoments = d_pm;
    a.bounds = d_bounds;
    a.tf = ctx->tf.as<float4>();
    a.step = rp->step_size;
    a.cx = cx;
    a.cy = cy;
    a.cz = cz;
    a.keys = ctx->ss_keys.as<unsigned long long>();
    a.cache = d_cache;
    CK(launch_ss_cache(a, ctx->error_flag.as<int>(), ctx->stream), "single-scattering cache launch");
    ctx->launches += 2;
    return store_ss_cache(ctx, d_cache, cx, cy, cz, dmin, dmax, cudaMemcpyDeviceToDevice);
}

} // namespace

int mraygb_upload_single_scattering_cache(mraygb_context *ctx, const float *data, int nx, int ny, int nz,
                                          const float dmin[3], const float dmax[3], int data_on_device)
{
    CHECK_CTX();
    if (!data || !dmin || !dmax)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    int rc = check_texture3d(ctx, nx, ny, nz, "single-scattering cache");
    if (rc)
        return rc;
    for (int i = 0; i < 3; ++i)
        if (!(dmax[i] > dmin[i]))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "empty domain along axis %d", i);
    if ((rc = store_ss_cache(ctx, data, nx, ny, nz, dmin, dmax,
                             data_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice)))
        return rc;
    if (!data_on_device)
        CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

int mraygb_stage_reconstruct_single_scattering_cache(mraygb_context *ctx, const mraygb_camera *light_cam,
                                                     const mraygb_reconstruction_params *rp, int width, int height,
                                                     int m, const float domain_min[3], const float domain_max[3],
                                                     const uint32_t *d_index, const float *d_pmoments,
                                                     const uint16_t *d_bounds, float *d_cache)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_ss_cache(ctx, light_cam, rp, domain_min, domain_max)))
        return rc;
    if (!d_pmoments)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL multipliers");
    return run_ss_cache(ctx, light_cam, rp, width, height, m, domain_min, domain_max, d_index, d_pmoments, d_bounds,
                        d_cache);
}

int mraygb_reconstruct_single_scattering_cache(mraygb_context *ctx, const mraygb_camera *light_cam,
                                               const mraygb_reconstruction_params *rp, int width, int height, int m,
                                               const float domain_min[3], const float domain_max[3],
                                               const uint32_t *h_index, const float *h_data, uint64_t data_size,
                                               const uint16_t *h_bounds, int prediction_code, int coding_warp,
                                               const uint16_t *h_coding_params, float *h_cache)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_ss_cache(ctx, light_cam, rp, domain_min, domain_max)))
        return rc;
    const uint32_t *d_index;
    const uint16_t *d_bounds, *d_cp;
    if ((rc = upload_moment_image(ctx, width, height, m, h_index, h_data, data_size, h_bounds, prediction_code,
                                  coding_warp, h_coding_params, &d_index, &d_bounds, &d_cp)))
        return rc;
    if ((rc = run_prepare(ctx, width, height, m, d_index, ctx->compact.as<float>(), prediction_code, coding_warp,
                          d_cp, rp->bias, ctx->pmoments.as<float>())))
        return rc;
    if ((rc = run_ss_cache(ctx, light_cam, rp, width, height, m, domain_min, domain_max, d_index,
                           ctx->pmoments.as<float>(), d_bounds, nullptr)))
        return rc;
    if (h_cache)
    {
        const size_t nvox = (size_t)rp->ss.cache_size_x * rp->ss.cache_size_y * rp->ss.cache_size_z;
        CK(cudaMemcpyAsync(h_cache, ctx->ss_linear.ptr, nvox * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "cache download");
    }
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

namespace
{

// ref_from_rec_params (src/parameters.h:379-390)
mraygb_reference_params ref_from_rec(const mraygb_reconstruction_params &r)
{
    mraygb_reference_params o{};
    o.step_size = r.step_size;
    o.medium_emission = r.medium_emission;
    o.medium_scattering = r.medium_scattering;
    o.early_ray_termination = r.early_ray_termination;
    o.data_min = r.data_min;
    o.data_max = r.data_max;
    o.ss = r.ss;
    return o;
}

int validate_reference_cached(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp)
{
    if (!rp)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "reconstruction parameters are NULL");
    const mraygb_reference_params ref = ref_from_rec(*rp);
    int rc = validate_reference(ctx, cam, &ref);
    if (rc)
        return rc;
    if (rp->ss.enable && rp->medium_scattering > 0.0f && !ctx->has_ss_cache)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT,
                    "single scattering needs a transmittance cache (mraygb_reconstruct_single_scattering_cache or "
                    "mraygb_upload_single_scattering_cache)");
    return MRAYGB_OK;
}

} // namespace

int mraygb_stage_generate_reference_reconstructed_ss(mraygb_context *ctx, const mraygb_camera *cam,
                                                     const mraygb_reconstruction_params *rp, int width, int height,
                                                     float *d_rgba)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, 1);
    if (rc)
        return rc;
    if ((rc = validate_reference_cached(ctx, cam, rp)))
        return rc;
    if (!d_rgba)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL colour buffer");
    const mraygb_reference_params ref = ref_from_rec(*rp);
    return run_reference(ctx, cam, &ref, width, height, d_rgba, nullptr, true);
}

int mraygb_generate_reference_reconstructed_ss(mraygb_context *ctx, const mraygb_camera *cam,
                                               const mraygb_reconstruction_params *rp, int width, int height,
                                               float *h_rgba, uint8_t *h_rgba8)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, 1);
    if (rc)
        return rc;
    if ((rc = validate_reference_cached(ctx, cam, rp)))
        return rc;
    if (!h_rgba && !h_rgba8)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "no output");
    const mraygb_reference_params ref = ref_from_rec(*rp);
    const size_t P = (size_t)width * (size_t)height;
    CK(ctx->rgba.reserve(P * 4 * sizeof(float)), "colour buffer allocation");
    if (h_rgba8)
        CK(ctx->rgba8.reserve(P * 4), "u8 colour buffer allocation");
    if ((rc = run_reference(ctx, cam, &ref, width, height, ctx->rgba.as<float>(),
                            h_rgba8 ? ctx->rgba8.as<uint8_t>() : nullptr, true)))
        return rc;
    if (h_rgba)
        CK(cudaMemcpyAsync(h_rgba, ctx->rgba.ptr, P * 4 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "colour download");
    if (h_rgba8)
        CK(cudaMemcpyAsync(h_rgba8, ctx->rgba8.ptr, P * 4, cudaMemcpyDeviceToHost, ctx->stream), "u8 colour download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

// ---- the moment-image file format ------------------------------------------------------------------------------

namespace
{

constexpr float kPlainLo = (float)(-1.0 / 3.14159265358979323846); // quantize(..., -1.0 / M_PI, 1.0 / M_PI)
constexpr float kPlainHi = (float)(1.0 / 3.14159265358979323846);

int host_threads()
{
    const unsigned t = std::thread::hardware_concurrency();
    return t ? (int)t : 1;
}

// the bits of each moment index: the prediction-coding table (given, else [16, bits, ...],
// get_prediction_coding_quantization_table, moment_quantization.cpp:186-203) or `bits` for every index
std::vector<uint8_t> payload_table(const mraygb_moment_image &mi, int bits, const uint8_t *quant_table)
{
    std::vector<uint8_t> t((size_t)mi.num_moments, (uint8_t)bits);
    if (mi.prediction_code)
    {
        if (quant_table)
            std::memcpy(t.data(), quant_table, t.size());
        else if (!t.empty())
            t[0] = 16;
    }
    return t;
}

int check_file_image(mraygb_context *ctx, const mraygb_moment_image *mi, int bits, int entropy,
                     const uint8_t *quant_table)
{
    if (!mi)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL moment image");
    if (mi->width <= 0 || mi->height <= 0 || mi->width > 65535 || mi->height > 65535)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "image size %dx%d outside 1..65535", mi->width, mi->height);
    if (mi->num_moments < 1 || mi->num_moments > 255)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "num_moments %d outside 1..255 (the file stores it in a byte)",
                    mi->num_moments);
    if (bits < 1 || bits > 32)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "quantization bits %d outside 1..32", bits);
    if (!mi->data)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL moment data");
    const size_t P = (size_t)mi->width * (size_t)mi->height;
    if (mi->is_compact)
    {
        if (!mi->index)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "a compact image needs its index");
        for (size_t p = 0; p < P; ++p)
            if (mi->index[p + 1] < mi->index[p] || mi->index[p + 1] - mi->index[p] > (uint32_t)mi->num_moments)
                return fail(ctx, MRAYGB_INVALID_ARGUMENT, "pixel %zu holds %lld moments (0..%d)", p,
                            (long long)mi->index[p + 1] - (long long)mi->index[p], mi->num_moments);
        if (mi->data_size < mi->index[P])
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "data_size %llu is below the index's %u",
                        (unsigned long long)mi->data_size, mi->index[P]);
    }
    else
    {
        if (mi->prediction_code)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "prediction coding needs a compact image");
        if (entropy)
            return fail(ctx, MRAYGB_NOT_SUPPORTED, "the entropy coder writes compact images only");
        if (mi->data_size < P * (size_t)mi->num_moments)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "a static image needs W*H*m floats");
    }
    if (entropy)
    {
        if (mi->prediction_code && !quant_table)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT,
                        "entropy coding of a prediction-coded image needs the quantization table");
        const std::vector<uint8_t> t = payload_table(*mi, bits, quant_table);
        for (int l = 1; l < mi->num_moments; ++l)
            if (t[l] < 1 || t[l] > 14)
                return fail(ctx, MRAYGB_INVALID_ARGUMENT,
                            "entropy coding takes 1..14 bits per code (moment index %d has %d)", l, (int)t[l]);
    }
    return MRAYGB_OK;
}

// the payload of a compact image: floats, packed codes or entropy-coded streams (write_moment_image,
// moment_image_io.cpp:398-436)
int compact_payload(mraygb_context *ctx, const mraygb_moment_image &mi, int bits, int entropy,
                    const uint8_t *quant_table, std::vector<uint8_t> &payload)
{
    const int P = mi.width * mi.height;
    const int m = mi.num_moments;
    const size_t nd = mi.index[P];
    if (!entropy && bits == 32)
    {
        payload.resize(nd * sizeof(float));
        if (nd)
            std::memcpy(payload.data(), mi.data, nd * sizeof(float));
        return MRAYGB_OK;
    }
    const std::vector<uint8_t> table = payload_table(mi, bits, quant_table);
    const float lo1 = mi.prediction_code ? 0.f : kPlainLo, hi1 = mi.prediction_code ? 1.f : kPlainHi;
    CK(ctx->index.reserve(((size_t)P + 1) * sizeof(uint32_t)), "index buffer allocation");
    CK(ctx->compact.reserve((nd ? nd : 1) * sizeof(float)), "moment buffer allocation");
    CK(cudaMemcpyAsync(ctx->index.ptr, mi.index, ((size_t)P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       ctx->stream),
       "index upload");
    if (nd)
        CK(cudaMemcpyAsync(ctx->compact.ptr, mi.data, nd * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
           "moment upload");
    const uint8_t *d_table;
    const uint32_t *d_prefix;
    int rc = upload_table(ctx, m, table.data(), &d_table, &d_prefix);
    if (rc)
        return rc;
    if (entropy)
    {
        // u16 codes on the device, the arithmetic coder on host threads
        CK(ctx->file_codes.reserve((nd ? nd : 1) * sizeof(uint16_t)), "code buffer allocation");
        CK(launch_symbols(P, ctx->index.as<uint32_t>(), ctx->compact.as<float>(), d_table, lo1, hi1,
                          ctx->file_codes.as<uint16_t>(), ctx->stream),
           "code launch");
        ctx->launches += 1;
        std::vector<uint16_t> codes(nd ? nd : 1);
        CK(cudaMemcpyAsync(codes.data(), ctx->file_codes.ptr, nd * sizeof(uint16_t), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "code download");
        CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        payload = entropy_encode(mi.width, mi.height, m, mi.index, codes.data(), table.data(), host_threads());
        return MRAYGB_OK;
    }
    uint64_t total_bits = 0;
    if ((rc = run_bit_offsets(ctx, P, ctx->index.as<uint32_t>(), d_prefix, &total_bits)))
        return rc;
    const uint64_t word_bytes = ((total_bits + 31) / 32) * 4;
    CK(ctx->packed.reserve(word_bytes ? word_bytes : 4), "packed buffer allocation");
    if (word_bytes)
        CK(cudaMemsetAsync(ctx->packed.ptr, 0, word_bytes, ctx->stream), "clearing the packed buffer");
    CK(launch_pack(P, ctx->index.as<uint32_t>(), ctx->compact.as<float>(), d_table, d_prefix,
                   ctx->bit_offset.as<unsigned long long>(), ctx->packed.as<uint32_t>(), ctx->stream, lo1, hi1),
       "pack launch");
    ctx->launches += 1;
    payload.resize(total_bits / 8); // pack_bits emits whole bytes only
    if (!payload.empty())
        CK(cudaMemcpyAsync(payload.data(), ctx->packed.ptr, payload.size(), cudaMemcpyDeviceToHost, ctx->stream),
           "packed download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

// write_static_image (moment_image_io.cpp:438-491): the payload follows the sections without a size prefix
int static_payload(mraygb_context *ctx, const mraygb_moment_image &mi, int compress, int bits,
                   std::vector<uint8_t> &out)
{
    const size_t count = (size_t)mi.width * (size_t)mi.height * (size_t)mi.num_moments;
    const uint8_t *raw = reinterpret_cast<const uint8_t *>(mi.data);
    if (!compress)
    {
        out.insert(out.end(), raw, raw + count * sizeof(float));
        return MRAYGB_OK;
    }
    if (bits == 32)
    {
        std::vector<uint8_t> block(count * sizeof(float));
        const size_t r = lz4_compress(raw, count * sizeof(float), block.data(), block.size());
        if (r == 0 || r >= block.size())
            out.insert(out.end(), raw, raw + count); // (sic) the reference writes one byte per float here
        else
            out.insert(out.end(), block.begin(), block.begin() + (long)r);
        return MRAYGB_OK;
    }
    // the bits byte, then the byte-aligned codes as one LZ4 block (its capacity, four times the codes, always holds it)
    out.push_back((uint8_t)bits);
    const size_t code_bytes = count * (size_t)((bits + 7) / 8);
    CK(ctx->compact.reserve((count ? count : 1) * sizeof(float)), "moment buffer allocation");
    CK(ctx->packed.reserve(code_bytes ? code_bytes : 4), "code buffer allocation");
    if (count)
    {
        CK(cudaMemcpyAsync(ctx->compact.ptr, mi.data, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
           "moment upload");
        CK(launch_static_quantize(count, mi.num_moments, ctx->compact.as<float>(), bits, kPlainLo, kPlainHi,
                                  ctx->packed.as<uint8_t>(), ctx->stream),
           "quantize launch");
        ctx->launches += 1;
    }
    std::vector<uint8_t> codes(code_bytes);
    if (code_bytes)
        CK(cudaMemcpyAsync(codes.data(), ctx->packed.ptr, code_bytes, cudaMemcpyDeviceToHost, ctx->stream),
           "code download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    std::vector<uint8_t> block(code_bytes * 4 + 16);
    const size_t r = lz4_compress(codes.data(), code_bytes, block.data(), code_bytes * 4);
    if (r == 0 || r >= code_bytes * 4)
        out.insert(out.end(), codes.begin(), codes.end());
    else
        out.insert(out.end(), block.begin(), block.begin() + (long)r);
    return MRAYGB_OK;
}

int encode_file(mraygb_context *ctx, const mraygb_moment_image *mi, int compress, int bits, int entropy,
                const uint8_t *quant_table, std::vector<uint8_t> &out)
{
    int rc = check_file_image(ctx, mi, bits, entropy, quant_table);
    if (rc)
        return rc;
    const size_t P = (size_t)mi->width * (size_t)mi->height;
    const int m = mi->num_moments;
    FileHeader h;
    h.width = (uint16_t)mi->width;
    h.height = (uint16_t)mi->height;
    h.moments = (uint8_t)m;
    h.coding_warp = (uint8_t)mi->coding_warp;
    h.bits = (uint8_t)((bits & 0xff) | (entropy ? 64 : 0) | (quant_table ? 128 : 0));
    h.flags = (uint8_t)((compress ? 1 : 0) | (mi->is_compact ? 2 : 0) | (mi->prediction_code ? 4 : 0) |
                        (mi->bounds ? 16 : 0) | (mi->error_bounds ? 32 : 0) | (mi->coding_params ? 128 : 0));
    for (int i = 0; i < 3; ++i)
    {
        h.dmin[i] = mi->domain_min[i];
        h.dmax[i] = mi->domain_max[i];
    }
    out.clear();
    put_header(out, h);
    if (quant_table)
        put_section(out, quant_table, (size_t)m, compress != 0);
    if (mi->is_compact)
    {
        std::vector<uint8_t> counts(P);
        for (size_t p = 0; p < P; ++p)
            counts[p] = (uint8_t)(mi->index[p + 1] - mi->index[p]);
        put_section(out, counts.data(), P, compress != 0);
    }
    if (mi->bounds)
        put_section(out, reinterpret_cast<const uint8_t *>(mi->bounds), P * 4, compress != 0);
    if (mi->error_bounds)
        put_section(out, reinterpret_cast<const uint8_t *>(mi->error_bounds), P * 2, compress != 0);
    if (mi->coding_params)
        put_section(out, reinterpret_cast<const uint8_t *>(mi->coding_params), (size_t)(m - 1) * 4, compress != 0);
    if (!mi->is_compact)
        return static_payload(ctx, *mi, compress, bits, out);
    std::vector<uint8_t> payload;
    if ((rc = compact_payload(ctx, *mi, bits, entropy, quant_table, payload)))
        return rc;
    put_section(out, payload.data(), payload.size(), compress != 0);
    return MRAYGB_OK;
}

int decode_file(mraygb_context *ctx, const uint8_t *file, size_t n, mraygb_moment_image *mi, uint8_t *quant_table,
                int *has_quant_table)
{
    if (!file || !mi)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    FileHeader h;
    if (!get_header(file, n, h))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the file is shorter than its header");
    const bool sizes_only = mi->data == nullptr;
    const int W = h.width, H = h.height, m = h.moments;
    const size_t P = (size_t)W * (size_t)H;
    const bool compressed = h.compressed();
    const int bits = h.quantization_bits();
    if (W == 0 || H == 0 || m == 0)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "empty image %dx%d with %d moments in the header", W, H, m);
    if (bits < 1 || bits > 32)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "quantization bits %d in the header (1..32)", bits);
    mi->width = W;
    mi->height = H;
    mi->num_moments = m;
    mi->coding_warp = h.coding_warp;
    mi->is_compact = h.compact();
    mi->prediction_code = h.prediction_coded();
    mi->has_bounds = h.has_bounds();
    mi->has_error_bounds = h.has_error_bounds();
    mi->has_coding_params = h.has_coding_params();
    for (int i = 0; i < 3; ++i)
    {
        mi->domain_min[i] = h.dmin[i];
        mi->domain_max[i] = h.dmax[i];
    }
    size_t pos = kFileHeaderBytes;
    std::vector<uint8_t> table((size_t)m, 0);
    if (has_quant_table)
        *has_quant_table = h.has_table() ? 1 : 0;
    if (h.has_table())
    {
        if (!get_section(file, n, &pos, (size_t)m, compressed, table.data()))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated quantization table");
        if (quant_table)
            std::memcpy(quant_table, table.data(), (size_t)m);
    }
    std::vector<uint32_t> index;
    if (h.compact())
    {
        std::vector<uint8_t> counts(P, 0);
        if (!get_section(file, n, &pos, P, compressed, counts.data()))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated index");
        index.resize(P + 1);
        uint64_t sum = 0;
        for (size_t p = 0; p < P; ++p)
        {
            if (counts[p] > m)
                return fail(ctx, MRAYGB_INVALID_ARGUMENT, "pixel %zu holds %d moments, the header %d", p,
                            (int)counts[p], m);
            index[p] = (uint32_t)sum;
            sum += counts[p];
        }
        if (sum >= (1ull << 32))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the index exceeds u32");
        index[P] = (uint32_t)sum;
        mi->data_size = sum;
    }
    else
    {
        if (h.prediction_coded())
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "a static image cannot be prediction coded");
        mi->data_size = (uint64_t)P * (uint64_t)m;
    }
    if (sizes_only)
        return MRAYGB_OK;
    if (h.compact() && !mi->index)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL index for a compact image");
    if ((h.has_bounds() && !mi->bounds) || (h.has_error_bounds() && !mi->error_bounds) ||
        (h.has_coding_params() && !mi->coding_params))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the file holds bounds, error bounds or coding parameters the "
                                                  "call gives no buffer for");
    if (h.compact())
        std::memcpy(mi->index, index.data(), (P + 1) * sizeof(uint32_t));
    if (h.has_bounds())
    {
        std::memset(mi->bounds, 0, P * 4);
        if (!get_section(file, n, &pos, P * 4, compressed, reinterpret_cast<uint8_t *>(mi->bounds)))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated bounds");
    }
    if (h.has_error_bounds())
    {
        std::memset(mi->error_bounds, 0, P * 2);
        if (!get_section(file, n, &pos, P * 2, compressed, reinterpret_cast<uint8_t *>(mi->error_bounds)))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated error bounds");
    }
    if (h.has_coding_params())
    {
        std::memset(mi->coding_params, 0, (size_t)(m - 1) * 4);
        if (!get_section(file, n, &pos, (size_t)(m - 1) * 4, compressed,
                         reinterpret_cast<uint8_t *>(mi->coding_params)))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated coding parameters");
    }
    const size_t nd = (size_t)mi->data_size;
    std::memset(mi->data, 0, nd * sizeof(float));
    if (!h.compact())
    {
        // read_static_image (moment_image_io.cpp:197-252)
        if (!compressed)
        {
            if (n - pos < nd * sizeof(float))
                return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated moment data");
            std::memcpy(mi->data, file + pos, nd * sizeof(float));
            return MRAYGB_OK;
        }
        if (bits < 32)
            return fail(ctx, MRAYGB_NOT_SUPPORTED,
                        "a compressed, quantized static image: the reference's writer puts the bits before the block "
                        "and its reader decodes from that byte");
        if (lz4_decompress(file + pos, n - pos, reinterpret_cast<uint8_t *>(mi->data), nd * sizeof(float)) < 0)
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "malformed LZ4 block");
        return MRAYGB_OK;
    }
    // read_moment_image (moment_image_io.cpp:158-185)
    std::vector<uint8_t> bytes;
    if (!get_payload(file, n, &pos, nd * 4, compressed, bytes))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "truncated moment payload");
    const bool entropy = h.entropy_coded();
    if (!entropy && bits == 32)
    {
        std::memcpy(mi->data, bytes.data(), std::min(bytes.size(), nd * sizeof(float)));
        return MRAYGB_OK;
    }
    mraygb_moment_image shape = *mi;
    if (entropy && h.prediction_coded() && !h.has_table())
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "an entropy-coded prediction-coded image without its table");
    const std::vector<uint8_t> bit_table = payload_table(shape, bits, h.has_table() ? table.data() : nullptr);
    const float lo1 = h.prediction_coded() ? 0.f : kPlainLo, hi1 = h.prediction_coded() ? 1.f : kPlainHi;
    if (entropy)
        for (int l = 1; l < m; ++l)
            if (bit_table[l] < 1 || bit_table[l] > 14)
                return fail(ctx, MRAYGB_INVALID_ARGUMENT, "entropy-coded moment index %d with %d bits", l,
                            (int)bit_table[l]);
    const int iP = (int)P;
    CK(ctx->index.reserve((P + 1) * sizeof(uint32_t)), "index buffer allocation");
    CK(ctx->compact.reserve((nd ? nd : 1) * sizeof(float)), "moment buffer allocation");
    CK(cudaMemcpyAsync(ctx->index.ptr, index.data(), (P + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
       "index upload");
    const uint8_t *d_table;
    const uint32_t *d_prefix;
    int rc = upload_table(ctx, m, bit_table.data(), &d_table, &d_prefix);
    if (rc)
        return rc;
    if (entropy)
    {
        std::vector<uint16_t> codes(nd ? nd : 1, 0);
        if (!entropy_decode(bytes.data(), bytes.size(), W, H, m, index.data(), bit_table.data(), codes.data(),
                            host_threads()))
            return fail(ctx, MRAYGB_INVALID_ARGUMENT, "malformed entropy-coded payload");
        CK(ctx->file_codes.reserve((nd ? nd : 1) * sizeof(uint16_t)), "code buffer allocation");
        CK(cudaMemcpyAsync(ctx->file_codes.ptr, codes.data(), nd * sizeof(uint16_t), cudaMemcpyHostToDevice,
                           ctx->stream),
           "code upload");
        CK(launch_desymbols(iP, ctx->index.as<uint32_t>(), ctx->file_codes.as<uint16_t>(), d_table, lo1, hi1,
                            ctx->compact.as<float>(), ctx->stream),
           "dequantize launch");
        ctx->launches += 1;
    }
    else
    {
        uint64_t total_bits = 0;
        if ((rc = run_bit_offsets(ctx, iP, ctx->index.as<uint32_t>(), d_prefix, &total_bits)))
            return rc;
        CK(ctx->packed.reserve(bytes.size() ? bytes.size() : 1), "packed buffer allocation");
        if (!bytes.empty())
            CK(cudaMemcpyAsync(ctx->packed.ptr, bytes.data(), bytes.size(), cudaMemcpyHostToDevice, ctx->stream),
               "packed upload");
        CK(launch_unpack(iP, ctx->index.as<uint32_t>(), d_table, d_prefix, ctx->bit_offset.as<unsigned long long>(),
                         ctx->packed.as<uint8_t>(), bytes.size(), ctx->compact.as<float>(), ctx->stream, lo1, hi1),
           "unpack launch");
        ctx->launches += 1;
    }
    if (nd)
        CK(cudaMemcpyAsync(mi->data, ctx->compact.ptr, nd * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "moment download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return MRAYGB_OK;
}

} // namespace

// host allocations and threads of the file format report failure as a status, never as an exception across the C ABI
#define HOST_GUARD(body)                                                                                            \
    try                                                                                                             \
    {                                                                                                               \
        body                                                                                                        \
    }                                                                                                               \
    catch (const std::bad_alloc &)                                                                                  \
    {                                                                                                               \
        return fail(ctx, MRAYGB_OUT_OF_MEMORY, "host allocation failed");                                          \
    }                                                                                                               \
    catch (const std::exception &e_)                                                                                \
    {                                                                                                               \
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "host failure: %s", e_.what());                                   \
    }

int mraygb_encode_moment_image(mraygb_context *ctx, const mraygb_moment_image *mi, int compress,
                               int quantization_bits, int entropy_coding, const uint8_t *quant_table,
                               uint64_t *h_bytes)
{
    CHECK_CTX();
    if (!h_bytes)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL size output");
    int rc;
    HOST_GUARD(rc = encode_file(ctx, mi, compress, quantization_bits, entropy_coding, quant_table, ctx->encoded);)
    if (rc)
    {
        ctx->encoded.clear();
        return rc;
    }
    *h_bytes = ctx->encoded.size();
    return MRAYGB_OK;
}

int mraygb_copy_encoded(mraygb_context *ctx, uint8_t *out, uint64_t capacity)
{
    CHECK_CTX();
    if (!out || capacity < ctx->encoded.size())
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the buffer holds %llu bytes, %llu needed",
                    (unsigned long long)capacity, (unsigned long long)ctx->encoded.size());
    if (!ctx->encoded.empty())
        std::memcpy(out, ctx->encoded.data(), ctx->encoded.size());
    return MRAYGB_OK;
}

int mraygb_decode_moment_image(mraygb_context *ctx, const uint8_t *bytes, uint64_t n, mraygb_moment_image *mi,
                               uint8_t *quant_table, int *has_quant_table)
{
    CHECK_CTX();
    HOST_GUARD(return decode_file(ctx, bytes, (size_t)n, mi, quant_table, has_quant_table);)
}

int mraygb_write_moment_image(mraygb_context *ctx, const char *path, const mraygb_moment_image *mi, int compress,
                              int quantization_bits, int entropy_coding, const uint8_t *quant_table)
{
    CHECK_CTX();
    if (!path)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL path");
    std::vector<uint8_t> bytes;
    int rc;
    HOST_GUARD(rc = encode_file(ctx, mi, compress, quantization_bits, entropy_coding, quant_table, bytes);)
    if (rc)
        return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "cannot open %s for writing", path);
    const size_t w = bytes.empty() ? 0 : std::fwrite(bytes.data(), 1, bytes.size(), f);
    const bool ok = std::fclose(f) == 0 && w == bytes.size();
    return ok ? MRAYGB_OK : fail(ctx, MRAYGB_INVALID_ARGUMENT, "cannot write %s", path);
}

int mraygb_load_moment_image(mraygb_context *ctx, const char *path, mraygb_moment_image *mi, uint8_t *quant_table,
                             int *has_quant_table)
{
    CHECK_CTX();
    if (!path)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL path");
    FILE *f = std::fopen(path, "rb");
    if (!f)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "cannot open %s", path);
    std::vector<uint8_t> bytes;
    bool read_ok = true;
    try
    {
        uint8_t chunk[1 << 16];
        size_t r;
        while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0)
            bytes.insert(bytes.end(), chunk, chunk + r);
    }
    catch (const std::exception &)
    {
        read_ok = false;
    }
    std::fclose(f);
    if (!read_ok)
        return fail(ctx, MRAYGB_OUT_OF_MEMORY, "host allocation failed reading %s", path);
    HOST_GUARD(return decode_file(ctx, bytes.data(), bytes.size(), mi, quant_table, has_quant_table);)
}

uint64_t mraygb_lz4_compress(const uint8_t *src, uint64_t n, uint8_t *dst, uint64_t cap)
{
    if ((!src && n) || !dst || n >= (1ull << 31))
        return 0;
    return lz4_compress(src, (size_t)n, dst, (size_t)cap);
}

int64_t mraygb_lz4_decompress(const uint8_t *src, uint64_t n, uint8_t *dst, uint64_t cap)
{
    if (!src || (!dst && cap))
        return -1;
    return lz4_decompress(src, (size_t)n, dst, (size_t)cap);
}

int mraygb_entropy_encode(int width, int height, int num_moments, const uint32_t *index, const uint16_t *codes,
                          const uint8_t *table, int threads, uint8_t *out, uint64_t capacity, uint64_t *h_bytes)
{
    if (width <= 0 || height <= 0 || num_moments < 1 || num_moments > 255 || !index || !codes || !table || !h_bytes)
        return MRAYGB_INVALID_ARGUMENT;
    for (int l = 1; l < num_moments; ++l)
        if (table[l] < 1 || table[l] > 14)
            return MRAYGB_INVALID_ARGUMENT;
    const size_t P = (size_t)width * (size_t)height;
    for (size_t p = 0; p < P; ++p)
        if (index[p + 1] < index[p] || index[p + 1] - index[p] > (uint32_t)num_moments)
            return MRAYGB_INVALID_ARGUMENT;
    try
    {
        const std::vector<uint8_t> bytes =
            entropy_encode(width, height, num_moments, index, codes, table, threads > 0 ? threads : host_threads());
        *h_bytes = bytes.size();
        if (out && capacity >= bytes.size() && !bytes.empty())
            std::memcpy(out, bytes.data(), bytes.size());
        return MRAYGB_OK;
    }
    catch (const std::exception &)
    {
        return MRAYGB_OUT_OF_MEMORY;
    }
}

int mraygb_entropy_decode(const uint8_t *bytes, uint64_t n, int width, int height, int num_moments,
                          const uint32_t *index, const uint8_t *table, int threads, uint16_t *codes)
{
    if (!bytes || width <= 0 || height <= 0 || num_moments < 1 || num_moments > 255 || !index || !table || !codes)
        return MRAYGB_INVALID_ARGUMENT;
    for (int l = 1; l < num_moments; ++l)
        if (table[l] < 1 || table[l] > 14)
            return MRAYGB_INVALID_ARGUMENT;
    const size_t P = (size_t)width * (size_t)height;
    for (size_t p = 0; p < P; ++p)
        if (index[p + 1] < index[p] || index[p + 1] - index[p] > (uint32_t)num_moments)
            return MRAYGB_INVALID_ARGUMENT;
    try
    {
        return entropy_decode(bytes, (size_t)n, width, height, num_moments, index, table, codes,
                              threads > 0 ? threads : host_threads())
                   ? MRAYGB_OK
                   : MRAYGB_INVALID_ARGUMENT;
    }
    catch (const std::exception &)
    {
        return MRAYGB_OUT_OF_MEMORY;
    }
}

int mraygb_upload_uncertainty_table(mraygb_context *ctx, const float *table_rgba256x256)
{
    CHECK_CTX();
    if (!table_rgba256x256)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL uncertainty table");
    CK(ctx->unc_table.reserve(256 * 256 * sizeof(float4)), "uncertainty table allocation");
    CK(cudaMemcpyAsync(ctx->unc_table.ptr, table_rgba256x256, 256 * 256 * sizeof(float4), cudaMemcpyHostToDevice,
                       ctx->stream),
       "uncertainty table upload");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    ctx->has_unc_table = true;
    return MRAYGB_OK;
}

int mraygb_stage_reconstruct_uncertainty(mraygb_context *ctx, const mraygb_camera *cam,
                                         const mraygb_uncertainty_params *up, int mode, int width, int height, int m,
                                         const float domain_min[3], const float domain_max[3],
                                         const uint32_t *d_index, const float *d_pmoments, const uint16_t *d_bounds,
                                         const uint16_t *d_error_bounds, float *d_rgba)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_uncertainty(ctx, up, mode)))
        return rc;
    if (!cam || !domain_min || !domain_max || !d_pmoments || !d_error_bounds || !d_rgba)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    return run_uncertainty(ctx, cam, up, mode, width, height, m, domain_min, domain_max, d_index, d_pmoments,
                           d_bounds, d_error_bounds, d_rgba, nullptr);
}

int mraygb_reconstruct_uncertainty(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_uncertainty_params *up,
                                   int mode, int width, int height, int m, const float domain_min[3],
                                   const float domain_max[3], const uint32_t *h_index, const float *h_data,
                                   uint64_t data_size, const uint16_t *h_bounds, const uint16_t *h_error_bounds,
                                   int prediction_code, int coding_warp, const uint16_t *h_coding_params,
                                   float *h_rgba, uint8_t *h_rgba8)
{
    CHECK_CTX();
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_uncertainty(ctx, up, mode)))
        return rc;
    if (!cam || !domain_min || !domain_max || !h_error_bounds || (!h_rgba && !h_rgba8))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL argument");
    const size_t P = (size_t)width * (size_t)height;
    const uint32_t *d_index;
    const uint16_t *d_bounds, *d_cp;
    if ((rc = upload_moment_image(ctx, width, height, m, h_index, h_data, data_size, h_bounds, prediction_code,
                                  coding_warp, h_coding_params, &d_index, &d_bounds, &d_cp)))
        return rc;
    CK(ctx->error_bounds.reserve(P * sizeof(uint16_t)), "error bound buffer allocation");
    CK(cudaMemcpyAsync(ctx->error_bounds.ptr, h_error_bounds, P * sizeof(uint16_t), cudaMemcpyHostToDevice,
                       ctx->stream),
       "error bound upload");
    CK(ctx->rgba.reserve(P * 4 * sizeof(float)), "colour buffer allocation");
    if (h_rgba8)
        CK(ctx->rgba8.reserve(P * 4), "u8 colour buffer allocation");
    rc = run_prepare(ctx, width, height, m, d_index, ctx->compact.as<float>(), prediction_code, coding_warp, d_cp,
                     up->rec.bias, ctx->pmoments.as<float>());
    if (rc)
        return rc;
    rc = run_uncertainty(ctx, cam, up, mode, width, height, m, domain_min, domain_max, d_index,
                         ctx->pmoments.as<float>(), d_bounds, ctx->error_bounds.as<uint16_t>(),
                         ctx->rgba.as<float>(), h_rgba8 ? ctx->rgba8.as<uint8_t>() : nullptr);
    if (rc)
        return rc;
    if (h_rgba)
        CK(cudaMemcpyAsync(h_rgba, ctx->rgba.ptr, P * 4 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "colour download");
    if (h_rgba8)
        CK(cudaMemcpyAsync(h_rgba8, ctx->rgba8.ptr, P * 4, cudaMemcpyDeviceToHost, ctx->stream), "u8 colour download");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return check_device_error_flag(ctx);
}

} // extern "C"

// ---- differentiation form ------------------------------------------------------------------------------------

namespace
{

int validate_diff(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                  const mraygb_reconstruction_params *rp, int width, int height, int m)
{
    int rc = check_image(ctx, width, height, m);
    if (rc)
        return rc;
    if ((rc = validate_gen(ctx, gp)))
        return rc;
    if (!cam || !rp)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "camera or reconstruction parameters are NULL");
    if (gp->compact_image || gp->prediction_coding || !gp->transform_to_bounds)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT,
                    "the differentiation form needs compact_image = 0, prediction_coding = 0, transform_to_bounds = 1");
    if (m > 64)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "the differentiation form supports up to 64 moments (got %d)", m);
    if (!(rp->step_size > 0.f))
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "reconstruction step_size must be > 0");
    if (rp->ss.enable && rp->medium_scattering > 0.0f)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "the differentiation form has no single scattering");
    if (ctx->volume == mraygb_context::NONE)
        return fail(ctx, MRAYGB_NO_VOLUME, "no volume uploaded");
    return MRAYGB_OK;
}

} // namespace

int mraygb_diff_forward(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                        const mraygb_reconstruction_params *rp, int width, int height, int m, const float *d_tf,
                        float *d_moments, float *d_bounds4, float *d_pmoments, float *d_rgba)
{
    CHECK_CTX();
    int rc = validate_diff(ctx, cam, gp, rp, width, height, m);
    if (rc)
        return rc;
    if (!d_tf || !d_moments || !d_bounds4 || !d_pmoments || !d_rgba)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL device buffer");
    if ((reinterpret_cast<uintptr_t>(d_bounds4) | reinterpret_cast<uintptr_t>(d_rgba) |
         reinterpret_cast<uintptr_t>(d_tf)) & 15u)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "d_tf, d_bounds4 and d_rgba must be 16-byte aligned");
    const size_t P = (size_t)width * (size_t)height;
    CK(ctx->bounds.reserve(2 * P * sizeof(uint16_t)), "bounds buffer allocation");
    rc = run_generate_moments(ctx, cam, gp, width, height, m, d_moments, ctx->bounds.as<uint16_t>(), nullptr,
                              reinterpret_cast<float4 *>(d_bounds4));
    if (rc)
        return rc;
    ctx->diff_key.valid = false;
    if (ctx->precision == MRAYGB_PRECISION_FP32)
    {
        // the FP32 multipliers, keeping what the preparation adjoint reads
        rc = run_prepare_keep(ctx, width, height, m, d_moments, rp->bias, d_pmoments);
        if (rc)
            return rc;
        ctx->diff_key = {true, d_moments, d_pmoments, width, height, m, rp->bias};
    }
    else
    {
        rc = run_prepare(ctx, width, height, m, nullptr, d_moments, 0, MRAYGB_CODING_WARP_NONE, nullptr, rp->bias,
                         d_pmoments);
        if (rc)
            return rc;
    }
    return run_reconstruct(ctx, cam, rp, width, height, m, ctx->dmin, ctx->dmax, nullptr, d_pmoments, nullptr, d_rgba,
                           nullptr, reinterpret_cast<const float4 *>(d_bounds4),
                           reinterpret_cast<const float4 *>(d_tf), 1);
}

int mraygb_diff_backward(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                         const mraygb_reconstruction_params *rp, int width, int height, int m, const float *d_tf,
                         const float *d_moments, const float *d_bounds4, const float *d_pmoments, const float *d_rgba,
                         const float *d_grad_rgba, float *d_grad_tf, float *d_grad_volume)
{
    CHECK_CTX();
    int rc = validate_diff(ctx, cam, gp, rp, width, height, m);
    if (rc)
        return rc;
    if (!d_tf || !d_moments || !d_bounds4 || !d_pmoments || !d_rgba || !d_grad_rgba || !d_grad_tf)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "NULL device buffer");
    if ((reinterpret_cast<uintptr_t>(d_bounds4) | reinterpret_cast<uintptr_t>(d_rgba) |
         reinterpret_cast<uintptr_t>(d_tf) | reinterpret_cast<uintptr_t>(d_grad_rgba) |
         reinterpret_cast<uintptr_t>(d_grad_tf)) & 15u)
        return fail(ctx, MRAYGB_INVALID_ARGUMENT, "float4 buffers must be 16-byte aligned");
    if (d_grad_volume && ctx->volume != mraygb_context::GRID)
        return fail(ctx, MRAYGB_NOT_SUPPORTED, "density gradients need a regular grid (particles: transfer function "
                                               "gradient only)");
    const size_t P = (size_t)width * (size_t)height;
    CK(ctx->adj_lambda.reserve(P * (size_t)m * sizeof(float)), "adjoint buffer allocation");
    CK(ctx->adj_bounds.reserve(P * sizeof(float2)), "adjoint buffer allocation");
    if (d_grad_volume)
    {
        const auto &k = ctx->diff_key;
        if (!(k.valid && k.moments == d_moments && k.pmoments == d_pmoments && k.width == width &&
              k.height == height && k.m == m && k.bias == rp->bias))
        {
            // the last forward kept nothing for these buffers (another precision form, or other buffers since):
            // run the FP32 preparation again for its arrays, its multipliers into the adjoint buffer (overwritten
            // below by the re-march adjoint)
            rc = run_prepare_keep(ctx, width, height, m, d_moments, rp->bias, ctx->adj_lambda.as<float>());
            if (rc)
                return rc;
            ctx->diff_key.valid = false;
        }
    }
    const DeviceCamera dc = to_device_camera(*cam);
    ReconAdjArgs a;
    a.cam = &dc;
    a.width = width;
    a.height = height;
    a.m = m;
    for (int i = 0; i < 3; ++i)
    {
        a.dmin[i] = ctx->dmin[i];
        a.dmax[i] = ctx->dmax[i];
    }
    a.pmoments = d_pmoments;
    a.bounds4 = reinterpret_cast<const float4 *>(d_bounds4);
    a.tf = reinterpret_cast<const float4 *>(d_tf);
    a.step = rp->step_size;
    a.emission = rp->medium_emission;
    a.ert = rp->early_ray_termination;
    a.rgba = reinterpret_cast<const float4 *>(d_rgba);
    a.grad_rgba = reinterpret_cast<const float4 *>(d_grad_rgba);
    a.grad_lambda = ctx->adj_lambda.as<float>();
    a.grad_bounds = ctx->adj_bounds.as<float2>();
    a.grad_tf = reinterpret_cast<float4 *>(d_grad_tf);
    a.tf_linear = ctx->diff_tf_sampling == MRAYGB_DIFF_TF_LINEAR;
    CK(launch_reconstruct_adjoint(a, ctx->error_flag.as<int>(), ctx->stream), "re-march adjoint launch");
    ctx->launches += 1;
    if (!d_grad_volume)
        return MRAYGB_OK;
    CK(launch_prepare_adjoint((int)P, m, ctx->diff_keep.as<float2>(), rp->bias, ctx->adj_lambda.as<float>(),
                              ctx->adj_lambda.as<float>(), ctx->stream),
       "preparation adjoint launch");
    CK(launch_generate_adjoint(grid_view(ctx), d_grad_volume, dc, *gp, width, height, m, d_moments,
                               reinterpret_cast<const float4 *>(d_bounds4), ctx->adj_lambda.as<float>(),
                               ctx->adj_bounds.as<float2>(), ctx->error_flag.as<int>(), ctx->stream),
       "generation adjoint launch");
    ctx->launches += 2;
    return MRAYGB_OK;
}
