/*
 * ORACLE — test infrastructure only.
 *
 * A C-ABI harness around the reference's OWN CPU implementation (TobiasRp/mray, compiled from its sources
 * where they lie by oracle/Makefile into oracle/_ref/).  It is used in the development container to pin
 * the C restatement (mray_oracle.c) and to write the golden fixtures under tests/golden/.  It only calls
 * the reference's functions; it computes nothing of its own except copying data in and out and, for the
 * float colour output, the per-pixel loop of reconstruct_host (moment_raymarcher.cpp:283-327) without its
 * final u8 store.
 */
#include "../include/mraygb_types.h"

#include "moment_raymarcher.h"
#include "raymarch_generate.h"
#include "raymarch_reconstruct.h"
#include "raymarch_reference.h"
#include "moment_compaction.h"
#include "moment_image.h"
#include "moment_image_sample.h"
#include "moment_quantization.h"
#include "coding_transform.h"
#include "moment_prediction_coding.h"
#include "mese/MESE_dynamic.h"
#include "mese/MESE_4_10.h"
#include "transfer_function.h"
#include "color_image.h"
#include "volume.h"
#include "cut/raytracing.h"
#include "single_scattering_image.h"
#include "single_scattering_cache.h"
#include "moment_image_io.h"
#include "moment_image_coding.h"

#include <omp.h>

#include <chrono>
#include <cstring>

/* defined in transfer_function.cpp without a header declaration */
TransferFunction preintegrate(const array<Vec4f, TransferFunction::RESOLUTION> &tf1d, float step_size);

namespace
{
cut::Camera to_camera(const mraygb_camera *c)
{
    cut::Camera cam;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            cam.transform[i][j] = c->transform[i][j];
    cam.position = Vec3f(c->position[0], c->position[1], c->position[2]);
    cam.right = Vec3f(c->right[0], c->right[1], c->right[2]);
    cam.up = Vec3f(c->up[0], c->up[1], c->up[2]);
    cam.dir = Vec3f(c->dir[0], c->dir[1], c->dir[2]);
    cam.scale = c->scale;
    cam.aspect = c->aspect;
    cam.znear = c->znear;
    cam.orthographic = c->orthographic != 0;
    return cam;
}

GenerationParameters to_gen(const mraygb_generation_params *g)
{
    GenerationParameters p;
    p.step_size = g->step_size;
    p.step_size_write_samples = g->step_size_write_samples;
    p.data_min = g->data_min;
    p.data_max = g->data_max;
    p.error_threshold = g->error_threshold;
    p.bias = g->bias;
    p.compact_image = g->compact_image != 0;
    p.prediction_coding = g->prediction_coding != 0;
    p.compress = g->compress != 0;
    p.entropy_coding = g->entropy_coding != 0;
    p.quantization_bits = g->quantization_bits;
    p.coding_warp = g->coding_warp;
    p.quantization_curve_sampling = g->quantization_curve_sampling;
    p.transform_to_bounds = g->transform_to_bounds != 0;
    p.transform_bound_eps = g->transform_bound_eps;
    return p;
}

SingleScatteringParameters to_ss(const mraygb_single_scattering_params &s);

ReconstructionParameters to_rec(const mraygb_reconstruction_params *r)
{
    ReconstructionParameters p;
    p.bias = r->bias;
    p.medium_emission = r->medium_emission;
    p.medium_scattering = r->medium_scattering;
    p.early_ray_termination = r->early_ray_termination;
    p.data_min = r->data_min;
    p.data_max = r->data_max;
    p.step_size = r->step_size;
    p.step_size_write_samples = r->step_size_write_samples;
    p.use_truncated_fourier = r->use_truncated_fourier != 0;
    p.ss = to_ss(r->ss);
    return p;
}

Range<Vec3f> to_range(const float *mn, const float *mx)
{
    return Range<Vec3f>(Vec3f(mn[0], mn[1], mn[2]), Vec3f(mx[0], mx[1], mx[2]));
}

/* A MomentImageHost from flat arrays (compact when index != nullptr). */
MomentImageHost make_mi(int w, int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                        const uint16_t *bounds, int prediction_code, int coding_warp, const uint16_t *coding_params,
                        const float *dmin, const float *dmax)
{
    MomentImageHost mi(w, h, m, index != nullptr, bounds != nullptr);
    if (index)
    {
        std::memcpy(mi.index.data(), index, sizeof(uint32_t) * (size_t(w) * h + 1));
        mi.is_compact = true;
    }
    mi.data.assign(data, data + data_size);
    if (bounds)
        for (size_t i = 0; i < size_t(w) * h; ++i)
        {
            mi.bounds[i].lower = bounds[2 * i];
            mi.bounds[i].upper = bounds[2 * i + 1];
        }
    mi.prediction_code = prediction_code != 0;
    mi.coding_warp = static_cast<CodingWarpType>(coding_warp);
    if (prediction_code && coding_warp == CODING_WARP_DEFAULT_TRANSFORMED && coding_params)
        for (int i = 0; i < m - 1; ++i)
            mi.coding_params.push_back(CodingParamType{coding_params[2 * i], coding_params[2 * i + 1]});
    if (dmin)
        mi.domain = to_range(dmin, dmax);
    return mi;
}

SingleScatteringParameters to_ss(const mraygb_single_scattering_params &s)
{
    SingleScatteringParameters p;
    p.enable = s.enable != 0;
    p.use_cache = s.use_cache != 0;
    p.cache_size_x = s.cache_size_x;
    p.cache_size_y = s.cache_size_y;
    p.cache_size_z = s.cache_size_z;
    p.step_size_factor = s.step_size_factor;
    p.henyey_greenstein_g = s.henyey_greenstein_g;
    p.direction_x = s.direction_x;
    p.direction_y = s.direction_y;
    p.direction_z = s.direction_z;
    p.intensity_r = s.intensity_r;
    p.intensity_g = s.intensity_g;
    p.intensity_b = s.intensity_b;
    return p;
}

ReferenceParameters to_ref(const mraygb_reference_params *r)
{
    ReferenceParameters p;
    p.step_size = r->step_size;
    p.medium_emission = r->medium_emission;
    p.medium_scattering = r->medium_scattering;
    p.early_ray_termination = r->early_ray_termination;
    p.data_min = r->data_min;
    p.data_max = r->data_max;
    p.ss.enable = r->ss.enable != 0;
    p.ss.use_cache = r->ss.use_cache != 0;
    p.ss.cache_size_x = r->ss.cache_size_x;
    p.ss.cache_size_y = r->ss.cache_size_y;
    p.ss.cache_size_z = r->ss.cache_size_z;
    p.ss.step_size_factor = r->ss.step_size_factor;
    p.ss.henyey_greenstein_g = r->ss.henyey_greenstein_g;
    p.ss.direction_x = r->ss.direction_x;
    p.ss.direction_y = r->ss.direction_y;
    p.ss.direction_z = r->ss.direction_z;
    p.ss.intensity_r = r->ss.intensity_r;
    p.ss.intensity_g = r->ss.intensity_g;
    p.ss.intensity_b = r->ss.intensity_b;
    return p;
}

ErrorReconstructionParameters to_err(const mraygb_error_params *e)
{
    ErrorReconstructionParameters p;
    p.error_type = e->error_type;
    p.error_percentile = e->error_percentile;
    p.bias = e->bias;
    p.data_min = e->data_min;
    p.data_max = e->data_max;
    p.step_size = e->step_size;
    return p;
}

UncertaintyReconstructionParameters to_unc(const mraygb_uncertainty_params *u)
{
    UncertaintyReconstructionParameters p;
    p.rec = to_rec(&u->rec);
    p.bound_interpolation = u->bound_interpolation;
    p.error_type = u->error_type;
    return p;
}

TransferFunction make_tf2d(const float *table)
{
    TransferFunction tf;
    for (int i = 0; i < TransferFunction::RESOLUTION * TransferFunction::RESOLUTION; ++i)
        tf.data[i] = Vec4f(table[4 * i], table[4 * i + 1], table[4 * i + 2], table[4 * i + 3]);
    return tf;
}

TransferFunction make_tf(const float *row)
{
    TransferFunction tf;
    for (int y = 0; y < TransferFunction::RESOLUTION; ++y)
        for (int x = 0; x < TransferFunction::RESOLUTION; ++x)
            tf.data[y * TransferFunction::RESOLUTION + x] =
                Vec4f(row[4 * x], row[4 * x + 1], row[4 * x + 2], row[4 * x + 3]);
    return tf;
}
} // namespace

// transfer_function.cpp defines the two filters of read_from_disk_uncertainty without declaring them in a header
TransferFunction box_filter(array<Vec4f, TransferFunction::RESOLUTION> tf1d, float step_size);
TransferFunction gaussian_filter(array<Vec4f, TransferFunction::RESOLUTION> tf1d, float step_size);

extern "C" {

/* generate() -> generate_host (moment_raymarcher.cpp:121-183) with the MomentImageHost that main.cpp:300
 * builds.  out_data needs W*H*m floats. */
int ref_generate_grid(const mraygb_camera *c, const mraygb_generation_params *g, const float *vol, int nx, int ny,
                      int nz, const float *dmin, const float *dmax, int w, int h, int m, float *out_data,
                      uint32_t *out_index, uint16_t *out_bounds, uint16_t *out_coding_params, uint64_t *out_size,
                      int *out_flags)
{
    auto gp = to_gen(g);
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    MomentImageHost mi(w, h, m, gp.compact_image, gp.transform_to_bounds);
    mi.domain = grid.domain;
    generate(to_camera(c), grid, mi, gp);
    std::memcpy(out_data, mi.data.data(), sizeof(float) * mi.data.size());
    *out_size = mi.data.size();
    if (out_index && !mi.index.empty())
        std::memcpy(out_index, mi.index.data(), sizeof(uint32_t) * mi.index.size());
    if (out_bounds && mi.has_bounds())
        for (size_t i = 0; i < mi.bounds.size(); ++i)
        {
            out_bounds[2 * i] = mi.bounds[i].lower;
            out_bounds[2 * i + 1] = mi.bounds[i].upper;
        }
    if (out_coding_params)
        for (size_t i = 0; i < mi.coding_params.size(); ++i)
        {
            out_coding_params[2 * i] = mi.coding_params[i].param1;
            out_coding_params[2 * i + 1] = mi.coding_params[i].param2;
        }
    out_flags[0] = mi.is_compact;
    out_flags[1] = mi.prediction_code;
    out_flags[2] = mi.coding_warp;
    out_flags[3] = mi.has_bounds();
    return 0;
}

/* A RegularGrid held between calls (the CPU baseline times the path, not the copy of the volume). */
void *ref_grid_create(const float *vol, int nx, int ny, int nz, const float *dmin, const float *dmax)
{
    return new RegularGrid(Vec3i(nx, ny, nz), to_range(dmin, dmax),
                           std::vector<float>(vol, vol + size_t(nx) * ny * nz), RegularGrid::DataType::F32);
}
void ref_grid_destroy(void *grid) { delete static_cast<RegularGrid *>(grid); }
/* the grid's own sample buffer (RegularGrid::data, the std::vector the reference's loaders fill) */
const float *ref_grid_data(const void *grid) { return static_cast<const RegularGrid *>(grid)->data.data(); }

/* The generate and reconstruct flows of main.cpp (generate() with compaction and prediction coding, the codes of
 * quantize_prediction_coding with `table`, dequantize_prediction_coding, reconstruct()) restricted to the rows
 * y = row0 (mod row_step) of a W x H image, with the reference's own code: the per-pixel body of generate_host
 * (moment_raymarcher.cpp:129-157: generate_ray and compute_num_moments) on the sampled rows, then
 * MomentImageHost::compact and prediction_encode (the other pixels hold no moments), the quantizer and its inverse,
 * and the per-pixel body of reconstruct_host (moment_raymarcher.cpp:296-325) on the sampled rows.  OpenMP over the
 * sampled pixels (the reference's loops go over rows, which a sample of a few rows would leave to a few threads).
 * out_rgba: W*H*4 floats or nullptr; returns the number of sampled rays. */
int64_t ref_pipeline_rows(const void *grid_handle, const mraygb_camera *c, const mraygb_generation_params *g,
                          const mraygb_reconstruction_params *r, int w, int h, int m, int row0, int row_step,
                          const uint8_t *table, const float *tf_row, float *out_rgba)
{
    const RegularGrid &grid = *static_cast<const RegularGrid *>(grid_handle);
    auto gp = to_gen(g);
    auto params = to_rec(r);
    auto cam = to_camera(c);
    MomentImageHost img(w, h, m, gp.compact_image, gp.transform_to_bounds);
    img.domain = grid.domain;
    const int nrows = row0 < h ? (h - 1 - row0) / row_step + 1 : 0;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = 0; i < int64_t(nrows) * w; ++i)
    {
        const int y = row0 + int(i / w) * row_step;
        const int x = int(i % w);
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            auto idx = img.get_idx(x, y);
            vector<float> trig_moments(m, 0.0f);
            auto b = generate_ray(grid, get_eye_ray(cam, ndc), cam.znear, trig_moments.data(), &img.data[idx], m, gp);
            if (img.has_bounds())
                img.bounds[y * w + x] = b;
            if (gp.compact_image)
            {
                vector<float_complex> t0(m), t1(m), t2(m);
                compute_num_moments(img, x, y, gp.error_threshold, t0.data(), t1.data(), t2.data());
            }
        }
    }
    // the rows not sampled hold no moments
    if (gp.compact_image)
        for (int y = 0; y < h; ++y)
            if (y < row0 || (y - row0) % row_step != 0)
                for (int x = 0; x < w; ++x)
                    img.index[y * w + x] = 0;
    if (gp.compact_image)
        img.compact();
    if (gp.prediction_coding)
        img.prediction_encode(gp.coding_warp, gp.bias);
    if (table && gp.prediction_coding)
    {
        std::vector<Byte> t(table, table + m);
        auto qs = moment_quantization::quantize_prediction_coding(img, t);
        moment_quantization::dequantize_prediction_coding(img, t, qs);
    }
    auto tf = make_tf(tf_row);
    NoSingleScattering ss;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = 0; i < int64_t(nrows) * w; ++i)
    {
        const int y = row0 + int(i / w) * row_step;
        const int x = int(i % w);
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color;
            if (img.get_num_moments(x, y) == 0)
                color = reconstruct_zero_ray(tf);
            else
            {
                auto pm = img.prepare_moments(x, y, params.bias);
                MESEReconstructionDefault rec(pm.size(), pm.data(), img.get_bounds(x, y));
                color = reconstruct_ray(cut::get_eye_ray(cam, ndc), img.domain, cam.znear, rec, tf, ss, params);
            }
            if (out_rgba)
            {
                float *o = out_rgba + 4 * (size_t(y) * w + x);
                o[0] = color.x;
                o[1] = color.y;
                o[2] = color.z;
                o[3] = color.w;
            }
        }
    }
    return int64_t(nrows) * w;
}

/* Wall-clock milliseconds of the reference's own generate() and reconstruct() calls (moment_raymarcher.cpp:
 * 168-183, 329-337) on a grid held between calls, as main.cpp's --generate / --reconstruct make them: a fresh
 * MomentImageHost per generate (outside the timing), then reconstruct of the image generate returned.  They
 * dispatch to whatever generate_device / reconstruct_device the library was linked with: the reference's
 * moment_raymarcher.cu (Makefile refcuda) or the drop-in shim over libmraygb.so (Makefile shim).  out_ms holds
 * 2 * steps values (generate, reconstruct per step); out_rgba8 (W*H*4 bytes, or nullptr) the last colours. */
int ref_time_flow(const void *grid_handle, const mraygb_camera *c, const mraygb_generation_params *g,
                  const mraygb_reconstruction_params *r, int w, int h, int m, const float *tf_row, int warmup,
                  int steps, double *out_ms, uint8_t *out_rgba8, uint64_t *out_data_size)
{
    const RegularGrid &grid = *static_cast<const RegularGrid *>(grid_handle);
    auto gp = to_gen(g);
    auto params = to_rec(r);
    auto cam = to_camera(c);
    auto tf = make_tf(tf_row);
    ColorImageHost cimg(w, h);
    for (int i = 0; i < warmup + steps; ++i)
    {
        MomentImageHost img(w, h, m, gp.compact_image, gp.transform_to_bounds);
        const auto t0 = std::chrono::steady_clock::now();
        generate(cam, grid, img, gp);
        const auto t1 = std::chrono::steady_clock::now();
        reconstruct(cam, img, tf, cimg, params);
        const auto t2 = std::chrono::steady_clock::now();
        if (i >= warmup)
        {
            out_ms[2 * (i - warmup)] = std::chrono::duration<double, std::milli>(t1 - t0).count();
            out_ms[2 * (i - warmup) + 1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
        }
        if (out_data_size)
            *out_data_size = img.data.size();
    }
    if (out_rgba8)
        std::memcpy(out_rgba8, cimg.rgba.data(), 4 * size_t(w) * h);
    return 0;
}

/* Particles::sample (volume.cpp:83-94) at npts points, with the grid Particles builds (volume.cpp:55-81). */
int ref_particles_sample(const float *x, const float *y, const float *z, const float *v, uint64_t n, float h,
                         const float *dmin, const float *dmax, const float *pts, uint64_t npts, float *out)
{
    Particles parts(to_range(dmin, dmax), std::vector<float>(x, x + n), std::vector<float>(y, y + n),
                    std::vector<float>(z, z + n), std::vector<float>(v, v + n), h);
    for (uint64_t i = 0; i < npts; ++i)
        out[i] = parts.sample(Vec3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    return 0;
}

/* generate() over Particles -> generate_host (moment_raymarcher.cpp:121-175). */
int ref_generate_particles(const mraygb_camera *c, const mraygb_generation_params *g, const float *x, const float *y,
                           const float *z, const float *v, uint64_t n, float h, const float *dmin, const float *dmax,
                           int w, int hgt, int m, float *out_data, uint32_t *out_index, uint16_t *out_bounds,
                           uint64_t *out_size)
{
    auto gp = to_gen(g);
    Particles parts(to_range(dmin, dmax), std::vector<float>(x, x + n), std::vector<float>(y, y + n),
                    std::vector<float>(z, z + n), std::vector<float>(v, v + n), h);
    MomentImageHost mi(w, hgt, m, gp.compact_image, gp.transform_to_bounds);
    mi.domain = parts.domain;
    generate(to_camera(c), parts, mi, gp);
    std::memcpy(out_data, mi.data.data(), sizeof(float) * mi.data.size());
    *out_size = mi.data.size();
    if (out_index && !mi.index.empty())
        std::memcpy(out_index, mi.index.data(), sizeof(uint32_t) * mi.index.size());
    if (out_bounds && mi.has_bounds())
        for (size_t i = 0; i < mi.bounds.size(); ++i)
        {
            out_bounds[2 * i] = mi.bounds[i].lower;
            out_bounds[2 * i + 1] = mi.bounds[i].upper;
        }
    return 0;
}

/* reconstruct() -> reconstruct_host (moment_raymarcher.cpp:283-337): u8 RGBA as the reference stores it. */
int ref_reconstruct_u8(const mraygb_camera *c, const mraygb_reconstruction_params *r, int w, int h, int m,
                       const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                       int prediction_code, int coding_warp, const uint16_t *coding_params, const float *dmin,
                       const float *dmax, const float *tf_row, uint8_t *out_rgba8)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    auto tf = make_tf(tf_row);
    ColorImageHost img(w, h);
    reconstruct(to_camera(c), mi, tf, img, to_rec(r));
    std::memcpy(out_rgba8, img.rgba.data(), 4 * size_t(w) * h);
    return 0;
}

/* The per-pixel body of reconstruct_host (moment_raymarcher.cpp:296-325, MESE branch) keeping the float colour. */
int ref_reconstruct_float(const mraygb_camera *c, const mraygb_reconstruction_params *r, int w, int h, int m,
                          const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                          int prediction_code, int coding_warp, const uint16_t *coding_params, const float *dmin,
                          const float *dmax, const float *tf_row, float *out_rgba)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    auto tf = make_tf(tf_row);
    auto cam = to_camera(c);
    auto params = to_rec(r);
    NoSingleScattering ss;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color;
            if (mi.get_num_moments(x, y) == 0)
                color = reconstruct_zero_ray(tf);
            else
            {
                auto pm = mi.prepare_moments(x, y, params.bias);
                MESEReconstructionDefault rec(pm.size(), pm.data(), mi.get_bounds(x, y));
                color = reconstruct_ray(cut::get_eye_ray(cam, ndc), mi.domain, cam.znear, rec, tf, ss, params);
            }
            float *o = out_rgba + 4 * (size_t(y) * w + x);
            o[0] = color.x;
            o[1] = color.y;
            o[2] = color.z;
            o[3] = color.w;
        }
    return 0;
}

/* MomentImageHost::prepare_moments (moment_image.cpp:154-183) for every pixel; output in the data layout. */
int ref_prepare_moments(int w, int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                        int prediction_code, int coding_warp, const uint16_t *coding_params, float bias, float *out)
{
    auto mi =
        make_mi(w, h, m, index, data, data_size, nullptr, prediction_code, coding_warp, coding_params, nullptr, nullptr);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            if (mi.get_num_moments(x, y) == 0)
                continue;
            auto pm = mi.prepare_moments(x, y, bias);
            std::memcpy(out + mi.get_idx(x, y), pm.data(), sizeof(float) * pm.size());
        }
    return 0;
}

/* MomentImageHost::prediction_encode (moment_image.cpp:96-152), in place. */
int ref_prediction_encode(int w, int h, int m, const uint32_t *index, float *data, uint64_t data_size, int warp,
                          float bias, uint16_t *out_coding_params)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, 0, warp, nullptr, nullptr, nullptr);
    mi.prediction_encode(warp, bias);
    std::memcpy(data, mi.data.data(), sizeof(float) * data_size);
    if (out_coding_params)
        for (size_t i = 0; i < mi.coding_params.size(); ++i)
        {
            out_coding_params[2 * i] = mi.coding_params[i].param1;
            out_coding_params[2 * i + 1] = mi.coding_params[i].param2;
        }
    return 0;
}

/* find_coding_transform_parameters (coding_transform.h:37-68). */
int ref_find_coding_transform_parameters(int w, int h, int m, const uint32_t *index, const float *data,
                                         uint64_t data_size, float *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, 0, 0, nullptr, nullptr, nullptr);
    auto p = find_coding_transform_parameters(mi);
    std::memcpy(out, p.data(), sizeof(float) * p.size());
    return 0;
}

/* moment_quantization::quantize_prediction_coding (moment_quantization.cpp:239-276).  Returns the byte count;
 * out may be nullptr. */
uint64_t ref_quantize_prediction_coding(int w, int h, int m, const uint32_t *index, const float *data,
                                        uint64_t data_size, const uint8_t *table, uint8_t *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, 1, 0, nullptr, nullptr, nullptr);
    std::vector<Byte> t(table, table + m);
    auto bytes = moment_quantization::quantize_prediction_coding(mi, t);
    if (out)
        std::memcpy(out, bytes.data(), bytes.size());
    return bytes.size();
}

/* sample_moment_image (moment_image_sample.h:33-62) of a compact image: s x s pixels.  s_index receives s*s+1
 * offsets, s_data (may be nullptr) the compact data; returns the data size. */
uint64_t ref_sample_moment_image(int w, int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                                 int s, uint32_t *s_index, float *s_data)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, 1, 0, nullptr, nullptr, nullptr);
    auto simg = sample_moment_image(mi, s, s);
    std::memcpy(s_index, simg.index.data(), sizeof(uint32_t) * simg.index.size());
    if (s_data)
        std::memcpy(s_data, simg.data.data(), sizeof(float) * simg.data.size());
    return simg.data.size();
}

/* Per-pixel rRMSE of compute_coding_error (measure_coding_error.cpp:143-182) against compute_reference
 * (:92-141) for the image whose moment idx is quantized to b bits (apply_quantization, :41-66; idx < 0: none),
 * evaluated with the reference's MomentImageHost, transform_dequantization_real, decode and
 * exponentialToTrigonometricMoments.  measure_coding_error.cpp itself includes the HDF5 headers and is not
 * compiled here, so its two loops are spelled out below around those calls.  errors[i] belongs to the i-th
 * non-empty pixel in row-major order; returns the number of non-empty pixels. */
uint32_t ref_coding_errors(int w, int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                           int warp, const uint16_t *coding_params, int idx, int b, float *errors)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, 1, warp, coding_params, nullptr, nullptr);
    const std::vector<float> params = mi.get_coding_params();
    auto trig = [&](const float *in, int n, std::vector<float> &out) {
        std::vector<float_complex> code(n), e(n), poly(n), tmp(n);
        transform_dequantization_real(n, in, code.data(), WarpParameters{mi.coding_warp, params.data()});
        decode(n, code.data(), e.data(), poly.data(), tmp.data());
        exponentialToTrigonometricMoments(n, tmp.data(), e.data());
        out.resize(n);
        for (int l = 0; l < n; ++l)
            out[l] = tmp[l].x;
    };
    uint32_t k = 0;
    std::vector<float> ref, q, in;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            int n = mi.get_num_moments(x, y);
            if (n <= 0)
                continue;
            const float *src = &mi.data[mi.get_idx(x, y)];
            trig(src, n, ref);
            in.assign(src, src + n);
            if (idx >= 0 && n > idx)
            {
                float p = std::pow(2.0f, float(b));
                in[idx] = std::floor(in[idx] * p) / p;
            }
            trig(in.data(), n, q);
            float sum = 0.0f;
            for (int l = 0; l < n; ++l)
            {
                float diff = ref[l] - q[l];
                sum += diff * diff;
            }
            errors[k++] = sqrtf(sum) / ref[0];
        }
    return k;
}

/* reconstruct_error (moment_raymarcher.cpp:552-560, host form :516-539) over a float grid: the u16 error bounds. */
int ref_reconstruct_error(const mraygb_camera *c, const mraygb_error_params *e, const float *vol, int nx, int ny,
                          int nz, const float *dmin, const float *dmax, int w, int h, int m, const uint32_t *index,
                          const float *data, uint64_t data_size, const uint16_t *bounds, int prediction_code,
                          int coding_warp, const uint16_t *coding_params, uint16_t *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    mi.add_error_bounds();
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    reconstruct_error(to_camera(c), grid, mi, to_err(e));
    std::memcpy(out, mi.error_bounds.data(), sizeof(uint16_t) * mi.error_bounds.size());
    return 0;
}

/* read_from_disk_uncertainty's filters (transfer_function.cpp:151-248) on a float 1D table: 256 x 256 RGBA. */
int ref_uncertainty_tf(const float *tf1d, float step_size, int error_type, float *out)
{
    array<Vec4f, TransferFunction::RESOLUTION> t;
    for (int i = 0; i < TransferFunction::RESOLUTION; ++i)
        t[i] = Vec4f(tf1d[4 * i], tf1d[4 * i + 1], tf1d[4 * i + 2], tf1d[4 * i + 3]);
    auto tf = (error_type == RMSE) ? gaussian_filter(t, step_size) : box_filter(t, step_size);
    for (size_t i = 0; i < tf.data.size(); ++i)
    {
        out[4 * i] = tf.data[i].x;
        out[4 * i + 1] = tf.data[i].y;
        out[4 * i + 2] = tf.data[i].z;
        out[4 * i + 3] = tf.data[i].w;
    }
    return 0;
}

/* reconstruct_uncertainty_interpolation (mode 0, on a preintegrated row) / reconstruct_uncertainty_convolution
 * (mode 1, on a 256 x 256 table) (moment_raymarcher.cpp:562-717): u8 RGBA as the reference stores it. */
int ref_reconstruct_uncertainty_u8(const mraygb_camera *c, const mraygb_uncertainty_params *u, int mode, int w,
                                   int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                                   const uint16_t *bounds, const uint16_t *error_bounds, int prediction_code,
                                   int coding_warp, const uint16_t *coding_params, const float *dmin,
                                   const float *dmax, const float *table, uint8_t *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    mi.add_error_bounds();
    std::memcpy(mi.error_bounds.data(), error_bounds, sizeof(uint16_t) * size_t(w) * h);
    auto tf = mode == 0 ? make_tf(table) : make_tf2d(table);
    ColorImageHost img(w, h);
    if (mode == 0)
        reconstruct_uncertainty_interpolation(to_camera(c), mi, tf, img, to_unc(u));
    else
        reconstruct_uncertainty_convolution(to_camera(c), mi, tf, img, to_unc(u));
    std::memcpy(out, img.rgba.data(), 4 * size_t(w) * h);
    return 0;
}

/* The per-pixel bodies of the two uncertainty renderers (MESE branches, moment_raymarcher.cpp:581-604, 660-688)
 * keeping the float colour. */
int ref_reconstruct_uncertainty_float(const mraygb_camera *c, const mraygb_uncertainty_params *u, int mode, int w,
                                      int h, int m, const uint32_t *index, const float *data, uint64_t data_size,
                                      const uint16_t *bounds, const uint16_t *error_bounds, int prediction_code,
                                      int coding_warp, const uint16_t *coding_params, const float *dmin,
                                      const float *dmax, const float *table, float *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    mi.add_error_bounds();
    std::memcpy(mi.error_bounds.data(), error_bounds, sizeof(uint16_t) * size_t(w) * h);
    auto tf = mode == 0 ? make_tf(table) : make_tf2d(table);
    auto cam = to_camera(c);
    auto params = to_unc(u);
    NoSingleScattering ss;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color;
            if (mi.get_num_moments(x, y) == 0)
                color = reconstruct_zero_ray(tf);
            else
            {
                auto pm = mi.prepare_moments(x, y, params.rec.bias);
                MESEReconstructionDefault mese(pm.size(), pm.data(), mi.get_bounds(x, y));
                auto ray = cut::get_eye_ray(cam, ndc);
                if (mode == 0)
                {
                    ErrorBoundMESEReconstruction<MESEReconstructionDefault> bound_rec(mese, mi.get_error_bound(x, y));
                    ErrorBoundInterpolator<ErrorBoundMESEReconstruction<MESEReconstructionDefault>> interp(
                        bound_rec, params.bound_interpolation);
                    color = reconstruct_ray(ray, mi.domain, cam.znear, interp, tf, ss, params.rec);
                }
                else if (params.error_type == MAX_ERROR)
                {
                    ErrorBoundMESEReconstruction<MESEReconstructionDefault> bound_rec(mese, mi.get_error_bound(x, y));
                    color = reconstruct_ray_uncertainty_tf(ray, mi.domain, cam.znear, bound_rec, tf, ss, params.rec);
                }
                else
                {
                    MeanStdDevMESEReconstruction<MESEReconstructionDefault> bound_rec(mese, mi.get_error_bound(x, y));
                    color = reconstruct_ray_uncertainty_tf(ray, mi.domain, cam.znear, bound_rec, tf, ss, params.rec);
                }
            }
            float *o = out + 4 * (size_t(y) * w + x);
            o[0] = color.x;
            o[1] = color.y;
            o[2] = color.z;
            o[3] = color.w;
        }
    return 0;
}

/* generate_reference (moment_raymarcher.cpp:74-80 -> reference_host :45-61) over a float grid: u8 RGBA. */
int ref_generate_reference_u8(const mraygb_camera *c, const mraygb_reference_params *r, const float *vol, int nx,
                              int ny, int nz, const float *dmin, const float *dmax, int w, int h, const float *tf_row,
                              uint8_t *out)
{
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    auto tf = make_tf(tf_row);
    ColorImageHost img(w, h);
    generate_reference(to_camera(c), tf, grid, img, to_ref(r));
    std::memcpy(out, img.rgba.data(), 4 * size_t(w) * h);
    return 0;
}

/* The per-pixel body of reference_host (reference_ray with SingleScatteringBruteForce) keeping the float colour. */
int ref_generate_reference_float(const mraygb_camera *c, const mraygb_reference_params *r, const float *vol, int nx,
                                 int ny, int nz, const float *dmin, const float *dmax, int w, int h,
                                 const float *tf_row, float *out)
{
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    auto tf = make_tf(tf_row);
    auto cam = to_camera(c);
    auto params = to_ref(r);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color = reference_ray(grid, cut::get_eye_ray(cam, ndc), cam.znear, tf, SingleScatteringBruteForce{},
                                        params);
            float *o = out + 4 * (size_t(y) * w + x);
            o[0] = color.x;
            o[1] = color.y;
            o[2] = color.z;
            o[3] = color.w;
        }
    return 0;
}

/* ---- single scattering from the transmittance cache ---- */

// defined in moment_raymarcher.cpp:217-258 without a header declaration
extern "C++" SingleScatteringCacheHost reconstruct_single_scattering_cache(const SingleScatteringImageHost &ss,
                                                                           const TransferFunction &tf,
                                                                           const ReconstructionParameters &params);

/* reconstruct_single_scattering_cache (moment_raymarcher.cpp:217-258) on one OpenMP thread, so that its racing
 * writes come in the loop's order; out: cache_size_z*y*x floats. */
int ref_ss_cache(const mraygb_camera *light, const mraygb_reconstruction_params *r, int w, int h, int m,
                 const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                 int prediction_code, int coding_warp, const uint16_t *coding_params, const float *dmin,
                 const float *dmax, const float *tf_row, float *out)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    SingleScatteringImageHost ss(to_camera(light), mi);
    auto tf = make_tf(tf_row);
    const int threads = omp_get_max_threads();
    omp_set_num_threads(1);
    auto cache = reconstruct_single_scattering_cache(ss, tf, to_rec(r));
    omp_set_num_threads(threads);
    const Vec3i sz = cache.cache.size;
    for (int z = 0; z < sz.z; ++z)
        for (int y = 0; y < sz.y; ++y)
            for (int x = 0; x < sz.x; ++x)
                out[(size_t(z) * sz.y + y) * sz.x + x] = cache.cache.get(x, y, z);
    return 0;
}

SingleScatteringCacheHost make_cache(const float *cache, int cx, int cy, int cz, const float *cmin, const float *cmax)
{
    return SingleScatteringCacheHost(RegularGrid(Vec3i(cx, cy, cz), to_range(cmin, cmax),
                                                 std::vector<float>(cache, cache + size_t(cx) * cy * cz),
                                                 RegularGrid::DataType::F32));
}

/* The per-pixel body of reconstruct_host with a SingleScatteringCacheHost (moment_raymarcher.cpp:283-327) keeping
 * the float colour. */
int ref_reconstruct_cached_float(const mraygb_camera *c, const mraygb_reconstruction_params *r, int w, int h, int m,
                                 const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                                 int prediction_code, int coding_warp, const uint16_t *coding_params,
                                 const float *dmin, const float *dmax, const float *tf_row, const float *cache, int cx,
                                 int cy, int cz, const float *cmin, const float *cmax, float *out_rgba)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    auto tf = make_tf(tf_row);
    auto cam = to_camera(c);
    auto params = to_rec(r);
    auto ss = make_cache(cache, cx, cy, cz, cmin, cmax);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color;
            if (mi.get_num_moments(x, y) == 0)
                color = reconstruct_zero_ray(tf);
            else
            {
                auto pm = mi.prepare_moments(x, y, params.bias);
                MESEReconstructionDefault rec(pm.size(), pm.data(), mi.get_bounds(x, y));
                color = reconstruct_ray(cut::get_eye_ray(cam, ndc), mi.domain, cam.znear, rec, tf, ss, params);
            }
            float *o = out_rgba + 4 * (size_t(y) * w + x);
            o[0] = color.x;
            o[1] = color.y;
            o[2] = color.z;
            o[3] = color.w;
        }
    return 0;
}

/* reconstruct(cam, mi, tf, img, ss, params) (moment_raymarcher.cpp:339-351) end to end, u8 RGBA, the cache built
 * on one OpenMP thread. */
int ref_reconstruct_ss_u8(const mraygb_camera *c, const mraygb_reconstruction_params *r, int w, int h, int m,
                          const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                          int prediction_code, int coding_warp, const uint16_t *coding_params, const float *dmin,
                          const float *dmax, const mraygb_camera *light, int lw, int lh, int lm,
                          const uint32_t *lindex, const float *ldata, uint64_t ldata_size, const uint16_t *lbounds,
                          int lprediction_code, int lcoding_warp, const uint16_t *lcoding_params, const float *tf_row,
                          uint8_t *out_rgba8)
{
    auto mi = make_mi(w, h, m, index, data, data_size, bounds, prediction_code, coding_warp, coding_params, dmin,
                      dmax);
    auto lmi = make_mi(lw, lh, lm, lindex, ldata, ldata_size, lbounds, lprediction_code, lcoding_warp, lcoding_params,
                       dmin, dmax);
    SingleScatteringImageHost ss(to_camera(light), lmi);
    auto tf = make_tf(tf_row);
    ColorImageHost img(w, h);
    const int threads = omp_get_max_threads();
    omp_set_num_threads(1);
    reconstruct(to_camera(c), mi, tf, img, ss, to_rec(r));
    omp_set_num_threads(threads);
    std::memcpy(out_rgba8, img.rgba.data(), 4 * size_t(w) * h);
    return 0;
}

/* The per-pixel body of generate_reference_reconstructed_ss (moment_raymarcher.cpp:259-281: reference_host with
 * the cache and ref_from_rec_params) keeping the float colour. */
int ref_generate_reference_cached_float(const mraygb_camera *c, const mraygb_reconstruction_params *r,
                                        const float *vol, int nx, int ny, int nz, const float *dmin, const float *dmax,
                                        int w, int h, const float *tf_row, const float *cache, int cx, int cy, int cz,
                                        const float *cmin, const float *cmax, float *out)
{
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    auto tf = make_tf(tf_row);
    auto cam = to_camera(c);
    auto params = ref_from_rec_params(to_rec(r));
    auto ss = make_cache(cache, cx, cy, cz, cmin, cmax);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
            Vec4f color = reference_ray(grid, cut::get_eye_ray(cam, ndc), cam.znear, tf, ss, params);
            float *o = out + 4 * (size_t(y) * w + x);
            o[0] = color.x;
            o[1] = color.y;
            o[2] = color.z;
            o[3] = color.w;
        }
    return 0;
}

/* ---- the moment-image file format (moment_image_io.cpp, moment_image_coding.cpp) ---- */

namespace
{
MomentImageHost file_image(int w, int h, int m, int compact, int pc, int warp, const float *dmin, const float *dmax,
                           const uint32_t *index, const float *data, uint64_t data_size, const uint16_t *bounds,
                           const uint16_t *error_bounds, const uint16_t *coding_params)
{
    auto mi = make_mi(w, h, m, compact ? index : nullptr, data, data_size, bounds, pc, warp, coding_params, dmin, dmax);
    if (error_bounds)
        mi.error_bounds.assign(error_bounds, error_bounds + size_t(w) * h);
    return mi;
}
} // namespace

/* write_moment_image (moment_image_io.cpp:510-529); table: installed as the global prediction-coding table first
 * (set_prediction_coding_quantization_table; NULL leaves the global state as it is, and once set it stays set) */
int ref_write_moment_image(const char *path, int w, int h, int m, int compact, int pc, int warp, const float *dmin,
                           const float *dmax, const uint32_t *index, const float *data, uint64_t data_size,
                           const uint16_t *bounds, const uint16_t *error_bounds, const uint16_t *coding_params,
                           int compress, int bits, int entropy, const uint8_t *table)
{
    auto mi = file_image(w, h, m, compact, pc, warp, dmin, dmax, index, data, data_size, bounds, error_bounds,
                         coding_params);
    if (table)
        moment_quantization::set_prediction_coding_quantization_table(std::vector<Byte>(table, table + m));
    write_moment_image(mi, std::string(path), compress != 0, (Byte)bits, entropy != 0);
    return 0;
}

/* load_moment_image (moment_image_io.cpp:291-310).  info: w, h, m, compact, pc, warp, has bounds, has error
 * bounds, has coding params; with data NULL only info, domain (6 floats) and *data_size are written. */
int ref_load_moment_image(const char *path, int *info, float *domain, uint64_t *data_size, uint32_t *index,
                          float *data, uint16_t *bounds, uint16_t *error_bounds, uint16_t *coding_params)
{
    auto mi = load_moment_image(std::string(path));
    info[0] = mi.width;
    info[1] = mi.height;
    info[2] = mi.num_moments;
    info[3] = mi.is_compact;
    info[4] = mi.prediction_code;
    info[5] = mi.coding_warp;
    info[6] = mi.has_bounds();
    info[7] = mi.has_error_bounds();
    info[8] = mi.has_coding_params();
    domain[0] = mi.domain.min.x;
    domain[1] = mi.domain.min.y;
    domain[2] = mi.domain.min.z;
    domain[3] = mi.domain.max.x;
    domain[4] = mi.domain.max.y;
    domain[5] = mi.domain.max.z;
    *data_size = mi.data.size();
    if (!data)
        return 0;
    std::memcpy(data, mi.data.data(), mi.data.size() * sizeof(float));
    if (mi.is_compact && index)
        std::memcpy(index, mi.index.data(), mi.index.size() * sizeof(uint32_t));
    if (mi.has_bounds() && bounds)
        for (size_t i = 0; i < mi.bounds.size(); ++i)
        {
            bounds[2 * i] = mi.bounds[i].lower;
            bounds[2 * i + 1] = mi.bounds[i].upper;
        }
    if (mi.has_error_bounds() && error_bounds)
        std::memcpy(error_bounds, mi.error_bounds.data(), mi.error_bounds.size() * sizeof(uint16_t));
    if (mi.has_coding_params() && coding_params)
        for (size_t i = 0; i < mi.coding_params.size(); ++i)
        {
            coding_params[2 * i] = mi.coding_params[i].param1;
            coding_params[2 * i + 1] = mi.coding_params[i].param2;
        }
    return 0;
}

/* entropy_encode (moment_image_coding.cpp:206-221) of a compact image with the table given; returns the size, the
 * bytes when out holds them */
uint64_t ref_entropy_encode(int w, int h, int m, const uint32_t *index, const float *data, uint64_t data_size, int pc,
                            const uint8_t *table, uint8_t *out, uint64_t capacity)
{
    auto mi = make_mi(w, h, m, index, data, data_size, nullptr, pc, 1, nullptr, nullptr, nullptr);
    auto bytes = entropy_encode(mi, std::vector<Byte>(table, table + m));
    if (out && capacity >= bytes.size())
        std::memcpy(out, bytes.data(), bytes.size());
    return bytes.size();
}

/* ---- MESE primitives (mese/MESE_dynamic.h) ---- */
void ref_trig_to_exp(int n, const float *trig, float *exp_out)
{
    trigonometricToExponentialMoments(n, reinterpret_cast<float_complex *>(exp_out), trig);
}
void ref_exp_to_trig(int n, const float *exp_in, float *trig_out)
{
    exponentialToTrigonometricMoments(n, reinterpret_cast<float_complex *>(trig_out),
                                      const_cast<float_complex *>(reinterpret_cast<const float_complex *>(exp_in)));
}
void ref_levinson(int n, const float *col, float *sol)
{
    std::vector<float_complex> tmp(n);
    levinsonsAlgorithm(n, reinterpret_cast<float_complex *>(sol), const_cast<float_complex *>(reinterpret_cast<const float_complex *>(col)),
                       tmp.data());
}
void ref_prepare_lagrange(int n, const float *trig, float *out)
{
    std::vector<float_complex> a(n), b(n), c(n);
    prepareMESELagrange(n, out, trig, a.data(), b.data(), c.data());
}
float ref_evaluate_mese(int n, float phase, const float *lagrange) { return evaluateMESELagrange(n, phase, lagrange); }
float ref_fast_atan(float x) { return fast_atan(x); }
void ref_autocorrelation(int n, const float *sig, float *out)
{
    computeAutocorrelation(n, reinterpret_cast<float_complex *>(out), const_cast<float_complex *>(reinterpret_cast<const float_complex *>(sig)));
}
void ref_correlation(int n, const float *lhs, const float *rhs, float *out)
{
    computeCorrelation(n, reinterpret_cast<float_complex *>(out), const_cast<float_complex *>(reinterpret_cast<const float_complex *>(lhs)),
                       const_cast<float_complex *>(reinterpret_cast<const float_complex *>(rhs)));
}
void ref_imaginary_correlation(int n, const float *lhs, const float *rhs, float *out)
{
    computeImaginaryCorrelation(n, out, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(lhs)),
                                const_cast<float_complex *>(reinterpret_cast<const float_complex *>(rhs)));
}
void ref_encode(int n, const float *exp_in, float *code)
{
    std::vector<float_complex> poly(n), tmp(n);
    encode(n, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(exp_in)), reinterpret_cast<float_complex *>(code), poly.data(),
           tmp.data());
}
void ref_decode(int n, const float *code, float *exp_out, float *poly)
{
    std::vector<float_complex> tmp(n);
    decode(n, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(code)), reinterpret_cast<float_complex *>(exp_out),
           reinterpret_cast<float_complex *>(poly), tmp.data());
}
void ref_transform_quantization_real(int n, const float *code, float c0, float *out)
{
    transform_quantization_real(n, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(code)), c0, out);
}
void ref_transform_quantization_real_warp(int n, float *inout, int warp, const float *params)
{
    transform_quantization_real_warp(n, inout, WarpParameters{warp, params});
}
void ref_transform_dequantization_real(int n, const float *in, float *code, int warp, const float *params)
{
    transform_dequantization_real(n, in, reinterpret_cast<float_complex *>(code), WarpParameters{warp, params});
}
int ref_determine_best_number_moments(int n, const float *moments, float thr)
{
    std::vector<float_complex> a(n), b(n), c(n);
    return determine_best_number_moments(n, moments, thr, a.data(), b.data(), c.data());
}
void ref_evaluate_unknown_moments(int n, const float *exp_in, int max_moments, float *new_exp)
{
    std::vector<float_complex> lev(max_moments);
    evaluate_unknown_moments(n, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(exp_in)), max_moments,
                             reinterpret_cast<float_complex *>(new_exp), lev.data());
}
void ref_exponential_to_bounded_moments(int n, const float *exp_in, float *bounded, int known)
{
    exponential_to_bounded_moments(n, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(exp_in)),
                                   reinterpret_cast<float_complex *>(bounded), known);
}
float ref_rmse(int n, int m, const float *pred, const float *target)
{
    return rmse(n, m, const_cast<float_complex *>(reinterpret_cast<const float_complex *>(pred)), target);
}

/* ---- the independent fixed-size MESE code (mese/MESE_4_10.h) used by the reference's tests ---- */
void ref_fixed_prepare_lagrange(int n, const float *trig, float *out)
{
    if (n == 4)
        prepareReflectanceSpectrumLagrange4(out, trig);
    else
        prepareReflectanceSpectrumLagrange10(out, trig);
}
float ref_fixed_evaluate_lagrange(int n, float phase, const float *lagrange)
{
    return n == 4 ? evaluateReflectanceSpectrumLagrange4(phase, lagrange)
                  : evaluateReflectanceSpectrumLagrange10(phase, lagrange);
}
void ref_fixed_trig_to_exp(int n, const float *trig, float *exp_out)
{
    if (n == 4)
        trigonometricToExponentialMoments4(reinterpret_cast<float_complex *>(exp_out), trig);
    else
        trigonometricToExponentialMoments10(reinterpret_cast<float_complex *>(exp_out), trig);
}
void ref_fixed_levinson(int n, const float *col, float *sol)
{
    if (n == 4)
        levinsonsAlgorithm4(reinterpret_cast<float_complex *>(sol), const_cast<float_complex *>(reinterpret_cast<const float_complex *>(col)));
    else
        levinsonsAlgorithm10(reinterpret_cast<float_complex *>(sol), const_cast<float_complex *>(reinterpret_cast<const float_complex *>(col)));
}

/* ---- helpers and overload probes ---- */
void ref_euler_exp(float x, float *out)
{
    auto e = euler_exp(x);
    out[0] = e.x;
    out[1] = e.y;
}
float ref_exp_overload(float x)
{
    using namespace cut;
    return exp(-x);
}
float ref_grid_sample(const float *vol, int nx, int ny, int nz, const float *dmin, const float *dmax, const float *p)
{
    RegularGrid grid(Vec3i(nx, ny, nz), to_range(dmin, dmax), std::vector<float>(vol, vol + size_t(nx) * ny * nz),
                     RegularGrid::DataType::F32);
    return grid.sample(Vec3f(p[0], p[1], p[2]));
}
int ref_eye_ray(const mraygb_camera *c, int x, int y, int w, int h, const float *dmin, const float *dmax,
                float *out /* origin[3], dir[3], t_near, t_far */)
{
    auto cam = to_camera(c);
    Vec2f ndc(x / static_cast<float>(w) * 2.f - 1.f, y / static_cast<float>(h) * 2.f - 1.f);
    auto ray = cut::get_eye_ray(cam, ndc);
    float tn, tf;
    int hit = cut::intersect_AABB(ray, Vec3f(dmin[0], dmin[1], dmin[2]), Vec3f(dmax[0], dmax[1], dmax[2]), tn, tf);
    out[0] = ray.origin.x;
    out[1] = ray.origin.y;
    out[2] = ray.origin.z;
    out[3] = ray.dir.x;
    out[4] = ray.dir.y;
    out[5] = ray.dir.z;
    out[6] = tn;
    out[7] = tf;
    return hit;
}
/* read_from_disk's table (transfer_function.cpp:46-97) from 256 RGBA floats; writes row 0 and returns 1 when
 * every row equals row 0. */
int ref_preintegrate(const float *tf1d, float step, float *row_out)
{
    array<Vec4f, TransferFunction::RESOLUTION> t;
    for (int i = 0; i < 256; ++i)
        t[i] = Vec4f(tf1d[4 * i], tf1d[4 * i + 1], tf1d[4 * i + 2], tf1d[4 * i + 3]);
    auto tf = std::make_unique<TransferFunction>(preintegrate(t, step));
    for (int x = 0; x < 256; ++x)
    {
        auto v = tf->data[x];
        row_out[4 * x] = v.x;
        row_out[4 * x + 1] = v.y;
        row_out[4 * x + 2] = v.z;
        row_out[4 * x + 3] = v.w;
    }
    int same = 1;
    for (int y = 1; y < 256 && same; ++y)
        for (int x = 0; x < 256; ++x)
        {
            Vec4f a = tf->data[y * 256 + x];
            Vec4f b = tf->data[x];
            if (a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w)
            {
                same = 0;
                break;
            }
        }
    return same;
}
float ref_tf_sample(const float *row, float fs, float bs, float *out)
{
    auto tf = std::make_unique<TransferFunction>(make_tf(row));
    auto v = tf->sample(fs, bs);
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
    out[3] = v.w;
    return v.w;
}

} // extern "C"
