// Reference-side shim: the reference's CUDA seam (generate_device / reconstruct_device, declared in
// src/moment_raymarcher.cuh:48-54) implemented over the mraygb C ABI.  A maintainer of the reference builds
// this file in place of src/moment_raymarcher.cu's generate/reconstruct launchers and links libmraygb.so;
// main.cpp, the CLI and eval/mray_cli.py stay unchanged.  It only converts containers and maps a failure
// status to the reference's behaviour (a message and std::terminate, as CHECK_CUDA does).
//
// Compiled against the reference's headers only (tests/test_shim_compiles.py checks that it compiles).

#include "moment_raymarcher.cuh"
#include "moment_quantization.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <mutex>

#include "mraygb.h"

namespace
{

mraygb_context *context()
{
    static mraygb_context *ctx = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        if (mraygb_create(0, &ctx) != MRAYGB_OK)
        {
            std::fprintf(stderr, "mraygb: cannot create a context on device 0\n");
            std::terminate();
        }
    });
    return ctx;
}

// MRAYGB_SHIM_TIMING=1 prints the wall time of each phase of the seam calls to stderr (a maintainer's view of
// where a generate / reconstruct call spends its time: copies, conversions, the library's own work)
struct PhaseTimer
{
    const char *call;
    bool on;
    std::chrono::steady_clock::time_point t;
    explicit PhaseTimer(const char *c) : call(c), on(std::getenv("MRAYGB_SHIM_TIMING") != nullptr)
    {
        t = std::chrono::steady_clock::now();
    }
    void mark(const char *phase)
    {
        if (!on)
            return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "mraygb shim %s: %s %.2f ms\n", call, phase,
                     std::chrono::duration<double, std::milli>(now - t).count());
        t = now;
    }
};

void check(int status)
{
    if (status != MRAYGB_OK)
    {
        std::fprintf(stderr, "mraygb error %d: %s\n", status, mraygb_last_error(context()));
        std::terminate();
    }
}

mraygb_camera to_c(const cut::Camera &c)
{
    mraygb_camera o{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            o.transform[i][j] = c.transform[i][j];
    const Vec3f *v[4] = {&c.position, &c.right, &c.up, &c.dir};
    float *d[4] = {o.position, o.right, o.up, o.dir};
    for (int k = 0; k < 4; ++k)
    {
        d[k][0] = v[k]->x;
        d[k][1] = v[k]->y;
        d[k][2] = v[k]->z;
    }
    o.scale = c.scale;
    o.aspect = c.aspect;
    o.znear = c.znear;
    o.orthographic = c.orthographic ? 1 : 0;
    return o;
}

mraygb_generation_params to_c(const GenerationParameters &p)
{
    mraygb_generation_params o{};
    o.step_size = p.step_size;
    o.step_size_write_samples = p.step_size_write_samples;
    o.data_min = p.data_min;
    o.data_max = p.data_max;
    o.error_threshold = p.error_threshold;
    o.bias = p.bias;
    o.compact_image = p.compact_image;
    o.prediction_coding = p.prediction_coding;
    o.compress = p.compress;
    o.entropy_coding = p.entropy_coding;
    o.quantization_bits = p.quantization_bits;
    o.coding_warp = p.coding_warp;
    o.quantization_curve_sampling = p.quantization_curve_sampling;
    o.transform_to_bounds = p.transform_to_bounds;
    o.transform_bound_eps = p.transform_bound_eps;
    return o;
}

mraygb_single_scattering_params to_c(const SingleScatteringParameters &p)
{
    mraygb_single_scattering_params o{};
    o.enable = p.enable;
    o.use_cache = p.use_cache;
    o.cache_size_x = p.cache_size_x;
    o.cache_size_y = p.cache_size_y;
    o.cache_size_z = p.cache_size_z;
    o.step_size_factor = p.step_size_factor;
    o.henyey_greenstein_g = p.henyey_greenstein_g;
    o.direction_x = p.direction_x;
    o.direction_y = p.direction_y;
    o.direction_z = p.direction_z;
    o.intensity_r = p.intensity_r;
    o.intensity_g = p.intensity_g;
    o.intensity_b = p.intensity_b;
    return o;
}

mraygb_reconstruction_params to_c(const ReconstructionParameters &p)
{
    mraygb_reconstruction_params o{};
    o.bias = p.bias;
    o.medium_emission = p.medium_emission;
    o.medium_scattering = p.medium_scattering;
    o.early_ray_termination = p.early_ray_termination;
    o.data_min = p.data_min;
    o.data_max = p.data_max;
    o.step_size = p.step_size;
    o.step_size_write_samples = p.step_size_write_samples;
    o.use_truncated_fourier = p.use_truncated_fourier;
    o.ss = to_c(p.ss);
    return o;
}

} // namespace

namespace
{

// the moment image of the volume uploaded last, written into the reference's container
void generate_uploaded(const cut::Camera &cam, const Range<Vec3f> &domain, MomentImageHost &img,
                       const GenerationParameters &params)
{
    PhaseTimer timer("generate");
    const auto c = to_c(cam);
    const auto g = to_c(params);
    img.domain = domain;
    img.data.resize(size_t(img.width) * img.height * img.num_moments);
    if (params.compact_image)
        img.index.resize(size_t(img.width) * img.height + 1);
    if (params.transform_to_bounds)
        img.bounds.resize(size_t(img.width) * img.height);
    std::vector<uint16_t> bounds(params.transform_to_bounds ? 2 * size_t(img.width) * img.height : 0);
    std::vector<uint16_t> cp(img.num_moments > 1 ? 2 * size_t(img.num_moments - 1) : 1);
    timer.mark("host buffers");
    uint64_t size = 0;
    check(mraygb_generate(context(), &c, &g, img.width, img.height, img.num_moments, img.data.data(),
                          params.compact_image ? img.index.data() : nullptr,
                          params.transform_to_bounds ? bounds.data() : nullptr, cp.data(), &size));
    timer.mark("mraygb_generate");
    img.data.resize(size);
    for (size_t i = 0; i < img.bounds.size() && !bounds.empty(); ++i)
    {
        img.bounds[i].lower = bounds[2 * i];
        img.bounds[i].upper = bounds[2 * i + 1];
    }
    timer.mark("bounds conversion");
    img.is_compact = params.compact_image;
    img.prediction_code = params.prediction_coding;
    img.coding_warp = static_cast<CodingWarpType>(params.coding_warp);
    img.coding_params.clear();
    if (params.prediction_coding && params.coding_warp == CODING_WARP_DEFAULT_TRANSFORMED)
        for (int i = 0; i + 1 < img.num_moments; ++i)
            img.coding_params.push_back(CodingParamType{cp[2 * i], cp[2 * i + 1]});
}

} // namespace

void generate_device(cut::Camera cam, const RegularGrid &volume, MomentImageHost &img,
                     const GenerationParameters &params)
{
    if (volume.type != RegularGrid::DataType::F32)
    {
        std::fprintf(stderr, "mraygb: only float grids are supported\n");
        std::terminate();
    }
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    PhaseTimer timer("generate_device");
    check(mraygb_upload_grid(context(), volume.data.data(), volume.size.x, volume.size.y, volume.size.z, dmin, dmax,
                             0));
    timer.mark("mraygb_upload_grid");
    generate_uploaded(cam, volume.domain, img, params);
}

void generate_device(cut::Camera cam, const Particles &volume, MomentImageHost &img,
                     const GenerationParameters &params)
{
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_particles(context(), volume.x.data(), volume.y.data(), volume.z.data(),
                                  volume.values.data(), volume.size(), volume.smoothing_length, dmin, dmax, 0));
    generate_uploaded(cam, volume.domain, img, params);
}

void reconstruct_device(cut::Camera cam, const MomentImageHost &mi, const TransferFunction &tf, ColorImageHost &cimg,
                        const ReconstructionParameters &params)
{
    // preintegrate() / read_from_disk() tables have 256 equal rows; the first row is the whole table
    PhaseTimer timer("reconstruct_device");
    check(mraygb_upload_tf(context(), reinterpret_cast<const float *>(tf.data.data())));
    const auto c = to_c(cam);
    const auto r = to_c(params);
    const float dmin[3] = {mi.domain.min.x, mi.domain.min.y, mi.domain.min.z};
    const float dmax[3] = {mi.domain.max.x, mi.domain.max.y, mi.domain.max.z};
    std::vector<uint16_t> bounds;
    for (const auto &b : mi.bounds)
    {
        bounds.push_back(b.lower);
        bounds.push_back(b.upper);
    }
    std::vector<uint16_t> cp;
    for (const auto &p : mi.coding_params)
    {
        cp.push_back(p.param1);
        cp.push_back(p.param2);
    }
    static_assert(sizeof(ColorImageHost::rgba8_t) == 4, "rgba8_t is four bytes");
    timer.mark("tf upload and bounds conversion");
    check(mraygb_reconstruct(context(), &c, &r, mi.width, mi.height, mi.num_moments, dmin, dmax,
                             mi.is_compact ? mi.index.data() : nullptr, mi.data.data(), mi.data.size(),
                             bounds.empty() ? nullptr : bounds.data(), mi.prediction_code, mi.coding_warp,
                             cp.empty() ? nullptr : cp.data(), nullptr,
                             reinterpret_cast<uint8_t *>(cimg.rgba.data())));
    timer.mark("mraygb_reconstruct");
}

namespace
{

mraygb_error_params to_c(const ErrorReconstructionParameters &p)
{
    mraygb_error_params o{};
    o.error_type = p.error_type;
    o.error_percentile = p.error_percentile;
    o.bias = p.bias;
    o.data_min = p.data_min;
    o.data_max = p.data_max;
    o.step_size = p.step_size;
    o.compress = p.compress;
    o.entropy_coding = p.entropy_coding;
    o.quantization_bits = p.quantization_bits;
    return o;
}

mraygb_uncertainty_params to_c(const UncertaintyReconstructionParameters &p)
{
    mraygb_uncertainty_params o{};
    o.rec = to_c(p.rec);
    o.bound_interpolation = p.bound_interpolation;
    o.error_type = p.error_type;
    return o;
}

// the moment image's u16 arrays as the C ABI takes them
struct ImageArrays
{
    std::vector<uint16_t> bounds, cp;
    explicit ImageArrays(const MomentImageHost &mi)
    {
        for (const auto &b : mi.bounds)
        {
            bounds.push_back(b.lower);
            bounds.push_back(b.upper);
        }
        for (const auto &p : mi.coding_params)
        {
            cp.push_back(p.param1);
            cp.push_back(p.param2);
        }
    }
};

void error_uploaded(const cut::Camera &cam, MomentImageHost &mi, const ErrorReconstructionParameters &params)
{
    const auto c = to_c(cam);
    const auto e = to_c(params);
    ImageArrays arr(mi);
    mi.error_bounds.resize(size_t(mi.width) * mi.height);
    check(mraygb_reconstruct_error(context(), &c, &e, mi.width, mi.height, mi.num_moments,
                                   mi.is_compact ? mi.index.data() : nullptr, mi.data.data(), mi.data.size(),
                                   arr.bounds.empty() ? nullptr : arr.bounds.data(), mi.prediction_code,
                                   mi.coding_warp, arr.cp.empty() ? nullptr : arr.cp.data(), mi.error_bounds.data(),
                                   nullptr));
}

void uncertainty(const cut::Camera &cam, const MomentImageHost &mi, ColorImageHost &cimg,
                 const UncertaintyReconstructionParameters &params, int mode)
{
    const auto c = to_c(cam);
    const auto u = to_c(params);
    ImageArrays arr(mi);
    const float dmin[3] = {mi.domain.min.x, mi.domain.min.y, mi.domain.min.z};
    const float dmax[3] = {mi.domain.max.x, mi.domain.max.y, mi.domain.max.z};
    check(mraygb_reconstruct_uncertainty(context(), &c, &u, mode, mi.width, mi.height, mi.num_moments, dmin, dmax,
                                         mi.is_compact ? mi.index.data() : nullptr, mi.data.data(), mi.data.size(),
                                         arr.bounds.empty() ? nullptr : arr.bounds.data(), mi.error_bounds.data(),
                                         mi.prediction_code, mi.coding_warp, arr.cp.empty() ? nullptr : arr.cp.data(),
                                         nullptr, reinterpret_cast<uint8_t *>(cimg.rgba.data())));
}

} // namespace

namespace
{

mraygb_reference_params to_c(const ReferenceParameters &p)
{
    mraygb_reference_params o{};
    o.step_size = p.step_size;
    o.medium_emission = p.medium_emission;
    o.medium_scattering = p.medium_scattering;
    o.early_ray_termination = p.early_ray_termination;
    o.data_min = p.data_min;
    o.data_max = p.data_max;
    o.ss = to_c(p.ss);
    return o;
}

void reference_uploaded(const cut::Camera &cam, const TransferFunction &tf, ColorImageHost &img,
                        const ReferenceParameters &params)
{
    check(mraygb_upload_tf(context(), reinterpret_cast<const float *>(tf.data.data())));
    const auto c = to_c(cam);
    const auto r = to_c(params);
    check(mraygb_generate_reference(context(), &c, &r, img.width, img.height, nullptr,
                                    reinterpret_cast<uint8_t *>(img.rgba.data())));
}

} // namespace

// generate_reference_device (src/moment_raymarcher.cuh:38-41) for both volume types
void generate_reference_device(cut::Camera cam, const RegularGrid &volume, const TransferFunction &tf,
                               ColorImageHost &img, const ReferenceParameters &params)
{
    if (volume.type != RegularGrid::DataType::F32)
    {
        std::fprintf(stderr, "mraygb: only float grids are supported\n");
        std::terminate();
    }
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_grid(context(), volume.data.data(), volume.size.x, volume.size.y, volume.size.z, dmin, dmax,
                             0));
    reference_uploaded(cam, tf, img, params);
}

void generate_reference_device(cut::Camera cam, const Particles &volume, const TransferFunction &tf,
                               ColorImageHost &img, const ReferenceParameters &params)
{
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_particles(context(), volume.x.data(), volume.y.data(), volume.z.data(),
                                  volume.values.data(), volume.size(), volume.smoothing_length, dmin, dmax, 0));
    reference_uploaded(cam, tf, img, params);
}

// reconstruct_error_device (src/moment_raymarcher.cuh:73-76) for both volume types: fills mi.error_bounds
void reconstruct_error_device(cut::Camera cam, const RegularGrid &volume, MomentImageHost &mi,
                              const ErrorReconstructionParameters &params)
{
    if (volume.type != RegularGrid::DataType::F32)
    {
        std::fprintf(stderr, "mraygb: only float grids are supported\n");
        std::terminate();
    }
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_grid(context(), volume.data.data(), volume.size.x, volume.size.y, volume.size.z, dmin, dmax,
                             0));
    error_uploaded(cam, mi, params);
}

void reconstruct_error_device(cut::Camera cam, const Particles &volume, MomentImageHost &mi,
                              const ErrorReconstructionParameters &params)
{
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_particles(context(), volume.x.data(), volume.y.data(), volume.z.data(),
                                  volume.values.data(), volume.size(), volume.smoothing_length, dmin, dmax, 0));
    error_uploaded(cam, mi, params);
}

namespace
{

// The transmittance cache of the light's image (reconstruct_single_scattering_cache_device in the reference's
// launchers), kept in the context for the call that follows.
void ss_cache_uploaded(const SingleScatteringImageHost &ss, const ReconstructionParameters &params)
{
    const auto lc = to_c(ss.cam);
    const auto r = to_c(params);
    const MomentImageHost &mi = ss.img;
    const float dmin[3] = {mi.domain.min.x, mi.domain.min.y, mi.domain.min.z};
    const float dmax[3] = {mi.domain.max.x, mi.domain.max.y, mi.domain.max.z};
    ImageArrays arr(mi);
    check(mraygb_reconstruct_single_scattering_cache(
        context(), &lc, &r, mi.width, mi.height, mi.num_moments, dmin, dmax, mi.is_compact ? mi.index.data() : nullptr,
        mi.data.data(), mi.data.size(), arr.bounds.empty() ? nullptr : arr.bounds.data(), mi.prediction_code,
        mi.coding_warp, arr.cp.empty() ? nullptr : arr.cp.data(), nullptr));
}

void reference_cached_uploaded(const cut::Camera &cam, const TransferFunction &tf, ColorImageHost &img,
                               const SingleScatteringImageHost &ss, const ReconstructionParameters &params)
{
    check(mraygb_upload_tf(context(), reinterpret_cast<const float *>(tf.data.data())));
    ss_cache_uploaded(ss, params);
    const auto c = to_c(cam);
    const auto r = to_c(params);
    check(mraygb_generate_reference_reconstructed_ss(context(), &c, &r, img.width, img.height, nullptr,
                                                     reinterpret_cast<uint8_t *>(img.rgba.data())));
}

} // namespace

// reconstruct_device with a SingleScatteringImageHost (src/moment_raymarcher.cuh:56-57): the cache of the light's
// image, then the re-march sampling it (params.ss.use_cache; the marched form returns MRAYGB_NOT_SUPPORTED)
void reconstruct_device(cut::Camera cam, const MomentImageHost &mi, const TransferFunction &tf, ColorImageHost &cimg,
                        const SingleScatteringImageHost &ss, const ReconstructionParameters &params)
{
    check(mraygb_upload_tf(context(), reinterpret_cast<const float *>(tf.data.data())));
    ss_cache_uploaded(ss, params);
    const auto c = to_c(cam);
    const auto r = to_c(params);
    const float dmin[3] = {mi.domain.min.x, mi.domain.min.y, mi.domain.min.z};
    const float dmax[3] = {mi.domain.max.x, mi.domain.max.y, mi.domain.max.z};
    ImageArrays arr(mi);
    check(mraygb_reconstruct(context(), &c, &r, mi.width, mi.height, mi.num_moments, dmin, dmax,
                             mi.is_compact ? mi.index.data() : nullptr, mi.data.data(), mi.data.size(),
                             arr.bounds.empty() ? nullptr : arr.bounds.data(), mi.prediction_code, mi.coding_warp,
                             arr.cp.empty() ? nullptr : arr.cp.data(), nullptr,
                             reinterpret_cast<uint8_t *>(cimg.rgba.data())));
}

// generate_reference_reconstructed_ss_device (src/moment_raymarcher.cuh:59-64) for both volume types
void generate_reference_reconstructed_ss_device(cut::Camera cam, const TransferFunction &tf, const RegularGrid &volume,
                                                ColorImageHost &img, const SingleScatteringImageHost &ss,
                                                const ReconstructionParameters &params)
{
    if (volume.type != RegularGrid::DataType::F32)
    {
        std::fprintf(stderr, "mraygb: only float grids are supported\n");
        std::terminate();
    }
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_grid(context(), volume.data.data(), volume.size.x, volume.size.y, volume.size.z, dmin, dmax,
                             0));
    reference_cached_uploaded(cam, tf, img, ss, params);
}

void generate_reference_reconstructed_ss_device(cut::Camera cam, const TransferFunction &tf, const Particles &volume,
                                                ColorImageHost &img, const SingleScatteringImageHost &ss,
                                                const ReconstructionParameters &params)
{
    const float dmin[3] = {volume.domain.min.x, volume.domain.min.y, volume.domain.min.z};
    const float dmax[3] = {volume.domain.max.x, volume.domain.max.y, volume.domain.max.z};
    check(mraygb_upload_particles(context(), volume.x.data(), volume.y.data(), volume.z.data(),
                                  volume.values.data(), volume.size(), volume.smoothing_length, dmin, dmax, 0));
    reference_cached_uploaded(cam, tf, img, ss, params);
}

// reconstruct_uncertainty_interpolation_device / _convolution_device (src/moment_raymarcher.cuh:78-86); the
// single-scattering overload stays with the reference's launcher (it marches the light's image, not the cache)
void reconstruct_uncertainty_interpolation_device(cut::Camera cam, const MomentImageHost &mi,
                                                  const TransferFunction &tf, ColorImageHost &cimg,
                                                  const UncertaintyReconstructionParameters &params)
{
    check(mraygb_upload_tf(context(), reinterpret_cast<const float *>(tf.data.data())));
    uncertainty(cam, mi, cimg, params, 0);
}

void reconstruct_uncertainty_convolution_device(cut::Camera cam, const MomentImageHost &mi, const TransferFunction &tf,
                                                ColorImageHost &cimg,
                                                const UncertaintyReconstructionParameters &params)
{
    check(mraygb_upload_uncertainty_table(context(), reinterpret_cast<const float *>(tf.data.data())));
    uncertainty(cam, mi, cimg, params, 1);
}

// create_quantization_table (src/measure_coding_error.cpp:374-438) over the C ABI: the same table for the same
// (already sampled) image, installed as the reference's global prediction-coding table.  measure_coding_error.cpp
// also holds the offline curve study that main.cpp:770 calls, so this is a second name: main.cpp:322 calls it in
// place of create_quantization_table.
void create_quantization_table_gb300(const MomentImageHost &img, int start_bits)
{
    std::vector<uint16_t> cp;
    for (const auto &p : img.coding_params)
    {
        cp.push_back(p.param1);
        cp.push_back(p.param2);
    }
    std::vector<Byte> table(img.num_moments);
    check(mraygb_create_quantization_table(context(), img.width, img.height, img.num_moments, img.index.data(),
                                           img.data.data(), img.data.size(), img.coding_warp,
                                           cp.empty() ? nullptr : cp.data(), start_bits, 0, table.data(), nullptr));
    moment_quantization::set_prediction_coding_quantization_table(table);
}
