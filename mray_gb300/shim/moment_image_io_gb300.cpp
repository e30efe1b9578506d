// Reference-side shim for the moment-image file format: load_moment_image / write_moment_image (declared in
// src/moment_image_io.h:30-33) over the mraygb C ABI.  A maintainer builds this file in place of
// src/moment_image_io.cpp (and src/moment_image_coding.cpp, src/entropy_coding/): liblz4 is then no longer needed.
// The reference's global prediction-coding table (moment_quantization.cpp:166-223) is passed to the library when it
// is set, and set from a file that holds one, as the reference's reader does.
//
// Compiled against the reference's headers only (tests/test_shim_compiles.py checks that it compiles).

#include "moment_image_io.h"
#include "moment_quantization.h"

#include <cstdio>
#include <exception>
#include <mutex>

#include "mraygb.h"

namespace
{

mraygb_context *io_context()
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

void io_check(int status)
{
    if (status != MRAYGB_OK)
    {
        std::fprintf(stderr, "mraygb error %d: %s\n", status, mraygb_last_error(io_context()));
        std::terminate();
    }
}

} // namespace

void write_moment_image(const MomentImageHost &mi, const std::string filename, bool compress, Byte quantizationBits,
                        bool entropy_coding)
{
    mraygb_moment_image c{};
    c.width = mi.width;
    c.height = mi.height;
    c.num_moments = mi.num_moments;
    c.is_compact = mi.is_compact;
    c.prediction_code = mi.prediction_code;
    c.coding_warp = mi.coding_warp;
    c.domain_min[0] = mi.domain.min.x;
    c.domain_min[1] = mi.domain.min.y;
    c.domain_min[2] = mi.domain.min.z;
    c.domain_max[0] = mi.domain.max.x;
    c.domain_max[1] = mi.domain.max.y;
    c.domain_max[2] = mi.domain.max.z;
    c.data_size = mi.data.size();
    c.index = mi.is_compact ? const_cast<uint32_t *>(mi.index.data()) : nullptr;
    c.data = const_cast<float *>(mi.data.data());
    std::vector<uint16_t> bounds, cp;
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
    c.bounds = bounds.empty() ? nullptr : bounds.data();
    c.error_bounds = mi.has_error_bounds() ? const_cast<uint16_t *>(mi.error_bounds.data()) : nullptr;
    c.coding_params = cp.empty() ? nullptr : cp.data();
    std::vector<Byte> table;
    if (moment_quantization::uses_prediction_coding_quantization_table())
        table = moment_quantization::get_prediction_coding_quantization_table();
    io_check(mraygb_write_moment_image(io_context(), filename.c_str(), &c, compress, quantizationBits, entropy_coding,
                                       table.empty() ? nullptr : table.data()));
}

MomentImageHost load_moment_image(const std::string filename)
{
    mraygb_moment_image c{};
    int has_table = 0;
    std::vector<Byte> table(255, 0);
    io_check(mraygb_load_moment_image(io_context(), filename.c_str(), &c, table.data(), &has_table));
    MomentImageHost mi(c.width, c.height, c.num_moments, c.is_compact, c.has_bounds);
    mi.is_compact = c.is_compact;
    mi.prediction_code = c.prediction_code;
    mi.coding_warp = c.coding_warp;
    mi.domain = Range<Vec3f>(Vec3f(c.domain_min[0], c.domain_min[1], c.domain_min[2]),
                             Vec3f(c.domain_max[0], c.domain_max[1], c.domain_max[2]));
    mi.data.resize(c.data_size);
    std::vector<uint16_t> bounds(c.has_bounds ? 2 * size_t(c.width) * c.height : 0);
    std::vector<uint16_t> cp(c.has_coding_params ? 2 * size_t(c.num_moments - 1) : 0);
    if (c.has_error_bounds)
        mi.error_bounds.resize(size_t(c.width) * c.height);
    if (c.is_compact)
        mi.index.resize(size_t(c.width) * c.height + 1);
    c.index = c.is_compact ? mi.index.data() : nullptr;
    c.data = mi.data.data();
    c.bounds = bounds.empty() ? nullptr : bounds.data();
    c.error_bounds = c.has_error_bounds ? mi.error_bounds.data() : nullptr;
    c.coding_params = cp.empty() ? nullptr : cp.data();
    io_check(mraygb_load_moment_image(io_context(), filename.c_str(), &c, nullptr, nullptr));
    for (size_t i = 0; 2 * i < bounds.size(); ++i)
    {
        mi.bounds[i].lower = bounds[2 * i];
        mi.bounds[i].upper = bounds[2 * i + 1];
    }
    for (size_t i = 0; 2 * i < cp.size(); ++i)
        mi.coding_params.push_back(CodingParamType{cp[2 * i], cp[2 * i + 1]});
    if (has_table)
        moment_quantization::set_prediction_coding_quantization_table(
            std::vector<Byte>(table.begin(), table.begin() + c.num_moments));
    return mi;
}
