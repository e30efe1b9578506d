/*
 * ORACLE — test infrastructure only.
 *
 * The rest of the reference's CUDA seam for the drop-in test build (oracle/Makefile shim): the reference's own CPU
 * code compiled with CUDA_SUPPORT, its generate()/reconstruct() dispatching to mray_gb300/shim/*.cpp over
 * libmraygb.so.  moment_raymarcher.cpp also references the device launchers of paths outside the moment-image hot
 * path (sample images, ray histograms, resampling; src/moment_raymarcher.cu); a maintainer keeps the reference's
 * own .cu files for those.  Here they stop with a message, and the device sort the particle grid uses
 * (src/particle_grid.cu via cut/sort_util.h) is the reference's host sort of the non-CUDA build.
 */
#include "moment_raymarcher.cuh"
#include "cut/sort_util.cuh"

#include <cstdio>
#include <exception>
#include <algorithm>
#include <numeric>

namespace
{
[[noreturn]] void unsupported(const char *what)
{
    std::fprintf(stderr, "%s: outside the drop-in test build\n", what);
    std::terminate();
}
} // namespace

namespace cut
{
namespace device
{
void getSortedIndices(const vector<uint32_t> &values, vector<uint32_t> &valueIndices)
{
    valueIndices.resize(values.size());
    std::iota(valueIndices.begin(), valueIndices.end(), 0);
    std::sort(valueIndices.begin(), valueIndices.end(), [&](int lhs, int rhs) { return values[lhs] < values[rhs]; });
}
} // namespace device
} // namespace cut

void generate_samples_device(cut::Camera, const RegularGrid &, SamplesImageHost &, const GenerationParameters &)
{
    unsupported("generate_samples_device");
}
void generate_samples_device(cut::Camera, const Particles &, SamplesImageHost &, const GenerationParameters &)
{
    unsupported("generate_samples_device");
}
void reconstruct_samples_device(cut::Camera, const MomentImageHost &, SamplesImageHost &,
                                const ReconstructionParameters &)
{
    unsupported("reconstruct_samples_device");
}
void reconstruct_rayhistogram_device(cut::Camera, const RayHistogramImageHost &, const TransferFunction &,
                                     ColorImageHost &, const RayHistogramReconstructionParameters &)
{
    unsupported("reconstruct_rayhistogram_device");
}
void reconstruct_rayhistogram_samples_device(cut::Camera, const RayHistogramImageHost &, SamplesImageHost &,
                                             const RayHistogramReconstructionParameters &)
{
    unsupported("reconstruct_rayhistogram_samples_device");
}
void reconstruct_resampled_device(cut::Camera, const MomentImageHost &, const TransferFunction &, ColorImageHost &,
                                  const vector<cut::Camera> &, const string &, Vec3f,
                                  const ResamplingReconstructionParameters &)
{
    unsupported("reconstruct_resampled_device");
}
void reconstruct_uncertainty_interpolation_device(cut::Camera, const MomentImageHost &, const TransferFunction &,
                                                  ColorImageHost &, const SingleScatteringImageHost &,
                                                  const UncertaintyReconstructionParameters &)
{
    unsupported("reconstruct_uncertainty_interpolation_device (single scattering)");
}
