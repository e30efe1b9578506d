// Launchers shared between the translation units of the library (not part of the C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mraygb_types.h"

namespace mraygb
{

struct GridView;
struct DeviceCamera;

// generate.cu
cudaError_t launch_generate_grid(const GridView &grid, const DeviceCamera &cam, const mraygb_generation_params &gp,
                                 int width, int height, int m, bool kahan, float *moments, uint16_t *bounds,
                                 uint32_t *counts, int *error_flag, cudaStream_t stream);

// mese.cu
cudaError_t mese_init_constants();
// determine_best_number_moments for every pixel whose count is non-zero (error threshold > 0)
cudaError_t launch_count_moments(int num_pixels, int m, float error_threshold, const float *moments,
                                 uint32_t *counts, cudaStream_t stream);
// Lagrange multipliers; fp64 selects the FP64 form
cudaError_t launch_prepare(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                           int coding_warp, const uint16_t *coding_params, float bias, bool fp64, float *pmoments,
                           cudaStream_t stream);

// scan.cu
// exclusive scan of n u32 counts into out[0..n] (out[n] = total); scratch must hold scan_scratch_words(n)
size_t scan_scratch_words(size_t n);
cudaError_t launch_exclusive_scan(const uint32_t *counts, uint32_t *out, size_t n, uint32_t *scratch,
                                  cudaStream_t stream, int *launches);
cudaError_t launch_compact_copy(int num_pixels, int m, const uint32_t *counts, const uint32_t *index,
                                const float *moments, float *compact, cudaStream_t stream);

// reconstruct.cu
struct ReconArgs
{
    const DeviceCamera *cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const float4 *tf;
    float step, emission, ert;
    float *rgba;
    uint8_t *rgba8;
};
cudaError_t launch_reconstruct(const ReconArgs &a, int *error_flag, cudaStream_t stream);

} // namespace mraygb
