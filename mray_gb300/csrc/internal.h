// Launchers shared between the translation units of the library (not part of the C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mraygb_types.h"

namespace mraygb
{

struct GridView;
struct ParticleView;
struct ParticleHView;
struct ParticleGridParams;
struct DeviceCamera;

// generate.cu
cudaError_t launch_generate_grid(const GridView &grid, const DeviceCamera &cam, const mraygb_generation_params &gp,
                                 int width, int height, int m, bool kahan, float *moments, uint16_t *bounds,
                                 uint32_t *counts, float4 *bounds4, int *error_flag, cudaStream_t stream);

cudaError_t launch_generate_particles(const ParticleView &parts, const DeviceCamera &cam,
                                      const mraygb_generation_params &gp, int width, int height, int m, bool kahan,
                                      float *moments, uint16_t *bounds, uint32_t *counts, float4 *bounds4,
                                      int *error_flag, cudaStream_t stream);
cudaError_t launch_generate_particles_h(const ParticleHView &parts, const DeviceCamera &cam,
                                        const mraygb_generation_params &gp, int width, int height, int m, bool kahan,
                                        float *moments, uint16_t *bounds, uint32_t *counts, float4 *bounds4,
                                        int *error_flag, cudaStream_t stream);

// particles.cu: the particle grid build
ParticleGridParams particle_grid_params(const float mn[3], const float mx[3], float h);
size_t particle_minmax_scratch_floats(uint64_t n);
// min (out6[0..2]) and max (out6[3..5]) of the positions
cudaError_t launch_particle_minmax(const float *x, const float *y, const float *z, uint64_t n, float *scratch,
                                   float *out6, cudaStream_t stream);
// cell of every particle and per-cell counts (counts zeroed by the caller)
cudaError_t launch_particle_cells(const float *x, const float *y, const float *z, uint64_t n,
                                  const ParticleGridParams &g, uint32_t *cell_of, uint32_t *counts,
                                  cudaStream_t stream);
// stable LSD radix sort of n cell keys (< total) with the particle index as payload; keys and keys_alt are
// overwritten, *sorted_vals points at vals or vals_alt.  hist holds particle_radix_hist_words(n) words, hist_scan
// one more, scan_scratch scan_scratch_words(particle_radix_hist_words(n)).
size_t particle_radix_hist_words(uint32_t n);
cudaError_t launch_particle_sort(uint32_t n, uint32_t total, uint32_t *keys, uint32_t *keys_alt, uint32_t *vals,
                                 uint32_t *vals_alt, uint32_t *hist, uint32_t *hist_scan, uint32_t *scan_scratch,
                                 uint32_t **sorted_vals, cudaStream_t stream, int *launches);
// pts[i] = (x, y, z, v)[order[i]]
// per-particle smoothing lengths: out2 = (bits of the largest valid h, count of h not finite and > 0); the records'
// (1 / h, 1 / h^3) in sorted order
cudaError_t launch_particle_h_range(uint64_t n, const float *h, unsigned int *out2, cudaStream_t stream);
cudaError_t launch_particle_gather_h(uint64_t n, const uint32_t *order, const float *h, float2 *inv_h,
                                     cudaStream_t stream);
cudaError_t launch_particle_gather(uint64_t n, const uint32_t *order, const float *x, const float *y, const float *z,
                                   const float *v, float4 *pts, cudaStream_t stream);

// libm_trig_host.cpp: the device copy of the sinf / cosf exception table (libm_trig_core.h)
struct LibmTrigTable
{
    const uint32_t *offsets; // n_buckets + 1
    const uint16_t *entries;
};
// the table of the current device, uploaded on first use (thread safe)
cudaError_t libm_trig_device_table(LibmTrigTable *out);

// fp32_rate.cu: the measured FP32 FMA rate (TFLOP/s) of the current device
size_t fp32_rate_scratch_floats(int sm_count);
cudaError_t measure_fp32_rate(int sm_count, cudaStream_t stream, float *scratch, double *tflops);

// mese.cu
cudaError_t mese_init_constants();
// cosf / sinf of the MESE algebra (the host C library's results) over n floats
cudaError_t launch_libm_sincosf(uint64_t n, const float *x, float *s, float *c, cudaStream_t stream);
// determine_best_number_moments for every pixel whose count is non-zero (error threshold > 0)
cudaError_t launch_count_moments(int num_pixels, int m, float error_threshold, const float *moments,
                                 uint32_t *counts, cudaStream_t stream);
// per-pixel part of prediction coding, in place on the compact moment data
cudaError_t launch_prediction_encode(int num_pixels, int m, const uint32_t *index, float *data, float bias,
                                     cudaStream_t stream);
// mese_f64.cu: the FP64 preparation
cudaError_t mese_f64_init_constants(const LibmTrigTable &trig);
cudaError_t launch_prepare_f64(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                               int coding_warp, const uint16_t *coding_params, float bias, float *pmoments,
                               cudaStream_t stream);
// mese_ff.cu: the float-float preparation
cudaError_t mese_ff_init_constants(const LibmTrigTable &trig);
cudaError_t launch_prepare_ff(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                              int coding_warp, const uint16_t *coding_params, float bias, float *pmoments,
                              cudaStream_t stream);
// Lagrange multipliers; fp64 selects the FP64 form
cudaError_t launch_prepare(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                           int coding_warp, const uint16_t *coding_params, float bias, bool fp64, float *pmoments,
                           cudaStream_t stream);

// uncertainty.cu: error bounds, the uncertainty table, uncertainty rendering
struct ErrorArgs
{
    const DeviceCamera *cam;
    int width, height, m;
    const uint32_t *index;  // compact index or null
    const float *pmoments;  // Lagrange multipliers in the data layout
    const uint16_t *bounds; // 2*W*H u16 or null
    float step, data_min, data_max;
    int percentile;
    uint16_t *error_bounds; // W*H u16
    float *errors;          // W*H floats or null
};
cudaError_t launch_error_bounds_grid(const GridView &grid, const ErrorArgs &a, int error_type, int *error_flag,
                                     cudaStream_t stream);
cudaError_t launch_error_bounds_particles(const ParticleView &parts, const ErrorArgs &a, int error_type,
                                          int *error_flag, cudaStream_t stream);
// 256 x 256 RGBA, [y][x]
cudaError_t launch_uncertainty_tf(const float4 *tf1d, float step, int error_type, float4 *table, cudaStream_t stream);
struct UncertaintyArgs
{
    const DeviceCamera *cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const uint16_t *error_bounds;
    const float4 *tf;    // mode 0: preintegrated row
    const float4 *table; // mode 1: uncertainty table
    float step, emission, ert, interp;
    int mode, error_type;
    float *rgba;
    uint8_t *rgba8;
};
cudaError_t launch_uncertainty(const UncertaintyArgs &a, int *error_flag, cudaStream_t stream);

// reference.cu: direct volume rendering of the resident volume (the ground truth)
struct ReferenceArgs
{
    const DeviceCamera *cam;
    int width, height;
    const mraygb_reference_params *rp;
    const float4 *tf; // preintegrated row
    float *rgba;      // W*H float4 or null
    uint8_t *rgba8;   // W*H uchar4 or null
    // single scattering from the transmittance cache instead of the brute-force march (null: brute force)
    const GridView *ss_cache = nullptr;
};
cudaError_t launch_reference_grid(const GridView &grid, const ReferenceArgs &a, int *error_flag, cudaStream_t stream);
cudaError_t launch_reference_particles(const ParticleView &parts, const ReferenceArgs &a, int *error_flag,
                                       cudaStream_t stream);

// quant_curve.cu: the data-dependent quantization table's error means for every (index, bits) pair
cudaError_t quant_curve_init_constants(const LibmTrigTable &trig);
// scratch bytes for an sx x sy sample, bits bmin .. bmin + nb - 1, rows_per_pass moment indices per pass
size_t quant_curve_scratch_bytes(int sx, int sy, int m, int nb, size_t rows_per_pass);
// d_means[(idx - 1) * nb + (b - bmin)] for idx in [1, m): the mean rRMSE of quantizing moment idx to b bits
cudaError_t launch_quant_curve(int width, int height, int m, const uint32_t *index, const float *data, int warp,
                               const uint16_t *coding_params, int sx, int sy, int bmin, int nb,
                               size_t rows_per_pass, void *scratch, float *d_means, cudaStream_t stream,
                               int *launches);

// scan.cu
// exclusive scan of n u32 counts into out[0..n] (out[n] = total); scratch must hold scan_scratch_words(n)
size_t scan_scratch_words(size_t n);
cudaError_t launch_exclusive_scan(const uint32_t *counts, uint32_t *out, size_t n, uint32_t *scratch,
                                  cudaStream_t stream, int *launches);
cudaError_t launch_exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, size_t n,
                                      unsigned long long *scratch, cudaStream_t stream, int *launches);
cudaError_t launch_compact_copy(int num_pixels, int m, const uint32_t *counts, const uint32_t *index,
                                const float *moments, float *compact, cudaStream_t stream);

// coding.cu
int coding_minmax_blocks(int num_pixels);
cudaError_t launch_coding_params(int num_pixels, int m, const uint32_t *index, const float *data, uint64_t total,
                                 float2 *partial, uint16_t *params_u16, float *params_f, cudaStream_t stream);
cudaError_t launch_coding_warp(int num_pixels, const uint32_t *index, float *data, int warp_type,
                               const float *params, cudaStream_t stream);
cudaError_t launch_pixel_bits(int num_pixels, const uint32_t *index, const uint32_t *prefix_bits,
                              unsigned long long *bits, cudaStream_t stream);
// codes of moment index l >= 1 over [lo1, hi1] (prediction codes: [0, 1]; the plain quantizer: [-1/pi, 1/pi]); the
// zeroth moment over [0, 1]
cudaError_t launch_pack(int num_pixels, const uint32_t *index, const float *data, const uint8_t *table,
                        const uint32_t *prefix_bits, const unsigned long long *bit_offset, uint32_t *words,
                        cudaStream_t stream, float lo1 = 0.f, float hi1 = 1.f);
cudaError_t launch_unpack(int num_pixels, const uint32_t *index, const uint8_t *table, const uint32_t *prefix_bits,
                          const unsigned long long *bit_offset, const uint8_t *bytes, unsigned long long num_bytes,
                          float *data, cudaStream_t stream, float lo1 = 0.f, float hi1 = 1.f);
// u16 codes in the layout of the moment data, for the entropy coder, and back
cudaError_t launch_symbols(int num_pixels, const uint32_t *index, const float *data, const uint8_t *table, float lo1,
                           float hi1, uint16_t *symbols, cudaStream_t stream);
cudaError_t launch_desymbols(int num_pixels, const uint32_t *index, const uint16_t *symbols, const uint8_t *table,
                             float lo1, float hi1, float *data, cudaStream_t stream);
// byte-aligned codes of an image without compaction (count = W*H*m values)
cudaError_t launch_static_quantize(size_t count, int m, const float *data, int bits, float lo1, float hi1,
                                   uint8_t *out, cudaStream_t stream);

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
    // per-pixel (lo, hi, ., .) float bounds instead of the u16 ones
    const float4 *bounds4 = nullptr;
    // the differentiation form's density and transfer function (exact atan, cubic B-spline row; with diff_tf_linear
    // the row linear in the front density)
    int diff_form = 0;
    int diff_tf_linear = 0;
    // single scattering from the transmittance cache (null: none): in-scattered light of intensity ss->intensity
    // and phase function ss->henyey_greenstein_g, weighted by the medium's scattering coefficient
    const GridView *ss_cache = nullptr;
    const mraygb_single_scattering_params *ss = nullptr;
    float scattering = 0.f;
};
cudaError_t launch_reconstruct(const ReconArgs &a, int *error_flag, cudaStream_t stream);

// scattering.cu: the single-scattering transmittance cache of a light moment image (prepared moments)
struct SsCacheArgs
{
    const DeviceCamera *cam; // the light's camera
    int width, height, m;
    float dmin[3], dmax[3]; // the image's domain, also the cache's
    const uint32_t *index;
    const float *pmoments;
    const uint16_t *bounds;
    const float4 *tf;
    float step;
    int cx, cy, cz;
    unsigned long long *keys; // cx*cy*cz scratch
    float *cache;             // cx*cy*cz floats, x fastest
};
cudaError_t launch_ss_cache(const SsCacheArgs &a, int *error_flag, cudaStream_t stream);

// adjoint.cu: the differentiation form's adjoints (non-compact images, float bounds, linear transfer function)
struct ReconAdjArgs
{
    const DeviceCamera *cam;
    int width, height, m;
    float dmin[3], dmax[3];
    const float *pmoments;
    const float4 *bounds4;
    const float4 *tf;
    float step, emission, ert;
    const float4 *rgba, *grad_rgba;
    float *grad_lambda;
    float2 *grad_bounds;
    float4 *grad_tf;
    int tf_linear = 0; // the transfer-function row linear in the front density instead of the cubic B-spline
};
cudaError_t launch_reconstruct_adjoint(const ReconAdjArgs &a, int *error_flag, cudaStream_t stream);
// the FP32 multipliers of W*H*m moments (m <= 64) and, per pixel, the 2m float2 that the preparation adjoint reads
cudaError_t launch_prepare_keep(int num_pixels, int m, const float *data, float bias, float *pmoments, float2 *keep,
                                cudaStream_t stream);
// d loss / d moments from d loss / d Lagrange multipliers and the arrays launch_prepare_keep kept (grad_moments may
// alias grad_lambda)
cudaError_t launch_prepare_adjoint(int num_pixels, int m, const float2 *keep, float bias, const float *grad_lambda,
                                   float *grad_moments, cudaStream_t stream);
// d loss / d voxel density, accumulated into grad_volume
cudaError_t launch_generate_adjoint(const GridView &grid, float *grad_volume, const DeviceCamera &cam,
                                    const mraygb_generation_params &gp, int width, int height, int m,
                                    const float *moments, const float4 *bounds4, const float *grad_moments,
                                    const float2 *grad_bounds, int *error_flag, cudaStream_t stream);

} // namespace mraygb
