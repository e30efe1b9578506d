/*
 * mraygb — GB300-native (sm_103a) moment-image generation, prediction coding / quantization and
 * bounded-MESE reconstruction: the data-parallel hot path of TobiasRp/mray behind a C ABI.
 *
 * Two layers:
 *
 *  1. The drop-in host API (mraygb_generate / mraygb_reconstruct) takes and returns HOST buffers, with the
 *     shapes of the reference's CUDA seam:
 *        void generate_device(cut::Camera, const RegularGrid &, MomentImageHost &, const GenerationParameters &);
 *        void generate_device(cut::Camera, const Particles &, MomentImageHost &, const GenerationParameters &);
 *        void reconstruct_device(cut::Camera, const MomentImageHost &, const TransferFunction &,
 *                                ColorImageHost &, const ReconstructionParameters &);
 *     (src/moment_raymarcher.cuh:48-54, dispatched from src/moment_raymarcher.cpp:168-183 and 329-337).
 *     The volume and transfer function stay resident in the context between calls.
 *
 *  2. The stage API (mraygb_stage_*) runs one step of the path on DEVICE pointers, ordered on the context's
 *     stream, with no host synchronisation unless a size has to come back to the host.
 *
 * Every entry point returns an mraygb_status; on failure mraygb_last_error() describes it.  Nothing aborts
 * the process (the reference terminates on CUDA errors, src/cut/cuda_common.cpp:32-53).  A context may be
 * used by one host thread at a time; independent contexts are independent.
 *
 * No CUDA or torch types appear in these signatures: streams are passed as void* (a cudaStream_t).
 */
#ifndef MRAYGB_H
#define MRAYGB_H

#include <stddef.h>
#include <stdint.h>

#include "mraygb_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mraygb_context mraygb_context;

typedef enum mraygb_status
{
    MRAYGB_OK = 0,
    MRAYGB_INVALID_ARGUMENT = 1,
    MRAYGB_OUT_OF_MEMORY = 2,
    MRAYGB_CUDA_ERROR = 3,
    MRAYGB_DEVICE_TIMEOUT = 4,
    MRAYGB_NUMERICAL = 5,
    MRAYGB_NOT_SUPPORTED = 6,
    MRAYGB_NO_VOLUME = 7
} mraygb_status;

/* Arithmetic forms of the path. */
typedef enum mraygb_precision
{
    /* the reference's method in FP32 (moment sums in plain FP32, FP32 Levinson / MESE preparation) */
    MRAYGB_PRECISION_FP32 = 0,
    /* FP32 ray marching with compensated (Kahan) moment sums; MESE preparation (Levinson recursion,
     * Toeplitz / Herglotz correlations) in FP64 */
    MRAYGB_PRECISION_COMPENSATED_FP64_MESE = 1,
    /* as COMPENSATED_FP64_MESE with the FP64 steps of the preparation (exponential moments, Levinson's
     * recursion) in float-float arithmetic (about 48 significant bits) and its correlation tail in FP32 on the
     * rounded results (prediction-coded moments: the decode recursion in float-float).  No counterpart in the
     * reference. */
    MRAYGB_PRECISION_COMPENSATED_FF_MESE = 2
} mraygb_precision;

/* Largest moment count (the reference's file format stores counts in 8 bits: src/main.cpp:288-293). */
#define MRAYGB_MAX_MOMENTS 255

/* ---- context -------------------------------------------------------------------------------------------- */

/* Creates a context on CUDA device `device` with its own non-blocking stream. */
int mraygb_create(int device, mraygb_context **out);
void mraygb_destroy(mraygb_context *ctx);
/* The last error message of this context ("" when none). */
const char *mraygb_last_error(const mraygb_context *ctx);
/* Orders all later work of this context on `stream` (a cudaStream_t; NULL restores the context's own; the legacy
 * default stream is cudaStreamLegacy, since NULL does not select it). */
int mraygb_set_stream(mraygb_context *ctx, void *stream);
void *mraygb_get_stream(const mraygb_context *ctx);
int mraygb_synchronize(mraygb_context *ctx);
/* Selects the arithmetic form (mraygb_precision) for later generate / prepare calls. */
int mraygb_set_precision(mraygb_context *ctx, int precision);
/* Number of this library's kernels launched by the context so far. */
uint64_t mraygb_kernel_launches(const mraygb_context *ctx);
/* The FP32 roof the marching kernels are measured against: the rate of a chain of fused multiply-adds with no
 * memory traffic on every SM of the context's device (two launches of about 10 ms on the context's stream, the
 * second timed with CUDA events), in TFLOP/s (an FMA counts as two).  No counterpart in the reference. */
int mraygb_measure_fp32_rate(mraygb_context *ctx, double *h_tflops);

/* ---- resident inputs ------------------------------------------------------------------------------------ */

/* A regular grid (RegularGrid, src/volume.h:31-123): float32, x fastest, z slowest, on the box [dmin, dmax].
 * `data` is a host pointer, or a device pointer when data_on_device != 0 (then it is copied, not adopted).
 * Replaces the per-call upload of RegularGridDevice (src/volume_device.cuh:52-97). */
int mraygb_upload_grid(mraygb_context *ctx, const float *data, int nx, int ny, int nz, const float dmin[3],
                       const float dmax[3], int data_on_device);

/* SPH particles (Particles, src/volume.h:125-157) with one smoothing length h, marched inside the box
 * [dmin, dmax] (Particles::domain).  x, y, z, v are n floats each: host pointers, or device pointers when
 * data_on_device != 0 (copied, not adopted).  The library builds the reference's uniform particle grid on the
 * device (Particles::create_grid, src/volume.cpp:55-81: cell size h, origin at the particles' minimum, 4x4x4
 * tiled cells), with the particles of a cell kept in their input order; it replaces the per-call upload of
 * ParticlesDevice (src/volume_device.cuh:135-186).  The particles replace a grid uploaded before, and the other
 * way round: generation samples the volume uploaded last.  1 <= n <= 2^31. */
int mraygb_upload_particles(mraygb_context *ctx, const float *x, const float *y, const float *z, const float *v,
                            uint64_t n, float h, const float dmin[3], const float dmax[3], int data_on_device);

/* SPH particles with a smoothing length per particle h[i] (n floats, host or device like x, y, z, v; each finite
 * and > 0) and the Wendland C2 kernel W(q) ~ (1 - q)^4 (1 + 4q) / h^3 for q = r / h < 1: a variant that the
 * reference does not have (its Particles carry one smoothing length and the cubic spline), so its parity is
 * checked against the oracle's restatement only.  The grid is the reference's grid with the largest h as its cell
 * size; samples are sum W v / sum W over the 27 neighbour cells, as the reference's sampler normalises.
 * Generation (mraygb_generate / mraygb_stage_generate_moments) samples it; the error-bound and reference
 * renderers return MRAYGB_NOT_SUPPORTED for it. */
int mraygb_upload_particles_h(mraygb_context *ctx, const float *x, const float *y, const float *z, const float *v,
                              const float *h, uint64_t n, const float dmin[3], const float dmax[3], int data_on_device);

/* The transfer-function table that reconstruction samples: 256 RGBA float entries of one row of
 * TransferFunction::data (src/transfer_function.h:30-60).  read_from_disk / preintegrate build tables whose
 * 256 rows are all equal (src/transfer_function.cpp:46-97), so one row is the whole table. */
int mraygb_upload_tf(mraygb_context *ctx, const float *table_rgba256);

/* ---- drop-in host API ----------------------------------------------------------------------------------- */

/* generate_device(cam, RegularGrid or Particles, MomentImageHost, GenerationParameters) over the volume
 * uploaded last.
 *   h_data         : capacity for W*H*m floats; receives the (compact, prediction-coded) moment data
 *   h_index        : W*H+1 u32 when gp->compact_image, else may be NULL      (MomentImageHost::index)
 *   h_bounds       : 2*W*H u16 (lower, upper) when gp->transform_to_bounds   (MomentImageHost::bounds)
 *   h_coding_params: 2*(m-1) u16 when prediction coded with the default warp (MomentImageHost::coding_params)
 *   h_data_size    : receives the number of floats written to h_data
 * The moment image's remaining flags follow from gp: is_compact = compact_image, prediction_code =
 * prediction_coding, coding_warp = coding_warp, domain = the grid's box. */
int mraygb_generate(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp, int width,
                    int height, int num_moments, float *h_data, uint32_t *h_index, uint16_t *h_bounds,
                    uint16_t *h_coding_params, uint64_t *h_data_size);

/* reconstruct_device(cam, MomentImageHost, TransferFunction, ColorImageHost, ReconstructionParameters) with
 * the uploaded transfer function.  The moment image is given by its members (h_index NULL = not compact,
 * h_bounds NULL = no bounds, h_coding_params NULL unless prediction coded with the default warp).
 *   h_rgba  : W*H*4 floats (the colour before the u8 store), or NULL
 *   h_rgba8 : W*H*4 bytes as ColorImageHost stores them (clamp + truncate, src/color_image.h:41-47), or NULL */
int mraygb_reconstruct(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp,
                       int width, int height, int num_moments, const float domain_min[3], const float domain_max[3],
                       const uint32_t *h_index, const float *h_data, uint64_t data_size, const uint16_t *h_bounds,
                       int prediction_code, int coding_warp, const uint16_t *h_coding_params, float *h_rgba,
                       uint8_t *h_rgba8);

/* moment_quantization::quantize_prediction_coding(mi, table) (src/moment_quantization.cpp:239-276 with
 * pack_bits :92-114) for a compact, prediction-coded image in host memory: per pixel in row-major order and per
 * moment index l ascending, code = trunc(clamp(v, 0, 1) * (2^table[l] - 1)), packed LSB first.  Like the
 * reference's packer it emits whole bytes only.  *h_nbytes receives the byte count; h_out (capacity bytes) may
 * be NULL to query the size. */
int mraygb_quantize_prediction_coding(mraygb_context *ctx, int width, int height, int num_moments,
                                      const uint32_t *h_index, const float *h_data, uint64_t data_size,
                                      const uint8_t *h_table, uint8_t *h_out, uint64_t capacity, uint64_t *h_nbytes);

/* dequantize_prediction_coding (src/moment_quantization.cpp:278-332 with unpack_bits :116-152) for a compact image
 * in host memory: the packed codes (num_bytes, as the quantizer wrote them) back to values in [0, 1], written to
 * h_data (data_size = index[W*H] floats), which the reconstruction then reads as the prediction-coded moments
 * (load_moment_image does this for a quantized file, src/moment_image_io.cpp). */
int mraygb_dequantize_prediction_coding(mraygb_context *ctx, int width, int height, int num_moments,
                                        const uint32_t *h_index, const uint8_t *h_table, const uint8_t *h_bytes,
                                        uint64_t num_bytes, float *h_data, uint64_t data_size);

/* create_quantization_table (src/measure_coding_error.cpp:374-438) as main.cpp:318-327 runs it before the codes
 * are written: on the sample_moment_image (src/moment_image_sample.h:33-62) of a compact, prediction-coded
 * moment image.  With sampling > 0 the sample is s x s pixels, s = min(W, sampling) = min(H, sampling), pixel
 * (x, y) of the sample being pixel (x * (W / s), y * (H / s)) of the image (the reference's
 * quantization_curve_sampling, 64 by default); the reference indexes a w x h sample as h x w, so a non-square
 * sample (min(W, sampling) != min(H, sampling)) returns MRAYGB_NOT_SUPPORTED.  With sampling <= 0 the whole
 * image is the sample (create_quantization_table applied to the image as given).
 *   h_table : num_moments bytes: [0] = 16, [1] = start_bits, then per index the fewest bits (>= 2, at most the
 *             previous index's) whose mean rRMSE stays below that of index 1 at start_bits.  The reference
 *             installs the table as its global quantization table (set_prediction_coding_quantization_table);
 *             here the caller passes it to mraygb_(stage_)quantize_prediction_coding.
 *   h_means : num_moments * 32 floats or NULL: the mean rRMSE of quantizing moment idx to b bits at
 *             [idx * 32 + b], for every idx in [1, m) and b in [min(2, start_bits), start_bits]; NaN elsewhere.
 * num_moments >= 2, start_bits in 1..31; the data must be prediction coded (residuals in [0, 1]). */
int mraygb_create_quantization_table(mraygb_context *ctx, int width, int height, int num_moments,
                                     const uint32_t *h_index, const float *h_data, uint64_t data_size,
                                     int coding_warp, const uint16_t *h_coding_params, int start_bits, int sampling,
                                     uint8_t *h_table, float *h_means);

/* reconstruct_error (src/moment_raymarcher.cpp:541-560; host form :516-539, GPU :693-752) over the volume uploaded
 * last: per pixel the Lagrange multipliers of its moments (prepare_moments with ep->bias), then along the eye ray
 * at t = t_near, t_near + step, ... <= t_far (src/raymarch_reconstruct.h:322-378) the bounded-MESE density at
 * phase(t) against the volume's mapped density at t, reduced by ep->error_type: the maximum, the RMSE or the P^2
 * estimate of the ep->error_percentile-th percentile (src/error_measures.h:30-229) of the absolute differences.
 *   h_error_bounds : W*H u16 as MomentImageHost::set_error_bound stores them (e * 65535 truncated,
 *                    src/moment_image.h:102-106)
 *   h_errors       : W*H floats before the u16 store, or NULL
 * Pixels without moments get 0 (the reference evaluates an empty multiplier array there). */
int mraygb_reconstruct_error(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_error_params *ep, int width,
                             int height, int num_moments, const uint32_t *h_index, const float *h_data,
                             uint64_t data_size, const uint16_t *h_bounds, int prediction_code, int coding_warp,
                             const uint16_t *h_coding_params, uint16_t *h_error_bounds, float *h_errors);

/* read_from_disk_uncertainty (src/transfer_function.cpp:233-248) on a float 1D table (read_tf's output: 256 RGBA):
 * box_filter (:151-186) for MRAYGB_ERROR_MAX and MRAYGB_ERROR_PERCENTILE, gaussian_filter (:188-231) for
 * MRAYGB_ERROR_RMSE, built on the device as a 256 x 256 RGBA table ([y][x]) that stays resident for the convolution
 * renderer.  h_table (256 * 256 * 4 floats) receives it when non-NULL. */
int mraygb_upload_uncertainty_tf(mraygb_context *ctx, const float *tf1d_rgba256, float step_size, int error_type,
                                 float *h_table);

/* A 256 x 256 RGBA uncertainty table given whole ([y][x], the layout of TransferFunction::data,
 * src/transfer_function.h:30-34), for callers that hold read_from_disk_uncertainty's result already (the seam
 * reconstruct_uncertainty_convolution_device takes the table, src/moment_raymarcher.cuh:84-86). */
int mraygb_upload_uncertainty_table(mraygb_context *ctx, const float *table_rgba256x256);

/* reconstruct_uncertainty_interpolation (mode 0) and reconstruct_uncertainty_convolution (mode 1)
 * (src/moment_raymarcher.cpp:562-717, GPU :755-950) with the error bounds of mraygb_reconstruct_error.  Mode 0
 * marches the density lerp(clamp(rho - e), clamp(rho + e), bound_interpolation) (ErrorBoundInterpolator,
 * src/reconstruction_techniques.h:99-155) with the transfer function of mraygb_upload_tf; mode 1 looks up the pair
 * (clamp(rho - e), clamp(rho + e)) for MRAYGB_ERROR_MAX, (rho, e) otherwise, in the table of
 * mraygb_upload_uncertainty_tf (reconstruct_ray_uncertainty_tf, src/raymarch_reconstruct.h:203-259).  Image
 * arguments and outputs as mraygb_reconstruct. */
int mraygb_reconstruct_uncertainty(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_uncertainty_params *up,
                                   int mode, int width, int height, int num_moments, const float domain_min[3],
                                   const float domain_max[3], const uint32_t *h_index, const float *h_data,
                                   uint64_t data_size, const uint16_t *h_bounds, const uint16_t *h_error_bounds,
                                   int prediction_code, int coding_warp, const uint16_t *h_coding_params,
                                   float *h_rgba, uint8_t *h_rgba8);

/* generate_reference (src/moment_raymarcher.cpp:64-80; GPU src/moment_raymarcher.cu:65-114): direct volume
 * rendering of the volume uploaded last with the transfer function of mraygb_upload_tf (reference_ray,
 * src/raymarch_reference.h:93-160), the ground truth of the moment path.  With rp->ss.enable and a positive
 * medium_scattering every sample marches a secondary ray towards the light (the brute-force transmittance of
 * raymarch_reference.h:40-75; the cache is mraygb_generate_reference_reconstructed_ss).  Outputs as
 * mraygb_reconstruct. */
int mraygb_generate_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp,
                              int width, int height, float *h_rgba, uint8_t *h_rgba8);

/* ---- single scattering: the transmittance cache ----------------------------------------------------------
 * The cache is a float grid of rp->ss.cache_size_x * _y * _z voxels (x fastest) over the domain of the light's
 * moment image, held by the context (SingleScatteringCacheHost, src/single_scattering_cache.h:33-59).  A
 * reconstruction with rp->ss.enable, rp->ss.use_cache and a positive medium_scattering samples it (trilinear,
 * RegularGrid::sample) at every sample for the in-scattered light T_ss * henyey_greenstein * intensity
 * (inscattering, src/raymarch_reconstruct.h:36-46 and 112-125); the marched form (use_cache = 0) returns
 * MRAYGB_NOT_SUPPORTED. */

/* reconstruct_single_scattering_cache(ss, tf, params) (src/moment_raymarcher.cpp:217-258): the moment image
 * rendered from the light (SingleScatteringImageHost::img, given by its members as in mraygb_reconstruct, the
 * light's camera light_cam) is prepared and re-marched with the transfer function of mraygb_upload_tf at
 * rp->step_size; every sample writes exp(-tau) into the voxel int((q - min) / (max - min) * size) of its position
 * q (ScatterGridHost::scatter, src/scatter_grid.h:54-66).  Where several samples reach a voxel the result is that
 * of the reference's loop run sequentially: the last pixel in row-major order, and its last sample there, wins
 * (the reference's parallel loop leaves the order open).  Voxels no sample reaches hold 0.  The cache becomes the
 * context's; h_cache (cache_size_x*y*z floats) receives a copy, or may be NULL. */
int mraygb_reconstruct_single_scattering_cache(mraygb_context *ctx, const mraygb_camera *light_cam,
                                               const mraygb_reconstruction_params *rp, int width, int height,
                                               int num_moments, const float domain_min[3], const float domain_max[3],
                                               const uint32_t *h_index, const float *h_data, uint64_t data_size,
                                               const uint16_t *h_bounds, int prediction_code, int coding_warp,
                                               const uint16_t *h_coding_params, float *h_cache);

/* A cache made elsewhere (SingleScatteringCacheHost(RegularGrid)): nx*ny*nz floats, x fastest, on the box
 * [dmin, dmax]; host pointer, or device pointer when data_on_device != 0 (copied). */
int mraygb_upload_single_scattering_cache(mraygb_context *ctx, const float *data, int nx, int ny, int nz,
                                          const float dmin[3], const float dmax[3], int data_on_device);

/* generate_reference_reconstructed_ss (src/moment_raymarcher.cpp:259-281): generate_reference of the volume
 * uploaded last with ref_from_rec_params(rp) (src/parameters.h:379-390), the in-scattered light's transmittance
 * sampled from the context's cache at each sample (compute_transmittance, src/raymarch_reference.h:77-86) instead
 * of marched.  Outputs as mraygb_reconstruct. */
int mraygb_generate_reference_reconstructed_ss(mraygb_context *ctx, const mraygb_camera *cam,
                                               const mraygb_reconstruction_params *rp, int width, int height,
                                               float *h_rgba, uint8_t *h_rgba8);

/* ---- the moment-image file format ------------------------------------------------------------------------
 * write_moment_image / load_moment_image (src/moment_image_io.cpp:291-529) with the entropy coder of
 * src/moment_image_coding.cpp:98-234: the same bytes for the same image and options, except that compressed
 * sections are LZ4 blocks of this library's encoder (any LZ4 decoder reads them; LZ4_compress_default would choose
 * other matches).  Quantization and dequantization of the payload run on the GPU; LZ4 and the arithmetic coder
 * (one stream per moment index, on host threads) on the host.  `quant_table` (num_moments bytes) stands for the
 * reference's global prediction-coding table (moment_quantization.cpp:166-223): NULL = none set, so the header's
 * table flag is 0 and prediction codes use [16, bits, bits, ...]; entropy coding of a prediction-coded image needs
 * it.  Entropy coding needs table entries of 1..14 bits for moment indices >= 1. */

/* Encodes the image into a buffer held by the context; *h_bytes receives its size.  mraygb_copy_encoded copies it
 * out (capacity >= the size). */
int mraygb_encode_moment_image(mraygb_context *ctx, const mraygb_moment_image *mi, int compress,
                               int quantization_bits, int entropy_coding, const uint8_t *quant_table,
                               uint64_t *h_bytes);
int mraygb_copy_encoded(mraygb_context *ctx, uint8_t *out, uint64_t capacity);

/* Decodes a file held in memory.  With mi->data NULL only the shape, flags, data_size and has_* fields are filled
 * (and the table, when the file holds one: *has_quant_table = 1 and num_moments bytes into quant_table if it is not
 * NULL); call again with index (compact images), data and the arrays the file holds.  A static image written with
 * compression and quantization cannot be read (the reference's writer puts a byte before its block that its reader
 * does not expect): MRAYGB_NOT_SUPPORTED. */
int mraygb_decode_moment_image(mraygb_context *ctx, const uint8_t *bytes, uint64_t n, mraygb_moment_image *mi,
                               uint8_t *quant_table, int *has_quant_table);

/* The same through files (write_moment_image(mi, filename, compress, quantizationBits, entropy_coding) and
 * load_moment_image(filename)); loading reads the file on each call. */
int mraygb_write_moment_image(mraygb_context *ctx, const char *path, const mraygb_moment_image *mi, int compress,
                              int quantization_bits, int entropy_coding, const uint8_t *quant_table);
int mraygb_load_moment_image(mraygb_context *ctx, const char *path, mraygb_moment_image *mi, uint8_t *quant_table,
                             int *has_quant_table);

/* Host-only pieces of the format (no context, no GPU): an LZ4 block of n bytes (returns its size, 0 when it does
 * not fit in cap) and back (returns the decoded size, -1 for a malformed block); the entropy-coded payload of u16
 * codes in the layout of the moment data (index: W*H+1 offsets; the size into *h_bytes, the bytes when out holds
 * them) and back (returns MRAYGB_OK or MRAYGB_INVALID_ARGUMENT for a malformed payload).  threads <= 0: all host
 * threads. */
uint64_t mraygb_lz4_compress(const uint8_t *src, uint64_t n, uint8_t *dst, uint64_t cap);
int64_t mraygb_lz4_decompress(const uint8_t *src, uint64_t n, uint8_t *dst, uint64_t cap);
int mraygb_entropy_encode(int width, int height, int num_moments, const uint32_t *index, const uint16_t *codes,
                          const uint8_t *table, int threads, uint8_t *out, uint64_t capacity, uint64_t *h_bytes);
int mraygb_entropy_decode(const uint8_t *bytes, uint64_t n, int width, int height, int num_moments,
                          const uint32_t *index, const uint8_t *table, int threads, uint16_t *codes);

/* ---- stage API: device pointers, ordered on the context stream ------------------------------------------ */

/* Per-ray moments over the uploaded grid (generate_ray, src/raymarch_generate.h:69-148, driven as
 * generate_moments_kernel, src/moment_raymarcher.cu:163-185).
 *   d_moments: W*H*m floats (non-compact layout; missed rays get zeros)
 *   d_bounds : 2*W*H u16, written when gp->transform_to_bounds (may be NULL otherwise)
 *   d_counts : W*H u32 moment counts for compaction (compute_num_moments, src/moment_compaction.h:147-174),
 *              written when gp->compact_image (may be NULL otherwise). */
int mraygb_stage_generate_moments(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                                  int width, int height, int num_moments, float *d_moments, uint16_t *d_bounds,
                                  uint32_t *d_counts);

/* MomentImageDevice::compact (src/moment_image_device.cu:83-110): exclusive scan of the counts into
 * d_index[W*H+1] and copy of the moments into the compact buffer (capacity floats).  *h_total receives the
 * compact size (one device->host read of 4 bytes). */
int mraygb_stage_compact(mraygb_context *ctx, int width, int height, int num_moments, const uint32_t *d_counts,
                         const float *d_moments, uint32_t *d_index, float *d_compact, uint64_t capacity,
                         uint64_t *h_total);

/* cosf / sinf as the MESE algebra evaluates them on the device: the zeroth-moment phase of
 * trigonometricToExponentialMoments (src/mese/MESE_dynamic.h:38-40) and of transform_dequantization_real
 * (src/moment_prediction_coding.h:103-104), which the reference takes from the host C library.  For every float
 * x in [-pi, pi] the results equal the C library's of the machine that built this library, bit for bit (a
 * double-precision evaluation corrected by a table generated from that library at build time); outside that
 * interval, the double-precision functions rounded to float.  n floats of d_x in, d_sin and d_cos out. */
int mraygb_stage_libm_sincosf(mraygb_context *ctx, const float *d_x, float *d_sin, float *d_cos, uint64_t n);

/* MomentImageDevice::prediction_encode (src/moment_image_device.cu:166-195; host form
 * MomentImageHost::prediction_encode, src/moment_image.cpp:96-152) in place on a compact image: bias lerp,
 * trigonometric -> exponential moments, Levinson-style encode, projection to the real line, coding parameters
 * (per-index |min|, |max - min| / 2 over the image, ceil-quantized to u16, written to d_coding_params[2(m-1)]
 * for the default warp) and the warp of every residual to [0, 1]. */
int mraygb_stage_prediction_encode(mraygb_context *ctx, int width, int height, int num_moments,
                                   const uint32_t *d_index, float *d_data, uint64_t data_size, int coding_warp,
                                   float bias, uint16_t *d_coding_params);

/* quantize_prediction_coding on device buffers: d_out must hold ceil(bits / 32) * 4 bytes (capacity);
 * *h_nbytes receives the number of valid bytes (whole bytes, as the reference's packer). */
int mraygb_stage_quantize_prediction_coding(mraygb_context *ctx, int width, int height, int num_moments,
                                            const uint32_t *d_index, const float *d_data, const uint8_t *h_table,
                                            uint8_t *d_out, uint64_t capacity, uint64_t *h_nbytes);

/* dequantize_prediction_coding (src/moment_quantization.cpp:278-332 with unpack_bits :135-160): codes back to
 * values in [0, 1] in the compact layout; codes the stream does not hold read as 0. */
int mraygb_stage_dequantize_prediction_coding(mraygb_context *ctx, int width, int height, int num_moments,
                                              const uint32_t *d_index, const uint8_t *h_table,
                                              const uint8_t *d_bytes, uint64_t num_bytes, float *d_data);

/* mraygb_create_quantization_table on device buffers (d_coding_params: 2(m-1) u16 for the default warp).  The
 * table and the means are returned in host memory; the call waits for the stream. */
int mraygb_stage_create_quantization_table(mraygb_context *ctx, int width, int height, int num_moments,
                                           const uint32_t *d_index, const float *d_data, int coding_warp,
                                           const uint16_t *d_coding_params, int start_bits, int sampling,
                                           uint8_t *h_table, float *h_means);

/* mraygb_reconstruct_error on the Lagrange multipliers of mraygb_stage_prepare_moments (d_errors may be NULL). */
int mraygb_stage_reconstruct_error(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_error_params *ep,
                                   int width, int height, int num_moments, const uint32_t *d_index,
                                   const float *d_pmoments, const uint16_t *d_bounds, uint16_t *d_error_bounds,
                                   float *d_errors);

/* mraygb_reconstruct_uncertainty on the Lagrange multipliers of mraygb_stage_prepare_moments: d_rgba W*H*4 floats. */
int mraygb_stage_reconstruct_uncertainty(mraygb_context *ctx, const mraygb_camera *cam,
                                         const mraygb_uncertainty_params *up, int mode, int width, int height,
                                         int num_moments, const float domain_min[3], const float domain_max[3],
                                         const uint32_t *d_index, const float *d_pmoments, const uint16_t *d_bounds,
                                         const uint16_t *d_error_bounds, float *d_rgba);

/* mraygb_generate_reference into device memory: d_rgba W*H*4 floats. */
int mraygb_stage_generate_reference(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reference_params *rp,
                                    int width, int height, float *d_rgba);

/* mraygb_reconstruct_single_scattering_cache from the light image's multipliers (mraygb_stage_prepare_moments)
 * in device memory; d_cache receives the cache (cache_size_x*y*z floats) or may be NULL. */
int mraygb_stage_reconstruct_single_scattering_cache(mraygb_context *ctx, const mraygb_camera *light_cam,
                                                     const mraygb_reconstruction_params *rp, int width, int height,
                                                     int num_moments, const float domain_min[3],
                                                     const float domain_max[3], const uint32_t *d_index,
                                                     const float *d_pmoments, const uint16_t *d_bounds,
                                                     float *d_cache);

/* mraygb_generate_reference_reconstructed_ss into device memory: d_rgba W*H*4 floats. */
int mraygb_stage_generate_reference_reconstructed_ss(mraygb_context *ctx, const mraygb_camera *cam,
                                                     const mraygb_reconstruction_params *rp, int width, int height,
                                                     float *d_rgba);

/* Compaction that allocates nothing, for callers that must not call cudaMalloc / cudaFree while they work:
 * renderers and services that reserve all device memory up front in their own pool or arena (where an
 * allocation can stall every stream on the device, exceed the pool's budget or fragment memory the pool
 * manages).  It has no counterpart in the reference.  Same result as mraygb_stage_compact, but without a
 * context: it runs on the current device and on `stream` (a cudaStream_t, NULL for the default stream), and
 * the scan's block sums live in a fixed device array of 16448 words (64 KiB) that each GPU loading the library
 * holds until the process exits.  Limit: W * H <= 16,777,216 pixels (4096 x 4096); larger images return
 * MRAYGB_INVALID_ARGUMENT.  The first call on a device looks up the array's device address (set-up) and keeps
 * it for the life of the process: after cudaDeviceReset, or with a non-primary driver context current on that
 * device, the kept address is not valid, so such callers must not use this entry point.  Every call reads the
 * compact size back and waits for `stream`, so it blocks the calling thread and cannot be used inside stream
 * capture.  All calls share the array: calls that overlap on the GPU race on it and must be ordered by the
 * caller.  Failures are reported by the return code only (there is no context to hold a message). */
int mraygb_stage_compact_noalloc(void *stream, int width, int height, int num_moments, const uint32_t *d_counts,
                                 const float *d_moments, uint32_t *d_index, float *d_compact, uint64_t capacity,
                                 uint64_t *h_total);

/* Lagrange multipliers per pixel (prepare_moments_device, src/moment_image_device.cu:306-335): the moment data
 * in the compact layout (d_index) or, with d_index NULL, the W*H*m layout; output in the same layout. */
int mraygb_stage_prepare_moments(mraygb_context *ctx, int width, int height, int num_moments, const uint32_t *d_index,
                                 const float *d_data, int prediction_code, int coding_warp,
                                 const uint16_t *d_coding_params, float bias, float *d_pmoments);

/* MESE re-march per pixel (reconstruct_moments_kernel, src/moment_raymarcher.cu:339-384) with the uploaded
 * transfer function; d_rgba: W*H*4 floats; d_rgba8: W*H*4 bytes or NULL. */
int mraygb_stage_reconstruct(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_reconstruction_params *rp,
                             int width, int height, int num_moments, const float domain_min[3],
                             const float domain_max[3], const uint32_t *d_index, const float *d_pmoments,
                             const uint16_t *d_bounds, float *d_rgba, uint8_t *d_rgba8);

/* ---- differentiation form -------------------------------------------------------------------------------
 * No counterpart in the reference.  The moment-image method with four changes that make an image-space loss
 * smooth almost everywhere in the volume and the transfer function: no compaction (every pixel keeps m moments),
 * the re-march reads the unquantized per-pixel density bounds, the MESE density uses the exact arctangent, and the
 * transfer-function row is sampled in the front density at the texel centres of the reference's GPU texture
 * (TransferFunctionDevice::sample, src/transfer_function_device.cuh:30-65: u = 256 fs - 1/2, clamp to edge), as a
 * uniform cubic B-spline (the default: the loss is then smooth where a density crosses an entry) or linearly, the
 * GPU path's own interpolation with exact weights (mraygb_set_diff_tf_sampling).  All buffers are device pointers
 * on the context's stream. */

enum
{
    MRAYGB_DIFF_TF_BSPLINE = 0, /* the row as a uniform cubic B-spline in the front density */
    MRAYGB_DIFF_TF_LINEAR = 1   /* the row linear in the front density (the reference's GPU sampling) */
};

/* Selects the differentiation form's transfer-function sampling for the later forward and backward calls of the
 * context (MRAYGB_DIFF_TF_BSPLINE by default).  A backward must run with the sampling of its forward. */
int mraygb_set_diff_tf_sampling(mraygb_context *ctx, int sampling);

/* Forward over the volume uploaded last: generate (gp->compact_image = 0, prediction_coding = 0,
 * transform_to_bounds = 1; m <= 64), Lagrange multipliers in the context's precision form, re-march with the
 * transfer-function row d_tf (256 RGBA floats).  Writes d_moments (W*H*m), d_bounds4 (W*H*4: lo, hi and the
 * samples' min, max), d_pmoments (W*H*m) and d_rgba (W*H*4), which the backward reads.  16-byte aligned float4
 * buffers.  In the FP32 precision form the context also keeps, for these buffers, the preparation's Levinson
 * solution and exponential moments (W*H*2m complex floats), which the backward's preparation adjoint reads. */
int mraygb_diff_forward(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                        const mraygb_reconstruction_params *rp, int width, int height, int m, const float *d_tf,
                        float *d_moments, float *d_bounds4, float *d_pmoments, float *d_rgba);

/* Adjoint of mraygb_diff_forward for the loss gradient d_grad_rgba (W*H*4): adds d loss / d transfer-function row
 * to d_grad_tf (256*4) and, when d_grad_volume is not NULL (regular grids only), d loss / d voxel density to
 * d_grad_volume (nx*ny*nz).  The forward's buffers must be unchanged.  When the context's kept preparation arrays
 * belong to other buffers (another forward ran since, or the forward ran in another precision form), the volume
 * gradient first runs the FP32 preparation of d_moments again to rebuild them. */
int mraygb_diff_backward(mraygb_context *ctx, const mraygb_camera *cam, const mraygb_generation_params *gp,
                         const mraygb_reconstruction_params *rp, int width, int height, int m, const float *d_tf,
                         const float *d_moments, const float *d_bounds4, const float *d_pmoments, const float *d_rgba,
                         const float *d_grad_rgba, float *d_grad_tf, float *d_grad_volume);

#ifdef __cplusplus
}
#endif

#endif /* MRAYGB_H */
