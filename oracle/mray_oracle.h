/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C, CPU restatement of the reference (TobiasRp/mray) moment-image
 * hot path: ray setup, volume sampling, moment generation, compaction,
 * prediction coding, quantization and bit packing, MESE preparation and the
 * MESE re-march.  It exists to check the CUDA product and to time the CPU
 * baseline; the product never links, loads or calls it.
 *
 * Every function comes in two precisions compiled from one body
 * (oracle_body.inc):
 *   *_f32 : the reference's own float arithmetic, operation for operation
 *           (including the places where the reference promotes to double),
 *           built with -ffp-contract=off so that it reproduces the
 *           reference's compiled CPU path;
 *   *_f64 : the same method evaluated in double precision with exact
 *           constants (the FP64 oracle the new precision form is compared
 *           against).
 * Each function cites the reference file:line it follows.
 */
#ifndef MRAY_ORACLE_H
#define MRAY_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/mraygb_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Regular grid (src/volume.h:31-123): x fastest, z slowest, float data. */
typedef struct oracle_grid
{
    const float *data;
    int nx, ny, nz;
    float dmin[3], dmax[3];
} oracle_grid;

/* SPH particles (src/volume.h:125-157) with the reference's uniform grid (src/particle_grid.cuh:64-403): cell
 * size = smoothing length, origin = the particles' minimum, 4x4x4-tiled cell order.  Built by
 * oracle_particles_create, which sorts the particles by cell (stable: original order inside a cell) and keeps the
 * first particle of every cell as a CSR start array. */
typedef struct oracle_particles
{
    float *x, *y, *z, *v; /* sorted by cell */
    uint64_t n;
    float h, inv_h;
    float dmin[3], dmax[3]; /* the ray box (the loader's domain) */
    float gmin[3];
    float inv_cell, r2;
    int sx, sy, sz, tz;
    uint32_t total;
    uint32_t *cell_start; /* total + 1 */
    float *hh;            /* per-particle smoothing lengths, sorted like x (Wendland C2 variant), or NULL */
} oracle_particles;

oracle_particles *oracle_particles_create(const float *x, const float *y, const float *z, const float *v, uint64_t n,
                                          float h, const float dmin[3], const float dmax[3]);
/* The variant with a smoothing length per particle and the Wendland C2 kernel (not in the reference, whose
 * particles carry one smoothing length): the same grid with the largest h as its cell size; a particle contributes
 * (1 - q)^4 (1 + 4q) / h^3 at q = r / h < 1 (and r^2 below the largest h squared, the cells' radius test). */
oracle_particles *oracle_particles_create_h(const float *x, const float *y, const float *z, const float *v,
                                            const float *h, uint64_t n, const float dmin[3], const float dmax[3]);
void oracle_particles_destroy(oracle_particles *p);
/* cell order of the grid (UniformGridDevice::getIndexFromCell, particle_grid.cuh:64-83) */
uint32_t oracle_particles_cell_index(const oracle_particles *p, int cx, int cy, int cz);

/* Options that select between reference-faithful and exact evaluation. */
typedef struct oracle_options
{
    int exact_atan;   /* 0: fast_atan polynomial (reference), 1: atan()   */
    int nthreads;     /* OpenMP threads (<=0: runtime default)            */
    int row_begin;    /* first image row processed                        */
    int row_end;      /* one past the last row (<=0: image height)        */
    int row_step;     /* process every row_step-th row (<=0: 1)           */
    /* The differentiation form (a variant of the method whose loss is smooth almost everywhere in its inputs;
     * combine with exact_atan = 1):
     *   tf_bspline : 1: reconstruct samples the transfer function row as a uniform cubic B-spline in the front
     *                density, knots at the texel centres of the reference's GPU texture (u = 256 fs - 1/2); 2:
     *                linearly in the front density at those texel centres (the texture's sampling, exact weights);
     *   bounds_out : generate writes the per-pixel density bounds (lo, hi) unquantized, 2*W*H of R;
     *   bounds_in  : reconstruct reads (lo, hi) from here (2*W*H of R) instead of the u16 bounds. */
    int tf_bspline;
    void *bounds_out;
    const void *bounds_in;
    /* generate only: columns col_begin, col_begin + col_step, ... below col_end (col_end <= 0: the width) */
    int col_begin, col_end, col_step;
    /* reconstruct and generate_reference: the single-scattering transmittance cache (NULL: none; generate_reference
     * then marches the transmittance when rp->ss.enable) */
    const oracle_grid *ss_cache;
    /* reconstruct only: added to every reconstructed density before the transfer-function lookup (0: the method).
     * The reference's CPU sampling of the table (transfer_function.h:44-59) takes the texel pair from the front
     * density and the blend weight from the back density's fractional part, so the colour jumps where a density
     * crosses a multiple of 1/256; a small offset shows which pixels sit on such a jump. */
    double density_offset;
    /* reconstruct only: per-pixel offsets (W*H of R) used instead of density_offset when not NULL */
    const void *density_offsets;
} oracle_options;

#define ORACLE_DECL(R, SFX)                                                                                         \
    /* per-ray generation over an image (moment_raymarcher.cpp:121-166, raymarch_generate.h:69-148)         */      \
    void oracle_generate_moments_particles_##SFX(const mraygb_camera *cam, const mraygb_generation_params *gp,     \
                                                 const oracle_particles *parts, int width, int height,              \
                                                 int num_moments, R *moments, uint16_t *bounds, uint32_t *counts,   \
                                                 const oracle_options *opt);                                         \
    R oracle_particles_sample_##SFX(const oracle_particles *parts, const R p[3]);                                   \
    void oracle_generate_moments_##SFX(const mraygb_camera *cam, const mraygb_generation_params *gp,               \
                                       const oracle_grid *grid, int width, int height, int num_moments,              \
                                       R *moments, uint16_t *bounds, uint32_t *counts, const oracle_options *opt);   \
    /* Lagrange multipliers per pixel (moment_image.cpp:154-183); data in the working precision              */    \
    void oracle_prepare_moments_##SFX(int width, int height, int num_moments, const uint32_t *index,               \
                                      const R *data, int prediction_code, int coding_warp,                           \
                                      const uint16_t *coding_params, float bias, R *pmoments,                        \
                                      const oracle_options *opt);                                                    \
    /* MESE re-march per pixel, float RGBA before the u8 store (moment_raymarcher.cpp:283-327)               */      \
    void oracle_reconstruct_##SFX(const mraygb_camera *cam, const mraygb_reconstruction_params *rp,                \
                                  int width, int height, int num_moments, const float domain_min[3],                 \
                                  const float domain_max[3], const uint32_t *index, const R *pmoments,               \
                                  const uint16_t *bounds, const R *tf_table, R *rgba,                                 \
                                  const oracle_options *opt);                                                        \
    /* an error measure fed value by value, error() after each update (error_measures.h:30-229)               */   \
    void oracle_error_stream_##SFX(int type, int percentile, int n, const R *values, R *out);                      \
    /* the single-scattering transmittance cache of a light image, sequential (moment_raymarcher.cpp:217-258) */   \
    void oracle_ss_cache_##SFX(const mraygb_camera *light_cam, const mraygb_reconstruction_params *rp, int width,    \
                               int height, int num_moments, const float domain_min[3], const float domain_max[3],    \
                               const uint32_t *index, const R *pmoments, const uint16_t *bounds,                     \
                               const R *tf_table, float *cache);                                                     \
    /* MESE primitives (mese/MESE_dynamic.h)                                                                  */    \
    void oracle_trig_to_exp_##SFX(int n, const R *trig, R *exp_out /* 2n */);                                     \
    void oracle_exp_to_trig_##SFX(int n, const R *exp_in /* 2n */, R *trig_out /* 2n */);                         \
    void oracle_levinson_##SFX(int n, const R *first_col /* 2n */, R *solution /* 2n */);                         \
    void oracle_prepare_lagrange_##SFX(int n, const R *trig, R *lagrange);                                        \
    R oracle_evaluate_mese_##SFX(int n, R phase, const R *lagrange, int exact_atan);                              \
    R oracle_fast_atan_##SFX(R x);                                                                                 \
    void oracle_autocorrelation_##SFX(int n, const R *signal /* 2n */, R *out /* 2n */);                          \
    void oracle_correlation_##SFX(int n, const R *lhs, const R *rhs, R *out);                                     \
    void oracle_imaginary_correlation_##SFX(int n, const R *lhs, const R *rhs, R *out /* n */);                   \
    /* prediction coding (moment_prediction_coding.h)                                                         */    \
    void oracle_encode_##SFX(int n, const R *exp_in, R *code);                                                     \
    void oracle_decode_##SFX(int n, const R *code, R *exp_out, R *eval_poly);                                     \
    void oracle_transform_quantization_real_##SFX(int n, const R *code, R c0, R *out);                            \
    void oracle_transform_dequantization_real_##SFX(int n, const R *in, R *code, int warp, const R *params);      \
    /* moment compaction (moment_compaction.h)                                                                 */   \
    int oracle_determine_best_number_moments_##SFX(int n, const R *moments, R error_threshold);                  \
    void oracle_count_moments_##SFX(int num_pixels, int m, const R *moments, const uint32_t *counts_in,          \
                                    R error_threshold, uint32_t *counts_out, int nthreads);                        \
    void oracle_evaluate_unknown_moments_##SFX(int n, const R *exp_in, int max_moments, R *new_exp);              \
    void oracle_exponential_to_bounded_moments_##SFX(int n, const R *exp_in, R *bounded, int known);             \
    R oracle_rmse_##SFX(int n, int m, const R *pred /* complex */, const R *target);                              \
    /* volume / ray helpers                                                                                    */   \
    R oracle_grid_sample_##SFX(const oracle_grid *grid, const R p[3]);                                            \
    void oracle_eye_ray_##SFX(const mraygb_camera *cam, int x, int y, int width, int height, R origin[3],         \
                              R dir[3]);                                                                           \
    int oracle_intersect_aabb_##SFX(const R origin[3], const R dir[3], const float bmin[3], const float bmax[3],  \
                                    R *t_near, R *t_far);                                                          \
    void oracle_tf_sample_##SFX(const R *tf_table, R fs, R bs, R out[4]);                                           \
    void oracle_tf_sample_bspline_##SFX(const R *tf_table, R fs, R out[4]);                                         \
    void oracle_tf_sample_linear_##SFX(const R *tf_table, R fs, R out[4]);                                          \
    /* quantization curve (measure_coding_error.cpp:92-192, 357-438) on a compact prediction-coded image       */   \
    R oracle_measure_idx_error_##SFX(int width, int height, int num_moments, const uint32_t *index, const R *data, \
                                     int coding_warp, const uint16_t *coding_params, int idx, int b, R *errors,     \
                                     uint32_t *size, int nthreads);                                                 \
    int oracle_create_quantization_table_##SFX(int width, int height, int num_moments, const uint32_t *index,      \
                                               const R *data, int coding_warp, const uint16_t *coding_params,       \
                                               int start_bits, uint8_t *table, R *means, int nthreads);     \
    /* error bounds and uncertainty rendering (moment_raymarcher.cpp:516-706)                                */    \
    void oracle_reconstruct_error_##SFX(const mraygb_camera *cam, const mraygb_error_params *ep,                  \
                                        const oracle_grid *grid, const oracle_particles *parts, int width,         \
                                        int height, int num_moments, const uint32_t *index, const R *data,          \
                                        int prediction_code, int coding_warp, const uint16_t *coding_params,        \
                                        const uint16_t *bounds, R *errors, uint16_t *error_bounds,                  \
                                        const oracle_options *opt);                                                  \
    void oracle_uncertainty_tf_##SFX(const R *tf1d, float step_size, int error_type, R *table);                  \
    void oracle_reconstruct_uncertainty_##SFX(const mraygb_camera *cam, const mraygb_uncertainty_params *up,      \
                                              int mode, int width, int height, int num_moments,                    \
                                              const float domain_min[3], const float domain_max[3],                \
                                              const uint32_t *index, const R *data, int prediction_code,           \
                                              int coding_warp, const uint16_t *coding_params,                      \
                                              const uint16_t *bounds, const uint16_t *error_bounds, const R *T,    \
                                              R *rgba, const oracle_options *opt);                         \
    /* reference direct volume rendering (moment_raymarcher.cpp:45-79)                                      */     \
    void oracle_generate_reference_##SFX(const mraygb_camera *cam, const mraygb_reference_params *rp,             \
                                         const oracle_grid *grid, const oracle_particles *parts, int width,        \
                                         int height, const R *T, R *rgba, const oracle_options *opt);

ORACLE_DECL(float, f32)
ORACLE_DECL(double, f64)

/* ---- integer / byte work and float-only container steps ---------------------------------------------------- */

/* MomentImageHost::compact (moment_image.cpp:69-94).  counts[W*H] -> index[W*H+1]; data is copied from the
 * W*H*m layout to the compact layout.  Returns the compact size. */
uint64_t oracle_compact(int width, int height, int num_moments, const uint32_t *counts, const float *moments,
                        uint32_t *index, float *compact);

/* MomentImageHost::prediction_encode (moment_image.cpp:96-152) on a compact image, in place.  Writes the
 * 2(m-1) u16 coding parameters when warp == DEFAULT_TRANSFORMED. */
void oracle_prediction_encode(int width, int height, int num_moments, const uint32_t *index, float *data,
                              uint64_t data_size, int coding_warp, float bias, uint16_t *coding_params,
                              const oracle_options *opt);

/* find_coding_transform_parameters (coding_transform.h:37-68), float params 2(m-1). */
void oracle_find_coding_transform_parameters(int width, int height, int num_moments, const uint32_t *index,
                                             const float *data, uint64_t data_size, float *params);
/* CodingParamType::quantize (coding_params.h:56-66). */
void oracle_quantize_coding_params(int num_params, const float *params, uint16_t *q);

/* quantize / dequantize (moment_quantization.cpp:37-66). */
uint32_t oracle_quantize(float value, int num_bits, float vmin, float vmax);
float oracle_dequantize(uint32_t q, int num_bits, float vmin, float vmax);

/* quantize_prediction_coding (moment_quantization.cpp:239-276) + pack_bits (:92-114).
 * table[m] = bits per index.  Returns the number of bytes written (the trailing partial byte is dropped,
 * as the reference's packer does).  out may be NULL to query the size. */
uint64_t oracle_quantize_prediction_coding(int width, int height, int num_moments, const uint32_t *index,
                                           const float *data, const uint8_t *table, uint8_t *out);
/* dequantize_prediction_coding (moment_quantization.cpp:278-332) + unpack_bits (:116-152). */
void oracle_dequantize_prediction_coding(int width, int height, int num_moments, const uint32_t *index,
                                         const uint8_t *table, const uint8_t *bytes, uint64_t num_bytes,
                                         float *data);
/* Test switch: cosf / sinf of the f32 prediction-coding dequantization from the C library (0, the default, as the
 * reference's CPU build) or correctly rounded (1). */
void oracle_set_rounded_trig(int on);
/* sample_moment_image (moment_image_sample.h:33-62) followed by MomentImageHost::compact (moment_image.cpp:69-94)
 * for a compact image: pixel (x, y) of the s x s sample is pixel (x * (W / s), y * (H / s)) of the image.
 * s_index[s*s+1]; s_data may be NULL to query the compact size, which is returned. */
uint64_t oracle_sample_moment_image(int width, int height, const uint32_t *index, const float *data, int s,
                                    uint32_t *s_index, float *s_data);
/* get_prediction_coding_quantization_table default (moment_quantization.cpp:186-203). */
void oracle_default_quantization_table(int num_moments, int num_bits, uint8_t *table);

/* TransferFunction preintegrate (transfer_function.cpp:46-97): the table row that every row equals.
 * tf1d: 256 RGBA floats; out: 256 RGBA floats. */
void oracle_preintegrate(const float *tf1d, float step_size, float *table);

/* ColorImageHost::set_color: clamp and truncate to u8 (color_image.h:41-47, 60-65). */
void oracle_rgba_to_u8(uint64_t num_pixels, const float *rgba, uint8_t *out);

/* The C library's cosf / sinf over n floats (OpenMP), as trigonometricToExponentialMoments calls them
 * (mese/MESE_dynamic.h:38-40). */
void oracle_libm_sincosf(uint64_t n, const float *x, float *s, float *c);

/* euler_exp as the reference's CPU build resolves it (complex_algebra.h:155-158). */
void oracle_euler_exp_f32(float x, float out[2]);

#ifdef __cplusplus
}
#endif

#endif /* MRAY_ORACLE_H */
