/*
 * Plain-old-data mirrors of the parameter and camera types that mray's moment
 * raymarcher API takes (TobiasRp/mray).  Field order, types and meaning follow
 * the reference field for field so that a shim around the reference's C++
 * signatures is a member-wise copy:
 *
 *   mraygb_camera                 <- cut::Camera            (src/cut/camera.h:39-55)
 *   mraygb_generation_params      <- GenerationParameters   (src/parameters.h:49-70)
 *   mraygb_reconstruction_params  <- ReconstructionParameters (src/parameters.h:231-247)
 *   mraygb_error_params           <- ErrorReconstructionParameters (src/parameters.h:124-137)
 *   mraygb_uncertainty_params     <- UncertaintyReconstructionParameters (src/parameters.h:319-325)
 *   mraygb_single_scattering_params <- SingleScatteringParameters (src/parameters.h:173-193)
 *   mraygb_reference_params       <- ReferenceParameters (src/parameters.h:339-350)
 *   mraygb_moment_image           <- MomentImageHost (src/moment_image.h:33-147), as arrays
 *
 * C++ `bool` members are stored as uint8_t (same size and alignment under the
 * Itanium and AAPCS64 ABIs).  No CUDA or torch types appear here.
 */
#ifndef MRAYGB_TYPES_H
#define MRAYGB_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cut::Camera (src/cut/camera.h:39-55).  transform is row-major, m[row][col],
 * exactly as cut::Mat4f stores it.  The inverse view transform of the
 * reference is not needed on this path and is not mirrored. */
typedef struct mraygb_camera
{
    float transform[4][4];
    float position[3];
    float right[3];
    float up[3];
    float dir[3];
    float scale;
    float aspect;
    float znear;
    int32_t orthographic;
} mraygb_camera;

/* GenerationParameters (src/parameters.h:49-70), same defaults. */
typedef struct mraygb_generation_params
{
    float step_size;               /* 1.0  */
    float step_size_write_samples; /* 1.5  (unused on this path) */
    float data_min;                /* 0.0  */
    float data_max;                /* 1.0  */
    float error_threshold;         /* 1.0  */
    float bias;                    /* 1e-4 */
    uint8_t compact_image;         /* 1 */
    uint8_t prediction_coding;     /* 1 */
    uint8_t compress;              /* 0 (file format; not on this path) */
    uint8_t entropy_coding;        /* 0 (file format; not on this path) */
    uint8_t quantization_bits;     /* 32 */
    uint8_t pad0[3];
    int32_t coding_warp;           /* 0 = CODING_WARP_DEFAULT_TRANSFORMED, 1 = CODING_WARP_NONE */
    int32_t quantization_curve_sampling; /* 64 (unused on this path) */
    uint8_t transform_to_bounds;   /* 0 */
    uint8_t pad1[3];
    float transform_bound_eps;     /* 0.01 */
} mraygb_generation_params;

/* SingleScatteringParameters (src/parameters.h:173-193), same defaults.  The direction is used as given (the
 * reference does not normalise it). */
typedef struct mraygb_single_scattering_params
{
    uint8_t enable;           /* 0 */
    uint8_t use_cache;        /* 1 (reconstruction samples the transmittance cache; 0, the marched form, is
                                 not supported) */
    uint8_t pad0[2];
    int32_t cache_size_x;     /* 128 */
    int32_t cache_size_y;     /* 128 */
    int32_t cache_size_z;     /* 128 */
    float step_size_factor;   /* 1.0 */
    float henyey_greenstein_g; /* 0.0 */
    float direction_x;        /* 0.0 */
    float direction_y;        /* -1.0 */
    float direction_z;        /* 0.1 */
    float intensity_r;        /* 1.0 */
    float intensity_g;        /* 1.0 */
    float intensity_b;        /* 1.0 */
} mraygb_single_scattering_params;

/* ReconstructionParameters (src/parameters.h:231-247), same defaults and the
 * same layout (the single-scattering block starts at byte 36). */
typedef struct mraygb_reconstruction_params
{
    float bias;                    /* 1e-6 */
    float medium_emission;         /* 0.1  */
    float medium_scattering;       /* 0.1  */
    float early_ray_termination;   /* 0.95 */
    float data_min;                /* 0.0  */
    float data_max;                /* 1.0  */
    float step_size;               /* 0.01 */
    float step_size_write_samples; /* 1.5 (unused on this path) */
    uint8_t use_truncated_fourier; /* 0 (must be 0: MESE only) */
    uint8_t pad0[3];
    mraygb_single_scattering_params ss;
} mraygb_reconstruction_params;

/* Error measures of the per-pixel error bound (src/common.h:152-157). */
enum
{
    MRAYGB_ERROR_MAX = 0,
    MRAYGB_ERROR_RMSE = 1,
    MRAYGB_ERROR_PERCENTILE = 2
};

/* ErrorReconstructionParameters (src/parameters.h:124-137), same defaults. */
typedef struct mraygb_error_params
{
    int32_t error_type;       /* 2 = MRAYGB_ERROR_PERCENTILE */
    int32_t error_percentile; /* 90 */
    float bias;               /* 1e-6 */
    float data_min;           /* 0.0 */
    float data_max;           /* 1.0 */
    float step_size;          /* 0.01 */
    uint8_t compress;         /* 0 (file format; not on this path) */
    uint8_t entropy_coding;   /* 0 (file format; not on this path) */
    uint8_t quantization_bits; /* 32 (file format; not on this path) */
    uint8_t pad0[1];
} mraygb_error_params;

/* UncertaintyReconstructionParameters (src/parameters.h:319-325), same defaults. */
typedef struct mraygb_uncertainty_params
{
    mraygb_reconstruction_params rec;
    float bound_interpolation; /* 0.5 */
    int32_t error_type;        /* 1 = MRAYGB_ERROR_RMSE */
} mraygb_uncertainty_params;

/* ReferenceParameters (src/parameters.h:339-350), same defaults. */
typedef struct mraygb_reference_params
{
    float step_size;             /* 1.0 */
    float medium_emission;       /* 0.1 */
    float medium_scattering;     /* 0.1 */
    float early_ray_termination; /* 0.95 */
    float data_min;              /* 0.0 */
    float data_max;              /* 1.0 */
    mraygb_single_scattering_params ss;
} mraygb_reference_params;

/* MomentImageHost (src/moment_image.h:33-147) as plain arrays, for the file-format calls.  Writing reads the
 * arrays given (NULL = the image has none; index is required when is_compact); loading fills the scalar fields and
 * the has_* flags first, then the arrays the caller provides. */
typedef struct mraygb_moment_image
{
    int32_t width, height, num_moments;
    uint8_t is_compact, prediction_code;
    uint8_t has_bounds, has_error_bounds; /* loading: the file holds them */
    uint8_t has_coding_params;            /* loading: the file holds them */
    uint8_t pad0[3];
    int32_t coding_warp;
    float domain_min[3], domain_max[3];
    uint64_t data_size;      /* floats in data (compact: index[W*H]; else W*H*num_moments) */
    uint32_t *index;         /* W*H + 1 offsets when is_compact */
    float *data;             /* data_size floats */
    uint16_t *bounds;        /* 2*W*H (lower, upper) */
    uint16_t *error_bounds;  /* W*H */
    uint16_t *coding_params; /* 2*(num_moments - 1) (param1, param2) */
} mraygb_moment_image;

/* Coding warps (src/coding_params.h:35-42). */
enum
{
    MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED = 0,
    MRAYGB_CODING_WARP_NONE = 1
};

#ifdef __cplusplus
}
#endif

#endif /* MRAYGB_TYPES_H */
