"""mray_gb300: the moment-image hot path of TobiasRp/mray (moment generation, compaction, prediction coding and
quantization, bounded-MESE reconstruction) as hand-written sm_103a CUDA behind a C ABI (include/mraygb.h).

The Python layer mirrors the reference's raymarcher API (generate / reconstruct and the moment-image, colour-image,
grid and transfer-function containers) and calls the C ABI through ctypes.
"""
from .types import (CODING_WARP_DEFAULT_TRANSFORMED, CODING_WARP_NONE, ERROR_PERCENTILE, MAX_ERROR, RMSE, Camera,
                    ErrorReconstructionParameters, GenerationParameters, ReconstructionParameters,
                    ReferenceParameters, SingleScatteringParameters, UncertaintyReconstructionParameters)
from .raymarcher import (DIFF_TF_BSPLINE, DIFF_TF_LINEAR, MAX_MOMENTS, PRECISION_COMPENSATED_FF_MESE, PRECISION_COMPENSATED_FP64_MESE, PRECISION_FP32, ColorImageHost, Context,
                         MomentImageHost, Particles, RegularGrid, TransferFunction, default_context, default_quantization_table,
                         generate, preintegrate, quantize_prediction_coding, dequantize_prediction_coding,
                         reconstruct,
                         create_quantization_table, UncertaintyTransferFunction, read_from_disk_uncertainty,
                         reconstruct_error, reconstruct_uncertainty_interpolation, reconstruct_uncertainty_convolution,
                         generate_reference, SingleScatteringImageHost, SingleScatteringCacheHost,
                         reconstruct_single_scattering_cache, generate_reference_reconstructed_ss,
                         write_moment_image, load_moment_image, lz4_compress, lz4_decompress, entropy_encode,
                         entropy_decode)
from ._lib import MrayError

__all__ = [
    "Camera", "GenerationParameters", "ReconstructionParameters", "CODING_WARP_DEFAULT_TRANSFORMED",
    "CODING_WARP_NONE", "ColorImageHost", "Context", "MomentImageHost", "Particles", "RegularGrid", "TransferFunction",
    "default_context", "default_quantization_table", "create_quantization_table", "quantize_prediction_coding", "dequantize_prediction_coding", "generate", "preintegrate", "reconstruct", "MrayError", "PRECISION_FP32",
    "PRECISION_COMPENSATED_FP64_MESE", "PRECISION_COMPENSATED_FF_MESE", "MAX_MOMENTS", "DIFF_TF_BSPLINE",
    "DIFF_TF_LINEAR",
    "ErrorReconstructionParameters", "UncertaintyReconstructionParameters", "MAX_ERROR", "RMSE", "ERROR_PERCENTILE",
    "UncertaintyTransferFunction", "read_from_disk_uncertainty", "reconstruct_error",
    "reconstruct_uncertainty_interpolation", "reconstruct_uncertainty_convolution", "generate_reference",
    "ReferenceParameters", "SingleScatteringParameters", "SingleScatteringImageHost", "SingleScatteringCacheHost",
    "reconstruct_single_scattering_cache", "generate_reference_reconstructed_ss", "write_moment_image",
    "load_moment_image", "lz4_compress", "lz4_decompress", "entropy_encode", "entropy_decode",
]
