"""Loads ``libmraygb.so`` (the CUDA library behind ``include/mraygb.h``) and declares its C ABI for ctypes.

There is no fallback: if the library cannot be built or loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from .types import (Camera, ErrorReconstructionParameters, GenerationParameters, MomentImageArrays,
                    ReconstructionParameters, ReferenceParameters, UncertaintyReconstructionParameters)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmraygb.so")

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "CUDA_ERROR", 4: "DEVICE_TIMEOUT", 5: "NUMERICAL",
          6: "NOT_SUPPORTED", 7: "NO_VOLUME"}

# every symbol include/mraygb.h declares
EXPORTS = [
    "mraygb_create", "mraygb_destroy", "mraygb_last_error", "mraygb_set_stream", "mraygb_get_stream",
    "mraygb_synchronize", "mraygb_set_precision", "mraygb_kernel_launches", "mraygb_upload_grid", "mraygb_upload_particles", "mraygb_upload_particles_h",
    "mraygb_upload_tf",
    "mraygb_generate", "mraygb_reconstruct", "mraygb_stage_generate_moments", "mraygb_stage_compact",
    "mraygb_stage_prepare_moments", "mraygb_stage_reconstruct", "mraygb_quantize_prediction_coding",
    "mraygb_stage_prediction_encode", "mraygb_stage_quantize_prediction_coding",
    "mraygb_stage_dequantize_prediction_coding", "mraygb_stage_compact_noalloc", "mraygb_diff_forward",
    "mraygb_diff_backward", "mraygb_create_quantization_table", "mraygb_stage_create_quantization_table",
    "mraygb_reconstruct_error", "mraygb_stage_reconstruct_error", "mraygb_upload_uncertainty_tf",
    "mraygb_reconstruct_uncertainty", "mraygb_stage_reconstruct_uncertainty", "mraygb_upload_uncertainty_table",
    "mraygb_generate_reference", "mraygb_stage_generate_reference", "mraygb_reconstruct_single_scattering_cache",
    "mraygb_stage_reconstruct_single_scattering_cache", "mraygb_upload_single_scattering_cache",
    "mraygb_generate_reference_reconstructed_ss", "mraygb_stage_generate_reference_reconstructed_ss",
    "mraygb_encode_moment_image", "mraygb_copy_encoded", "mraygb_decode_moment_image", "mraygb_write_moment_image",
    "mraygb_load_moment_image", "mraygb_lz4_compress", "mraygb_lz4_decompress", "mraygb_entropy_encode",
    "mraygb_entropy_decode", "mraygb_stage_libm_sincosf", "mraygb_dequantize_prediction_coding",
    "mraygb_measure_fp32_rate", "mraygb_set_diff_tf_sampling",
]

_lock = threading.Lock()
_lib = None


class MrayError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def _declare(L):
    P = C.POINTER
    vp = C.c_void_p
    i = C.c_int
    L.mraygb_create.argtypes = [i, P(vp)]
    L.mraygb_destroy.argtypes = [vp]
    L.mraygb_destroy.restype = None
    L.mraygb_last_error.argtypes = [vp]
    L.mraygb_last_error.restype = C.c_char_p
    L.mraygb_set_stream.argtypes = [vp, vp]
    L.mraygb_get_stream.argtypes = [vp]
    L.mraygb_get_stream.restype = vp
    L.mraygb_synchronize.argtypes = [vp]
    L.mraygb_set_precision.argtypes = [vp, i]
    L.mraygb_set_diff_tf_sampling.argtypes = [vp, i]
    L.mraygb_kernel_launches.argtypes = [vp]
    L.mraygb_kernel_launches.restype = C.c_uint64
    L.mraygb_upload_grid.argtypes = [vp, vp, i, i, i, C.c_float * 3, C.c_float * 3, i]
    L.mraygb_upload_particles.argtypes = [vp, vp, vp, vp, vp, C.c_uint64, C.c_float, C.c_float * 3, C.c_float * 3, i]
    L.mraygb_upload_particles_h.argtypes = [vp, vp, vp, vp, vp, vp, C.c_uint64, C.c_float * 3, C.c_float * 3, i]
    L.mraygb_upload_tf.argtypes = [vp, vp]
    L.mraygb_generate.argtypes = [vp, P(Camera), P(GenerationParameters), i, i, i, vp, vp, vp, vp,
                                  P(C.c_uint64)]
    L.mraygb_reconstruct.argtypes = [vp, P(Camera), P(ReconstructionParameters), i, i, i, C.c_float * 3,
                                     C.c_float * 3, vp, vp, C.c_uint64, vp, i, i, vp, vp, vp]
    L.mraygb_stage_generate_moments.argtypes = [vp, P(Camera), P(GenerationParameters), i, i, i, vp, vp, vp]
    L.mraygb_stage_compact.argtypes = [vp, i, i, i, vp, vp, vp, vp, C.c_uint64, P(C.c_uint64)]
    L.mraygb_stage_prepare_moments.argtypes = [vp, i, i, i, vp, vp, i, i, vp, C.c_float, vp]
    L.mraygb_stage_reconstruct.argtypes = [vp, P(Camera), P(ReconstructionParameters), i, i, i, C.c_float * 3,
                                           C.c_float * 3, vp, vp, vp, vp, vp]
    u64 = C.c_uint64
    L.mraygb_quantize_prediction_coding.argtypes = [vp, i, i, i, vp, vp, u64, vp, vp, u64, P(u64)]
    L.mraygb_dequantize_prediction_coding.argtypes = [vp, i, i, i, vp, vp, vp, u64, vp, u64]
    L.mraygb_measure_fp32_rate.argtypes = [vp, P(C.c_double)]
    L.mraygb_stage_libm_sincosf.argtypes = [vp, vp, vp, vp, u64]
    L.mraygb_stage_prediction_encode.argtypes = [vp, i, i, i, vp, vp, u64, i, C.c_float, vp]
    L.mraygb_stage_quantize_prediction_coding.argtypes = [vp, i, i, i, vp, vp, vp, vp, u64, P(u64)]
    L.mraygb_stage_dequantize_prediction_coding.argtypes = [vp, i, i, i, vp, vp, vp, u64, vp]
    L.mraygb_stage_compact_noalloc.argtypes = [vp, i, i, i, vp, vp, vp, vp, u64, P(u64)]
    G, RP = P(GenerationParameters), P(ReconstructionParameters)
    L.mraygb_diff_forward.argtypes = [vp, P(Camera), G, RP, i, i, i, vp, vp, vp, vp, vp]
    L.mraygb_diff_backward.argtypes = [vp, P(Camera), G, RP, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
    L.mraygb_create_quantization_table.argtypes = [vp, i, i, i, vp, vp, u64, i, vp, i, i, vp, vp]
    L.mraygb_stage_create_quantization_table.argtypes = [vp, i, i, i, vp, vp, i, vp, i, i, vp, vp]
    EP, UP = P(ErrorReconstructionParameters), P(UncertaintyReconstructionParameters)
    f3 = C.c_float * 3
    L.mraygb_reconstruct_error.argtypes = [vp, P(Camera), EP, i, i, i, vp, vp, u64, vp, i, i, vp, vp, vp]
    L.mraygb_stage_reconstruct_error.argtypes = [vp, P(Camera), EP, i, i, i, vp, vp, vp, vp, vp]
    L.mraygb_upload_uncertainty_tf.argtypes = [vp, vp, C.c_float, i, vp]
    L.mraygb_upload_uncertainty_table.argtypes = [vp, vp]
    L.mraygb_generate_reference.argtypes = [vp, P(Camera), P(ReferenceParameters), i, i, vp, vp]
    L.mraygb_stage_generate_reference.argtypes = [vp, P(Camera), P(ReferenceParameters), i, i, vp]
    L.mraygb_reconstruct_single_scattering_cache.argtypes = [vp, P(Camera), RP, i, i, i, f3, f3, vp, vp, u64, vp, i,
                                                             i, vp, vp]
    L.mraygb_stage_reconstruct_single_scattering_cache.argtypes = [vp, P(Camera), RP, i, i, i, f3, f3, vp, vp, vp, vp]
    L.mraygb_upload_single_scattering_cache.argtypes = [vp, vp, i, i, i, f3, f3, i]
    L.mraygb_generate_reference_reconstructed_ss.argtypes = [vp, P(Camera), RP, i, i, vp, vp]
    L.mraygb_stage_generate_reference_reconstructed_ss.argtypes = [vp, P(Camera), RP, i, i, vp]
    L.mraygb_reconstruct_uncertainty.argtypes = [vp, P(Camera), UP, i, i, i, i, f3, f3, vp, vp, u64, vp, vp, i, i, vp,
                                                 vp, vp]
    MI = P(MomentImageArrays)
    L.mraygb_encode_moment_image.argtypes = [vp, MI, i, i, i, vp, P(u64)]
    L.mraygb_copy_encoded.argtypes = [vp, vp, u64]
    L.mraygb_decode_moment_image.argtypes = [vp, vp, u64, MI, vp, P(i)]
    L.mraygb_write_moment_image.argtypes = [vp, C.c_char_p, MI, i, i, i, vp]
    L.mraygb_load_moment_image.argtypes = [vp, C.c_char_p, MI, vp, P(i)]
    L.mraygb_lz4_compress.argtypes = [vp, u64, vp, u64]
    L.mraygb_lz4_decompress.argtypes = [vp, u64, vp, u64]
    L.mraygb_entropy_encode.argtypes = [i, i, i, vp, vp, vp, i, vp, u64, P(u64)]
    L.mraygb_entropy_decode.argtypes = [vp, u64, i, i, i, vp, vp, i, vp]
    L.mraygb_stage_reconstruct_uncertainty.argtypes = [vp, P(Camera), UP, i, i, i, i, f3, f3, vp, vp, vp, vp, vp]
    special = ("mraygb_destroy", "mraygb_last_error", "mraygb_get_stream", "mraygb_kernel_launches",
               "mraygb_lz4_compress", "mraygb_lz4_decompress")
    for name in EXPORTS:
        if name not in special:
            getattr(L, name).restype = C.c_int
    L.mraygb_lz4_compress.restype = u64
    L.mraygb_lz4_decompress.restype = C.c_int64


def load(build_if_missing: bool = True):
    """The loaded library; builds it in-tree first when it is missing (nvcc required)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise OSError(f"{LIB_PATH} is missing; run mray_gb300.build.build()")
                from . import build as _build
                _build.build()
            _lib = C.CDLL(LIB_PATH)
            _declare(_lib)
        return _lib


def check(ctx_handle, status: int) -> None:
    if status != 0:
        msg = load().mraygb_last_error(ctx_handle)
        raise MrayError(status, msg.decode() if msg else "")
