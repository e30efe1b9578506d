"""ctypes mirrors of ``include/mraygb_types.h``.

The structures follow the reference's parameter and camera types field for field:

* :class:`Camera`                   -- ``cut::Camera`` (src/cut/camera.h:39-55)
* :class:`GenerationParameters`     -- ``GenerationParameters`` (src/parameters.h:49-70)
* :class:`ReconstructionParameters` -- ``ReconstructionParameters`` (src/parameters.h:231-247)

Defaults are the reference's defaults.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

CODING_WARP_DEFAULT_TRANSFORMED = 0
CODING_WARP_NONE = 1
# error measures of the per-pixel error bound (common.h:152-157)
MAX_ERROR = 0
RMSE = 1
ERROR_PERCENTILE = 2


class Camera(C.Structure):
    """``cut::Camera``: row-major ``transform`` (m[row][col]) plus the orthographic frame."""

    _fields_ = [
        ("transform", (C.c_float * 4) * 4),
        ("position", C.c_float * 3),
        ("right", C.c_float * 3),
        ("up", C.c_float * 3),
        ("dir", C.c_float * 3),
        ("scale", C.c_float),
        ("aspect", C.c_float),
        ("znear", C.c_float),
        ("orthographic", C.c_int32),
    ]

    @staticmethod
    def orthographic_camera(position, right, up, direction, znear=0.0):
        """An orthographic camera as ``cut::load_from_file`` fills it (camera.cpp:38-58)."""
        c = Camera()
        for i in range(4):
            for j in range(4):
                c.transform[i][j] = 1.0 if i == j else 0.0
        for i in range(3):
            c.position[i] = float(position[i])
            c.right[i] = float(right[i])
            c.up[i] = float(up[i])
            c.dir[i] = float(direction[i])
        c.scale = 1.0
        c.aspect = 1.0
        c.znear = float(znear)
        c.orthographic = 1
        return c

    @staticmethod
    def perspective_camera(transform, scale, aspect, znear=0.0):
        """A perspective camera as ``cut::load_from_file`` fills it (camera.cpp:59-72): camera->world
        ``transform`` (4x4, row-major), ``scale`` = tan(fov/2), position from the last column."""
        t = np.asarray(transform, dtype=np.float32).reshape(4, 4)
        c = Camera()
        for i in range(4):
            for j in range(4):
                c.transform[i][j] = float(t[i, j])
        for i in range(3):
            c.position[i] = float(t[i, 3])
            c.right[i] = 0.0
            c.up[i] = 0.0
            c.dir[i] = 0.0
        c.scale = float(scale)
        c.aspect = float(aspect)
        c.znear = float(znear)
        c.orthographic = 0
        return c


class GenerationParameters(C.Structure):
    """``GenerationParameters`` (parameters.h:49-70) with the reference's defaults."""

    _fields_ = [
        ("step_size", C.c_float),
        ("step_size_write_samples", C.c_float),
        ("data_min", C.c_float),
        ("data_max", C.c_float),
        ("error_threshold", C.c_float),
        ("bias", C.c_float),
        ("compact_image", C.c_uint8),
        ("prediction_coding", C.c_uint8),
        ("compress", C.c_uint8),
        ("entropy_coding", C.c_uint8),
        ("quantization_bits", C.c_uint8),
        ("pad0", C.c_uint8 * 3),
        ("coding_warp", C.c_int32),
        ("quantization_curve_sampling", C.c_int32),
        ("transform_to_bounds", C.c_uint8),
        ("pad1", C.c_uint8 * 3),
        ("transform_bound_eps", C.c_float),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.step_size = 1.0
        self.step_size_write_samples = 1.5
        self.data_min = 0.0
        self.data_max = 1.0
        self.error_threshold = 1.0
        self.bias = 1e-4
        self.compact_image = 1
        self.prediction_coding = 1
        self.compress = 0
        self.entropy_coding = 0
        self.quantization_bits = 32
        self.coding_warp = 0
        self.quantization_curve_sampling = 64
        self.transform_to_bounds = 0
        self.transform_bound_eps = 0.01
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class SingleScatteringParameters(C.Structure):
    """``SingleScatteringParameters`` (parameters.h:173-193) with the reference's defaults."""

    _fields_ = [
        ("enable", C.c_uint8),
        ("use_cache", C.c_uint8),
        ("pad0", C.c_uint8 * 2),
        ("cache_size_x", C.c_int32),
        ("cache_size_y", C.c_int32),
        ("cache_size_z", C.c_int32),
        ("step_size_factor", C.c_float),
        ("henyey_greenstein_g", C.c_float),
        ("direction_x", C.c_float),
        ("direction_y", C.c_float),
        ("direction_z", C.c_float),
        ("intensity_r", C.c_float),
        ("intensity_g", C.c_float),
        ("intensity_b", C.c_float),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.enable = 0
        self.use_cache = 1
        self.cache_size_x = self.cache_size_y = self.cache_size_z = 128
        self.step_size_factor = 1.0
        self.henyey_greenstein_g = 0.0
        self.direction_x, self.direction_y, self.direction_z = 0.0, -1.0, 0.1
        self.intensity_r = self.intensity_g = self.intensity_b = 1.0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class ReconstructionParameters(C.Structure):
    """``ReconstructionParameters`` (parameters.h:231-247) with the reference's defaults and layout; the
    truncated-Fourier variant is not part of this path and must stay 0.  Single scattering (``ss.enable``) samples
    the transmittance cache of the context (``reconstruct_single_scattering_cache``)."""

    _fields_ = [
        ("bias", C.c_float),
        ("medium_emission", C.c_float),
        ("medium_scattering", C.c_float),
        ("early_ray_termination", C.c_float),
        ("data_min", C.c_float),
        ("data_max", C.c_float),
        ("step_size", C.c_float),
        ("step_size_write_samples", C.c_float),
        ("use_truncated_fourier", C.c_uint8),
        ("pad0", C.c_uint8 * 3),
        ("ss", SingleScatteringParameters),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.bias = 1e-6
        self.medium_emission = 0.1
        self.medium_scattering = 0.1
        self.early_ray_termination = 0.95
        self.data_min = 0.0
        self.data_max = 1.0
        self.step_size = 0.01
        self.step_size_write_samples = 1.5
        self.use_truncated_fourier = 0
        self.ss = SingleScatteringParameters()
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class ErrorReconstructionParameters(C.Structure):
    """``ErrorReconstructionParameters`` (parameters.h:124-137) with the reference's defaults; the file-format
    fields (compress, entropy_coding, quantization_bits) are carried but not used on this path."""

    _fields_ = [
        ("error_type", C.c_int32),
        ("error_percentile", C.c_int32),
        ("bias", C.c_float),
        ("data_min", C.c_float),
        ("data_max", C.c_float),
        ("step_size", C.c_float),
        ("compress", C.c_uint8),
        ("entropy_coding", C.c_uint8),
        ("quantization_bits", C.c_uint8),
        ("pad0", C.c_uint8 * 1),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.error_type = ERROR_PERCENTILE
        self.error_percentile = 90
        self.bias = 1e-6
        self.data_min = 0.0
        self.data_max = 1.0
        self.step_size = 0.01
        self.compress = 0
        self.entropy_coding = 0
        self.quantization_bits = 32
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class UncertaintyReconstructionParameters(C.Structure):
    """``UncertaintyReconstructionParameters`` (parameters.h:319-325) with the reference's defaults."""

    _fields_ = [
        ("rec", ReconstructionParameters),
        ("bound_interpolation", C.c_float),
        ("error_type", C.c_int32),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.rec = ReconstructionParameters()
        self.bound_interpolation = 0.5
        self.error_type = RMSE
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class ReferenceParameters(C.Structure):
    """``ReferenceParameters`` (parameters.h:339-350) with the reference's defaults."""

    _fields_ = [
        ("step_size", C.c_float),
        ("medium_emission", C.c_float),
        ("medium_scattering", C.c_float),
        ("early_ray_termination", C.c_float),
        ("data_min", C.c_float),
        ("data_max", C.c_float),
        ("ss", SingleScatteringParameters),
    ]

    def __init__(self, **kw):
        super().__init__()
        self.step_size = 1.0
        self.medium_emission = 0.1
        self.medium_scattering = 0.1
        self.early_ray_termination = 0.95
        self.data_min = 0.0
        self.data_max = 1.0
        self.ss = SingleScatteringParameters()
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class MomentImageArrays(C.Structure):
    """``mraygb_moment_image``: a MomentImageHost (moment_image.h:33-147) as plain arrays for the file-format calls."""

    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("num_moments", C.c_int32),
        ("is_compact", C.c_uint8),
        ("prediction_code", C.c_uint8),
        ("has_bounds", C.c_uint8),
        ("has_error_bounds", C.c_uint8),
        ("has_coding_params", C.c_uint8),
        ("pad0", C.c_uint8 * 3),
        ("coding_warp", C.c_int32),
        ("domain_min", C.c_float * 3),
        ("domain_max", C.c_float * 3),
        ("data_size", C.c_uint64),
        ("index", C.c_void_p),
        ("data", C.c_void_p),
        ("bounds", C.c_void_p),
        ("error_bounds", C.c_void_p),
        ("coding_params", C.c_void_p),
    ]
