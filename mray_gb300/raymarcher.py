"""Host-side mirror of the reference's moment raymarcher interface, running on the CUDA library.

The names, argument meaning and error behaviour follow the reference (TobiasRp/mray):

* :class:`MomentImageHost`   -- src/moment_image.h:33-147 (index / bounds / coding params / data)
* :class:`ColorImageHost`    -- src/color_image.h:30-71 (u8 RGBA, plus the float colour before the u8 store)
* :class:`RegularGrid`       -- src/volume.h:31-123
* :class:`TransferFunction`  -- src/transfer_function.h:30-60, built by :func:`preintegrate`
  (src/transfer_function.cpp:46-97)
* :func:`generate`           -- generate(cam, volume, mi, params), src/moment_raymarcher.h:48-49
* :func:`reconstruct`        -- reconstruct(cam, mi, tf, img, params), src/moment_raymarcher.h:61-64

All compute runs in ``libmraygb.so``; there is no CPU path.  :class:`Context` exposes the C ABI's stage calls on
device pointers (ints or CUDA tensors).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from .types import (Camera, ErrorReconstructionParameters, GenerationParameters, MomentImageArrays,
                    ReconstructionParameters,
                    ReferenceParameters, UncertaintyReconstructionParameters)

PRECISION_FP32 = 0
PRECISION_COMPENSATED_FP64_MESE = 1
PRECISION_COMPENSATED_FF_MESE = 2
MAX_MOMENTS = 255
# the differentiation form's transfer-function row (mraygb_set_diff_tf_sampling)
DIFF_TF_BSPLINE = 0
DIFF_TF_LINEAR = 1


def _dptr(x) -> Optional[int]:
    """A device address from None, an int or a CUDA tensor."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x.data_ptr()
    raise TypeError(f"cannot take a device pointer of {type(x)}")


def _hptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class RegularGrid:
    """RegularGrid: float32 data indexed [z, y, x] on the box [domain_min, domain_max]."""

    def __init__(self, data: np.ndarray, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0)):
        self.data = data
        self.domain_min = tuple(float(v) for v in domain_min)
        self.domain_max = tuple(float(v) for v in domain_max)

    @property
    def size(self):
        nz, ny, nx = self.data.shape
        return (nx, ny, nz)


class Particles:
    """Particles (volume.h:125-157): SPH particles x, y, z with scalar values, one smoothing length, marched inside
    the box [domain_min, domain_max]."""

    def __init__(self, domain_min, domain_max, x, y, z, values, smoothing_length: float):
        self.domain_min = tuple(float(v) for v in domain_min)
        self.domain_max = tuple(float(v) for v in domain_max)
        self.x, self.y, self.z, self.values = x, y, z, values
        self.smoothing_length = float(smoothing_length)

    def size(self) -> int:
        return len(self.x)

    def get_step_size(self) -> float:
        """Particles::get_step_size: half the smoothing length."""
        return float(np.float32(self.smoothing_length) * np.float32(0.5))


class TransferFunction:
    """TransferFunction: ``table`` is one row (256 x RGBA float) of the 256 x 256 table, all rows being equal."""

    RESOLUTION = 256

    def __init__(self, table: np.ndarray):
        t = np.ascontiguousarray(table, dtype=np.float32)
        if t.shape != (256, 4):
            raise ValueError("transfer function table must be 256 x 4")
        self.table = t


class UncertaintyTransferFunction:
    """read_from_disk_uncertainty's table (transfer_function.cpp:233-248): the 1D table (read_tf's output, 256 x RGBA
    float), the step size and the error type that selects the box or the Gaussian filter.  The 256 x 256 table is
    built on the device (``Context.upload_uncertainty_tf``)."""

    def __init__(self, tf1d: np.ndarray, step_size: float, error_type: int):
        t = np.ascontiguousarray(tf1d, dtype=np.float32)
        if t.shape != (256, 4):
            raise ValueError("transfer function table must be 256 x 4")
        self.tf1d, self.step_size, self.error_type = t, float(step_size), int(error_type)


def read_from_disk_uncertainty(tf1d: np.ndarray, step_size: float, error_type: int) -> UncertaintyTransferFunction:
    """read_from_disk_uncertainty(filepath, step_size, error_type) on the table the file holds."""
    return UncertaintyTransferFunction(tf1d, step_size, error_type)


def preintegrate(tf1d: np.ndarray, step_size: float) -> TransferFunction:
    """preintegrate (transfer_function.cpp:46-97): entry x = (rgb_x * a_x s, a_x s), s = step_size (float
    arithmetic, as the reference's)."""
    t = np.ascontiguousarray(tf1d, dtype=np.float32)
    w = t[:, 3] * np.float32(step_size)
    out = np.empty_like(t)
    out[:, 0] = t[:, 0] * w
    out[:, 1] = t[:, 1] * w
    out[:, 2] = t[:, 2] * w
    out[:, 3] = w
    return TransferFunction(out)


class MomentImageHost:
    """MomentImageHost (moment_image.h:33-147)."""

    def __init__(self, width: int, height: int, num_moments: int, create_index: bool = True,
                 create_bounds: bool = False):
        self.width = int(width)
        self.height = int(height)
        self.num_moments = int(num_moments)
        self.is_compact = False
        self.prediction_code = False
        self.coding_warp = 0
        self.domain_min = (0.0, 0.0, 0.0)
        self.domain_max = (1.0, 1.0, 1.0)
        self.index = np.zeros(self.width * self.height + 1, dtype=np.uint32) if create_index else None
        self.bounds = np.zeros((self.width * self.height, 2), dtype=np.uint16) if create_bounds else None
        self.coding_params: Optional[np.ndarray] = None
        self.error_bounds: Optional[np.ndarray] = None
        self.data = np.zeros(self.width * self.height * self.num_moments, dtype=np.float32)

    def add_error_bounds(self) -> None:
        """add_error_bounds (moment_image.h:100): one u16 error bound per pixel."""
        self.error_bounds = np.zeros(self.width * self.height, dtype=np.uint16)

    def has_error_bounds(self) -> bool:
        return self.error_bounds is not None

    def get_error_bound(self, x: int, y: int) -> float:
        return float(np.float32(self.error_bounds[y * self.width + x]) / np.float32(65535.0))

    def has_bounds(self) -> bool:
        return self.bounds is not None

    def get_idx(self, x: int, y: int) -> int:
        if self.is_compact:
            return int(self.index[y * self.width + x])
        return (y * self.width + x) * self.num_moments

    def get_num_moments(self, x: int, y: int) -> int:
        if self.is_compact:
            p = y * self.width + x
            return int(self.index[p + 1] - self.index[p])
        return self.num_moments

    def get_bounds(self, x: int, y: int):
        if self.bounds is None:
            return (0.0, 1.0)
        b = self.bounds[y * self.width + x]
        return (np.float32(b[0]) / np.float32(65535.0), np.float32(b[1]) / np.float32(65535.0))


class SingleScatteringImageHost:
    """SingleScatteringImageHost (single_scattering_image.h:50-106): the light's camera and the moment image
    rendered from it (generate with that camera)."""

    def __init__(self, cam: Camera, img: "MomentImageHost"):
        self.cam = cam
        self.img = img


class SingleScatteringCacheHost:
    """SingleScatteringCacheHost (single_scattering_cache.h:33-59): the transmittance towards the light as a
    RegularGrid (float32 [z, y, x] over the light image's domain)."""

    def __init__(self, cache: RegularGrid):
        self.cache = cache


class ColorImageHost:
    """ColorImageHost: u8 RGBA as the reference stores it, plus ``rgba_float`` (the colour before the store)."""

    def __init__(self, width: int, height: int):
        self.width = int(width)
        self.height = int(height)
        self.rgba = np.zeros((self.height, self.width, 4), dtype=np.uint8)
        self.rgba_float = np.zeros((self.height, self.width, 4), dtype=np.float32)


class Context:
    """One mraygb_context: a device, a stream, the resident volume and transfer function."""

    def __init__(self, device: int = 0, precision: int = PRECISION_FP32):
        self._L = _lib.load()
        h = C.c_void_p()
        st = self._L.mraygb_create(int(device), C.byref(h))
        if st != 0:
            raise _lib.MrayError(st, f"cannot create a context on device {device}")
        self._h = h
        self.device = device
        self._grid_key = None
        self._tf_key = None
        self.precision = precision

    # ---- lifetime ----
    def close(self):
        if getattr(self, "_h", None):
            self._L.mraygb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        _lib.check(self._h, st)

    # ---- settings ----
    @property
    def precision(self) -> int:
        return self._precision

    @precision.setter
    def precision(self, value: int):
        self._check(self._L.mraygb_set_precision(self._h, int(value)))
        self._precision = int(value)

    @property
    def diff_tf_sampling(self) -> int:
        """The differentiation form's transfer-function row: DIFF_TF_BSPLINE (default) or DIFF_TF_LINEAR."""
        return getattr(self, "_diff_tf_sampling", DIFF_TF_BSPLINE)

    @diff_tf_sampling.setter
    def diff_tf_sampling(self, value: int):
        self._check(self._L.mraygb_set_diff_tf_sampling(self._h, int(value)))
        self._diff_tf_sampling = int(value)

    def set_stream(self, stream) -> None:
        """Orders later work on ``stream``: a torch.cuda.Stream (torch's default stream included), a cudaStream_t as
        an int, or None for the context's own stream."""
        if stream is not None and hasattr(stream, "cuda_stream"):
            # torch's default stream has the handle 0, which the C ABI reads as "the context's own stream": pass
            # cudaStreamLegacy (1) for it instead
            stream = stream.cuda_stream or 1
        self._check(self._L.mraygb_set_stream(self._h, stream))

    def synchronize(self) -> None:
        self._check(self._L.mraygb_synchronize(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(self._L.mraygb_kernel_launches(self._h))

    # ---- resident inputs ----
    def upload_grid(self, volume, domain_min, domain_max) -> None:
        """Uploads a [z, y, x] float32 volume (numpy array or CUDA tensor)."""
        if hasattr(volume, "data_ptr"):
            nz, ny, nx = volume.shape
            self._check(self._L.mraygb_upload_grid(self._h, _dptr(volume), nx, ny, nz, _f3(domain_min),
                                                   _f3(domain_max), 1))
        else:
            v = np.ascontiguousarray(volume, dtype=np.float32)
            nz, ny, nx = v.shape
            self._check(self._L.mraygb_upload_grid(self._h, _hptr(v), nx, ny, nz, _f3(domain_min), _f3(domain_max),
                                                   0))
        self._grid_key = None

    def upload_particles(self, x, y, z, v, smoothing_length: float, domain_min, domain_max) -> None:
        """Uploads SPH particles (four float32 arrays: numpy arrays or CUDA tensors) and builds their cell grid on
        the device; they replace an uploaded grid."""
        if hasattr(x, "data_ptr"):
            n = x.numel()
            ptrs = [_dptr(a) for a in (x, y, z, v)]
            on_device = 1
        else:
            arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, v)]
            n = arrs[0].size
            ptrs = [_hptr(a) for a in arrs]
            on_device = 0
        self._check(self._L.mraygb_upload_particles(self._h, *ptrs, n, float(smoothing_length), _f3(domain_min),
                                                    _f3(domain_max), on_device))

    def upload_particles_h(self, x, y, z, v, h, domain_min, domain_max) -> None:
        """SPH particles with a smoothing length per particle (five float32 arrays: numpy arrays or CUDA tensors)
        and the Wendland C2 kernel (mraygb_upload_particles_h); they replace an uploaded volume."""
        if hasattr(x, "data_ptr"):
            n = x.numel()
            ptrs = [_dptr(a) for a in (x, y, z, v, h)]
            on_device = 1
        else:
            arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, v, h)]
            n = arrs[0].size
            ptrs = [_hptr(a) for a in arrs]
            on_device = 0
        self._check(self._L.mraygb_upload_particles_h(self._h, *ptrs, n, _f3(domain_min), _f3(domain_max),
                                                      on_device))

    def upload_tf(self, table) -> None:
        t = np.ascontiguousarray(table, dtype=np.float32)
        if t.shape != (256, 4):
            raise ValueError("transfer function table must be 256 x 4")
        self._check(self._L.mraygb_upload_tf(self._h, _hptr(t)))
        self._tf_key = None

    # ---- drop-in host calls ----
    def generate(self, cam: Camera, gp: GenerationParameters, width: int, height: int, num_moments: int,
                 out: Optional[MomentImageHost] = None) -> MomentImageHost:
        mi = out or MomentImageHost(width, height, num_moments, bool(gp.compact_image),
                                    bool(gp.transform_to_bounds))
        cap = width * height * num_moments
        if mi.data.size < cap:
            mi.data = np.zeros(cap, dtype=np.float32)
        if gp.compact_image and mi.index is None:
            mi.index = np.zeros(width * height + 1, dtype=np.uint32)
        if gp.transform_to_bounds and mi.bounds is None:
            mi.bounds = np.zeros((width * height, 2), dtype=np.uint16)
        cp = np.zeros(max(2 * (num_moments - 1), 1), dtype=np.uint16)
        size = C.c_uint64()
        self._check(self._L.mraygb_generate(self._h, C.byref(cam), C.byref(gp), width, height, num_moments,
                                            _hptr(mi.data), _hptr(mi.index) if gp.compact_image else None,
                                            _hptr(mi.bounds) if gp.transform_to_bounds else None, _hptr(cp),
                                            C.byref(size)))
        mi.data = mi.data[:size.value]
        mi.is_compact = bool(gp.compact_image)
        mi.prediction_code = bool(gp.prediction_coding)
        mi.coding_warp = int(gp.coding_warp)
        mi.coding_params = cp[:2 * (num_moments - 1)] if (gp.prediction_coding and gp.coding_warp == 0) else None
        return mi

    def reconstruct(self, cam: Camera, rp: ReconstructionParameters, mi: MomentImageHost,
                    img: Optional[ColorImageHost] = None) -> ColorImageHost:
        img = img or ColorImageHost(mi.width, mi.height)
        data = np.ascontiguousarray(mi.data, dtype=np.float32)
        index = np.ascontiguousarray(mi.index, dtype=np.uint32) if mi.is_compact else None
        bounds = np.ascontiguousarray(mi.bounds, dtype=np.uint16) if mi.bounds is not None else None
        cp = np.ascontiguousarray(mi.coding_params, dtype=np.uint16) if mi.coding_params is not None else None
        self._check(self._L.mraygb_reconstruct(self._h, C.byref(cam), C.byref(rp), mi.width, mi.height,
                                               mi.num_moments, _f3(mi.domain_min), _f3(mi.domain_max), _hptr(index),
                                               _hptr(data), data.size, _hptr(bounds), int(mi.prediction_code),
                                               int(mi.coding_warp), _hptr(cp), _hptr(img.rgba_float),
                                               _hptr(img.rgba)))
        return img

    def _image_arrays(self, mi: MomentImageHost):
        data = np.ascontiguousarray(mi.data, dtype=np.float32)
        index = np.ascontiguousarray(mi.index, dtype=np.uint32) if mi.is_compact else None
        bounds = np.ascontiguousarray(mi.bounds, dtype=np.uint16) if mi.bounds is not None else None
        cp = np.ascontiguousarray(mi.coding_params, dtype=np.uint16) if mi.coding_params is not None else None
        return data, index, bounds, cp

    def reconstruct_error(self, cam: Camera, ep: ErrorReconstructionParameters, mi: MomentImageHost,
                          return_errors: bool = False):
        """reconstruct_error(cam, volume, mi, params) over the volume uploaded last (moment_raymarcher.cpp:541-560):
        fills mi.error_bounds (u16 per pixel) and, with ``return_errors``, returns the float errors [H, W]."""
        if mi.error_bounds is None:
            mi.add_error_bounds()
        data, index, bounds, cp = self._image_arrays(mi)
        eb = np.zeros(mi.width * mi.height, dtype=np.uint16)
        errors = np.zeros((mi.height, mi.width), dtype=np.float32) if return_errors else None
        self._check(self._L.mraygb_reconstruct_error(self._h, C.byref(cam), C.byref(ep), mi.width, mi.height,
                                                     mi.num_moments, _hptr(index), _hptr(data), data.size,
                                                     _hptr(bounds), int(mi.prediction_code), int(mi.coding_warp),
                                                     _hptr(cp), _hptr(eb), _hptr(errors)))
        mi.error_bounds = eb
        return errors

    def upload_uncertainty_tf(self, utf: UncertaintyTransferFunction, return_table: bool = False):
        """The uncertainty table of ``utf`` built on the device and kept resident; with ``return_table`` also
        returned as [256 (y), 256 (x), 4]."""
        table = np.zeros((256, 256, 4), dtype=np.float32) if return_table else None
        self._check(self._L.mraygb_upload_uncertainty_tf(self._h, _hptr(utf.tf1d), utf.step_size, utf.error_type,
                                                         _hptr(table)))
        return table

    def upload_uncertainty_table(self, table) -> None:
        """A whole 256 x 256 RGBA uncertainty table ([y][x]) as the convolution renderer's table."""
        t = np.ascontiguousarray(table, dtype=np.float32)
        if t.shape != (256, 256, 4):
            raise ValueError("uncertainty table must be 256 x 256 x 4")
        self._check(self._L.mraygb_upload_uncertainty_table(self._h, _hptr(t)))

    def reconstruct_uncertainty(self, cam: Camera, up: UncertaintyReconstructionParameters, mode: int,
                                mi: MomentImageHost, img: Optional[ColorImageHost] = None) -> ColorImageHost:
        """mode 0: reconstruct_uncertainty_interpolation with the transfer function of ``upload_tf``; mode 1:
        reconstruct_uncertainty_convolution with the table of ``upload_uncertainty_tf``
        (moment_raymarcher.cpp:562-717)."""
        if mi.error_bounds is None:
            raise ValueError("the moment image has no error bounds (reconstruct_error first)")
        img = img or ColorImageHost(mi.width, mi.height)
        data, index, bounds, cp = self._image_arrays(mi)
        eb = np.ascontiguousarray(mi.error_bounds, dtype=np.uint16)
        self._check(self._L.mraygb_reconstruct_uncertainty(self._h, C.byref(cam), C.byref(up), int(mode), mi.width,
                                                           mi.height, mi.num_moments, _f3(mi.domain_min),
                                                           _f3(mi.domain_max), _hptr(index), _hptr(data), data.size,
                                                           _hptr(bounds), _hptr(eb), int(mi.prediction_code),
                                                           int(mi.coding_warp), _hptr(cp), _hptr(img.rgba_float),
                                                           _hptr(img.rgba)))
        return img

    def generate_reference(self, cam: Camera, rp: ReferenceParameters, width: int, height: int,
                           img: Optional[ColorImageHost] = None) -> ColorImageHost:
        """generate_reference (moment_raymarcher.cpp:64-80) over the volume and transfer function uploaded last."""
        img = img or ColorImageHost(width, height)
        self._check(self._L.mraygb_generate_reference(self._h, C.byref(cam), C.byref(rp), width, height,
                                                      _hptr(img.rgba_float), _hptr(img.rgba)))
        return img

    def stage_generate_reference(self, cam, rp, width, height, rgba):
        self._check(self._L.mraygb_stage_generate_reference(self._h, C.byref(cam), C.byref(rp), width, height,
                                                            _dptr(rgba)))

    # ---- the moment-image file format ----
    def encode_moment_image(self, mi: MomentImageHost, compress: bool, quantization_bits: int,
                            entropy_coding: bool = False, table=None) -> bytes:
        """The bytes write_moment_image(mi, filename, compress, quantizationBits, entropy_coding) writes
        (moment_image_io.cpp:510-529); ``table`` stands for the reference's global prediction-coding table."""
        arrs, keep = _image_arrays_c(mi)
        t = None if table is None else np.ascontiguousarray(table, dtype=np.uint8)
        n = C.c_uint64()
        self._check(self._L.mraygb_encode_moment_image(self._h, C.byref(arrs), int(compress), int(quantization_bits),
                                                       int(entropy_coding), _hptr(t), C.byref(n)))
        out = np.zeros(max(n.value, 1), dtype=np.uint8)
        self._check(self._L.mraygb_copy_encoded(self._h, _hptr(out), out.size))
        del keep
        return out[:n.value].tobytes()

    def decode_moment_image(self, data: bytes):
        """load_moment_image on bytes (moment_image_io.cpp:291-310): (MomentImageHost, table or None)."""
        buf = np.frombuffer(data, dtype=np.uint8)
        arrs = MomentImageArrays()
        has_table = C.c_int()
        table = np.zeros(256, dtype=np.uint8)
        self._check(self._L.mraygb_decode_moment_image(self._h, _hptr(buf), buf.size, C.byref(arrs), _hptr(table),
                                                       C.byref(has_table)))
        mi, keep = _image_from_c(arrs)
        self._check(self._L.mraygb_decode_moment_image(self._h, _hptr(buf), buf.size, C.byref(arrs), None, None))
        del keep
        return mi, (table[:mi.num_moments].copy() if has_table.value else None)

    def write_moment_image(self, filename: str, mi: MomentImageHost, compress: bool, quantization_bits: int,
                           entropy_coding: bool = False, table=None) -> None:
        arrs, keep = _image_arrays_c(mi)
        t = None if table is None else np.ascontiguousarray(table, dtype=np.uint8)
        self._check(self._L.mraygb_write_moment_image(self._h, str(filename).encode(), C.byref(arrs), int(compress),
                                                      int(quantization_bits), int(entropy_coding), _hptr(t)))
        del keep

    def load_moment_image(self, filename: str):
        arrs = MomentImageArrays()
        has_table = C.c_int()
        table = np.zeros(256, dtype=np.uint8)
        path = str(filename).encode()
        self._check(self._L.mraygb_load_moment_image(self._h, path, C.byref(arrs), _hptr(table), C.byref(has_table)))
        mi, keep = _image_from_c(arrs)
        self._check(self._L.mraygb_load_moment_image(self._h, path, C.byref(arrs), None, None))
        del keep
        return mi, (table[:mi.num_moments].copy() if has_table.value else None)

    # ---- single scattering: the transmittance cache ----
    def reconstruct_single_scattering_cache(self, light_cam: Camera, rp: ReconstructionParameters,
                                            mi: MomentImageHost, return_cache: bool = True):
        """reconstruct_single_scattering_cache(ss, tf, params) (moment_raymarcher.cpp:217-258) of the light's
        moment image with the transfer function uploaded last.  The cache stays in the context for
        reconstruct / generate_reference_reconstructed_ss; returns it as float32 [z, y, x] (or None)."""
        data, index, bounds, cp = self._image_arrays(mi)
        ss = rp.ss
        cache = np.zeros((ss.cache_size_z, ss.cache_size_y, ss.cache_size_x), dtype=np.float32) \
            if return_cache else None
        self._check(self._L.mraygb_reconstruct_single_scattering_cache(
            self._h, C.byref(light_cam), C.byref(rp), mi.width, mi.height, mi.num_moments, _f3(mi.domain_min),
            _f3(mi.domain_max), _hptr(index), _hptr(data), data.size, _hptr(bounds), int(mi.prediction_code),
            int(mi.coding_warp), _hptr(cp), _hptr(cache)))
        return cache

    def stage_reconstruct_single_scattering_cache(self, light_cam, rp, width, height, num_moments, domain_min,
                                                  domain_max, index, pmoments, bounds, cache=None):
        self._check(self._L.mraygb_stage_reconstruct_single_scattering_cache(
            self._h, C.byref(light_cam), C.byref(rp), width, height, num_moments, _f3(domain_min), _f3(domain_max),
            _dptr(index), _dptr(pmoments), _dptr(bounds), _dptr(cache)))

    def upload_single_scattering_cache(self, cache, domain_min, domain_max) -> None:
        """A transmittance cache made elsewhere: float32 [z, y, x] (numpy array or CUDA tensor) on the box."""
        if hasattr(cache, "data_ptr"):
            nz, ny, nx = cache.shape
            self._check(self._L.mraygb_upload_single_scattering_cache(self._h, _dptr(cache), nx, ny, nz,
                                                                      _f3(domain_min), _f3(domain_max), 1))
        else:
            c = np.ascontiguousarray(cache, dtype=np.float32)
            nz, ny, nx = c.shape
            self._check(self._L.mraygb_upload_single_scattering_cache(self._h, _hptr(c), nx, ny, nz,
                                                                      _f3(domain_min), _f3(domain_max), 0))

    def generate_reference_reconstructed_ss(self, cam: Camera, rp: ReconstructionParameters, width: int,
                                            height: int, img: Optional[ColorImageHost] = None) -> ColorImageHost:
        """generate_reference_reconstructed_ss (moment_raymarcher.cpp:259-281) over the volume, transfer function
        and transmittance cache of the context."""
        img = img or ColorImageHost(width, height)
        self._check(self._L.mraygb_generate_reference_reconstructed_ss(self._h, C.byref(cam), C.byref(rp), width,
                                                                       height, _hptr(img.rgba_float),
                                                                       _hptr(img.rgba)))
        return img

    def stage_generate_reference_reconstructed_ss(self, cam, rp, width, height, rgba):
        self._check(self._L.mraygb_stage_generate_reference_reconstructed_ss(self._h, C.byref(cam), C.byref(rp),
                                                                             width, height, _dptr(rgba)))

    def quantize_prediction_coding(self, mi: MomentImageHost, table, out: Optional[np.ndarray] = None) -> np.ndarray:
        """quantize_prediction_coding(mi, table) (moment_quantization.cpp:239-276): the packed code bytes, as a view
        of ``out`` (a caller's uint8 buffer, e.g. pinned, of at least the packed size) or of a new array."""
        if not mi.is_compact:
            raise ValueError("quantize_prediction_coding needs a compact moment image")
        t = np.ascontiguousarray(table, dtype=np.uint8)
        if t.size < mi.num_moments:
            raise ValueError("the quantization table needs one entry per moment index")
        data = np.ascontiguousarray(mi.data, dtype=np.float32)
        index = np.ascontiguousarray(mi.index, dtype=np.uint32)
        if out is None:
            # an upper bound of the packed size (every stored value at the widest code); the library reports the
            # exact size and the copy back touches only those bytes
            out = np.empty(max((data.size * int(t[:mi.num_moments].max()) + 7) // 8, 1), dtype=np.uint8)
        elif out.dtype != np.uint8 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous uint8 array")
        n = C.c_uint64()
        self._check(self._L.mraygb_quantize_prediction_coding(self._h, mi.width, mi.height, mi.num_moments,
                                                              _hptr(index), _hptr(data), data.size, _hptr(t),
                                                              _hptr(out), out.size, C.byref(n)))
        return out[:n.value]

    def dequantize_prediction_coding(self, mi: MomentImageHost, table, qs) -> None:
        """dequantize_prediction_coding(mi, table, qs) (moment_quantization.cpp:278-332): the codes back into
        mi.data (values in [0, 1]; the image keeps its index and coding parameters)."""
        if not mi.is_compact:
            raise ValueError("dequantize_prediction_coding needs a compact moment image")
        t = np.ascontiguousarray(table, dtype=np.uint8)
        if t.size < mi.num_moments:
            raise ValueError("the quantization table needs one entry per moment index")
        index = np.ascontiguousarray(mi.index, dtype=np.uint32)
        q = np.ascontiguousarray(qs, dtype=np.uint8)
        size = int(index[-1])
        data = mi.data if (isinstance(mi.data, np.ndarray) and mi.data.dtype == np.float32 and mi.data.size >= size
                           and mi.data.flags.c_contiguous) else np.empty(size, dtype=np.float32)
        data = data[:size]
        self._check(self._L.mraygb_dequantize_prediction_coding(self._h, mi.width, mi.height, mi.num_moments,
                                                                _hptr(index), _hptr(t), _hptr(q), q.size,
                                                                _hptr(data), size))
        mi.data = data

    def create_quantization_table(self, mi: MomentImageHost, start_bits: int, sampling: int = 0,
                                  return_means: bool = False):
        """create_quantization_table(img, start_bits) (measure_coding_error.cpp:374-438) on a compact
        prediction-coded image; with ``sampling`` > 0 on its sample_moment_image (main.cpp:318-327).  Returns the
        table (u8 per moment index) and, with ``return_means``, the mean rRMSE of every (index, bits) pair as an
        (m, 32) array (NaN where not evaluated)."""
        if not mi.is_compact or mi.index is None:
            raise ValueError("create_quantization_table needs a compact moment image")
        if not mi.prediction_code:
            raise ValueError("create_quantization_table needs a prediction-coded moment image")
        m = mi.num_moments
        data = np.ascontiguousarray(mi.data, dtype=np.float32)
        index = np.ascontiguousarray(mi.index, dtype=np.uint32)
        cp = None if mi.coding_params is None else np.ascontiguousarray(mi.coding_params, dtype=np.uint16)
        table = np.zeros(m, dtype=np.uint8)
        means = np.zeros((m, 32), dtype=np.float32) if return_means else None
        self._check(self._L.mraygb_create_quantization_table(self._h, mi.width, mi.height, m, _hptr(index),
                                                             _hptr(data), data.size, int(mi.coding_warp), _hptr(cp),
                                                             int(start_bits), int(sampling), _hptr(table),
                                                             _hptr(means)))
        return (table, means) if return_means else table

    # ---- stage calls on device pointers ----
    def stage_reconstruct_error(self, cam, ep, width, height, num_moments, index, pmoments, bounds, error_bounds,
                                errors=None):
        self._check(self._L.mraygb_stage_reconstruct_error(self._h, C.byref(cam), C.byref(ep), width, height,
                                                           num_moments, _dptr(index), _dptr(pmoments), _dptr(bounds),
                                                           _dptr(error_bounds), _dptr(errors)))

    def stage_reconstruct_uncertainty(self, cam, up, mode, width, height, num_moments, domain_min, domain_max, index,
                                      pmoments, bounds, error_bounds, rgba):
        self._check(self._L.mraygb_stage_reconstruct_uncertainty(self._h, C.byref(cam), C.byref(up), int(mode),
                                                                 width, height, num_moments, _f3(domain_min),
                                                                 _f3(domain_max), _dptr(index), _dptr(pmoments),
                                                                 _dptr(bounds), _dptr(error_bounds), _dptr(rgba)))

    def stage_create_quantization_table(self, width, height, num_moments, index, data, coding_warp, coding_params,
                                        start_bits, sampling=64, return_means=False):
        """mraygb_stage_create_quantization_table: the table (and the means) of a compact prediction-coded image
        in device memory; see :meth:`create_quantization_table`."""
        table = np.zeros(num_moments, dtype=np.uint8)
        means = np.zeros((num_moments, 32), dtype=np.float32) if return_means else None
        self._check(self._L.mraygb_stage_create_quantization_table(self._h, width, height, num_moments,
                                                                   _dptr(index), _dptr(data), int(coding_warp),
                                                                   _dptr(coding_params), int(start_bits),
                                                                   int(sampling), _hptr(table), _hptr(means)))
        return (table, means) if return_means else table

    def stage_generate_moments(self, cam, gp, width, height, num_moments, moments, bounds=None, counts=None):
        self._check(self._L.mraygb_stage_generate_moments(self._h, C.byref(cam), C.byref(gp), width, height,
                                                          num_moments, _dptr(moments), _dptr(bounds),
                                                          _dptr(counts)))

    def stage_compact(self, width, height, num_moments, counts, moments, index, compact, capacity=None) -> int:
        total = C.c_uint64()
        if capacity is None:
            capacity = compact.numel() if hasattr(compact, "numel") else width * height * num_moments
        self._check(self._L.mraygb_stage_compact(self._h, width, height, num_moments, _dptr(counts), _dptr(moments),
                                                 _dptr(index), _dptr(compact), int(capacity), C.byref(total)))
        return int(total.value)

    def measure_fp32_rate(self) -> float:
        """The FP32 FMA roof of the device in TFLOP/s (mraygb_measure_fp32_rate)."""
        v = C.c_double()
        self._check(self._L.mraygb_measure_fp32_rate(self._h, C.byref(v)))
        return float(v.value)

    def stage_libm_sincosf(self, x, s, c):
        """cosf / sinf of the MESE algebra on device float32 tensors (the host C library's results on [-pi, pi])."""
        self._check(self._L.mraygb_stage_libm_sincosf(self._h, _dptr(x), _dptr(s), _dptr(c), int(x.numel())))

    def stage_prediction_encode(self, width, height, num_moments, index, data, data_size, coding_warp=0,
                                bias=1e-4, coding_params=None):
        self._check(self._L.mraygb_stage_prediction_encode(self._h, width, height, num_moments, _dptr(index),
                                                           _dptr(data), int(data_size), int(coding_warp),
                                                           float(bias), _dptr(coding_params)))

    def stage_quantize_prediction_coding(self, width, height, num_moments, index, data, table, out,
                                         capacity=None) -> int:
        t = np.ascontiguousarray(table, dtype=np.uint8)
        n = C.c_uint64()
        if capacity is None:
            capacity = out.numel() * out.element_size()
        self._check(self._L.mraygb_stage_quantize_prediction_coding(self._h, width, height, num_moments,
                                                                    _dptr(index), _dptr(data), _hptr(t), _dptr(out),
                                                                    int(capacity), C.byref(n)))
        return int(n.value)

    def stage_dequantize_prediction_coding(self, width, height, num_moments, index, table, packed, num_bytes,
                                           data):
        t = np.ascontiguousarray(table, dtype=np.uint8)
        self._check(self._L.mraygb_stage_dequantize_prediction_coding(self._h, width, height, num_moments,
                                                                      _dptr(index), _hptr(t), _dptr(packed),
                                                                      int(num_bytes), _dptr(data)))

    def stage_prepare_moments(self, width, height, num_moments, index, data, pmoments, prediction_code=False,
                              coding_warp=0, coding_params=None, bias=1e-6):
        self._check(self._L.mraygb_stage_prepare_moments(self._h, width, height, num_moments, _dptr(index),
                                                         _dptr(data), int(prediction_code), int(coding_warp),
                                                         _dptr(coding_params), float(bias), _dptr(pmoments)))

    def stage_reconstruct(self, cam, rp, width, height, num_moments, domain_min, domain_max, index, pmoments,
                          bounds, rgba, rgba8=None):
        self._check(self._L.mraygb_stage_reconstruct(self._h, C.byref(cam), C.byref(rp), width, height,
                                                     num_moments, _f3(domain_min), _f3(domain_max), _dptr(index),
                                                     _dptr(pmoments), _dptr(bounds), _dptr(rgba), _dptr(rgba8)))

    # ---- differentiation form (device buffers: CUDA tensors or addresses) ----
    def diff_forward(self, cam, gp, rp, width, height, num_moments, tf, moments, bounds4, pmoments, rgba) -> None:
        self._check(self._L.mraygb_diff_forward(self._h, C.byref(cam), C.byref(gp), C.byref(rp), width, height,
                                                num_moments, _dptr(tf), _dptr(moments), _dptr(bounds4),
                                                _dptr(pmoments), _dptr(rgba)))

    def diff_backward(self, cam, gp, rp, width, height, num_moments, tf, moments, bounds4, pmoments, rgba, grad_rgba,
                      grad_tf, grad_volume=None) -> None:
        self._check(self._L.mraygb_diff_backward(self._h, C.byref(cam), C.byref(gp), C.byref(rp), width, height,
                                                 num_moments, _dptr(tf), _dptr(moments), _dptr(bounds4),
                                                 _dptr(pmoments), _dptr(rgba), _dptr(grad_rgba), _dptr(grad_tf),
                                                 _dptr(grad_volume)))


def _image_arrays_c(mi: MomentImageHost):
    """The mraygb_moment_image view of a MomentImageHost, and the arrays that must stay alive while it is used."""
    a = MomentImageArrays()
    a.width, a.height, a.num_moments = mi.width, mi.height, mi.num_moments
    a.is_compact, a.prediction_code, a.coding_warp = int(mi.is_compact), int(mi.prediction_code), int(mi.coding_warp)
    for i in range(3):
        a.domain_min[i], a.domain_max[i] = mi.domain_min[i], mi.domain_max[i]
    data = np.ascontiguousarray(mi.data, dtype=np.float32)
    index = np.ascontiguousarray(mi.index, dtype=np.uint32) if mi.is_compact else None
    bounds = np.ascontiguousarray(mi.bounds, dtype=np.uint16) if mi.bounds is not None else None
    eb = np.ascontiguousarray(mi.error_bounds, dtype=np.uint16) if mi.error_bounds is not None else None
    cp = np.ascontiguousarray(mi.coding_params, dtype=np.uint16) if mi.coding_params is not None else None
    a.data_size = data.size
    a.index, a.data = _addr(index), _addr(data)
    a.bounds, a.error_bounds, a.coding_params = _addr(bounds), _addr(eb), _addr(cp)
    return a, (data, index, bounds, eb, cp)


def _addr(a):
    return None if a is None else a.ctypes.data


def _image_from_c(a: MomentImageArrays):
    """A MomentImageHost with the arrays a decoded header asks for, pointed to by ``a``."""
    mi = MomentImageHost(a.width, a.height, a.num_moments, bool(a.is_compact), bool(a.has_bounds))
    mi.is_compact, mi.prediction_code, mi.coding_warp = bool(a.is_compact), bool(a.prediction_code), a.coding_warp
    mi.domain_min = tuple(float(a.domain_min[i]) for i in range(3))
    mi.domain_max = tuple(float(a.domain_max[i]) for i in range(3))
    mi.data = np.zeros(a.data_size, dtype=np.float32)
    if not mi.is_compact:
        mi.index = None
    if a.has_error_bounds:
        mi.add_error_bounds()
    mi.coding_params = np.zeros(2 * (mi.num_moments - 1), dtype=np.uint16) if a.has_coding_params else None
    a.index, a.data = _addr(mi.index), _addr(mi.data)
    a.bounds, a.error_bounds, a.coding_params = _addr(mi.bounds), _addr(mi.error_bounds), _addr(mi.coding_params)
    return mi, None


def lz4_compress(data: bytes) -> bytes:
    """An LZ4 block of ``data`` (the compression of the file format's sections)."""
    L = _lib.load()
    src = np.frombuffer(data, dtype=np.uint8)
    cap = src.size + src.size // 255 + 16
    dst = np.zeros(cap, dtype=np.uint8)
    n = L.mraygb_lz4_compress(_hptr(src) if src.size else None, src.size, _hptr(dst), cap)
    if n == 0:
        raise _lib.MrayError(1, "LZ4 block does not fit")
    return dst[:n].tobytes()


def lz4_decompress(block: bytes, size: int) -> bytes:
    L = _lib.load()
    src = np.frombuffer(block, dtype=np.uint8)
    dst = np.zeros(max(size, 1), dtype=np.uint8)
    r = L.mraygb_lz4_decompress(_hptr(src), src.size, _hptr(dst), size)
    if r < 0:
        raise _lib.MrayError(1, "malformed LZ4 block")
    return dst[:r].tobytes()


def entropy_encode(width: int, height: int, num_moments: int, index, codes, table, threads: int = 0) -> bytes:
    """The entropy-coded payload (moment_image_coding.cpp:206-221) of u16 codes in the layout of the moment data."""
    L = _lib.load()
    idx = np.ascontiguousarray(index, dtype=np.uint32)
    c = np.ascontiguousarray(codes, dtype=np.uint16)
    t = np.ascontiguousarray(table, dtype=np.uint8)
    n = C.c_uint64()
    st = L.mraygb_entropy_encode(width, height, num_moments, _hptr(idx), _hptr(c), _hptr(t), threads, None, 0,
                                 C.byref(n))
    if st:
        raise _lib.MrayError(st, "entropy_encode: invalid arguments")
    out = np.zeros(max(n.value, 1), dtype=np.uint8)
    L.mraygb_entropy_encode(width, height, num_moments, _hptr(idx), _hptr(c), _hptr(t), threads, _hptr(out), out.size,
                            C.byref(n))
    return out[:n.value].tobytes()


def entropy_decode(payload: bytes, width: int, height: int, num_moments: int, index, table,
                   threads: int = 0) -> np.ndarray:
    L = _lib.load()
    buf = np.frombuffer(payload, dtype=np.uint8)
    idx = np.ascontiguousarray(index, dtype=np.uint32)
    t = np.ascontiguousarray(table, dtype=np.uint8)
    codes = np.zeros(max(int(idx[-1]), 1), dtype=np.uint16)
    st = L.mraygb_entropy_decode(_hptr(buf), buf.size, width, height, num_moments, _hptr(idx), _hptr(t), threads,
                                 _hptr(codes))
    if st:
        raise _lib.MrayError(st, "malformed entropy-coded payload")
    return codes[:int(idx[-1])]


_default: dict = {}


def default_context(device: int = 0) -> Context:
    ctx = _default.get(device)
    if ctx is None:
        ctx = _default[device] = Context(device)
    return ctx


def generate(cam: Camera, volume, mi: MomentImageHost, params: GenerationParameters,
             context: Optional[Context] = None) -> None:
    """generate(cam, volume, mi, params) for a RegularGrid or Particles (moment_raymarcher.h:48-49): fills ``mi``
    in place."""
    ctx = context or default_context()
    if isinstance(volume, Particles):
        ctx.upload_particles(volume.x, volume.y, volume.z, volume.values, volume.smoothing_length,
                             volume.domain_min, volume.domain_max)
    else:
        ctx.upload_grid(volume.data, volume.domain_min, volume.domain_max)
    out = ctx.generate(cam, params, mi.width, mi.height, mi.num_moments, out=mi)
    mi.domain_min, mi.domain_max = volume.domain_min, volume.domain_max
    assert out is mi


def quantize_prediction_coding(mi: MomentImageHost, table, context: Optional[Context] = None,
                               out: Optional[np.ndarray] = None) -> np.ndarray:
    """moment_quantization::quantize_prediction_coding(mi, table) on the GPU (``out``: an optional caller buffer)."""
    return (context or default_context()).quantize_prediction_coding(mi, table, out)


def dequantize_prediction_coding(mi: MomentImageHost, table, qs, context: Optional[Context] = None) -> None:
    """moment_quantization::dequantize_prediction_coding(mi, table, qs) on the GPU (into mi.data)."""
    (context or default_context()).dequantize_prediction_coding(mi, table, qs)


def create_quantization_table(img: MomentImageHost, start_bits: int, context: Optional[Context] = None,
                              sampling: int = 0) -> np.ndarray:
    """create_quantization_table(img, start_bits) (measure_coding_error.cpp:374-438): the data-dependent table
    for a compact prediction-coded image.  The reference installs it as its global table; here it is returned for
    :func:`quantize_prediction_coding`.  ``sampling`` > 0 first takes sample_moment_image(img, s, s) with
    s = min(width, sampling) = min(height, sampling), as main.cpp:318-327 does with quantization_curve_sampling."""
    return (context or default_context()).create_quantization_table(img, start_bits, sampling)


def default_quantization_table(num_moments: int, num_bits: int) -> np.ndarray:
    """get_prediction_coding_quantization_table without a loaded table (moment_quantization.cpp:186-203):
    16 bits for index 0, num_bits for the rest."""
    return np.array([16] + [num_bits] * (num_moments - 1), dtype=np.uint8)[:num_moments]


def reconstruct(cam: Camera, mi: MomentImageHost, tf: TransferFunction, img: ColorImageHost,
                params: ReconstructionParameters, context: Optional[Context] = None,
                ss: Optional[SingleScatteringImageHost] = None) -> None:
    """reconstruct(cam, mi, tf, img, params) and, with ``ss``, reconstruct(cam, mi, tf, img, ss, params)
    (moment_raymarcher.h:61-64, moment_raymarcher.cpp:329-351): fills ``img`` in place.  With ``ss`` the
    transmittance cache of the light's image is built first and sampled for the in-scattered light."""
    ctx = context or default_context()
    ctx.upload_tf(tf.table)
    if ss is not None:
        ctx.reconstruct_single_scattering_cache(ss.cam, params, ss.img, return_cache=False)
    ctx.reconstruct(cam, params, mi, img)


def write_moment_image(mi: MomentImageHost, filename: str, compress: bool, quantization_bits: int,
                       entropy_coding: bool = False, table=None, context: Optional[Context] = None) -> None:
    """write_moment_image(mi, filename, compress, quantizationBits, entropy_coding) (moment_image_io.h:32-33);
    ``table``: the prediction-coding table the reference keeps globally (set_prediction_coding_quantization_table)."""
    (context or default_context()).write_moment_image(filename, mi, compress, quantization_bits, entropy_coding, table)


def load_moment_image(filename: str, context: Optional[Context] = None):
    """load_moment_image(filename) (moment_image_io.h:30): (MomentImageHost, the table the file holds or None)."""
    return (context or default_context()).load_moment_image(filename)


def reconstruct_single_scattering_cache(ss: SingleScatteringImageHost, tf: TransferFunction,
                                        params: ReconstructionParameters,
                                        context: Optional[Context] = None) -> SingleScatteringCacheHost:
    """reconstruct_single_scattering_cache(ss, tf, params) (moment_raymarcher.cpp:217-258)."""
    ctx = context or default_context()
    ctx.upload_tf(tf.table)
    cache = ctx.reconstruct_single_scattering_cache(ss.cam, params, ss.img)
    return SingleScatteringCacheHost(RegularGrid(cache, ss.img.domain_min, ss.img.domain_max))


def generate_reference_reconstructed_ss(cam: Camera, tf: TransferFunction, volume, img: ColorImageHost,
                                        ss: SingleScatteringImageHost, params: ReconstructionParameters,
                                        context: Optional[Context] = None) -> None:
    """generate_reference_reconstructed_ss(cam, tf, volume, img, ss, params) (moment_raymarcher.cpp:259-281): the
    reference renderer with the single-scattering transmittance of the light image's cache."""
    ctx = context or default_context()
    ctx.upload_tf(tf.table)
    ctx.reconstruct_single_scattering_cache(ss.cam, params, ss.img, return_cache=False)
    _upload_volume(ctx, volume)
    ctx.generate_reference_reconstructed_ss(cam, params, img.width, img.height, img)


def _upload_volume(ctx: Context, volume) -> None:
    if isinstance(volume, Particles):
        ctx.upload_particles(volume.x, volume.y, volume.z, volume.values, volume.smoothing_length,
                             volume.domain_min, volume.domain_max)
    else:
        ctx.upload_grid(volume.data, volume.domain_min, volume.domain_max)


def reconstruct_error(cam: Camera, volume, mi: MomentImageHost, params: ErrorReconstructionParameters,
                      context: Optional[Context] = None) -> None:
    """reconstruct_error(cam, volume, mi, params) for a RegularGrid or Particles (moment_raymarcher.h:73-76): fills
    mi.error_bounds in place."""
    ctx = context or default_context()
    _upload_volume(ctx, volume)
    ctx.reconstruct_error(cam, params, mi)


def reconstruct_uncertainty_interpolation(cam: Camera, mi: MomentImageHost, tf: TransferFunction,
                                          img: ColorImageHost, params: UncertaintyReconstructionParameters,
                                          context: Optional[Context] = None) -> None:
    """reconstruct_uncertainty_interpolation(cam, mi, tf, img, params) (moment_raymarcher.h:78-79)."""
    ctx = context or default_context()
    ctx.upload_tf(tf.table)
    ctx.reconstruct_uncertainty(cam, params, 0, mi, img)


def reconstruct_uncertainty_convolution(cam: Camera, mi: MomentImageHost, tf: UncertaintyTransferFunction,
                                        img: ColorImageHost, params: UncertaintyReconstructionParameters,
                                        context: Optional[Context] = None) -> None:
    """reconstruct_uncertainty_convolution(cam, mi, tf, img, params) (moment_raymarcher.h:84-85) with the table of
    read_from_disk_uncertainty."""
    ctx = context or default_context()
    ctx.upload_uncertainty_tf(tf)
    ctx.reconstruct_uncertainty(cam, params, 1, mi, img)


def generate_reference(cam: Camera, tf: TransferFunction, volume, img: ColorImageHost, params: ReferenceParameters,
                       context: Optional[Context] = None) -> None:
    """generate_reference(cam, tf, volume, img, params) (moment_raymarcher.h, moment_raymarcher.cpp:64-80): direct
    volume rendering of a RegularGrid or Particles into ``img``."""
    ctx = context or default_context()
    _upload_volume(ctx, volume)
    ctx.upload_tf(tf.table)
    ctx.generate_reference(cam, params, img.width, img.height, img)
