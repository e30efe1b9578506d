"""ORACLE -- test infrastructure only.

ctypes front end of the C restatement of the reference's CPU path (``oracle/mray_oracle.c``, built by
``oracle/Makefile`` into ``oracle/_build/liboracle.so``) and, where it was built, of the reference's own CPU
code (``oracle/_ref/libmrayref.so``).  Imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` only; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libmrayref.so")
REF_REL_LIB_PATH = os.path.join(HERE, "_ref", "libmrayref_release.so")

_lock = threading.Lock()
_lib = None
_ref = None
_ref_rel = None

fp = np.ctypeslib.ndpointer


class Options(C.Structure):
    _fields_ = [("exact_atan", C.c_int), ("nthreads", C.c_int), ("row_begin", C.c_int), ("row_end", C.c_int),
                ("row_step", C.c_int), ("tf_bspline", C.c_int), ("bounds_out", C.c_void_p),
                ("bounds_in", C.c_void_p), ("col_begin", C.c_int), ("col_end", C.c_int), ("col_step", C.c_int),
                ("ss_cache", C.c_void_p), ("density_offset", C.c_double), ("density_offsets", C.c_void_p)]


class Grid(C.Structure):
    _fields_ = [("data", C.c_void_p), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dmin", C.c_float * 3), ("dmax", C.c_float * 3)]


def build(force: bool = False) -> None:
    """Compile liboracle.so (and the reference library when its sources exist)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def build_ref() -> bool:
    """Compile the reference's own CPU path into oracle/_ref (only where the reference sources were staged)."""
    from stage_reference import reference_src

    src = reference_src()
    if src is None:
        return False
    jobs = str(min(16, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-j", jobs, "-C", HERE, "ref", "refrel", f"REF={src}"], check=True)
    return os.path.exists(REF_LIB_PATH)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(LIB_PATH)
            _declare(_lib)
        return _lib


def ref_lib():
    """The reference's own CPU code, or None where it cannot be built."""
    global _ref
    with _lock:
        if _ref is None:
            if not os.path.exists(REF_LIB_PATH) and not build_ref():
                return None
            _ref = C.CDLL(REF_LIB_PATH)
        return _ref


def ref_release_lib():
    """The reference's own CPU code built with its Release flags (timing only), or None where it cannot be built."""
    global _ref_rel
    with _lock:
        if _ref_rel is None:
            if not os.path.exists(REF_REL_LIB_PATH) and not build_ref():
                return None
            if not os.path.exists(REF_REL_LIB_PATH):
                return None
            L = C.CDLL(REF_REL_LIB_PATH)
            from mray_gb300.types import Camera, GenerationParameters, ReconstructionParameters

            L.ref_grid_create.restype = C.c_void_p
            L.ref_grid_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
            L.ref_grid_destroy.argtypes = [C.c_void_p]
            L.ref_grid_destroy.restype = None
            L.ref_pipeline_rows.restype = C.c_int64
            L.ref_pipeline_rows.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(GenerationParameters),
                                            C.POINTER(ReconstructionParameters), C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
            _ref_rel = L
        return _ref_rel


class RefPipeline:
    """The reference's own generate -> compaction -> prediction coding -> quantize / dequantize -> reconstruct flow
    (Release build) over row samples of an image, on a grid held between calls (timing of the CPU baseline)."""

    def __init__(self, volume, dmin, dmax):
        self.L = ref_release_lib()
        if self.L is None:
            raise OSError("the reference's CPU path is not built (its sources are not staged)")
        self._vol = np.ascontiguousarray(volume, dtype=np.float32)
        nz, ny, nx = self._vol.shape
        dmn = np.asarray(dmin, dtype=np.float32)
        dmx = np.asarray(dmax, dtype=np.float32)
        self.handle = self.L.ref_grid_create(_ptr(self._vol), nx, ny, nz, _ptr(dmn), _ptr(dmx))
        self._vol = None

    def rows(self, cam, gen, rec, width, height, m, row0, row_step, table, tf_row, rgba=None):
        t = np.ascontiguousarray(table, dtype=np.uint8) if table is not None else None
        row = np.ascontiguousarray(tf_row, dtype=np.float32)
        return int(self.L.ref_pipeline_rows(self.handle, C.byref(cam), C.byref(gen), C.byref(rec), width, height, m,
                                            row0, row_step, _ptr(t) if t is not None else None, _ptr(row),
                                            _ptr(rgba) if rgba is not None else None))

    def close(self):
        if self.handle:
            self.L.ref_grid_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


class ParticleSet:
    """oracle_particles: the reference's uniform particle grid built by the oracle (owns its C memory)."""

    def __init__(self, x, y, z, v, h, dmin, dmax):
        """h: one smoothing length (the reference's particles), or one per particle (the Wendland C2 variant)."""
        L = lib()
        self._keep = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, v)]
        self.n = self._keep[0].size
        self.dmin, self.dmax = tuple(dmin), tuple(dmax)
        if np.ndim(h) == 0:
            self.h = float(h)
            self.handle = L.oracle_particles_create(*[_ptr(a) for a in self._keep], self.n, self.h,
                                                    (C.c_float * 3)(*dmin), (C.c_float * 3)(*dmax))
        else:
            hs = np.ascontiguousarray(h, dtype=np.float32)
            self._keep.append(hs)
            self.h = float(hs.max())
            self.handle = L.oracle_particles_create_h(*[_ptr(a) for a in self._keep], self.n,
                                                      (C.c_float * 3)(*dmin), (C.c_float * 3)(*dmax))
        if not self.handle:
            raise ValueError("no particles")

    def __del__(self):
        if getattr(self, "handle", None):
            lib().oracle_particles_destroy(self.handle)
            self.handle = None


def _declare(L):
    from mray_gb300.types import Camera, GenerationParameters, ReconstructionParameters

    P = C.POINTER
    for sfx, R in (("f32", C.c_float), ("f64", C.c_double)):
        f = getattr(L, f"oracle_generate_moments_{sfx}")
        f.argtypes = [P(Camera), P(GenerationParameters), P(Grid), C.c_int, C.c_int, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_void_p, P(Options)]
        f.restype = None
        f = getattr(L, f"oracle_prepare_moments_{sfx}")
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_float,
                      C.c_void_p, P(Options)]
        f.restype = None
        f = getattr(L, f"oracle_reconstruct_{sfx}")
        f.argtypes = [P(Camera), P(ReconstructionParameters), C.c_int, C.c_int, C.c_int, C.c_float * 3,
                      C.c_float * 3, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, P(Options)]
        f.restype = None
        getattr(L, f"oracle_evaluate_mese_{sfx}").restype = R
        getattr(L, f"oracle_evaluate_mese_{sfx}").argtypes = [C.c_int, R, C.c_void_p, C.c_int]
        getattr(L, f"oracle_fast_atan_{sfx}").restype = R
        getattr(L, f"oracle_fast_atan_{sfx}").argtypes = [R]
        getattr(L, f"oracle_determine_best_number_moments_{sfx}").argtypes = [C.c_int, C.c_void_p, R]
        getattr(L, f"oracle_determine_best_number_moments_{sfx}").restype = C.c_int
        getattr(L, f"oracle_count_moments_{sfx}").argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, R,
                                                              C.c_void_p, C.c_int]
        getattr(L, f"oracle_count_moments_{sfx}").restype = None
        getattr(L, f"oracle_rmse_{sfx}").argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        getattr(L, f"oracle_rmse_{sfx}").restype = R
        getattr(L, f"oracle_transform_quantization_real_{sfx}").argtypes = [C.c_int, C.c_void_p, R, C.c_void_p]
        getattr(L, f"oracle_grid_sample_{sfx}").argtypes = [P(Grid), C.c_void_p]
        getattr(L, f"oracle_grid_sample_{sfx}").restype = R
        getattr(L, f"oracle_tf_sample_{sfx}").argtypes = [C.c_void_p, R, R, C.c_void_p]
        getattr(L, f"oracle_tf_sample_bspline_{sfx}").argtypes = [C.c_void_p, R, C.c_void_p]
        getattr(L, f"oracle_tf_sample_linear_{sfx}").argtypes = [C.c_void_p, R, C.c_void_p]
    L.oracle_particles_create.restype = C.c_void_p
    L.oracle_particles_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_float,
                                          C.c_float * 3, C.c_float * 3]
    L.oracle_particles_create_h.restype = C.c_void_p
    L.oracle_particles_create_h.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                            C.c_float * 3, C.c_float * 3]
    L.oracle_particles_destroy.argtypes = [C.c_void_p]
    for sfx, R in (("f32", C.c_float), ("f64", C.c_double)):
        f = getattr(L, f"oracle_generate_moments_particles_{sfx}")
        f.argtypes = [P(Camera), P(GenerationParameters), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_void_p, P(Options)]
        f.restype = None
        getattr(L, f"oracle_particles_sample_{sfx}").argtypes = [C.c_void_p, C.c_void_p]
        getattr(L, f"oracle_particles_sample_{sfx}").restype = R
    L.oracle_compact.restype = C.c_uint64
    L.oracle_compact.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.oracle_prediction_encode.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                           C.c_float, C.c_void_p, P(Options)]
    L.oracle_find_coding_transform_parameters.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                          C.c_uint64, C.c_void_p]
    L.oracle_quantize.restype = C.c_uint32
    L.oracle_quantize.argtypes = [C.c_float, C.c_int, C.c_float, C.c_float]
    L.oracle_dequantize.restype = C.c_float
    L.oracle_dequantize.argtypes = [C.c_uint32, C.c_int, C.c_float, C.c_float]
    L.LZ4_compress_default.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.LZ4_decompress_safe.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.oracle_quantize_prediction_coding.restype = C.c_uint64
    L.oracle_quantize_prediction_coding.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                    C.c_void_p]
    L.oracle_dequantize_prediction_coding.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                      C.c_void_p, C.c_uint64, C.c_void_p]
    L.oracle_preintegrate.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
    L.oracle_rgba_to_u8.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p]
    for sfx in ("f32", "f64"):
        getattr(L, f"oracle_reconstruct_error_{sfx}").argtypes = [
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        getattr(L, f"oracle_uncertainty_tf_{sfx}").argtypes = [C.c_void_p, C.c_float, C.c_int, C.c_void_p]
        getattr(L, f"oracle_reconstruct_uncertainty_{sfx}").argtypes = [
            C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float * 3, C.c_float * 3, C.c_void_p,
            C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    for sfx in ("f32", "f64"):
        getattr(L, f"oracle_error_stream_{sfx}").argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        getattr(L, f"oracle_ss_cache_{sfx}").argtypes = [
            P(Camera), P(ReconstructionParameters), C.c_int, C.c_int, C.c_int, C.c_float * 3, C.c_float * 3,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        getattr(L, f"oracle_generate_reference_{sfx}").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                                   C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                                   C.c_void_p]
    L.oracle_libm_sincosf.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
    L.oracle_libm_sincosf.restype = None
    L.oracle_set_rounded_trig.argtypes = [C.c_int]
    L.oracle_set_rounded_trig.restype = None
    L.oracle_sample_moment_image.restype = C.c_uint64
    L.oracle_sample_moment_image.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                             C.c_void_p]
    for sfx, R in (("f32", C.c_float), ("f64", C.c_double)):
        f = getattr(L, f"oracle_measure_idx_error_{sfx}")
        f.restype = R
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                      C.c_void_p, C.c_void_p, C.c_int]
        f = getattr(L, f"oracle_create_quantization_table_{sfx}")
        f.restype = C.c_int
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_int]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _grid(volume, dmin, dmax):
    g = Grid()
    v = np.ascontiguousarray(volume, dtype=np.float32)
    g.data = v.ctypes.data
    g.nz, g.ny, g.nx = v.shape
    for i in range(3):
        g.dmin[i] = dmin[i]
        g.dmax[i] = dmax[i]
    return g, v


def options(nthreads=0, rows=None, exact_atan=False):
    o = Options()
    o.exact_atan = int(exact_atan)
    o.nthreads = int(nthreads)
    if rows is None:
        o.row_begin, o.row_end, o.row_step = 0, 0, 1
    else:
        o.row_begin, o.row_end, o.row_step = rows
    return o


def _dt(precision):
    return np.float32 if precision == "f32" else np.float64


# --------------------------------------------------------------------------------------------------------------
# pipeline stages
# --------------------------------------------------------------------------------------------------------------

def generate_moments(cam, gp, volume, dmin, dmax, width, height, m, precision="f32", nthreads=0, rows=None,
                     float_bounds=False, cols=None):
    """generate_host's per-pixel loop: returns (moments[H,W,m], bounds[H,W,2] u16, counts[H,W] u32), and with
    float_bounds the unquantized bounds[H,W,2] in the working precision as a fourth value."""
    L = lib()
    dt = _dt(precision)
    g, keep = _grid(volume, dmin, dmax)
    moments = np.zeros((height, width, m), dtype=dt)
    bounds = np.zeros((height, width, 2), dtype=np.uint16)
    counts = np.zeros((height, width), dtype=np.uint32)
    o = options(nthreads, rows)
    if cols is not None:
        o.col_begin, o.col_end, o.col_step = cols
    bf = np.zeros((height, width, 2), dtype=dt) if float_bounds else None
    o.bounds_out = bf.ctypes.data if float_bounds else None
    getattr(L, f"oracle_generate_moments_{precision}")(C.byref(cam), C.byref(gp), C.byref(g), width, height, m,
                                                       _ptr(moments), _ptr(bounds), _ptr(counts), C.byref(o))
    del keep
    if float_bounds:
        return moments, bounds, counts, bf
    return moments, bounds, counts


def generate_moments_particles(cam, gp, parts: ParticleSet, width, height, m, precision="f32", nthreads=0,
                               rows=None):
    """generate_host's per-pixel loop over SPH particles: (moments[H,W,m], bounds[H,W,2] u16, counts[H,W] u32)."""
    L = lib()
    dt = _dt(precision)
    moments = np.zeros((height, width, m), dtype=dt)
    bounds = np.zeros((height, width, 2), dtype=np.uint16)
    counts = np.zeros((height, width), dtype=np.uint32)
    o = options(nthreads, rows)
    getattr(L, f"oracle_generate_moments_particles_{precision}")(C.byref(cam), C.byref(gp), parts.handle, width,
                                                                 height, m, _ptr(moments), _ptr(bounds),
                                                                 _ptr(counts), C.byref(o))
    return moments, bounds, counts


def particles_sample(parts: ParticleSet, points, precision="f32"):
    """Particles::sample at each point (N x 3)."""
    L = lib()
    dt = _dt(precision)
    pts = np.ascontiguousarray(points, dtype=dt)
    f = getattr(L, f"oracle_particles_sample_{precision}")
    return np.array([f(parts.handle, _ptr(pts[i])) for i in range(pts.shape[0])], dtype=dt)


def compact(counts, moments):
    """MomentImageHost::compact: returns (index[W*H+1] u32, data[total] f32)."""
    L = lib()
    h, w, m = moments.shape
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    mo = np.ascontiguousarray(moments, dtype=np.float32)
    index = np.zeros(w * h + 1, dtype=np.uint32)
    total = int(L.oracle_compact(w, h, m, _ptr(counts), _ptr(mo), _ptr(index), None))
    data = np.zeros(max(total, 1), dtype=np.float32)[:total]
    if total:
        L.oracle_compact(w, h, m, _ptr(counts), _ptr(mo), _ptr(index), _ptr(data))
    return index, data


def prediction_encode(width, height, m, index, data, coding_warp=0, bias=1e-4, nthreads=0):
    """MomentImageHost::prediction_encode on a copy; returns (data, coding_params u16[2(m-1)])."""
    L = lib()
    d = np.array(data, dtype=np.float32, copy=True)
    cp = np.zeros(max(2 * (m - 1), 1), dtype=np.uint16)
    o = options(nthreads)
    L.oracle_prediction_encode(width, height, m, _ptr(np.ascontiguousarray(index, dtype=np.uint32)), _ptr(d),
                               d.size, coding_warp, bias, _ptr(cp), C.byref(o))
    return d, cp[:2 * (m - 1)]


def count_moments(moments, counts_in, error_threshold, precision="f32", nthreads=0):
    """compute_num_moments with an error threshold: per pixel of moments[H, W, m] (or [P, m]) whose counts_in is
    non-zero, determine_best_number_moments; returns u32 counts."""
    L = lib()
    m = moments.shape[-1]
    mo = np.ascontiguousarray(moments, dtype=_dt(precision)).reshape(-1, m)
    cin = np.ascontiguousarray(counts_in, dtype=np.uint32).reshape(-1)
    out = np.zeros(mo.shape[0], dtype=np.uint32)
    getattr(L, f"oracle_count_moments_{precision}")(mo.shape[0], m, _ptr(mo), _ptr(cin), error_threshold,
                                                     _ptr(out), nthreads)
    return out


def libm_sincosf(x):
    """The C library's (sinf(x), cosf(x)) for a float32 array."""
    xs = np.ascontiguousarray(x, dtype=np.float32)
    s = np.empty_like(xs)
    c = np.empty_like(xs)
    lib().oracle_libm_sincosf(xs.size, _ptr(xs), _ptr(s), _ptr(c))
    return s, c


def find_coding_transform_parameters(width, height, m, index, data):
    L = lib()
    d = np.ascontiguousarray(data, dtype=np.float32)
    out = np.zeros(max(2 * (m - 1), 1), dtype=np.float32)
    L.oracle_find_coding_transform_parameters(width, height, m, _ptr(np.ascontiguousarray(index, dtype=np.uint32)),
                                              _ptr(d), d.size, _ptr(out))
    return out[:2 * (m - 1)]


def quantize_prediction_coding(width, height, m, index, data, table):
    L = lib()
    idx = np.ascontiguousarray(index, dtype=np.uint32)
    d = np.ascontiguousarray(data, dtype=np.float32)
    t = np.ascontiguousarray(table, dtype=np.uint8)
    n = int(L.oracle_quantize_prediction_coding(width, height, m, _ptr(idx), _ptr(d), _ptr(t), None))
    out = np.zeros(max(n, 1), dtype=np.uint8)
    L.oracle_quantize_prediction_coding(width, height, m, _ptr(idx), _ptr(d), _ptr(t), _ptr(out))
    return out[:n]


def entropy_codes(width, height, m, index, data, table, prediction_code):
    """The symbols the reference's entropy coder codes (moment_image_coding.cpp:110-143), as u16 in the layout of
    the moment data: quantize(value, table[l], 0, 1) for the zeroth moment and for prediction codes, else over
    [-1/pi, 1/pi]."""
    L = lib()
    idx = np.asarray(index, dtype=np.int64)
    d = np.asarray(data, dtype=np.float32)
    lo = np.float32(0.0) if prediction_code else np.float32(-1.0 / np.pi)
    hi = np.float32(1.0) if prediction_code else np.float32(1.0 / np.pi)
    out = np.zeros(d.size, dtype=np.uint16)
    for p in range(width * height):
        for l in range(int(idx[p + 1] - idx[p])):
            a, b = (0.0, 1.0) if l == 0 else (float(lo), float(hi))
            out[idx[p] + l] = L.oracle_quantize(float(d[idx[p] + l]), int(table[l]), a, b) & 0xffff
    return out


def lz4_compress(data: bytes) -> bytes:
    """The oracle's own LZ4 block encoder (oracle/lz4_ref.c)."""
    L = lib()
    src = np.frombuffer(data, dtype=np.uint8)
    cap = src.size + src.size // 255 + 16
    dst = np.zeros(cap, dtype=np.uint8)
    n = L.LZ4_compress_default(_ptr(src) if src.size else None, _ptr(dst), src.size, cap)
    return dst[:n].tobytes()


def lz4_decompress(block: bytes, size: int):
    """The oracle's LZ4 block decoder: the bytes, or None for a malformed block."""
    L = lib()
    src = np.frombuffer(block, dtype=np.uint8)
    dst = np.zeros(max(size, 1), dtype=np.uint8)
    r = L.LZ4_decompress_safe(_ptr(src), _ptr(dst), src.size, size)
    return None if r < 0 else dst[:r].tobytes()


def dequantize_prediction_coding(width, height, m, index, table, packed, size):
    L = lib()
    out = np.zeros(max(size, 1), dtype=np.float32)
    b = np.ascontiguousarray(packed, dtype=np.uint8)
    L.oracle_dequantize_prediction_coding(width, height, m, _ptr(np.ascontiguousarray(index, dtype=np.uint32)),
                                          _ptr(np.ascontiguousarray(table, dtype=np.uint8)), _ptr(b), b.size,
                                          _ptr(out))
    return out[:size]


def unpack_codes(width, height, m, index, table, packed):
    """The integer codes of a packed prediction-coding stream (pack_bits, moment_quantization.cpp:92-114: LSB-first,
    pixels in row-major order, moment index ascending), one per stored moment; -1 for a code cut off by the
    dropped trailing partial byte."""
    idx = np.asarray(index, dtype=np.int64)
    counts = np.diff(idx)
    tab = np.asarray(table, dtype=np.int64)
    total = int(idx[-1])
    starts = np.repeat(idx[:-1], counts)
    l = np.arange(total, dtype=np.int64) - starts
    widths = tab[l]
    offs = np.zeros(total, dtype=np.int64)
    if total:
        offs[1:] = np.cumsum(widths)[:-1]
    bits = np.unpackbits(np.asarray(packed, dtype=np.uint8), bitorder="little").astype(np.int64)
    nbits = bits.size
    codes = np.zeros(total, dtype=np.int64)
    for k in range(int(tab.max()) if total else 0):
        pos = offs + k
        take = (k < widths) & (pos < nbits)
        codes[take] |= bits[pos[take]] << k
    codes[offs + widths > nbits] = -1
    return codes


def default_quantization_table(m, bits):
    return np.array([16] + [bits] * (m - 1), dtype=np.uint8)[:m]


class rounded_trig:
    """Within the block, the f32 prediction-coding dequantization takes correctly rounded cos / sin instead of the
    C library's cosf / sinf (for comparing a device implementation operation by operation)."""

    def __enter__(self):
        lib().oracle_set_rounded_trig(1)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_rounded_trig(0)


def sample_moment_image(width, height, index, data, s):
    """sample_moment_image(img, s, s) + compact on a compact image: returns (index[s*s+1], data)."""
    L = lib()
    idx = np.ascontiguousarray(index, dtype=np.uint32)
    d = np.ascontiguousarray(data, dtype=np.float32)
    s_index = np.zeros(s * s + 1, dtype=np.uint32)
    n = int(L.oracle_sample_moment_image(width, height, _ptr(idx), _ptr(d), s, _ptr(s_index), None))
    s_data = np.zeros(max(n, 1), dtype=np.float32)
    L.oracle_sample_moment_image(width, height, _ptr(idx), _ptr(d), s, _ptr(s_index), _ptr(s_data))
    return s_index, s_data[:n]


def _coding_params(cp, m):
    return None if cp is None else np.ascontiguousarray(cp, dtype=np.uint16)[:2 * (m - 1)]


def measure_idx_error(width, height, m, index, data, coding_warp, coding_params, idx, b, precision="f32",
                      nthreads=0):
    """measure_idx_error on a compact prediction-coded image: (mean rRMSE, per-pixel rRMSE of the non-empty
    pixels in row-major order) for moment idx quantized to b bits (idx < 0: nothing quantized)."""
    L = lib()
    dt = _dt(precision)
    idx_a = np.ascontiguousarray(index, dtype=np.uint32)
    d = np.ascontiguousarray(data, dtype=dt)
    cp = _coding_params(coding_params, m)
    errors = np.zeros(max(int(np.count_nonzero(np.diff(idx_a.astype(np.int64)))), 1), dtype=dt)
    size = C.c_uint32()
    mean = getattr(L, f"oracle_measure_idx_error_{precision}")(width, height, m, _ptr(idx_a), _ptr(d), coding_warp,
                                                               _ptr(cp), idx, b, _ptr(errors), C.byref(size),
                                                               nthreads)
    return float(mean), errors[:size.value]


def create_quantization_table(width, height, m, index, data, coding_warp, coding_params, start_bits,
                              precision="f32", nthreads=0):
    """create_quantization_table on a compact prediction-coded image: returns (table[m] u8, means[m, 32] of the
    evaluations the search made (NaN elsewhere), number of evaluations)."""
    L = lib()
    dt = _dt(precision)
    table = np.zeros(m, dtype=np.uint8)
    means = np.zeros((m, 32), dtype=dt)
    cp = _coding_params(coding_params, m)
    n = getattr(L, f"oracle_create_quantization_table_{precision}")(
        width, height, m, _ptr(np.ascontiguousarray(index, dtype=np.uint32)),
        _ptr(np.ascontiguousarray(data, dtype=dt)), coding_warp, _ptr(cp), start_bits, _ptr(table), _ptr(means),
        nthreads)
    return table, means, int(n)


def prepare_moments(width, height, m, index, data, prediction_code=False, coding_warp=0, coding_params=None,
                    bias=1e-6, precision="f32", nthreads=0, rows=None):
    """MomentImageHost::prepare_moments for every pixel; returns the Lagrange multipliers in the data layout."""
    L = lib()
    d = np.ascontiguousarray(data, dtype=_dt(precision))
    out = np.zeros(max(d.size, 1), dtype=_dt(precision))
    cp = None if coding_params is None else np.ascontiguousarray(coding_params, dtype=np.uint16)
    idx = None if index is None else np.ascontiguousarray(index, dtype=np.uint32)
    o = options(nthreads, rows)
    getattr(L, f"oracle_prepare_moments_{precision}")(width, height, m, _ptr(idx), _ptr(d), int(prediction_code),
                                                      coding_warp, _ptr(cp), bias, _ptr(out), C.byref(o))
    return out[:d.size]


def error_stream(error_type, percentile, values, precision="f32"):
    """ErrorMax / ErrorRMSE / ErrorPercentile (error_measures.h) fed update(0, v) for each value: error() after
    each update."""
    L = lib()
    v = np.ascontiguousarray(values, dtype=_dt(precision))
    out = np.zeros(v.size, dtype=_dt(precision))
    getattr(L, f"oracle_error_stream_{precision}")(int(error_type), int(percentile), v.size, _ptr(v), _ptr(out))
    return out


def ss_cache(light_cam, rp, width, height, m, dmin, dmax, index, pmoments, bounds, tf_table, precision="f32"):
    """reconstruct_single_scattering_cache, run sequentially: the transmittance cache of a light image's
    multipliers, float32[cache_size_z, cache_size_y, cache_size_x] over [dmin, dmax]."""
    L = lib()
    dt = _dt(precision)
    pm = np.ascontiguousarray(pmoments, dtype=dt)
    idx = None if index is None else np.ascontiguousarray(index, dtype=np.uint32)
    b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.uint16)
    t = np.ascontiguousarray(tf_table, dtype=dt)
    out = np.zeros((rp.ss.cache_size_z, rp.ss.cache_size_y, rp.ss.cache_size_x), dtype=np.float32)
    getattr(L, f"oracle_ss_cache_{precision}")(C.byref(light_cam), C.byref(rp), width, height, m,
                                               (C.c_float * 3)(*dmin), (C.c_float * 3)(*dmax), _ptr(idx), _ptr(pm),
                                               _ptr(b), _ptr(t), _ptr(out))
    return out


def _cache_option(o, cache):
    """cache = (values[z, y, x], dmin, dmax) or None; returns what must stay alive while the call runs."""
    if cache is None:
        return None
    g, keep = _grid(*cache)
    o.ss_cache = C.addressof(g)
    return g, keep


def reconstruct(cam, rp, width, height, m, dmin, dmax, index, pmoments, bounds, tf_table, precision="f32",
                nthreads=0, rows=None, exact_atan=False, tf_bspline=False, float_bounds=None, cache=None,
                density_offset=0.0):
    """reconstruct_host with float RGBA: returns rgba[H,W,4].  tf_bspline / float_bounds select the
    differentiation form (transfer-function row as a cubic B-spline in the front density, or with tf_bspline = 2
    linear in it; unquantized bounds[H,W,2]).  cache = (values[z, y, x], dmin, dmax): single scattering from that transmittance cache when
    rp.ss.enable.  density_offset (a scalar, or one value per pixel [H, W]) is added to every reconstructed density (a
    probe of the colour's sensitivity to the densities; 0 is the method)."""
    L = lib()
    dt = _dt(precision)
    pm = np.ascontiguousarray(pmoments, dtype=dt)
    idx = None if index is None else np.ascontiguousarray(index, dtype=np.uint32)
    b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.uint16)
    t = np.ascontiguousarray(tf_table, dtype=dt)
    out = np.zeros((height, width, 4), dtype=dt)
    o = options(nthreads, rows, exact_atan)
    o.tf_bspline = int(tf_bspline)
    bf = None if float_bounds is None else np.ascontiguousarray(float_bounds, dtype=dt)
    o.bounds_in = None if bf is None else bf.ctypes.data
    offs = None
    if np.ndim(density_offset) == 0:
        o.density_offset = float(density_offset)
    else:
        offs = np.ascontiguousarray(np.broadcast_to(density_offset, (height, width)), dtype=dt)
        o.density_offsets = offs.ctypes.data
    keep = _cache_option(o, cache)
    getattr(L, f"oracle_reconstruct_{precision}")(C.byref(cam), C.byref(rp), width, height, m,
                                                  (C.c_float * 3)(*dmin), (C.c_float * 3)(*dmax), _ptr(idx),
                                                  _ptr(pm), _ptr(b), _ptr(t), _ptr(out), C.byref(o))
    del keep
    return out


def reconstruct_error(cam, ep, volume, dmin, dmax, width, height, m, index, data, prediction_code=False,
                      coding_warp=0, coding_params=None, bounds=None, precision="f32", nthreads=0, rows=None,
                      particles=None):
    """reconstruct_error_host: per pixel the error measure of the MESE reconstruction against the volume (a grid,
    or ``particles`` when given).  Returns (errors[H,W] in the working precision, error bounds[H,W] u16)."""
    L = lib()
    dt = _dt(precision)
    g, keep = (_grid(volume, dmin, dmax) if particles is None else (None, None))
    idx = None if index is None else np.ascontiguousarray(index, dtype=np.uint32)
    d = np.ascontiguousarray(data, dtype=dt)
    cp = None if coding_params is None else np.ascontiguousarray(coding_params, dtype=np.uint16)
    b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.uint16)
    errors = np.zeros((height, width), dtype=dt)
    eb = np.zeros((height, width), dtype=np.uint16)
    o = options(nthreads, rows)
    getattr(L, f"oracle_reconstruct_error_{precision}")(
        C.byref(cam), C.byref(ep), C.byref(g) if g is not None else None,
        particles.handle if particles is not None else None, width, height, m, _ptr(idx), _ptr(d),
        int(prediction_code), int(coding_warp), _ptr(cp), _ptr(b), _ptr(errors), _ptr(eb), C.byref(o))
    del keep
    return errors, eb


def uncertainty_tf(tf1d, step_size, error_type, precision="f32"):
    """read_from_disk_uncertainty's table for a float 1D table: box filter (MAX_ERROR, ERROR_PERCENTILE) or
    Gaussian filter (RMSE); returns [256 (y), 256 (x), 4]."""
    L = lib()
    dt = _dt(precision)
    src = np.ascontiguousarray(tf1d, dtype=dt)
    out = np.zeros((256, 256, 4), dtype=dt)
    getattr(L, f"oracle_uncertainty_tf_{precision}")(_ptr(src), step_size, int(error_type), _ptr(out))
    return out


def reconstruct_uncertainty(cam, up, mode, width, height, m, dmin, dmax, index, data, error_bounds,
                            prediction_code=False, coding_warp=0, coding_params=None, bounds=None, table=None,
                            precision="f32", nthreads=0, rows=None):
    """reconstruct_uncertainty_interpolation (mode 0, ``table`` = the preintegrated row) or _convolution (mode 1,
    ``table`` = the 256 x 256 uncertainty table): float RGBA[H,W,4]."""
    L = lib()
    dt = _dt(precision)
    idx = None if index is None else np.ascontiguousarray(index, dtype=np.uint32)
    d = np.ascontiguousarray(data, dtype=dt)
    cp = None if coding_params is None else np.ascontiguousarray(coding_params, dtype=np.uint16)
    b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.uint16)
    eb = np.ascontiguousarray(error_bounds, dtype=np.uint16)
    t = np.ascontiguousarray(table, dtype=dt)
    out = np.zeros((height, width, 4), dtype=dt)
    o = options(nthreads, rows)
    getattr(L, f"oracle_reconstruct_uncertainty_{precision}")(
        C.byref(cam), C.byref(up), int(mode), width, height, m, (C.c_float * 3)(*dmin), (C.c_float * 3)(*dmax),
        _ptr(idx), _ptr(d), int(prediction_code), int(coding_warp), _ptr(cp), _ptr(b), _ptr(eb), _ptr(t), _ptr(out),
        C.byref(o))
    return out


def generate_reference(cam, rp, volume, dmin, dmax, width, height, tf_table, precision="f32", nthreads=0,
                       rows=None, particles=None, cache=None):
    """reference_host: direct volume rendering of the volume (a grid, or ``particles`` when given) with the
    preintegrated row; float RGBA[H,W,4].  cache = (values[z, y, x], dmin, dmax): the single-scattering
    transmittance from that cache instead of the brute-force march (generate_reference_reconstructed_ss)."""
    L = lib()
    dt = _dt(precision)
    g, keep = (_grid(volume, dmin, dmax) if particles is None else (None, None))
    t = np.ascontiguousarray(tf_table, dtype=dt)
    out = np.zeros((height, width, 4), dtype=dt)
    o = options(nthreads, rows)
    keep_cache = _cache_option(o, cache)
    getattr(L, f"oracle_generate_reference_{precision}")(
        C.byref(cam), C.byref(rp), C.byref(g) if g is not None else None,
        particles.handle if particles is not None else None, width, height, _ptr(t), _ptr(out), C.byref(o))
    del keep, keep_cache
    return out


def ref_from_rec(rp):
    """ref_from_rec_params (parameters.h:379-390)."""
    from mray_gb300.types import ReferenceParameters

    return ReferenceParameters(step_size=rp.step_size, medium_emission=rp.medium_emission,
                               medium_scattering=rp.medium_scattering, early_ray_termination=rp.early_ray_termination,
                               data_min=rp.data_min, data_max=rp.data_max, ss=rp.ss)


def tf_sample_diff(tf_table, fs, linear=False, precision="f64"):
    """The differentiation form's transfer-function row at front density fs: the cubic B-spline or (linear) the
    GPU texture's linear interpolation, both at the texel centres u = 256 fs - 1/2; RGBA."""
    L = lib()
    t = np.ascontiguousarray(tf_table, dtype=_dt(precision)).reshape(-1)
    out = np.zeros(4, dtype=_dt(precision))
    getattr(L, f"oracle_tf_sample_{'linear' if linear else 'bspline'}_{precision}")(_ptr(t), fs, _ptr(out))
    return out


def preintegrate(tf1d, step_size):
    L = lib()
    src = np.ascontiguousarray(tf1d, dtype=np.float32)
    out = np.zeros((256, 4), dtype=np.float32)
    L.oracle_preintegrate(_ptr(src), step_size, _ptr(out))
    return out


def rgba_to_u8(rgba):
    L = lib()
    src = np.ascontiguousarray(rgba, dtype=np.float32)
    out = np.zeros(src.shape, dtype=np.uint8)
    L.oracle_rgba_to_u8(src.size // 4, _ptr(src), _ptr(out))
    return out


def generate(cam, gp, volume, dmin, dmax, width, height, m, precision="f32", nthreads=0):
    """The whole reference ``generate()`` on the CPU (moment_raymarcher.cpp:121-166): per-pixel moments, counts,
    compaction and prediction coding as the parameters ask.  Returns a dict like a MomentImageHost."""
    moments, bounds, counts = generate_moments(cam, gp, volume, dmin, dmax, width, height, m, precision, nthreads)
    res = {"width": width, "height": height, "num_moments": m, "bounds": bounds if gp.transform_to_bounds else None,
           "raw_moments": moments, "counts": counts, "is_compact": bool(gp.compact_image),
           "prediction_code": False, "coding_warp": int(gp.coding_warp), "coding_params": None}
    if gp.compact_image:
        index, data = compact(counts, moments.astype(np.float32))
        res["index"], res["data"] = index, data
        if gp.prediction_coding:
            d, cp = prediction_encode(width, height, m, index, data, gp.coding_warp, gp.bias, nthreads)
            res["data"], res["prediction_code"] = d, True
            res["coding_params"] = cp if gp.coding_warp == 0 else None
    else:
        res["index"], res["data"] = None, moments.reshape(-1)
    return res


def workload_generate(wl, precision="f32", nthreads=0):
    return generate(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width, wl.height,
                    wl.num_moments, precision, nthreads)


def workload_reconstruct(wl, mi, precision="f32", nthreads=0, exact_atan=False):
    """prepare + MESE re-march of a moment image from :func:`generate`."""
    tf = preintegrate(wl.tf1d, wl.tf_step)
    pm = prepare_moments(wl.width, wl.height, wl.num_moments, mi["index"], mi["data"], mi["prediction_code"],
                         mi["coding_warp"], mi["coding_params"], wl.rec.bias, precision, nthreads)
    return reconstruct(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                       mi["index"], pm, mi["bounds"], tf, precision, nthreads, exact_atan=exact_atan)


def preintegrate_r(tf1d, step_size, precision="f64"):
    """The preintegrated row (rgb a s, a s) in the working precision (float: the reference's own arithmetic)."""
    if precision == "f32":
        return preintegrate(tf1d, step_size)
    t = np.asarray(tf1d, dtype=np.float64)
    w = t[:, 3] * float(step_size)
    return np.concatenate([t[:, :3] * w[:, None], w[:, None]], axis=1)


def diff_forward(cam, gp, rp, volume, dmin, dmax, width, height, m, tf_table, precision="f64", nthreads=0,
                 exact_atan=True, rows=None, tf_linear=False):
    """The differentiation form's forward on the CPU: generate without compaction, unquantized bounds,
    Lagrange multipliers, re-march with exact atan and the transfer-function row as a cubic B-spline in the
    front density (with tf_linear: linear in it, the GPU texture's sampling with exact weights).  Returns
    rgba[H,W,4] in the working precision; with rows = (begin, end, step) only those rows (the others stay zero)."""
    moments, _, _, bf = generate_moments(cam, gp, volume, dmin, dmax, width, height, m, precision, nthreads,
                                         rows=rows, float_bounds=True)
    pm = prepare_moments(width, height, m, None, moments.reshape(-1), False, 1, None, rp.bias, precision, nthreads,
                         rows=rows)
    return reconstruct(cam, rp, width, height, m, dmin, dmax, None, pm, None, tf_table, precision, nthreads,
                       rows=rows, exact_atan=exact_atan, tf_bspline=2 if tf_linear else 1, float_bounds=bf)
