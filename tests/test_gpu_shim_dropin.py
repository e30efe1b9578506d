"""The drop-in through the reference's own caller.

oracle/Makefile `shim` compiles the reference's CPU sources with CUDA_SUPPORT, so that its generate() and
reconstruct() (moment_raymarcher.cpp:168-183, 329-337) dispatch to generate_device / reconstruct_device, and links
the shim mray_gb300/shim/moment_raymarcher_gb300.cpp (those two functions over the C ABI) and libmraygb.so in place
of the reference's moment_raymarcher.cu.  The reference's own harness entry points (ref_generate_grid: generate()
into the MomentImageHost that main.cpp builds; ref_reconstruct_u8: reconstruct() into a ColorImageHost) then run
the GPU path exactly as the reference's CLI would.  Bar: the same bytes as the ctypes path (mray_gb300.generate /
reconstruct) on the same inputs -- the seam adds nothing and loses nothing.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import small_mixing, small_ml

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE, "_ref", "libmrayref_shim.so")


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


@pytest.fixture(scope="module")
def shim_lib():
    from stage_reference import reference_src

    src = reference_src()
    if src is None:
        pytest.skip("the reference's sources are not staged")
    jobs = str(min(16, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-j", jobs, "-C", ORACLE, "shim", f"REF={src}"], check=True)
    L = C.CDLL(LIB)
    L.ref_generate_grid.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                    C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_reconstruct_u8.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_uint64, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
    return L


def _through_reference(L, wl):
    """generate() and reconstruct() of the reference's own code, dispatching to the shim."""
    import mray_gb300 as M

    W, H, m = wl.width, wl.height, wl.num_moments
    vol = np.ascontiguousarray(wl.volume, dtype=np.float32)
    nz, ny, nx = vol.shape
    dmin = np.asarray(wl.domain_min, np.float32)
    dmax = np.asarray(wl.domain_max, np.float32)
    data = np.zeros(W * H * m, np.float32)
    index = np.zeros(W * H + 1, np.uint32)
    bounds = np.zeros(2 * W * H, np.uint16)
    cp = np.zeros(2 * m, np.uint16)
    size = C.c_uint64()
    flags = np.zeros(4, np.int32)
    L.ref_generate_grid(C.byref(wl.camera), C.byref(wl.gen), _p(vol), nx, ny, nz, _p(dmin), _p(dmax), W, H, m,
                        _p(data), _p(index), _p(bounds), _p(cp), C.byref(size), _p(flags))
    data = data[:size.value].copy()
    pc = int(flags[1])
    tf = M.preintegrate(wl.tf1d, wl.tf_step).table.astype(np.float32)
    u8 = np.zeros((H, W, 4), np.uint8)
    L.ref_reconstruct_u8(C.byref(wl.camera), C.byref(wl.rec), W, H, m, _p(index), _p(data), data.size, _p(bounds), pc,
                         int(flags[2]), _p(cp if pc else None), _p(dmin), _p(dmax), _p(tf), _p(u8))
    return dict(data=data, index=index, bounds=bounds.reshape(-1, 2), coding_params=cp[:2 * (m - 1)], flags=flags,
                rgba8=u8)


def _through_ctypes(ctx, wl):
    import mray_gb300 as M

    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(wl.width, wl.height, wl.num_moments, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=ctx)
    img = M.ColorImageHost(wl.width, wl.height)
    M.reconstruct(wl.camera, mi, M.preintegrate(wl.tf1d, wl.tf_step), img, wl.rec, context=ctx)
    return mi, img


@pytest.mark.parametrize("case", ["ml-m31", "ml-m31-pc", "mixing-m64-pc"])
def test_generate_and_reconstruct_through_the_reference_caller(shim_lib, gpu_context, case):
    import mray_gb300 as M

    wl = small_ml(96, 80, 31) if case.startswith("ml") else small_mixing(64, 48, 64, 96)
    wl.gen.prediction_coding = 1 if case.endswith("pc") else 0
    gpu_context.precision = M.PRECISION_FP32
    ref = _through_reference(shim_lib, wl)
    mi, img = _through_ctypes(gpu_context, wl)
    assert bool(ref["flags"][0]) == mi.is_compact and bool(ref["flags"][1]) == mi.prediction_code
    assert np.array_equal(ref["index"], mi.index)
    assert np.array_equal(ref["bounds"], mi.bounds.reshape(-1, 2))
    assert np.array_equal(ref["data"].view(np.uint32), mi.data.view(np.uint32))
    if mi.prediction_code:
        assert np.array_equal(ref["coding_params"], mi.coding_params)
    assert np.array_equal(ref["rgba8"], img.rgba)
