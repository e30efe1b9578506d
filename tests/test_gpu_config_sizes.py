"""Parity at the configurations' own sizes.

* Configuration 1 in full (64^3 Marschner-Lobb, 512^2 orthographic, 31 moments), through the drop-in host API,
  against the oracle's whole image: bounds and compaction index exact, moments within 1e-4 (the bar of
  test_gpu_path.py), the colour of every pixel held to the RGBA bar, and, with prediction coding and 10-bit codes,
  the end-to-end code figures against the codes of the FP64 moments.
* Configuration 2 (512^3 mixing layer, 1024^2 perspective, 64 moments) on 2048 sampled pixels (16 rows x 128
  columns): the GPU renders the whole image, the oracle the sampled pixels.

RGBA bar per pixel (helpers.rgba_agreement): within 1e-3 of the reference's FP32 colour, or at least as close to the
FP64 evaluation of the same method as the reference's own FP32 colour is.
"""
import numpy as np
import pytest

import oracle as O
from helpers import moment_rel_err, rgba_agreement

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RGBA_TOL = 1e-3


def _config1(prediction_coding=False):
    from mray_gb300 import workloads as W

    wl = W.ml_workload(n=64, width=512, height=512, num_moments=31, seed=11)
    wl.gen.prediction_coding = 1 if prediction_coding else 0
    return wl


def _fp64_image(wl, rows=None, cols=None):
    """FP64 evaluation of the same method: moments, compaction of them, multipliers and re-march in double."""
    W, H, m = wl.width, wl.height, wl.num_moments
    gen = wl.gen
    m64, b64, c64 = O.generate_moments(wl.camera, gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f64",
                                       rows=rows, cols=cols)
    idx64, _ = O.compact(c64, m64.astype(np.float32))
    data64 = m64.reshape(-1, m)[c64.reshape(-1) > 0].reshape(-1)
    pm64 = O.prepare_moments(W, H, m, idx64, data64, False, 1, None, wl.rec.bias, "f64", rows=rows)
    rgba64 = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx64, pm64, b64,
                           O.preintegrate(wl.tf1d, wl.tf_step), "f64", rows=rows)
    return m64, b64, c64, rgba64


def test_config1_full_image(gpu_context):
    import mray_gb300 as M

    wl = _config1()
    W, H, m = wl.width, wl.height, wl.num_moments
    gpu_context.precision = M.PRECISION_FP32
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(W, H, m, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    img = M.ColorImageHost(W, H)
    M.reconstruct(wl.camera, mi, M.preintegrate(wl.tf1d, wl.tf_step), img, wl.rec, context=gpu_context)

    ref = O.workload_generate(wl, "f32")
    assert np.array_equal(mi.index, ref["index"])
    assert np.array_equal(mi.bounds.reshape(-1), ref["bounds"].reshape(-1))
    counts = np.diff(ref["index"].astype(np.int64)).reshape(H, W)
    ours = np.zeros((H, W, m), np.float32)
    theirs = np.zeros_like(ours)
    for arr, src in ((ours, mi.data), (theirs, ref["data"])):
        arr.reshape(-1, m)[counts.reshape(-1) > 0] = src.reshape(-1, m)
    m64, b64, _, rgba64 = _fp64_image(wl)
    hit = counts > 0
    own = moment_rel_err(theirs, m64, m64[..., 0])
    err = moment_rel_err(ours, theirs, theirs[..., 0])
    assert np.all(err[hit] <= 1e-4 + own[hit]), f"max excess {(err - own)[hit].max():.3e}"
    rgba32 = O.workload_reconstruct(wl, ref, "f32")
    ok = rgba_agreement(img.rgba_float, rgba32, rgba64, RGBA_TOL)
    diff = np.abs(img.rgba_float.astype(np.float64) - rgba32).max(axis=-1)
    print(f"config 1, {W}x{H}: max |dRGBA| vs reference FP32 {diff.max():.2e}, pixels outside the bar "
          f"{int((~ok).sum())} of {ok.size}")
    assert ok.all(), f"{int((~ok).sum())} pixels outside the RGBA bar"


def test_config1_prediction_coded_codes_end_to_end(gpu_context):
    """Volume -> 10-bit codes at configuration 1's full size: the fraction of codes that differ from the
    reference's, and from the codes of the FP64 moments (encoded with the reference's FP32 arithmetic)."""
    import mray_gb300 as M

    wl = _config1(prediction_coding=True)
    W, H, m = wl.width, wl.height, wl.num_moments
    gpu_context.precision = M.PRECISION_FP32
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(W, H, m, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    table = M.default_quantization_table(m, 10)
    codes = M.quantize_prediction_coding(mi, table, context=gpu_context)
    ref = O.workload_generate(wl, "f32")
    assert np.array_equal(mi.index, ref["index"])
    codes_ref = O.quantize_prediction_coding(W, H, m, ref["index"], ref["data"], table)
    m64, b64, _ = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f64")
    counts = np.diff(ref["index"].astype(np.int64))
    data64 = m64.reshape(-1, m)[counts > 0].reshape(-1).astype(np.float32)
    enc64, _ = O.prediction_encode(W, H, m, ref["index"], data64, 0, wl.gen.bias)
    codes_exact = O.quantize_prediction_coding(W, H, m, ref["index"], enc64, table)
    a, b, e = (O.unpack_codes(W, H, m, ref["index"], table, c) for c in (codes, codes_ref, codes_exact))
    same = np.repeat(np.all(b64.reshape(-1, 2) == ref["bounds"].reshape(-1, 2), axis=-1), counts)
    ours_vs_ref = float(np.mean(a != b))
    ours_vs_exact = float(np.mean((a != e)[same]))
    ref_vs_exact = float(np.mean((b != e)[same]))
    print(f"config 1 10-bit codes ({a.size}): ours vs reference {ours_vs_ref:.3%}, ours vs exact {ours_vs_exact:.3%}, "
          f"reference vs exact {ref_vs_exact:.3%}")
    assert ours_vs_exact <= ref_vs_exact + 0.002


def test_config2_sampled_pixels(gpu_context):
    import mray_gb300 as M
    from mray_gb300 import workloads as W_

    wl = W_.mixing_layer_workload(n=512, width=1024, height=1024, num_moments=64, modes=64, seed=21)
    W, H, m = wl.width, wl.height, wl.num_moments
    P = W * H
    rows, cols = (0, H, H // 16), (0, W, W // 128)
    gpu_context.precision = M.PRECISION_FP32
    gpu_context.upload_grid(torch.from_numpy(wl.volume).cuda(), wl.domain_min, wl.domain_max)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf)
    d_mo = torch.zeros(P * m, device="cuda")
    d_b = torch.zeros(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.zeros(P, dtype=torch.int32, device="cuda")
    d_idx = torch.zeros(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.zeros(P * m, device="cuda")
    d_pm = torch.zeros(P * m, device="cuda")
    d_rgba = torch.zeros(P * 4, device="cuda")
    gpu_context.stage_generate_moments(wl.camera, wl.gen, W, H, m, d_mo, d_b, d_c)
    gpu_context.stage_compact(W, H, m, d_c, d_mo, d_idx, d_cm)
    gpu_context.stage_prepare_moments(W, H, m, d_idx, d_cm, d_pm, bias=wl.rec.bias)
    gpu_context.stage_reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
    gpu_context.synchronize()
    sel = np.zeros((H, W), bool)
    sel[rows[0]:rows[1]:rows[2], cols[0]:cols[1]:cols[2]] = True
    mo = d_mo.cpu().numpy().reshape(H, W, m)
    b = d_b.cpu().numpy().view(np.uint16).reshape(H, W, 2)
    c = d_c.cpu().numpy().view(np.uint32).reshape(H, W)
    rgba = d_rgba.cpu().numpy().reshape(H, W, 4)

    m32, b32, c32 = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f32",
                                       rows=rows, cols=cols)
    assert np.array_equal(b[sel], b32[sel]) and np.array_equal(c[sel], c32[sel])
    m64, b64, c64, rgba64 = _fp64_image(wl, rows, cols)
    hit = sel & (c32 > 0)
    same = hit & np.all(b32 == b64, axis=-1)
    err64 = moment_rel_err(mo, m64, m64[..., 0])[same]
    assert err64.max() <= 1e-4, f"max rel err vs f64 {err64.max():.3e}"
    # the reference's FP32 colours of the sampled pixels, from its own moments of those pixels
    idx32, _ = O.compact(c32, m32)
    data32 = m32.reshape(-1, m)[c32.reshape(-1) > 0].reshape(-1)
    pm32 = O.prepare_moments(W, H, m, idx32, data32, False, 1, None, wl.rec.bias, "f32", rows=rows)
    rgba32 = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx32, pm32, b32, tf, "f32",
                           rows=rows)
    ok = rgba_agreement(rgba[sel], rgba32[sel], rgba64[sel], RGBA_TOL)
    d64 = np.abs(rgba[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    d32 = np.abs(rgba32[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    print(f"config 2 sampled: vs FP64 ours max {d64.max():.2e} rms {np.sqrt((d64 ** 2).mean()):.2e}; reference FP32 "
          f"max {d32.max():.2e} rms {np.sqrt((d32 ** 2).mean()):.2e}; outside the bar {int((~ok).sum())} of {ok.size}")
    assert ok.all()
