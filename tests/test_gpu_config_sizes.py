"""Parity at the configurations' own sizes.

* Configuration 1 in full (64^3 Marschner-Lobb, 512^2 orthographic, 31 moments), through the drop-in host API,
  against the oracle's whole image: bounds and compaction index exact, moments within 1e-4 (the bar of
  test_gpu_path.py), the colour of every pixel held to the RGBA bar, and, with prediction coding and 10-bit codes,
  the end-to-end code figures against the codes of the FP64 moments.
* Configuration 2 (512^3 mixing layer, 1024^2 perspective, 64 moments) on 2048 sampled pixels (16 rows x 128
  columns): the GPU renders the whole image, the oracle the sampled pixels.
* Configuration 3 (256^3 Marschner-Lobb, 512^2, 31 moments, the differentiation form): the adjoint of the L2 loss
  against central differences of the FP64 oracle (loss over 8 sampled rows) and of the GPU forward (whole image).
* Configuration 5 (16M SPH particles, 256^3 cells, 1024^2, 64 moments) on 16 sampled rows.

RGBA bar per pixel (helpers.rgba_agreement), met by every pixel: within 1e-3 of the reference's FP32 colour; or at
least as close to the FP64 evaluation of the same method as the reference's own FP32 colour is; or within 1e-3 plus
the FP64 colour's change under a +-1e-5 shift of all densities (pixels on a jump of the reference's transfer-function
lookup).
"""
import numpy as np
import pytest

import oracle as O
from helpers import fp32_density_bound, fp64_sensitivity, moment_rel_err, rgba_agreement

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RGBA_TOL = 1e-3


def _config1(prediction_coding=False):
    from mray_gb300 import workloads as W

    wl = W.ml_workload(n=64, width=512, height=512, num_moments=31, seed=11)
    wl.gen.prediction_coding = 1 if prediction_coding else 0
    return wl


def _fp64_image(wl, rows=None, cols=None, sensitivity=False):
    """FP64 evaluation of the same method: moments, compaction of them, multipliers and re-march in double (and, when
    asked, the colour's sensitivity to a +-1e-5 shift of the densities, helpers.fp64_sensitivity)."""
    W, H, m = wl.width, wl.height, wl.num_moments
    gen = wl.gen
    m64, b64, c64 = O.generate_moments(wl.camera, gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f64",
                                       rows=rows, cols=cols)
    idx64, _ = O.compact(c64, m64.astype(np.float32))
    data64 = m64.reshape(-1, m)[c64.reshape(-1) > 0].reshape(-1)
    pm64 = O.prepare_moments(W, H, m, idx64, data64, False, 1, None, wl.rec.bias, "f64", rows=rows)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    rgba64 = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx64, pm64, b64, tf, "f64",
                           rows=rows)
    if not sensitivity:
        return m64, b64, c64, rgba64
    sens = fp64_sensitivity(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx64, pm64, b64, tf, rows)
    return m64, b64, c64, rgba64, sens


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
    m64, b64, _, rgba64, sens = _fp64_image(wl, sensitivity=True)
    hit = counts > 0
    own = moment_rel_err(theirs, m64, m64[..., 0])
    err = moment_rel_err(ours, theirs, theirs[..., 0])
    assert np.all(err[hit] <= 1e-4 + own[hit]), f"max excess {(err - own)[hit].max():.3e}"
    rgba32 = O.workload_reconstruct(wl, ref, "f32")
    ok = rgba_agreement(img.rgba_float, rgba32, rgba64, RGBA_TOL, sens)
    plain = rgba_agreement(img.rgba_float, rgba32, rgba64, RGBA_TOL)
    diff = np.abs(img.rgba_float.astype(np.float64) - rgba32).max(axis=-1)
    print(f"config 1, {W}x{H}: max |dRGBA| vs reference FP32 {diff.max():.2e}; pixels held only by the "
          f"transfer-function jump clause {int((ok & ~plain).sum())} of {ok.size}")
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
    m64, b64, c64, rgba64, sens = _fp64_image(wl, rows, cols, sensitivity=True)
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
    ok = rgba_agreement(rgba[sel], rgba32[sel], rgba64[sel], RGBA_TOL, sens[sel])
    d64 = np.abs(rgba[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    d32 = np.abs(rgba32[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    print(f"config 2 sampled: vs FP64 ours max {d64.max():.2e} rms {np.sqrt((d64 ** 2).mean()):.2e}; reference FP32 "
          f"max {d32.max():.2e} rms {np.sqrt((d32 ** 2).mean()):.2e}; outside the bar {int((~ok).sum())} of {ok.size}")
    assert ok.all()


def _config3():
    from mray_gb300 import workloads as W

    return W.diff_workload(n=256, width=512, height=512, num_moments=31)


def test_config3_adjoint_against_fp64_central_differences(gpu_context):
    """Configuration 3 (256^3 Marschner-Lobb, 512^2, 31 moments, L2 loss against a target rendered with the
    perturbed transfer function), the loss taken over every 64th row (8 rows of 512 pixels, which the FP64 oracle
    renders in well under a second): the GPU adjoint, fed the FP64 forward's residual on those rows, against central
    differences (eps = 2^-10, about 1e-3, Richardson-combined with 2 eps) of the FP64 oracle on 32 seeded parameters
    (16 transfer-function entries, 16 voxels).  Bar: 1e-3 relative per parameter."""
    from helpers import GpuRender, pick_parameters, richardson

    wl, target_tf = _config3()
    W, H, m = wl.width, wl.height, wl.num_moments
    rows = (0, H, 64)
    table = O.preintegrate(wl.tf1d, wl.tf_step).astype(np.float64)
    R = GpuRender(gpu_context, wl)
    target = R.forward(wl.volume, O.preintegrate(target_tf, wl.tf_step))
    sel = np.zeros((H, W, 1), bool)
    sel[rows[0]:rows[1]:rows[2]] = True

    def fwd64(v, t):
        return O.diff_forward(wl.camera, wl.gen, wl.rec, v, wl.domain_min, wl.domain_max, W, H, m, t, "f64",
                              rows=rows)

    rgba64 = fwd64(wl.volume, table)
    R.forward(wl.volume, table)
    gtf, gvol = R.backward(np.where(sel, 2.0 * (rgba64 - target), 0.0))
    params = pick_parameters(np.random.default_rng(31), gvol, gtf, 16, 16)

    def loss(v, t):
        return float((np.where(sel, fwd64(v, t) - target, 0.0) ** 2).sum())

    fd = np.array([richardson(loss, wl, table, kind, idx, 2.0 ** -10) for kind, idx in params])
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    rel = np.abs(ad - fd) / np.abs(fd)
    print(f"config 3 adjoint vs FP64 central differences: max rel err {rel.max():.2e} over {len(params)} parameters")
    assert rel.max() <= 1e-3, f"max rel err {rel.max():.3e} at {params[int(rel.argmax())]}"


def test_config3_adjoint_against_gpu_central_differences(gpu_context):
    """Configuration 3 on the whole image: the adjoint of the L2 loss against central differences (eps = 1e-3,
    Richardson-combined with 2 eps) of the FP32 GPU forward itself, on 16 seeded transfer-function entries whose
    gradient is at least a tenth of the largest.  A table entry moves every pixel's colour the same way, so the FP32
    forward's own rounding averages out of L(p + eps) - L(p - eps).  A single voxel moves a few rays by about as much
    as the FP32 forward's rounding does (up to 1e-3 of RGBA through the MESE reconstruction), so voxels are checked
    against the FP64 oracle's differences above.  Tolerance 1e-2."""
    from helpers import GpuRender, richardson

    wl, target_tf = _config3()
    table = O.preintegrate(wl.tf1d, wl.tf_step).astype(np.float64)
    R = GpuRender(gpu_context, wl)
    target = R.forward(wl.volume, O.preintegrate(target_tf, wl.tf_step))
    rgba = R.forward(wl.volume, table)
    gtf, _ = R.backward(2.0 * (rgba - target), volume_grad=False)
    rng = np.random.default_rng(37)
    tf_ok = np.argwhere(np.abs(gtf) > 0.1 * np.abs(gtf).max())
    params = [("tf", tuple(tf_ok[i])) for i in rng.choice(len(tf_ok), min(16, len(tf_ok)), replace=False)]

    def loss(v, t):
        return ((R.forward(v, t) - target) ** 2).sum()

    fd = np.array([richardson(loss, wl, table, kind, idx, 1e-3) for kind, idx in params])
    ad = np.array([gtf[idx] for _, idx in params])
    rel = np.abs(ad - fd) / np.abs(fd)
    print(f"config 3 adjoint vs FP32 GPU central differences: max rel err {rel.max():.2e} over {len(params)} "
          f"transfer-function entries")
    assert rel.max() <= 1e-2, f"max rel err {rel.max():.3e} at {params[int(rel.argmax())]}"


def _colour(wl, mo, bo, co, precision, rows, sensitivity=False, delta=1e-5):
    """Compaction, multipliers and re-march of the given moments in the given precision on the sampled rows (and,
    when asked, the FP64 colour's sensitivity to a +-delta shift of the densities, delta a scalar or per pixel)."""
    W, H, m = wl.width, wl.height, wl.num_moments
    idx, _ = O.compact(co, mo.astype(np.float32))
    data = mo.reshape(-1, m)[co.reshape(-1) > 0].reshape(-1)
    pm = O.prepare_moments(W, H, m, idx, data, False, 1, None, wl.rec.bias, precision, rows=rows)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    rgba = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx, pm, bo, tf, precision,
                         rows=rows)
    if not sensitivity:
        return rgba
    return rgba, fp64_sensitivity(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, idx, pm, bo, tf, rows,
                                  delta=delta)


def test_config5_sph_sampled_rows(gpu_context):
    """Configuration 5 (16M SPH particles: 70 % uniform, 30 % in 200 Gaussian clusters; one smoothing length 1/256,
    so 256^3 cells; 1024^2 perspective, 64 moments) on every 64th row (16 rows of 1024 pixels): the GPU bins the
    particles and renders the whole image, the oracle bins them the reference's way and renders the sampled rows.
    Bars: bounds and counts exact; moments within 1e-4 of the reference's FP32 moments widened by its own FP32 error,
    and no further from the FP64 oracle than that; every sampled pixel's colour within the RGBA bar, its jump clause
    with a density shift of the size of the FP32 errors of the moments and of the MESE series."""
    import mray_gb300 as M
    from mray_gb300 import workloads as W_

    wl = W_.sph_cluster_workload()
    W, H, m = wl.width, wl.height, wl.num_moments
    P = W * H
    rows = (0, H, 64)
    gpu_context.precision = M.PRECISION_FP32
    gpu_context.upload_particles(*[torch.from_numpy(a).cuda() for a in (wl.x, wl.y, wl.z, wl.v)], wl.h,
                                 wl.domain_min, wl.domain_max)
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
    sel[rows[0]:rows[1]:rows[2]] = True
    mo = d_mo.cpu().numpy().reshape(H, W, m)
    b = d_b.cpu().numpy().view(np.uint16).reshape(H, W, 2)
    c = d_c.cpu().numpy().view(np.uint32).reshape(H, W)
    rgba = d_rgba.cpu().numpy().reshape(H, W, 4)

    parts = O.ParticleSet(wl.x, wl.y, wl.z, wl.v, wl.h, wl.domain_min, wl.domain_max)
    m32, b32, c32 = O.generate_moments_particles(wl.camera, wl.gen, parts, W, H, m, "f32", rows=rows)
    m64, b64, c64 = O.generate_moments_particles(wl.camera, wl.gen, parts, W, H, m, "f64", rows=rows)
    del parts
    assert np.array_equal(b[sel], b32[sel]) and np.array_equal(c[sel], c32[sel])
    hit = sel & (c32 > 0)
    assert hit.sum() > 1000
    own = moment_rel_err(m32, m64, m64[..., 0])
    err = moment_rel_err(mo, m32, m32[..., 0])
    assert np.all(err[hit] <= 1e-4 + own[hit]), f"max excess {(err - own)[hit].max():.3e}"
    # against FP64: no further from it than the reference's FP32 moments are, plus 1e-4 (the particle densities
    # themselves are FP32 sums of up to hundreds of kernel weights, about 3e-4 off in the reference's arithmetic)
    same = hit & np.all(b32 == b64, axis=-1)
    err64 = moment_rel_err(mo, m64, m64[..., 0])
    assert np.all(err64[same] <= 1e-4 + own[same]), f"max excess vs f64 {(err64 - own)[same].max():.3e}"
    # The jump clause of the RGBA bar with a density shift per pixel of the larger of: our moments' distance from
    # FP64 (relative to m_0, times the density span), and how far any FP32 evaluation of the MESE series can move
    # the density (helpers.fp32_density_bound from the reference's FP32 multipliers: ~1e-5 on most pixels, up to
    # a few 1e-2 on the 1 % whose multipliers reach 1e4 and cancel).
    span = (b64[..., 1].astype(np.float64) - b64[..., 0]) / 65535.0
    idx32, _ = O.compact(c32, m32)
    pm32 = O.prepare_moments(W, H, m, idx32, m32.reshape(-1, m)[c32.reshape(-1) > 0].reshape(-1), False, 1, None,
                             wl.rec.bias, "f32", rows=rows)
    delta = np.maximum(fp32_density_bound(W, H, m, idx32, pm32, b32), np.where(same, err64 * span, 0.0))
    err64, own64 = err64[same], own[same]
    rgba32 = _colour(wl, m32, b32, c32, "f32", rows)
    rgba64, sens = _colour(wl, m64, b64, c64, "f64", rows, sensitivity=True, delta=delta)
    ok = rgba_agreement(rgba[sel], rgba32[sel], rgba64[sel], RGBA_TOL, sens[sel])
    d64 = np.abs(rgba[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    d32 = np.abs(rgba32[sel].astype(np.float64) - rgba64[sel]).max(axis=-1)
    print(f"config 5 sampled ({int(hit.sum())} rays hit): moments vs FP64 ours max {err64.max():.2e}, reference FP32 "
          f"max {own64.max():.2e}; RGBA vs FP64 ours "
          f"max {d64.max():.2e} rms {np.sqrt((d64 ** 2).mean()):.2e}, reference FP32 max {d32.max():.2e} rms "
          f"{np.sqrt((d32 ** 2).mean()):.2e}; outside the bar {int((~ok).sum())} of {ok.size}")
    assert ok.all()
