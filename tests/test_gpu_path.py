"""GPU parity of the moment-image path against the oracle (the reference's CPU method restated, f32 bit-exact
with the reference's own build; f64 the same method in double).

Tolerances (from the target of the build): moments within 1e-4 relative (per pixel, relative to m_0), RGBA
within 1e-3 absolute per channel, integer outputs (bounds, counts, index) exact.
"""
import numpy as np
import pytest

import oracle as O
from helpers import (fp32_density_bound, fp64_sensitivity, moment_rel_err, moments_bounds_agree, rgba_agreement,
                     small_mixing, small_ml)

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MOMENT_TOL = 1e-4
RGBA_TOL = 1e-3


def _dev(a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _gpu_moments(ctx, wl, precision=0):
    import mray_gb300 as M

    ctx.precision = precision
    ctx.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    W, H, m = wl.width, wl.height, wl.num_moments
    mo = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
    b = torch.zeros(2 * W * H, dtype=torch.int16, device="cuda")
    c = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    ctx.stage_generate_moments(wl.camera, wl.gen, W, H, m, mo, b, c)
    ctx.synchronize()
    ctx.precision = M.PRECISION_FP32
    return (mo.cpu().numpy().reshape(H, W, m), b.cpu().numpy().view(np.uint16).reshape(H, W, 2),
            c.cpu().numpy().view(np.uint32).reshape(H, W))


CASES = [
    dict(kind="ml", width=96, height=80, m=31, seed=11),
    dict(kind="ml", width=64, height=48, m=8, seed=5),
    dict(kind="ml", width=40, height=40, m=1, seed=3),
    dict(kind="ml", width=33, height=17, m=64, seed=9),
    dict(kind="mix", width=48, height=40, m=64, n=96, seed=21),
    # beyond 64 moments, up to the reference's limit of 255 (main.cpp:288-293): the 32- and 64-moment-per-lane
    # generate instances and the 128- and 256-entry preparation and re-march instances
    dict(kind="mix", width=24, height=20, m=128, n=64, seed=23),
    dict(kind="mix", width=20, height=16, m=255, n=64, seed=29),
]


def _case(c):
    if c["kind"] == "ml":
        return small_ml(c["width"], c["height"], c["m"], c["seed"])
    return small_mixing(c["width"], c["height"], c["m"], c["n"], c["seed"])


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['kind']}-{c['width']}x{c['height']}-m{c['m']}")
@pytest.mark.parametrize("transform", [1, 0])
def test_generate_moments_match_oracle(gpu_context, case, transform):
    wl = _case(case)
    wl.gen.transform_to_bounds = transform
    mo, b, c = _gpu_moments(gpu_context, wl)
    ref_m, ref_b, ref_c = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max,
                                             wl.width, wl.height, wl.num_moments, "f32")
    # same sample positions and densities as the reference: bounds and compaction counts are exact
    if transform:
        assert np.array_equal(b, ref_b)
    assert np.array_equal(c, ref_c)
    hit = ref_c > 0
    assert hit.sum() > 0
    # Against the reference's FP32 moments: within 1e-4 relative, widened per pixel by the reference's own
    # FP32 rounding error (its distance to the FP64 evaluation of the same method).  On long noisy rays that
    # error alone exceeds 1e-4 (the reference differences two O(S/j^2) terms per step); these kernels stay
    # within 1e-4 of the FP64 result there.
    ref64, b64, _ = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width,
                                       wl.height, wl.num_moments, "f64")
    own = moment_rel_err(ref_m, ref64, ref64[..., 0])
    err = moment_rel_err(mo, ref_m, ref_m[..., 0])
    assert np.all(err[hit] <= MOMENT_TOL + own[hit]), f"max excess {(err - own)[hit].max():.3e}"
    same = hit & (moments_bounds_agree(ref_b, b64) if transform else hit)
    err64 = moment_rel_err(mo, ref64, ref64[..., 0])[same]
    assert err64.max() <= MOMENT_TOL, f"max rel err vs f64 {err64.max():.3e}"
    # missed rays carry zero moments
    assert np.all(mo[~hit] == 0.0)


@pytest.mark.parametrize("case", CASES[:2] + CASES[4:], ids=lambda c: f"{c['kind']}-m{c['m']}")
def test_generate_moments_vs_fp64_oracle(gpu_context, case):
    """The compensated form against the FP64 oracle of the same method."""
    import mray_gb300 as M

    wl = _case(case)
    mo, b, c = _gpu_moments(gpu_context, wl, precision=M.PRECISION_COMPENSATED_FP64_MESE)
    ref_m, ref_b, ref_c = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width,
                                             wl.height, wl.num_moments, "f64")
    hit = (ref_c > 0) & (c > 0) & moments_bounds_agree(b, ref_b)
    err = moment_rel_err(mo, ref_m, ref_m[..., 0])[hit]
    assert err.max() <= MOMENT_TOL, f"max rel err vs f64 {err.max():.3e}"


def test_compaction_matches_oracle(gpu_context):
    wl = small_ml(96, 80, 31)
    mo, b, c = _gpu_moments(gpu_context, wl)
    W, H, m = wl.width, wl.height, wl.num_moments
    d_c = _dev(c.reshape(-1).view(np.int32))
    d_m = _dev(mo.reshape(-1))
    d_idx = torch.zeros(W * H + 1, dtype=torch.int32, device="cuda")
    d_out = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
    total = gpu_context.stage_compact(W, H, m, d_c, d_m, d_idx, d_out)
    gpu_context.synchronize()
    idx_ref, data_ref = O.compact(c, mo)
    assert total == data_ref.size
    assert np.array_equal(d_idx.cpu().numpy().view(np.uint32), idx_ref)
    assert np.array_equal(d_out.cpu().numpy()[:total], data_ref)


@pytest.mark.parametrize("n", [1, 2047, 2048, 2049, 5000, 1 << 20, (1 << 22) + 3])
def test_scan_sizes(gpu_context, n):
    """Exclusive scan of counts through compaction for sizes around the 2048-element tile and multi-level cases."""
    rng = np.random.default_rng(n)
    W = min(n, 4096)
    H = (n + W - 1) // W
    P = W * H
    counts = np.zeros(P, np.uint32)
    counts[:n] = rng.integers(0, 2, size=n) * 3
    m = 3
    mo = rng.standard_normal(P * m).astype(np.float32)
    d_idx = torch.zeros(P + 1, dtype=torch.int32, device="cuda")
    d_out = torch.zeros(P * m, dtype=torch.float32, device="cuda")
    total = gpu_context.stage_compact(W, H, m, _dev(counts.view(np.int32)), _dev(mo), d_idx, d_out)
    gpu_context.synchronize()
    ref = np.zeros(P + 1, dtype=np.uint64)
    ref[1:] = np.cumsum(counts.astype(np.uint64))
    assert total == int(ref[-1])
    assert np.array_equal(d_idx.cpu().numpy().view(np.uint32).astype(np.uint64), ref)
    keep = np.repeat(counts > 0, m)
    assert np.array_equal(d_out.cpu().numpy()[:total], mo[keep])


def _oracle_image(wl):
    mi = O.workload_generate(wl, "f32")
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    return mi, tf


@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[3], CASES[4], CASES[5], CASES[6]],
                         ids=lambda c: f"{c['kind']}-m{c['m']}")
def test_prepare_and_reconstruct_from_same_moments(gpu_context, case):
    """Same compact moment image in: GPU Lagrange multipliers and re-march against the oracle's."""
    wl = _case(case)
    mi, tf = _oracle_image(wl)
    W, H, m = wl.width, wl.height, wl.num_moments
    gpu_context.upload_tf(tf)
    d_idx = _dev(mi["index"].view(np.int32))
    d_data = _dev(mi["data"])
    d_pm = torch.zeros_like(d_data)
    gpu_context.stage_prepare_moments(W, H, m, d_idx, d_data, d_pm, bias=wl.rec.bias)
    pm_ref = O.prepare_moments(W, H, m, mi["index"], mi["data"], bias=wl.rec.bias, precision="f32")
    d_b = _dev(mi["bounds"].reshape(-1).view(np.int16))
    d_rgba = torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")

    def oracle_march(pm, precision):
        return O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, mi["index"],
                             pm.astype(np.float32 if precision == "f32" else np.float64), mi["bounds"], tf, precision)

    # the per-pixel bar: two FP32 evaluations of an ill-conditioned series (64-moment mixing layer: multipliers of
    # 1e4..1e6 that cancel) or a sample on a jump of the transfer-function lookup can differ by more than 1e-3, so a
    # pixel may instead be within 1e-3 plus the FP64 colour's change under a shift of the densities by the FP32
    # evaluation bound of its series (helpers.fp32_density_bound)
    sens = fp64_sensitivity(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, mi["index"],
                            pm_ref.astype(np.float64), mi["bounds"], tf,
                            delta=fp32_density_bound(W, H, m, mi["index"], pm_ref, mi["bounds"]))

    # 1. the march alone, from the oracle's multipliers
    gpu_context.stage_reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, d_idx, _dev(pm_ref), d_b,
                                  d_rgba)
    gpu_context.synchronize()
    rgba = d_rgba.cpu().numpy().reshape(H, W, 4)
    ok = rgba_agreement(rgba, oracle_march(pm_ref, "f32"), oracle_march(pm_ref, "f64"), RGBA_TOL, sens)
    assert ok.all(), f"{(~ok).sum()} pixels outside the RGBA bar"
    # 2. the multipliers: the reference's arithmetic operation by operation, bit for bit
    gpu_context.stage_reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_rgba)
    gpu_context.synchronize()
    rgba2 = d_rgba.cpu().numpy().reshape(H, W, 4)
    pm = d_pm.cpu().numpy()
    assert np.array_equal(pm.view(np.uint32), pm_ref.view(np.uint32)), \
        f"{int((pm.view(np.uint32) != pm_ref.view(np.uint32)).sum())} of {pm.size} multipliers differ"
    ok2 = rgba_agreement(rgba2, oracle_march(pm, "f32"), oracle_march(pm, "f64"), RGBA_TOL, sens)
    assert ok2.all(), f"{(~ok2).sum()} pixels outside the RGBA bar"
    if m <= 31:
        # well-conditioned moment counts: the whole prepare + march within 1e-3 of the reference
        assert np.abs(rgba2 - oracle_march(pm_ref, "f32")).max() <= RGBA_TOL


def _full_oracle(wl, sensitivity=False):
    """The reference's FP32 pipeline and the FP64 evaluation of the same method (same sample positions); with
    sensitivity, also the FP64 colour's change under the FP32 density bound of each pixel."""
    ref = O.workload_generate(wl, "f32")
    rgba32 = O.workload_reconstruct(wl, ref, "f32")
    m64, b64, c64 = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width,
                                       wl.height, wl.num_moments, "f64")
    idx64, _ = O.compact(c64, m64.astype(np.float32))
    data64 = m64.reshape(-1, wl.num_moments)[c64.reshape(-1) > 0].reshape(-1)
    pm64 = O.prepare_moments(wl.width, wl.height, wl.num_moments, idx64, data64.astype(np.float32), bias=wl.rec.bias,
                             precision="f64")
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    rgba64 = O.reconstruct(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                           idx64, pm64, b64, tf, "f64")
    if not sensitivity:
        return ref, rgba32, rgba64
    sens = fp64_sensitivity(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                            idx64, pm64, b64, tf,
                            delta=fp32_density_bound(wl.width, wl.height, wl.num_moments, idx64, pm64, b64))
    return ref, rgba32, rgba64, sens


def test_dropin_generate_reconstruct_ml(gpu_context):
    """mraygb_generate + mraygb_reconstruct (host buffers in and out) against the reference method end to end."""
    import mray_gb300 as M

    wl = small_ml(96, 80, 31)
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(wl.width, wl.height, wl.num_moments, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    ref, rgba32, rgba64, sens = _full_oracle(wl, sensitivity=True)
    assert mi.is_compact and np.array_equal(mi.index, ref["index"])
    assert np.array_equal(mi.bounds.reshape(-1), ref["bounds"].reshape(-1))
    counts = np.diff(ref["index"].astype(np.int64)).reshape(wl.height, wl.width)
    ours = np.zeros((wl.height, wl.width, wl.num_moments), np.float32)
    theirs = np.zeros_like(ours)
    for arr, src in ((ours, mi.data), (theirs, ref["data"])):
        flat = arr.reshape(-1, wl.num_moments)
        flat[counts.reshape(-1) > 0] = src.reshape(-1, wl.num_moments)
    err = moment_rel_err(ours, theirs, theirs[..., 0])[counts > 0]
    assert err.max() <= MOMENT_TOL

    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    assert np.array_equal(tf.table, O.preintegrate(wl.tf1d, wl.tf_step))
    img = M.ColorImageHost(wl.width, wl.height)
    M.reconstruct(wl.camera, mi, tf, img, wl.rec, context=gpu_context)
    ok = rgba_agreement(img.rgba_float, rgba32, rgba64, RGBA_TOL, sens)
    assert ok.all(), f"{(~ok).sum()} pixels outside the RGBA bar"
    # the stored u8 colour: within one step of the reference's on 99.9 % of the channels
    assert np.mean(np.abs(img.rgba.astype(int) - O.rgba_to_u8(rgba32).astype(int)) <= 1) >= 0.999


@pytest.mark.parametrize("prediction_coding", [0, 1])
def test_dropin_empty_image(gpu_context, prediction_coding):
    """A view that misses the volume: every count zero, an empty compact image, empty codes, and every pixel the
    zero ray's colour (the transfer function at density 0 with alpha 0, reconstruct_zero_ray,
    raymarch_reconstruct.h:127-131), as the oracle gives it."""
    import mray_gb300 as M
    from mray_gb300 import workloads as W

    wl = small_mixing(24, 20, 16, 64, seed=3)
    wl.camera = W.perspective_camera(eye=(3.0, 3.0, 3.0), target=(6.0, 6.0, 6.0), fov_deg=30.0)
    wl.gen.prediction_coding = prediction_coding
    wl.gen.quantization_bits = 10 if prediction_coding else 32
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(wl.width, wl.height, wl.num_moments, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    ref = O.workload_generate(wl, "f32")
    assert mi.data.size == 0 and np.all(mi.index == 0) and np.array_equal(mi.index, ref["index"])
    if prediction_coding:
        table = M.default_quantization_table(wl.num_moments, 10)
        qs = M.quantize_prediction_coding(mi, table, context=gpu_context)
        assert qs.size == 0
        M.dequantize_prediction_coding(mi, table, qs, context=gpu_context)
        assert mi.data.size == 0
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    img = M.ColorImageHost(wl.width, wl.height)
    M.reconstruct(wl.camera, mi, tf, img, wl.rec, context=gpu_context)
    rgba32 = O.workload_reconstruct(wl, ref, "f32")
    assert np.array_equal(img.rgba_float, rgba32.astype(np.float32))
    assert np.all(img.rgba_float[..., 3] == 0.0)


def test_dropin_rejects_bad_arguments(gpu_context):
    import mray_gb300 as M

    wl = small_ml(16, 16, 4)
    gpu_context.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    with pytest.raises(M.MrayError):
        gpu_context.generate(wl.camera, M.GenerationParameters(step_size=0.0), 16, 16, 4)
    with pytest.raises(M.MrayError):
        gpu_context.generate(wl.camera, wl.gen, 16, 16, 256)
    with pytest.raises(M.MrayError):
        gpu_context.generate(wl.camera, wl.gen, 0, 16, 4)
