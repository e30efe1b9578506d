"""GPU prediction coding, coding parameters, quantization and bit packing against the oracle.

Bar: from the same input moments, the prediction-coded floats, the u16 coding parameters, the 10-bit codes and
the packed bytes are bit-identical to the reference's CPU arithmetic (the device performs its float operations in
its order and takes cosf / sinf with the C library's results).  From the same volume, the moments themselves
differ from the reference's in their last bits, so the end-to-end code mismatch is measured and bounded.
"""
import numpy as np
import pytest

import oracle as O
from helpers import fp32_density_bound, fp64_sensitivity, rgba_agreement, small_mixing, small_ml

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _ragged_image(seed=0, width=40, height=24, m=16):
    """A compact image with random per-pixel counts 0..m (the error-threshold compaction case), from real
    moments of the Marschner-Lobb case."""
    wl = small_ml(width, height, m, seed=seed + 3)
    mo, b, c = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, width, height, m, "f32")
    rng = np.random.default_rng(seed)
    counts = np.where(c > 0, rng.integers(0, m + 1, size=c.shape), 0).astype(np.uint32)
    index, data = O.compact(counts, mo)
    return width, height, m, index, data


def _encode_gpu(ctx, W, H, m, index, data, warp, bias):
    d_idx = _dev(index.view(np.int32))
    d_data = _dev(data)
    d_cp = torch.zeros(max(2 * (m - 1), 1), dtype=torch.int16, device="cuda")
    ctx.stage_prediction_encode(W, H, m, d_idx, d_data, data.size, coding_warp=warp, bias=bias, coding_params=d_cp)
    ctx.synchronize()
    return d_data.cpu().numpy(), d_cp.cpu().numpy().view(np.uint16)[:2 * (m - 1)]


@pytest.mark.parametrize("warp", [0, 1])
@pytest.mark.parametrize("ragged_seed", [None, 1, 2])
def test_prediction_encode_matches_oracle(gpu_context, warp, ragged_seed):
    if ragged_seed is None:
        wl = small_ml(96, 80, 31)
        mi = O.workload_generate(wl, "f32")
        W, H, m, index, data = wl.width, wl.height, wl.num_moments, mi["index"], mi["data"]
    else:
        W, H, m, index, data = _ragged_image(ragged_seed)
    bias = 5e-5
    ours, cp = _encode_gpu(gpu_context, W, H, m, index, data, warp, bias)
    ref, cp_ref = O.prediction_encode(W, H, m, index, data, warp, bias)
    # the encoded (and, with the default warp, warped) floats: bit for bit
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), \
        f"{int((ours.view(np.uint32) != ref.view(np.uint32)).sum())} of {ref.size} floats differ"
    if warp == 0:
        assert np.array_equal(cp, cp_ref)
    # the 10-bit codes packed by the GPU equal the reference packer's codes of the reference's floats
    table = O.default_quantization_table(m, 10)
    d_out = torch.zeros(ours.size * 4 + 16, dtype=torch.uint8, device="cuda")
    n = gpu_context.stage_quantize_prediction_coding(W, H, m, _dev(index.view(np.int32)), _dev(ours), table, d_out)
    gpu_context.synchronize()
    b = O.quantize_prediction_coding(W, H, m, index, ref, table)
    assert n == b.size
    assert np.array_equal(d_out.cpu().numpy()[:n], b)


@pytest.mark.parametrize("warp", [0, 1])
@pytest.mark.parametrize("m", [1, 2, 64, 255])
def test_prediction_encode_moment_counts(gpu_context, warp, m):
    """The same bar at the ends of the moment range: one and two moments (no or one coding-parameter pair) and 64
    and 255 (the reference's limit), on a compact image with random per-pixel counts."""
    W, H, m, index, data = _ragged_image(seed=m, width=24, height=16, m=m)
    ours, cp = _encode_gpu(gpu_context, W, H, m, index, data, warp, 5e-5)
    ref, cp_ref = O.prediction_encode(W, H, m, index, data, warp, 5e-5)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), \
        f"{int((ours.view(np.uint32) != ref.view(np.uint32)).sum())} of {ref.size} floats differ"
    if warp == 0:
        assert np.array_equal(cp, cp_ref)
    table = O.default_quantization_table(m, 10)
    d_out = torch.zeros(ours.size * 4 + 16, dtype=torch.uint8, device="cuda")
    n = gpu_context.stage_quantize_prediction_coding(W, H, m, _dev(index.view(np.int32)), _dev(ours), table, d_out)
    gpu_context.synchronize()
    b = O.quantize_prediction_coding(W, H, m, index, ref, table)
    assert n == b.size
    assert np.array_equal(d_out.cpu().numpy()[:n], b)


TABLES = {
    "16_10": lambda m: O.default_quantization_table(m, 10),
    "16_12": lambda m: O.default_quantization_table(m, 12),
    "ragged_bits": lambda m: np.array([16] + [8 + (i % 9) for i in range(1, m)], dtype=np.uint8)[:m],
    "32": lambda m: np.full(m, 32, dtype=np.uint8),
    "odd": lambda m: np.array([13] + [7] * (m - 1), dtype=np.uint8)[:m],
}


@pytest.mark.parametrize("table_name", list(TABLES))
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_quantize_pack_bit_exact(gpu_context, table_name, seed):
    """Same prediction-coded floats in: identical codes and identical packed bytes (the trailing partial byte
    dropped as the reference's packer does)."""
    W, H, m, index, data = _ragged_image(seed)
    rng = np.random.default_rng(seed)
    # values around [0, 1] including the clamp edges and exact code boundaries
    vals = rng.uniform(-0.1, 1.1, size=data.size).astype(np.float32)
    vals[::17] = 0.0
    vals[::19] = 1.0
    vals[::23] = np.float32(511) / np.float32(1023)
    table = TABLES[table_name](m)
    ref = O.quantize_prediction_coding(W, H, m, index, vals, table)
    d_out = torch.zeros(vals.size * 4 + 16, dtype=torch.uint8, device="cuda")
    n = gpu_context.stage_quantize_prediction_coding(W, H, m, _dev(index.view(np.int32)), _dev(vals), table, d_out)
    gpu_context.synchronize()
    assert n == ref.size
    assert np.array_equal(d_out.cpu().numpy()[:n], ref)


@pytest.mark.parametrize("table_name", ["16_10", "ragged_bits", "32"])
def test_dequantize_round_trip(gpu_context, table_name):
    W, H, m, index, data = _ragged_image(4)
    rng = np.random.default_rng(4)
    vals = rng.uniform(0.0, 1.0, size=data.size).astype(np.float32)
    table = TABLES[table_name](m)
    packed = O.quantize_prediction_coding(W, H, m, index, vals, table)
    ref = O.dequantize_prediction_coding(W, H, m, index, table, packed, vals.size)
    d_out = torch.zeros(max(vals.size, 1), dtype=torch.float32, device="cuda")
    d_packed = _dev(np.concatenate([packed, np.zeros(8, np.uint8)]))
    gpu_context.stage_dequantize_prediction_coding(W, H, m, _dev(index.view(np.int32)), table, d_packed, packed.size,
                                                   d_out)
    gpu_context.synchronize()
    assert np.array_equal(d_out.cpu().numpy()[:vals.size], ref)


def test_quantize_host_api_matches_reference_packer(gpu_context):
    import mray_gb300 as M

    W, H, m, index, data = _ragged_image(5)
    mi = M.MomentImageHost(W, H, m, True)
    mi.is_compact, mi.prediction_code = True, True
    mi.index, mi.data = index, np.clip(data, 0, 1).astype(np.float32)
    table = M.default_quantization_table(m, 10)
    ours = M.quantize_prediction_coding(mi, table, context=gpu_context)
    assert np.array_equal(ours, O.quantize_prediction_coding(W, H, m, index, mi.data, table))


def test_dequantize_host_api_matches_reference_unpacker(gpu_context):
    """mraygb_dequantize_prediction_coding (dequantize_prediction_coding on host buffers): the oracle's floats."""
    import mray_gb300 as M

    W, H, m, index, data = _ragged_image(6)
    table = M.default_quantization_table(m, 10)
    vals = np.random.default_rng(6).uniform(0.0, 1.0, size=data.size).astype(np.float32)
    packed = O.quantize_prediction_coding(W, H, m, index, vals, table)
    mi = M.MomentImageHost(W, H, m, True)
    mi.is_compact, mi.prediction_code = True, True
    mi.index, mi.data = index, np.zeros(data.size, np.float32)
    M.dequantize_prediction_coding(mi, table, packed, context=gpu_context)
    ref = O.dequantize_prediction_coding(W, H, m, index, table, packed, data.size)
    assert np.array_equal(mi.data, ref)


def test_measured_fp32_rate_is_plausible(gpu_context):
    """The FP32 FMA roof: within the GB300's nominal 152 SMs x 128 lanes x 2 FLOP x 2.07 GHz = 80.6 TFLOP/s."""
    rate = gpu_context.measure_fp32_rate()
    assert 20.0 < rate < 85.0, rate


@pytest.mark.parametrize("warp", [0, 1])
def test_dropin_generate_prediction_coded_then_reconstruct(gpu_context, warp):
    """generate with prediction_coding (the reference's default), codes at 10 bits, reconstruct from the
    prediction-coded image; compared with the reference method end to end."""
    import mray_gb300 as M

    wl = small_ml(96, 80, 31)
    wl.gen.prediction_coding = 1
    wl.gen.coding_warp = warp
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(wl.width, wl.height, wl.num_moments, True, True)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    ref = O.workload_generate(wl, "f32")
    assert mi.prediction_code and np.array_equal(mi.index, ref["index"])
    if warp == 0:
        assert np.abs(mi.coding_params.astype(int) - ref["coding_params"].astype(int)).max() <= 1
    # the encoding amplifies the moments' last-bit differences (the reference's FP32 rounding) by the
    # prediction coding's Levinson recursion; with the same input moments it is the reference's arithmetic
    # bit for bit (test_prediction_encode_matches_oracle)
    assert np.abs(mi.data.astype(np.float64) - ref["data"]).max() <= 2e-3
    table = M.default_quantization_table(wl.num_moments, 10)
    codes = M.quantize_prediction_coding(mi, table, context=gpu_context)
    codes_ref = O.quantize_prediction_coding(wl.width, wl.height, wl.num_moments, ref["index"], ref["data"], table)
    assert codes.size == codes_ref.size
    # end to end (volume -> codes): the moments differ from the reference's FP32 moments in their last bits, and a
    # code flips wherever that carries an encoded value across a code boundary.  Both code streams are compared with
    # the codes the reference's FP32 encoding gives for the FP64 moments rounded to float (pixels whose u16 bounds
    # agree in both precisions): ours must agree with those at least as often as the reference's do.
    W, H, m = wl.width, wl.height, wl.num_moments
    m64, b64, _ = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, W, H, m, "f64")
    counts = np.diff(ref["index"].astype(np.int64))
    data64 = m64.reshape(-1, m)[counts > 0].reshape(-1).astype(np.float32)
    enc64, _ = O.prediction_encode(W, H, m, ref["index"], data64, warp, wl.gen.bias)
    codes_exact = O.quantize_prediction_coding(W, H, m, ref["index"], enc64, table)
    a, b, e = (O.unpack_codes(W, H, m, ref["index"], table, c) for c in (codes, codes_ref, codes_exact))
    pix_same = np.all(b64.reshape(-1, 2) == ref["bounds"].reshape(-1, 2), axis=-1)
    same = np.repeat(pix_same, counts)
    ours_vs_ref = float(np.mean(a != b))
    ours_vs_exact = float(np.mean((a != e)[same]))
    ref_vs_exact = float(np.mean((b != e)[same]))
    print(f"10-bit codes differing (warp {warp}, {a.size} codes): ours vs reference {ours_vs_ref:.3%}, ours vs "
          f"exact {ours_vs_exact:.3%}, reference vs exact {ref_vs_exact:.3%}")
    assert ours_vs_exact <= ref_vs_exact + 0.002
    # reconstruct from the prediction-coded image (prepare_moments_from_pred_coding)
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    img = M.ColorImageHost(wl.width, wl.height)
    M.reconstruct(wl.camera, mi, tf, img, wl.rec, context=gpu_context)
    rgba_ref = O.workload_reconstruct(wl, ref, "f32")
    pm64 = O.prepare_moments(wl.width, wl.height, wl.num_moments, ref["index"], ref["data"], True, warp,
                             ref["coding_params"], wl.rec.bias, "f64")
    rgba64 = O.reconstruct(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                           ref["index"], pm64, ref["bounds"], O.preintegrate(wl.tf1d, wl.tf_step), "f64")
    diff = np.abs(img.rgba_float - rgba_ref).max(axis=-1)
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    sens = fp64_sensitivity(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                            ref["index"], pm64, ref["bounds"], tf,
                            delta=fp32_density_bound(wl.width, wl.height, wl.num_moments, ref["index"], pm64,
                                                     ref["bounds"]))
    ok = rgba_agreement(img.rgba_float, rgba_ref, rgba64, 1e-3, sens)
    assert np.quantile(diff, 0.99) <= 1e-3
    assert ok.all(), f"{(~ok).sum()} pixels outside the RGBA bar"


def test_prepare_from_prediction_coding_same_input(gpu_context):
    """prepare_moments_from_pred_coding on the same prediction-coded floats: the re-march matches the oracle."""
    wl = small_ml(64, 48, 16)
    wl.gen.prediction_coding = 1
    ref = O.workload_generate(wl, "f32")
    W, H, m = wl.width, wl.height, wl.num_moments
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf)
    d_idx = _dev(ref["index"].view(np.int32))
    d_data = _dev(ref["data"])
    d_pm = torch.zeros_like(d_data)
    d_cp = _dev(ref["coding_params"].view(np.int16))
    gpu_context.stage_prepare_moments(W, H, m, d_idx, d_data, d_pm, prediction_code=True, coding_warp=0,
                                      coding_params=d_cp, bias=wl.rec.bias)
    gpu_context.synchronize()
    pm_ref = O.prepare_moments(W, H, m, ref["index"], ref["data"], True, 0, ref["coding_params"], wl.rec.bias)
    pm = d_pm.cpu().numpy()
    rgba = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, ref["index"], pm, ref["bounds"],
                         tf, "f32")
    rgba_ref = O.reconstruct(wl.camera, wl.rec, W, H, m, wl.domain_min, wl.domain_max, ref["index"], pm_ref,
                             ref["bounds"], tf, "f32")
    assert np.abs(rgba - rgba_ref).max() <= 1e-3
    # the multipliers themselves: the reference's arithmetic, bit for bit
    assert np.array_equal(pm.view(np.uint32), pm_ref.view(np.uint32))
