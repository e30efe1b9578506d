"""The large configuration at its full size (1024^3 mixing layer with 256 modes, 2048^2 perspective view, 64
moments, prediction coding, 10-bit codes): checks that do not need the oracle to run the whole image.

* sampled pixels: the oracle runs generate on every 16th column of every 128th row (2048 rays); the u16 bounds
  and compaction counts there are exact, the moments within 1e-4 of the FP64 evaluation;
* prediction coding: the oracle's encode of the GPU's compact moments gives the GPU's prediction-coded floats and
  coding parameters, bit for bit, over the whole image;
* codes: the oracle's quantizer and bit packer applied to the GPU's prediction-coded floats of the whole image
  give the GPU's bytes, bit for bit, and unpacking them gives the same floats on both sides;
* compaction: the index is the exclusive scan of the counts, every non-empty pixel keeps all 64 moments;
* the data-dependent quantization table of the 64 x 64 sample (quantization_curve_sampling's default) equals the
  oracle's.
"""
import numpy as np
import pytest

import oracle as O
from helpers import moment_rel_err, moments_bounds_agree

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, WIDTH, HEIGHT, M_MOM = 1024, 2048, 2048, 64
ROWS = (0, HEIGHT, 128)
COLS = (0, WIDTH, 16)


@pytest.fixture(scope="module")
def large(gpu_context):
    import mray_gb300 as Mg
    from mray_gb300 import workloads as W

    ctx = gpu_context
    ctx.precision = Mg.PRECISION_FP32
    gen, rec, cam, tf1d, tf_step = W.mixing_layer_setup(N, WIDTH, HEIGHT, prediction_coding=True)
    dmin, dmax = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    vol = W.mixing_layer_device(N, modes=256, seed=21)
    torch.cuda.synchronize()
    ctx.upload_grid(vol, dmin, dmax)
    vol_host = vol.cpu().numpy()
    del vol
    P = WIDTH * HEIGHT
    m = M_MOM
    d_mo = torch.zeros(P * m, device="cuda")
    d_b = torch.zeros(2 * P, dtype=torch.int16, device="cuda")
    d_c = torch.zeros(P, dtype=torch.int32, device="cuda")
    d_idx = torch.zeros(P + 1, dtype=torch.int32, device="cuda")
    d_cm = torch.zeros(P * m, device="cuda")
    d_cp = torch.zeros(2 * m, dtype=torch.int16, device="cuda")
    table = Mg.default_quantization_table(m, 10)
    d_codes = torch.zeros(P * (16 + 10 * (m - 1)) // 8 + 64, dtype=torch.uint8, device="cuda")
    ctx.stage_generate_moments(cam, gen, WIDTH, HEIGHT, m, d_mo, d_b, d_c)
    total = ctx.stage_compact(WIDTH, HEIGHT, m, d_c, d_mo, d_idx, d_cm)
    ctx.synchronize()
    compact = d_cm[:total].cpu().numpy()
    ctx.stage_prediction_encode(WIDTH, HEIGHT, m, d_idx, d_cm, total, 0, gen.bias, d_cp)
    ctx.synchronize()
    coded = d_cm[:total].cpu().numpy()
    nbytes = ctx.stage_quantize_prediction_coding(WIDTH, HEIGHT, m, d_idx, d_cm, table, d_codes)
    d_deq = torch.zeros(total, device="cuda")
    ctx.stage_dequantize_prediction_coding(WIDTH, HEIGHT, m, d_idx, table, d_codes, nbytes, d_deq)
    ctx.synchronize()
    out = dict(gen=gen, cam=cam, vol=vol_host, dmin=dmin, dmax=dmax, table=table, total=total,
               d_index=d_idx, d_coded=d_cm, d_coding_params=d_cp, coding_params=d_cp.cpu().numpy().view(np.uint16),
               moments=d_mo.cpu().numpy().reshape(HEIGHT, WIDTH, m),
               bounds=d_b.cpu().numpy().view(np.uint16).reshape(HEIGHT, WIDTH, 2),
               counts=d_c.cpu().numpy().view(np.uint32).reshape(HEIGHT, WIDTH),
               index=d_idx.cpu().numpy().view(np.uint32), compact=compact, coded=coded,
               codes=d_codes[:nbytes].cpu().numpy(), dequantized=d_deq.cpu().numpy())
    return out


def test_large_sampled_pixels_match_oracle(large):
    g = large
    ref_m, ref_b, ref_c = O.generate_moments(g["cam"], g["gen"], g["vol"], g["dmin"], g["dmax"], WIDTH, HEIGHT, M_MOM,
                                             "f32", rows=ROWS, cols=COLS)
    m64, b64, _ = O.generate_moments(g["cam"], g["gen"], g["vol"], g["dmin"], g["dmax"], WIDTH, HEIGHT, M_MOM, "f64",
                                     rows=ROWS, cols=COLS)
    sel = (slice(ROWS[0], ROWS[1], ROWS[2]), slice(COLS[0], COLS[1], COLS[2]))
    assert np.array_equal(g["bounds"][sel], ref_b[sel])
    assert np.array_equal(g["counts"][sel], ref_c[sel])
    hit = ref_c[sel] > 0
    assert hit.sum() > 256
    same = hit & moments_bounds_agree(ref_b[sel], b64[sel])
    err = moment_rel_err(g["moments"][sel], m64[sel], m64[sel][..., 0])[same]
    assert err.max() <= 1e-4, f"max rel err vs f64 {err.max():.3e}"


def test_large_compaction(large):
    g = large
    counts = g["counts"].reshape(-1).astype(np.uint64)
    assert np.array_equal(g["index"][1:].astype(np.uint64), np.cumsum(counts))
    assert g["index"][0] == 0 and int(g["index"][-1]) == g["total"]
    assert set(np.unique(counts)) <= {0, M_MOM}


def test_large_prediction_encode_bit_exact(large):
    """The reference's prediction encode (oracle) on the GPU's compact moments of the whole 2048^2 image: the same
    prediction-coded floats and coding parameters, bit for bit."""
    g = large
    ref, cp_ref = O.prediction_encode(WIDTH, HEIGHT, M_MOM, g["index"], g["compact"], 0, g["gen"].bias)
    assert np.array_equal(g["coding_params"][:2 * (M_MOM - 1)], cp_ref)
    diff = int(np.count_nonzero(ref.view(np.uint32) != g["coded"].view(np.uint32)))
    assert diff == 0, f"{diff} of {ref.size} prediction-coded floats differ"


def test_large_codes_bit_exact(large):
    """The reference's quantizer and packer (oracle) on the GPU's prediction-coded floats: the same bytes."""
    g = large
    ref = O.quantize_prediction_coding(WIDTH, HEIGHT, M_MOM, g["index"], g["coded"], g["table"])
    assert ref.size == g["codes"].size
    assert np.array_equal(ref, g["codes"])
    # unpacking: the oracle's dequantization of the bytes equals the GPU's, and re-quantizing it is the identity
    deq = O.dequantize_prediction_coding(WIDTH, HEIGHT, M_MOM, g["index"], g["table"], g["codes"], g["total"])
    assert np.array_equal(deq, g["dequantized"])
    again = O.quantize_prediction_coding(WIDTH, HEIGHT, M_MOM, g["index"], g["dequantized"], g["table"])
    assert np.array_equal(again, g["codes"])


def test_large_quantization_table(large, gpu_context):
    """create_quantization_table on the sample_moment_image(64, 64) of the full prediction-coded image."""
    g = large
    d_coded = g["d_coded"]
    table, means = gpu_context.stage_create_quantization_table(WIDTH, HEIGHT, M_MOM, g["d_index"], d_coded, 0,
                                                               g["d_coding_params"], 10, sampling=64,
                                                               return_means=True)
    s_index, s_data = O.sample_moment_image(WIDTH, HEIGHT, g["index"], g["coded"], 64)
    ref_table, ref_means, _ = O.create_quantization_table(64, 64, M_MOM, s_index, s_data, 0, g["coding_params"], 10)
    seen = np.isfinite(ref_means)
    assert np.array_equal(means[seen], ref_means[seen])
    assert table.tolist() == ref_table.tolist()


def test_large_codes_end_to_end_sampled(large):
    """Volume -> 10-bit codes on the sampled pixels of the large configuration: the codes of the GPU's moments, of
    the reference's FP32 moments (oracle) and of the FP64 moments rounded to float, each prediction coded with the
    reference's encoder (bit-exact with the GPU's on the same moments, test above) and quantized with the fixed
    table.  The warp is the plain one (CODING_WARP_NONE), so every pixel's codes depend on its own moments only.
    Ours must agree with the codes of the FP64 moments at least as often as the reference's do."""
    g = large
    sel = (slice(ROWS[0], ROWS[1], ROWS[2]), slice(COLS[0], COLS[1], COLS[2]))
    ref_m, ref_b, ref_c = O.generate_moments(g["cam"], g["gen"], g["vol"], g["dmin"], g["dmax"], WIDTH, HEIGHT, M_MOM,
                                             "f32", rows=ROWS, cols=COLS)
    m64, b64, _ = O.generate_moments(g["cam"], g["gen"], g["vol"], g["dmin"], g["dmax"], WIDTH, HEIGHT, M_MOM, "f64",
                                     rows=ROWS, cols=COLS)
    keep = (ref_c[sel] > 0) & np.all(ref_b[sel] == b64[sel], axis=-1)
    n = int(keep.sum())
    assert n > 256
    index = np.arange(n + 1, dtype=np.uint32) * M_MOM
    codes = []
    for mom in (g["moments"][sel][keep], ref_m[sel][keep], m64[sel][keep].astype(np.float32)):
        enc, _ = O.prediction_encode(n, 1, M_MOM, index, mom.reshape(-1), 1, g["gen"].bias)
        packed = O.quantize_prediction_coding(n, 1, M_MOM, index, enc, g["table"])
        codes.append(O.unpack_codes(n, 1, M_MOM, index, g["table"], packed))
    ours, ref, exact = codes
    ours_vs_exact = float(np.mean(ours != exact))
    ref_vs_exact = float(np.mean(ref != exact))
    print(f"large configuration, {n} sampled pixels: 10-bit codes differing from those of the FP64 moments, ours "
          f"{ours_vs_exact:.3%}, the reference's FP32 {ref_vs_exact:.3%}; ours against the reference's "
          f"{float(np.mean(ours != ref)):.3%}")
    assert ours_vs_exact <= ref_vs_exact + 0.002
