"""Error-threshold compaction on the GPU against the oracle: determine_best_number_moments per pixel
(moment_compaction.h:113-174, the reference's GPU form compute_num_moments_kernel, moment_raymarcher.cu:187-208),
then the compaction index.  Every shipped evaluation configuration runs generate with error_threshold = 0.01.

Bar: the per-pixel counts and the index are integers and must be equal.  Same moments in (the GPU's), so the
comparison isolates the count; the end-to-end counts from the volume (moments that differ from the reference's in
their last bits, which can move a pixel's rRMSE across the threshold) are reported and bounded separately.
"""
import numpy as np
import pytest

import oracle as O
from helpers import small_mixing, small_ml

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _gpu_generate(ctx, wl):
    ctx.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    W, H, m = wl.width, wl.height, wl.num_moments
    mo = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
    b = torch.zeros(2 * W * H, dtype=torch.int16, device="cuda")
    c = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    ctx.stage_generate_moments(wl.camera, wl.gen, W, H, m, mo, b, c)
    idx = torch.zeros(W * H + 1, dtype=torch.int32, device="cuda")
    out = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
    total = ctx.stage_compact(W, H, m, c, mo, idx, out)
    ctx.synchronize()
    return (mo.cpu().numpy().reshape(H * W, m), b.cpu().numpy().view(np.uint16).reshape(H * W, 2),
            c.cpu().numpy().view(np.uint32), idx.cpu().numpy().view(np.uint32), out.cpu().numpy()[:total])


def _case(kind, m):
    if kind == "ml":
        wl = small_ml(96, 80, m, seed=11)
    else:
        wl = small_mixing(64, 64, m, n=96, seed=21)
    wl.gen.compact_image = 1
    wl.gen.transform_to_bounds = 1
    return wl


@pytest.mark.parametrize("thr", [0.01, 0.001])
@pytest.mark.parametrize("m", [8, 31, 64, 128, 255])
@pytest.mark.parametrize("kind", ["ml", "mixing"])
def test_threshold_counts_match_oracle(gpu_context, kind, m, thr):
    wl = _case(kind, m)
    wl.gen.error_threshold = thr
    mo, b, counts, index, data = _gpu_generate(gpu_context, wl)
    nonzero = b[:, 0] != b[:, 1]
    assert nonzero.sum() > 0
    ref = O.count_moments(mo, nonzero.astype(np.uint32), thr)
    assert np.array_equal(counts, ref), f"{int((counts != ref).sum())} of {counts.size} counts differ"
    # the search moved the counts (the threshold is active) and kept every non-empty pixel non-empty
    assert np.all(counts[nonzero] >= 1) and np.all(counts[~nonzero] == 0)
    assert np.any(counts[nonzero] < m)
    idx_ref, data_ref = O.compact(counts.reshape(wl.height, wl.width), mo.reshape(wl.height, wl.width, m))
    assert np.array_equal(index, idx_ref)
    assert np.array_equal(data, data_ref)


@pytest.mark.parametrize("m", [31, 64])
def test_threshold_counts_end_to_end(gpu_context, m):
    """From the volume.  The moments differ from the reference's FP32 moments in their last bits (the reference's
    own FP32 error reaches 2.8e-4 relative on 64-moment noisy rays), and a count flips wherever that moves a pixel's
    rRMSE across the threshold.  Both are compared with the counts that the reference's FP32 search gives for the
    FP64 moments rounded to float: ours must agree with those at least as often as the reference's do."""
    wl = _case("ml" if m == 31 else "mixing", m)
    wl.gen.error_threshold = 0.01
    mo, b, counts, index, data = _gpu_generate(gpu_context, wl)
    _, ref_b, ref_c = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width,
                                         wl.height, m, "f32")
    assert np.array_equal(b, ref_b.reshape(-1, 2))
    m64, b64, _ = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, wl.width,
                                     wl.height, m, "f64")
    nonzero = b[:, 0] != b[:, 1]
    same = np.all(b64.reshape(-1, 2) == b, axis=-1)
    exact = O.count_moments(m64.reshape(-1, m).astype(np.float32), nonzero.astype(np.uint32), 0.01)
    ref_c = ref_c.reshape(-1)
    ours_vs_ref = float(np.mean(counts != ref_c))
    ours_vs_exact = float(np.mean((counts != exact)[same]))
    ref_vs_exact = float(np.mean((ref_c != exact)[same]))
    print(f"m={m}: counts differing, ours vs reference {ours_vs_ref:.3%}, ours vs exact {ours_vs_exact:.3%}, "
          f"reference vs exact {ref_vs_exact:.3%}")
    assert ours_vs_exact <= ref_vs_exact + 0.002
