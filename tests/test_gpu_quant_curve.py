"""The data-dependent quantization table (create_quantization_table, measure_coding_error.cpp:374-438, on the
sample_moment_image main.cpp:318-327 takes) against the oracle, through the C ABI.

The GPU evaluates every (index, bits) pair the search can reach; the oracle runs the reference's sequential search.
The device's per-pixel arithmetic is the reference CPU build's operation for operation, with cosf / sinf taking the
C library's results, so every mean the search evaluated is bit-identical and so is the table.
"""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _golden(key):
    g = np.load(os.path.join(GOLDEN, "quant_curve.npz"))
    W, H, m, s = (int(v) for v in g[f"{key}_shape"])
    return W, H, m, s, g[f"{key}_index"], g[f"{key}_data"], g[f"{key}_coding_params"]


def _stage(ctx, W, H, m, index, data, warp, cp, start_bits, sampling):
    d_cp = _dev(cp.view(np.int16)) if cp is not None else None
    return ctx.stage_create_quantization_table(W, H, m, _dev(index.view(np.int32)), _dev(data), warp, d_cp,
                                               start_bits, sampling=sampling, return_means=True)


def _check_against_oracle(table, means, W, H, m, index, data, warp, cp, start_bits, s):
    s_index, s_data = O.sample_moment_image(W, H, index, data, s) if s else (index, data)
    sw = s or W
    sh = s or H
    ref_table, ref_means, ref_evals = O.create_quantization_table(sw, sh, m, s_index, s_data, warp, cp, start_bits)
    seen = np.isfinite(ref_means)
    assert seen.sum() == ref_evals
    same = means[seen] == ref_means[seen]
    assert same.all(), f"{(~same).sum()} of {seen.sum()} means differ from the oracle's"
    assert table.tolist() == ref_table.tolist()
    return ref_table


@pytest.mark.parametrize("key,start_bits", [("mix", 10), ("mix", 16), ("mix", 3), ("mlthr", 10), ("mlthr", 7)])
def test_table_matches_oracle(gpu_context, key, start_bits):
    W, H, m, s, index, data, cp = _golden(key)
    table, means = _stage(gpu_context, W, H, m, index, data, 0, cp, start_bits, s)
    ref = _check_against_oracle(table, means, W, H, m, index, data, 0, cp, start_bits, s)
    assert ref[0] == 16 and ref[1] == start_bits
    # every reachable pair is evaluated on the GPU, visited or not
    bmin = min(2, start_bits)
    assert np.all(np.isfinite(means[1:, bmin:start_bits + 1]))
    assert np.all(np.isnan(means[0])) and np.all(np.isnan(means[:, start_bits + 1:]))


def test_ragged_counts_and_short_pixels(gpu_context):
    """Error-threshold compaction leaves pixels with fewer moments than the index being quantized: their error is
    0 and they still count in the mean (compute_coding_error visits every non-empty pixel)."""
    W, H, m, s, index, data, cp = _golden("mlthr")
    s_index, _ = O.sample_moment_image(W, H, index, data, s)
    counts = np.diff(s_index.astype(np.int64))
    assert counts.min() < m // 2 < counts.max()
    table, means = _stage(gpu_context, W, H, m, index, data, 0, cp, 10, s)
    _check_against_oracle(table, means, W, H, m, index, data, 0, cp, 10, s)


def test_whole_image_without_sampling(gpu_context):
    """sampling <= 0: create_quantization_table on the image as given (any shape)."""
    W, H, m, s, index, data, cp = _golden("mlthr")
    table, means = _stage(gpu_context, W, H, m, index, data, 0, cp, 9, 0)
    _check_against_oracle(table, means, W, H, m, index, data, 0, cp, 9, 0)


def test_host_call_equals_stage_call(gpu_context):
    import mray_gb300 as Mg

    W, H, m, s, index, data, cp = _golden("mix")
    mi = Mg.MomentImageHost(W, H, m, True)
    mi.index, mi.data, mi.is_compact = index.copy(), data.copy(), True
    mi.prediction_code, mi.coding_warp, mi.coding_params = True, 0, cp.copy()
    t_host, m_host = gpu_context.create_quantization_table(mi, 10, sampling=s, return_means=True)
    t_stage, m_stage = _stage(gpu_context, W, H, m, index, data, 0, cp, 10, s)
    assert t_host.tolist() == t_stage.tolist()
    assert np.array_equal(m_host, m_stage, equal_nan=True)
    assert Mg.create_quantization_table(mi, 10, context=gpu_context, sampling=s).tolist() == t_host.tolist()


def test_coding_warp_none(gpu_context):
    """Residuals warped by x / 2 + 1 / 2 (CODING_WARP_NONE) need no coding parameters."""
    from mray_gb300 import workloads as Wl

    wl = Wl.mixing_layer_workload(n=40, width=32, height=32, num_moments=32, modes=16, seed=5, name="qc_warp_none")
    wl.gen.prediction_coding = 0
    mi = O.workload_generate(wl, "f32")
    data, _ = O.prediction_encode(wl.width, wl.height, wl.num_moments, mi["index"], mi["data"], coding_warp=1,
                                  bias=wl.gen.bias)
    assert data.min() >= 0 and data.max() <= 1
    table, means = _stage(gpu_context, wl.width, wl.height, wl.num_moments, mi["index"], data, 1, None, 10, 16)
    _check_against_oracle(table, means, wl.width, wl.height, wl.num_moments, mi["index"], data, 1, None, 10, 16)


def test_gpu_pipeline_image_at_default_sampling(gpu_context):
    """The GPU's own prediction-coded 128x128 image, sampled 64 x 64 (quantization_curve_sampling's default)."""
    from helpers import small_mixing

    wl = small_mixing(128, 128, 64, 96)
    wl.gen.prediction_coding = 1
    mi = O.workload_generate(wl, "f32")
    table, means = _stage(gpu_context, wl.width, wl.height, 64, mi["index"], mi["data"], 0, mi["coding_params"],
                          10, 64)
    ref = _check_against_oracle(table, means, wl.width, wl.height, 64, mi["index"], mi["data"], 0,
                                mi["coding_params"], 10, 64)
    assert ref[-1] < 10


def test_errors(gpu_context):
    import mray_gb300 as Mg

    W, H, m, s, index, data, cp = _golden("mix")
    d_index, d_data, d_cp = _dev(index.view(np.int32)), _dev(data), _dev(cp.view(np.int16))

    def call(width=W, height=H, mm=m, idx=d_index, warp=0, cpp=d_cp, bits=10, sampling=s):
        return gpu_context.stage_create_quantization_table(width, height, mm, idx, d_data, warp, cpp, bits, sampling)

    with pytest.raises(Mg.MrayError) as e:  # a 32x16 sample: the reference indexes it as 16x32
        call(height=H // 2, sampling=64)
    assert e.value.status == 6
    for kwargs in (dict(mm=1), dict(bits=0), dict(bits=32), dict(idx=None), dict(cpp=None), dict(warp=5)):
        with pytest.raises(Mg.MrayError) as e:
            call(**kwargs)
        assert e.value.status == 1, kwargs
    # the context stays usable
    assert call().tolist()[:2] == [16, 10]
