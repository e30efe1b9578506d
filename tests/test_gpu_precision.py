"""The precision forms' MESE preparation against the FP64 oracle of the same method, on the same compact moment
image (the reference's FP32 moments): the FP64 form (native FP64) and the float-float form (float pairs for the
exponential moments and Levinson's recursion, FP32 correlation tail)."""
import numpy as np
import pytest

import oracle as O
from helpers import small_mixing, small_ml

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _lambda_err(pm, pm64, index):
    """Per pixel max_k |lambda_k - lambda64_k| / max_k |lambda64_k|."""
    out = []
    for p in range(index.size - 1):
        a, b = int(index[p]), int(index[p + 1])
        if b > a:
            out.append(np.abs(pm[a:b] - pm64[a:b]).max() / max(np.abs(pm64[a:b]).max(), 1e-30))
    return np.array(out)


CASES = [("ml", 31), ("mix", 64), ("mix", 128), ("mix", 255)]


@pytest.mark.parametrize("form", ["fp64", "ff"])
@pytest.mark.parametrize("pc", [0, 1], ids=["std", "prediction_coded"])
@pytest.mark.parametrize("kind,m", CASES)
def test_precision_prepare_matches_fp64_oracle(gpu_context, form, pc, kind, m):
    import mray_gb300 as M

    wl = small_ml(64, 56, m) if kind == "ml" else small_mixing(48, 40, m, 96)
    wl.gen.prediction_coding = pc
    mi = O.workload_generate(wl, "f32")
    W, H = wl.width, wl.height
    d_idx = _dev(mi["index"].view(np.int32))
    d_data = _dev(mi["data"])
    d_pm = torch.zeros_like(d_data)
    cp = mi["coding_params"]
    d_cp = _dev(cp.view(np.int16)) if cp is not None else None
    gpu_context.precision = (M.PRECISION_COMPENSATED_FP64_MESE if form == "fp64"
                             else M.PRECISION_COMPENSATED_FF_MESE)
    gpu_context.stage_prepare_moments(W, H, m, d_idx, d_data, d_pm, prediction_code=pc, coding_warp=0,
                                      coding_params=d_cp, bias=wl.rec.bias)
    gpu_context.synchronize()
    gpu_context.precision = M.PRECISION_FP32
    pm = d_pm.cpu().numpy().astype(np.float64)
    pm64 = O.prepare_moments(W, H, m, mi["index"], mi["data"], bool(pc), 0, cp, wl.rec.bias, "f64")
    err = _lambda_err(pm, pm64, mi["index"])
    # FP64: the same arithmetic up to contraction and the sincos of the first exponential moment; float-float:
    # 48-bit steps, then the FP32 tail and the float result.  The tail's correlations sum m products in FP32, so
    # its rounding grows with m: the bar scales with m above 64 moments (measured at 255 moments: p99 5.5e-6, max
    # 1.8e-5, against 2e-5 / 8e-5)
    tol = 1e-6 if form == "fp64" else 2e-5 * max(1.0, m / 64.0)
    assert np.quantile(err, 0.99) <= tol / 4 and err.max() <= tol, f"p99 {np.quantile(err, .99):.2e} max {err.max():.2e}"
    # the FP32 preparation, for scale: the precision forms are far closer to FP64
    gpu_context.stage_prepare_moments(W, H, m, d_idx, d_data, d_pm, prediction_code=pc, coding_warp=0,
                                      coding_params=d_cp, bias=wl.rec.bias)
    gpu_context.synchronize()
    err32 = _lambda_err(d_pm.cpu().numpy().astype(np.float64), pm64, mi["index"])
    assert np.median(err) < np.median(err32)
