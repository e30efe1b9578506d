"""The device cosf / sinf of the MESE algebra against the host C library, for every float of [-pi, pi].

The reference computes the zeroth-moment phase's cosine and sine with the C library's cosf / sinf
(mese/MESE_dynamic.h:38-40, moment_prediction_coding.h:103-104).  Everything the prediction coding, the
error-threshold count and the FP32 preparation produce depends on those two values, so the device must return
the C library's results bit for bit.  Bar: identical bits for all 2 * 1,078,530,012 floats of [-pi, pi].
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_ABS_BITS = 0x40490FDB  # (float)pi
CHUNK = 1 << 25


def _check_range(ctx, lo, hi, sign):
    """Bits [lo, hi) with the given sign bit, on the device and in the C library."""
    x_dev = torch.empty(CHUNK, dtype=torch.float32, device="cuda")
    s_dev = torch.empty_like(x_dev)
    c_dev = torch.empty_like(x_dev)
    bad = 0
    for start in range(lo, hi, CHUNK):
        n = min(CHUNK, hi - start)
        bits = np.arange(start, start + n, dtype=np.uint32)
        if sign:
            bits |= np.uint32(0x80000000)
        x = bits.view(np.float32)
        x_dev[:n].copy_(torch.from_numpy(x))
        ctx.stage_libm_sincosf(x_dev[:n], s_dev[:n], c_dev[:n])
        ctx.synchronize()
        s_ref, c_ref = O.libm_sincosf(x)
        s = s_dev[:n].cpu().numpy()
        c = c_dev[:n].cpu().numpy()
        bad += int(np.count_nonzero(s.view(np.uint32) != s_ref.view(np.uint32)))
        bad += int(np.count_nonzero(c.view(np.uint32) != c_ref.view(np.uint32)))
    return bad


@pytest.mark.parametrize("sign", [0, 1])
def test_libm_sincosf_exhaustive(gpu_context, sign):
    bad = _check_range(gpu_context, 0, MAX_ABS_BITS + 1, sign)
    assert bad == 0, f"{bad} results differ from the C library's"


def test_libm_sincosf_outside_interval(gpu_context):
    """Beyond [-pi, pi] (never reached by the moments of a non-negative density) the results stay within one ulp of
    the C library's."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(3.1416, 1e4, 100000), -rng.uniform(3.1416, 1e4, 100000)]).astype(np.float32)
    x_dev = torch.from_numpy(x).cuda()
    s_dev = torch.empty_like(x_dev)
    c_dev = torch.empty_like(x_dev)
    gpu_context.stage_libm_sincosf(x_dev, s_dev, c_dev)
    gpu_context.synchronize()
    s_ref, c_ref = O.libm_sincosf(x)
    for got, ref in ((s_dev.cpu().numpy(), s_ref), (c_dev.cpu().numpy(), c_ref)):
        ulps = np.abs(got.view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64))
        assert ulps.max() <= 1
