"""mraygb_stage_compact_noalloc: the compaction entry point for callers that cannot allocate device memory while
they work (their memory is reserved up front in their own pool).  It must give exactly what the allocating entry
point gives, on consecutive calls (the shared scratch array keeps the previous call's contents), and must reject
images above its fixed limit.  Collected last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _noalloc(L, stream, W, H, m, counts, moments, index, compact):
    total = C.c_uint64()
    st = L.mraygb_stage_compact_noalloc(stream, W, H, m, counts.data_ptr(), moments.data_ptr(), index.data_ptr(),
                                        compact.data_ptr(), compact.numel(), C.byref(total))
    return st, int(total.value)


# (4096, 4096, 1) is the limit: the only size whose scan takes three levels and nearly all 16448 words of the
# array (16394); (2111, 37, 31) spans several 2048-pixel tiles with a ragged last tile.
@pytest.mark.parametrize("shape", [(517, 389, 7), (1024, 1024, 4), (2111, 37, 31), (4096, 4096, 1)])
def test_noalloc_compaction_matches_the_allocating_entry_point(shape):
    import mray_gb300 as M
    from mray_gb300 import _lib

    L = _lib.load()
    W, H, m = shape
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    ctx = M.Context(0)
    ctx.set_stream(stream)
    try:
        rng = np.random.default_rng(W * H + m)
        for call in range(2):  # two calls in a row: the second must not see the first's scratch contents
            counts = (rng.integers(0, m + 1, size=W * H) * (rng.random(W * H) < 0.8 - 0.3 * call)).astype(np.int32)
            moments = torch.from_numpy(rng.standard_normal(W * H * m).astype(np.float32)).cuda()
            d_counts = torch.from_numpy(counts).cuda()
            idx_a = torch.zeros(W * H + 1, dtype=torch.int32, device="cuda")
            out_a = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
            idx_b = torch.full((W * H + 1,), -1, dtype=torch.int32, device="cuda")
            out_b = torch.full((W * H * m,), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            total_a = ctx.stage_compact(W, H, m, d_counts, moments, idx_a, out_a)
            ctx.synchronize()
            st, total_b = _noalloc(L, stream.cuda_stream, W, H, m, d_counts, moments, idx_b, out_b)
            stream.synchronize()
            assert st == 0
            assert total_b == total_a == int(counts.sum())
            assert torch.equal(idx_a, idx_b)
            assert torch.equal(out_a[:total_a], out_b[:total_b])
    finally:
        ctx.close()


def test_noalloc_rejects_images_above_its_limit():
    from mray_gb300 import _lib

    L = _lib.load()
    tiny = torch.zeros(8, dtype=torch.int32, device="cuda")
    tinyf = torch.zeros(8, dtype=torch.float32, device="cuda")
    total = C.c_uint64()
    st = L.mraygb_stage_compact_noalloc(None, 4097, 4096, 1, tiny.data_ptr(), tinyf.data_ptr(), tiny.data_ptr(),
                                        tinyf.data_ptr(), 8, C.byref(total))
    assert st == 1  # MRAYGB_INVALID_ARGUMENT, before any device work
