"""Moment-image files through the C ABI against the reference's write_moment_image / load_moment_image
(moment_image_io.cpp:291-529; fixture tests/golden/file_format.npz, written by the reference with its LZ4 calls
served by oracle/lz4_ref.c): raw, quantized (prediction codes and the plain quantizer) and entropy-coded payloads,
compact and static images, with and without compression and the global quantization table.

Uncompressed files are byte-identical to the reference's.  Compressed sections are LZ4 blocks of this library's
encoder, so those files are compared by content: the header, and every image the reference's loader returned equals
what this loader returns for the reference's file and for its own (bit-exact floats)."""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# name, image, compress, bits, entropy, with the table (the same cases as tests/golden/make_golden.py)
CASES = [
    ("pc_raw", "pc", 0, 32, 0, False), ("pc_raw_lz4", "pc", 1, 32, 0, False), ("pc_q10", "pc", 0, 10, 0, False),
    ("pc_q10_lz4", "pc", 1, 10, 0, False), ("plain_raw", "plain", 0, 32, 0, False),
    ("plain_q12", "plain", 0, 12, 0, False), ("plain_q12_lz4", "plain", 1, 12, 0, False),
    ("plain_ac10", "plain", 0, 10, 1, False), ("plain_ac10_lz4", "plain", 1, 10, 1, False),
    ("static_raw", "static", 0, 32, 0, False), ("static_lz4", "static", 1, 32, 0, False),
    ("static_q16_lz4", "static", 1, 16, 0, False),
    ("pc_table", "pc", 0, 10, 0, True), ("pc_table_ac", "pc", 0, 10, 1, True), ("pc_table_ac_lz4", "pc", 1, 10, 1, True),
    ("plain_q12_table", "plain", 0, 12, 0, True),
]


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "file_format.npz"))


def _image(M, g, kind):
    Wd, H, m = (int(v) for v in g["shape"])
    dom = g["domain"]
    compact = kind != "static"
    mi = M.MomentImageHost(Wd, H, m, compact, compact)
    mi.data = g[f"{kind}_data"].copy()
    mi.is_compact = compact
    mi.domain_min, mi.domain_max = tuple(map(float, dom[0])), tuple(map(float, dom[1]))
    if compact:
        mi.index = g[f"{kind}_index"].copy()
        mi.bounds = g[f"{kind}_bounds"].reshape(-1, 2).copy()
    if kind == "pc":
        mi.prediction_code, mi.coding_warp, mi.coding_params = True, 0, g["pc_coding_params"].copy()
    if kind == "plain":
        mi.error_bounds = g["error_bounds"].copy()
    return mi


def _whole_codes(mi, bits, entropy, table):
    """Values whose packed code lies inside the payload's whole bytes (quantize_prediction_coding and quantize pack
    codes in the order of the moment data and drop a trailing partial byte, moment_quantization.cpp:68-114)."""
    n = mi.data.size
    if bits == 32 or entropy or not mi.is_compact:
        return np.ones(n, bool)
    counts = np.diff(mi.index.astype(np.int64))
    l = np.arange(n) - np.repeat(mi.index[:-1].astype(np.int64), counts)
    if mi.prediction_code:
        t = table if table is not None else np.array([16] + [bits] * (mi.num_moments - 1))
        per = np.asarray(t, np.int64)[l]
    else:
        per = np.full(n, bits, np.int64)
    end = np.cumsum(per)
    return end <= (end[-1] // 8) * 8


def _same_image(a, b):
    assert (a.width, a.height, a.num_moments, a.is_compact, a.prediction_code, a.coding_warp) == \
        (b.width, b.height, b.num_moments, b.is_compact, b.prediction_code, b.coding_warp)
    assert np.array_equal(a.data.view(np.uint32), b.data.view(np.uint32))
    for field in ("index", "bounds", "error_bounds", "coding_params"):
        x, y = getattr(a, field), getattr(b, field)
        assert (x is None) == (y is None), field
        if x is not None:
            assert np.array_equal(x, y), field


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_files_against_reference(gpu_context, g, case):
    import mray_gb300 as M

    name, kind, compress, bits, entropy, use_table = case
    mi = _image(M, g, kind)
    table = g["table"] if use_table else None
    ours = gpu_context.encode_moment_image(mi, compress, bits, entropy, table)
    ref = g[f"file_{name}"].tobytes()
    assert ours[:32] == ref[:32]  # the header
    if not compress:
        assert ours == ref
    if name == "static_q16_lz4":
        # the bits byte, then one LZ4 block of the byte-aligned codes: the same codes in both
        size = mi.width * mi.height * mi.num_moments * 2
        assert ours[32] == ref[32] == 16
        assert O.lz4_decompress(ours[33:], size) == O.lz4_decompress(ref[33:], size) is not None
        with pytest.raises(M.MrayError) as e:  # the reference's reader decodes from the bits byte
            gpu_context.decode_moment_image(ref)
        assert e.value.status == 6
        return
    info = g[f"loaded_{name}_info"]
    loaded = g[f"loaded_{name}_data"]
    whole = _whole_codes(mi, bits, entropy, table)
    for data in (ref, ours):
        back, t = gpu_context.decode_moment_image(data)
        assert [back.width, back.height, back.num_moments, back.is_compact, back.prediction_code,
                back.coding_warp, back.bounds is not None, back.error_bounds is not None,
                back.coding_params is not None] == [int(v) for v in info]
        assert np.array_equal(back.data[whole].view(np.uint32), loaded[whole].view(np.uint32))
        # the code cut by the packer's last partial byte: the reference reads past its unpacked codes there
        # (moment_quantization.cpp:316-327, undefined); this loader gives 0
        assert np.all(back.data[~whole] == 0)
        assert (t is not None) == use_table
        if use_table:
            assert np.array_equal(t, g["table"])
    back_ref, _ = gpu_context.decode_moment_image(ref)
    back_ours, _ = gpu_context.decode_moment_image(ours)
    _same_image(back_ref, back_ours)
    if bits == 32 and not entropy:
        _same_image(back_ours, mi)


def test_path_calls_and_module_functions(gpu_context, g, tmp_path):
    import mray_gb300 as M

    mi = _image(M, g, "pc")
    path = str(tmp_path / "pc.mom")
    M.write_moment_image(mi, path, True, 10, True, table=g["table"], context=gpu_context)
    with open(path, "rb") as f:
        assert f.read() == gpu_context.encode_moment_image(mi, True, 10, True, g["table"])
    back, table = M.load_moment_image(path, context=gpu_context)
    assert np.array_equal(table, g["table"])
    assert np.array_equal(back.data, g["loaded_pc_table_ac_lz4_data"])


def test_large_image_round_trips(gpu_context):
    """A 256 x 256, 64-moment prediction-coded image from the GPU pipeline: packed 10-bit codes and the entropy
    coder with a ragged table both come back as the oracle's dequantize(quantize(x)), bit for bit; the entropy coder
    beats the packed codes on size."""
    import mray_gb300 as M
    from helpers import small_mixing

    wl = small_mixing(256, 256, 64, 96)
    wl.gen.prediction_coding = 1
    gpu_context.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    mi = gpu_context.generate(wl.camera, wl.gen, wl.width, wl.height, 64)
    mi.domain_min, mi.domain_max = wl.domain_min, wl.domain_max
    sizes = {}
    for table, entropy in ((np.array([16] + [10] * 63, np.uint8), False),
                           (np.array([16] + [14, 12, 11] + [10] * 20 + [8] * 40, np.uint8), False),
                           (np.array([16] + [14, 12, 11] + [10] * 20 + [8] * 40, np.uint8), True)):
        packed = O.quantize_prediction_coding(wl.width, wl.height, 64, mi.index, mi.data, table)
        want = O.dequantize_prediction_coding(wl.width, wl.height, 64, mi.index, table, packed, mi.data.size)
        if entropy:
            # the packed stream drops its trailing partial byte (pack_bits, moment_quantization.cpp:92-114), so the
            # last code or two read back as 0 there; the entropy coder keeps every code whole
            cut = np.flatnonzero(O.unpack_codes(wl.width, wl.height, 64, mi.index, table, packed) < 0)
            syms = O.entropy_codes(wl.width, wl.height, 64, mi.index, mi.data, table, True)
            last = mi.index[np.searchsorted(mi.index, cut, side="right") - 1]
            want = want.copy()
            for i, l in zip(cut, cut - last):
                want[i] = O.lib().oracle_dequantize(int(syms[i]), int(table[l]), 0.0, 1.0)
        for compress in (False, True):
            blob = gpu_context.encode_moment_image(mi, compress, 10, entropy, table)
            back, t = gpu_context.decode_moment_image(blob)
            assert np.array_equal(back.data.view(np.uint32), want.view(np.uint32)), (entropy, compress)
            assert np.array_equal(back.index, mi.index) and np.array_equal(back.bounds, mi.bounds)
            assert np.array_equal(back.coding_params, mi.coding_params)
            assert np.array_equal(t, table)
            sizes[(int(table[1]), entropy, compress)] = len(blob)
    # the arithmetic coder takes fewer bytes than the packed codes of the same table
    assert sizes[(14, True, False)] < sizes[(14, False, False)]


def test_errors(gpu_context, g):
    import mray_gb300 as M

    pc = _image(M, g, "pc")
    with pytest.raises(M.MrayError) as e:  # entropy coding of prediction codes needs the table
        gpu_context.encode_moment_image(pc, False, 10, True, None)
    assert e.value.status == 1
    with pytest.raises(M.MrayError) as e:  # more than 14 bits per entropy-coded symbol
        gpu_context.encode_moment_image(_image(M, g, "plain"), False, 15, True, None)
    assert e.value.status == 1
    with pytest.raises(M.MrayError) as e:
        gpu_context.encode_moment_image(pc, False, 33, False, None)
    assert e.value.status == 1
    ref = g["file_pc_q10_lz4"].tobytes()
    for cut in (10, 40, len(ref) // 2):
        with pytest.raises(M.MrayError) as e:
            gpu_context.decode_moment_image(ref[:cut])
        assert e.value.status == 1
    # the context stays usable
    back, _ = gpu_context.decode_moment_image(ref)
    whole = _whole_codes(pc, 10, False, None)
    assert np.array_equal(back.data[whole], g["loaded_pc_q10_lz4_data"][whole])


@pytest.mark.parametrize("m", [1, 255])
@pytest.mark.parametrize("compact,pc", [(True, True), (True, False), (False, False)], ids=["pc", "plain", "static"])
def test_round_trip_at_the_moment_limits(gpu_context, m, compact, pc):
    """One moment and 255 (the file's 8-bit moment count, moment_image_io.cpp:346-359): raw files round-trip bit for
    bit, compressed or not; quantized and entropy-coded compact images decode to the image's shape and index, and a
    second encoding of the decoded image gives the same file size.  Static images: raw files (their quantized files
    are taken apart by a bits byte, tested above)."""
    import mray_gb300 as M
    from helpers import small_mixing

    wl = small_mixing(20, 16, m, 64, seed=m)
    wl.gen.compact_image = int(compact)
    wl.gen.prediction_coding = int(pc)
    wl.gen.transform_to_bounds = int(compact)
    grid = M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max)
    mi = M.MomentImageHost(wl.width, wl.height, m, compact, compact)
    M.generate(wl.camera, grid, mi, wl.gen, context=gpu_context)
    for compress in (0, 1):
        back, _ = gpu_context.decode_moment_image(gpu_context.encode_moment_image(mi, compress, 32))
        _same_image(back, mi)
    if not compact:
        return
    for bits, entropy in ((10, 0), (16, 0), (10, 1)):
        table = np.array([16] + [bits] * (m - 1), dtype=np.uint8)[:m] if pc else None
        back, _ = gpu_context.decode_moment_image(gpu_context.encode_moment_image(mi, 1, bits, entropy, table))
        assert (back.width, back.height, back.num_moments, back.data.size) == (mi.width, mi.height, m, mi.data.size)
        assert np.array_equal(back.index, mi.index)
        assert np.all(np.isfinite(back.data))
        if not entropy:
            assert len(gpu_context.encode_moment_image(back, 1, bits, entropy, table)) > 0
            assert len(gpu_context.encode_moment_image(back, 0, bits, entropy, table)) == \
                len(gpu_context.encode_moment_image(mi, 0, bits, entropy, table))
