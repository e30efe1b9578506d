"""The host pieces of the moment-image file format, on the CPU: the entropy-coded payload against the reference's
own entropy_encode (moment_image_coding.cpp:206-221, fixture tests/golden/file_format.npz) byte for byte, its
decoder, and the LZ4 block codec against the oracle's independent LZ4 implementation (oracle/lz4_ref.c).
The GPU quantization of the payload and whole files are tested in test_gpu_file_format.py."""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "file_format.npz"))


@pytest.fixture(scope="module")
def M():
    import mray_gb300 as M

    return M


def _codes(g, kind):
    Wd, H, m = (int(v) for v in g["shape"])
    table = g[f"entropy_{kind}_table"]
    return O.entropy_codes(Wd, H, m, g[f"{kind}_index"], g[f"{kind}_data"], table, kind == "pc"), table


@pytest.mark.parametrize("kind", ["plain", "pc"])
@pytest.mark.parametrize("threads", [1, 5])
def test_entropy_payload_equals_reference(g, M, kind, threads):
    """One adaptive arithmetic-coded stream per moment index (2^bits symbols: 10 bits for the plain image, the
    ragged 5..14-bit table for the prediction-coded one): the same bytes as the reference's coder."""
    Wd, H, m = (int(v) for v in g["shape"])
    codes, table = _codes(g, kind)
    ours = M.entropy_encode(Wd, H, m, g[f"{kind}_index"], codes, table, threads=threads)
    assert ours == g[f"entropy_{kind}"].tobytes()


@pytest.mark.parametrize("kind", ["plain", "pc"])
def test_entropy_decode_of_reference_payload(g, M, kind):
    Wd, H, m = (int(v) for v in g["shape"])
    codes, table = _codes(g, kind)
    back = M.entropy_decode(g[f"entropy_{kind}"].tobytes(), Wd, H, m, g[f"{kind}_index"], table)
    assert np.array_equal(back, codes)


def test_entropy_round_trip_many_symbols(M):
    """A larger ragged image: skewed symbol statistics (many model rebuilds and count halvings past 2^17), counts
    from 0 to m, 14-bit alphabets."""
    rng = np.random.default_rng(3)
    Wd, H, m = 96, 80, 9
    counts = rng.integers(0, m + 1, Wd * H)
    index = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    table = np.array([16, 14, 12, 10, 8, 6, 4, 2, 1], np.uint8)
    codes = np.zeros(int(index[-1]), np.uint16)
    for p in range(Wd * H):
        for l in range(counts[p]):
            b = int(table[l])
            codes[index[p] + l] = min(int(rng.geometric(0.05)), (1 << b) - 1) if l else rng.integers(0, 1 << 16)
    payload = M.entropy_encode(Wd, H, m, index, codes, table)
    assert np.array_equal(M.entropy_decode(payload, Wd, H, m, index, table), codes)
    # the zeroth codes are stored as they are, the skewed streams compress
    assert len(payload) < 2 * codes.size


def test_entropy_rejects_bad_input(M):
    index = np.array([0, 2, 4], np.uint32)
    codes = np.zeros(4, np.uint16)
    with pytest.raises(M.MrayError):
        M.entropy_encode(2, 1, 2, index, codes, np.array([16, 15], np.uint8))  # 2^15 symbols: above 2^14
    with pytest.raises(M.MrayError):
        M.entropy_encode(2, 1, 2, np.array([0, 3, 4], np.uint32), codes, np.array([16, 8], np.uint8))
    good = M.entropy_encode(2, 1, 2, index, codes, np.array([16, 8], np.uint8))
    with pytest.raises(M.MrayError):
        M.entropy_decode(good[:5], 2, 1, 2, index, np.array([16, 8], np.uint8))


def _inputs():
    rng = np.random.default_rng(11)
    text = (b"moment images of a mixing layer; " * 5000)[:150000]
    yield "empty", b""
    yield "short", b"0123456789ab"
    yield "thirteen", b"aaaaaaaaaaaaa"
    yield "zeros", bytes(300000)
    yield "random", rng.integers(0, 256, 70000, dtype=np.uint8).tobytes()
    yield "text", text
    far = rng.integers(0, 256, 40000, dtype=np.uint8).tobytes()
    yield "repeat_beyond_window", far + bytes(70000) + far  # the repeat is 110 KB back: outside the 64 KiB window
    yield "codes", (rng.integers(0, 1024, 200000) // 3).astype(np.uint16).tobytes()


@pytest.mark.parametrize("name,data", list(_inputs()), ids=[n for n, _ in _inputs()])
def test_lz4_against_independent_codec(M, name, data):
    ours = M.lz4_compress(data)
    assert O.lz4_decompress(ours, len(data)) == data
    assert M.lz4_decompress(ours, len(data)) == data
    theirs = O.lz4_compress(data)
    assert M.lz4_decompress(theirs, len(data)) == data
    if name in ("zeros", "text"):
        assert len(ours) < len(data) // 20


def test_lz4_malformed_blocks(M):
    data = (b"abcdefgh" * 1000) + bytes(range(256))
    block = M.lz4_compress(data)
    for cut in (1, 2, len(block) // 2, len(block) - 1):
        with pytest.raises(M.MrayError):
            M.lz4_decompress(block[:cut], len(data))
    with pytest.raises(M.MrayError):  # the output does not fit
        M.lz4_decompress(block, len(data) - 1)
    with pytest.raises(M.MrayError):  # an offset before the start of the output
        M.lz4_decompress(bytes([0x10, 0x41, 0x05, 0x00]), 100)


def test_reference_file_headers(g):
    """The header fields of the reference's files (moment_image_io.cpp:471-508) for the layouts the GPU tests read."""
    Wd, H, m = (int(v) for v in g["shape"])
    for name in ("pc_q10_lz4", "plain_ac10", "static_raw", "pc_table_ac"):
        f = g[f"file_{name}"]
        assert int(f[0]) | (int(f[1]) << 8) == Wd and int(f[2]) | (int(f[3]) << 8) == H and f[4] == m
    assert g["file_pc_q10_lz4"][6] == 1 | 2 | 4 | 16 | 128  # compressed, compact, prediction coded, bounds, params
    assert g["file_plain_ac10"][7] == 10 | 64  # 10 bits, entropy coded
    assert g["file_static_raw"][6] == 0 and g["file_static_raw"][7] == 32
    assert g["file_pc_table_ac"][7] == 10 | 64 | 128  # and the table follows the header
    assert g["file_plain_q12_table"][7] == 12 | 128  # the global table is written for a plain image too


def test_reference_coding_test_ramp(g, M):
    """The reference's own entropy-coding test (tests/test_moment_image_coding.cpp:30-64): a 16 x 16 ramp in ten
    prediction-coded moments, table [16, 11, ...]; the payload equals the reference's coder's and decodes to within
    0.1 of the input, as that test asks (here: to the quantizer's own resolution)."""
    data, table = g["entropy_ramp_data"], g["entropy_ramp_table"]
    Wd = H = 16
    m = 10
    index = np.arange(0, Wd * H * m + 1, m, dtype=np.uint32)
    codes = O.entropy_codes(Wd, H, m, index, data, table, True)
    payload = M.entropy_encode(Wd, H, m, index, codes, table)
    assert payload == g["entropy_ramp"].tobytes()
    back = M.entropy_decode(payload, Wd, H, m, index, table)
    L = O.lib()
    dec = np.array([L.oracle_dequantize(int(back[i]), int(table[i % m]), 0.0, 1.0) for i in range(back.size)])
    assert np.abs(dec - data).max() <= 0.1
    assert np.abs(dec - data)[np.arange(back.size) % m > 0].max() <= 1.0 / (2 ** 11 - 1)
