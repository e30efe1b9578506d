"""The oracle pinned to the reference's own CPU implementation (CPU only).

The fixtures in tests/golden/ were written by tests/golden/make_golden.py from the reference compiled from its
sources.  The oracle's f32 body must reproduce them bit for bit (it performs the reference's float operations in
the reference's order, built without contraction); the assertions of the reference's own unit tests are
re-checked on the same inputs.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
from mray_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def P(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture(scope="module")
def L():
    return O.lib()


@pytest.fixture(scope="module")
def ka():
    return load("known_answers.npz")


# ---- tests/test_mese.cpp ------------------------------------------------------------------------------------

@pytest.mark.parametrize("name", ["m4", "m10"])
def test_mese_prepare_and_evaluate(L, ka, name):
    mom = ka[f"mese_{name}_moments"]
    n = mom.size
    pm = np.zeros(n, np.float32)
    L.oracle_prepare_lagrange_f32(n, P(mom), P(pm))
    assert np.array_equal(pm, ka[f"mese_{name}_lagrange_dynamic"])
    # test_mese.cpp:31-57: the fixed-size code and the dynamic code agree on the value (ASSERT_FLOAT_EQ)
    p = np.float32(-np.pi + np.pi * 0.5)
    v = L.oracle_evaluate_mese_f32(n, float(p), P(ka[f"mese_{name}_lagrange_fixed"]), 0)
    assert np.float32(v) == ka[f"mese_{name}_value_dynamic"]
    assert abs(float(ka[f"mese_{name}_value_fixed"]) - float(v)) <= 4 * np.spacing(np.float32(v))


def test_mese_prepare_against_fixed_size_code(L, ka):
    """test_mese.cpp:185-206: the dynamic preparation within 1e-2 of the fixed-size code."""
    mom = ka["prep4_moments"]
    pm = np.zeros(4, np.float32)
    L.oracle_prepare_lagrange_f32(4, P(mom), P(pm))
    assert np.array_equal(pm, ka["prep4_dynamic"])
    assert np.abs(pm - ka["prep4_fixed"]).max() < 1e-2


@pytest.mark.parametrize("name", ["m4", "m10"])
def test_trig_to_exp_and_levinson_pinned(L, ka, name):
    mom = ka[f"mese_{name}_moments"]
    n = mom.size
    e = np.zeros(2 * n, np.float32)
    L.oracle_trig_to_exp_f32(n, P(mom), P(e))
    assert np.array_equal(e, ka[f"mese_{name}_exp_dynamic"])
    sol = np.zeros(2 * n, np.float32)
    L.oracle_levinson_f32(n, P(ka[f"mese_{name}_exp_fixed"]), P(sol))
    assert np.array_equal(sol, ka[f"mese_{name}_levinson_dynamic"])


def test_trig_to_exp_and_levinson_against_fixed_size_code(L, ka):
    """test_mese.cpp:59-75 (exponential moments, ASSERT_FLOAT_EQ) and :115-133 (Levinson within 1e-2)."""
    mom = ka["prep4_moments"]
    e = np.zeros(8, np.float32)
    L.oracle_trig_to_exp_f32(4, P(mom), P(e))
    assert np.array_equal(e, ka["prep4_exp_dynamic"])
    fixed = ka["prep4_exp_fixed"]
    assert np.all(np.abs(e - fixed) <= 4 * np.spacing(np.maximum(np.abs(e), np.abs(fixed))))
    sol = np.zeros(8, np.float32)
    L.oracle_levinson_f32(4, P(fixed), P(sol))
    assert np.array_equal(sol, ka["prep4_levinson_dynamic"])
    assert np.abs(sol - ka["prep4_levinson_fixed"]).max() < 1e-2


def test_exp_trig_round_trip(L, ka):
    trig = ka["roundtrip28_trig"]
    e = np.zeros(56, np.float32)
    L.oracle_trig_to_exp_f32(28, P(trig), P(e))
    assert np.array_equal(e, ka["roundtrip28_exp"])
    back = np.zeros(56, np.float32)
    L.oracle_exp_to_trig_f32(28, P(e), P(back))
    assert np.array_equal(back, ka["roundtrip28_back"])
    assert np.abs(back[0::2] - trig).max() < 0.01  # test_mese.cpp:111-112


def test_correlations(L, ka):
    lhs, rhs = ka["corr_lhs"], ka["corr_rhs"]
    a = np.zeros(8, np.float32)
    L.oracle_autocorrelation_f32(4, P(lhs), P(a))
    c = np.zeros(8, np.float32)
    L.oracle_correlation_f32(4, P(lhs), P(rhs), P(c))
    ic = np.zeros(4, np.float32)
    L.oracle_imaginary_correlation_f32(4, P(lhs), P(rhs), P(ic))
    assert np.array_equal(a, ka["autocorr"])
    assert np.array_equal(c, ka["corr"])
    assert np.array_equal(ic, ka["imag_corr"])


def test_fast_atan(L, ka):
    ys = np.array([L.oracle_fast_atan_f32(float(x)) for x in ka["fast_atan_x"]], np.float32)
    assert np.array_equal(ys, ka["fast_atan_y"])
    # "maximal absolute error around 1.1e-5" (complex_algebra.h:133); measured 1.21e-5
    assert np.abs(ys.astype(np.float64) - np.arctan(ka["fast_atan_x"].astype(np.float64))).max() < 1.25e-5


# ---- tests/test_prediction_coding.cpp -----------------------------------------------------------------------

@pytest.mark.parametrize("name", ["pc5", "pc5b"])
def test_prediction_coding_round_trip(L, ka, name):
    trig = ka[f"{name}_trig"]
    n = trig.size
    e = np.zeros(2 * n, np.float32)
    L.oracle_trig_to_exp_f32(n, P(trig), P(e))
    assert np.array_equal(e, ka[f"{name}_exp"])
    code = np.zeros(2 * n, np.float32)
    L.oracle_encode_f32(n, P(e), P(code))
    assert np.array_equal(code, ka[f"{name}_code"])
    dec = np.zeros(2 * n, np.float32)
    poly = np.zeros(2 * n, np.float32)
    L.oracle_decode_f32(n, P(code), P(dec), P(poly))
    assert np.array_equal(dec, ka[f"{name}_decoded"])
    assert np.array_equal(poly, ka[f"{name}_decoded_poly"])
    # test_prediction_coding.cpp:59-66: decoded exponential moments within 1e-6, m_1 = 0 stays exactly 0
    assert np.abs(dec - e).max() <= 1e-6
    if trig[1] == 0:
        assert e[2] == 0 and e[3] == 0 and code[2] == 0 and code[3] == 0
    real = np.zeros(n, np.float32)
    L.oracle_transform_quantization_real_f32(n, P(code), float(trig[0]), P(real))
    assert np.array_equal(real, ka[f"{name}_real"])
    # transform_quantization_real_warp with CODING_WARP_NONE: x * 0.5 + 0.5, clamped to [0, 1]
    warped = real.copy()
    warped[1:] = np.clip(real[1:] * np.float32(0.5) + np.float32(0.5), 0, 1)
    assert np.array_equal(warped, ka[f"{name}_warped_none"])
    back = np.zeros(2 * n, np.float32)
    L.oracle_transform_dequantization_real_f32(n, P(warped), P(back), 1, None)
    assert np.array_equal(back, ka[f"{name}_back_warp_none"])
    # test_prediction_coding.cpp:93-99: the real projection round trip within 1e-7 (indices >= 1)
    assert np.abs(back[2:] - code[2:]).max() <= 1e-7


# ---- tests/test_coding_transform.cpp ------------------------------------------------------------------------

def test_coding_transform_known_answer(ka):
    params = O.find_coding_transform_parameters(16, 1, 10, ka["ramp_index"], ka["ramp_data"])
    assert np.array_equal(params, ka["ramp_params"])
    assert np.abs(params[0::2] - 0.6).max() < 1e-6 and np.abs(params[1::2] - 0.5).max() < 1e-6


# ---- tests/test_moment_compaction.cpp -----------------------------------------------------------------------

def test_compaction_rrmse(L, ka):
    trig, e = ka["compaction_trig"], ka["compaction_exp"]
    got = np.zeros(20, np.float32)
    L.oracle_trig_to_exp_f32(10, P(trig), P(got))
    assert np.array_equal(got, e)
    rm = {}
    for n in (2, 8):
        ext = np.zeros(20, np.float32)
        L.oracle_evaluate_unknown_moments_f32(n, P(e), 10, P(ext))
        assert np.array_equal(ext, ka[f"compaction_ext{n}"])
        b = np.zeros(20, np.float32)
        b[0:2 * n:2] = trig[:n]
        L.oracle_exponential_to_bounded_moments_f32(10, P(ext), P(b), n)
        assert np.array_equal(b, ka[f"compaction_bounded{n}"])
        rm[n] = np.float32(L.oracle_rmse_f32(n, 10, P(b), P(trig)))
        assert rm[n] == ka[f"compaction_rmse{n}"]
    assert rm[8] < rm[2]  # test_moment_compaction.cpp:62
    for thr in (0.0, 0.05, 0.01, 0.001):
        assert L.oracle_determine_best_number_moments_f32(10, P(trig), thr) == int(ka[f"compaction_best_{thr}"])


# ---- tests/test_moment_image.cpp ----------------------------------------------------------------------------

def test_compaction_index_arithmetic():
    """test_moment_image.cpp:31-63: counts x per pixel of an 8x4 image with 10 moments."""
    w, h, m = 8, 4, 10
    counts = np.tile(np.arange(w, dtype=np.uint32), h).reshape(h, w)
    mo = np.zeros((h, w, m), np.float32)
    for x in range(w):
        mo[:, x, :x] = x / 8.0
    index, data = O.compact(counts, mo)
    assert data.size == counts.sum()
    assert np.array_equal(np.diff(index.astype(np.int64)).reshape(h, w), counts.astype(np.int64))
    assert index[1] == 0 and index[2] == 1 and index[3] == 3 and index[4] == 6


def test_quantize_dequantize_16bit():
    """test_moment_image.cpp:153-184: 16-bit prediction-coding quantization round trip within 1e-2."""
    w, h, m = 8, 4, 10
    counts = np.array([[x + 1 if x > 0 else 0 for x in range(w)]] * h, np.uint32)
    mo = np.zeros((h, w, m), np.float32)
    for x in range(w):
        mo[:, x, :x] = x / 8.0
    index, data = O.compact(counts, mo)
    table = O.default_quantization_table(m, 16)
    q = O.quantize_prediction_coding(w, h, m, index, data, table)
    back = O.dequantize_prediction_coding(w, h, m, index, table, q, data.size)
    for y in range(h):
        for x in range(w):
            i0 = index[y * w + x]
            for l in range(x):
                assert abs(back[i0 + l] - x / 8.0) < 1e-2


# ---- probes: overload choices, TF, sampling, rays -------------------------------------------------------------

def test_probes_match_reference_build():
    pr = load("probes.npz")
    L = O.lib()
    e = np.zeros(2, np.float32)
    for x, ref in zip(pr["euler_x"], pr["euler_y"]):
        L.oracle_euler_exp_f32(C.c_float(x), P(e))
        assert np.array_equal(e, ref)
    table = O.preintegrate(pr["tf1d"], 0.05)
    assert np.array_equal(table, pr["tf_row"]) and int(pr["tf_rows_equal"]) == 1
    out = np.zeros(4, np.float32)
    L.oracle_tf_sample_f32.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
    for (fs, bs), ref in zip(pr["tf_fs_bs"], pr["tf_samples"]):
        L.oracle_tf_sample_f32(P(table), fs, bs, P(out))
        assert np.array_equal(out, ref)
    vol = W.marschner_lobb(16)
    g, keep = O._grid(vol, (-1, -1, -1), (1, 1, 1))
    for p, ref in zip(pr["grid_points"], pr["grid_samples"]):
        assert np.float32(L.oracle_grid_sample_f32(C.byref(g), P(np.ascontiguousarray(p)))) == ref


def test_eye_rays_match_reference_build():
    pr = load("probes.npz")
    L = O.lib()
    L.oracle_eye_ray_f32.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.oracle_intersect_aabb_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    dmin = np.array([-1, -1, -1], np.float32)
    dmax = np.array([1, 1, 1], np.float32)
    for key, cam in (("ortho", W.ortho_camera(11)),
                     ("persp", W.perspective_camera((1.9, -1.1, 1.45), (0, 0, 0), 38.0, 1.0))):
        rays, hits = pr[f"rays_{key}"], pr[f"hits_{key}"]
        o = np.zeros(3, np.float32)
        d = np.zeros(3, np.float32)
        tn = C.c_float()
        tf = C.c_float()
        for y in range(9):
            for x in range(12):
                L.oracle_eye_ray_f32(C.byref(cam), x, y, 12, 9, P(o), P(d))
                hit = L.oracle_intersect_aabb_f32(P(o), P(d), P(dmin), P(dmax), C.byref(tn), C.byref(tf))
                assert np.array_equal(o, rays[x, y, :3]) and np.array_equal(d, rays[x, y, 3:6])
                assert hit == hits[x, y]
                assert np.float32(tn.value) == rays[x, y, 6] and np.float32(tf.value) == rays[x, y, 7]


# ---- whole pipeline ------------------------------------------------------------------------------------------

@pytest.mark.parametrize("fixture,kind", [("pipeline_ml.npz", "ml"), ("pipeline_mix.npz", "mix")])
def test_pipeline_bit_exact(fixture, kind):
    g = load(fixture)
    if kind == "ml":
        wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    else:
        wl = W.mixing_layer_workload(n=40, width=32, height=32, num_moments=64, modes=16, seed=5, name="golden_mix")
    tf = O.preintegrate(wl.tf1d, wl.tf_step)
    assert np.array_equal(tf, g["tf_table"])
    for pc in (0, 1):
        wl.gen.prediction_coding = pc
        mi = O.workload_generate(wl, "f32")
        k = f"pc{pc}"
        assert np.array_equal(mi["index"], g[f"{k}_index"])
        assert np.array_equal(mi["bounds"].reshape(-1), g[f"{k}_bounds"])
        assert np.array_equal(mi["data"], g[f"{k}_data"])
        if pc:
            assert np.array_equal(mi["coding_params"], g[f"{k}_coding_params"])
        pm = O.prepare_moments(wl.width, wl.height, wl.num_moments, mi["index"], mi["data"], bool(pc), 0,
                               mi["coding_params"], wl.rec.bias, "f32")
        assert np.array_equal(pm, g[f"{k}_pmoments"])
        rgba = O.reconstruct(wl.camera, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                             mi["index"], pm, mi["bounds"], tf, "f32")
        assert np.array_equal(rgba, g[f"{k}_rgba"])
        assert np.array_equal(O.rgba_to_u8(rgba), g[f"{k}_rgba8"])
        if pc:
            table = O.default_quantization_table(wl.num_moments, 10)
            q = O.quantize_prediction_coding(wl.width, wl.height, wl.num_moments, mi["index"], mi["data"], table)
            assert np.array_equal(q, g[f"{k}_codes_16_10"])


def test_quantize_tables_bit_exact():
    g = load("quantize.npz")
    Wd, H, m = (int(v) for v in g["shape"])
    for name in ("t16_10", "t_ragged", "t32", "t_odd"):
        q = O.quantize_prediction_coding(Wd, H, m, g["index"], g["values"], g[f"{name}_table"])
        assert np.array_equal(q, g[f"{name}_bytes"]), name


def test_fp64_oracle_agrees_with_fp32_on_smooth_case():
    """The f64 body is the same method: on the smooth Marschner-Lobb case the reference's FP32 moments sit within
    1e-4 (relative to m_0) of it."""
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11)
    m32, b32, c32 = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, 48, 40, 16, "f32")
    m64, b64, c64 = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, 48, 40, 16, "f64")
    hit = c32 > 0
    assert np.array_equal(c32, c64)
    err = np.abs(m32 - m64).max(axis=-1) / np.maximum(np.abs(m64[..., 0]), 1e-3)
    assert err[hit].max() < 1e-4


def _particle_fixture(g, prefix):
    from mray_gb300.types import Camera, GenerationParameters

    x, y, z, v = (np.ascontiguousarray(a) for a in g[f"{prefix}_xyzv"])
    dmin, dmax = g[f"{prefix}_domain"]
    parts = O.ParticleSet(x, y, z, v, float(g[f"{prefix}_h"]), tuple(dmin), tuple(dmax))
    cam = Camera.from_buffer_copy(g[f"{prefix}_camera"].tobytes())
    gen = GenerationParameters.from_buffer_copy(g[f"{prefix}_gen"].tobytes())
    return parts, cam, gen


def _particle_generate(parts, cam, gen, shape):
    Wd, H, m = (int(s) for s in shape)
    moments, bounds, counts = O.generate_moments_particles(cam, gen, parts, Wd, H, m, "f32")
    index, data = O.compact(counts, moments)
    return index, data, bounds.reshape(-1)


def test_particles_lattice_bit_exact():
    """One particle per grid cell: the reference's sort order is unique, so sample and moments are bit-exact."""
    g = load("particles.npz")
    parts, cam, gen = _particle_fixture(g, "lattice")
    s = O.particles_sample(parts, g["lattice_points"], "f32")
    assert np.array_equal(s, g["lattice_samples"])
    index, data, bounds = _particle_generate(parts, cam, gen, g["lattice_shape"])
    assert np.array_equal(index, g["lattice_index"])
    assert np.array_equal(bounds, g["lattice_bounds"])
    assert np.array_equal(data, g["lattice_data"])


def test_particles_clustered_within_summation_order():
    """Several particles per cell: the reference's std::sort leaves their order (and so the float summation
    order) unspecified; the oracle uses the input order.  Samples agree to a few ulp, the u16 bounds and the
    compaction exactly where the samples' bounds do."""
    g = load("particles.npz")
    parts, cam, gen = _particle_fixture(g, "cluster")
    s = O.particles_sample(parts, g["cluster_points"], "f32")
    ref = g["cluster_samples"]
    assert np.max(np.abs(s - ref) / np.maximum(np.abs(ref), 1e-30)) < 2e-6
    index, data, bounds = _particle_generate(parts, cam, gen, g["cluster_shape"])
    assert np.array_equal(index, g["cluster_index"])
    assert np.max(np.abs(bounds.astype(np.int64) - g["cluster_bounds"].astype(np.int64))) <= 1
    assert np.allclose(data, g["cluster_data"], rtol=0, atol=2e-5)


# ---- the data-dependent quantization curve (measure_coding_error.cpp) --------------------------------------------

def _sequential_mean(values):
    """get_mean (measure_coding_error.cpp:184-192): a float running sum divided by the count."""
    acc = np.float32(0)
    for v in values:
        acc = np.float32(acc + v)
    return np.float32(acc / np.float32(len(values)))


@pytest.mark.parametrize("key", ["mix", "mlthr"])
def test_quant_curve_sample_and_errors_bit_exact(key):
    g = load("quant_curve.npz")
    Wd, H, m, s = (int(v) for v in g[f"{key}_shape"])
    s_index, s_data = O.sample_moment_image(Wd, H, g[f"{key}_index"], g[f"{key}_data"], s)
    assert np.array_equal(s_index, g[f"{key}_s_index"])
    assert np.array_equal(s_data, g[f"{key}_s_data"])
    counts = np.diff(s_index.astype(np.int64))
    if key == "mlthr":  # error-threshold compaction leaves ragged moment counts
        assert len(set(counts[counts > 0].tolist())) > 3
    checked = 0
    for name in g.files:
        if not name.startswith(f"{key}_err_"):
            continue
        idx, b = (int(v) for v in name.split("_")[-2:])
        mean, errors = O.measure_idx_error(s, s, m, s_index, s_data, 0, g[f"{key}_coding_params"], idx, b)
        assert np.array_equal(errors, g[name]), name
        assert np.float32(mean) == _sequential_mean(g[name]), name
        checked += 1
    assert checked >= 7


def test_quant_curve_search_rule():
    """The table is create_quantization_table's search (measure_coding_error.cpp:400-435) over the means the oracle
    evaluated: [16, start_bits, ...]; each later index starts at the previous index's bits and steps down to 2 bits
    while the mean rRMSE stays below the threshold (the mean of index 1 at start_bits)."""
    g = load("quant_curve.npz")
    Wd, H, m, s = (int(v) for v in g["mix_shape"])
    for start_bits in (10, 6):
        table, means, evals = O.create_quantization_table(s, s, m, g["mix_s_index"], g["mix_s_data"], 0,
                                                          g["mix_coding_params"], start_bits)
        assert table[0] == 16 and table[1] == start_bits
        thr = means[1, start_bits]
        assert np.isfinite(thr) and thr > 0
        expect, visited = [16, start_bits], 1
        for idx in range(2, m):
            t = expect[-1]
            for b in range(expect[-1], 1, -1):
                visited += 1
                assert np.isfinite(means[idx, b]), (idx, b)
                if means[idx, b] >= thr:
                    break
                t = b
            expect.append(t)
        assert table.tolist() == expect
        assert evals == visited == np.count_nonzero(np.isfinite(means))
        assert 2 <= table[-1] < start_bits  # the curve does go down on this image


# ---- error bounds and uncertainty rendering (moment_raymarcher.cpp:516-717) ---------------------------------------

def test_error_bounds_and_uncertainty_bit_exact():
    from mray_gb300.types import ErrorReconstructionParameters, UncertaintyReconstructionParameters

    g = load("uncertainty.npz")
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    Wd, H, m = wl.width, wl.height, wl.num_moments
    tables = {et: O.uncertainty_tf(wl.tf1d, wl.tf_step, et) for et in (0, 1)}
    for et in (0, 1):
        assert np.array_equal(tables[et][::17], g[f"table{et}_rows"]), et
    row = O.preintegrate(wl.tf1d, wl.tf_step)
    for pc in (0, 1):
        idx, data, b = g[f"pc{pc}_index"], g[f"pc{pc}_data"], g[f"pc{pc}_bounds"]
        cp = g["pc1_coding_params"] if pc else None
        for et, pct in ((0, 90), (1, 90), (2, 90), (2, 50)):
            ep = ErrorReconstructionParameters(error_type=et, error_percentile=pct, step_size=wl.rec.step_size,
                                               bias=wl.rec.bias)
            _, eb = O.reconstruct_error(wl.camera, ep, wl.volume, wl.domain_min, wl.domain_max, Wd, H, m, idx, data,
                                        pc, 0, cp, b)
            assert np.array_equal(eb.reshape(-1), g[f"pc{pc}_eb{et}_{pct}"]), (pc, et, pct)
            assert eb.max() > 0
        for mode, et in ((0, 1), (1, 0), (1, 1), (1, 2)):
            up = UncertaintyReconstructionParameters(rec=wl.rec, error_type=et, bound_interpolation=0.3)
            table = row if mode == 0 else tables[1 if et == 1 else 0]
            rgba = O.reconstruct_uncertainty(wl.camera, up, mode, Wd, H, m, wl.domain_min, wl.domain_max, idx, data,
                                             g[f"pc{pc}_eb{et}_90"], pc, 0, cp, b, table)
            assert np.array_equal(rgba, g[f"pc{pc}_unc{mode}_{et}"]), (pc, mode, et)
    # the P^2 estimate moves with the percentile and stays below the maximum on average
    pct50, pct90 = g["pc0_eb2_50"].astype(float), g["pc0_eb2_90"].astype(float)
    assert pct50.mean() < pct90.mean() <= g["pc0_eb0_90"].astype(float).mean()


# ---- reference direct volume rendering (raymarch_reference.h) ------------------------------------------------------

def test_reference_dvr_bit_exact():
    from mray_gb300.types import ReferenceParameters, SingleScatteringParameters

    g = load("reference_dvr.npz")
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    row = O.preintegrate(wl.tf1d, wl.tf_step)
    cases = {"plain": dict(enable=0), "ss": dict(enable=1, henyey_greenstein_g=0.3, step_size_factor=2.0,
                                                   direction_x=0.3, direction_y=-1.0, direction_z=0.2)}
    for name, ss in cases.items():
        rp = ReferenceParameters(step_size=wl.rec.step_size, medium_emission=1.0, early_ray_termination=0.99,
                                 medium_scattering=0.5, ss=SingleScatteringParameters(**ss))
        rgba = O.generate_reference(wl.camera, rp, wl.volume, wl.domain_min, wl.domain_max, wl.width, wl.height, row)
        assert np.array_equal(rgba, g[f"{name}_rgba"]), name
    # in-scattered light brightens the image where the medium scatters
    assert g["ss_rgba"][..., :3].mean() > g["plain_rgba"][..., :3].mean()


# ---- single scattering from the transmittance cache (moment_raymarcher.cpp:217-351) ---------------------------------

def test_single_scattering_cache_bit_exact():
    """The cache of the light image (the reference's loop on one thread: the last write to a voxel wins), the
    re-march sampling it (float and the whole reconstruct(..., ss, ...) as u8) and the reference renderer sampling
    it, against the reference's own code."""
    from helpers import single_scattering_case

    g = load("single_scattering.npz")
    wl, light, rp = single_scattering_case()
    lw, lh, m = (int(v) for v in g["light_shape"])
    row = O.preintegrate(wl.tf1d, wl.tf_step)
    dmin, dmax = wl.domain_min, wl.domain_max
    lpm = O.prepare_moments(lw, lh, m, g["light_index"], g["light_data"], True, 0, g["light_coding_params"], rp.bias)
    cache = O.ss_cache(light, rp, lw, lh, m, dmin, dmax, g["light_index"], lpm, g["light_bounds"], row)
    assert np.array_equal(cache, g["cache"])
    epm = O.prepare_moments(wl.width, wl.height, m, g["eye_index"], g["eye_data"], bias=rp.bias)
    rgba = O.reconstruct(wl.camera, rp, wl.width, wl.height, m, dmin, dmax, g["eye_index"], epm, g["eye_bounds"], row,
                         cache=(cache, dmin, dmax))
    assert np.array_equal(rgba, g["rgba"])
    assert np.array_equal(O.rgba_to_u8(rgba), g["rgba8"])
    ref = O.generate_reference(wl.camera, O.ref_from_rec(rp), wl.volume, dmin, dmax, wl.width, wl.height, row,
                               cache=(cache, dmin, dmax))
    assert np.array_equal(ref, g["reference_rgba"])
    # the in-scattered light is there: without single scattering the image is darker
    rp.ss.enable = 0
    plain = O.reconstruct(wl.camera, rp, wl.width, wl.height, m, dmin, dmax, g["eye_index"], epm, g["eye_bounds"],
                          row)
    assert g["rgba"][..., :3].mean() > plain[..., :3].mean()
    # a transmittance in (0, 1] everywhere the light image reaches
    assert 0.0 < cache.min() and cache.max() <= 1.0


def test_single_scattering_cache_last_write_wins():
    """Many light pixels per voxel (a 3 x 2 x 4 cache): the rows decide in order.  Where one row of the light image
    writes, its values replace the earlier rows'; the other voxels keep the earlier rows' values."""
    from helpers import single_scattering_case

    g = load("single_scattering.npz")
    wl, light, rp = single_scattering_case(cache_size=(3, 2, 4))
    lw, lh, m = (int(v) for v in g["light_shape"])
    row = O.preintegrate(wl.tf1d, wl.tf_step)
    lpm = O.prepare_moments(lw, lh, m, g["light_index"], g["light_data"], True, 0, g["light_coding_params"], rp.bias)
    full = O.ss_cache(light, rp, lw, lh, m, wl.domain_min, wl.domain_max, g["light_index"], lpm, g["light_bounds"],
                      row)
    idx = g["light_index"].astype(np.int64)

    def rows(r0, r1):
        """the light image with only rows r0 .. r1 - 1 kept (the other pixels empty)"""
        keep = idx.copy()
        keep[:r0 * lw + 1] = idx[r0 * lw]
        keep[r1 * lw + 1:] = idx[r1 * lw]
        return O.ss_cache(light, rp, lw, lh, m, wl.domain_min, wl.domain_max, keep.astype(np.uint32), lpm,
                          g["light_bounds"], row)

    r = lh // 2
    upto, before, only = rows(0, r + 1), rows(0, r), rows(r, r + 1)
    hit = only != 0
    assert hit.any() and not hit.all()
    # where row r writes, its values win over the earlier rows'; elsewhere the earlier rows' stay
    assert np.array_equal(upto[hit], only[hit])
    assert np.array_equal(upto[~hit], before[~hit])
    assert not np.array_equal(before[hit], only[hit])
    assert np.array_equal(rows(0, lh), full)


# ---- tests/test_error_measures.cpp ------------------------------------------------------------------------------

def test_p2_percentile_worked_example():
    """The reference's own check of its P-squared median (tests/test_error_measures.cpp:29-87, the worked example of
    Jain and Chlamtac, with the paper's typo corrected as the reference does): the estimate after each of updates
    6..20 within 0.01."""
    values = [0.02, 0.15, 0.74, 3.39, 0.83, 22.37, 10.15, 15.43, 38.62, 15.92, 34.60, 10.28, 1.47, 0.40, 0.05, 11.39,
              0.27, 0.42, 0.09, 11.37]
    expected = [0.74, 0.74, 2.18, 4.75, 4.75, 9.28, 9.28, 9.28, 9.28, 6.3, 6.3, 6.3, 6.3, 4.44, 4.44]
    for precision in ("f32", "f64"):
        est = O.error_stream(2, 50, np.array(values, np.float32), precision)
        assert np.allclose(est[5:], expected, atol=0.01), (precision, est[5:])
    # max and RMSE on the same stream
    v = np.array(values, np.float32)
    assert O.error_stream(0, 50, v)[-1] == v.max()
    assert abs(O.error_stream(1, 50, v, "f64")[-1] - np.sqrt(np.mean(v.astype(np.float64) ** 2))) < 1e-12
