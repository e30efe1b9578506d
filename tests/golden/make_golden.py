"""Writes the golden fixtures of tests/golden/ from the reference's OWN CPU implementation.

The reference (TobiasRp/mray) is compiled from its sources by oracle/Makefile (`make ref`, sources staged by
oracle/stage_reference.py) into oracle/_ref/libmrayref.so together with a small C-ABI harness.  This script calls it
on seeded inputs and stores inputs and outputs as small .npz files:

  known_answers.npz   the inputs of the reference's own unit tests (tests/test_mese.cpp, test_prediction_coding.cpp,
                      test_coding_transform.cpp, test_moment_compaction.cpp) with the outputs of the dynamic MESE
                      code and of the independent fixed-size MESE code (mese/MESE_4_10.h) they compare against
  probes.npz          euler_exp / exp(-x) as the reference's build evaluates them, TF tables and samples,
                      grid samples and eye rays
  pipeline_ml.npz     generate() -> (compaction, prediction coding) -> prepare -> reconstruct on a Marschner-Lobb
                      64^3 volume, 48x40 orthographic image, 16 moments
  pipeline_mix.npz    the same on a 40^3 mixing layer, 32x32 perspective image, 64 moments
  quantize.npz        quantize_prediction_coding of a ragged compact image under several bit tables
  particles.npz       Particles::sample and generate() over SPH particles: a jittered lattice with one particle
                      per grid cell (so the reference's unstable sort by cell cannot change the summation order)
                      and a clustered set
  quant_curve.npz     prediction-coded images from generate() (one with error-threshold compaction), their
                      sample_moment_image and the per-pixel rRMSE of compute_coding_error for several (index, bits)
                      pairs (measure_coding_error.cpp needs HDF5, so the harness composes its loop from the
                      reference's own sample_moment_image, transform_dequantization_real, decode and
                      exponentialToTrigonometricMoments)
  reference_dvr.npz   generate_reference's direct volume rendering of the Marschner-Lobb volume, without and with
                      brute-force single scattering
  uncertainty.npz     error bounds of reconstruct_error (max, RMSE, P^2 percentile at 90 and 50), rows of the two
                      uncertainty tables of read_from_disk_uncertainty and the float colours of the interpolation
                      and convolution renderers on the Marschner-Lobb pipeline image

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from mray_gb300 import workloads as W  # noqa: E402

P = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731


def f32(*v):
    return np.array(v, dtype=np.float32)


def cplx(values):
    a = np.zeros(2 * len(values), dtype=np.float32)
    for i, v in enumerate(values):
        a[2 * i], a[2 * i + 1] = np.float32(complex(v).real), np.float32(complex(v).imag)
    return a


def declare(ref):
    u64, f, vp = C.c_uint64, C.c_float, C.c_void_p
    ref.ref_particles_sample.argtypes = [vp, vp, vp, vp, u64, f, vp, vp, vp, u64, vp]
    ref.ref_generate_particles.argtypes = [vp, vp, vp, vp, vp, vp, u64, f, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp,
                                           vp, vp]
    i = C.c_int
    ref.ref_reconstruct_error.argtypes = [vp, vp, vp, i, i, i, vp, vp, i, i, i, vp, vp, u64, vp, i, i, vp, vp]
    ref.ref_uncertainty_tf.argtypes = [vp, f, i, vp]
    ref.ref_reconstruct_uncertainty_float.argtypes = [vp, vp, i, i, i, i, vp, vp, u64, vp, vp, i, i, vp, vp, vp, vp,
                                                      vp]
    ref.ref_generate_reference_float.argtypes = [vp, vp, vp, i, i, i, vp, vp, i, i, vp, vp]
    ref.ref_ss_cache.argtypes = [vp, vp, i, i, i, vp, vp, u64, vp, i, i, vp, vp, vp, vp, vp]
    ref.ref_write_moment_image.argtypes = [C.c_char_p, i, i, i, i, i, i, vp, vp, vp, vp, u64, vp, vp, vp, i, i, i, vp]
    ref.ref_load_moment_image.argtypes = [C.c_char_p, vp, vp, vp, vp, vp, vp, vp, vp]
    ref.ref_entropy_encode.restype = u64
    ref.ref_entropy_encode.argtypes = [i, i, i, vp, vp, u64, i, vp, vp, u64]
    ref.ref_reconstruct_cached_float.argtypes = [vp, vp, i, i, i, vp, vp, u64, vp, i, i, vp, vp, vp, vp, vp, i, i, i,
                                                 vp, vp, vp]
    ref.ref_reconstruct_ss_u8.argtypes = [vp, vp, i, i, i, vp, vp, u64, vp, i, i, vp, vp, vp, vp, i, i, i, vp, vp,
                                          u64, vp, i, i, vp, vp, vp]
    ref.ref_generate_reference_cached_float.argtypes = [vp, vp, vp, i, i, i, vp, vp, i, i, vp, vp, i, i, i, vp, vp,
                                                        vp]
    ref.ref_sample_moment_image.restype = u64
    ref.ref_sample_moment_image.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, u64, C.c_int, vp, vp]
    ref.ref_coding_errors.restype = C.c_uint32
    ref.ref_coding_errors.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, u64, C.c_int, vp, C.c_int, C.c_int, vp]
    ref.ref_evaluate_mese.restype = C.c_float
    ref.ref_evaluate_mese.argtypes = [C.c_int, C.c_float, C.c_void_p]
    ref.ref_fixed_evaluate_lagrange.restype = C.c_float
    ref.ref_fixed_evaluate_lagrange.argtypes = [C.c_int, C.c_float, C.c_void_p]
    ref.ref_fast_atan.restype = C.c_float
    ref.ref_fast_atan.argtypes = [C.c_float]
    ref.ref_rmse.restype = C.c_float
    ref.ref_rmse.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    ref.ref_determine_best_number_moments.argtypes = [C.c_int, C.c_void_p, C.c_float]
    ref.ref_transform_quantization_real.argtypes = [C.c_int, C.c_void_p, C.c_float, C.c_void_p]
    ref.ref_euler_exp.argtypes = [C.c_float, C.c_void_p]
    ref.ref_exp_overload.restype = C.c_float
    ref.ref_exp_overload.argtypes = [C.c_float]
    ref.ref_grid_sample.restype = C.c_float
    ref.ref_preintegrate.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
    ref.ref_tf_sample.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
    ref.ref_tf_sample.restype = C.c_float
    ref.ref_quantize_prediction_coding.restype = C.c_uint64
    ref.ref_generate_grid.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    for name in ("ref_reconstruct_float", "ref_reconstruct_u8"):
        getattr(ref, name).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_uint64, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    ref.ref_prepare_moments.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                        C.c_int, C.c_void_p, C.c_float, C.c_void_p]
    ref.ref_prediction_encode.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                          C.c_float, C.c_void_p]
    ref.ref_find_coding_transform_parameters.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                         C.c_uint64, C.c_void_p]
    ref.ref_quantize_prediction_coding.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint64,
                                                   C.c_void_p, C.c_void_p]


def known_answers(ref):
    out = {}
    # tests/test_mese.cpp:31-57: fixed (MESE_4_10) vs dynamic preparation and evaluation at p = -pi/2
    for name, mom in (("m4", f32(0.5, 0.25, 0.25, 0.1)),
                      ("m10", f32(0.22008814, 0.0, 0.01400074, 0.00271224, 0.00426201, 0, 0, 0, 0, 0))):
        n = mom.size
        pm_fixed = np.zeros(n, np.float32)
        ref.ref_fixed_prepare_lagrange(n, P(mom), P(pm_fixed))
        pm_dyn = np.zeros(n, np.float32)
        ref.ref_prepare_lagrange(n, P(mom), P(pm_dyn))
        p = np.float32(-np.pi + np.pi * 0.5)
        out[f"mese_{name}_moments"] = mom
        out[f"mese_{name}_lagrange_fixed"] = pm_fixed
        out[f"mese_{name}_lagrange_dynamic"] = pm_dyn
        out[f"mese_{name}_value_fixed"] = np.float32(ref.ref_fixed_evaluate_lagrange(n, p, P(pm_fixed)))
        out[f"mese_{name}_value_dynamic"] = np.float32(ref.ref_evaluate_mese(n, p, P(pm_fixed)))
        e_fixed = np.zeros(2 * n, np.float32)
        ref.ref_fixed_trig_to_exp(n, P(mom), P(e_fixed))
        e_dyn = np.zeros(2 * n, np.float32)
        ref.ref_trig_to_exp(n, P(mom), P(e_dyn))
        out[f"mese_{name}_exp_fixed"] = e_fixed
        out[f"mese_{name}_exp_dynamic"] = e_dyn
        sol_fixed = np.zeros(2 * n, np.float32)
        ref.ref_fixed_levinson(n, P(e_fixed), P(sol_fixed))
        sol_dyn = np.zeros(2 * n, np.float32)
        ref.ref_levinson(n, P(e_fixed), P(sol_dyn))
        out[f"mese_{name}_levinson_fixed"] = sol_fixed
        out[f"mese_{name}_levinson_dynamic"] = sol_dyn
    # tests/test_mese.cpp:185-206: the 4-moment preparation compared with the fixed-size code
    prep4 = f32(0.22008814, 0.0, 0.01400074, 0.00271224)
    pf = np.zeros(4, np.float32)
    ref.ref_fixed_prepare_lagrange(4, P(prep4), P(pf))
    pd = np.zeros(4, np.float32)
    ref.ref_prepare_lagrange(4, P(prep4), P(pd))
    out.update(prep4_moments=prep4, prep4_fixed=pf, prep4_dynamic=pd)
    # tests/test_mese.cpp:59-75 and 115-133: exponential moments and Levinson on the same 4 moments
    ef = np.zeros(8, np.float32)
    ref.ref_fixed_trig_to_exp(4, P(prep4), P(ef))
    ed = np.zeros(8, np.float32)
    ref.ref_trig_to_exp(4, P(prep4), P(ed))
    lf = np.zeros(8, np.float32)
    ref.ref_fixed_levinson(4, P(ef), P(lf))
    ld = np.zeros(8, np.float32)
    ref.ref_levinson(4, P(ef), P(ld))
    out.update(prep4_exp_fixed=ef, prep4_exp_dynamic=ed, prep4_levinson_fixed=lf, prep4_levinson_dynamic=ld)
    # tests/test_mese.cpp:94-113: 28-moment exp <-> trig round trip
    trig28 = f32(5.2070445e-01, 7.4165657e-02, -1.3283056e-02, 1.2487045e-02, 1.3437086e-02, -9.5647079e-04,
                 -1.2216626e-03, 2.1146263e-03, -5.4606516e-04, 1.0199437e-02, 1.1894707e-02, -1.9188672e-02,
                 -5.5241492e-03, 2.8166445e-02, 6.7452774e-03, -1.9198583e-02, 4.3223342e-03, -6.1640824e-04,
                 7.8988671e-03, 2.4080461e-02, -9.6553434e-03, -1.9514188e-02, 1.1532067e-02, -4.1229022e-03,
                 2.3510400e-02, 1.7623754e-02, -1.4590423e-02, 1.1135901e-03)
    e28 = np.zeros(56, np.float32)
    ref.ref_trig_to_exp(28, P(trig28), P(e28))
    t28 = np.zeros(56, np.float32)
    ref.ref_exp_to_trig(28, P(e28), P(t28))
    out["roundtrip28_trig"], out["roundtrip28_exp"], out["roundtrip28_back"] = trig28, e28, t28
    # tests/test_mese.cpp:135-183: correlations on "any random signal"
    sig = cplx([2, 4, 8, 16])
    rhs = cplx([1, 42, 0.1, 0.2])
    a = np.zeros(8, np.float32)
    ref.ref_autocorrelation(4, P(sig), P(a))
    c = np.zeros(8, np.float32)
    ref.ref_correlation(4, P(sig), P(rhs), P(c))
    ic = np.zeros(4, np.float32)
    ref.ref_imaginary_correlation(4, P(sig), P(rhs), P(ic))
    out.update(corr_lhs=sig, corr_rhs=rhs, autocorr=a, corr=c, imag_corr=ic)
    # tests/test_prediction_coding.cpp:30-100: encode / decode / real projection
    for name, trig in (("pc5", f32(0.22, 0.0, 0.014, 0.0027, 0.004)),
                       ("pc5b", f32(0.22008814, 0.0, 0.01400074, 0.00271224, 0.00426201))):
        n = trig.size
        e = np.zeros(2 * n, np.float32)
        ref.ref_trig_to_exp(n, P(trig), P(e))
        code = np.zeros(2 * n, np.float32)
        ref.ref_encode(n, P(e), P(code))
        dec = np.zeros(2 * n, np.float32)
        poly = np.zeros(2 * n, np.float32)
        ref.ref_decode(n, P(code), P(dec), P(poly))
        real = np.zeros(n, np.float32)
        ref.ref_transform_quantization_real(n, P(code), trig[0], P(real))
        warped = real.copy()
        ref.ref_transform_quantization_real_warp(n, P(warped), 1, None)
        back = np.zeros(2 * n, np.float32)
        ref.ref_transform_dequantization_real(n, P(warped), P(back), 1, None)
        out.update({f"{name}_trig": trig, f"{name}_exp": e, f"{name}_code": code, f"{name}_decoded": dec,
                    f"{name}_decoded_poly": poly, f"{name}_real": real, f"{name}_warped_none": warped,
                    f"{name}_back_warp_none": back})
    # tests/test_coding_transform.cpp:32-62: ramp x/15 - 0.6 over 16 pixels x 10 moments -> (0.6, 0.5)
    w, h, m = 16, 1, 10
    counts = np.full(w * h, m, np.uint32)
    raw = np.repeat((np.arange(w, dtype=np.float32) / np.float32(w - 1) - np.float32(0.6)), m).astype(np.float32)
    index = np.zeros(w * h + 1, np.uint32)
    index[1:] = np.cumsum(counts)
    params = np.zeros(2 * (m - 1), np.float32)
    ref.ref_find_coding_transform_parameters(w, h, m, P(index), P(raw), raw.size, P(params))
    out.update(ramp_index=index, ramp_data=raw, ramp_params=params)
    # tests/test_moment_compaction.cpp:30-66: extrapolated tail rmse for n = 2 and n = 8
    trig10 = f32(1.9176584e-01, -3.7339486e-02, -1.4143054e-02, -1.6614912e-02, -2.2262430e-02, -1.2005451e-02,
                 -7.5180288e-03, 2.5505440e-02, 2.8378680e-02, 1.6212923e-02)
    e10 = np.zeros(20, np.float32)
    ref.ref_trig_to_exp(10, P(trig10), P(e10))
    out["compaction_trig"], out["compaction_exp"] = trig10, e10
    for n in (2, 8):
        ext = np.zeros(20, np.float32)
        ref.ref_evaluate_unknown_moments(n, P(e10), 10, P(ext))
        b = np.zeros(20, np.float32)
        b[0:2 * n:2] = trig10[:n]
        ref.ref_exponential_to_bounded_moments(10, P(ext), P(b), n)
        out[f"compaction_ext{n}"] = ext
        out[f"compaction_bounded{n}"] = b
        out[f"compaction_rmse{n}"] = np.float32(ref.ref_rmse(n, 10, P(b), P(trig10)))
    for thr in (0.0, 0.05, 0.01, 0.001):
        out[f"compaction_best_{thr}"] = np.int32(ref.ref_determine_best_number_moments(10, P(trig10), thr))
    xs = np.linspace(-40, 40, 801).astype(np.float32)
    out["fast_atan_x"] = xs
    out["fast_atan_y"] = np.array([ref.ref_fast_atan(float(x)) for x in xs], np.float32)
    return out


def probes(ref):
    out = {}
    rng = np.random.default_rng(0)
    xs = rng.uniform(-200, 0, 4000).astype(np.float32)
    e = np.zeros((xs.size, 2), np.float32)
    for i, x in enumerate(xs):
        ref.ref_euler_exp(float(x), P(e[i]))
    out["euler_x"], out["euler_y"] = xs, e
    ts = rng.uniform(0, 20, 2000).astype(np.float32)
    out["exp_x"] = ts
    out["exp_y"] = np.array([ref.ref_exp_overload(float(t)) for t in ts], np.float32)
    tf1d = W.transfer_function(7)
    row = np.zeros((256, 4), np.float32)
    same = ref.ref_preintegrate(P(tf1d), C.c_float(0.05), P(row))
    out["tf1d"], out["tf_row"], out["tf_rows_equal"] = tf1d, row, np.int32(same)
    fb = rng.uniform(-0.05, 1.05, size=(500, 2)).astype(np.float32)
    s = np.zeros((500, 4), np.float32)
    for i in range(500):
        ref.ref_tf_sample(P(row), float(fb[i, 0]), float(fb[i, 1]), P(s[i]))
    out["tf_fs_bs"], out["tf_samples"] = fb, s
    vol = W.marschner_lobb(16)
    pts = rng.uniform(-1.2, 1.2, size=(800, 3)).astype(np.float32)
    dmin, dmax = f32(-1, -1, -1), f32(1, 1, 1)
    ref.ref_grid_sample.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    out["grid_points"] = pts
    out["grid_samples"] = np.array([ref.ref_grid_sample(P(vol), 16, 16, 16, P(dmin), P(dmax), P(p)) for p in pts],
                                   np.float32)
    rays = []
    for cam in (W.ortho_camera(11), W.perspective_camera((1.9, -1.1, 1.45), (0, 0, 0), 38.0, 1.0)):
        r = np.zeros((12, 9, 8), np.float32)
        hits = np.zeros((12, 9), np.int32)
        ref.ref_eye_ray.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        for y in range(9):
            for x in range(12):
                hits[x, y] = ref.ref_eye_ray(C.byref(cam), x, y, 12, 9, P(dmin), P(dmax), P(r[x, y]))
        rays.append((r, hits))
    out["rays_ortho"], out["hits_ortho"] = rays[0]
    out["rays_persp"], out["hits_persp"] = rays[1]
    return out


def pipeline(ref, wl):
    out = {}
    Wd, H, m = wl.width, wl.height, wl.num_moments
    vol = np.ascontiguousarray(wl.volume)
    nz, ny, nx = vol.shape
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    tf = np.zeros((256, 4), np.float32)
    ref.ref_preintegrate(P(np.ascontiguousarray(wl.tf1d)), C.c_float(wl.tf_step), P(tf))
    out["tf_table"] = tf
    for pc in (0, 1):
        wl.gen.prediction_coding = pc
        data = np.zeros(Wd * H * m, np.float32)
        index = np.zeros(Wd * H + 1, np.uint32)
        bounds = np.zeros(2 * Wd * H, np.uint16)
        cp = np.zeros(2 * m, np.uint16)
        size = C.c_uint64()
        flags = np.zeros(4, np.int32)
        ref.ref_generate_grid(C.byref(wl.camera), C.byref(wl.gen), P(vol), nx, ny, nz, P(dmin), P(dmax), Wd, H, m,
                              P(data), P(index), P(bounds), P(cp), C.byref(size), P(flags))
        data = data[:size.value].copy()
        key = f"pc{pc}"
        out[f"{key}_index"], out[f"{key}_bounds"], out[f"{key}_data"] = index, bounds, data
        if pc:
            out[f"{key}_coding_params"] = cp[:2 * (m - 1)].copy()
        cpp = cp if pc else None
        pm = np.zeros(max(data.size, 1), np.float32)
        ref.ref_prepare_moments(Wd, H, m, P(index), P(data), data.size, pc, 0, P(cpp), C.c_float(wl.rec.bias), P(pm))
        out[f"{key}_pmoments"] = pm[:data.size]
        rgba = np.zeros((H, Wd, 4), np.float32)
        ref.ref_reconstruct_float(C.byref(wl.camera), C.byref(wl.rec), Wd, H, m, P(index), P(data), data.size,
                                  P(bounds), pc, 0, P(cpp), P(dmin), P(dmax), P(tf), P(rgba))
        out[f"{key}_rgba"] = rgba
        u8 = np.zeros((H, Wd, 4), np.uint8)
        ref.ref_reconstruct_u8(C.byref(wl.camera), C.byref(wl.rec), Wd, H, m, P(index), P(data), data.size,
                               P(bounds), pc, 0, P(cpp), P(dmin), P(dmax), P(tf), P(u8))
        out[f"{key}_rgba8"] = u8
        if pc:
            table = np.array([16] + [10] * (m - 1), np.uint8)
            n = ref.ref_quantize_prediction_coding(Wd, H, m, P(index), P(data), data.size, P(table), None)
            q = np.zeros(max(n, 1), np.uint8)
            ref.ref_quantize_prediction_coding(Wd, H, m, P(index), P(data), data.size, P(table), P(q))
            out[f"{key}_codes_16_10"] = q[:n]
    wl.gen.prediction_coding = 0
    return out


def _particle_case(ref, prefix, x, y, z, v, h, dmin, dmax, cam, gen, Wd, H, m, rng):
    out = {}
    n = x.size
    out[f"{prefix}_xyzv"] = np.stack([x, y, z, v])
    out[f"{prefix}_h"] = np.float32(h)
    out[f"{prefix}_domain"] = np.stack([dmin, dmax])
    lo, hi = dmin - np.float32(0.05), dmax + np.float32(0.05)
    pts = (lo + (hi - lo) * rng.random((400, 3))).astype(np.float32)
    pts[:50] = np.stack([x[:50], y[:50], z[:50]], axis=1)  # exactly on particles (zero distance)
    samples = np.zeros(pts.shape[0], np.float32)
    ref.ref_particles_sample(P(x), P(y), P(z), P(v), n, C.c_float(h), P(dmin), P(dmax), P(pts), pts.shape[0],
                             P(samples))
    out[f"{prefix}_points"], out[f"{prefix}_samples"] = pts, samples
    data = np.zeros(Wd * H * m, np.float32)
    index = np.zeros(Wd * H + 1, np.uint32)
    bounds = np.zeros(2 * Wd * H, np.uint16)
    size = C.c_uint64()
    ref.ref_generate_particles(C.byref(cam), C.byref(gen), P(x), P(y), P(z), P(v), n, C.c_float(h), P(dmin),
                               P(dmax), Wd, H, m, P(data), P(index), P(bounds), C.byref(size))
    out[f"{prefix}_camera"] = np.frombuffer(bytes(cam), np.uint8).copy()
    out[f"{prefix}_gen"] = np.frombuffer(bytes(gen), np.uint8).copy()
    out[f"{prefix}_shape"] = np.array([Wd, H, m], np.int32)
    out[f"{prefix}_data"], out[f"{prefix}_index"], out[f"{prefix}_bounds"] = data[:size.value].copy(), index, bounds
    return out


def particles(ref):
    out = {}
    rng = np.random.default_rng(77)
    # one particle per cell: positions (i + 0.25 + 0.5 u) h, so (p - min) / h stays inside [i, i + 0.5)
    side, h = 10, np.float32(0.1)
    ii = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 3)
    pos = ((ii + 0.25 + 0.5 * rng.random(ii.shape)) * float(h)).astype(np.float32)
    pos[0] = np.float32(0.25) * h  # cell (0, 0, 0): the grid origin is exactly 0.25 h on every axis
    perm = rng.permutation(pos.shape[0])
    pos = pos[perm]
    x, y, z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    v = rng.lognormal(0.0, 0.5, size=x.size).astype(np.float32)
    gmin = np.array([x.min(), y.min(), z.min()], np.float32)
    inv = np.float32(1.0 / float(h))
    cells = ((pos - gmin).astype(np.float32) * inv).astype(np.int32)
    assert len({tuple(c) for c in cells}) == x.size, "lattice cells collide"
    wl = W.sph_workload(n=64, h=float(h), width=24, height=20, num_moments=8, seed=3)
    dmin, dmax = f32(0, 0, 0), f32(1, 1, 1)
    gen = wl.gen
    gen.step_size = float(h) / 2
    gen.data_min, gen.data_max = 0.3, 3.0
    out.update(_particle_case(ref, "lattice", x, y, z, v, float(h), dmin, dmax, wl.camera, gen, 24, 20, 8, rng))
    # clustered: 70 % uniform, 30 % in Gaussian clusters; ties inside a cell (summation order unpinned)
    wl = W.sph_workload(n=3000, h=1.0 / 16, width=24, height=20, num_moments=8, seed=9)
    out.update(_particle_case(ref, "cluster", wl.x, wl.y, wl.z, wl.v, wl.h, f32(*wl.domain_min), f32(*wl.domain_max),
                              wl.camera, wl.gen, 24, 20, 8, rng))
    return out


def quantize(ref):
    out = {}
    rng = np.random.default_rng(42)
    Wd, H, m = 23, 11, 12
    counts = rng.integers(0, m + 1, size=Wd * H).astype(np.uint32)
    index = np.zeros(Wd * H + 1, np.uint32)
    index[1:] = np.cumsum(counts)
    vals = rng.uniform(-0.1, 1.1, size=int(index[-1])).astype(np.float32)
    vals[::7] = 1.0
    vals[::11] = 0.0
    out["index"], out["values"] = index, vals
    tables = {"t16_10": [16] + [10] * (m - 1), "t_ragged": [16] + [5 + i for i in range(m - 1)],
              "t32": [32] * m, "t_odd": [13] + [3] * (m - 1)}
    for name, t in tables.items():
        t = np.array(t, np.uint8)
        n = ref.ref_quantize_prediction_coding(Wd, H, m, P(index), P(vals), vals.size, P(t), None)
        q = np.zeros(max(n, 1), np.uint8)
        ref.ref_quantize_prediction_coding(Wd, H, m, P(index), P(vals), vals.size, P(t), P(q))
        out[f"{name}_table"], out[f"{name}_bytes"] = t, q[:n]
    out["shape"] = np.array([Wd, H, m], np.int32)
    return out


QC_PAIRS = [(1, 10), (2, 10), (3, 9), (7, 6), (15, 4), (30, 3), (63, 2), (5, 16), (-1, 0)]


def _qc_image(ref, wl):
    Wd, H, m = wl.width, wl.height, wl.num_moments
    vol = np.ascontiguousarray(wl.volume)
    nz, ny, nx = vol.shape
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    data = np.zeros(Wd * H * m, np.float32)
    index = np.zeros(Wd * H + 1, np.uint32)
    bounds = np.zeros(2 * Wd * H, np.uint16)
    cp = np.zeros(2 * m, np.uint16)
    size = C.c_uint64()
    flags = np.zeros(4, np.int32)
    ref.ref_generate_grid(C.byref(wl.camera), C.byref(wl.gen), P(vol), nx, ny, nz, P(dmin), P(dmax), Wd, H, m,
                          P(data), P(index), P(bounds), P(cp), C.byref(size), P(flags))
    return index, data[:size.value].copy(), cp[:2 * (m - 1)].copy()


def quant_curve(ref):
    """Prediction-coded images from the reference's generate, their sample_moment_image and the per-pixel rRMSE
    of compute_coding_error for a set of (index, bits) pairs, from the reference's own building blocks."""
    out = {}
    mix = W.mixing_layer_workload(n=40, width=32, height=32, num_moments=64, modes=16, seed=5, name="golden_mix")
    ml = W.ml_workload(n=64, width=48, height=48, num_moments=24, seed=11, name="golden_ml_thr")
    ml.gen.error_threshold = 5e-2  # error-threshold compaction: ragged moment counts (2 .. 22)
    for key, wl, s in (("mix", mix, 16), ("mlthr", ml, 24)):
        wl.gen.prediction_coding = 1
        Wd, H, m = wl.width, wl.height, wl.num_moments
        index, data, cp = _qc_image(ref, wl)
        out[f"{key}_shape"] = np.array([Wd, H, m, s], np.int32)
        out[f"{key}_index"], out[f"{key}_data"], out[f"{key}_coding_params"] = index, data, cp
        s_index = np.zeros(s * s + 1, np.uint32)
        n = ref.ref_sample_moment_image(Wd, H, m, P(index), P(data), data.size, s, P(s_index), None)
        s_data = np.zeros(max(n, 1), np.float32)
        ref.ref_sample_moment_image(Wd, H, m, P(index), P(data), data.size, s, P(s_index), P(s_data))
        out[f"{key}_s_index"], out[f"{key}_s_data"] = s_index, s_data[:n]
        nonempty = int(np.count_nonzero(np.diff(s_index.astype(np.int64))))
        for idx, b in QC_PAIRS:
            if idx >= m:
                continue
            e = np.zeros(max(nonempty, 1), np.float32)
            k = ref.ref_coding_errors(s, s, m, P(s_index), P(s_data), n, 0, P(cp), idx, b, P(e))
            out[f"{key}_err_{idx}_{b}"] = e[:k]
    return out


def uncertainty(ref):
    """Error bounds (reconstruct_error, three measures and two percentiles), the two uncertainty tables of
    read_from_disk_uncertainty (every 17th row) and the two uncertainty renderers, from the reference's own code on
    the Marschner-Lobb pipeline image (standard and prediction coding)."""
    from mray_gb300.types import ErrorReconstructionParameters, UncertaintyReconstructionParameters

    out = {}
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    Wd, H, m = wl.width, wl.height, wl.num_moments
    vol = np.ascontiguousarray(wl.volume)
    nz, ny, nx = vol.shape
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    tf1d = np.ascontiguousarray(wl.tf1d, np.float32)
    for et in (0, 1):
        t = np.zeros((256, 256, 4), np.float32)
        ref.ref_uncertainty_tf(P(tf1d), C.c_float(wl.tf_step), et, P(t))
        out[f"table{et}_rows"] = t[::17].copy()
    row = np.zeros((256, 4), np.float32)
    ref.ref_preintegrate(P(tf1d), C.c_float(wl.tf_step), P(row))
    for pc in (0, 1):
        wl.gen.prediction_coding = pc
        index, data, cp = _qc_image(ref, wl)
        bounds = np.zeros(2 * Wd * H, np.uint16)
        d2 = np.zeros(Wd * H * m, np.float32)
        i2 = np.zeros(Wd * H + 1, np.uint32)
        cp2 = np.zeros(2 * m, np.uint16)
        size = C.c_uint64()
        flags = np.zeros(4, np.int32)
        ref.ref_generate_grid(C.byref(wl.camera), C.byref(wl.gen), P(vol), nx, ny, nz, P(dmin), P(dmax), Wd, H, m,
                              P(d2), P(i2), P(bounds), P(cp2), C.byref(size), P(flags))
        cpp = cp if pc else None
        for et, pct in ((0, 90), (1, 90), (2, 90), (2, 50)):
            ep = ErrorReconstructionParameters(error_type=et, error_percentile=pct, step_size=wl.rec.step_size,
                                               bias=wl.rec.bias)
            eb = np.zeros(Wd * H, np.uint16)
            ref.ref_reconstruct_error(C.byref(wl.camera), C.byref(ep), P(vol), nx, ny, nz, P(dmin), P(dmax), Wd, H,
                                      m, P(index), P(data), data.size, P(bounds), pc, 0, P(cpp), P(eb))
            out[f"pc{pc}_eb{et}_{pct}"] = eb
        for mode, et in ((0, 1), (1, 0), (1, 1), (1, 2)):
            up = UncertaintyReconstructionParameters(rec=wl.rec, error_type=et, bound_interpolation=0.3)
            if mode == 0:
                table = row
            else:
                table = np.zeros((256, 256, 4), np.float32)
                ref.ref_uncertainty_tf(P(tf1d), C.c_float(wl.tf_step), 1 if et == 1 else 0, P(table))
            eb = out[f"pc{pc}_eb{et}_90"]
            rgba = np.zeros((H, Wd, 4), np.float32)
            ref.ref_reconstruct_uncertainty_float(C.byref(wl.camera), C.byref(up), mode, Wd, H, m, P(index), P(data),
                                                  data.size, P(bounds), P(eb), pc, 0, P(cpp), P(dmin), P(dmax),
                                                  P(np.ascontiguousarray(table)), P(rgba))
            out[f"pc{pc}_unc{mode}_{et}"] = rgba
        out[f"pc{pc}_index"], out[f"pc{pc}_data"], out[f"pc{pc}_bounds"] = index, data, bounds
        if pc:
            out["pc1_coding_params"] = cp
    wl.gen.prediction_coding = 0
    return out


def reference_dvr(ref):
    """generate_reference (direct volume rendering of the volume itself) without and with brute-force single
    scattering, float colours from the reference's own reference_ray on the Marschner-Lobb volume."""
    from mray_gb300.types import ReferenceParameters, SingleScatteringParameters

    out = {}
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    vol = np.ascontiguousarray(wl.volume)
    nz, ny, nx = vol.shape
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    row = np.zeros((256, 4), np.float32)
    ref.ref_preintegrate(P(np.ascontiguousarray(wl.tf1d, np.float32)), C.c_float(wl.tf_step), P(row))
    cases = {"plain": dict(enable=0), "ss": dict(enable=1, henyey_greenstein_g=0.3, step_size_factor=2.0,
                                                   direction_x=0.3, direction_y=-1.0, direction_z=0.2)}
    for name, ss in cases.items():
        rp = ReferenceParameters(step_size=wl.rec.step_size, medium_emission=1.0, early_ray_termination=0.99,
                                 medium_scattering=0.5, ss=SingleScatteringParameters(**ss))
        rgba = np.zeros((wl.height, wl.width, 4), np.float32)
        ref.ref_generate_reference_float(C.byref(wl.camera), C.byref(rp), P(vol), nx, ny, nz, P(dmin), P(dmax),
                                         wl.width, wl.height, P(row), P(rgba))
        out[f"{name}_rgba"] = rgba
    return out


def _ref_image(ref, cam, gen, vol, dmin, dmax, Wd, H, m):
    """generate() through the reference: (index, data, bounds, coding params or None)."""
    nz, ny, nx = vol.shape
    data = np.zeros(Wd * H * m, np.float32)
    index = np.zeros(Wd * H + 1, np.uint32)
    bounds = np.zeros(2 * Wd * H, np.uint16)
    cp = np.zeros(2 * m, np.uint16)
    size = C.c_uint64()
    flags = np.zeros(4, np.int32)
    ref.ref_generate_grid(C.byref(cam), C.byref(gen), P(vol), nx, ny, nz, P(dmin), P(dmax), Wd, H, m, P(data),
                          P(index), P(bounds), P(cp), C.byref(size), P(flags))
    return index, data[:size.value].copy(), bounds, (cp[:2 * (m - 1)].copy() if gen.prediction_coding else None)


def single_scattering(ref):
    """Single scattering from the transmittance cache: the cache of a light image (reconstruct_single_scattering_
    cache on one thread, so that its racing writes come in the loop's order), the re-march sampling it
    (reconstruct_host with the cache, float and the whole reconstruct(..., ss, ...) as u8) and the reference
    renderer sampling it (generate_reference_reconstructed_ss), all from the reference's own code."""
    from mray_gb300.types import GenerationParameters, ReconstructionParameters, SingleScatteringParameters

    out = {}
    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    vol = np.ascontiguousarray(wl.volume)
    nz, ny, nx = vol.shape
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    row = np.zeros((256, 4), np.float32)
    ref.ref_preintegrate(P(np.ascontiguousarray(wl.tf1d, np.float32)), C.c_float(wl.tf_step), P(row))
    # the eye image (compact, bounds) and the light image (compact, bounds, prediction coded, threshold 0.01)
    m = wl.num_moments
    eye = _ref_image(ref, wl.camera, wl.gen, vol, dmin, dmax, wl.width, wl.height, m)
    light = W.light_camera((0.3, -1.0, 0.2))
    lw, lh = 40, 36
    lgen = GenerationParameters(step_size=wl.gen.step_size, error_threshold=0.01, bias=wl.gen.bias, compact_image=1,
                                prediction_coding=1, transform_to_bounds=1, transform_bound_eps=0.005)
    lim = _ref_image(ref, light, lgen, vol, dmin, dmax, lw, lh, m)
    ssp = SingleScatteringParameters(enable=1, use_cache=1, cache_size_x=24, cache_size_y=20, cache_size_z=16,
                                     henyey_greenstein_g=0.3, direction_x=light.dir[0], direction_y=light.dir[1],
                                     direction_z=light.dir[2], intensity_r=0.9, intensity_g=0.8, intensity_b=0.7)
    rp = ReconstructionParameters(step_size=wl.rec.step_size, bias=wl.rec.bias, medium_emission=1.0,
                                  medium_scattering=0.5, early_ray_termination=0.99, ss=ssp)
    cs = (ssp.cache_size_z, ssp.cache_size_y, ssp.cache_size_x)
    cache = np.zeros(cs, np.float32)
    ref.ref_ss_cache(C.byref(light), C.byref(rp), lw, lh, m, P(lim[0]), P(lim[1]), lim[1].size, P(lim[2]), 1, 0,
                     P(lim[3]), P(dmin), P(dmax), P(row), P(cache))
    rgba = np.zeros((wl.height, wl.width, 4), np.float32)
    ref.ref_reconstruct_cached_float(C.byref(wl.camera), C.byref(rp), wl.width, wl.height, m, P(eye[0]), P(eye[1]),
                                     eye[1].size, P(eye[2]), 0, 0, None, P(dmin), P(dmax), P(row), P(cache),
                                     ssp.cache_size_x, ssp.cache_size_y, ssp.cache_size_z, P(dmin), P(dmax), P(rgba))
    u8 = np.zeros((wl.height, wl.width, 4), np.uint8)
    ref.ref_reconstruct_ss_u8(C.byref(wl.camera), C.byref(rp), wl.width, wl.height, m, P(eye[0]), P(eye[1]),
                              eye[1].size, P(eye[2]), 0, 0, None, P(dmin), P(dmax), C.byref(light), lw, lh, m,
                              P(lim[0]), P(lim[1]), lim[1].size, P(lim[2]), 1, 0, P(lim[3]), P(row), P(u8))
    refss = np.zeros((wl.height, wl.width, 4), np.float32)
    ref.ref_generate_reference_cached_float(C.byref(wl.camera), C.byref(rp), P(vol), nx, ny, nz, P(dmin), P(dmax),
                                            wl.width, wl.height, P(row), P(cache), ssp.cache_size_x, ssp.cache_size_y,
                                            ssp.cache_size_z, P(dmin), P(dmax), P(refss))
    out.update(eye_index=eye[0], eye_data=eye[1], eye_bounds=eye[2], light_index=lim[0], light_data=lim[1],
               light_bounds=lim[2], light_coding_params=lim[3], light_shape=np.array([lw, lh, m], np.int32),
               cache=cache, rgba=rgba, rgba8=u8, reference_rgba=refss)
    return out


FILE_CASES = [
    # name, image, compress, bits, entropy, install the table first (once set, the reference keeps it)
    ("pc_raw", "pc", 0, 32, 0, False), ("pc_raw_lz4", "pc", 1, 32, 0, False), ("pc_q10", "pc", 0, 10, 0, False),
    ("pc_q10_lz4", "pc", 1, 10, 0, False), ("plain_raw", "plain", 0, 32, 0, False),
    ("plain_q12", "plain", 0, 12, 0, False), ("plain_q12_lz4", "plain", 1, 12, 0, False),
    ("plain_ac10", "plain", 0, 10, 1, False), ("plain_ac10_lz4", "plain", 1, 10, 1, False),
    ("static_raw", "static", 0, 32, 0, False), ("static_lz4", "static", 1, 32, 0, False),
    ("static_q16_lz4", "static", 1, 16, 0, False),
    ("pc_table", "pc", 0, 10, 0, True), ("pc_table_ac", "pc", 0, 10, 1, True), ("pc_table_ac_lz4", "pc", 1, 10, 1, True),
    ("plain_q12_table", "plain", 0, 12, 0, True),
]
FILE_TABLE = [16, 14, 13, 12, 11, 10, 10, 9, 8, 7, 6, 5]


def file_format(ref):
    """Moment-image files written by the reference's write_moment_image (its LZ4 calls served by oracle/lz4_ref.c)
    and read back by its load_moment_image, for compact images with and without prediction coding and a static
    image, raw, quantized, entropy coded, with and without compression and the global quantization table; and the
    entropy-coded payloads on their own."""
    import tempfile

    wl = W.ml_workload(n=64, width=20, height=16, num_moments=12, seed=11, name="golden_file")
    vol = np.ascontiguousarray(wl.volume)
    dmin, dmax = f32(*wl.domain_min), f32(*wl.domain_max)
    Wd, H, m = wl.width, wl.height, wl.num_moments
    P_ = Wd * H
    rng = np.random.default_rng(7)
    images = {}
    wl.gen.prediction_coding = 1
    images["pc"] = _ref_image(ref, wl.camera, wl.gen, vol, dmin, dmax, Wd, H, m)
    wl.gen.prediction_coding = 0
    images["plain"] = _ref_image(ref, wl.camera, wl.gen, vol, dmin, dmax, Wd, H, m)
    wl.gen.compact_image = 0
    wl.gen.transform_to_bounds = 0
    st = _ref_image(ref, wl.camera, wl.gen, vol, dmin, dmax, Wd, H, m)
    images["static"] = (None, np.ascontiguousarray(st[1][:P_ * m]), None, None)
    error_bounds = rng.integers(0, 65536, P_).astype(np.uint16)
    out = {"shape": np.array([Wd, H, m], np.int32), "domain": np.stack([dmin, dmax]),
           "table": np.array(FILE_TABLE, np.uint8), "error_bounds": error_bounds}
    for k, (index, data, bounds, cp) in images.items():
        out[f"{k}_data"] = data
        if index is not None:
            out[f"{k}_index"], out[f"{k}_bounds"] = index, bounds
        if cp is not None:
            out[f"{k}_coding_params"] = cp
    table = np.array(FILE_TABLE, np.uint8)
    with tempfile.TemporaryDirectory() as tmp:
        for name, kind, compress, bits, entropy, use_table in FILE_CASES:
            index, data, bounds, cp = images[kind]
            path = os.path.join(tmp, name + ".mom").encode()
            eb = error_bounds if kind == "plain" else None
            ref.ref_write_moment_image(path, Wd, H, m, int(index is not None), int(kind == "pc"), 0, P(dmin),
                                       P(dmax), P(index), P(data), data.size, P(bounds), P(eb), P(cp), compress,
                                       bits, entropy, P(table) if use_table else None)
            with open(path, "rb") as f:
                out[f"file_{name}"] = np.frombuffer(f.read(), np.uint8).copy()
            if name == "static_q16_lz4":
                continue  # the reference's reader decodes this one from the wrong byte
            info = np.zeros(9, np.int32)
            dom = np.zeros(6, np.float32)
            size = C.c_uint64()
            ref.ref_load_moment_image(path, P(info), P(dom), C.byref(size), None, None, None, None, None)
            d = np.zeros(size.value, np.float32)
            idx = np.zeros(P_ + 1, np.uint32)
            b = np.zeros(2 * P_, np.uint16)
            e = np.zeros(P_, np.uint16)
            c = np.zeros(2 * (m - 1), np.uint16)
            ref.ref_load_moment_image(path, P(info), P(dom), C.byref(size), P(idx), P(d), P(b), P(e), P(c))
            out[f"loaded_{name}_info"], out[f"loaded_{name}_data"] = info, d
    # the entropy-coded payloads alone
    for kind, pc, tab in (("plain", 0, np.full(m, 10, np.uint8)), ("pc", 1, table)):
        index, data = images[kind][0], images[kind][1]
        n = ref.ref_entropy_encode(Wd, H, m, P(index), P(data), data.size, pc, P(tab), None, 0)
        buf = np.zeros(n, np.uint8)
        ref.ref_entropy_encode(Wd, H, m, P(index), P(data), data.size, pc, P(tab), P(buf), n)
        out[f"entropy_{kind}"], out[f"entropy_{kind}_table"] = buf, tab
    # the reference's own coding test (tests/test_moment_image_coding.cpp:30-64): a 16 x 16 ramp x / 16 in all ten
    # moments, prediction coded, table [16, 11, ...]
    rw, rm = 16, 10
    ramp = np.repeat((np.arange(rw, dtype=np.float32) / np.float32(rw))[None, :, None], rw, axis=0)
    ramp = np.ascontiguousarray(np.repeat(ramp, rm, axis=2).reshape(-1))
    ridx = np.arange(0, rw * rw * rm + 1, rm, dtype=np.uint32)
    rtab = np.array([16] + [11] * (rm - 1), np.uint8)
    n = ref.ref_entropy_encode(rw, rw, rm, P(ridx), P(ramp), ramp.size, 1, P(rtab), None, 0)
    buf = np.zeros(n, np.uint8)
    ref.ref_entropy_encode(rw, rw, rm, P(ridx), P(ramp), ramp.size, 1, P(rtab), P(buf), n)
    out["entropy_ramp"], out["entropy_ramp_data"], out["entropy_ramp_table"] = buf, ramp, rtab
    return out


def main():
    ref = O.ref_lib()
    if ref is None:
        raise SystemExit("the reference sources are not available; cannot write golden fixtures")
    declare(ref)
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **known_answers(ref))
    np.savez_compressed(os.path.join(HERE, "probes.npz"), **probes(ref))
    ml = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    np.savez_compressed(os.path.join(HERE, "pipeline_ml.npz"), **pipeline(ref, ml))
    mix = W.mixing_layer_workload(n=40, width=32, height=32, num_moments=64, modes=16, seed=5, name="golden_mix")
    np.savez_compressed(os.path.join(HERE, "pipeline_mix.npz"), **pipeline(ref, mix))
    np.savez_compressed(os.path.join(HERE, "quantize.npz"), **quantize(ref))
    np.savez_compressed(os.path.join(HERE, "particles.npz"), **particles(ref))
    np.savez_compressed(os.path.join(HERE, "quant_curve.npz"), **quant_curve(ref))
    np.savez_compressed(os.path.join(HERE, "uncertainty.npz"), **uncertainty(ref))
    np.savez_compressed(os.path.join(HERE, "reference_dvr.npz"), **reference_dvr(ref))
    np.savez_compressed(os.path.join(HERE, "single_scattering.npz"), **single_scattering(ref))
    np.savez_compressed(os.path.join(HERE, "file_format.npz"), **file_format(ref))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
