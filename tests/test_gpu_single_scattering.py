"""Single scattering from the transmittance cache through the C ABI: the cache of a light moment image
(reconstruct_single_scattering_cache, moment_raymarcher.cpp:217-258), the re-march sampling it (reconstruct with a
SingleScatteringImageHost, :339-351) and the reference renderer sampling it (generate_reference_reconstructed_ss,
:259-281), against the oracle pinned to the reference's own code (tests/golden/single_scattering.npz).

Every sample lands in the reference's voxel (positions and voxel indices are the reference's float operations) and
the cache keeps the value of the last pixel in row-major order, as the reference's loop run sequentially does; the
transmittance written there differs from the oracle's by the rounding of the MESE density and of exp, held like the
re-march's colours: within 1e-3 of the FP32 oracle, or at least as close to the FP64 evaluation of the same method.
"""
import os

import numpy as np
import pytest

import oracle as O
from helpers import light_generation_parameters, rgba_agreement, single_scattering_case

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-3
REF_TOL = 1e-4


def _golden():
    return np.load(os.path.join(GOLDEN, "single_scattering.npz"))


def _light_image(M, g, wl):
    lw, lh, m = (int(v) for v in g["light_shape"])
    mi = M.MomentImageHost(lw, lh, m, True, True)
    mi.index, mi.data, mi.is_compact = g["light_index"].copy(), g["light_data"].copy(), True
    mi.bounds = g["light_bounds"].reshape(-1, 2).copy()
    mi.prediction_code, mi.coding_warp, mi.coding_params = True, 0, g["light_coding_params"].copy()
    mi.domain_min, mi.domain_max = wl.domain_min, wl.domain_max
    return mi


def _eye_image(M, g, wl):
    mi = M.MomentImageHost(wl.width, wl.height, wl.num_moments, True, True)
    mi.index, mi.data, mi.is_compact = g["eye_index"].copy(), g["eye_data"].copy(), True
    mi.bounds = g["eye_bounds"].reshape(-1, 2).copy()
    mi.domain_min, mi.domain_max = wl.domain_min, wl.domain_max
    return mi


def _oracle_caches(light, rp, mi, row):
    """The FP32 oracle's cache and the FP64 evaluation of the same method (same sample positions)."""
    cp = mi.coding_params if mi.prediction_code else None
    out = []
    for precision in ("f32", "f64"):
        pm = O.prepare_moments(mi.width, mi.height, mi.num_moments, mi.index, mi.data, mi.prediction_code,
                               mi.coding_warp, cp, rp.bias, precision=precision)
        out.append(O.ss_cache(light, rp, mi.width, mi.height, mi.num_moments, mi.domain_min, mi.domain_max, mi.index,
                              pm, mi.bounds, row.astype(np.float32 if precision == "f32" else np.float64),
                              precision=precision))
    return out


def cache_agreement(ours, c32, c64, tol=TOL):
    d32 = np.abs(ours.astype(np.float64) - c32)
    d64 = np.abs(ours.astype(np.float64) - c64)
    own = np.abs(c32.astype(np.float64) - c64)
    return (d32 <= tol) | (d64 <= np.maximum(tol, own))


def _check_cache(cache, c32, c64, min_frac=0.999):
    # the same voxels are written (an underflowed exp(-tau) = 0 reads as unwritten)
    written = (cache > 1e-30) | (c32 > 1e-30)
    assert np.array_equal(cache[written] != 0, c32[written] != 0)
    ok = cache_agreement(cache, c32, c64)
    assert ok.mean() >= min_frac, f"{(~ok).sum()} of {ok.size} voxels off; max diff {np.abs(cache - c32).max():.2e}"


def test_cache_matches_golden(gpu_context):
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    lmi = _light_image(M, g, wl)
    cache = gpu_context.reconstruct_single_scattering_cache(light, rp, lmi)
    c32, c64 = _oracle_caches(light, rp, lmi, tf.table)
    assert np.array_equal(c32, g["cache"])
    _check_cache(cache, c32, c64)


@pytest.mark.parametrize("cache_size,light_shape", [((3, 2, 4), (40, 36)), ((17, 9, 31), (64, 48)),
                                                    ((64, 64, 64), (96, 96)), ((128, 128, 128), (33, 65))],
                         ids=["3x2x4", "17x9x31", "64cube", "128cube-sparse"])
def test_cache_collisions_and_coverage(gpu_context, cache_size, light_shape):
    """From dozens of samples per voxel (a 3 x 2 x 4 cache) to a cache the light image covers sparsely (most
    voxels never written and left 0): the same voxels, and in each the last writer's transmittance."""
    import mray_gb300 as M

    wl, light, rp = single_scattering_case(cache_size=cache_size, light_shape=light_shape)
    lw, lh = light_shape
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    gpu_context.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    lmi = gpu_context.generate(light, light_generation_parameters(wl), lw, lh, wl.num_moments)
    lmi.domain_min, lmi.domain_max = wl.domain_min, wl.domain_max
    cache = gpu_context.reconstruct_single_scattering_cache(light, rp, lmi)
    c32, c64 = _oracle_caches(light, rp, lmi, tf.table)
    _check_cache(cache, c32, c64)
    if cache_size == (128, 128, 128):
        assert (c32 == 0).mean() > 0.5


def test_stage_cache_from_device_image(gpu_context):
    """The stage call from multipliers in device memory, with the cache written to a device buffer too; the same
    grid as the host call."""
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    lmi = _light_image(M, g, wl)
    host = gpu_context.reconstruct_single_scattering_cache(light, rp, lmi)
    d_idx = torch.from_numpy(lmi.index.view(np.int32)).cuda()
    d_data = torch.from_numpy(lmi.data).cuda()
    d_cp = torch.from_numpy(lmi.coding_params.view(np.int16)).cuda()
    d_b = torch.from_numpy(lmi.bounds.reshape(-1).view(np.int16)).cuda()
    d_pm = torch.zeros_like(d_data)
    gpu_context.stage_prepare_moments(lmi.width, lmi.height, lmi.num_moments, d_idx, d_data, d_pm,
                                      prediction_code=True, coding_warp=0, coding_params=d_cp, bias=rp.bias)
    d_cache = torch.full((16, 20, 24), -1.0, device="cuda")
    gpu_context.stage_reconstruct_single_scattering_cache(light, rp, lmi.width, lmi.height, lmi.num_moments,
                                                          wl.domain_min, wl.domain_max, d_idx, d_pm, d_b, d_cache)
    gpu_context.synchronize()
    assert np.array_equal(d_cache.cpu().numpy(), host)


def test_reconstruct_with_cache(gpu_context):
    """The re-march with the golden cache uploaded: against the reference's colours and the FP32 / FP64 oracles on
    the same cache."""
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    gpu_context.upload_single_scattering_cache(g["cache"], wl.domain_min, wl.domain_max)
    emi = _eye_image(M, g, wl)
    img = gpu_context.reconstruct(wl.camera, rp, emi)
    cache = (g["cache"], wl.domain_min, wl.domain_max)
    m = wl.num_moments

    def march(precision):
        pm = O.prepare_moments(wl.width, wl.height, m, emi.index, emi.data, bias=rp.bias, precision=precision)
        return O.reconstruct(wl.camera, rp, wl.width, wl.height, m, wl.domain_min, wl.domain_max, emi.index, pm,
                             emi.bounds, tf.table.astype(pm.dtype), precision, cache=cache)

    r32 = march("f32")
    assert np.array_equal(r32, g["rgba"])
    ok = rgba_agreement(img.rgba_float, r32, march("f64"), TOL)
    assert ok.mean() >= 0.998, f"{(~ok).sum()} pixels"
    assert np.mean(np.abs(img.rgba.astype(int) - g["rgba8"].astype(int)) <= 1) >= 0.999
    # the same cache uploaded from device memory gives the same image
    gpu_context.upload_single_scattering_cache(torch.from_numpy(g["cache"].copy()).cuda(), wl.domain_min,
                                               wl.domain_max)
    assert np.array_equal(gpu_context.reconstruct(wl.camera, rp, emi).rgba_float, img.rgba_float)
    # the in-scattered light is there
    rp.ss.enable = 0
    plain = gpu_context.reconstruct(wl.camera, rp, emi)
    assert img.rgba_float[..., :3].mean() > plain.rgba_float[..., :3].mean() + 0.05


def test_dropin_reconstruct_with_light_image(gpu_context):
    """reconstruct(cam, mi, tf, img, ss, params): the cache built from the light image, then the re-march; the
    whole call against the reference's u8 image."""
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    img = M.ColorImageHost(wl.width, wl.height)
    ss = M.SingleScatteringImageHost(light, _light_image(M, g, wl))
    M.reconstruct(wl.camera, _eye_image(M, g, wl), tf, img, rp, context=gpu_context, ss=ss)
    assert np.mean(np.abs(img.rgba.astype(int) - g["rgba8"].astype(int)) <= 1) >= 0.999
    grid = M.reconstruct_single_scattering_cache(ss, tf, rp, context=gpu_context)
    assert grid.cache.data.shape == (16, 20, 24) and grid.cache.domain_min == wl.domain_min


def test_reference_with_cache(gpu_context):
    """generate_reference_reconstructed_ss: the reference renderer sampling the golden cache, then the whole call
    building its own cache from the light image."""
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    gpu_context.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
    gpu_context.upload_single_scattering_cache(g["cache"], wl.domain_min, wl.domain_max)
    img = gpu_context.generate_reference_reconstructed_ss(wl.camera, rp, wl.width, wl.height)
    d = np.abs(img.rgba_float - g["reference_rgba"])
    assert d.max() <= REF_TOL, f"max diff {d.max():.2e}"
    d_rgba = torch.zeros(wl.height * wl.width * 4, device="cuda")
    gpu_context.stage_generate_reference_reconstructed_ss(wl.camera, rp, wl.width, wl.height, d_rgba)
    gpu_context.synchronize()
    assert np.array_equal(d_rgba.cpu().numpy().reshape(wl.height, wl.width, 4), img.rgba_float)

    img2 = M.ColorImageHost(wl.width, wl.height)
    ss = M.SingleScatteringImageHost(light, _light_image(M, g, wl))
    M.generate_reference_reconstructed_ss(wl.camera, tf, M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max),
                                          img2, ss, rp, context=gpu_context)
    own = gpu_context.reconstruct_single_scattering_cache(light, rp, ss.img)
    ref = O.generate_reference(wl.camera, O.ref_from_rec(rp), wl.volume, wl.domain_min, wl.domain_max, wl.width,
                               wl.height, tf.table, cache=(own, wl.domain_min, wl.domain_max))
    assert np.abs(img2.rgba_float - ref).max() <= REF_TOL


def test_reference_with_cache_over_particles(gpu_context):
    """generate_reference_reconstructed_ss over SPH particles: the renderer samples the particles and the cache of a
    light image rendered from them."""
    import mray_gb300 as M
    from mray_gb300 import workloads as Wl

    swl = Wl.sph_workload(n=100_000, h=1.0 / 48, width=40, height=32, num_moments=12, seed=9)
    light = Wl.light_camera((0.3, -1.0, 0.2), center=(0.5, 0.5, 0.5), half_extent=0.9, distance=2.0)
    ssp = M.SingleScatteringParameters(enable=1, use_cache=1, cache_size_x=20, cache_size_y=18, cache_size_z=16,
                                       henyey_greenstein_g=-0.2, direction_x=light.dir[0], direction_y=light.dir[1],
                                       direction_z=light.dir[2])
    rp = M.ReconstructionParameters(step_size=swl.rec.step_size, bias=swl.rec.bias, medium_emission=1.0,
                                    medium_scattering=0.5, early_ray_termination=0.99, data_min=swl.gen.data_min,
                                    data_max=swl.gen.data_max, ss=ssp)
    tf = M.preintegrate(swl.tf1d, swl.tf_step)
    gpu_context.upload_tf(tf.table)
    gpu_context.upload_particles(swl.x, swl.y, swl.z, swl.v, swl.h, swl.domain_min, swl.domain_max)
    lmi = gpu_context.generate(light, swl.gen, 48, 48, swl.num_moments)
    lmi.domain_min, lmi.domain_max = swl.domain_min, swl.domain_max
    cache = gpu_context.reconstruct_single_scattering_cache(light, rp, lmi)
    assert 0.0 < cache.max() <= 1.0
    img = gpu_context.generate_reference_reconstructed_ss(swl.camera, rp, swl.width, swl.height)
    parts = O.ParticleSet(swl.x, swl.y, swl.z, swl.v, swl.h, swl.domain_min, swl.domain_max)
    ref = O.generate_reference(swl.camera, O.ref_from_rec(rp), None, swl.domain_min, swl.domain_max, swl.width,
                               swl.height, tf.table, particles=parts, cache=(cache, swl.domain_min, swl.domain_max))
    assert ref[..., 3].mean() > 0.05
    assert np.abs(img.rgba_float - ref).max() <= REF_TOL


def test_disabled_or_no_scattering_is_the_plain_march(gpu_context):
    """ss.enable = 0, or a medium that does not scatter: no in-scattering (raymarch_reconstruct.h:176-179), the
    plain re-march bit for bit, with a cache resident or not."""
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    gpu_context.upload_tf(tf.table)
    gpu_context.upload_single_scattering_cache(g["cache"], wl.domain_min, wl.domain_max)
    emi = _eye_image(M, g, wl)
    plain_rp = M.ReconstructionParameters(step_size=rp.step_size, bias=rp.bias, medium_emission=1.0,
                                          medium_scattering=0.0, early_ray_termination=0.99)
    plain = gpu_context.reconstruct(wl.camera, plain_rp, emi).rgba_float.copy()
    rp.medium_scattering = 0.0
    assert np.array_equal(gpu_context.reconstruct(wl.camera, rp, emi).rgba_float, plain)
    rp.medium_scattering = 0.5
    rp.ss.enable = 0
    plain_rp.medium_scattering = 0.5
    assert np.array_equal(gpu_context.reconstruct(wl.camera, rp, emi).rgba_float,
                          gpu_context.reconstruct(wl.camera, plain_rp, emi).rgba_float)


def test_errors():
    import mray_gb300 as M

    g = _golden()
    wl, light, rp = single_scattering_case()
    fresh = M.Context(0)
    try:
        tf = M.preintegrate(wl.tf1d, wl.tf_step)
        fresh.upload_tf(tf.table)
        emi = _eye_image(M, g, wl)
        with pytest.raises(M.MrayError) as e:  # no cache built or uploaded
            fresh.reconstruct(wl.camera, rp, emi)
        assert e.value.status == 1
        rp.ss.use_cache = 0  # the marched form
        with pytest.raises(M.MrayError) as e:
            fresh.reconstruct(wl.camera, rp, emi)
        assert e.value.status == 6
        rp.ss.use_cache = 1
        for bad in ((0, 20, 16), (24, -1, 16), (24, 20, 1 << 20)):
            rp.ss.cache_size_x, rp.ss.cache_size_y, rp.ss.cache_size_z = bad
            with pytest.raises(M.MrayError) as e:
                fresh.reconstruct_single_scattering_cache(light, rp, _light_image(M, g, wl), return_cache=False)
            assert e.value.status == 1, bad
        rp.ss.cache_size_x, rp.ss.cache_size_y, rp.ss.cache_size_z = 24, 20, 16
        with pytest.raises(M.MrayError) as e:  # an empty domain
            fresh.upload_single_scattering_cache(g["cache"], (0, 0, 0), (1, 0, 1))
        assert e.value.status == 1
        up = M.UncertaintyReconstructionParameters(rec=rp)
        emi.add_error_bounds()
        with pytest.raises(M.MrayError) as e:  # uncertainty rendering marches the light image: not supported
            fresh.reconstruct_uncertainty(wl.camera, up, 0, emi)
        assert e.value.status == 6
        # the context stays usable: build the cache, then reconstruct
        fresh.reconstruct_single_scattering_cache(light, rp, _light_image(M, g, wl), return_cache=False)
        img = fresh.reconstruct(wl.camera, rp, emi)
        assert np.mean(np.abs(img.rgba.astype(int) - g["rgba8"].astype(int)) <= 1) >= 0.999
    finally:
        fresh.close()
