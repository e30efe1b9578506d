"""The reference direct volume renderer (generate_reference, raymarch_reference.h) against the oracle, through the
C ABI: without single scattering, with brute-force single scattering, over a grid and over SPH particles.

Sample positions, densities and the compositing order are the reference's; the device's exp is CUDA's expf where
the reference's CPU build rounds the double function, so colours agree within a few float ulps of the accumulated
sums: held to 1e-4 per channel here (the re-march's bar is 1e-3).
"""
import numpy as np
import pytest

import oracle as O
from helpers import small_ml

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-4


def _params(M, wl, ss):
    sp = M.SingleScatteringParameters(enable=1, henyey_greenstein_g=0.3, step_size_factor=2.0, direction_x=0.3,
                                      direction_y=-1.0, direction_z=0.2) if ss else M.SingleScatteringParameters()
    return M.ReferenceParameters(step_size=wl.rec.step_size, medium_emission=1.0, early_ray_termination=0.99,
                                 medium_scattering=0.5, data_min=wl.gen.data_min, data_max=wl.gen.data_max, ss=sp)


@pytest.mark.parametrize("ss", [0, 1], ids=["plain", "single_scattering"])
def test_reference_dvr_grid(gpu_context, ss):
    import mray_gb300 as M

    wl = small_ml(96, 80, 8) if not ss else small_ml(48, 40, 8)
    rp = _params(M, wl, ss)
    tf = M.preintegrate(wl.tf1d, wl.tf_step)
    img = M.ColorImageHost(wl.width, wl.height)
    M.generate_reference(wl.camera, tf, M.RegularGrid(wl.volume, wl.domain_min, wl.domain_max), img, rp,
                         context=gpu_context)
    ref = O.generate_reference(wl.camera, rp, wl.volume, wl.domain_min, wl.domain_max, wl.width, wl.height, tf.table)
    assert ref[..., 3].mean() > 0.1
    d = np.abs(img.rgba_float - ref)
    assert d.max() <= TOL, f"max diff {d.max():.2e}"
    assert np.mean(np.abs(img.rgba.astype(int) - O.rgba_to_u8(ref).astype(int)) <= 1) == 1.0
    if ss:
        plain = O.generate_reference(wl.camera, _params(M, wl, 0), wl.volume, wl.domain_min, wl.domain_max,
                                     wl.width, wl.height, tf.table)
        assert img.rgba_float[..., :3].mean() > plain[..., :3].mean()


def test_reference_dvr_particles_and_stage_call(gpu_context):
    import mray_gb300 as M
    from mray_gb300 import workloads as Wl

    swl = Wl.sph_workload(n=200_000, h=1.0 / 64, width=48, height=40, num_moments=8, seed=5)
    rp = M.ReferenceParameters(step_size=swl.rec.step_size, medium_emission=1.0, early_ray_termination=0.99,
                               data_min=swl.gen.data_min, data_max=swl.gen.data_max)
    parts = O.ParticleSet(swl.x, swl.y, swl.z, swl.v, swl.h, swl.domain_min, swl.domain_max)
    tf = M.preintegrate(swl.tf1d, swl.tf_step)
    gpu_context.upload_particles(swl.x, swl.y, swl.z, swl.v, swl.h, swl.domain_min, swl.domain_max)
    gpu_context.upload_tf(tf.table)
    img = gpu_context.generate_reference(swl.camera, rp, 48, 40)
    ref = O.generate_reference(swl.camera, rp, None, swl.domain_min, swl.domain_max, 48, 40, tf.table,
                               particles=parts)
    assert ref[..., 3].mean() > 0.05
    assert np.abs(img.rgba_float - ref).max() <= TOL
    d_rgba = torch.zeros(48 * 40 * 4, device="cuda")
    gpu_context.stage_generate_reference(swl.camera, rp, 48, 40, d_rgba)
    gpu_context.synchronize()
    assert np.array_equal(d_rgba.cpu().numpy().reshape(40, 48, 4), img.rgba_float)


def test_reference_dvr_errors(gpu_context):
    import mray_gb300 as M

    wl = small_ml(16, 16, 8)
    fresh = M.Context(0)
    try:
        rp = _params(M, wl, 0)
        with pytest.raises(M.MrayError) as e:
            fresh.generate_reference(wl.camera, rp, 16, 16)
        assert e.value.status == 7  # no volume
        fresh.upload_grid(wl.volume, wl.domain_min, wl.domain_max)
        with pytest.raises(M.MrayError) as e:
            fresh.generate_reference(wl.camera, rp, 16, 16)
        assert e.value.status == 1  # no transfer function
        fresh.upload_tf(M.preintegrate(wl.tf1d, wl.tf_step).table)
        rp.step_size = 0.0
        with pytest.raises(M.MrayError) as e:
            fresh.generate_reference(wl.camera, rp, 16, 16)
        assert e.value.status == 1
        rp = _params(M, wl, 1)
        rp.ss.step_size_factor = 0.0
        with pytest.raises(M.MrayError) as e:
            fresh.generate_reference(wl.camera, rp, 16, 16)
        assert e.value.status == 1
    finally:
        fresh.close()
