"""The differentiation form on the GPU: its forward against the oracle, and the hand-written adjoint (re-march,
Lagrange-multiplier preparation, generation) against finite differences.

The differentiated method: no compaction, unquantized density bounds, exact arctangent, transfer-function row as
a cubic B-spline in the front density.  Two checks of the gradients:
  * the FP64 reference gradient: central differences (eps = 2^-10, exact in float storage) of the FP64 oracle of
    the same method, under a fixed linear image loss (the gradient is then the Jacobian alone, not the forward's
    residual), relative error <= 1e-3 per parameter on parameters whose gradient is not negligible;
  * under the configuration's L2 loss (target rendered with a perturbed transfer function) on 32 seeded parameters
    (16 transfer-function entries, 16 voxels): against central differences (eps about 1e-3) of the FP64 oracle,
    and against central differences (eps = 1e-3) of the FP32 GPU forward itself on the strong parameters.
The transfer-function row linear in the front density (the reference's GPU sampling) is checked the same way
against the oracle's FP64 form of that sampling.
"""
import numpy as np
import pytest

import oracle as O
from helpers import GpuRender, pick_parameters as _pick, richardson as _richardson

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _workload(n=40, width=40, height=36, m=16, seed=11):
    from mray_gb300 import workloads as W

    return W.diff_workload(n=n, width=width, height=height, num_moments=m, seed=seed)


def _oracle_rgba(wl, volume, table):
    return O.diff_forward(wl.camera, wl.gen, wl.rec, volume, wl.domain_min, wl.domain_max, wl.width, wl.height,
                          wl.num_moments, table, "f64")


@pytest.mark.parametrize("m", [8, 16, 31])
def test_diff_forward_matches_oracle(gpu_context, m):
    wl, _ = _workload(m=m)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    rgba = GpuRender(gpu_context, wl).forward(wl.volume, table)
    ref32 = O.diff_forward(wl.camera, wl.gen, wl.rec, wl.volume, wl.domain_min, wl.domain_max, wl.width, wl.height,
                           m, table, "f32")
    ref64 = _oracle_rgba(wl, wl.volume, table)
    assert np.abs(rgba - ref32).max() <= 1e-3
    assert np.abs(rgba - ref64).max() <= 1e-3
    assert rgba[..., 3].max() > 0.1  # the view sees the volume


def _fd64(wl, volume, table, weights, params, eps=2.0 ** -10):
    """Central differences of the FP64 oracle under the linear loss sum(weights * rgba), Richardson-combined."""
    t64 = table.astype(np.float64)

    def loss(v, t):
        return float((weights * _oracle_rgba(wl, v, t)).sum())

    return np.array([_richardson(loss, wl, t64, kind, idx, eps) for kind, idx in params])


@pytest.mark.parametrize("m", [1, 8, 16, 31])
def test_adjoint_against_fp64_reference_gradient(gpu_context, m):
    wl, _ = _workload(m=m)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    rng = np.random.default_rng(5)
    weights = rng.standard_normal((wl.height, wl.width, 4))
    R = GpuRender(gpu_context, wl)
    R.forward(wl.volume, table)
    gtf, gvol = R.backward(weights)
    params = _pick(rng, gvol, gtf, 8, 8)
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    fd = _fd64(wl, wl.volume, table, weights, params)
    rel = np.abs(ad - fd) / np.abs(fd)
    assert rel.max() <= 1e-3, f"max rel err {rel.max():.3e} at {params[int(rel.argmax())]}: ad {ad} fd {fd}"


def test_adjoint_64_moments_against_fp64_reference_gradient(gpu_context):
    """64 moments (two elements per lane in the preparation adjoint, the 64-moment instances of every adjoint
    kernel) under a random linear image loss against central differences of the FP64 oracle: voxels within 1e-3
    relative (measured 7e-5).  Table entries within 3e-3 (measured 1.9e-3 at worst, most below 5e-4): an entry's
    gradient sums the B-spline weights of its samples, which move with the FP32 forward's reconstructed densities,
    and at 64 moments the FP32 series (multipliers up to 1e4 cancelling to values of order one) moves those
    densities more than at 31 (at 31 moments 1e-3 holds above)."""
    wl, _ = _workload(m=64)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    rng = np.random.default_rng(5)
    weights = rng.standard_normal((wl.height, wl.width, 4))
    R = GpuRender(gpu_context, wl)
    R.forward(wl.volume, table)
    gtf, gvol = R.backward(weights)
    params = _pick(rng, gvol, gtf, 8, 8)
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    fd = _fd64(wl, wl.volume, table, weights, params)
    rel = np.abs(ad - fd) / np.abs(fd)
    is_tf = np.array([kind == "tf" for kind, _ in params])
    assert rel[~is_tf].max() <= 1e-3, f"voxels: max rel err {rel[~is_tf].max():.3e}: ad {ad[~is_tf]} fd {fd[~is_tf]}"
    assert rel[is_tf].max() <= 3e-3, f"tf: max rel err {rel[is_tf].max():.3e}: ad {ad[is_tf]} fd {fd[is_tf]}"


def _l2_setup(ctx):
    wl, target_tf = _workload(n=48, width=48, height=40, m=31)
    table = O.preintegrate(wl.tf1d, wl.tf_step).astype(np.float64)
    R = GpuRender(ctx, wl)
    target = R.forward(wl.volume, O.preintegrate(target_tf, wl.tf_step))
    return wl, table, R, target


def test_l2_adjoint_against_fp64_central_differences(gpu_context):
    """The L2 loss of the configuration (target rendered with the perturbed transfer function): the GPU adjoint,
    fed the FP64 forward's residual, against central differences (eps = 2^-10, about 1e-3, Richardson-combined
    with 2 eps) of the FP64 oracle on 32 seeded parameters (16 transfer-function entries, 16 voxels)."""
    wl, table, R, target = _l2_setup(gpu_context)
    rgba64 = _oracle_rgba(wl, wl.volume, table)
    R.forward(wl.volume, table)
    gtf, gvol = R.backward(2.0 * (rgba64 - target))
    params = _pick(np.random.default_rng(17), gvol, gtf, 16, 16)

    def loss(v, t):
        return ((_oracle_rgba(wl, v, t) - target) ** 2).sum()

    fd = np.array([_richardson(loss, wl, table, kind, idx, 2.0 ** -10) for kind, idx in params])
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    rel = np.abs(ad - fd) / np.abs(fd)
    assert rel.max() <= 1e-3, f"max rel err {rel.max():.3e} at {params[int(rel.argmax())]}"


def test_l2_adjoint_against_gpu_central_differences(gpu_context):
    """Central differences (eps = 1e-3, Richardson-combined with 2 eps) of the FP32 GPU forward itself on the
    seeded parameters whose gradient is at least a tenth of the largest of its kind.  Tolerance 1e-2: the FP32
    forward's own rounding moves L(p + eps) - L(p - eps) by a few 1e-3 of itself for a single voxel (measured with
    the oracle's FP32 and FP64 forms of the same method), so the 1e-3 bound is checked against the FP64 oracle's
    differences above and this test checks that the kernels' FP32 forward and adjoint agree with each other."""
    wl, table, R, target = _l2_setup(gpu_context)
    rgba = R.forward(wl.volume, table)
    gtf, gvol = R.backward(2.0 * (rgba - target))
    rng = np.random.default_rng(23)
    tf_ok = np.argwhere(np.abs(gtf) > 0.1 * np.abs(gtf).max())
    vox_ok = np.argwhere(np.abs(gvol) > 0.1 * np.abs(gvol).max())
    params = [("tf", tuple(tf_ok[i])) for i in rng.choice(len(tf_ok), min(16, len(tf_ok)), replace=False)]
    params += [("vox", tuple(vox_ok[i])) for i in rng.choice(len(vox_ok), min(16, len(vox_ok)), replace=False)]

    def loss(v, t):
        return ((R.forward(v, t) - target) ** 2).sum()

    fd = np.array([_richardson(loss, wl, table, kind, idx, 1e-3) for kind, idx in params])
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    rel = np.abs(ad - fd) / np.abs(fd)
    assert rel.max() <= 1e-2, f"max rel err {rel.max():.3e} at {params[int(rel.argmax())]}"


def _linear(ctx):
    import mray_gb300 as M

    class _Linear:
        def __enter__(self):
            ctx.diff_tf_sampling = M.DIFF_TF_LINEAR

        def __exit__(self, *exc):
            ctx.diff_tf_sampling = M.DIFF_TF_BSPLINE

    return _Linear()


def _oracle_rgba_linear(wl, volume, table):
    return O.diff_forward(wl.camera, wl.gen, wl.rec, volume, wl.domain_min, wl.domain_max, wl.width, wl.height,
                          wl.num_moments, table, "f64", tf_linear=True)


def test_linear_tf_forward_matches_oracle(gpu_context):
    """The transfer-function row sampled linearly in the front density (the reference's GPU texture sampling, exact
    weights): the forward against the oracle's FP32 and FP64 forms of the same sampling, and different from the
    B-spline row's image."""
    wl, _ = _workload(m=31)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    R = GpuRender(gpu_context, wl)
    spline = R.forward(wl.volume, table)
    with _linear(gpu_context):
        rgba = R.forward(wl.volume, table)
    ref32 = O.diff_forward(wl.camera, wl.gen, wl.rec, wl.volume, wl.domain_min, wl.domain_max, wl.width, wl.height,
                           wl.num_moments, table, "f32", tf_linear=True)
    ref64 = _oracle_rgba_linear(wl, wl.volume, table)
    assert np.abs(rgba - ref32).max() <= 1e-3
    assert np.abs(rgba - ref64).max() <= 1e-3
    # the two rows render differently (the smooth table makes the difference small): the linear image is far closer to
    # the oracle's linear image than to the B-spline one
    assert np.abs(rgba - spline).max() > 10.0 * np.abs(rgba - ref64).max()


def test_linear_tf_adjoint_against_fp64_central_differences(gpu_context):
    """Gradients with the linear row against central differences (eps = 2^-10, Richardson-combined with 2 eps) of
    the FP64 oracle of the same sampling, under a random linear image loss.  The loss is smooth in the table entries
    (they enter the emission linearly and the transmittance through exp), but an entry's gradient sums the hat weights
    1 - |256 fs - 1/2 - i| of its samples, which move by 256 times the FP32 forward's density error (the B-spline's
    weights by at most half as much): 16 entries within 3e-3 relative (measured 1.8e-3 at worst, median 7e-5).  In a
    voxel the loss has a kink wherever one of the many samples whose reconstructed density the voxel moves crosses a
    texel centre, and central differences over eps cross some of them: 8 voxels within 1e-2 relative (measured
    7.3e-3)."""
    wl, _ = _workload(m=16)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    rng = np.random.default_rng(29)
    weights = rng.standard_normal((wl.height, wl.width, 4))
    R = GpuRender(gpu_context, wl)
    with _linear(gpu_context):
        R.forward(wl.volume, table)
        gtf, gvol = R.backward(weights)
    params = _pick(rng, gvol, gtf, 16, 8)
    t64 = table.astype(np.float64)

    def loss(v, t):
        return float((weights * _oracle_rgba_linear(wl, v, t)).sum())

    fd = np.array([_richardson(loss, wl, t64, kind, idx, 2.0 ** -10) for kind, idx in params])
    ad = np.array([gtf[idx] if kind == "tf" else gvol[idx] for kind, idx in params])
    rel = np.abs(ad - fd) / np.abs(fd)
    is_tf = np.array([kind == "tf" for kind, _ in params])
    print(f"linear row: tf max rel err {rel[is_tf].max():.2e} (median {np.median(rel[is_tf]):.1e}), voxels "
          f"{rel[~is_tf].max():.2e}")
    assert rel[is_tf].max() <= 3e-3, f"tf: max rel err {rel[is_tf].max():.3e}: ad {ad[is_tf]} fd {fd[is_tf]}"
    assert rel[~is_tf].max() <= 1e-2, f"voxels: max rel err {rel[~is_tf].max():.3e}: ad {ad[~is_tf]} fd {fd[~is_tf]}"


def test_preparation_adjoint_without_the_kept_arrays(gpu_context):
    """The forward keeps the preparation's Levinson solution and exponential moments for the backward on the same
    buffers.  A backward on buffers of an earlier forward (another forward ran since) and a backward after a
    forward in the float-float precision form prepare them again: the first must give the gradients of the kept
    path (up to the order of the float atomics), the second those of its own multipliers (within 1e-3 of the FP32
    forward's gradients)."""
    import mray_gb300 as M

    wl, _ = _workload(m=31)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    weights = np.random.default_rng(9).standard_normal((wl.height, wl.width, 4))
    R1, R2 = GpuRender(gpu_context, wl), GpuRender(gpu_context, wl)
    R1.forward(wl.volume, table)
    gtf, gvol = R1.backward(weights)
    R2.forward(wl.volume, table)
    gtf2, gvol2 = R1.backward(weights)
    assert np.allclose(gvol2, gvol, rtol=1e-5, atol=1e-6 * np.abs(gvol).max())
    assert np.allclose(gtf2, gtf, rtol=1e-5, atol=1e-6 * np.abs(gtf).max())
    gpu_context.precision = M.PRECISION_COMPENSATED_FF_MESE
    try:
        R1.forward(wl.volume, table)
        _, gvol3 = R1.backward(weights)
    finally:
        gpu_context.precision = M.PRECISION_FP32
    assert np.abs(gvol3 - gvol).max() <= 1e-3 * np.abs(gvol).max()


def test_autograd_function_and_tf1d_chain(gpu_context):
    """torch.autograd.Function: the same gradients as the direct calls, and through preintegrate_table to the 1D
    extinction / emission entries."""
    from mray_gb300.autograd import RenderSpec, preintegrate_table, render

    wl, target_tf = _workload(m=16)
    spec = RenderSpec(wl.camera, wl.gen, wl.rec, wl.width, wl.height, wl.num_moments, wl.domain_min, wl.domain_max,
                      gpu_context)
    vol = torch.from_numpy(wl.volume).cuda().requires_grad_(True)
    tf1d = torch.from_numpy(wl.tf1d.astype(np.float32)).cuda().requires_grad_(True)
    with torch.no_grad():
        target = render(vol, preintegrate_table(torch.from_numpy(target_tf).cuda(), wl.tf_step), spec)
    rgba = render(vol, preintegrate_table(tf1d, wl.tf_step), spec)
    loss = ((rgba - target) ** 2).sum()
    loss.backward()
    R = GpuRender(gpu_context, wl)
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    r = R.forward(wl.volume, table)
    gtf, gvol = R.backward(2.0 * (r - target.cpu().numpy()))
    assert np.allclose(vol.grad.cpu().numpy(), gvol, rtol=1e-4, atol=1e-6 * np.abs(gvol).max())
    # chain to the 1D table: d table / d tf1d by hand
    s = wl.tf_step
    t1 = wl.tf1d.astype(np.float64)
    expect = np.zeros_like(t1)
    expect[:, :3] = gtf[:, :3] * (t1[:, 3:4] * s)
    expect[:, 3] = (gtf[:, :3] * t1[:, :3]).sum(axis=1) * s + gtf[:, 3] * s
    assert np.allclose(tf1d.grad.cpu().numpy(), expect, rtol=1e-3, atol=1e-5 * np.abs(expect).max())


def test_diff_form_argument_errors(gpu_context):
    import mray_gb300 as M

    wl, _ = _workload(m=8)
    R = GpuRender(gpu_context, wl)
    R.forward(wl.volume, O.preintegrate(wl.tf1d, wl.tf_step))
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):
        gpu_context.diff_tf_sampling = 7
    wl.gen.compact_image = 1
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):
        R.forward(wl.volume, O.preintegrate(wl.tf1d, wl.tf_step))
    wl.gen.compact_image = 0
    # particles: transfer-function gradient only
    from mray_gb300 import workloads as Wk

    p = Wk.sph_workload(n=2000, h=1.0 / 16, width=wl.width, height=wl.height, num_moments=8)
    gpu_context.upload_particles(p.x, p.y, p.z, p.v, p.h, p.domain_min, p.domain_max)
    gtf = torch.zeros((256, 4), device="cuda")
    gvol = torch.zeros(8, device="cuda")
    g = torch.zeros_like(R.rgba)
    with pytest.raises(M.MrayError, match="NOT_SUPPORTED"):
        gpu_context.diff_backward(wl.camera, wl.gen, wl.rec, wl.width, wl.height, 8, R.tab, R.moments, R.bounds4,
                                  R.pm, R.rgba, g, gtf, gvol)
