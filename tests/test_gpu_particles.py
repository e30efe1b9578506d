"""GPU parity of moment generation over SPH particles against the oracle and the reference's fixtures.

The device builds the reference's uniform particle grid (cell size h, origin at the particles' minimum, 4x4x4
tiled cells) with the particles of a cell in input order, and samples with the 27-cell sum of Particles::sample.
The samples, and so the u16 bounds and the compaction counts, are bit-exact with the oracle; the moments meet
the same per-pixel tolerance as the grid path (1e-4 relative to m_0, widened by the reference's own FP32
error, and 1e-4 against the FP64 evaluation).
"""
import os

import numpy as np
import pytest

import oracle as O
from helpers import moment_rel_err, moments_bounds_agree

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MOMENT_TOL = 1e-4
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _gpu_particle_moments(ctx, x, y, z, v, h, dmin, dmax, cam, gen, W, H, m, precision=0, on_device=False):
    import mray_gb300 as M

    ctx.precision = precision
    per_particle = np.ndim(h) > 0
    if on_device:
        arrs = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
                for a in ((x, y, z, v, h) if per_particle else (x, y, z, v))]
        if per_particle:
            ctx.upload_particles_h(*arrs, dmin, dmax)
        else:
            ctx.upload_particles(*arrs, h, dmin, dmax)
    elif per_particle:
        ctx.upload_particles_h(x, y, z, v, h, dmin, dmax)
    else:
        ctx.upload_particles(x, y, z, v, h, dmin, dmax)
    mo = torch.zeros(W * H * m, dtype=torch.float32, device="cuda")
    b = torch.zeros(2 * W * H, dtype=torch.int16, device="cuda")
    c = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    ctx.stage_generate_moments(cam, gen, W, H, m, mo, b, c)
    ctx.synchronize()
    ctx.precision = M.PRECISION_FP32
    return (mo.cpu().numpy().reshape(H, W, m), b.cpu().numpy().view(np.uint16).reshape(H, W, 2),
            c.cpu().numpy().view(np.uint32).reshape(H, W))


def _check_against_oracle(ctx, x, y, z, v, h, dmin, dmax, cam, gen, W, H, m, **kw):
    mo, b, c = _gpu_particle_moments(ctx, x, y, z, v, h, dmin, dmax, cam, gen, W, H, m, **kw)
    parts = O.ParticleSet(x, y, z, v, h, dmin, dmax)
    ref_m, ref_b, ref_c = O.generate_moments_particles(cam, gen, parts, W, H, m, "f32")
    ref64, b64, _ = O.generate_moments_particles(cam, gen, parts, W, H, m, "f64")
    assert np.array_equal(b, ref_b)
    assert np.array_equal(c, ref_c)
    hit = ref_c > 0
    assert hit.sum() > 0
    own = moment_rel_err(ref_m, ref64, ref64[..., 0])
    err = moment_rel_err(mo, ref_m, ref_m[..., 0])
    assert np.all(err[hit] <= MOMENT_TOL + own[hit]), f"max excess {(err - own)[hit].max():.3e}"
    same = hit & moments_bounds_agree(ref_b, b64)
    err64 = moment_rel_err(mo, ref64, ref64[..., 0])[same]
    assert err64.max() <= MOMENT_TOL, f"max rel err vs f64 {err64.max():.3e}"
    return mo, b, c


def _fixture(prefix):
    from mray_gb300.types import Camera, GenerationParameters

    g = np.load(os.path.join(GOLDEN, "particles.npz"))
    x, y, z, v = (np.ascontiguousarray(a) for a in g[f"{prefix}_xyzv"])
    dmin, dmax = (tuple(float(t) for t in r) for r in g[f"{prefix}_domain"])
    cam = Camera.from_buffer_copy(g[f"{prefix}_camera"].tobytes())
    gen = GenerationParameters.from_buffer_copy(g[f"{prefix}_gen"].tobytes())
    return g, (x, y, z, v, float(g[f"{prefix}_h"]), dmin, dmax, cam, gen, *(int(s) for s in g[f"{prefix}_shape"]))


@pytest.mark.parametrize("prefix", ["lattice", "cluster"])
def test_particles_match_reference_fixture(gpu_context, prefix):
    """Against the reference's own generate() over Particles: index and bounds exact (the lattice has one
    particle per cell, the clustered set's bounds may move by one u16 step with the reference's sort order),
    compact moments within 1e-4 of m_0."""
    g, args = _fixture(prefix)
    mo, b, c = _check_against_oracle(gpu_context, *args)
    W, H, m = args[-3:]
    index, data = O.compact(c, mo)
    assert np.array_equal(index, g[f"{prefix}_index"])
    db = np.abs(b.reshape(-1).astype(np.int64) - g[f"{prefix}_bounds"].astype(np.int64)).max()
    assert db == 0 if prefix == "lattice" else db <= 1
    ref = g[f"{prefix}_data"]
    m0 = np.repeat(ref.reshape(-1, m)[:, :1], m, axis=1).reshape(-1)
    assert np.max(np.abs(data - ref) / np.maximum(np.abs(m0), 1e-3)) <= MOMENT_TOL


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("m", [16, 128])
def test_sph_workload_matches_oracle(gpu_context, precision, m):
    from mray_gb300 import workloads as W

    wl = W.sph_workload(n=20000, h=1.0 / 32, width=64 if m <= 64 else 32, height=56 if m <= 64 else 24,
                        num_moments=m, seed=31)
    _check_against_oracle(gpu_context, wl.x, wl.y, wl.z, wl.v, wl.h, wl.domain_min, wl.domain_max, wl.camera,
                          wl.gen, wl.width, wl.height, wl.num_moments, precision=precision)


def test_flat_particle_set(gpu_context):
    """All particles in one z plane: a grid one cell deep with 4x4x1 tiles (getIndexFromCell's flat case)."""
    from mray_gb300 import workloads as W

    wl = W.sph_workload(n=4000, h=1.0 / 24, width=40, height=40, num_moments=8, seed=5)
    z = np.full_like(wl.z, np.float32(0.5))
    dmin = (wl.domain_min[0], wl.domain_min[1], 0.45)
    dmax = (wl.domain_max[0], wl.domain_max[1], 0.55)
    _check_against_oracle(gpu_context, wl.x, wl.y, z, wl.v, wl.h, dmin, dmax, wl.camera, wl.gen, 40, 40, 8)


def test_crowded_cells_keep_input_order(gpu_context):
    """Thousands of particles in a few cells (one cell holds about a third of them): the device's radix sort
    keeps the input order inside a cell, so the float sums match the oracle's bit for bit (bounds exact), and
    two uploads give identical moments."""
    from mray_gb300 import workloads as W

    rng = np.random.default_rng(4)
    n = 6000
    h = 0.05
    base = rng.random((n, 3)).astype(np.float32)
    pos = np.where(rng.random((n, 1)) < 0.35, np.float32(0.5) + np.float32(0.3 * h) * base, base)
    pos = pos.astype(np.float32)
    v = rng.lognormal(0.0, 0.5, size=n).astype(np.float32)
    wl = W.sph_workload(n=64, h=h, width=40, height=32, num_moments=8, seed=2)
    wl.gen.step_size = h / 2
    wl.gen.data_min, wl.gen.data_max = 0.3, 3.0
    args = (pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), v, h, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0),
            wl.camera, wl.gen, 40, 32, 8)
    mo1, b1, c1 = _check_against_oracle(gpu_context, *args)
    mo2, b2, c2 = _gpu_particle_moments(gpu_context, *args, on_device=True)
    assert np.array_equal(mo1, mo2) and np.array_equal(b1, b2) and np.array_equal(c1, c2)


def test_particle_upload_errors(gpu_context):
    import mray_gb300 as M

    x = np.zeros(4, np.float32)
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):
        gpu_context.upload_particles(x[:0], x[:0], x[:0], x[:0], 0.1, (0, 0, 0), (1, 1, 1))
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):
        gpu_context.upload_particles(x, x, x, x, 0.0, (0, 0, 0), (1, 1, 1))
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):
        gpu_context.upload_particles(x, x, x, x, 0.1, (0, 0, 0), (1, 0, 1))
    far = np.array([0.0, 1.0, 0.0, 1.0], np.float32)
    with pytest.raises(M.MrayError, match="INVALID_ARGUMENT"):  # 10^12 cells
        gpu_context.upload_particles(far, far, far, x, 1e-4, (0, 0, 0), (1, 1, 1))
    # a failed upload leaves no volume behind
    mi_cam = M.Camera()
    gp = M.GenerationParameters(step_size=0.01)
    mo = torch.zeros(16, dtype=torch.float32, device="cuda")
    with pytest.raises(M.MrayError, match="NO_VOLUME"):
        gpu_context.stage_generate_moments(mi_cam, gp, 4, 4, 1, mo, None, None)


def _wendland_case(n=30000, seed=41, W=48, H=40, m=16):
    """The per-particle smoothing-length variant on a small case: clustered particles, h uniform in [0.03, 0.06]
    (about six particles per cell of the 0.06 grid), step 2^-6."""
    from mray_gb300 import workloads as W_

    wl = W_.sph_workload(n=n, h=0.06, width=W, height=H, num_moments=m, seed=seed)
    wl.h = np.random.default_rng(seed).uniform(0.03, 0.06, size=n).astype(np.float32)
    wl.gen.step_size = 2.0 ** -6
    return wl


@pytest.mark.parametrize("on_device", [False, True])
def test_wendland_variant_matches_oracle(gpu_context, on_device):
    """The Wendland C2 variant with a smoothing length per particle (parity unpinned: the reference has no such
    form; the oracle's restatement, oracle_particles_create_h, is the check): bounds and counts exact, moments
    within the particle path's bar against the oracle's FP32 and FP64 evaluations."""
    wl = _wendland_case()
    _check_against_oracle(gpu_context, wl.x, wl.y, wl.z, wl.v, wl.h, wl.domain_min, wl.domain_max, wl.camera,
                          wl.gen, wl.width, wl.height, wl.num_moments, on_device=on_device)


def test_wendland_variant_kahan_and_unsupported_paths(gpu_context):
    import mray_gb300 as M

    wl = _wendland_case(n=12000, seed=43, W=33, H=17, m=31)
    _check_against_oracle(gpu_context, wl.x, wl.y, wl.z, wl.v, wl.h, wl.domain_min, wl.domain_max, wl.camera,
                          wl.gen, wl.width, wl.height, wl.num_moments, precision=M.PRECISION_COMPENSATED_FF_MESE)
    # smoothing lengths must be finite and > 0
    for bad in (0.0, -0.01, np.nan, np.inf):
        h = wl.h.copy()
        h[17] = bad
        with pytest.raises(M.MrayError) as e:
            gpu_context.upload_particles_h(wl.x, wl.y, wl.z, wl.v, h, wl.domain_min, wl.domain_max)
        assert e.value.status == 1
    # the renderers without a per-particle form say so
    gpu_context.upload_particles_h(wl.x, wl.y, wl.z, wl.v, wl.h, wl.domain_min, wl.domain_max)
    rgba = torch.zeros(wl.width * wl.height * 4, device="cuda")
    gpu_context.upload_tf(O.preintegrate(wl.tf1d, wl.tf_step))
    from mray_gb300.types import ReferenceParameters

    rp = ReferenceParameters(step_size=wl.gen.step_size, data_min=wl.gen.data_min, data_max=wl.gen.data_max)
    with pytest.raises(M.MrayError) as e:
        gpu_context.stage_generate_reference(wl.camera, rp, wl.width, wl.height, rgba)
    assert e.value.status == 6
