"""The oracle's restatement of the per-particle smoothing-length variant (Wendland C2; not in the reference, so its
parity is unpinned) against a brute-force evaluation of its definition: for random points, every particle within its
own support (r < h_i, and r^2 below the largest h squared, the grid's radius test) weighted by
(1 - q)^4 (1 + 4q) / h_i^3, q = r / h_i, the weighted values summed and divided by the weight sum.  The grid search
must find exactly the particles of the brute-force sum: the FP64 form agrees to rounding; the FP32 form within the
rounding of its float sums."""
import numpy as np

import oracle as O


def _case(n=4000, seed=3):
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 3)).astype(np.float32)
    pts[: n // 3] = np.clip(0.5 + 0.05 * rng.standard_normal((n // 3, 3)), 0.0, 1.0).astype(np.float32)
    v = rng.lognormal(0.0, 0.5, n).astype(np.float32)
    h = rng.uniform(0.04, 0.12, n).astype(np.float32)
    return pts, v, h


def _brute(pts, v, h, p):
    d = pts.astype(np.float64) - p
    r2 = (d * d).sum(axis=1)
    r = np.sqrt(r2)
    hmax = np.float64(np.float32(h.max()) * np.float32(h.max()))
    q = r / h.astype(np.float64)
    take = (r2 < hmax) & (q < 1.0)
    w = (1.0 - q[take]) ** 4 * (1.0 + 4.0 * q[take]) / h.astype(np.float64)[take] ** 3
    return float((w * v[take]).sum() / w.sum()) if take.any() else 0.0, int(take.sum())


def test_wendland_restatement_against_brute_force():
    pts, v, h = _case()
    parts = O.ParticleSet(pts[:, 0], pts[:, 1], pts[:, 2], v, h, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    assert abs(parts.h - float(h.max())) == 0.0
    rng = np.random.default_rng(9)
    points = np.concatenate([rng.random((200, 3)), 0.5 + 0.03 * rng.standard_normal((100, 3))]).astype(np.float32)
    got64 = O.particles_sample(parts, points.astype(np.float64), "f64")
    got32 = O.particles_sample(parts, points, "f32")
    counts = []
    for i, p in enumerate(points.astype(np.float64)):
        want, k = _brute(pts, v, h, p)
        counts.append(k)
        assert abs(got64[i] - want) <= 1e-12 * max(1.0, abs(want)), (i, got64[i], want)
        assert abs(got32[i] - want) <= 2e-5 * max(1.0, abs(want)), (i, got32[i], want)
    assert min(counts) > 0 and max(counts) > 30  # sparse and crowded neighbourhoods both covered


def test_single_h_unchanged_by_the_variant():
    """The reference's form (one h, cubic spline) is untouched: a scalar h builds the cubic-spline grid."""
    pts, v, _ = _case(n=1500, seed=5)
    parts = O.ParticleSet(pts[:, 0], pts[:, 1], pts[:, 2], v, 0.08, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    p = np.array([[0.5, 0.5, 0.5]], np.float32)
    a = O.particles_sample(parts, p, "f32")[0]
    d = pts.astype(np.float64) - p[0]
    r = np.sqrt((d * d).sum(axis=1))
    x = r / np.float64(np.float32(1.0) / np.float32(0.08)) ** -1
    take = r * r < np.float64(np.float32(0.08) * np.float32(0.08))
    xs = x[take]
    w = 0.5641895835477563 * (1.0 - 1.5 * xs * xs * (1.0 - 0.5 * xs))
    assert abs(a - (w * v[take]).sum() / w.sum()) <= 2e-5 * abs(a)
