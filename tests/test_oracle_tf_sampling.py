"""The differentiation form's two transfer-function rows in the oracle (CPU only), against their definitions: the
linear row is the GPU texture's interpolation between the texel centres u = 256 fs - 1/2 (transfer_function_device.cuh:
30-65) with clamp to edge; the cubic B-spline row, on the same knots, reproduces constants and linear ramps away from
the clamped ends (the uniform cubic B-splines sum to one and their first moment is u)."""
import numpy as np

import oracle as O


def _linear_reference(table, fs):
    u = 256.0 * fs - 0.5
    i = int(np.floor(u))
    t = u - i
    x0, x1 = min(max(i, 0), 255), min(max(i + 1, 0), 255)
    return (1.0 - t) * table[x0] + t * table[x1]


def test_linear_row_is_the_texture_interpolation():
    rng = np.random.default_rng(3)
    table = rng.random((256, 4))
    points = np.concatenate([rng.random(200), [0.0, 1.0 / 1024, 1.0 / 512, 0.5, 1.0 - 1.0 / 512, 1.0, -0.01, 1.01]])
    for fs in points:
        np.testing.assert_allclose(O.tf_sample_diff(table, fs, linear=True), _linear_reference(table, fs),
                                   rtol=0, atol=1e-14)


def test_bspline_row_reproduces_constants_and_ramps():
    rng = np.random.default_rng(4)
    const = np.tile(rng.random(4), (256, 1))
    ramp = np.repeat(np.arange(256, dtype=np.float64)[:, None], 4, axis=1)
    for fs in rng.uniform(3.0 / 256, 1.0 - 3.0 / 256, 200):
        np.testing.assert_allclose(O.tf_sample_diff(const, fs), const[0], rtol=1e-14)
        np.testing.assert_allclose(O.tf_sample_diff(ramp, fs), np.full(4, 256.0 * fs - 0.5), rtol=0, atol=1e-11)
