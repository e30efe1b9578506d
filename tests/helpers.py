"""Shared helpers of the parity tests: error metrics and small seeded cases."""
from __future__ import annotations

import numpy as np


def moment_rel_err(a: np.ndarray, b: np.ndarray, ref_m0: np.ndarray) -> np.ndarray:
    """Per pixel max_j |a_j - b_j| / max(|m_0|, 1e-3): bounded trigonometric moments satisfy |m_j| <= m_0 for a
    non-negative signal, so m_0 is their natural scale."""
    d = np.abs(a.astype(np.float64) - b.astype(np.float64)).max(axis=-1)
    return d / np.maximum(np.abs(ref_m0.astype(np.float64)), 1e-3)


def small_ml(width=96, height=80, m=31, seed=11, n=64):
    from mray_gb300 import workloads as W

    return W.ml_workload(n=n, width=width, height=height, num_moments=m, seed=seed, name=f"ml{n}_{width}x{height}_m{m}")


def small_mixing(width=64, height=64, m=64, n=96, seed=21):
    from mray_gb300 import workloads as W

    return W.mixing_layer_workload(n=n, width=width, height=height, num_moments=m, seed=seed)


def rgba_agreement(ours: np.ndarray, ref32: np.ndarray, ref64: np.ndarray, tol: float = 1e-3) -> np.ndarray:
    """Per pixel: True where the colour matches the reference's FP32 result within ``tol`` (max over channels), or,
    where the reference's own FP32 result is further than ``tol`` from the FP64 evaluation of the same method, where
    ours is at least as close to that FP64 value as the reference's is."""
    d_ref = np.abs(ours.astype(np.float64) - ref32).max(axis=-1)
    d_64 = np.abs(ours.astype(np.float64) - ref64).max(axis=-1)
    own = np.abs(ref32.astype(np.float64) - ref64).max(axis=-1)
    return (d_ref <= tol) | (d_64 <= np.maximum(tol, own))


def moments_bounds_agree(b32: np.ndarray, b64: np.ndarray) -> np.ndarray:
    """Pixels whose u16 density bounds agree between the FP32 and FP64 evaluations (the bounds are truncated to
    u16, so a last-bit difference of the sampled extremes can move them one step)."""
    return np.all(b32 == b64, axis=-1)


def single_scattering_case(cache_size=(24, 20, 16), light_shape=(40, 36), direction=(0.3, -1.0, 0.2),
                           scattering=0.5):
    """The single-scattering case of tests/golden/single_scattering.npz: the 64^3 Marschner-Lobb volume seen by the
    48x40 golden camera, an orthographic light along ``direction`` and a light image of ``light_shape`` with the
    golden workload's moments.  Returns (workload, light camera, reconstruction parameters)."""
    from mray_gb300 import workloads as W
    from mray_gb300.types import ReconstructionParameters, SingleScatteringParameters

    wl = W.ml_workload(n=64, width=48, height=40, num_moments=16, seed=11, name="golden_ml")
    light = W.light_camera(direction)
    cx, cy, cz = cache_size
    ssp = SingleScatteringParameters(enable=1, use_cache=1, cache_size_x=cx, cache_size_y=cy, cache_size_z=cz,
                                     henyey_greenstein_g=0.3, direction_x=light.dir[0], direction_y=light.dir[1],
                                     direction_z=light.dir[2], intensity_r=0.9, intensity_g=0.8, intensity_b=0.7)
    rp = ReconstructionParameters(step_size=wl.rec.step_size, bias=wl.rec.bias, medium_emission=1.0,
                                  medium_scattering=scattering, early_ray_termination=0.99, ss=ssp)
    return wl, light, rp


def light_generation_parameters(wl):
    """The light image's generation: compact, bounds, prediction coded, error threshold 0.01 (the reference's
    single-scattering image settings, eval/turbine/turbine_single_scattering.json)."""
    from mray_gb300.types import GenerationParameters

    return GenerationParameters(step_size=wl.gen.step_size, error_threshold=0.01, bias=wl.gen.bias, compact_image=1,
                                prediction_coding=1, transform_to_bounds=1, transform_bound_eps=0.005)
