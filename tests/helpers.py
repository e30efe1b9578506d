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
