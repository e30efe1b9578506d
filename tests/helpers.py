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


def rgba_agreement(ours: np.ndarray, ref32: np.ndarray, ref64: np.ndarray, tol: float = 1e-3,
                   sensitivity: np.ndarray | None = None) -> np.ndarray:
    """The per-pixel RGBA bar.  True where the colour matches the reference's FP32 result within ``tol`` (max over
    channels); or, where the reference's own FP32 result is further than ``tol`` from the FP64 evaluation of the same
    method, where ours is at least as close to that FP64 value as the reference's is; or, with ``sensitivity`` (the
    FP64 colour's change under a shift of every reconstructed density by +-1e-5, :func:`fp64_sensitivity`), where
    ours is within ``tol`` plus that change of the FP64 colour.  The last clause covers the pixels where a sample
    sits on a jump of the reference's transfer-function lookup (texel pair from the front density, weight from the
    back density's fraction: the colour is discontinuous at every multiple of 1/256), where any two evaluations
    that differ in the last bits -- FP64 against FP64 included -- can land on either side."""
    d_ref = np.abs(ours.astype(np.float64) - ref32).max(axis=-1)
    d_64 = np.abs(ours.astype(np.float64) - ref64).max(axis=-1)
    own = np.abs(ref32.astype(np.float64) - ref64).max(axis=-1)
    ok = (d_ref <= tol) | (d_64 <= np.maximum(tol, own))
    if sensitivity is not None:
        ok |= d_64 <= tol + sensitivity
    return ok


def fp32_density_bound(width, height, m, index, pm, bounds, floor=1e-5):
    """Per pixel, a bound on how far an FP32 evaluation of the MESE density can stray: the series
    lambda_0 + 2 sum_k lambda_k cos(k p) evaluated in FP32 errs by about m eps sum |lambda|, and the density is
    lo + (hi - lo) (atan(S) / pi + 1/2), whose slope in S is at most (hi - lo) / pi.  At least ``floor``."""
    idx = np.asarray(index, dtype=np.int64)
    n = np.diff(idx)
    pmv = np.abs(np.asarray(pm, dtype=np.float64))
    csum = np.concatenate([[0.0], np.cumsum(pmv)])
    first = pmv[np.minimum(idx[:-1], max(pmv.size - 1, 0))] if pmv.size else np.zeros(n.size)
    lam = np.where(n > 0, 2.0 * (csum[idx[1:]] - csum[idx[:-1]]) - first, 0.0)
    b = np.asarray(bounds, dtype=np.float64).reshape(-1, 2) / 65535.0
    span = b[:, 1] - b[:, 0]
    bound = m * 2.0 ** -24 * lam * span / np.pi
    return np.maximum(bound, floor).reshape(height, width)


def fp64_sensitivity(cam, rp, width, height, m, dmin, dmax, index, pm64, bounds, tf, rows=None, delta=1e-5):
    """Per pixel, the largest change of the FP64 colour (max over channels) when every reconstructed density moves by
    +delta or -delta (the oracle's density_offset; delta a scalar or one value per pixel)."""
    import oracle as O

    base = O.reconstruct(cam, rp, width, height, m, dmin, dmax, index, pm64, bounds, tf, "f64", rows=rows)
    sens = np.zeros((height, width))
    for d in (delta, -np.asarray(delta)):
        c = O.reconstruct(cam, rp, width, height, m, dmin, dmax, index, pm64, bounds, tf, "f64", rows=rows,
                          density_offset=d)
        sens = np.maximum(sens, np.abs(c - base).max(axis=-1))
    return sens


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


# ---- the differentiation form: GPU forward / backward on fixed buffers and central differences ----

class GpuRender:
    """The GPU forward / backward of one workload on fixed device buffers."""

    def __init__(self, ctx, wl):
        import torch

        self.ctx, self.wl = ctx, wl
        W, H, m = wl.width, wl.height, wl.num_moments
        self.moments = torch.empty(W * H * m, device="cuda")
        self.bounds4 = torch.empty(W * H * 4, device="cuda")
        self.pm = torch.empty(W * H * m, device="cuda")
        self.rgba = torch.empty((H, W, 4), device="cuda")

    def forward(self, volume, table):
        import torch

        wl = self.wl
        self.vol = torch.from_numpy(np.ascontiguousarray(volume, dtype=np.float32)).cuda()
        self.tab = torch.from_numpy(np.ascontiguousarray(table, dtype=np.float32)).cuda()
        self.ctx.upload_grid(self.vol, wl.domain_min, wl.domain_max)
        self.ctx.diff_forward(wl.camera, wl.gen, wl.rec, wl.width, wl.height, wl.num_moments, self.tab, self.moments,
                              self.bounds4, self.pm, self.rgba)
        self.ctx.synchronize()
        return self.rgba.cpu().numpy().astype(np.float64)

    def backward(self, grad_rgba, volume_grad=True):
        import torch

        wl = self.wl
        g = torch.from_numpy(np.ascontiguousarray(grad_rgba, dtype=np.float32)).cuda()
        gtf = torch.zeros((256, 4), device="cuda")
        gvol = torch.zeros_like(self.vol) if volume_grad else None
        self.ctx.diff_backward(wl.camera, wl.gen, wl.rec, wl.width, wl.height, wl.num_moments, self.tab, self.moments,
                               self.bounds4, self.pm, self.rgba, g, gtf, gvol)
        self.ctx.synchronize()
        return gtf.cpu().numpy().astype(np.float64), (gvol.cpu().numpy().astype(np.float64) if volume_grad else None)


def pick_parameters(rng, grad_vol, grad_tf, n_tf, n_vox):
    """Seeded parameters whose gradient is not negligible (above 1 % of the largest of its kind)."""
    tf_ok = np.argwhere(np.abs(grad_tf) > 1e-2 * np.abs(grad_tf).max())
    vox_ok = np.argwhere(np.abs(grad_vol) > 1e-2 * np.abs(grad_vol).max())
    params = [("tf", tuple(tf_ok[i])) for i in rng.choice(len(tf_ok), n_tf, replace=False)]
    params += [("vox", tuple(vox_ok[i])) for i in rng.choice(len(vox_ok), n_vox, replace=False)]
    return params


def perturbed(wl, table, kind, idx, delta):
    v, t = wl.volume, table
    if kind == "vox":
        v = wl.volume.copy()
        v[idx] += np.float32(delta)
    else:
        t = table.copy()
        t[idx] += delta
    return v, t


def richardson(loss, wl, table, kind, idx, eps):
    """Central differences at eps and 2 eps combined as (4 D(eps) - D(2 eps)) / 3, which removes their eps^2
    truncation term: voxels near where rays enter the volume change the image strongly enough that D(1e-3) alone
    is off by a few 1e-3."""
    def d(e):
        return (loss(*perturbed(wl, table, kind, idx, e)) - loss(*perturbed(wl, table, kind, idx, -e))) / (2 * e)
    return (4.0 * d(eps) - d(2 * eps)) / 3.0
