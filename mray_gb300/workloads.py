"""Seeded synthetic inputs that stand in for the reference's datasets.

The reference evaluates on NetCDF / H5Part datasets (Marschner-Lobb, mixing layers, SPH runs) that are not
available here; these generators produce fields of the same shapes, sizes and value ranges:

* :func:`marschner_lobb`   -- the analytic Marschner-Lobb test function on [-1, 1]^3, sampled at the
  reference's corner-aligned voxel positions x_i = -1 + 2 i / N (src/volume.h:97-123 maps voxel i to
  min + i/N (max - min)).
* :func:`mixing_layer`     -- rho = 0.5 (1 + tanh((z - z0 - h(x, y)) / 0.02)) on [0, 1]^3, h a sum of seeded
  Fourier modes (wavenumbers 1..32, amplitude ~ k^(-5/3)), plus 5 % seeded Gaussian noise.
* :func:`transfer_function` -- a 256-entry RGBA table: extinction and emission each the sum of 4 seeded
  Gaussian bumps.
* cameras: a seeded orthographic view of the unit-diagonal cube and a perspective view.

Volumes are float32 arrays indexed ``[z, y, x]`` (x fastest in memory, as ``RegularGrid::read``).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .types import Camera, GenerationParameters, ReconstructionParameters


def marschner_lobb(n: int, alpha: float = 0.25, f_m: float = 6.0) -> np.ndarray:
    """rho(x,y,z) = (1 - sin(pi z / 2) + alpha (1 + cos(2 pi f_M cos(pi r / 2)))) / (2 (1 + alpha)),
    r = sqrt(x^2 + y^2), on [-1, 1]^3."""
    c = (-1.0 + 2.0 * np.arange(n, dtype=np.float64) / n)
    z = c[:, None, None]
    y = c[None, :, None]
    x = c[None, None, :]
    r = np.sqrt(x * x + y * y)
    rho = (1.0 - np.sin(np.pi * z / 2.0) + alpha * (1.0 + np.cos(2.0 * np.pi * f_m * np.cos(np.pi * r / 2.0))))
    rho = rho / (2.0 * (1.0 + alpha))
    return np.ascontiguousarray(np.broadcast_to(rho, (n, n, n)), dtype=np.float32)


def mixing_layer(n: int, modes: int = 64, seed: int = 1, noise: float = 0.05, z0: float = 0.5,
                 amplitude: float = 0.08, width: float = 0.02) -> np.ndarray:
    """A mixing-layer-like field on [0, 1]^3 (see the module docstring)."""
    rng = np.random.default_rng(seed)
    k = rng.uniform(1.0, 32.0, size=modes)
    theta = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    amp = k ** (-5.0 / 3.0)
    amp *= amplitude / np.sqrt(np.sum(amp * amp) / 2.0)
    c = np.arange(n, dtype=np.float64) / n
    xx, yy = np.meshgrid(c, c, indexing="xy")  # [y, x]
    h = np.zeros((n, n), dtype=np.float64)
    for i in range(modes):
        kx, ky = k[i] * np.cos(theta[i]), k[i] * np.sin(theta[i])
        h += amp[i] * np.cos(2.0 * np.pi * (kx * xx + ky * yy) + phase[i])
    h32 = h.astype(np.float32)
    out = np.empty((n, n, n), dtype=np.float32)
    zc = c.astype(np.float32)
    inv_w = np.float32(1.0 / width)
    for iz in range(n):
        np.tanh((zc[iz] - np.float32(z0) - h32) * inv_w, out=out[iz])
    out += np.float32(1.0)
    out *= np.float32(0.5)
    if noise > 0.0:
        nrng = np.random.default_rng(seed + 1000003)
        chunk = max(1, (1 << 24) // (n * n))
        for z in range(0, n, chunk):
            out[z:z + chunk] += np.float32(noise) * nrng.standard_normal(out[z:z + chunk].shape, dtype=np.float32)
    return out


def transfer_function(seed: int = 7, bumps: int = 4) -> np.ndarray:
    """A 256 x RGBA float table: alpha (extinction) and rgb (emission) are sums of seeded Gaussian bumps."""
    rng = np.random.default_rng(seed)
    s = np.arange(256, dtype=np.float64) / 256.0
    tf = np.zeros((256, 4), dtype=np.float64)
    for _ in range(bumps):
        c, w, a = rng.uniform(0.15, 0.9), rng.uniform(0.02, 0.08), rng.uniform(0.3, 1.0)
        tf[:, 3] += a * np.exp(-0.5 * ((s - c) / w) ** 2)
    tf[:, 3] /= tf[:, 3].max()
    for _ in range(bumps):
        c, w = rng.uniform(0.1, 0.95), rng.uniform(0.03, 0.12)
        col = rng.uniform(0.2, 1.0, size=3)
        tf[:, :3] += col[None, :] * np.exp(-0.5 * ((s - c) / w) ** 2)[:, None]
    tf[:, :3] /= max(1.0, tf[:, :3].max())
    return tf.astype(np.float32)


def _unit(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


def ortho_camera(seed: int, center=(0.0, 0.0, 0.0), half_extent: float = math.sqrt(3.0),
                 distance: float = 3.0) -> Camera:
    """A seeded orthographic view: unit direction d, right/up orthogonal to d spanning +-half_extent,
    position = center - distance * d."""
    rng = np.random.default_rng(seed)
    d = _unit(rng.normal(size=3))
    helper = np.array([0.0, 0.0, 1.0]) if abs(d[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    right = _unit(np.cross(d, helper))
    up = _unit(np.cross(right, d))
    pos = np.asarray(center, dtype=np.float64) - distance * d
    return Camera.orthographic_camera(pos, right * half_extent, up * half_extent, d)


def light_camera(direction, center=(0.0, 0.0, 0.0), half_extent: float = math.sqrt(3.0),
                 distance: float = 3.0) -> Camera:
    """An orthographic camera looking along ``direction``: the light of single scattering, whose image is the
    SingleScatteringImage and whose direction is SingleScatteringParameters' light direction
    (parse_ss_params, src/parameters.h:219-226)."""
    d = _unit(direction)
    helper = np.array([0.0, 0.0, 1.0]) if abs(d[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    right = _unit(np.cross(d, helper))
    up = _unit(np.cross(right, d))
    pos = np.asarray(center, dtype=np.float64) - distance * d
    return Camera.orthographic_camera(pos, right * half_extent, up * half_extent, d)


def look_at_transform(eye, target, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """Camera->world matrix (row-major) for a camera at ``eye`` looking at ``target``; the camera looks
    along -z in camera space (src/cut/raytracing.h:39-49)."""
    eye = np.asarray(eye, dtype=np.float64)
    f = _unit(np.asarray(target, dtype=np.float64) - eye)
    r = _unit(np.cross(f, up))
    u = np.cross(r, f)
    m = np.eye(4)
    m[:3, 0] = r
    m[:3, 1] = u
    m[:3, 2] = -f
    m[:3, 3] = eye
    return m


def perspective_camera(eye, target, fov_deg: float, aspect: float = 1.0, znear: float = 0.0) -> Camera:
    return Camera.perspective_camera(look_at_transform(eye, target), math.tan(math.radians(fov_deg) / 2.0),
                                     aspect, znear)


@dataclasses.dataclass
class Workload:
    """One configuration of the path: volume, view, image, moments and the two parameter blocks."""

    name: str
    volume: np.ndarray
    domain_min: tuple
    domain_max: tuple
    width: int
    height: int
    num_moments: int
    camera: Camera
    gen: GenerationParameters
    rec: ReconstructionParameters
    tf1d: np.ndarray
    tf_step: float  # step_size * preintegration_step_size_factor (main.cpp:100-105)

    @property
    def num_rays(self) -> int:
        return self.width * self.height


def ml_workload(n: int = 64, width: int = 512, height: int = 512, num_moments: int = 31, seed: int = 11,
                name: str = "ml64_512sq_m31_ortho") -> Workload:
    """Marschner-Lobb n^3 on [-1,1]^3, orthographic seeded view, 0.5-voxel steps, bounded moments
    (transform_to_bounds, eps 0.005), compaction with threshold 0, no prediction coding, bias 5e-5,
    emission 1.0, early termination 0.99 (eval/marschner_lobb/marschner_lobb.json)."""
    step = 0.5 * 2.0 / n
    gen = GenerationParameters(step_size=step, error_threshold=0.0, bias=5e-5, compact_image=1,
                               prediction_coding=0, transform_to_bounds=1, transform_bound_eps=0.005)
    rec = ReconstructionParameters(step_size=step, bias=5e-5, medium_emission=1.0, early_ray_termination=0.99)
    return Workload(name, marschner_lobb(n), (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), width, height, num_moments,
                    ortho_camera(seed), gen, rec, transfer_function(seed + 1), tf_step=0.05)


def mixing_layer_device(n: int, modes: int = 64, seed: int = 1, noise: float = 0.05, z0: float = 0.5,
                        amplitude: float = 0.08, width: float = 0.02, device: str = "cuda"):
    """The mixing-layer field of :func:`mixing_layer` built on the GPU with torch (for volumes too large to build
    on the host quickly, e.g. 1024^3): the same modes and formula; the 5 % noise comes from torch's seeded
    generator, so the values differ from the host version's while the distribution is the same."""
    import torch

    rng = np.random.default_rng(seed)
    k = rng.uniform(1.0, 32.0, size=modes)
    theta = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    amp = k ** (-5.0 / 3.0)
    amp *= amplitude / np.sqrt(np.sum(amp * amp) / 2.0)
    c = torch.arange(n, dtype=torch.float64, device=device) / n
    yy, xx = torch.meshgrid(c, c, indexing="ij")  # [y, x]
    h = torch.zeros((n, n), dtype=torch.float64, device=device)
    for i in range(modes):
        kx, ky = float(k[i] * np.cos(theta[i])), float(k[i] * np.sin(theta[i]))
        h += float(amp[i]) * torch.cos(2.0 * np.pi * (kx * xx + ky * yy) + float(phase[i]))
    h32 = h.float()
    zc = c.float()
    out = torch.empty((n, n, n), dtype=torch.float32, device=device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed + 1000003)
    for iz in range(n):
        sl = out[iz]
        torch.tanh((zc[iz] - z0 - h32) * (1.0 / width), out=sl)
        sl.add_(1.0).mul_(0.5)
        if noise > 0.0:
            sl.add_(noise * torch.randn((n, n), generator=gen, device=device, dtype=torch.float32))
    return out


def mixing_layer_setup(n: int, width: int, height: int, prediction_coding: bool = False, seed: int = 21):
    """The view and parameters of the mixing-layer workloads: (gen, rec, camera, tf1d, tf_step)."""
    step = 0.5 / n
    gen = GenerationParameters(step_size=step, error_threshold=0.0, bias=5e-5, compact_image=1,
                               prediction_coding=1 if prediction_coding else 0, transform_to_bounds=1,
                               transform_bound_eps=0.005, quantization_bits=10 if prediction_coding else 32,
                               coding_warp=0)
    rec = ReconstructionParameters(step_size=step, bias=5e-5, medium_emission=1.0, early_ray_termination=0.99)
    cam = perspective_camera(eye=(1.9, -1.1, 1.45), target=(0.5, 0.5, 0.5), fov_deg=38.0, aspect=width / height)
    return gen, rec, cam, transfer_function(seed + 1), 0.05 * (512.0 / n)


def mixing_layer_workload(n: int = 512, width: int = 1024, height: int = 1024, num_moments: int = 64,
                          modes: int = 64, seed: int = 21, prediction_coding: bool = False,
                          name: str | None = None) -> Workload:
    """Mixing layer n^3 on [0,1]^3, perspective view, 0.5-voxel steps."""
    gen, rec, cam, tf1d, tf_step = mixing_layer_setup(n, width, height, prediction_coding, seed)
    name = name or f"mixing_layer{n}_{width}x{height}_m{num_moments}_persp"
    return Workload(name, mixing_layer(n, modes=modes, seed=seed), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), width,
                    height, num_moments, cam, gen, rec, tf1d, tf_step=tf_step)


def diff_workload(n: int = 256, width: int = 512, height: int = 512, num_moments: int = 31, seed: int = 11,
                  noise: float = 0.05, name: str | None = None):
    """The differentiation form on a Marschner-Lobb n^3 volume with an orthographic seeded view: no compaction,
    early ray termination off (ert = 1: a march stops only where the transmittance is exactly 0), the preintegration
    step scaled with the sample count (0.05 * 64 / n).  Returns (workload, target_tf1d): the target transfer
    function carries seeded N(0, noise) perturbations on its 256 extinction (alpha) and 256 emission entries (one
    value per entry scaling the entry's rgb), clipped at 0.  The density range is [-0.1, 1.1], so that neither
    the density mapping nor the bounds transform clamps (both would put kinks into the loss)."""
    wl = ml_workload(n=n, width=width, height=height, num_moments=num_moments, seed=seed,
                     name=name or f"diff_ml{n}_{width}x{height}_m{num_moments}")
    wl.gen.compact_image = 0
    wl.gen.data_min, wl.gen.data_max = -0.1, 1.1
    wl.rec.early_ray_termination = 1.0
    wl.tf_step = 0.05 * 64.0 / n
    rng = np.random.default_rng(seed + 101)
    target = wl.tf1d.astype(np.float64).copy()
    target[:, 3] += rng.normal(0.0, noise, size=256)
    target[:, :3] *= (1.0 + rng.normal(0.0, noise, size=256))[:, None]
    return wl, np.clip(target, 0.0, None).astype(np.float32)


def sph_particles(n: int, seed: int = 31, clusters: int = 200, cluster_frac: float = 0.3):
    """Particles in the unit cube: (1 - cluster_frac) uniform and cluster_frac in seeded Gaussian clusters
    (sigma 0.01..0.05), clipped to the cube; values ~ LogNormal(0, 0.5).  Returns x, y, z, v (float32)."""
    rng = np.random.default_rng(seed)
    n_cl = int(n * cluster_frac)
    n_un = n - n_cl
    pts = np.empty((n, 3), dtype=np.float32)
    pts[:n_un] = rng.random((n_un, 3), dtype=np.float32)
    centres = rng.random((clusters, 3))
    sigmas = rng.uniform(0.01, 0.05, size=clusters)
    which = rng.integers(0, clusters, size=n_cl)
    pts[n_un:] = np.clip(centres[which] + sigmas[which, None] * rng.standard_normal((n_cl, 3)), 0.0, 1.0)
    v = rng.lognormal(0.0, 0.5, size=n).astype(np.float32)
    return pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), v


@dataclasses.dataclass
class ParticleWorkload:
    """A particle configuration: particles, one global smoothing length, view, image, moments, parameters."""

    name: str
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    v: np.ndarray
    h: float
    domain_min: tuple
    domain_max: tuple
    width: int
    height: int
    num_moments: int
    camera: Camera
    gen: GenerationParameters
    rec: ReconstructionParameters
    tf1d: np.ndarray
    tf_step: float


def sph_workload(n: int = 20000, h: float = 1.0 / 32, width: int = 64, height: int = 64, num_moments: int = 16,
                 seed: int = 31, name: str | None = None) -> ParticleWorkload:
    """SPH particles with one global smoothing length (the reference's grid: cell size = h); the ray box is the
    particles' bounding box (the loader's domain); step h / 2; data_min / data_max at the 1st / 99th
    percentiles of a seeded sample of the values."""
    x, y, z, v = sph_particles(n, seed)
    dmin = (float(x.min()), float(y.min()), float(z.min()))
    dmax = (float(x.max()), float(y.max()), float(z.max()))
    rng = np.random.default_rng(seed + 7)
    sample = v[rng.integers(0, n, size=min(n, 100000))]
    lo, hi = float(np.percentile(sample, 1)), float(np.percentile(sample, 99))
    step = h / 2
    gen = GenerationParameters(step_size=step, error_threshold=0.0, bias=5e-5, compact_image=1, prediction_coding=0,
                               transform_to_bounds=1, transform_bound_eps=0.005, data_min=lo, data_max=hi)
    rec = ReconstructionParameters(step_size=step, bias=5e-5, medium_emission=1.0, early_ray_termination=0.99)
    cam = perspective_camera(eye=(1.9, -1.1, 1.45), target=(0.5, 0.5, 0.5), fov_deg=38.0, aspect=width / height)
    name = name or f"sph{n}_h{h:g}_{width}x{height}_m{num_moments}"
    return ParticleWorkload(name, x, y, z, v, h, dmin, dmax, width, height, num_moments, cam, gen, rec,
                            transfer_function(seed + 1), tf_step=0.05)


def sph_wendland_workload(n: int = 16_000_000, h_range=(0.005, 0.02), width: int = 1024, height: int = 1024,
                          num_moments: int = 64, seed: int = 31) -> ParticleWorkload:
    """The SPH configuration as its text states it, a variant the reference does not have: the particles of
    :func:`sph_cluster_workload` with a seeded smoothing length per particle, uniform in ``h_range``, and the Wendland
    C2 kernel (``Context.upload_particles_h``).  Step 2^-9, below half the smallest smoothing length; ``h`` holds the
    per-particle array."""
    wl = sph_cluster_workload(n=n, h=1.0 / 256, width=width, height=height, num_moments=num_moments, seed=seed)
    rng = np.random.default_rng(seed + 11)
    wl.h = rng.uniform(h_range[0], h_range[1], size=n).astype(np.float32)
    wl.gen.step_size = 2.0 ** -9
    wl.rec.step_size = 2.0 ** -9
    wl.name = f"sph{n}_wendland_h{h_range[0]:g}-{h_range[1]:g}_{width}x{height}_m{num_moments}_persp"
    return wl


def sph_cluster_workload(n: int = 16_000_000, h: float = 1.0 / 256, width: int = 1024, height: int = 1024,
                         num_moments: int = 64, seed: int = 31) -> ParticleWorkload:
    """The SPH configuration: n particles (70 % uniform, 30 % in 200 seeded Gaussian clusters, LogNormal(0, 0.5)
    values) with one smoothing length h (the reference's particle grid: 1 / h cells per unit, 256^3 at h = 1/256),
    perspective view of the unit cube, 64 moments, step h / 2; data_min / data_max at the 1st / 99th percentiles of
    a seeded sample of 100000 values."""
    wl = sph_workload(n=64, h=h, width=width, height=height, num_moments=num_moments, seed=seed)
    x, y, z, v = sph_particles(n, seed)
    rng = np.random.default_rng(seed + 7)
    smp = v[rng.integers(0, n, size=min(n, 100000))]
    wl.gen.data_min, wl.gen.data_max = float(np.percentile(smp, 1)), float(np.percentile(smp, 99))
    wl.x, wl.y, wl.z, wl.v = x, y, z, v
    wl.domain_min = (float(x.min()), float(y.min()), float(z.min()))
    wl.domain_max = (float(x.max()), float(y.max()), float(z.max()))
    wl.name = f"sph{n}_h1/{round(1 / h)}_{width}x{height}_m{num_moments}_persp"
    return wl
