"""torch.autograd binding of the differentiation form: render(volume, tf_table) -> RGBA with a hand-written
adjoint (the CUDA kernels behind mraygb_diff_forward / mraygb_diff_backward).

The differentiated method is the moment-image path (generate -> Lagrange multipliers -> MESE re-march) without
compaction, with the unquantized per-pixel density bounds, the exact arctangent and the transfer-function row
sampled in the front density as a cubic B-spline (``RenderSpec.tf_sampling = DIFF_TF_BSPLINE``, the default) or
linearly as the reference's GPU texture samples it (``DIFF_TF_LINEAR``).  Gradients flow to the transfer-function
row (256 x RGBA, the preintegrated table) and to
the voxel densities; ``preintegrate_table`` builds that row from a 1D transfer function with torch operations, so
gradients reach the 1D extinction (alpha) and emission (rgb) tables through ordinary autograd.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import torch

from .raymarcher import DIFF_TF_BSPLINE, Context, default_context
from .types import Camera, GenerationParameters, ReconstructionParameters


def preintegrate_table(tf1d: torch.Tensor, step_size: float) -> torch.Tensor:
    """TransferFunction preintegration (transfer_function.cpp:46-97) as torch operations: entry x =
    (rgb_x a_x s, a_x s), s = step_size."""
    a = tf1d[:, 3:4] * step_size
    return torch.cat([tf1d[:, :3] * a, a], dim=1)


@dataclasses.dataclass
class RenderSpec:
    """Everything of one render except the two differentiated inputs."""

    camera: Camera
    gen: GenerationParameters
    rec: ReconstructionParameters
    width: int
    height: int
    num_moments: int
    domain_min: tuple
    domain_max: tuple
    context: Optional[Context] = None
    tf_sampling: int = DIFF_TF_BSPLINE

    def ctx(self) -> Context:
        return self.context or default_context(torch.cuda.current_device())


class MomentRender(torch.autograd.Function):
    @staticmethod
    def forward(fctx, volume: torch.Tensor, tf_table: torch.Tensor, spec: RenderSpec):
        ctx = spec.ctx()
        ctx.set_stream(torch.cuda.current_stream())
        vol = volume.detach().contiguous().float()
        tf = tf_table.detach().contiguous().float()
        ctx.upload_grid(vol, spec.domain_min, spec.domain_max)
        W, H, m = spec.width, spec.height, spec.num_moments
        dev = volume.device
        moments = torch.empty(W * H * m, dtype=torch.float32, device=dev)
        bounds4 = torch.empty(W * H * 4, dtype=torch.float32, device=dev)
        pmoments = torch.empty(W * H * m, dtype=torch.float32, device=dev)
        rgba = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
        ctx.diff_tf_sampling = spec.tf_sampling
        ctx.diff_forward(spec.camera, spec.gen, spec.rec, W, H, m, tf, moments, bounds4, pmoments, rgba)
        fctx.save_for_backward(vol, tf, moments, bounds4, pmoments, rgba)
        fctx.spec = spec
        fctx.need_volume = volume.requires_grad
        return rgba

    @staticmethod
    def backward(fctx, grad_rgba: torch.Tensor):
        vol, tf, moments, bounds4, pmoments, rgba = fctx.saved_tensors
        spec: RenderSpec = fctx.spec
        ctx = spec.ctx()
        ctx.set_stream(torch.cuda.current_stream())
        ctx.upload_grid(vol, spec.domain_min, spec.domain_max)  # the context may hold another volume by now
        W, H, m = spec.width, spec.height, spec.num_moments
        g = grad_rgba.contiguous().float()
        grad_tf = torch.zeros_like(tf)
        grad_vol = torch.zeros_like(vol) if fctx.need_volume else None
        ctx.diff_tf_sampling = spec.tf_sampling
        ctx.diff_backward(spec.camera, spec.gen, spec.rec, W, H, m, tf, moments, bounds4, pmoments, rgba, g, grad_tf,
                          grad_vol)
        return grad_vol, grad_tf, None


def render(volume: torch.Tensor, tf_table: torch.Tensor, spec: RenderSpec) -> torch.Tensor:
    """The differentiation form's image (H x W x RGBA float32) of a [z, y, x] CUDA volume and a 256 x 4
    transfer-function row, differentiable in both."""
    return MomentRender.apply(volume, tf_table, spec)
