"""torch.autograd.Function over bh_render_adjoint, for verification only.

``render_loss(theta, ...)`` returns the image loss mean((C - target)^2) of
the differentiable render at ``theta`` as a torch scalar whose backward is the
library's adjoint: ``torch.autograd.gradcheck``-style comparisons and
optimiser loops can drive the C ABI without any torch arithmetic on the hot
path (the forward and the gradient both come from one bh_render_adjoint
call). The library computes in its own precision; theta is float64.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import capi
from .render import Renderer


class _AdjointLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, renderer, c_scene, target, options, image):
        th = theta.detach().to("cpu", torch.float64).contiguous().numpy().reshape(1, capi.GRAD_COUNT)
        frames = (capi.AdjointFrame * 1)()
        frames[0].target = target.data_ptr()
        frames[0].image = image.data_ptr() if image is not None else None
        scenes = (capi.Scene * 1)(c_scene)
        res = renderer.render_adjoint(scenes, frames, th, options)[0]
        ctx.save_for_backward(torch.tensor(list(res.grad), dtype=torch.float64))
        return torch.tensor(res.loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None, None, None, None, None


def render_loss(theta: torch.Tensor, renderer: Renderer, c_scene: capi.Scene, target: torch.Tensor,
                options: capi.AdjointOptions | None = None, image: torch.Tensor | None = None) -> torch.Tensor:
    """Loss of the render at theta (10 float64) against target (H, W, 3)
    float32 CUDA tensor; differentiable in theta."""
    if not (target.is_cuda and target.dtype == torch.float32 and target.is_contiguous()):
        raise ValueError("target must be a contiguous float32 CUDA tensor of shape (H, W, 3)")
    h, w = c_scene.camera.height, c_scene.camera.width
    if tuple(target.shape) != (h, w, 3):
        raise ValueError(f"target shape {tuple(target.shape)} != {(h, w, 3)}")
    torch.cuda.current_stream().synchronize()
    return _AdjointLoss.apply(theta, renderer, c_scene, target, options, image)
