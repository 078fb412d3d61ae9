"""torch.autograd.Function over cvtpm_cost_adjoint: the aggregated ASW cost
(patch_eval_color_grad_weighted, cvt/cl/kernel/pmhstereo.cl:170-228) of
per-pixel planes as a differentiable function of the planes and both images.

A thin wrapper for tests and for callers that optimise planes or images by
gradient descent; the forward and the backward are the library's CUDA
kernels (the backward recomputes the window weights).
"""
from __future__ import annotations

import torch

from .stereo import PMHuberStereo


class AswCost(torch.autograd.Function):
    """cost = AswCost.apply(ctx_obj, img1, img2, planes, lr)

    img1, img2: (H, W, 4) float32 RGBA on the GPU; planes: (H, W, 4)
    (a, b, c, unused), d = a*x + b*y + c; returns the (H, W) cost.
    Gradients flow to planes (a, b, c; the 4th channel gets 0) and to the
    RGB channels of both images (alpha gets 0)."""

    @staticmethod
    def forward(ctx, stereo: PMHuberStereo, img1, img2, planes, lr: int = 1):
        cost, _, _, _ = stereo.cost_adjoint(img1.detach(), img2.detach(), planes.detach(), lr)
        ctx.save_for_backward(img1, img2, planes)
        ctx.stereo, ctx.lr = stereo, lr
        return cost

    @staticmethod
    def backward(ctx, grad_cost):
        img1, img2, planes = ctx.saved_tensors
        want_img = ctx.needs_input_grad[1] or ctx.needs_input_grad[2]
        _, dpl, d1, d2 = ctx.stereo.cost_adjoint(img1.detach(), img2.detach(), planes.detach(), ctx.lr,
                                                 dcost=grad_cost, want_planes=ctx.needs_input_grad[3],
                                                 want_images=want_img)
        return (None,
                d1 if ctx.needs_input_grad[1] else None,
                d2 if ctx.needs_input_grad[2] else None,
                dpl, None)


def asw_cost(stereo: PMHuberStereo, img1, img2, planes, lr: int = 1):
    return AswCost.apply(stereo, img1, img2, planes, lr)
