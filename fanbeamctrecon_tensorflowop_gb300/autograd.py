"""Differentiable operators: torch.autograd.Functions over the library's
hand-written adjoints.

Every operator is linear, so backward applies the exact transpose kernel to
the incoming gradient and nothing is saved for backward except the plan.
(The reference registers no gradient at all: utils.py imports ``ops`` and
never uses it, utils.py:5.)
"""
from __future__ import annotations

import torch

from .ops import ConePlan, FanPlan


class _ForwardProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, img: torch.Tensor, plan: FanPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = img.dim() == 2
        out = plan.fp(img)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        gi = ctx.plan.fp_adjoint(g.contiguous())
        return (gi[0] if ctx.squeeze else gi), None


class _ForwardProjectionAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = sino.dim() == 2
        out = plan.fp_adjoint(sino)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        gs = ctx.plan.fp(g.contiguous())
        return (gs[0] if ctx.squeeze else gs), None


class _BackProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = sino.dim() == 2
        out = plan.bp(sino)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        gs = ctx.plan.bp_adjoint(g.contiguous())
        return (gs[0] if ctx.squeeze else gs), None


class _FilteredBackProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = sino.dim() == 2
        out = plan.fbp(sino)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        gs = ctx.plan.fbp_adjoint(g.contiguous())
        return (gs[0] if ctx.squeeze else gs), None


class _FDKBackProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = sino.dim() == 2
        out = plan.fdk_bp(sino)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        # With one detector row the FDK op equals the weighted FBP, so its
        # transpose is the FBP transpose.
        gs = ctx.plan.fbp_adjoint(g.contiguous())
        return (gs[0] if ctx.squeeze else gs), None


def forward_project(img: torch.Tensor, plan: FanPlan) -> torch.Tensor:
    """Differentiable ray-driven FP; backward is the exact transpose."""
    return _ForwardProjection.apply(img, plan)


def forward_project_adjoint(sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
    """Differentiable FP transpose; backward is FP."""
    return _ForwardProjectionAdjoint.apply(sino, plan)


def back_project(sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
    """Differentiable unweighted BP; backward is its transpose."""
    return _BackProjection.apply(sino, plan)


def filtered_back_project(sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
    """Differentiable FBP; backward is its transpose (BP^T, then the filter)."""
    return _FilteredBackProjection.apply(sino, plan)


def fdk_back_project(sino: torch.Tensor, plan: FanPlan) -> torch.Tensor:
    """Differentiable reference FDK op; backward is its transpose."""
    return _FDKBackProjection.apply(sino, plan)


class _FDKCone(torch.autograd.Function):
    @staticmethod
    def forward(ctx, proj: torch.Tensor, plan: ConePlan) -> torch.Tensor:
        ctx.plan = plan
        ctx.squeeze = proj.dim() == 3
        out = plan.fdk(proj)
        return out[0] if ctx.squeeze else out

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        gp = ctx.plan.fdk_adjoint(g.contiguous())
        return (gp[0] if ctx.squeeze else gp), None


def fdk_cone(proj: torch.Tensor, plan: ConePlan) -> torch.Tensor:
    """Differentiable cone-beam FDK; backward is its exact transpose
    (CB_EA transpose, then the filter)."""
    return _FDKCone.apply(proj, plan)
