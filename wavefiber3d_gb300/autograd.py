"""torch.autograd bindings of the PO engine (the fitting side's entry point).

``far_field_intensity(solver, illum, samples)`` returns the intensity
patterns of a (7, n) tensor of surface samples (x, y, z, nx, ny, nz, area);
its backward pass calls the library's hand-written adjoint (po_grad), which
recomputes the forward solve and propagates dL/dI back to every sample.
``height_field_samples(hf_xy, ...)`` maps a fiber height field to samples
(util/geometry.h:76-179) with the adjoint of that map in its backward pass,
so a loss on the patterns differentiates down to the vertex coordinates.
Both run on the CUDA library only; there is no PyTorch re-implementation to
fall back on.
"""
from __future__ import annotations

import torch

from . import api


class _FarFieldIntensity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, samples, solver, illum):
        s = samples.detach().to(device="cuda", dtype=torch.float32).contiguous()
        out = solver.solve(tuple(s[k] for k in range(7)), illum)
        ctx.solver, ctx.illum = solver, illum
        ctx.save_for_backward(s)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (s,) = ctx.saved_tensors
        g = ctx.solver.grad(s, ctx.illum, grad_out)
        return g, None, None


def far_field_intensity(solver: "api.Solver", illum: "api.Illumination", samples: torch.Tensor) -> torch.Tensor:
    """Intensity [L][I][P][n_theta][n_phi] of the (7, n) samples, differentiable in the samples."""
    return _FarFieldIntensity.apply(samples, solver, illum)


class _HeightFieldSamples(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xy, period, unitz, ring_begin, ring_end):
        x = xy.detach().to(device="cuda", dtype=torch.float32).contiguous()
        out = api.height_field_points_tensor(x, period, unitz, ring_begin, ring_end)
        ctx.meta = (period, unitz, ring_begin, ring_end)
        ctx.save_for_backward(x)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (x,) = ctx.saved_tensors
        period, unitz, b, e = ctx.meta
        g = api.height_field_adjoint(x, period, unitz, b, e, grad_out)
        return g, None, None, None, None


def height_field_samples(xy: torch.Tensor, period: float, unitz: float, ring_begin: int = 0,
                         ring_end: int | None = None) -> torch.Tensor:
    """(7, n) samples of the height field xy [2][numel][numelvert], differentiable in xy."""
    ring_end = xy.shape[1] - 1 if ring_end is None else int(ring_end)
    return _HeightFieldSamples.apply(xy, float(period), float(unitz), int(ring_begin), ring_end)
