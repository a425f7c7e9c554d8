"""The adjoint of the ghost fill and its autograd binding.

The reference has no adjoint.  The fill is a linear map ``A`` of the field
data; ``fill_ghosts_adjoint`` applies ``A^T`` with the library's gather-form
kernel (``tam_fill_adjoint``), and ``GhostFill`` wraps the pair as a
``torch.autograd.Function`` -- the counterpart of the ChainRulesCore rrule
a Julia caller would define for ``fill_ghosts!`` (``src/ghosts.jl:1783``):
forward returns the filled copy, backward pulls the cotangent back through
``A^T``.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _native
from .ghosts import check_fill, device_schedule, run_axis, turns_variables
from .schedule import GhostSchedule, SELFIMAGE_TAG, UNIFY_TAG
from .storage import FieldSet


def fill_ghosts_adjoint(fs: FieldSet, schedule: GhostSchedule, y: Optional[torch.Tensor] = None,
                        *, scratch: Optional[torch.Tensor] = None,
                        stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """``y <- A^T y`` in place, ``y`` shaped like ``fs.work`` (default: ``fs.work``
    itself).  Stages run in reverse; every ghost's adjoint is pushed onto the
    points its value was computed from, then zeroed.  Over a seam whose axis
    projection turns variables, the projection's transpose runs between
    stage 0's transpose and stage P's."""
    check_fill(fs, schedule)
    y = fs.work if y is None else y
    if y.shape != fs.work.shape or y.dtype != fs.work.dtype or y.device != fs.work.device:
        raise ValueError("the adjoint vector must have the field set's shape, type and device")
    if not y.is_contiguous():
        raise ValueError("the adjoint vector must be contiguous")
    ds = device_schedule(schedule, y.device.index or 0)
    rotvars = getattr(fs, "rotvars", None)
    if schedule.axis and turns_variables(fs):
        # the fill is (stages >= 0) P (stages <= P), P the axis projection
        # between them; its transpose runs the three parts' transposes in
        # reverse order
        ds.run_adjoint(y, fs.nvars, fs.factors, UNIFY_TAG, _native.TAM_STAGE_ALL_LAST, stream,
                       scratch, rotvars=rotvars)
        run_axis(fs, schedule, stream, work=y, transpose=True)
        ds.run_adjoint(y, fs.nvars, fs.factors, _native.TAM_STAGE_ALL_FIRST, SELFIMAGE_TAG,
                       stream, scratch, rotvars=rotvars)
        return y
    ds.run_adjoint(y, fs.nvars, fs.factors, _native.TAM_STAGE_ALL_FIRST,
                   _native.TAM_STAGE_ALL_LAST, stream, scratch, rotvars=rotvars)
    return y


class GhostFill(torch.autograd.Function):
    """``out = A(x)``: the filled copy of ``x`` (the field set's layout), with
    ``d out / d x`` applied by the adjoint kernel."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, fs: FieldSet, schedule: GhostSchedule):
        from .ghosts import fill_ghosts
        check_fill(fs, schedule)
        out = x.detach().clone().contiguous()
        saved = fs.work
        try:
            fs.work = out
            fill_ghosts(fs, schedule)
        finally:
            fs.work = saved
        ctx.fs, ctx.schedule = fs, schedule
        return out

    @staticmethod
    def backward(ctx, grad: torch.Tensor):
        g = grad.detach().clone().contiguous()
        fill_ghosts_adjoint(ctx.fs, ctx.schedule, g)
        return g, None, None


def ghost_fill(x: torch.Tensor, fs: FieldSet, schedule: GhostSchedule) -> torch.Tensor:
    """Differentiable ghost fill of ``x`` (shaped like ``fs.work``)."""
    return GhostFill.apply(x, fs, schedule)
