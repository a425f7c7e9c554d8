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


def fill_pair_adjoint(pair, schedules, ya: Optional[torch.Tensor] = None,
                      yb: Optional[torch.Tensor] = None, *,
                      stream: Optional[torch.cuda.Stream] = None):
    """``(y_a, y_b) <- A^T (y_a, y_b)`` in place for a RotationPair's fill
    (``fill_pair``, without hooks), ``y_a`` and ``y_b`` shaped like the
    members' arrays (default: the arrays themselves).  The forward fill runs,
    tag by tag, the first member's stage and then the second's, each member's
    odd turns reading its partner's array; the transpose runs the tags from
    the last, the second member's stage transpose and then the first's, each
    adding its odd turns' transposes onto the partner's cotangent
    (``tam_fill_adjoint_alt``)."""
    from .storage import RotationPair
    if not isinstance(pair, RotationPair):
        raise TypeError("fill_pair_adjoint takes a RotationPair")
    sa, sb = schedules
    a, b = pair.a, pair.b
    check_fill(a, sa, pair=True)
    check_fill(b, sb, pair=True)
    ya = a.work if ya is None else ya
    yb = b.work if yb is None else yb
    for fs, y in ((a, ya), (b, yb)):
        if y.shape != fs.work.shape or y.dtype != fs.work.dtype or y.device != fs.work.device:
            raise ValueError("each adjoint vector must have its member's shape, type and device")
        if not y.is_contiguous():
            raise ValueError("the adjoint vectors must be contiguous")
    if ya.data_ptr() == yb.data_ptr():
        raise ValueError("the members' adjoint vectors must be distinct arrays")
    members = [(a, sa, pair.afactors, pair.arotvars, ya, yb),
               (b, sb, pair.bfactors, pair.brotvars, yb, ya)]
    dss = [device_schedule(s, y.device.index or 0) for _, s, _, _, y, _ in members]
    tags = sorted(set(sa.stage_tags) | set(sb.stage_tags))
    for tag in reversed(tags):
        for i in (1, 0):
            fs, s, fac, rv, y, alt = members[i]
            if tag in s.stage_tags:
                dss[i].run_adjoint(y, fs.nvars, fac, tag, tag, stream, rotvars=rv, alt=alt)
    return ya, yb


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
