"""The cell-wise boundary hook on the device: ``CellBoundary``
(``src/ghosts.jl:1166-1318``) with a built-in function of position.

The reference's ``CellBoundary(g)`` takes a per-cell function ``g(x, v, δ)``
the package launches as a kernel.  A function written above a C ABI cannot
be called from a compiled kernel, so the forms of ``g`` that Dirichlet data
and manufactured solutions use are built in: ``Constant(values)`` and
``Polynomial(terms)``, evaluated on the device in a fixed order of single
roundings.  Either runs between phase 1 and the prolongations, as every
hook does, over every ghost region facing out through an outer face, with
the position of a ghost formed exactly as ``nodeposition`` forms it.
``Relative(f)`` with such an ``f`` gives the relative form, run in parts
after the stages that fill what it reads.  ``wall = "prescribed"``
(``src/ghosts.jl:1378-1412, 1639-1652``) makes the hook write the wall
planes of vertex-like dimensions too, at their primaries, before stage P
and stage 0 (stage W), so that every copy of a prescribed point is one
number.
"""
from __future__ import annotations

import ctypes as C
from typing import Mapping, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .storage import FieldSet

MAX_TERMS = 20


class Constant:
    """``g(x, v) = values[v]``."""

    def __init__(self, values: Sequence[float]):
        self.values = [float(v) for v in values]


class Polynomial:
    """``g(x, v) = sum_q coef_q[v] * x1^a_q * x2^b_q * x3^c_q``, the terms in
    the given order: ``{(a, b, c): [coef for each variable], ...}``, at most
    20 terms.  Each term is ``((coef * x1^a) * x2^b) * x3^c`` with powers by
    repeated multiplication, summed in order from +0."""

    def __init__(self, terms: Mapping[Tuple[int, ...], Sequence[float]]):
        self.terms = [(tuple(int(e) for e in exps), [float(c) for c in coefs])
                      for exps, coefs in terms.items()]
        if len(self.terms) > MAX_TERMS:
            raise ValueError(f"a Polynomial holds at most {MAX_TERMS} terms")


class Relative:
    """The relative form (``src/ghosts.jl:1431-1475``): every ghost ``x_g``
    beyond an outer face becomes ``f(x_g) + (u(x_r) - f(x_r))``, ``x_r`` the
    nearest evolved point, evaluated in that order; ``f`` a ``Constant`` or
    a ``Polynomial``."""

    def __init__(self, f):
        if not isinstance(f, (Constant, Polynomial)):
            raise TypeError("Relative takes a Constant or a Polynomial")
        self.f = f


class CellBoundary:
    """The device hook: ``CellBoundary(Constant(...))``,
    ``CellBoundary(Polynomial(...))`` or ``CellBoundary(Relative(...))``,
    passed as ``fill_ghosts(..., boundary=hook)``."""

    def __init__(self, g, wall: str = "evolved"):
        if not isinstance(g, (Constant, Polynomial, Relative)):
            raise TypeError("CellBoundary takes a Constant, a Polynomial or a Relative of one: "
                            "a function written above the C ABI cannot run in the device "
                            "kernel")
        if wall not in ("evolved", "prescribed"):
            raise ValueError("wall must be 'evolved' (the wall plane of a vertex-like "
                             "dimension is an own point of the state, evolved by the "
                             "application, and the hook fills the ghosts beyond it) or "
                             "'prescribed' (the hook gives the wall plane its value too, a "
                             f"Dirichlet condition), got {wall!r}")
        self.relative = isinstance(g, Relative)
        self.g = g.f if self.relative else g
        self.prescribes_wall = wall == "prescribed"

    # -- the device side ---------------------------------------------------------
    def _fn(self, fs: FieldSet):
        fn = _native.tam_boundary_fn()
        fn.relative = 1 if self.relative else 0
        nv = fs.nvars
        if isinstance(self.g, Constant):
            if len(self.g.values) != nv:
                raise ValueError(f"Constant has {len(self.g.values)} values for {nv} variables")
            fn.kind = _native.TAM_BC_CONSTANT
            fn.nterms = 0
            coef = np.array(self.g.values, dtype=fs.T)
        else:
            fn.kind = _native.TAM_BC_POLYNOMIAL
            fn.nterms = len(self.g.terms)
            coef = np.zeros((nv, max(1, fn.nterms)), dtype=fs.T)
            for q, (exps, coefs) in enumerate(self.g.terms):
                if len(coefs) != nv:
                    raise ValueError(f"term {exps} has {len(coefs)} coefficients for {nv} "
                                     "variables")
                if len(exps) > fs.D and any(exps[fs.D:]):
                    raise ValueError(f"term {exps} has a power beyond dimension {fs.D}")
                for d in range(3):
                    fn.exps[q][d] = exps[d] if d < len(exps) else 0
                coef[:, q] = coefs
        return fn, coef

    def slots(self, schedule):
        """The stage tags after which this hook runs: phase 1 alone, or for
        the relative form every slot its regions need."""
        if not self.relative:
            return [1]
        return sorted({r.slot for r in schedule.boundaries})

    def apply_walls(self, fs: FieldSet, schedule, stream=None):
        """Stage W (``wall_boundary!``, ``src/ghosts.jl:1639-1652``): a hook
        that prescribes the wall writes the wall planes' primaries."""
        if not self.prescribes_wall or not schedule.walls:
            return
        table = region_table(fs, schedule, "walls")
        self._launch(fs, table[0], 0, len(schedule.walls), stream)

    def apply(self, fs: FieldSet, schedule, stream=None, slot: Optional[int] = None):
        """Fill the regions (for the relative form, those of ``slot``)."""
        table = region_table(fs, schedule)
        if table is None:
            return
        regions, spans = table
        if self.relative:
            first, count = spans.get(slot, (0, 0))
        else:
            first, count = 0, len(schedule.boundaries)
        self._launch(fs, regions, first, count, stream)

    def _launch(self, fs: FieldSet, regions, first: int, count: int, stream):
        if count == 0:
            return
        key = (np.dtype(fs.T).name, fs.nvars, fs.work.device.index)
        cache = self.__dict__.setdefault("_device", {})
        if key not in cache:
            fn, coef = self._fn(fs)
            # kept with the hook, so the launch may read it after this returns
            cache[key] = (fn, torch.from_numpy(np.ascontiguousarray(coef).ravel())
                          .to(fs.work.device))
        fn, dcoef = cache[key]
        s = stream if stream is not None else torch.cuda.current_stream(fs.work.device)
        stored = (C.c_int32 * 3)(*[fs.stored[d] if d < fs.D else 1 for d in range(3)])
        dtype = _native.TAM_F64 if fs.T == np.float64 else _native.TAM_F32
        rc = _native.lib().tam_boundary_apply(
            dtype, C.c_void_p(regions.data_ptr() + first * C.sizeof(_native.tam_boundary_region)),
            count, fn,
            C.c_void_p(dcoef.data_ptr()), C.c_void_p(fs.work.data_ptr()), fs.nvars, stored,
            C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _native.TamError(f"tam_boundary_apply failed ({rc})")


def ordered_regions(schedule, which: str = "boundaries"):
    """The hook regions (or stage W's, ``which="walls"``) ordered by slot
    (stably), and per slot its ``(first, count)`` in that order."""
    regions = sorted(getattr(schedule, which), key=lambda r: r.slot)
    spans = {}
    for i, r in enumerate(regions):
        a, n = spans.get(r.slot, (i, 0))
        spans[r.slot] = (a, n + 1)
    return regions, spans


def region_rows(fs: FieldSet, schedule, which: str = "boundaries"):
    """One ``tam_boundary_region`` per hook region, ordered by slot, with its
    block's nodeposition data (``src/storage.jl:1008-1017``)."""
    f = fs.forest
    D = fs.D
    ordered, _ = ordered_regions(schedule, which)
    rows = (_native.tam_boundary_region * max(1, len(ordered)))()
    for i, r in enumerate(ordered):
        k = f.leaves[r.block]
        lo, B = f.block_low(k), f.block_base(k)
        h = f.spacing(k.level, fs.T)
        row = rows[i]
        row.block = r.block
        for d in range(3):
            if d < D:
                a, z = r.region[d]
                row.first[d], row.n[d] = a, z - a + 1
                row.ghosts[d], row.stagger[d] = fs.G[d], fs.c[d]
                row.clamps[d] = r.clamps[d] if r.clamps else 0
                row.base[d], row.lo[d] = B[d], float(np.dtype(fs.T).type(lo[d]))
            else:
                row.first[d], row.n[d], row.ghosts[d], row.stagger[d] = 1, 1, 0, 0
                row.clamps[d] = 0
                row.base[d], row.lo[d] = 0, 0.0
        row.h = float(h)
    return rows


def region_table(fs: FieldSet, schedule, which: str = "boundaries"):
    """The regions as a device array ordered by slot, and the slots' spans,
    made once per schedule, element type and device."""
    regions = getattr(schedule, which)
    if not regions:
        return None
    cache = schedule.__dict__.setdefault("_boundary_regions", {})
    key = (which, np.dtype(fs.T).name, fs.work.device.index)
    if key not in cache:
        rows = region_rows(fs, schedule, which)
        raw = np.frombuffer(bytes(rows), dtype=np.uint8)[:C.sizeof(rows[0]) * len(regions)]
        cache[key] = (torch.from_numpy(raw.copy()).to(fs.work.device),
                      ordered_regions(schedule, which)[1])
    return cache[key]
