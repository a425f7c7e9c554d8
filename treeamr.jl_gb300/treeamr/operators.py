"""Interpolation operators and their exact rational weights.

Restates ``src/operators.jl``:

* ``Operators`` -- ``src/operators.jl:314-415`` (families ``PointValue`` and
  ``Conservative``; both orders required, no default).
* ``check_operators`` -- ``src/operators.jl:531-592``.
* ``lagrange_weights`` / ``unit_lagrange_weights`` -- ``src/operators.jl:627-682``:
  exact rationals, rounded once into the stencil's element type.
* ``conservative_prolong_weights`` -- ``src/schedule.jl:1097-1120``.
* ``boundedmode`` -- ``src/operators.jl:417-441``: how a group's kernel
  bounds what it computes (not at all, the bounded conservative
  prolongation, or the point-value interpolant clamped into its bracket).
"""
from __future__ import annotations

from fractions import Fraction
from functools import lru_cache
from typing import List, Sequence, Tuple

import numpy as np

from .forest import round_rational_f32

PointValue, Conservative = "PointValue", "Conservative"

UNBOUNDED, BOUNDED_CONSERVATIVE, BOUNDED_POINTVALUE = 0, 1, 2


class Operators:
    """The prolongation and restriction a schedule is built with.

    Both orders are required: ``Operators()`` raises, as the reference's
    constructor does (``src/operators.jl:338-344``)."""

    def __init__(self, *, prolongation=None, restriction=None, family=PointValue,
                 bounded=False, vertex_prolongation=None):
        for name, p in (("prolongation", prolongation), ("restriction", restriction)):
            if p is None:
                raise ValueError(
                    f"Operators has no default order: pass {name} explicitly. The order "
                    "must exceed the application's differencing order by two.")
        if family == PointValue:
            for name, p in (("prolongation", prolongation), ("restriction", restriction)):
                if p < 2:
                    raise ValueError(f"{name} order must be at least 2, got {p}")
                if p % 2:
                    raise ValueError(f"{name} order must be even for the point-value family, got {p}")
        elif family == Conservative:
            if prolongation < 1:
                raise ValueError(f"conservative prolongation order must be at least 1, got {prolongation}")
            if prolongation % 2 == 0:
                raise ValueError(f"conservative prolongation order must be odd, got {prolongation}")
            if restriction != 2:
                raise ValueError("conservative restriction is the exact volume average, so "
                                 f"restriction must be 2, got {restriction}")
        else:
            raise ValueError(f"unknown operator family {family!r}")
        if bounded and family == Conservative and prolongation not in (1, 3):
            raise ValueError("bounded = true with the conservative family needs prolongation = "
                             "3 or 1: the bounded prolongation is a limited order-3 "
                             f"reconstruction, and order 1 copies the parent; got {prolongation}")
        if bounded and vertex_prolongation is not None:
            raise ValueError("bounded = true together with vertex_prolongation is not "
                             "implemented: the bounded conservative prolongation is built for an "
                             "order-3 cell stencil in every dimension")
        if vertex_prolongation is not None:
            if family != Conservative:
                raise ValueError("vertex_prolongation is for the conservative family only")
            if vertex_prolongation < 2 or vertex_prolongation % 2:
                raise ValueError("vertex_prolongation must be even and at least 2")
        self.family = family
        self.prolongation = int(prolongation)
        self.restriction = int(restriction)
        self.bounded = bool(bounded)
        self.vertex_prolongation = 0 if vertex_prolongation is None else int(vertex_prolongation)

    def __repr__(self):
        vp = "" if not self.vertex_prolongation else f", vertex_prolongation={self.vertex_prolongation}"
        b = ", bounded=true" if self.bounded else ""
        return (f"Operators(prolongation={self.prolongation}, restriction={self.restriction}, "
                f"family={self.family}{b}{vp})")

    def vertex_order(self) -> int:
        return self.vertex_prolongation if self.family == Conservative else self.prolongation

    def ghost_layers_read(self) -> int:
        """``src/operators.jl:463-466``."""
        return (self.prolongation - 1) // 2 if self.family == Conservative else self.prolongation // 2


def check_operators(N: int, G: Sequence[int], c: Sequence[int], ops: Operators):
    """Per-dimension compatibility of ``N``, ``G`` and the orders
    (``src/operators.jl:531-592``)."""
    pr = ops.restriction
    needed = ops.ghost_layers_read()
    for d, (g, cd) in enumerate(zip(G, c)):
        if cd == 1:
            pv = ops.vertex_order()
            if pv == 0:
                raise ValueError("a Conservative field set with a vertex-like dimension "
                                 "needs vertex_prolongation")
            if g < pv // 2 - 1:
                raise ValueError(f"prolongation of order {pv} into a vertex-like dimension needs "
                                 f"G >= {pv // 2 - 1}, but G={tuple(G)} (dimension {d + 1})")
        else:
            if g < needed:
                raise ValueError(f"{ops.family} prolongation of order {ops.prolongation} needs "
                                 f"G >= {needed} ghost layers, but G={tuple(G)} (dimension {d + 1})")
            if N < 2 * g + pr // 2 - 1:
                raise ValueError(f"restriction of order {pr} into G={g} ghost layers needs "
                                 f"N >= {2 * g + pr // 2 - 1}, but N={N}")
            if N < pr:
                raise ValueError(f"restriction of order {pr} needs N >= {pr}, but N={N}")


def lagrange_weights(nodes: Sequence[Fraction], x: Fraction) -> List[Fraction]:
    """Exact weights ``w`` with ``sum(w[i] u(nodes[i])) == u(x)`` for every
    polynomial of degree below ``len(nodes)`` (``src/operators.jl:627-643``)."""
    nodes = [Fraction(n) for n in nodes]
    x = Fraction(x)
    n = len(nodes)
    out = []
    for i in range(n):
        num, den = Fraction(1), Fraction(1)
        for j in range(n):
            if j == i:
                continue
            num *= (x - nodes[j])
            den *= (nodes[i] - nodes[j])
        out.append(num / den)
    return out


@lru_cache(maxsize=None)
def unit_lagrange_weights(p: int, xi: Fraction) -> Tuple[Fraction, ...]:
    """Weights for the nodes ``0:p-1`` at ``xi``, memoised
    (``src/operators.jl:675-682``)."""
    return tuple(lagrange_weights([Fraction(j) for j in range(p)], Fraction(xi)))


def interpolation_weights(lo: int, p: int, x: Fraction, what: str) -> Tuple[Fraction, ...]:
    """Weights of the window ``lo:lo+p-1`` at ``x``; refuses extrapolation
    (``src/schedule.jl:908-916``)."""
    x = Fraction(x)
    if not (lo <= x <= lo + p - 1):
        raise ValueError(f"{what} would extrapolate: target {x} lies outside the source window "
                         f"[{lo}, {lo + p - 1}]. The block geometry cannot support this order.")
    return unit_lagrange_weights(p, x - lo)


@lru_cache(maxsize=None)
def conservative_prolong_weights(p: int) -> Tuple[Tuple[Fraction, ...], Tuple[Fraction, ...]]:
    """The low and high subcell weights of the order-``p`` conservative
    reconstruction (``src/schedule.jl:1097-1120``): interpolate the primitive
    through the ``p+1`` cell boundaries and difference it over each half."""
    r = (p - 1) // 2
    bounds = [Fraction(-r) - Fraction(1, 2) + i for i in range(p + 1)]
    # W(x) = sum_i L_i(x) W_i with W_i = sum_{t<i} ubar_t, so ubar_t carries
    # sum_{i>t} L_i(x); evaluated at the coarse cell's own centre.
    L = lagrange_weights(bounds, Fraction(0))
    tail = [sum(L[t + 1:p + 1], Fraction(0)) for t in range(p)]
    low = tuple(2 * (tail[t] - (1 if t < r else 0)) for t in range(p))
    high = tuple(2 * ((1 if t < r + 1 else 0) - tail[t]) for t in range(p))
    return low, high


def round_weights(ws: Sequence[Fraction], dtype) -> np.ndarray:
    """Each exact weight rounded once into ``dtype`` (``src/operators.jl:597-607``)."""
    dtype = np.dtype(dtype)
    if dtype == np.float64:
        return np.array([float(w) for w in ws], dtype=np.float64)
    if dtype == np.float32:
        return np.array([round_rational_f32(w.numerator, w.denominator) for w in ws],
                        dtype=np.float32)
    raise TypeError(f"unsupported element type {dtype}")


def boundedmode(ops: "Operators", kind: str, mirror, c) -> int:
    """The bound a group of ``kind`` takes (``src/operators.jl:431-441``):
    only an operator that can make a new extremum takes one.  Conservative
    order 1 copies the parent and a point-value width of 2 is linear
    interpolation, bounded already; injection (a vertex-like restriction) is
    a copy; a point-value restriction interpolates along every cell-like
    dimension."""
    if not ops.bounded:
        return UNBOUNDED
    if ops.family == Conservative:
        return BOUNDED_CONSERVATIVE if kind == "prolong" and ops.prolongation == 3 else UNBOUNDED
    if kind == "prolong" and ops.prolongation > 2:
        return BOUNDED_POINTVALUE
    if kind == "restrict" and ops.restriction > 2 and any(x == 0 for x in c):
        return BOUNDED_POINTVALUE
    return UNBOUNDED

