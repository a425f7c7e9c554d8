"""Rotating seams (a quarter turn, ``rotating = (d1, d2)``) and half-turn
seams (``halfturn = (d1, d2)``): the tree and the turned ghost fill.

Restated from the reference's ``test/rotate_tests.jl`` and
``test/halfturn_tests.jl`` with the unfolded-forest oracles of
``test/ghost_oracles.jl:770-1000, 1462-1560``: the quadrant (or half plane)
is checked against the full plane it is a part of, built from turned
``Fraction`` boxes, never from the seam's own key arithmetic.  The forest's
neighbours across the seam are the unfolded forest's turned back, every
orientation meeting every kind of neighbour; balance makes the seam
conforming; the ghosts of a quadrant filled through the turned transfers
equal the full plane's filled without a seam, for data covariant under the
turn; and on the GPU the turned fill is the oracle's bit for bit."""
import ctypes as C
import itertools
from fractions import Fraction

import numpy as np
import pytest

from treeamr.forest import (Forest, MortonKey, alldirections, childoffset, real_direction,
                            virtual_offset)

F = Fraction


# --- the unfolded-forest oracle ------------------------------------------------------

def rotate_box(box, r, d1, d2):
    """``R^r`` of the box about the axis at the origin of the ``(d1, d2)``
    plane, ``R(x1, x2) = (-x2, x1)`` (``test/ghost_oracles.jl:781-789``)."""
    lo, hi = list(box[0]), list(box[1])
    for _ in range(r % 4):
        nlo, nhi = list(lo), list(hi)
        nlo[d1], nlo[d2] = -hi[d2], lo[d1]
        nhi[d1], nhi[d2] = -lo[d2], hi[d1]
        lo, hi = nlo, nhi
    return tuple(lo), tuple(hi)


def box_orientation(box, d1, d2):
    lo, hi = box
    a, b = hi[d1] <= 0, hi[d2] <= 0
    return (2 if b else 1) if a else (3 if b else 0)


def leafbox(forest, k):
    rp = forest.root_position(k.root)
    s = F(1, 1 << k.level)
    lo = tuple(rp[d] + k.coords[d] * s for d in range(forest.D))
    return lo, tuple(x + s for x in lo)


def box_key(roots, box):
    lo, hi = box
    D = len(roots)
    size = hi[0] - lo[0]
    assert all(hi[d] - lo[d] == size for d in range(D)) and size.numerator == 1
    lvl = size.denominator.bit_length() - 1
    assert size.denominator == 1 << lvl
    pos = [int(np.floor(lo[d])) for d in range(D)]
    root, stride = 0, 1
    for d in range(D):
        root += pos[d] * stride
        stride *= roots[d]
    return MortonKey(root, lvl, tuple(int((lo[d] - pos[d]) * (1 << lvl)) for d in range(D)))


def unfolded_forest(quad):
    """``(full, image, back)`` of a rotating quadrant
    (``test/ghost_oracles.jl:827-846``)."""
    d1, d2 = quad.seam_plane()
    M = quad.roots[d1]
    D = quad.D
    roots = tuple(2 * M if d in (d1, d2) else quad.roots[d] for d in range(D))
    shift = tuple(M if d in (d1, d2) else 0 for d in range(D))

    def image(k, r):
        lo, hi = rotate_box(leafbox(quad, k), r, d1, d2)
        return box_key(roots, (tuple(x + s for x, s in zip(lo, shift)),
                               tuple(x + s for x, s in zip(hi, shift))))

    def back(kf, full):
        lo, hi = leafbox(full, kf)
        box = (tuple(x - s for x, s in zip(lo, shift)), tuple(x - s for x, s in zip(hi, shift)))
        r = box_orientation(box, d1, d2)
        return r, box_key(quad.roots, rotate_box(box, -r, d1, d2))

    refl = tuple((a == 1, b == 1) for a, b in quad.faces)
    leaves = [image(k, r) for k in quad.leaves for r in range(4)]
    full = Forest(roots, N=quad.N, periodic=quad.periodic, reflecting=refl, leaves=leaves)
    return full, image, (lambda kf: back(kf, full))


def halfturn_box(box, d1, d2, c):
    lo, hi = list(box[0]), list(box[1])
    nlo, nhi = list(lo), list(hi)
    nlo[d1], nhi[d1] = -hi[d1], -lo[d1]
    nlo[d2], nhi[d2] = 2 * c - hi[d2], 2 * c - lo[d2]
    return tuple(nlo), tuple(nhi)


def unfolded_halfturn_forest(half):
    """``test/ghost_oracles.jl:1484-1502``."""
    d1, d2 = half.seam_plane()
    M1, c = half.roots[d1], F(half.roots[d2], 2)
    D = half.D
    roots = tuple(2 * M1 if d == d1 else half.roots[d] for d in range(D))
    shift = tuple(M1 if d == d1 else 0 for d in range(D))

    def turn(box, r):
        return box if r == 0 else halfturn_box(box, d1, d2, c)

    def image(k, r):
        lo, hi = turn(leafbox(half, k), r)
        return box_key(roots, (tuple(x + s for x, s in zip(lo, shift)),
                               tuple(x + s for x, s in zip(hi, shift))))

    def back(kf, full):
        lo, hi = leafbox(full, kf)
        box = (tuple(x - s for x, s in zip(lo, shift)), tuple(x - s for x, s in zip(hi, shift)))
        r = 2 if box[1][d1] <= 0 else 0
        return r, box_key(half.roots, turn(box, r))

    refl = tuple((a == 1, b == 1) for a, b in half.faces)
    leaves = [image(k, r) for k in half.leaves for r in (0, 2)]
    full = Forest(roots, N=half.N, periodic=half.periodic, reflecting=refl, leaves=leaves)
    return full, image, (lambda kf: back(kf, full))


def neighbor_mismatches(quad, half=False):
    """``seam_neighbor_mismatches`` / ``halfturn_neighbor_mismatches``
    (``test/ghost_oracles.jl:860-900, 1508-1540``)."""
    d1, d2 = quad.seam_plane()
    full, image, back = (unfolded_halfturn_forest if half else unfolded_forest)(quad)
    bad = 0
    seen = {}
    for k in quad.leaves:
        for delta in alldirections(quad.D):
            r, keys = quad.turned_neighbors(k, delta)
            unfolded = full.oriented_neighbors(image(k, 0), delta)
            expected = [back(kf) for kf in unfolded]
            if not expected:
                lo, hi = leafbox(quad, k)
                s = hi[0] - lo[0]
                if half:
                    want = 2 if hi[d1] + s * delta[d1] <= 0 else 0
                else:
                    want = box_orientation((tuple(lo[d] + s * delta[d] for d in range(quad.D)),
                                            tuple(hi[d] + s * delta[d] for d in range(quad.D))),
                                           d1, d2)
                ok = not keys and r == want
            else:
                ok = all(e[0] == r for e in expected) and \
                    sorted(keys) == sorted(e[1] for e in expected) and \
                    all(kf.level <= k.level or
                        virtual_offset(childoffset(kq), r, d1, d2) == childoffset(kf)
                        for kf, (_, kq) in zip(unfolded, expected))
            bad += not ok
            kind = "none" if not keys else "same" if keys[0].level == k.level else \
                "coarser" if keys[0].level < k.level else "finer"
            seen[(r, kind)] = seen.get((r, kind), 0) + 1
    return bad, seen, full


def random_seam_forest(rng, D, *, plane, M, other="outer", nsteps, maxlvl, half=False,
                       M2=None):
    """``random_rotating_forest`` / ``random_halfturn_forest``
    (``test/ghost_oracles.jl:944-961, 1561-1590``)."""
    d1, d2 = plane
    roots = []
    for d in range(1, D + 1):
        if d == d1:
            roots.append(M)
        elif d == d2:
            roots.append(M2 if half else M)
        else:
            roots.append(int(rng.integers(1, 3)))
    inplane = lambda d: d + 1 in plane                           # noqa: E731
    periodic = tuple(not inplane(d) and other == "periodic" for d in range(D))
    reflecting = tuple((not inplane(d) and other == "reflecting", False) for d in range(D))
    kw = {"halfturn": plane} if half else {"rotating": plane}
    f = Forest(tuple(roots), N=4, periodic=periodic, reflecting=reflecting, **kw)
    for _ in range(nsteps):
        k = f.leaves[int(rng.integers(len(f.leaves)))]
        if k.level < maxlvl and rng.random() < 0.75:
            f.refine([k])
        elif k.level > 0:
            p = MortonKey(k.root, k.level - 1, tuple(c >> 1 for c in k.coords))
            kids = [MortonKey(p.root, p.level + 1, tuple(2 * c + o for c, o in zip(p.coords, off)))
                    for off in itertools.product((0, 1), repeat=D)]
            if all(f.isleaf(c) for c in kids):
                f.coarsen([p])
    return f


def seam_conforming(full, d1, d2):
    """Leaves sharing a face across an image of the seam are at one level
    (``test/ghost_oracles.jl:906-919``)."""
    M = full.roots[d1] // 2
    for kf in full.leaves:
        for d in (d1, d2):
            for s in (-1, 1):
                delta = tuple(s if e == d else 0 for e in range(full.D))
                hi = leafbox(full, kf)[1][d]
                for nf in full.oriented_neighbors(kf, delta):
                    across = (hi <= M) != (leafbox(full, nf)[1][d] <= M)
                    if across and nf.level != kf.level:
                        return False
    return True


# --- the tree ----------------------------------------------------------------------------

def test_a_seam_is_refused_where_it_cannot_be_glued():
    """``test/rotate_tests.jl:19-61``, ``test/halfturn_tests.jl:22-82``."""
    with pytest.raises(ValueError, match="at least two dimensions"):
        Forest((2,), N=4, rotating=(1, 2))
    with pytest.raises(ValueError, match="outside 1:2"):
        Forest((2, 2), N=4, rotating=(1, 3))
    with pytest.raises(ValueError, match="twice"):
        Forest((2, 2), N=4, rotating=(2, 2))
    with pytest.raises(ValueError, match="as many roots along dimension 1 as along 2"):
        Forest((2, 1), N=4, rotating=(1, 2))
    with pytest.raises(ValueError, match="dimension 2 is periodic"):
        Forest((2, 2), N=4, periodic=(False, True), rotating=(1, 2))
    with pytest.raises(ValueError, match="dimension 1 has a reflecting face"):
        Forest((2, 2), N=4, reflecting=((False, True), (False, False)), rotating=(1, 2))
    assert Forest((2, 2, 1), N=4, periodic=(False, False, True), rotating=(1, 2)).hasrotating()
    assert Forest((2, 1, 2), N=4, rotating=(3, 1)).rotating_dims() == (3, 1)
    assert Forest((2, 2), N=4).rotating == (0, 0)
    with pytest.raises(ValueError, match="both given"):
        Forest((2, 2), N=4, rotating=(1, 2), halfturn=(1, 2))
    with pytest.raises(ValueError, match="even number of roots"):
        Forest((1, 3), N=4, halfturn=(1, 2))
    h = Forest((1, 2), N=4, halfturn=(1, 2))
    assert h.hasrotating() and h.ishalfturn() and h.halfturn_dims() == (1, 2)
    assert h.rotating_dims() is None


@pytest.mark.parametrize("d1,d2", [(0, 1), (1, 0), (0, 2), (2, 1)])
def test_direction_and_offset_maps_turn_by_the_rotation(d1, d2):
    """``test/rotate_tests.jl:63-83``: against turned unit boxes."""
    for r in range(4):
        for delta in alldirections(3):
            unit = ((F(0),) * 3, tuple(F(x) for x in delta))
            lo, hi = rotate_box(unit, -r, d1, d2)
            assert real_direction(delta, r, d1, d2) == tuple(int(lo[d] + hi[d]) for d in range(3))
        for o in itertools.product((0, 1), repeat=3):
            box = (tuple(F(o[d] - 1) for d in range(3)), tuple(F(o[d]) for d in range(3)))
            lo, _ = rotate_box(box, r, d1, d2)
            assert virtual_offset(o, r, d1, d2) == tuple(int(lo[d]) + 1 for d in range(3))


def test_a_block_at_the_axis_is_its_own_neighbour():
    """``test/rotate_tests.jl:131-156``."""
    f = Forest((1, 1), N=4, rotating=(1, 2))
    k = f.leaves[0]
    assert f.turned_neighbors(k, (-1, 0)) == (1, [k])
    assert f.turned_neighbors(k, (0, -1)) == (3, [k])
    assert f.turned_neighbors(k, (-1, -1)) == (2, [k])
    assert f.turned_neighbors(k, (-1, 1)) == (1, [])
    assert f.turned_neighbors(k, (1, -1)) == (3, [])
    assert f.turned_neighbors(k, (1, 0)) == (0, [])
    octant = Forest((1, 1, 1), N=4, rotating=(1, 2),
                    reflecting=((False, False), (False, False), (True, False)))
    k = octant.leaves[0]
    assert octant.wall_direction(k, (-1, 0, -1))[0] == (-1, 0, 0)
    assert octant.turned_neighbors(k, (-1, 0, 0)) == (1, [k])


@pytest.mark.parametrize("D,plane,other", [(2, (1, 2), "outer"), (2, (2, 1), "outer"),
                                           (3, (1, 2), "outer"), (3, (1, 2), "periodic"),
                                           (3, (1, 2), "reflecting"), (3, (3, 1), "periodic"),
                                           (3, (2, 3), "reflecting")])
def test_the_seams_neighbours_are_the_unfolded_forests(D, plane, other):
    """``test/rotate_tests.jl:85-129``: random unbalanced quadrants, then
    balanced; every orientation meets every kind of neighbour."""
    rng = np.random.default_rng(1212 + D + 10 * plane[0] + len(other))
    seen = {}
    d1, d2 = plane[0] - 1, plane[1] - 1
    for trial in range(4 if D == 2 else 2):
        quad = random_seam_forest(rng, D, plane=plane, M=int(rng.integers(1, 3)), other=other,
                                  nsteps=30 if D == 2 else 12, maxlvl=3)
        bad, s, _ = neighbor_mismatches(quad)
        assert bad == 0
        for key, n in s.items():
            seen[key] = seen.get(key, 0) + n
        quad.balance()
        assert quad.isbalanced()
        bad, s, full = neighbor_mismatches(quad)
        assert bad == 0
        for key, n in s.items():
            seen[key] = seen.get(key, 0) + n
        assert full.isbalanced()
        assert seam_conforming(full, d1, d2)
    assert all(seen.get((r, "same"), 0) > 0 for r in range(4))
    assert all(seen.get((r, "none"), 0) > 0 for r in (0, 1, 3))


@pytest.mark.parametrize("D,plane,other", [(2, (1, 2), "outer"), (2, (2, 1), "outer"),
                                           (3, (1, 2), "periodic"), (3, (3, 2), "reflecting")])
def test_the_half_planes_neighbours_are_the_unfolded_forests(D, plane, other):
    """``test/halfturn_tests.jl:84-128``."""
    rng = np.random.default_rng(1414 + D + 10 * plane[0])
    seen = {}
    for trial in range(4 if D == 2 else 2):
        half = random_seam_forest(rng, D, plane=plane, M=int(rng.integers(1, 3)),
                                  M2=2 * int(rng.integers(1, 3)), other=other,
                                  nsteps=30 if D == 2 else 12, maxlvl=3, half=True)
        bad, s, _ = neighbor_mismatches(half, half=True)
        assert bad == 0
        for key, n in s.items():
            seen[key] = seen.get(key, 0) + n
        half.balance()
        assert half.isbalanced()
        bad, s, full = neighbor_mismatches(half, half=True)
        assert bad == 0
        for key, n in s.items():
            seen[key] = seen.get(key, 0) + n
        assert full.isbalanced()
    assert seen.get((2, "same"), 0) > 0 and seen.get((0, "same"), 0) > 0


# --- the turned fill -------------------------------------------------------------------

import torch                                                      # noqa: E402

import oracle                                                     # noqa: E402
from _helpers import nanbits                                      # noqa: E402
from treeamr import FieldSet, GhostSchedule, Operators            # noqa: E402
from treeamr.storage import composed_rotation                     # noqa: E402

OPS4 = Operators(prolongation=4, restriction=4)


def vector_rotation(D, plane):
    """A scalar and a vector's components (``test/ghost_oracles.jl:963-967``):
    the component along d1 becomes minus the one along d2, the one along d2
    the one along d1."""
    d1, d2 = plane
    return [1] + [-(1 + d2) if e == d1 else (1 + d1) if e == d2 else 1 + e
                  for e in range(1, D + 1)]


def vector_halfturn(D, plane):
    """``test/ghost_oracles.jl:1594``: the in-plane components negate."""
    return [1] + [-(1 + e) if e in plane else 1 + e for e in range(1, D + 1)]


def vector_parity(D, plane, other):
    """``test/ghost_oracles.jl:974-980``: reflecting at the low face of the
    dimension outside the plane, the component along its normal odd."""
    if other != "reflect_lo":
        return None
    z = 6 - plane[0] - plane[1]
    return [tuple("NoParity" if d + 1 != z else "OddParity" if v == z else "EvenParity"
                  for d in range(D)) for v in range(D + 1)]


def seam_forest(D, plane, other, *, half=False, N=8):
    """A quadrant (or half plane) refined to three levels at the seam and at
    the axis: 2 roots a side in the plane (the half plane 1 x 2), the third
    dimension periodic, outer or reflecting at its low face."""
    d1, d2 = plane
    roots = []
    for d in range(1, D + 1):
        roots.append((1 if d == d1 else 2) if half else 2 if d in plane else 1)
    periodic = tuple(other == "periodic" and d + 1 not in plane for d in range(D))
    reflecting = tuple((other == "reflect_lo" and d + 1 not in plane, False) for d in range(D))
    kw = {"halfturn": plane} if half else {"rotating": plane}
    f = Forest(tuple(roots), N=N, periodic=periodic, reflecting=reflecting, **kw)
    # refine the root at the axis, then its children touching the seam face
    f.refine([f.leaves[0]])
    f.balance()
    lo = [k for k in f.leaves if k.level == 1 and k.coords[d1 - 1] == 0 and k.root == 0]
    f.refine(lo[:1])
    f.balance()
    return f


def unfold_data(quad, fs, full, image, back, ff, q, half):
    """The full plane's own points: the quadrant's, turned.  Full leaf
    ``kf`` is quadrant leaf ``kq`` turned by ``r``, so its own point ``p``
    holds ``sign[v] * u_kq[sigma[v]](R^{-r} p)``, located with exact
    positions (cell centres, or vertices along a vertex-like dimension)."""
    D, N = quad.D, quad.N
    d1, d2 = quad.seam_plane()
    G = fs.G
    c = fs.c
    half_cell = [F(0) if c[d] else F(1, 2) for d in range(D)]
    host_q = fs.work.numpy()
    out = np.full(tuple(ff.work.shape), np.nan, dtype=fs.T)
    qindex = {k: i for i, k in enumerate(quad.leaves)}
    nv = fs.nvars
    for bf, kf in enumerate(full.leaves):
        r, kq = back(kf)
        bq = qindex[kq]
        steps = ((q,) if half else (q,) * r) if r else ()
        sigma, sign = composed_rotation(steps, nv)
        lof, _ = leafbox(full, kf)
        loq, _ = leafbox(quad, kq)
        h = F(1, N << kf.level)
        shift = tuple(quad.roots[d1] if (d == d1 or (d == d2 and not half)) else 0
                      for d in range(D))
        for I in itertools.product(*[range(N + c[d]) for d in range(D)]):
            x = [lof[d] + (I[d] + half_cell[d]) * h - shift[d] for d in range(D)]
            if r:
                if half:
                    cc = F(quad.roots[d2], 2)
                    x[d1], x[d2] = -x[d1], 2 * cc - x[d2]
                else:
                    for _ in range((4 - r) % 4):             # R^{-r} = R^{4-r}
                        x[d1], x[d2] = -x[d2], x[d1]
            Jf = [(x[d] - loq[d]) / h - half_cell[d] for d in range(D)]
            assert all(j.denominator == 1 for j in Jf)
            J = [int(j) for j in Jf]
            assert all(0 <= J[d] < N + c[d] for d in range(D))
            for v in range(nv):
                val = host_q[(bq, sigma[v] - 1) + tuple(G[d] + J[d] for d in reversed(range(D)))]
                out[(bf, v) + tuple(G[d] + I[d] for d in reversed(range(D)))] = \
                    fs.T.type(sign[v]) * val if sign[v] < 0 else val
    return out


def seam_fill(s, fs, host, *, one_tap=True, hook_zero=True, first=-1, last=0x7FFFFFFF):
    """The oracle's fill of a set over a seam, in place: stage P, the axis
    projection, stage 0 and phase 1, the hook regions set to zero, then the
    prolongations."""
    from treeamr.ghosts import turns_variables
    rv = fs.rotvars_host
    kw = dict(rotvars=rv, one_tap=one_tap)
    oracle.fill(s, host, fs.nvars, fs.factors_host, first=first, last=-1, **kw)
    if s.axis and turns_variables(fs):
        oracle.axis_project(s, host, fs.nvars, fs.factors_host, rv)
    oracle.fill(s, host, fs.nvars, fs.factors_host, first=0, last=1, **kw)
    if hook_zero:
        for r in s.boundaries:
            host[(r.block, slice(None)) +
                 tuple(slice(a - 1, z) for a, z in reversed(r.region))] = 0
    return oracle.fill(s, host, fs.nvars, fs.factors_host, first=2, last=last, **kw)


def quadrant_case(D, plane, other, *, half=False, T=np.float64, seed=3, C=None):
    """The quadrant's field set with NaN ghosts and random own points, its
    schedule, and the full plane's field set with the same data turned.  A
    set with a vertex-like dimension has its own points unified first (a
    fill, whose stage 0 makes the copies of a point one number through the
    turn and whose axis projection makes the axis its own image), so that
    the full plane's copies of a point agree."""
    quad = seam_forest(D, plane, other, half=half)
    q = (vector_halfturn if half else vector_rotation)(D, plane)
    kw = {"halfturn": q} if half else {"rotation": q}
    fs = FieldSet(quad, D + 1, G=2, T=T, parity=vector_parity(D, plane, other), centering=C,
                  **kw)
    rng = np.random.default_rng(seed)
    host = np.full(tuple(fs.work.shape), np.nan, dtype=T)
    own = (slice(None), slice(None)) + fs.interior()
    host[own] = rng.uniform(-1, 1, size=host[own].shape).astype(T)
    s = GhostSchedule(fs, OPS4)
    if any(fs.c):
        unified = seam_fill(s, fs, host.copy())
        host[own] = unified[own]
    fs.work = torch.from_numpy(host)
    full, image, back = (unfolded_halfturn_forest if half else unfolded_forest)(quad)
    ff = FieldSet(full, D + 1, G=2, T=T, parity=vector_parity(D, plane, other), centering=C)
    ff.work = torch.from_numpy(unfold_data(quad, fs, full, image, back, ff, q, half))
    return quad, fs, s, full, ff, image


SEAM_CASES = [(2, (1, 2), "none"), (2, (2, 1), "none"), (3, (1, 2), "periodic"),
              (3, (2, 1), "reflect_lo"), (3, (3, 1), "outer")]
HALF_CASES = [(2, (1, 2), "none"), (2, (2, 1), "none"), (3, (1, 2), "periodic"),
              (3, (3, 2), "reflect_lo")]
# more planes and faces, checked with the oracle on the CPU
MORE_SEAM_CASES = [(3, (1, 3), "outer"), (3, (3, 2), "reflect_lo")]
MORE_HALF_CASES = [(3, (2, 3), "reflect_lo"), (3, (3, 1), "periodic")]


@pytest.mark.parametrize("D,plane,other", SEAM_CASES + MORE_SEAM_CASES)
def test_a_rotating_quadrant_is_the_turned_full_plane(D, plane, other):
    """``test/rotate_tests.jl:437-456`` and ``:399-435``: every stored point
    of the quadrant after the fill, ghosts included, is the full plane's at
    the same place (the full plane holds the quadrant's data turned, and has
    no seam), to 1e-13 as in the reference: a turned stencil that reads a
    source's ghosts reads values the real frame summed in its own order.
    Every ghost the schedule writes is defined, and every kind of transfer
    crosses the seam."""
    quad, fs, s, full, ff, image = quadrant_case(D, plane, other)
    kinds = {(g.kind, g.orientation) for g in s.groups if g.orientation}
    assert {k for k, _ in kinds} == {"copy", "restrict", "prolong"}
    assert {r for _, r in kinds} >= {1, 3}
    got = zero_hook_fill(s, fs)
    want = zero_hook_fill(GhostSchedule(ff, OPS4), ff)
    _agree(quad, full, image, got, want)
    # every ghost is defined: no transfer read a ghost before it was written
    assert not np.isnan(got).any()


@pytest.mark.parametrize("D,plane,other", HALF_CASES + MORE_HALF_CASES)
def test_a_half_plane_is_the_turned_full_plane(D, plane, other):
    """``test/halfturn_tests.jl:349-377``."""
    quad, fs, s, full, ff, image = quadrant_case(D, plane, other, half=True)
    assert {g.orientation for g in s.groups} == {0, 2}
    got = zero_hook_fill(s, fs)
    want = zero_hook_fill(GhostSchedule(ff, OPS4), ff)
    _agree(quad, full, image, got, want)
    assert not np.isnan(got).any()


def zero_hook_fill(s, fs):
    """The oracle's fill with a hook that sets every outer-face region to
    zero, in both frames alike."""
    host = fs.work.numpy().copy()
    oracle.fill(s, host, fs.nvars, fs.factors_host, rotvars=fs.rotvars_host, last=1)
    for r in s.boundaries:
        host[(r.block, slice(None)) + tuple(slice(a - 1, z) for a, z in reversed(r.region))] = 0
    return oracle.fill(s, host, fs.nvars, fs.factors_host, rotvars=fs.rotvars_host, first=2)


def _agree(quad, full, image, got, want, tol=1e-13):
    findex = {k: i for i, k in enumerate(full.leaves)}
    worst = 0.0
    for b, k in enumerate(quad.leaves):
        g, w = got[b], want[findex[image(k, 0)]]
        assert np.array_equal(np.isnan(g), np.isnan(w)), (b, k)
        ok = ~np.isnan(g)
        worst = max(worst, float(np.max(np.abs(g[ok] - w[ok]), initial=0.0)))
    assert worst < tol, worst


@pytest.mark.parametrize("D,plane,other", SEAM_CASES[:3])
def test_the_schedule_partitions_the_ghosts_across_the_seam(D, plane, other):
    """``test/rotate_tests.jl:491-524``: every stored point outside the own
    range is written exactly once, by a transfer or by the hook."""
    quad, fs, s, *_ = quadrant_case(D, plane, other)
    counts = s.write_counts()
    N, G = quad.N, 2
    inside = np.ones(counts.shape[1:], bool)
    for ax in range(D):
        sl = [slice(None)] * D
        idx = np.arange(counts.shape[1 + ax])
        mask = (idx >= G) & (idx < G + N)
        shape = [1] * D
        shape[ax] = -1
        inside &= mask.reshape(shape)
    assert (counts[:, inside] == 0).all() and (counts[:, ~inside] == 1).all()


def test_seam_refusals():
    """A rotation map is required, checked, and its tables composed
    (``test/rotate_tests.jl:276-353``)."""
    f = Forest((2, 2), N=8, rotating=(1, 2))
    with pytest.raises(ValueError, match="needs `rotation`"):
        FieldSet(f, 3, G=1)
    with pytest.raises(ValueError, match="one entry per variable"):
        FieldSet(f, 3, G=1, rotation=(1, -3))
    with pytest.raises(ValueError, match="not a signed permutation"):
        FieldSet(f, 2, G=1, rotation=(1, 1))
    with pytest.raises(ValueError, match="turned four times"):
        FieldSet(f, 3, G=1, rotation=(2, 3, 1))
    assert FieldSet(f, 3, G=1, rotation=(1, -3, 2)).rotation == [1, -3, 2]
    assert FieldSet(Forest((2, 2), N=8), 1, G=1).rotvars is None
    # a vertex-like set over a seam is built: its axis is known to the schedule
    vs = GhostSchedule(FieldSet(f, 1, G=2, centering=("vertex", "vertex"), rotation=(1,)), OPS4)
    assert vs.axis and vs.axis_orbit == (0, 2, 1, 3)
    h = Forest((1, 2), N=8, halfturn=(1, 2))
    with pytest.raises(ValueError, match="needs `halfturn`"):
        FieldSet(h, 1, G=1)
    with pytest.raises(ValueError, match="applied twice"):
        FieldSet(h, 2, G=1, halfturn=(2, -1))
    fs = FieldSet(h, 3, G=1, halfturn=(1, -2, -3))
    assert fs.rotvars_host[:, 2].tolist() == [1, 2, 3]
    assert fs.factors_host[:, 2 * 9].tolist() == [1, -1, -1]


@pytest.mark.gpu
@pytest.mark.parametrize("case", [("q",) + c for c in SEAM_CASES] + [("h",) + c for c in HALF_CASES])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_turned_fill_bit_exact(cuda_lib, case, T):
    """The device fill across a seam, fused (the CPU form of the sum) and
    plain (the device form), is the oracle's bit for bit."""
    from treeamr import fill_ghosts
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h", T=T)
    host = fs.work.numpy().copy()
    fs.factors, fs.rotvars = fs.factors.cuda(), fs.rotvars.cuda()
    for method, one_tap in (("fused", True), ("plain", False)):
        expect = oracle.fill(s, host.copy(), fs.nvars, fs.factors_host,
                             rotvars=fs.rotvars_host, one_tap=one_tap)
        fs.work = torch.from_numpy(host.copy()).cuda()
        fill_ghosts(fs, s, method=method)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), method


@pytest.mark.gpu
def test_gpu_turned_fill_refusals(cuda_lib):
    """Without the variable table the library refuses a turned schedule,
    forward and adjoint; an asymmetric set is refused alone
    (``test/rotate_tests.jl:526-559``)."""
    from treeamr import fill_ghosts
    from treeamr.ghosts import device_schedule
    quad, fs, s, *_ = quadrant_case(2, (1, 2), "none")
    fs.work, fs.factors = fs.work.cuda(), fs.factors.cuda()
    rv = fs.rotvars
    fs.rotvars = None
    with pytest.raises(ValueError, match="variable table"):
        fill_ghosts(fs, s)
    ds = device_schedule(s, 0)
    rc = ds.lib.tam_fill(ds.handle, C.c_void_p(fs.work.data_ptr()), fs.nvars, fs.nblocks(),
                         C.c_void_p(fs.factors.data_ptr()), -1, 0x7FFFFFFF, None)
    assert rc != 0
    rc = ds.lib.tam_fill_adjoint(ds.handle, C.c_void_p(fs.work.data_ptr()), fs.nvars,
                                 fs.nblocks(), C.c_void_p(fs.factors.data_ptr()), -1,
                                 0x7FFFFFFF, None)
    assert rc != 0
    fs.rotvars = rv
    f = Forest((2, 2), N=8, rotating=(1, 2))
    asym = FieldSet(f, 1, G=(1, 2), rotation=(1,), device="cuda")
    with pytest.raises(ValueError, match="RotationPair"):
        fill_ghosts(asym, GhostSchedule(asym, Operators(prolongation=2, restriction=2)))


# --- RotationPair: asymmetric layouts -----------------------------------------------------

def unfold_member(quad, own_fs, partner_fs, full, back, ff, steps):
    """The full plane's own points of one member's layout: in quarter ``r``
    the composed map of ``steps[:r]`` applied to the quadrant data of the
    member itself (``r`` even) or of its partner (``r`` odd)."""
    D, N = quad.D, quad.N
    d1, d2 = quad.seam_plane()
    out = np.full(tuple(ff.work.shape), np.nan, dtype=own_fs.T)
    qindex = {k: i for i, k in enumerate(quad.leaves)}
    nv = own_fs.nvars
    for bf, kf in enumerate(full.leaves):
        r, kq = back(kf)
        src = partner_fs if r % 2 else own_fs
        hq = src.work.numpy()
        sigma, sign = composed_rotation(steps[:r], nv)
        lof, _ = leafbox(full, kf)
        loq, _ = leafbox(quad, kq)
        h = F(1, N << kf.level)
        shift = tuple(quad.roots[d1] if d in (d1, d2) else 0 for d in range(D))
        for I in itertools.product(range(N), repeat=D):
            x = [lof[d] + (I[d] + F(1, 2)) * h - shift[d] for d in range(D)]
            for _ in range((4 - r) % 4):
                x[d1], x[d2] = -x[d2], x[d1]
            J = [int((x[d] - loq[d]) / h - F(1, 2)) for d in range(D)]
            for v in range(nv):
                val = hq[(qindex[kq], sigma[v] - 1) +
                         tuple(src.G[d] + J[d] for d in reversed(range(D)))]
                out[(bf, v) + tuple(ff.G[d] + I[d] for d in reversed(range(D)))] = \
                    -val if sign[v] < 0 else val
    return out


def pair_case(D, plane, other, T=np.float64, seed=5):
    """A cell-centred pair whose ghost widths alone are swapped, the vector
    stored in swapped component orders so that the maps permute
    (``test/rotate_tests.jl:458-489``)."""
    from treeamr import RotationPair
    quad = seam_forest(D, plane, other)
    d1, d2 = plane[0] - 1, plane[1] - 1
    Ga = tuple(2 if d == d1 else 1 for d in range(D))
    Gb = tuple(2 if d == d2 else 1 for d in range(D))
    # a stores (s, v_1 .. v_D), b the same vector with its d1 and d2
    # components exchanged, w_{d1} = v_{d2} and w_{d2} = v_{d1}.  A quarter
    # turn takes v to (v'_{d1}, v'_{d2}) = (-v_{d2}, v_{d1}), so a's data at
    # R p come from b's at p as Q_a says, and b's from a's as Q_b says.
    nv = D + 1
    par = vector_parity(D, plane, other)
    qa = [1] + [-(2 + d1) if e == d1 else (2 + d2) if e == d2 else e + 2 for e in range(D)]
    qb = [1] + [(2 + d1) if e == d1 else -(2 + d2) if e == d2 else e + 2 for e in range(D)]
    perm_b = [0] + [1 + (d2 if e == d1 else d1 if e == d2 else e) for e in range(D)]
    parb = None if par is None else [par[perm_b[v]] for v in range(nv)]
    a = FieldSet(quad, nv, G=Ga, T=T, parity=par, rotation=qa)
    b = FieldSet(quad, nv, G=Gb, T=T, parity=parb, rotation=qb)
    rng = np.random.default_rng(seed)
    for fs in (a, b):
        host = np.full(tuple(fs.work.shape), np.nan, dtype=T)
        own = (slice(None), slice(None)) + tuple(slice(g, g + quad.N) for g in reversed(fs.G))
        host[own] = rng.uniform(-1, 1, size=host[own].shape).astype(T)
        fs.work = torch.from_numpy(host)
    pair = RotationPair(a, b)
    ops = Operators(prolongation=2, restriction=2)
    return quad, pair, (GhostSchedule(a, ops), GhostSchedule(b, ops)), ops


def oracle_pair_fill(pair, schedules, hook_zero=True):
    """The merged fill on the host: stage by stage, a then b, each turned
    group of odd orientation reading the partner's array."""
    a, b = pair.a, pair.b
    ha, hb = a.work.numpy().copy(), b.work.numpy().copy()
    sa, sb = schedules
    mem = [(sa, ha, hb, a, pair.afactors_host, pair.arotvars_host),
           (sb, hb, ha, b, pair.bfactors_host, pair.brotvars_host)]
    tags = sorted(set(sa.stage_tags) | set(sb.stage_tags))
    for phase in (0, 1):
        for tag in [t for t in tags if (t <= 1) == (phase == 0)]:
            for s, h, alt, fs, fac, rv in mem:
                oracle.fill(s, h, fs.nvars, fac, first=tag, last=tag, rotvars=rv, alt=alt)
        if phase == 0 and hook_zero:
            for s, h, *_ in mem:
                for r in s.boundaries:
                    h[(r.block, slice(None)) +
                      tuple(slice(x - 1, z) for x, z in reversed(r.region))] = 0
    return ha, hb


@pytest.mark.parametrize("D,plane,other", [(2, (1, 2), "none"), (2, (2, 1), "none"),
                                           (3, (1, 2), "reflect_lo"), (3, (3, 2), "periodic")])
def test_a_rotation_pair_is_the_turned_full_plane(D, plane, other):
    """``test/rotate_tests.jl:458-489``: a pair fill reads each set's ghosts
    across the seam out of the other through the composed maps; each set
    equals the full plane's set of its layout, which holds the quadrant's
    data turned, to 1e-13."""
    quad, pair, (sa, sb), ops = pair_case(D, plane, other)
    assert sa.odd_turns and sb.odd_turns
    ga, gb = oracle_pair_fill(pair, (sa, sb))
    full, image, back = unfolded_forest(quad)
    a, b = pair.a, pair.b
    for own, partner, got, steps in ((a, b, ga, (a.rotation, b.rotation, a.rotation)),
                                     (b, a, gb, (b.rotation, a.rotation, b.rotation))):
        ff = FieldSet(full, own.nvars, G=own.G, T=own.T, parity=own.parities)
        ff.work = torch.from_numpy(unfold_member(quad, own, partner, full, back, ff, steps))
        want = zero_hook_fill(GhostSchedule(ff, ops), ff)
        _agree(quad, full, image, got, want)
        assert not np.isnan(got).any()


def test_rotation_pair_refusals():
    """``test/rotate_tests.jl:355-397``."""
    from treeamr import RotationPair
    f = Forest((2, 2), N=8, rotating=(1, 2))
    A = lambda **kw: FieldSet(f, 1, G=(2, 1), rotation=(-1,), **kw)        # noqa: E731
    B = lambda **kw: FieldSet(f, 1, G=(1, 2), rotation=(1,), **kw)         # noqa: E731
    p = RotationPair(A(), B())
    assert p.arotvars_host.tolist() == [[1, 1, 1, 1]]
    assert p.afactors_host[0, [0, 9, 18, 27]].tolist() == [1, -1, -1, 1]
    assert p.bfactors_host[0, [0, 9, 18, 27]].tolist() == [1, 1, -1, -1]
    other = Forest((2, 2), N=8, rotating=(1, 2))
    with pytest.raises(ValueError, match="over one forest"):
        RotationPair(A(), FieldSet(other, 1, G=(1, 2), rotation=(1,)))
    with pytest.raises(ValueError, match="rotating seam"):
        plain = Forest((2, 2), N=8)
        RotationPair(FieldSet(plain, 1, G=(2, 1)), FieldSet(plain, 1, G=(1, 2)))
    with pytest.raises(ValueError, match="each other's layout"):
        RotationPair(A(), A())
    with pytest.raises(ValueError, match="turns into itself"):
        RotationPair(FieldSet(f, 1, G=1, rotation=(1,)), FieldSet(f, 1, G=1, rotation=(1,)))
    with pytest.raises(ValueError, match="same number of variables"):
        RotationPair(A(), FieldSet(f, 2, G=(1, 2), rotation=(1, 2)))
    with pytest.raises(ValueError, match="one element type"):
        RotationPair(A(), FieldSet(f, 1, G=(1, 2), rotation=(1,), T=np.float32))
    with pytest.raises(ValueError, match="not the identity"):
        RotationPair(FieldSet(f, 2, G=(2, 1), rotation=(-2, 1)),
                     FieldSet(f, 2, G=(1, 2), rotation=(1, 2)))


@pytest.mark.gpu
@pytest.mark.parametrize("D,plane,other", [(2, (1, 2), "none"), (3, (1, 2), "reflect_lo")])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_rotation_pair_bit_exact(cuda_lib, D, plane, other, T):
    """The device pair fill is the oracle's merged fill bit for bit."""
    from treeamr import fill_ghosts
    quad, pair, (sa, sb), ops = pair_case(D, plane, other, T=T)
    ea, eb = oracle_pair_fill(pair, (sa, sb), hook_zero=False)
    for fs in (pair.a, pair.b):
        fs.work, fs.factors = fs.work.cuda(), fs.factors.cuda()
    pair.to("cuda")
    fill_ghosts(pair, (sa, sb))
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(pair.a.work.cpu().numpy()), nanbits(ea))
    assert np.array_equal(nanbits(pair.b.work.cpu().numpy()), nanbits(eb))


@pytest.mark.parametrize("D,plane,other", [(2, (1, 2), "none"), (2, (2, 1), "none"),
                                           (3, (1, 2), "reflect_lo")])
def test_a_regrid_across_the_seam_is_the_full_planes(D, plane, other):
    """``test/rotate_tests.jl:561-604``: refining along the low face of d1
    near the axis makes conformity refine the image on the low face of d2;
    the regrid transfer's prolongations read their parents' ghosts across
    the seam, so the moved quadrant, filled again, is the full plane's
    regrid of the same leaves to 1e-13."""
    from test_regrid import oracle_regrid
    from treeamr.regrid import RegridTransfer
    quad, fs, s, full, ff, image = quadrant_case(D, plane, other)
    d1, d2 = quad.seam_plane()
    old_q, old_f = list(quad.leaves), list(full.leaves)
    hq = zero_hook_fill(s, fs)
    hf = zero_hook_fill(GhostSchedule(ff, OPS4), ff)
    marked = [k for k in quad.leaves if leafbox(quad, k)[0][d1] == 0 and
              leafbox(quad, k)[0][d2] < 1 and k.level < 3]
    assert marked
    quad.refine(marked)
    quad.balance()
    assert quad.isbalanced()
    # the full plane's regrid: the images of the quadrant's new leaves
    full, image, _ = unfolded_forest(quad)
    assert full.isbalanced() and seam_conforming(full, d1, d2)
    moved = []
    for forest, old, host, x in ((quad, old_q, hq, fs), (full, old_f, hf, ff)):
        t = RegridTransfer(forest, old, x.G, x.centering, x.T, OPS4)
        new = np.full((forest.nleaves(),) + tuple(x.work.shape[1:]), np.nan, x.T)
        moved.append(oracle_regrid(t, host, new, x.nvars))
    nq = FieldSet(quad, fs.nvars, G=2, parity=fs.parities, rotation=fs.rotation)
    nq.work = torch.from_numpy(moved[0])
    nf = FieldSet(full, ff.nvars, G=2, parity=ff.parities)
    nf.work = torch.from_numpy(moved[1])
    # the moved own points, then everything after a fill
    findex = {k: i for i, k in enumerate(full.leaves)}
    own = (slice(None),) + tuple(slice(2, 2 + quad.N) for _ in range(D))
    worst = 0.0
    for b, k in enumerate(quad.leaves):
        g, w = moved[0][b][own], moved[1][findex[image(k, 0)]][own]
        worst = max(worst, float(np.max(np.abs(g - w))))
    assert worst < 1e-13
    got = zero_hook_fill(GhostSchedule(nq, OPS4), nq)
    want = zero_hook_fill(GhostSchedule(nf, OPS4), nf)
    _agree(quad, full, image, got, want)


# --- the adjoint across the seam -------------------------------------------------------------

def _dot(a, b):
    return float(np.dot(a.ravel().astype(np.float64), b.ravel().astype(np.float64)))


@pytest.mark.parametrize("case", [("q",) + c for c in SEAM_CASES[:4] + MORE_SEAM_CASES] +
                         [("h",) + c for c in MORE_HALF_CASES] +
                         [("h",) + c for c in HALF_CASES[:3]])
def test_oracle_adjoint_dot_product_across_the_seam(case):
    """``<A x, y> = <x, A^T y>`` to 1e-13 with turned transfers, A the
    oracle's fill and A^T its scatter-form transpose through the axis map
    and the variable table."""
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h")
    rng = np.random.default_rng(17)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    ax = oracle.fill(s, x.copy(), fs.nvars, fs.factors_host, rotvars=fs.rotvars_host)
    aty = oracle.fill_adjoint(s, y.copy(), fs.nvars, fs.factors_host, rotvars=fs.rotvars_host)
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


@pytest.mark.gpu
@pytest.mark.parametrize("case", [("q",) + c for c in SEAM_CASES] +
                         [("h",) + c for c in HALF_CASES])
def test_gpu_adjoint_across_the_seam(cuda_lib, case):
    """The device adjoint of a turned schedule: the dot-product test against
    the device forward fill to 1e-13, and the oracle's scatter-form
    transpose to the sums' rounding."""
    from treeamr import fill_ghosts
    from treeamr.adjoint import fill_ghosts_adjoint
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h")
    rng = np.random.default_rng(23)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.factors, fs.rotvars = fs.factors.cuda(), fs.rotvars.cuda()
    fs.work = torch.from_numpy(x.copy()).cuda()
    fill_ghosts(fs, s)
    ax = fs.work.cpu().numpy()
    yd = torch.from_numpy(y.copy()).cuda()
    fs.work = torch.from_numpy(x.copy()).cuda()
    fill_ghosts_adjoint(fs, s, yd)
    torch.cuda.synchronize()
    aty = yd.cpu().numpy()
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    want = oracle.fill_adjoint(s, y.copy(), fs.nvars, fs.factors_host, rotvars=fs.rotvars_host)
    assert np.max(np.abs(aty - want)) < 1e-13


@pytest.mark.gpu
def test_gpu_adjoint_of_a_pair_member_is_refused(cuda_lib):
    from treeamr.adjoint import fill_ghosts_adjoint
    quad, pair, (sa, sb), ops = pair_case(2, (1, 2), "none")
    a = pair.a
    a.work, a.factors, a.rotvars = a.work.cuda(), a.factors.cuda(), a.rotvars.cuda()
    with pytest.raises(Exception, match="RotationPair"):
        fill_ghosts_adjoint(a, sa, torch.zeros_like(a.work))
    # the library itself: without the partner's cotangent the member is refused
    from treeamr.ghosts import device_schedule
    ds = device_schedule(sa, 0)
    with pytest.raises(Exception, match="tam_fill_adjoint_alt"):
        ds.run_adjoint(torch.zeros_like(a.work), a.nvars, a.factors, -1, 0x7FFFFFFF,
                       rotvars=a.rotvars)



# --- sets with vertex-like dimensions over a seam -----------------------------------------

VERTEX_CASES = [("q", 2, (1, 2), "none"), ("q", 2, (2, 1), "none"),
                ("q", 3, (1, 2), "periodic"), ("q", 3, (3, 1), "outer"),
                ("h", 2, (1, 2), "none"), ("h", 3, (1, 2), "periodic")]
# checked with the oracle on the CPU: a reflecting low face beside the seam
# puts stage P (an odd and an even variable across the wall) into the fill
MORE_VERTEX_CASES = [("q", 3, (1, 2), "reflect_lo"), ("h", 3, (3, 2), "reflect_lo"),
                     ("q", 3, (2, 3), "outer"), ("h", 3, (1, 3), "periodic")]


def _centering(D, plane, which):
    from treeamr.storage import vertexcentered
    if which == "vertex":
        return vertexcentered(D)
    # vertex-like along the plane's two dimensions only (symmetric in the turn)
    return tuple("vertex" if d + 1 in plane else "cell" for d in range(D))


@pytest.mark.parametrize("case", VERTEX_CASES + MORE_VERTEX_CASES)
@pytest.mark.parametrize("which", ["vertex", "plane"])
def test_a_vertex_like_quadrant_is_the_turned_full_plane(case, which):
    """``test/rotate_tests.jl:437-456`` for vertex-like sets: the seam
    planes are copies of each other through the turn (stage 0 across the
    seam) and the axis its own image (the projection); after a fill every
    stored point is the full plane's to 1e-13 and none is undefined."""
    kind, D, plane, other = case
    C = _centering(D, plane, which)
    quad, fs, s, full, ff, image = quadrant_case(D, plane, other, half=kind == "h", C=C)
    assert any(g.orientation and g.stage == 0 for g in s.groups)
    assert s.axis
    got = seam_fill(s, fs, fs.work.numpy().copy())
    want = seam_fill(GhostSchedule(ff, OPS4), ff, ff.work.numpy().copy())
    _agree(quad, full, image, got, want)
    assert not np.isnan(got).any()
    # the fill is idempotent on unified data: a second fill changes no bit
    again = seam_fill(s, fs, got.copy())
    assert np.array_equal(nanbits(again), nanbits(got))


@pytest.mark.parametrize("case", VERTEX_CASES[:3])
def test_the_vertex_schedule_partitions_the_ghosts_across_the_seam(case):
    """Every stored point outside the closed own box is written exactly once
    by a transfer or the hook (``test/rotate_tests.jl:491-524``)."""
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h",
                                    C=_centering(D, plane, "vertex"))
    counts = s.write_counts()
    N, G = quad.N, 2
    inside = np.ones(counts.shape[1:], bool)
    for ax in range(D):
        idx = np.arange(counts.shape[1 + ax])
        mask = (idx >= G) & (idx < G + N + 1)
        shape = [1] * D
        shape[ax] = -1
        inside &= mask.reshape(shape)
    assert (counts[:, inside] == 0).all() and (counts[:, ~inside] == 1).all()


@pytest.mark.gpu
@pytest.mark.parametrize("case", VERTEX_CASES)
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_vertex_like_fill_across_the_seam_bit_exact(cuda_lib, case, T):
    """The device fill of a vertex-like set over a seam (turned stage-0
    copies, the axis projection) is the oracle's bit for bit."""
    from treeamr import fill_ghosts
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h", T=T,
                                    C=_centering(D, plane, "vertex"))
    host = fs.work.numpy().copy()
    rng = np.random.default_rng(5)
    host[(slice(None), slice(None)) + fs.interior()] = \
        rng.uniform(-1, 1, size=host[(slice(None), slice(None)) + fs.interior()].shape)
    fs.factors, fs.rotvars = fs.factors.cuda(), fs.rotvars.cuda()
    for method, one_tap in (("fused", True), ("plain", False)):
        expect = seam_fill(s, fs, host.copy(), one_tap=one_tap, hook_zero=False)
        fs.work = torch.from_numpy(host.copy()).cuda()
        fill_ghosts(fs, s, method=method)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), method


# --- the adjoint across a vertex seam: the axis projection's transpose --------------------

def oracle_vertex_adjoint(s, fs, y):
    """``A^T y`` of ``seam_fill`` without the hook (the oracle's transposes
    of stages 0 and on, of the axis projection, then of stage P)."""
    from treeamr.ghosts import turns_variables
    rv = fs.rotvars_host
    oracle.fill_adjoint(s, y, fs.nvars, fs.factors_host, first=0, rotvars=rv)
    if s.axis and turns_variables(fs):
        oracle.axis_project_adjoint(s, y, fs.nvars, fs.factors_host, rv)
    return oracle.fill_adjoint(s, y, fs.nvars, fs.factors_host, last=-1, rotvars=rv)


@pytest.mark.parametrize("case", VERTEX_CASES + MORE_VERTEX_CASES)
def test_oracle_adjoint_dot_product_across_a_vertex_seam(case):
    """``<A x, y> = <x, A^T y>`` to 1e-13 where the fill holds the axis
    projection between stage P and stage 0, and the projection of the
    product's transposed tables is the oracle's scatter-form transpose."""
    from treeamr.ghosts import axis_transposed_tables, turns_variables
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h",
                                    C=_centering(D, plane, "vertex"))
    assert s.axis and turns_variables(fs)
    rng = np.random.default_rng(29)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    ax = seam_fill(s, fs, x.copy(), hook_zero=False)
    aty = oracle_vertex_adjoint(s, fs, y.copy())
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    # without the projection's transpose the test fails: the axis matters here
    wrong = oracle.fill_adjoint(s, y.copy(), fs.nvars, fs.factors_host, rotvars=fs.rotvars_host)
    assert abs(lhs - _dot(x, wrong)) > 1e-10 * max(abs(lhs), 1.0)
    # the product's transposed tables, run through the projection's own form
    ft, rt = axis_transposed_tables(fs)
    got = oracle.axis_project(s, y.copy(), fs.nvars, ft, rt)
    want = oracle.axis_project_adjoint(s, y.copy(), fs.nvars, fs.factors_host, fs.rotvars_host)
    assert np.max(np.abs(got - want)) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("case", VERTEX_CASES)
def test_gpu_adjoint_across_a_vertex_seam(cuda_lib, case):
    """The device adjoint over a vertex seam: the dot-product test against
    the device forward fill to 1e-13, and the oracle's transpose to the
    sums' rounding."""
    from treeamr import fill_ghosts
    from treeamr.adjoint import fill_ghosts_adjoint
    kind, D, plane, other = case
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h",
                                    C=_centering(D, plane, "vertex"))
    rng = np.random.default_rng(31)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.factors, fs.rotvars = fs.factors.cuda(), fs.rotvars.cuda()
    fs.work = torch.from_numpy(x.copy()).cuda()
    fill_ghosts(fs, s)
    ax = fs.work.cpu().numpy()
    yd = torch.from_numpy(y.copy()).cuda()
    fill_ghosts_adjoint(fs, s, yd)
    torch.cuda.synchronize()
    aty = yd.cpu().numpy()
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    want = oracle_vertex_adjoint(s, fs, y.copy())
    assert np.max(np.abs(aty - want)) < 1e-13


# --- turned and bounded members in a batch of forests -------------------------------------

def _batch_members(bounded=True):
    """Field sets of 3 Float64 variables over 2-D forests: a turned
    cell-centred quadrant, a vertex-like quadrant (its axis projected), a
    plain nested forest and, with ``bounded``, a bounded one; each with its
    schedule and random own points."""
    from _helpers import nested_forest
    from treeamr import FieldSet, GhostSchedule, Operators
    from treeamr.operators import Conservative
    out = []
    for C in (None, _centering(2, (1, 2), "vertex")):
        _, fs, s, *_ = quadrant_case(2, (1, 2), "none", C=C)
        out.append((fs, s))
    kinds = [OPS4] + ([Operators(prolongation=3, restriction=2, family=Conservative,
                                 bounded=True)] if bounded else [])
    for k, ops in enumerate(kinds):
        fs = FieldSet(nested_forest(2, N=8, periodic=(True, True)), 3, G=1 + (k == 0))
        fs.work = torch.from_numpy(
            np.random.default_rng(40 + k).uniform(-1, 1, size=tuple(fs.work.shape)))
        out.append((fs, GhostSchedule(fs, ops)))
    return out


@pytest.mark.gpu
def test_gpu_batch_of_turned_and_bounded_members(cuda_lib):
    """A batch holding turned quadrants (one cell-centred, one vertex-like
    whose axis is projected between stage P and stage 0), a plain set and a
    bounded one fills every member as its own fill does, bit for bit."""
    from treeamr import fill_ghosts
    from treeamr.batch import ForestBatch
    members = _batch_members()
    fss, scheds = [m[0] for m in members], [m[1] for m in members]
    assert any(g.bounded for g in scheds[3].groups) and scheds[1].axis
    batch = ForestBatch(fss, scheds)
    start = batch.arena.clone()
    batch.fill()
    alone = start.clone()
    for m, (fs, s) in enumerate(members):
        fs.work = batch.member_view(alone, m)
        fill_ghosts(fs, s)
    torch.cuda.synchronize()
    assert batch.device_status() == 0
    assert np.array_equal(nanbits(batch.arena.cpu().numpy()), nanbits(alone.cpu().numpy()))
    # and each turned member is the oracle's fill
    for m in (0, 1):
        fs, s = members[m]
        want = seam_fill(s, fs, batch.member_view(start, m).cpu().numpy().copy(),
                         hook_zero=False)
        got = batch.member_view(batch.arena, m).cpu().numpy()
        assert np.array_equal(nanbits(got), nanbits(want)), m


@pytest.mark.gpu
def test_gpu_batch_adjoint_of_turned_members(cuda_lib):
    """The batch's adjoint over turned members (the axis projection's
    transpose between stage 0's and stage P's) is each member's own adjoint
    bit for bit; a batch with a bounded member has none."""
    from treeamr.adjoint import fill_ghosts_adjoint
    from treeamr.batch import ForestBatch
    members = _batch_members(bounded=False)
    fss, scheds = [m[0] for m in members], [m[1] for m in members]
    batch = ForestBatch(fss, scheds)
    y = torch.rand(batch.arena.shape, dtype=batch.arena.dtype, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(8))
    got = y.clone()
    batch.fill_adjoint(got)
    alone = y.clone()
    for m, (fs, s) in enumerate(members):
        fill_ghosts_adjoint(fs, s, batch.member_view(alone, m))
    torch.cuda.synchronize()
    assert torch.equal(got.view(torch.int64), alone.view(torch.int64))
    with_bounded = _batch_members()
    b2 = ForestBatch([m[0] for m in with_bounded], [m[1] for m in with_bounded])
    with pytest.raises(Exception, match="not linear"):
        b2.fill_adjoint(b2.arena.clone())


@pytest.mark.gpu
def test_gpu_batch_refuses_a_pair_member_and_flags_a_bad_table(cuda_lib):
    """A RotationPair member reads its partner's array, which a batch does not
    hold: the library refuses it.  A variable table naming no variable is
    skipped by the solo launch and reported through the batch's error word."""
    from treeamr import _native
    from treeamr.batch import ForestBatch
    from treeamr.ghosts import device_schedule
    quad, pair, (sa, sb), ops = pair_case(2, (1, 2), "none")
    lib, ctx = _native.lib(), _native.context(0)
    h = device_schedule(sa, 0).handle
    out = C.c_void_p()
    rc = lib.tam_batch_create(ctx, (C.c_void_p * 1)(h.value), 1, (C.c_int64 * 1)(0),
                              (C.c_int64 * 1)(0), C.byref(out))
    assert rc != 0 and "RotationPair" in _native.last_error(ctx)
    fs, s = _batch_members(bounded=False)[0]
    batch = ForestBatch([fs], [s])
    batch.rotvars.zero_()
    batch.fill()
    assert batch.device_status() == _native.TAM_EINVAL
    assert batch.device_status() == 0   # read and cleared


# --- the adjoint of a RotationPair ------------------------------------------------------------

PAIR_ADJ_CASES = [(2, (1, 2), "none"), (2, (2, 1), "none"), (3, (1, 2), "reflect_lo"),
                  (3, (3, 2), "periodic")]


def oracle_pair_adjoint(pair, schedules, ya, yb):
    """The oracle's transpose of ``oracle_pair_fill`` without the hook: tag by
    tag from the last, b's stage transpose then a's, odd turns scattering
    onto the partner's cotangent."""
    sa, sb = schedules
    mem = [(sa, ya, yb, pair.a, pair.afactors_host, pair.arotvars_host),
           (sb, yb, ya, pair.b, pair.bfactors_host, pair.brotvars_host)]
    tags = sorted(set(sa.stage_tags) | set(sb.stage_tags))
    for tag in reversed(tags):
        for s, y, alt, fs, fac, rv in reversed(mem):
            oracle.fill_adjoint(s, y, fs.nvars, fac, first=tag, last=tag, rotvars=rv, alt=alt)
    return ya, yb


def _pair_vectors(pair, seed):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, size=tuple(fs.work.shape)) for fs in (pair.a, pair.b)]


@pytest.mark.parametrize("D,plane,other", PAIR_ADJ_CASES)
def test_oracle_adjoint_dot_product_of_a_rotation_pair(D, plane, other):
    """``<A x, y> = <x, A^T y>`` to 1e-13 over both members of a pair, whose
    odd turns read (and whose transposes add onto) the partner's array."""
    quad, pair, (sa, sb), ops = pair_case(D, plane, other)
    xa, xb = _pair_vectors(pair, 11)
    ya, yb = _pair_vectors(pair, 12)
    pair.a.work, pair.b.work = torch.from_numpy(xa.copy()), torch.from_numpy(xb.copy())
    axa, axb = oracle_pair_fill(pair, (sa, sb), hook_zero=False)
    ata, atb = oracle_pair_adjoint(pair, (sa, sb), ya.copy(), yb.copy())
    lhs = _dot(axa, ya) + _dot(axb, yb)
    rhs = _dot(xa, ata) + _dot(xb, atb)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


@pytest.mark.gpu
@pytest.mark.parametrize("D,plane,other", PAIR_ADJ_CASES)
def test_gpu_adjoint_of_a_rotation_pair(cuda_lib, D, plane, other):
    """The device adjoint of a pair fill (``fill_pair_adjoint``): the dot
    test against the device pair fill to 1e-13, and the oracle's transpose
    to the sums' rounding."""
    from treeamr.adjoint import fill_pair_adjoint
    from treeamr.ghosts import fill_pair
    quad, pair, (sa, sb), ops = pair_case(D, plane, other)
    for fs in (pair.a, pair.b):
        fs.factors = fs.factors.cuda()
    pair.to("cuda")
    xa, xb = _pair_vectors(pair, 13)
    ya, yb = _pair_vectors(pair, 14)
    pair.a.work = torch.from_numpy(xa.copy()).cuda()
    pair.b.work = torch.from_numpy(xb.copy()).cuda()
    fill_pair(pair, (sa, sb))
    axa, axb = pair.a.work.cpu().numpy(), pair.b.work.cpu().numpy()
    da, db = torch.from_numpy(ya.copy()).cuda(), torch.from_numpy(yb.copy()).cuda()
    fill_pair_adjoint(pair, (sa, sb), da, db)
    torch.cuda.synchronize()
    ata, atb = da.cpu().numpy(), db.cpu().numpy()
    lhs = _dot(axa, ya) + _dot(axb, yb)
    rhs = _dot(xa, ata) + _dot(xb, atb)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    wa, wb = oracle_pair_adjoint(pair, (sa, sb), ya.copy(), yb.copy())
    assert np.max(np.abs(ata - wa)) < 1e-13 and np.max(np.abs(atb - wb)) < 1e-13


# --- awkward data across the seam ---------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("case", [("q", 2, (1, 2), "none", None), ("q", 3, (1, 2), "periodic", None),
                                  ("h", 3, (1, 2), "periodic", None),
                                  ("q", 2, (1, 2), "none", "vertex")])
def test_gpu_awkward_data_across_the_seam(cuda_lib, case):
    """+-0, NaN, +-Inf and subnormals through turned copies, restrictions,
    prolongations and the axis projection (``test/ghost_tests.jl:507-560``):
    the device fill, fused and plain, is the oracle's bit for bit."""
    from _helpers import awkward_fill
    from treeamr import fill_ghosts
    kind, D, plane, other, which = case
    C = _centering(D, plane, which) if which else None
    quad, fs, s, *_ = quadrant_case(D, plane, other, half=kind == "h", C=C)
    host = awkward_fill(tuple(fs.work.shape), np.float64, seed=D + 7)
    fs.factors, fs.rotvars = fs.factors.cuda(), fs.rotvars.cuda()
    for method, one_tap in (("fused", True), ("plain", False)):
        expect = seam_fill(s, fs, host.copy(), one_tap=one_tap, hook_zero=False)
        fs.work = torch.from_numpy(host.copy()).cuda()
        fill_ghosts(fs, s, method=method)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), method


@pytest.mark.gpu
def test_gpu_a_table_naming_no_variable_is_flagged(cuda_lib):
    """A variable table naming no variable (every entry 0): the forward's
    solo launch and the adjoint's pass 2 skip the writes it would steer and
    set the schedule's error word, which the host reads and clears."""
    from treeamr import _native, fill_ghosts
    from treeamr.ghosts import device_schedule
    quad, fs, s, *_ = quadrant_case(2, (1, 2), "none")
    fs.factors = fs.factors.cuda()
    fs.rotvars = torch.zeros_like(fs.rotvars).cuda()
    fs.work = fs.work.cuda()
    ds = device_schedule(s, 0)
    ds.status(fs)
    fill_ghosts(fs, s)
    assert ds.status(fs) == _native.TAM_EINVAL
    assert ds.status(fs) == 0
    y = torch.ones_like(fs.work)
    ds.run_adjoint(y, fs.nvars, fs.factors, _native.TAM_STAGE_ALL_FIRST,
                   _native.TAM_STAGE_ALL_LAST, rotvars=fs.rotvars)
    assert ds.status(fs) == _native.TAM_EINVAL
    assert ds.status(fs) == 0
