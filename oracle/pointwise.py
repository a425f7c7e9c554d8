"""The point-by-point ghost fill: TEST INFRASTRUCTURE ONLY.

A second oracle, independent of the product's schedule: nothing here
imports ``treeamr.schedule`` or ``treeamr.operators``, and no
``GhostSchedule`` is built.  Only ``tests/`` call it.

- ``rebuild_forest``: the meshes' leaves rebuilt from their construction
  rules (refine every leaf of a pass's level that meets a predicate on its
  box, then the minimal 2:1 refinement across faces, edges and corners:
  ``src/forest.jl:1837-1908``), as a set of ``(level, anchor)``, the anchor
  being the node's integer coordinates at its level over the whole brick.
- ``morton_order``: the reference's leaf order (``src/morton.jl:454-482``):
  root (dimension 1 fastest), then the bit-interleaved coordinates with
  dimension 1 most significant.
- ``lagrange_table``: the order-p Lagrange weights at every quarter offset of
  a window of p unit-spaced nodes, in exact rationals, rounded once to
  nearest-even into the element type (``src/operators.jl:597-682``).
- ``fill``: ``pointwise.c``'s fill of a field set's own points, every ghost
  derived from the forest's geometry alone.

Parity: the point-by-point fill and the schedule replay (``fill_oracle.c``
over the product's ``GhostSchedule``) are compared bit for bit in
``tests/test_pointwise.py`` on the benchmark's meshes at reduced size, and the
GPU fill against this one at full size.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from fractions import Fraction
from typing import Dict, Iterable, List, Sequence, Set, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtam_pointwise.so")
SRC = os.path.join(HERE, "pointwise.c")

PW_REFLECT, PW_OUTFLOW = 1, 2

_lock = threading.Lock()
_lib = None


class pw_mesh(C.Structure):
    _fields_ = [("D", C.c_int32), ("N", C.c_int32), ("p", C.c_int32), ("vertex", C.c_int32),
                ("G", C.c_int32 * 3), ("S", C.c_int32 * 3), ("roots", C.c_int32 * 3),
                ("periodic", C.c_int32 * 3), ("face", (C.c_int32 * 2) * 3),
                ("nblocks", C.c_int64), ("nvars", C.c_int32),
                ("level", C.c_void_p), ("anchor", C.c_void_p), ("sigma", C.c_void_p)]


def build(force: bool = False) -> str:
    """gcc -O2 -fopenmp -ffp-contract=off: no fused multiply-add on any host."""
    with _lock:
        os.makedirs(BUILD_DIR, exist_ok=True)
        if not force and os.path.exists(LIB_PATH) and \
                os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
            return LIB_PATH
        tmp = LIB_PATH + ".tmp"
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-fPIC", "-shared", SRC, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"pointwise oracle build failed:\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(LIB_PATH)
        l.pw_fill.argtypes = [C.POINTER(pw_mesh), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_int]
        l.pw_fill.restype = C.c_int
        _lib = l
    return _lib


# ---- weights ------------------------------------------------------------------

def round_f32(q: Fraction) -> float:
    """``q`` rounded once to the nearest float32, ties to even."""
    if q == 0:
        return 0.0
    sign = -1.0 if q < 0 else 1.0
    q = abs(q)
    e = q.numerator.bit_length() - q.denominator.bit_length()
    if Fraction(2) ** e > q:
        e -= 1                                       # 2^e <= q < 2^(e+1)
    e = max(e, -126)                                 # subnormals share the last exponent
    scaled = q / Fraction(2) ** (e - 23)             # the significand in units of the last place
    m = scaled.numerator // scaled.denominator
    rem = scaled - m
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and m % 2 == 1):
        m += 1
    return sign * float(np.float32(m * 2.0 ** (e - 23)))


def lagrange_table(p: int, T) -> np.ndarray:
    """Row ``k`` (``k = 0 .. 4(p-1)``): the weights ``w_m``, ``m = 0..p-1``,
    with ``sum_m w_m u(m) = u(k/4)`` for every polynomial of degree < p,
    ``w_m = prod_{n != m} (k/4 - n) / (m - n)``, each rounded once into T."""
    T = np.dtype(T)
    rows = []
    for k in range(4 * (p - 1) + 1):
        x = Fraction(k, 4)
        row = []
        for mm in range(p):
            w = Fraction(1)
            for n in range(p):
                if n != mm:
                    w *= (x - n) / Fraction(mm - n)
            row.append(float(w) if T == np.float64 else round_f32(w))
        rows.append(row)
    return np.array(rows, dtype=T)


# ---- the forest ---------------------------------------------------------------

Leaf = Tuple[int, Tuple[int, ...]]


class Brick:
    """A brick of roots with its faces: ``periodic[d]``, and past a
    non-periodic face ``faces[d] = (lo, hi)`` in {PW_REFLECT, PW_OUTFLOW, 0}."""

    def __init__(self, roots: Sequence[int], N: int, periodic: Sequence[bool],
                 extents: Sequence[Tuple[float, float]]):
        self.roots = tuple(int(r) for r in roots)
        self.D = len(self.roots)
        self.N = int(N)
        self.periodic = tuple(bool(x) for x in periodic)
        self.extents = tuple((float(a), float(b)) for a, b in extents)

    def box(self, leaf: Leaf):
        """The leaf's box in coordinates: node spacing h = (hi - lo) / roots_1
        / N / 2^level (dimension 1's, rounded step by step), corners
        lo + anchor N h and lo + (anchor + 1) N h."""
        lvl, a = leaf
        lo0, hi0 = self.extents[0]
        h = (hi0 - lo0) / self.roots[0] / self.N / (1 << lvl)
        return tuple((self.extents[d][0] + a[d] * self.N * h,
                      self.extents[d][0] + (a[d] + 1) * self.N * h) for d in range(self.D))


def _directions(D):
    out = [()]
    for _ in range(D):
        out = [o + (s,) for o in out for s in (-1, 0, 1)]
    return [o for o in out if any(o)]


def _refine(leaves: Set[Leaf], leaf: Leaf, D: int):
    lvl, a = leaf
    leaves.discard(leaf)
    for off in range(1 << D):
        leaves.add((lvl + 1, tuple(2 * a[d] + ((off >> d) & 1) for d in range(D))))


def _covering(leaves: Set[Leaf], lvl: int, a: Tuple[int, ...]):
    """The leaf at or above node (lvl, a), or None when the node is refined."""
    for up in range(lvl + 1):
        k = (lvl - up, tuple(x >> up for x in a))
        if k in leaves:
            return k
    return None


def balance(leaves: Set[Leaf], brick: Brick) -> Set[Leaf]:
    """The minimal refinement in which leaves that touch (across a face, an
    edge or a corner, periodic faces included) differ by at most one level."""
    D = brick.D
    dirs = _directions(D)
    work = sorted(leaves, key=lambda k: -k[0])
    while work:
        nxt = set()
        for leaf in work:
            if leaf not in leaves:
                continue
            lvl, a = leaf
            if lvl < 2:
                continue
            for dl in dirs:
                n = list(a[d] + dl[d] for d in range(D))
                ok = True
                for d in range(D):
                    top = brick.roots[d] << lvl
                    if not 0 <= n[d] < top:
                        if brick.periodic[d]:
                            n[d] %= top
                        else:
                            ok = False
                if not ok:
                    continue
                c = _covering(leaves, lvl, tuple(n))
                if c is not None and c[0] < lvl - 1:
                    _refine(leaves, c, D)
                    nxt.update((c[0] + 1, tuple(2 * c[1][d] + ((off >> d) & 1)
                                                for d in range(D))) for off in range(1 << D))
                    nxt.add(leaf)
        work = sorted(nxt, key=lambda k: -k[0])
    return leaves


def rebuild_forest(brick: Brick, passes: Iterable[Tuple[int, callable]]) -> Set[Leaf]:
    """The roots, then per pass ``(level, pred)``: every leaf of that level
    whose box meets ``pred`` refined, then balanced."""
    D = brick.D
    leaves: Set[Leaf] = set()
    for idx in np.ndindex(*reversed(brick.roots)):
        leaves.add((0, tuple(reversed(idx))))
    for lvl, pred in passes:
        targets = [k for k in leaves if k[0] == lvl and pred(brick.box(k))]
        if not targets:
            continue
        for k in targets:
            _refine(leaves, k, D)
        balance(leaves, brick)
    return leaves


def morton_key(leaf: Leaf, roots: Sequence[int], maxbits: int = 32):
    """Root index (dimension 1 fastest), then the coordinates within the
    root, padded to ``maxbits`` bits and interleaved bit by bit from the
    top, dimension 1 first."""
    lvl, a = leaf
    D = len(a)
    rp = [x >> lvl for x in a]
    root = 0
    stride = 1
    for d in range(D):
        root += rp[d] * stride
        stride *= roots[d]
    loc = [(a[d] - (rp[d] << lvl)) << (maxbits - lvl) for d in range(D)]
    code = 0
    for bit in range(maxbits - 1, -1, -1):
        for d in range(D):
            code = (code << 1) | ((loc[d] >> bit) & 1)
    return (root, code, lvl)


def leaves_of(forest) -> List[Leaf]:
    """The product forest's leaves as ``(level, anchor)``, in its order."""
    out = []
    for k in forest.leaves:
        rp = forest.root_position(k.root)
        out.append((k.level, tuple((rp[d] << k.level) + k.coords[d] for d in range(forest.D))))
    return out


# ---- the fill -------------------------------------------------------------------

def fill(fs, data: np.ndarray, p: int, nthreads: int = None) -> np.ndarray:
    """The point-by-point fill of ``data`` (shape ``(nblocks, nvars,
    S_D..S_1)``, C order, the field set's element type): a new array whose
    own points are stages P and 0's and whose ghosts are derived from the
    forest.  Raises on a layout the point-by-point fill does not cover."""
    f = fs.forest
    D = f.D
    T = np.dtype(data.dtype)
    assert data.flags.c_contiguous and T in (np.float32, np.float64)
    if len(set(fs.c)) != 1:
        raise ValueError("the point-by-point fill takes all-cell or all-vertex sets")
    if f.hasrotating():
        raise ValueError("the point-by-point fill takes no seams")
    m = pw_mesh()
    m.D, m.N, m.p, m.vertex = D, f.N, p, fs.c[0]
    for d in range(3):
        m.G[d] = fs.G[d] if d < D else 0
        m.S[d] = fs.stored[d] if d < D else 1
        m.roots[d] = f.roots[d] if d < D else 1
        m.periodic[d] = int(f.periodic[d]) if d < D else 1
        for s in range(2):
            kind = f.faces[d][s] if d < D else 0
            # forest face kinds: 0 outer, 1 reflecting, 2 outflow
            m.face[d][s] = {0: 0, 1: PW_REFLECT, 2: PW_OUTFLOW}[kind]
    leaves = leaves_of(f)
    level = np.array([l for l, _ in leaves], dtype=np.int32)
    anchor = np.zeros((len(leaves), 3), dtype=np.int64)
    for b, (_, a) in enumerate(leaves):
        anchor[b, :D] = a
    nvars = fs.nvars
    sigma = np.ones((nvars, 3), dtype=np.int32)
    if fs.parities is not None:
        for v, par in enumerate(fs.parities):
            for d in range(D):
                sigma[v, d] = -1 if par[d] == "OddParity" else 1
    m.nblocks, m.nvars = len(leaves), nvars
    m.level, m.anchor, m.sigma = level.ctypes.data, anchor.ctypes.data, sigma.ctypes.data
    wtab = lagrange_table(p, T)
    out = np.empty_like(data)
    rc = lib().pw_fill(C.byref(m), T.itemsize, wtab.ctypes.data, data.ctypes.data,
                       out.ctypes.data, nthreads or os.cpu_count() or 1)
    if rc != 0:
        raise RuntimeError(f"pw_fill failed ({rc})")
    return out
