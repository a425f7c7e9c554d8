"""The schedule checked by a second, independent oracle (``oracle/pointwise``).

The oracle's replay (``fill_oracle.c``) runs the product's own
``GhostSchedule``; so does the GPU.  Here the meshes are rebuilt from their
construction rules without the product's forest code, and every ghost is
derived point by point from the forest's geometry (covering leaf, level
difference, window, weights from exact rationals, mirror and clamp images,
the primary copy of a shared vertex point), with no schedule at all.

- The rebuilt leaf sets equal the product's, at the benchmark's sizes, and
  the product's leaf order is the reference's curve order.
- The point-by-point fill equals the schedule replay bit for bit on the
  quadrant mesh and on the sphere, walls and batch meshes at reduced size
  (the GPU fill is compared with the point-by-point one at full size in
  ``test_fullsize.py``), and on 1-D to 3-D layouts, cell- and vertex-centred,
  periodic or with reflecting and outflow walls, orders 2, 4 and 6, ghost
  widths 1 to 3; and on 40 seeded random layouts (each dimension periodic
  or walled, either kind of wall on either side, random parities, Float32
  or Float64), whose leaves the oracle also rebuilds.
- A wrong order or a wrong parity is caught."""
import numpy as np
import pytest

import oracle
from _helpers import nanbits
from oracle import pointwise as pw
from treeamr import FieldSet, Operators, meshes
from treeamr.schedule import GhostSchedule
from treeamr.storage import vertexcentered


# ---- the meshes' construction rules, restated --------------------------------

def _meets_sphere(box, centre=(0.5, 0.5, 0.5), r=0.25):
    """The box meets the sphere: the nearest point of the box inside it and
    the farthest outside."""
    near2 = far2 = 0.0
    for (a, b), c in zip(box, centre):
        n = min(max(c, a), b)
        near2 += (n - c) ** 2
        far2 += max((a - c) ** 2, (b - c) ** 2)
    return near2 <= r * r <= far2


def _near(points):
    """The box contains one of the points or lies within one box width of it."""
    def pred(box):
        w = box[0][1] - box[0][0]
        return any(all(a - w <= q[d] <= b + w for d, (a, b) in enumerate(box)) for q in points)
    return pred


def sphere_leaves(roots=8, N=16, levels=3):
    brick = pw.Brick((roots,) * 3, N, (True,) * 3, ((0.0, 1.0),) * 3)
    return pw.rebuild_forest(brick, [(l, _meets_sphere) for l in range(levels)])


def walls_leaves(roots=8, N=32, levels=5):
    brick = pw.Brick((roots,) * 3, N, (False,) * 3, ((0.0, 1.0),) * 3)
    return pw.rebuild_forest(brick, [(l, _near(meshes.walls_points())) for l in range(levels)])


def batch_leaves(roots, N, levels, pts):
    brick = pw.Brick(roots, N, (True,) * 3, tuple((0.0, float(r)) for r in roots))
    return pw.rebuild_forest(brick, [(l, _near(pts)) for l in range(levels)])


def quadrant_leaves(seed=0):
    """4x4 periodic roots, a seeded quarter of them (in root order, dimension
    1 fastest) refined once, then balanced."""
    rng = np.random.default_rng(seed)
    roots = [(0, (i % 4, i // 4)) for i in range(16)]
    pick = set(int(i) for i in rng.choice(16, size=4, replace=False))
    brick = pw.Brick((4, 4), 8, (True, True), ((0.0, 4.0), (0.0, 4.0)))
    leaves = set(roots)
    for i in pick:
        pw._refine(leaves, roots[i], 2)
    return pw.balance(leaves, brick)


def _same_forest(f, leaves):
    mine = pw.leaves_of(f)
    assert set(mine) == leaves
    assert mine == sorted(mine, key=lambda k: pw.morton_key(k, f.roots))


def test_rebuilt_forests_equal_the_product_forests():
    _same_forest(meshes.quadrant_forest(), quadrant_leaves())
    _same_forest(meshes.sphere_forest(), sphere_leaves())
    _same_forest(meshes.walls_forest(), walls_leaves())
    for spec in meshes.forest_batch_specs():
        _same_forest(meshes.batch_forest(*spec), batch_leaves(*spec))


def test_lagrange_table_reproduces_cubics():
    """Every row of the order-4 table reproduces 1, x, x^2 and x^3 at its
    quarter offset to rounding, and rows at whole offsets are unit vectors."""
    for T in (np.float64, np.float32):
        W = pw.lagrange_table(4, T).astype(np.float64)
        for k in range(W.shape[0]):
            x = k / 4
            for e in range(4):
                assert abs(sum(W[k, m] * m ** e for m in range(4)) - x ** e) < 1e-5
            if k % 4 == 0:
                assert W[k].tolist() == [1.0 if m == k // 4 else 0.0 for m in range(4)]
    assert pw.round_f32(pw.Fraction(1, 3)) == float(np.float32(1 / 3))


# ---- the point-by-point fill against the schedule replay ---------------------

def _compare(fs, p, seed=5, ops=None):
    meshes.random_fill(fs, seed=seed)
    data = fs.work.numpy().copy()
    s = GhostSchedule(fs, ops or Operators(prolongation=p, restriction=p))
    replay = oracle.fill(s, data.copy(), fs.nvars, fs.factors_host, nthreads=8)
    point = pw.fill(fs, data, p)
    return int(np.count_nonzero(nanbits(point) != nanbits(replay)))


def test_quadrant_pointwise_equals_replay():
    f, fs, ops = meshes.quadrant_setup()
    assert _compare(fs, 4) == 0


@pytest.mark.parametrize("p", [4, 6])
def test_sphere_pointwise_equals_replay(p):
    f = meshes.sphere_forest(roots=4, N=16, levels=2)
    assert _compare(FieldSet(f, 2, G=3, T=np.float64), p) == 0


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_walls_pointwise_equals_replay(T):
    f = meshes.walls_forest(roots=4, N=16, levels=3)
    fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=meshes.walls_parities(), T=T)
    assert _compare(fs, 4) == 0


def test_batch_members_pointwise_equal_replay():
    for spec in meshes.forest_batch_specs()[:6]:
        fs = FieldSet(meshes.batch_forest(*spec), 2, G=2, T=np.float32)
        assert _compare(fs, 4) == 0, spec


def test_pointwise_comparison_catches_mistakes():
    """The comparison is not vacuous: a fill with another restriction order,
    or with the parities of the variables swapped, differs."""
    f = meshes.sphere_forest(roots=4, N=16, levels=2)
    fs = FieldSet(f, 1, G=3, T=np.float64)
    assert _compare(fs, 4, ops=Operators(prolongation=4, restriction=2)) > 0
    f = meshes.walls_forest(roots=4, N=16, levels=3)
    good = meshes.walls_parities()
    fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=good)
    meshes.random_fill(fs, seed=2)
    data = fs.work.numpy().copy()
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    replay = oracle.fill(s, data.copy(), 8, fs.factors_host, nthreads=8)
    bad = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=good[::-1])
    assert np.count_nonzero(nanbits(pw.fill(bad, data, 4)) != nanbits(replay)) > 0


# ---- more layouts: 1-D to 3-D, cell and vertex, walls, orders 2 to 6 ---------

def _layout(D, vertex, walls, N, G, levels, nvars=2):
    """A brick of 4 roots a side over the unit box, periodic, or with
    reflecting low and outflow high faces; ``levels`` passes refining the
    leaves within a box width of a point off the centre, each balanced.  With
    walls, variable 2 is odd in dimension 1."""
    from treeamr import Forest, EvenParity, OddParity
    kw = dict(N=N, extents=((0.0, 1.0),) * D)
    if walls:
        kw.update(reflecting=((True, False),) * D, outflow=((False, True),) * D)
    else:
        kw.update(periodic=(True,) * D)
    f = Forest((4,) * D, **kw)
    meshes.refine_where(f, _near([(0.3, 0.6, 0.45)[:D]]), range(levels))  # as rebuilt below
    parity = None
    if walls:
        parity = [(EvenParity,) * D,
                  tuple(OddParity if d == 0 else EvenParity for d in range(D))][:nvars]
    centering = vertexcentered(D) if vertex else None
    return FieldSet(f, nvars, G=G, centering=centering, parity=parity, T=np.float64)


LAYOUTS = [
    # D, vertex, walls, N, G, levels, p
    (1, False, False, 8, 2, 3, 4),
    (1, False, True, 8, 3, 3, 6),
    (1, True, False, 8, 2, 3, 4),
    (1, True, True, 16, 2, 3, 2),
    (2, False, True, 8, 2, 2, 4),
    (2, False, False, 8, 1, 2, 2),
    (2, True, True, 8, 2, 2, 4),
    (2, True, False, 16, 3, 2, 6),
    (3, False, True, 8, 2, 2, 4),
    (3, True, False, 8, 1, 2, 2),
    (3, True, True, 8, 3, 2, 6),
    (3, False, False, 8, 2, 3, 4),
    (2, False, True, 16, 3, 3, 6),
    (2, True, True, 8, 1, 3, 4),
    (1, False, False, 16, 1, 4, 2),
    (1, True, True, 8, 3, 4, 6),
]


@pytest.mark.parametrize("D,vertex,walls,N,G,levels,p", LAYOUTS)
def test_more_layouts_pointwise_equal_replay(D, vertex, walls, N, G, levels, p):
    """The schedule of each layout, replayed, equals the point-by-point fill
    derived from the forest's geometry, bit for bit."""
    fs = _layout(D, vertex, walls, N, G, levels)
    assert fs.forest.nleaves() > 4 ** D  # refined somewhere
    brick = pw.Brick((4,) * D, N, (not walls,) * D, ((0.0, 1.0),) * D)
    point = (0.3, 0.6, 0.45)[:D]
    _same_forest(fs.forest, pw.rebuild_forest(brick, [(l, _near([point]))
                                                      for l in range(levels)]))
    assert _compare(fs, p) == 0


def _random_layout(rng, dtype=None):
    """A seeded layout: 1 to 3 dimensions, cell or vertex, each dimension
    periodic or walled (reflecting or outflow on each side), N 8 or 16, an
    order of 2, 4 or 6 with the least ghost width it allows (or one more),
    one to three levels around two random points, random parities."""
    from treeamr import Forest, EvenParity, OddParity
    D = int(rng.integers(1, 4))
    vertex = bool(rng.integers(2))
    N = int(rng.choice([8, 16]))
    p = int(rng.choice([2, 4, 6]))
    periodic = tuple(bool(rng.integers(2)) for _ in range(D))
    kinds = [tuple(int(rng.integers(2)) for _ in range(2)) for _ in range(D)]
    reflecting = tuple((k[0] == 0 and not periodic[d], k[1] == 0 and not periodic[d])
                       for d, k in enumerate(kinds))
    outflow = tuple((k[0] == 1 and not periodic[d], k[1] == 1 and not periodic[d])
                    for d, k in enumerate(kinds))
    G = (max(1, p // 2 - 1) if vertex else p // 2) + int(rng.integers(2))
    from treeamr.operators import check_operators
    try:  # a layout the reference refuses (N too small for G and the order)
        check_operators(N, (G,) * D, (int(vertex),) * D, Operators(prolongation=p, restriction=p))
    except ValueError:
        N = 16
    levels = int(rng.integers(1, 4 if D < 3 else 3))
    points = [tuple(float(x) for x in rng.uniform(0.05, 0.95, size=D)) for _ in range(2)]
    f = Forest((4,) * D, N=N, periodic=periodic, reflecting=reflecting, outflow=outflow,
               extents=((0.0, 1.0),) * D)
    meshes.refine_where(f, _near(points), range(levels))
    nvars = 3
    parity = [tuple(OddParity if rng.integers(2) else EvenParity for _ in range(D))
              for _ in range(nvars)]
    fs = FieldSet(f, nvars, G=G, centering=vertexcentered(D) if vertex else None,
                  parity=parity, T=np.float64 if rng.integers(2) else np.float32)
    if dtype is not None:  # the same layout in another element type
        fs = FieldSet(f, nvars, G=G, centering=vertexcentered(D) if vertex else None,
                      parity=parity, T=dtype)
    brick = pw.Brick((4,) * D, N, periodic, ((0.0, 1.0),) * D)
    return fs, p, brick, [(l, _near(points)) for l in range(levels)]


@pytest.mark.parametrize("seed", range(40))
def test_random_layouts_pointwise_equal_replay(seed):
    """Seeded random layouts: the leaves rebuilt independently equal the
    product's, and the schedule replay equals the point-by-point fill bit for
    bit."""
    fs, p, brick, passes = _random_layout(np.random.default_rng(1000 + seed))
    _same_forest(fs.forest, pw.rebuild_forest(brick, passes))
    assert _compare(fs, p, seed=seed) == 0
