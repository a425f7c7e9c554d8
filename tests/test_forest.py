"""The tree: curve order, neighbours, balance (``test/tree_tests.jl``,
``test/oracles.jl:232-341``)."""
import itertools
import random

import pytest

from treeamr import Forest, MortonKey, alldirections, curve_key, sortedchildkeys


def bitplane_less(a: MortonKey, b: MortonKey) -> bool:
    """The naive bit-plane comparison of ``test/oracles.jl:232``."""
    if a.root != b.root:
        return a.root < b.root
    D = len(a.coords)
    for bit in range(31, -1, -1):
        for d in range(D):
            x = (a.coords[d] << (32 - a.level)) >> bit & 1
            y = (b.coords[d] << (32 - b.level)) >> bit & 1
            if x != y:
                return x < y
    return a.level < b.level


def test_curve_order_matches_bitplanes():
    rng = random.Random(3)
    keys = []
    for _ in range(300):
        D = 3
        lvl = rng.randint(0, 5)
        keys.append(MortonKey(rng.randint(0, 2), lvl, tuple(rng.randrange(1 << lvl) for _ in range(D))))
    for a, b in itertools.combinations(keys, 2):
        if a == b:
            continue
        assert (curve_key(a) < curve_key(b)) == bitplane_less(a, b)


def test_children_sorted():
    k = MortonKey(0, 2, (1, 2, 3))
    ch = sortedchildkeys(k)
    assert ch == sorted(ch, key=curve_key)


def test_alldirections_order():
    dirs = alldirections(2)
    assert dirs == [(-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1)]
    assert len(alldirections(3)) == 26


def test_neighbors_and_balance():
    f = Forest((2, 2), N=4, periodic=(True, True))
    assert f.nleaves() == 4
    k = f.leaves[0]
    # a lone periodic root in 1-D is its own neighbour
    g = Forest((1,), N=4, periodic=(True,))
    assert g.oriented_neighbors(g.leaves[0], (1,)) == [g.leaves[0]]
    # refining then balancing keeps 2:1
    f.refine(k)
    f.refine(f.leaves[0])
    assert not f.isbalanced()
    f.balance()
    assert f.isbalanced()
    # a finer neighbour across a face is 2^(D-1) leaves
    for b, leaf in enumerate(f.leaves):
        for d in alldirections(2):
            nb = f.oriented_neighbors(leaf, d)
            if nb and nb[0].level > leaf.level:
                assert len(nb) == 2 ** (2 - sum(1 for x in d if x))


def test_nonperiodic_face_has_no_neighbor():
    f = Forest((2,), N=4)
    assert f.oriented_neighbors(f.leaves[0], (-1,)) == []
    assert f.oriented_neighbors(f.leaves[0], (1,)) == [f.leaves[1]]


def test_wall_direction():
    f = Forest((2, 2), N=4, reflecting=((True, False), (False, False)),
               outflow=((False, True), (False, False)))
    k = f.leaves[0]                 # root (0, 0)
    dprime, walls = f.wall_direction(k, (-1, -1))
    assert dprime == (0, -1) and walls[0] == 1
    with pytest.raises(ValueError):
        Forest((2,), N=4, periodic=(True,), reflecting=((True, False),))
