"""Known-answer tests of the operators (``test/ghost_tests.jl:5-99``)."""
from fractions import Fraction as F

import numpy as np
import pytest

from treeamr import Operators
from treeamr.operators import (conservative_prolong_weights, interpolation_weights,
                               lagrange_weights, round_weights)
from treeamr.forest import round_rational_f32


def test_both_orders_required():
    with pytest.raises(ValueError, match="no default order"):
        Operators()
    with pytest.raises(ValueError, match="restriction"):
        Operators(prolongation=2)
    with pytest.raises(ValueError):
        Operators(restriction=2)
    for bad in (dict(prolongation=1, restriction=2), dict(prolongation=3, restriction=2),
                dict(prolongation=2, restriction=0)):
        with pytest.raises(ValueError):
            Operators(**bad)
    assert repr(Operators(prolongation=2, restriction=2)) == \
        "Operators(prolongation=2, restriction=2, family=PointValue)"


@pytest.mark.parametrize("nodes", [[F(0), F(1)], [F(-1), F(0), F(1), F(2)],
                                   [F(3), F(4), F(5), F(6)]])
def test_lagrange_exact_for_polynomials(nodes):
    p = len(nodes)
    for deg in range(p):
        for x in (F(-1, 4), F(1, 2), F(5, 4), F(9, 2)):
            w = lagrange_weights(nodes, x)
            assert sum(w[i] * nodes[i] ** deg for i in range(p)) == x ** deg
            assert sum(w) == 1


def test_lagrange_known_answers():
    assert lagrange_weights([F(0), F(1)], F(3, 4)) == [F(1, 4), F(3, 4)]
    assert lagrange_weights([F(0), F(1)], F(1, 2)) == [F(1, 2), F(1, 2)]
    assert lagrange_weights([F(0), F(1), F(2), F(3)], F(3, 2)) == \
        [F(-1, 16), F(9, 16), F(9, 16), F(-1, 16)]
    assert list(interpolation_weights(1, 4, F(5, 2), "test")) == \
        [F(-1, 16), F(9, 16), F(9, 16), F(-1, 16)]
    assert list(interpolation_weights(1, 4, F(4), "test")) == [0, 0, 0, 1]
    with pytest.raises(ValueError):
        interpolation_weights(1, 4, F(9, 2), "test")
    with pytest.raises(ValueError):
        interpolation_weights(1, 4, F(1, 2), "test")


def test_conservative_family():
    ops = Operators(prolongation=3, restriction=2, family="Conservative")
    assert ops.family == "Conservative"
    with pytest.raises(ValueError):
        Operators(prolongation=2, restriction=2, family="Conservative")
    with pytest.raises(ValueError, match="exact volume average"):
        Operators(prolongation=3, restriction=4, family="Conservative")
    for p in (1, 3, 5):
        low, high = conservative_prolong_weights(p)
        assert len(low) == len(high) == p
        assert sum(low) == 1 and sum(high) == 1
        centre = [F(1) if t == (p - 1) // 2 else F(0) for t in range(p)]
        assert [(a + b) / 2 for a, b in zip(low, high)] == centre
    low, high = conservative_prolong_weights(3)
    assert list(low) == [F(1, 8), 1, F(-1, 8)]
    assert list(high) == [F(-1, 8), 1, F(1, 8)]
    assert conservative_prolong_weights(1) == ((F(1),), (F(1),))


def test_weights_round_once():
    # 1/3 and 1/10 rounded once, directly to each type
    w = round_weights([F(1, 3), F(1, 10), F(-7, 128)], np.float64)
    assert list(w) == [1 / 3, 0.1, -7 / 128]
    w32 = round_weights([F(1, 3), F(1, 10)], np.float32)
    assert w32.dtype == np.float32
    assert w32[0] == np.float32(1 / 3) and w32[1] == np.float32(0.1)
    # a rational whose float64 rounding sits on a float32 tie: one rounding
    # to float32 must not be the float64 one rounded again
    num = (1 << 25) + 1 + 1                      # 2^25 + 2 over 2^25: ...
    q = F((1 << 24) * 2 + 1, 1 << 25) + F(1, 1 << 60)
    direct = round_rational_f32(q.numerator, q.denominator)
    assert abs(F(float(direct)) - q) <= abs(F(float(np.float32(float(q)))) - q)
