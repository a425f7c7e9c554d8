"""The full-size property checks (``tests/_props.py``) on reduced meshes of the
same construction, with the oracle's fill on the host: the sphere mesh at
4^3 roots and 2 levels, the walls mesh at 4^3 roots, N=16 and 3 levels."""
import numpy as np

from _props import sphere_polynomial_error, walls_properties
from treeamr import FieldSet, GhostSchedule, Operators, meshes
from treeamr.storage import vertexcentered


def test_sphere_polynomial_exact_oracle():
    f = meshes.sphere_forest(roots=4, N=16, levels=2)
    fs = FieldSet(f, 2, G=3, T=np.float64)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    worst, scale = sphere_polynomial_error(fs, sched, "oracle")
    assert worst <= 1e-10 * scale, (worst, scale)


def test_walls_polynomial_and_outflow_oracle():
    f = meshes.walls_forest(roots=4, N=16, levels=3)
    assert max(k.level for k in f.leaves) == 3
    fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=meshes.walls_parities(),
                  T=np.float64)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    worst, scale, bad = walls_properties(fs, sched, "oracle", margin=1.0 / 16)
    assert worst <= 1e-10 * scale, (worst, scale)
    assert bad == 0
