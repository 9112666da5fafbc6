"""Scatterer file -> corner-graded polygon mesh -> GPU operators, against the
oracle's assembly of the same panels (examples/roots_brent_polygon.cpp:72-121 and
examples/find_resonances.cpp:111-124 build their meshes this way)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("rf", [0.25, 0.5])
def test_graded_L_shape_operator_matches_oracle(tmp_path, rf):
    f = tmp_path / "L.dat"
    f.write_text("0,0\n2,0\n2,1\n1,1\n1,2\n0,2\n")
    x, y = geometry.read_scatterer(str(f), scale=0.5)
    kinds, par = geometry.polygon_graded(x, y, 60, rf)
    ok, opar = O.polygon_panels_graded(*O.read_scatterer(str(f), 0.5), 60, rf)
    assert np.array_equal(par, opar)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=9))
    oso = O.SolutionsOperator(O.Builder(kinds, par, 9))
    got = so.gen_sol_op_2nd_der(3.7, 1.0, 5.0)
    ref = oso.gen_sol_op(3.7, 1.0, 5.0, d=2)
    for a, b in zip(got, ref):
        assert rel(a, b) < 1e-12
    s = api.sv_dense([list(got)], d=2)[0]
    r = O.sv_derivs(*ref)
    assert abs(s[0] - r[0]) <= 1e-12 * r[0] * 10
    assert abs(s[1] - r[1]) <= 1e-8 * max(1.0, abs(r[1]))


def test_chosen_panel_count_mesh():
    x, y = geometry.star_polygon(9, seed=5)
    n = geometry.choose_num_panels(x, y, k_max=4.0, degf=10.0, rfac=0.5)
    kinds, par = geometry.polygon_graded(x, y, n, 0.5)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=7))
    oso = O.SolutionsOperator(O.Builder(kinds, par, 7))
    assert rel(so.gen_sol_op(2.2, 1.0, 9.0), oso.gen_sol_op(2.2, 1.0, 9.0)[0]) < 1e-12
