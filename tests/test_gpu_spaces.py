"""Discontinuous P0 spaces on the GPU (DiscontinuousSpace<0>,
include/discontinuous_space.hpp:33-127) against the oracle's restatement of
GalerkinBuilder::assembleDense, including its non-square branch
(source/galerkin_builder.cpp:966-1009), at 1e-12 relative Frobenius.

The first three tests are the reference's own operator unit tests
(test/googletest/single_layer_test.cpp:22-73, double_layer_test.cpp,
hypersingular_test.cpp): circle r = 0.25 split into 50 arcs, Gauss order 11, k = 1,
c = 5, P0 test / P1 trial (P1 / P1 for the hypersingular operator).  Their golden
rows are not in the reference tree, so the row is checked against the oracle at the
reference's own tolerance (5e-4 in the 2-norm) and the whole matrix at 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402

P0, P1 = C.SPACE_P0, C.SPACE_P1


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _both(mesh, order, test, trial):
    kinds, par = mesh
    return (api.GalerkinBuilder(api.BuilderData(mesh, test, trial, order)),
            O.Builder(kinds, par, order, qtest=test, qtrial=trial))


@pytest.mark.parametrize("layer,name,test,trial", [
    (api.LayerType_SINGLE, "V", P0, P1),
    (api.LayerType_DOUBLE, "K", P0, P1),
    (api.LayerType_HYPERSINGULAR, "W", P1, P1)])
def test_reference_unit_test_configurations(layer, name, test, trial):
    gb, ob = _both(geometry.circle(0.25, 50), 11, test, trial)
    gb.assembleDense(1.0, 5.0, layer, 0)
    got = {"V": gb.getSingleLayer, "K": gb.getDoubleLayer, "W": gb.getHypersingular}[name](0)
    ref = ob.assemble(1.0, 5.0, {"V": O.LAYER_SINGLE, "K": O.LAYER_DOUBLE, "W": O.LAYER_HYPERSINGULAR}[name], 0)[name][0]
    assert got.shape == ref.shape == (50, 50)
    assert np.linalg.norm(got[0] - ref[0]) < 5e-4
    assert rel(got, ref) <= 1e-12


MESHES = {
    "circle": lambda: geometry.circle(0.25, 24),
    "polygon": lambda: geometry.polygon(*geometry.star_polygon(10, seed=4), 31),
}


@pytest.mark.parametrize("mesh", sorted(MESHES))
@pytest.mark.parametrize("spaces", [(P0, P1), (P1, P0), (P0, P0)])
@pytest.mark.parametrize("k", [2.3, 1.7 + 0.4j])
def test_all_layers_and_derivatives_vs_oracle(mesh, spaces, k):
    gb, ob = _both(MESHES[mesh](), 9, *spaces)
    gb.assembleDense(k, 4.0, api.LayerType_ALL, 2)
    ref = ob.assemble(k, 4.0, O.LAYER_ALL, 2)
    for t in range(3):
        assert rel(gb.getDoubleLayer(t), ref["K"][t]) <= 1e-12, ("K", t)
        assert rel(gb.getHypersingular(t), ref["W"][t]) <= 1e-12, ("W", t)
        assert rel(gb.getSingleLayer(t), ref["V"][t]) <= 1e-12, ("V", t)


@pytest.mark.parametrize("spaces", [(P0, P1), (P1, P0), (P0, P0)])
@pytest.mark.parametrize("layers", [api.LayerType_ALL, api.LayerType_SINGLE | api.LayerType_HYPERSINGULAR])
def test_submatrix_vs_oracle(spaces, layers):
    """The sub-matrix rule with P0 spaces, including the non-square double layer's
    ordered pairs and a block straddling the diagonal."""
    gb, ob = _both(geometry.polygon(*geometry.star_polygon(9, seed=6), 26), 7, *spaces)
    for row, col, rows, cols in [(3, 8, 9, 12), (10, 2, 6, 5), (0, 0, 26, 7)]:
        gb.assembleDense(2.9, 3.0, layers, 1, row, col, rows, cols)
        ref = ob.assemble(2.9, 3.0, layers, 1, row, col, rows, cols)
        for t in range(2):
            if layers & api.LayerType_DOUBLE:
                assert rel(gb.getDoubleLayer(t), ref["K"][t]) <= 1e-12
            assert rel(gb.getHypersingular(t), ref["W"][t]) <= 1e-12
            assert rel(gb.getSingleLayer(t), ref["V"][t]) <= 1e-12


@pytest.mark.parametrize("spaces,proj", [((P0, P1), False), ((P1, P0), False), ((P0, P0), True), ((P0, P0), False)])
def test_solutions_operator_with_p0_spaces(spaces, proj):
    mesh = geometry.circle(0.25, 20)
    data = api.BuilderData(mesh, spaces[0], spaces[1], 9)
    so = api.SolutionsOperator(data, proj=proj)
    oso = O.SolutionsOperator(O.Builder(*mesh, 9, qtest=spaces[0], qtrial=spaces[1]), proj=proj)
    np.testing.assert_allclose(so.mass_matrix(), oso.M, rtol=0, atol=1e-14 * np.abs(oso.M).max())
    T = so.gen_sol_op_2nd_der(3.1, 1.0, 6.0)
    R = oso.gen_sol_op(3.1, 1.0, 6.0, d=2)
    for a, b in zip(T, R):
        assert rel(a, b) <= 1e-12


def test_projection_refused_for_p0_x_p1():
    data = api.BuilderData(geometry.circle(0.25, 12), P0, P1, 7)
    with pytest.raises(C.HbemError) as e:
        api.SolutionsOperator(data, proj=True)
    assert e.value.status == 7 and "symmetric" in str(e.value)
