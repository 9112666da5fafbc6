"""Assembly launches of few wavenumbers split each coincident / adjacent panel pair
over several CTAs (k_singular_part + k_singular_join; option "singular_split").  The
split changes only the order of the quadrature sums: T, T', T'' agree with the
one-CTA-per-pair launch to rounding (1e-14 relative Frobenius) and with the oracle's
GalerkinBuilder / gen_sol_op restatement at the usual 1e-12."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _split(on):
    C.check(C.lib().hbem_set_option(b"singular_split", on))


def test_option_round_trip():
    v = ctypes.c_int(-1)
    C.check(C.lib().hbem_get_option(b"singular_split", ctypes.byref(v)))
    assert v.value == 1


MESHES = {
    "circle": lambda: geometry.circle(0.25, 50),
    "polygon": lambda: geometry.polygon(*geometry.star_polygon(12, seed=5), 40),
}


@pytest.mark.parametrize("mesh", sorted(MESHES))
@pytest.mark.parametrize("k", [5.2339, 3.1 + 0.2j])
def test_split_matches_one_cta_per_pair_and_oracle(mesh, k):
    kinds, par = MESHES[mesh]()
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=11))
    try:
        _split(0)
        ref = so.gen_sol_op_2nd_der(k, 1.0, 23.4)
    finally:
        _split(1)
    got = so.gen_sol_op_2nd_der(k, 1.0, 23.4)
    for a, b in zip(got, ref):
        assert rel(a, b) <= 1e-14
    R = O.SolutionsOperator(O.Builder(kinds, par, 11)).gen_sol_op(k, 1.0, 23.4, d=2)
    for a, b in zip(got, R):
        assert rel(a, b) <= 1e-12


def test_split_batches_of_one_to_four_wavenumbers():
    # the split applies while pairs x jobs stay below four CTAs per SM
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    for nk in (1, 2, 3, 4):
        ks = np.linspace(2.0, 7.0, nk)
        try:
            _split(0)
            ref = so.sweep_sigma(ks, 1.0, 23.4, d=2)
        finally:
            _split(1)
        got = so.sweep_sigma(ks, 1.0, 23.4, d=2)
        np.testing.assert_allclose(got[:, 0], ref[:, 0], rtol=1e-12)
        np.testing.assert_allclose(got[:, 1], ref[:, 1], rtol=1e-9, atol=1e-12)
