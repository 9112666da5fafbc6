"""Dense sigma_min, sigma', sigma'' by FP32 Jacobi + FP64 refinement of the near
singular triplets (the default for matrices up to order 100) against the oracle's
restatement of direct::sv_2nd_der and against the FP64-polished Jacobi kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _mats(kinds, par, order, ks, c_i):
    oso = O.SolutionsOperator(O.Builder(kinds, par, order))
    return [oso.gen_sol_op(k, 1.0, c_i, d=2) for k in ks]


def _check(out, refs):
    for o, ref in zip(out, refs):
        assert abs(o[0] - ref[0]) <= 1e-10 * ref[0]
        assert abs(o[1] - ref[1]) <= 1e-8 * max(abs(ref[1]), 1e-3)
        assert abs(o[2] - ref[2]) <= 1e-8 * max(abs(ref[2]), 1e-3)


@pytest.mark.parametrize("case", ["circle", "polygon"])
def test_fast_dense_sigma_vs_oracle(case):
    """circle N = 50 (T of order 100, the sweep's workload, with the circle's
    degenerate singular pairs) and a star polygon N = 48 at several wavenumbers,
    near and away from resonances."""
    if case == "circle":
        kinds, par = geometry.circle(0.25, 50)
        mats = _mats(kinds, par, 11, [0.9, 2.35, 4.07, 6.31, 8.8, 9.97], 23.4)
    else:
        kinds, par = geometry.polygon(*geometry.star_polygon(12, seed=7), 48)
        mats = _mats(kinds, par, 9, [1.0, 3.3, 5.5, 7.25], 9.0)
    refs = [O.sv_derivs(*m) for m in mats]
    C.check(C.lib().hbem_set_option(b"svd_fast", 1))
    fast = api.sv_dense(mats, d=2)
    _check(fast, refs)
    C.check(C.lib().hbem_set_option(b"svd_fast", 0))
    try:
        full = api.sv_dense(mats, d=2)
    finally:
        C.check(C.lib().hbem_set_option(b"svd_fast", 1))
    _check(full, refs)
    assert np.max(np.abs(fast[:, 0] - full[:, 0]) / full[:, 0]) < 1e-11


def test_fast_dense_sigma_orders_below_block():
    """n smaller than the near block's cap (n = 8) and n = 2."""
    kinds, par = geometry.circle(0.25, 4)
    mats = _mats(kinds, par, 5, [1.1, 2.2], 23.4)
    refs = [O.sv_derivs(*m) for m in mats]
    _check(api.sv_dense(mats, d=2), refs)
    rng = np.random.default_rng(4)
    T = [rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)) for _ in range(3)]
    ms = [[T[0], T[1], T[2]]]
    _check(api.sv_dense(ms, d=2), [O.sv_derivs(*ms[0])])
