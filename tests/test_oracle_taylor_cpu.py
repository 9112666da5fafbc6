"""The premise of the plain search's points near a point just evaluated (a Newton step
of at most 1e-6, a root's two check points at -/+ tol): T and T' there equal the
Taylor polynomials of T, T', T'' at the evaluated point,
    T(k + h) ~ T + h T' + h^2/2 T'',   T'(k + h) ~ T' + h T'',
to 1e-13 / 1e-11 relative for |h| <= 1e-6.  Checked with the oracle's restatement of
gen_sol_op_2nd_der (gen_sol_op.cpp) on the bench circle near its sharpest resonance
and on a star polygon of lines."""
import numpy as np
import pytest

from oracle import oracle as O


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _polygon():
    # a 7-point star polygon split into 28 lines (the oracle's own panel helper)
    t = np.linspace(0.0, 2.0 * np.pi, 8)[:-1]
    r = 0.25 * (1.0 + 0.3 * np.cos(3.0 * t))
    return O.polygon_panels(r * np.cos(t), r * np.sin(t), 28)


@pytest.mark.parametrize("case", ["circle", "polygon"])
def test_taylor_polynomials_match_the_oracles_operators(case):
    if case == "circle":
        kinds, par = O.circle_panels(0.25, 50)
        order, k, c_i = 11, 6.2386115757, 23.4
    else:
        kinds, par = _polygon()
        order, k, c_i = 9, 4.1, 9.0
    so = O.SolutionsOperator(O.Builder(kinds, par, order))
    T, T1, T2 = so.gen_sol_op(k, 1.0, c_i, d=2)
    for h in (-1e-6, 2e-8, 1e-6):
        A, A1 = so.gen_sol_op(k + h, 1.0, c_i, d=1)
        assert rel(T + h * (T1 + 0.5 * h * T2), A) <= 1e-13, h
        assert rel(T1 + h * T2, A1) <= 1e-11, h
