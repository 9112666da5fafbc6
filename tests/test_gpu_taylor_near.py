"""The plain search evaluates points within 1e-6 of a point it has just evaluated (a
root's two sign-change check points, a Newton step of at most 1e-6) from that point's
T, T', T'' by their Taylor polynomials instead of assembling them.  Here the premise:
on the bench scatterer (circle N = 50, order 11, c_i = 23.4) near a sharp resonance,
the Taylor matrices equal the assembled T(k + h), T'(k + h) to 1e-13 / 1e-11 relative
for |h| <= 1e-6, and sigma, sigma' from them agree with the assembled ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("k", [5.2339513479, 1.9305983898])
def test_taylor_matrices_match_assembly(k):
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    T, T1, T2 = so.gen_sol_op_2nd_der(k, 1.0, 23.4)
    for h in (-1e-6, -2e-8, 1e-8, 3e-7, 1e-6):
        A, A1 = so.gen_sol_op_1st_der(k + h, 1.0, 23.4)
        Tt = T + h * (T1 + 0.5 * h * T2)
        T1t = T1 + h * T2
        assert rel(Tt, A) <= 1e-13, h
        assert rel(T1t, A1) <= 1e-11, h
        got = api.sv_dense([[Tt, T1t]], d=1)[0]
        ref = api.sv_dense([[A, A1]], d=1)[0]
        assert abs(got[0] - ref[0]) <= 1e-12 * ref[0] + 1e-15
        assert abs(got[1] - ref[1]) <= 1e-9 * max(1.0, abs(ref[1]))
