"""The paired (two-CTA cluster) form of the dense sigma kernel against the one-CTA form.

Launches of at most `svd_pair_max` matrices run each matrix on a cluster of two CTAs:
the FP32 Jacobi and the FP64 LU run side by side, the inverse iterations and T X are
split by columns.  Every column goes through the one-CTA kernel's arithmetic in the
same order, so the two forms must agree bit for bit: here on single matrices and small
batches with first and second derivatives, with the kept singular vectors, and through
the plain resonance search (warm-started V pool, Newton lanes, bracket ends)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402


def _get(name):
    v = ctypes.c_int(-1)
    C.check(C.lib().hbem_get_option(name.encode(), ctypes.byref(v)))
    return v.value


def _with_pair_max(m, fn):
    old = _get("svd_pair_max")
    C.check(C.lib().hbem_set_option(b"svd_pair_max", m))
    try:
        return fn()
    finally:
        C.check(C.lib().hbem_set_option(b"svd_pair_max", old))


def test_option_round_trip_and_refusal():
    old = _get("svd_pair_max")
    assert old >= 1
    _with_pair_max(3, lambda: None)
    assert _get("svd_pair_max") == old
    with pytest.raises(C.HbemError):
        C.check(C.lib().hbem_set_option(b"svd_pair_max", -1))


def _mats(mesh, ks, c_o, c_i, d):
    so = api.SolutionsOperator(api.BuilderData(mesh, order=9))
    out = []
    for k in ks:
        if d == 2:
            out.append(list(so.gen_sol_op_2nd_der(k, c_o, c_i)))
        elif d == 1:
            out.append(list(so.gen_sol_op_1st_der(k, c_o, c_i)))
        else:
            out.append([so.gen_sol_op(k, c_o, c_i)])
    return out


@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("nmat", [1, 3])
def test_paired_equals_single_cta(d, nmat):
    ks = np.linspace(2.1, 6.3, nmat)
    cases = [(geometry.circle(0.25, 50), 1.0, 23.4),              # degenerate pairs (circle)
             (geometry.polygon(*geometry.star_polygon(9, seed=3), 41), 1.0, 4.0)]
    for mesh, c_o, c_i in cases:
        Ts = _mats(mesh, ks, c_o, c_i, d)
        single = _with_pair_max(0, lambda: api.sv_dense(Ts, d=d))
        paired = _with_pair_max(16, lambda: api.sv_dense(Ts, d=d))
        np.testing.assert_array_equal(paired, single)
        assert np.all(np.isfinite(paired[:, :d + 1]))


def test_paired_small_odd_orders():
    # kb = min(n, 12) columns split 6 + 6 for n >= 12, unevenly for odd kb below
    rng = np.random.default_rng(5)
    for n in (3, 5, 11, 13):
        Ts = []
        for _ in range(2):
            A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
            B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
            Ts.append([A, B, 0.5 * B @ B])
        single = _with_pair_max(0, lambda: api.sv_dense(Ts, d=2))
        paired = _with_pair_max(16, lambda: api.sv_dense(Ts, d=2))
        np.testing.assert_array_equal(paired, single)


def test_plain_search_identical_with_and_without_pairs():
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))

    def run():
        return so.find_resonances_plain_verified(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)

    a = _with_pair_max(0, run)
    b = _with_pair_max(16, run)
    assert a[0].size == 10
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]
    np.testing.assert_array_equal(a[3], b[3])
