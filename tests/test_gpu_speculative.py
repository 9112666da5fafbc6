"""The plain search's Newton rounds with speculative bisection points against the
same search without them: the same roots, the same grid, the same evaluation
count (speculation only changes which round a value is computed in)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry, _capi as C  # noqa: E402
from helmholtzbem_gb300._capi import check  # noqa: E402


def _both(so, *args, **kw):
    check(C.lib().hbem_set_option(b"plain_speculate", 1))
    fast = so.find_resonances_plain(*args, **kw)
    check(C.lib().hbem_set_option(b"plain_speculate", 0))
    try:
        slow = so.find_resonances_plain(*args, **kw)
    finally:
        check(C.lib().hbem_set_option(b"plain_speculate", 1))
    return fast, slow


@pytest.mark.parametrize("N,c_i,npoints", [(50, 23.4, 200), (40, 9.0, 120), (24, 23.4, 64)])
def test_speculative_newton_matches_plain_rounds(N, c_i, npoints):
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, N), order=11))
    (r1, g1, n1), (r0, g0, n0) = _both(so, 0.5, 10.0, npoints, 1.0, c_i, tol=1e-8)
    assert r0.size > 0
    assert r1.size == r0.size
    # sigma at a wavenumber does not depend on the batch it was computed in, so each
    # candidate's iterates agree (to rounding of the batched evaluation)
    assert np.max(np.abs(r1 - r0)) <= 1e-10
    assert n1 == n0
    assert np.array_equal(np.isnan(g1), np.isnan(g0))
    assert np.max(np.abs(g1[:, 0] - g0[:, 0]) / g0[:, 0]) <= 1e-13
    ends = ~np.isnan(g0[:, 1])
    assert np.max(np.abs(g1[ends, 1] - g0[ends, 1])) <= 1e-10 * max(1.0, np.max(np.abs(g0[ends, 1])))


def test_plain_search_repeats():
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 30), order=9))
    a = so.find_resonances_plain(0.5, 8.0, 96, 1.0, 23.4, tol=1e-8)
    b = so.find_resonances_plain(0.5, 8.0, 96, 1.0, 23.4, tol=1e-8)
    assert np.array_equal(a[0], b[0]) and a[2] == b[2] and np.array_equal(a[1], b[1], equal_nan=True)


@pytest.mark.parametrize("N,c_i,npoints", [(50, 23.4, 200), (36, 9.0, 96)])
def test_warm_started_jacobi_matches_cold(N, c_i, npoints):
    """Bracket ends and Newton points start the dense kernel's FP32 Jacobi from the
    V set of the nearest evaluated wavenumber: the same roots (the FP64 refinement
    after the Jacobi stage sets the accuracy, not the start)."""
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, N), order=11))
    check(C.lib().hbem_set_option(b"plain_warm_start", 1))
    r1, g1, n1 = so.find_resonances_plain(0.5, 10.0, npoints, 1.0, c_i, tol=1e-8)
    check(C.lib().hbem_set_option(b"plain_warm_start", 0))
    try:
        r0, g0, n0 = so.find_resonances_plain(0.5, 10.0, npoints, 1.0, c_i, tol=1e-8)
    finally:
        check(C.lib().hbem_set_option(b"plain_warm_start", 1))
    assert r0.size > 0 and r1.size == r0.size and n1 == n0
    assert np.max(np.abs(r1 - r0)) <= 1e-10
    assert np.max(np.abs(g1[:, 0] - g0[:, 0]) / g0[:, 0]) <= 1e-12
    ends = ~np.isnan(g0[:, 1])
    assert np.max(np.abs(g1[ends, 1] - g0[ends, 1])) <= 1e-9 * max(1.0, np.max(np.abs(g0[ends, 1])))


def test_batched_plain_search_with_speculation_matches_plain_rounds():
    """The plain search over several scatterers in lock step (speculative bisection
    points in the late rounds) against the same search without speculation."""
    from helmholtzbem_gb300 import learned as L
    cases = [L.draw(s) for s in (20101, 20102, 20103, 20104)]
    ops = [L.operator(a, b) for (a, b, _, _) in cases]
    lo = [c[3] for c in cases]
    hi = [c[3] + 2.0 for c in cases]
    ci = [c[2] for c in cases]
    check(C.lib().hbem_set_option(b"plain_speculate", 1))
    r1, n1 = api.find_resonances_plain_multi(ops, lo, hi, 96, 1.0, ci, tol=1e-8)
    check(C.lib().hbem_set_option(b"plain_speculate", 0))
    try:
        r0, n0 = api.find_resonances_plain_multi(ops, lo, hi, 96, 1.0, ci, tol=1e-8)
    finally:
        check(C.lib().hbem_set_option(b"plain_speculate", 1))
    assert n1 == n0 and sum(len(r) for r in r0) > 0
    for a, b in zip(r1, r0):
        assert len(a) == len(b)
        if len(a):
            assert np.max(np.abs(np.asarray(a) - np.asarray(b))) <= 1e-10


def test_async_newton_matches_lock_step():
    """The plain search's Newton phase with every candidate on its own stream (the
    default) against the lock-step rounds: the same roots to 1e-10 and the same number
    of evaluations, on the bench workload (circle N = 50, order 11, 200 points)."""
    from helmholtzbem_gb300 import _capi as C, api, geometry
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    a_roots, a_grid, a_nev = so.find_resonances_plain(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)
    C.check(C.lib().hbem_set_option(b"plain_async", 0))
    try:
        l_roots, l_grid, l_nev = so.find_resonances_plain(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)
    finally:
        C.check(C.lib().hbem_set_option(b"plain_async", 1))
    assert a_roots.size == l_roots.size == 10
    assert np.max(np.abs(np.sort(a_roots) - np.sort(l_roots))) <= 1e-10
    assert a_nev == l_nev
    np.testing.assert_array_equal(a_grid[:, 0], l_grid[:, 0])


def test_verified_search_checks_every_root():
    """hbem_find_resonances_plain_verified: the roots of the plain search, each with
    sigma' at root -/+ tol -- evaluated beside the other candidates' iterations with
    the candidates on their own streams, in one batch after the search in lock step --
    equal to the separate evaluation to the dense kernel's accuracy, with the sign
    change of every root of the bench workload."""
    from helmholtzbem_gb300 import _capi as C, api, geometry
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    plain, _, nev = so.find_resonances_plain(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)
    for async_on in (1, 0):
        C.check(C.lib().hbem_set_option(b"plain_async", async_on))
        try:
            roots, _, nev2, chk = so.find_resonances_plain_verified(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)
        finally:
            C.check(C.lib().hbem_set_option(b"plain_async", 1))
        assert roots.size == plain.size == 10 and nev2 == nev
        assert np.max(np.abs(np.sort(roots) - np.sort(plain))) <= 1e-10
        assert np.all(chk[:, 0] <= 0) and np.all(chk[:, 1] >= 0)
        sep = np.stack([so.sweep_sigma(roots - 1e-8, 1.0, 23.4, d=1)[:, 1],
                        so.sweep_sigma(roots + 1e-8, 1.0, 23.4, d=1)[:, 1]], axis=1)
        assert np.max(np.abs(chk - sep)) <= 1e-10   # sigma' there is ~1e-7 .. 1e-6
