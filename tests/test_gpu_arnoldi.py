"""arnoldi::sv / sv_1st_der / sv_2nd_der on the GPU (block iteration, one CTA per
matrix or the batched global-memory LU) against the oracle: the ARPACK call of the
reference, the dense SVD and the perturbation-theory derivatives, plus the block
iteration's own iteration counts."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402
from helmholtzbem_gb300._capi import HbemError, check  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _circle(ks, npan=50, order=11, d=0):
    kinds, par = geometry.circle(0.25, npan)
    oso = O.SolutionsOperator(O.Builder(kinds, par, order))
    return [oso.gen_sol_op(k, 1.0, 23.4, d=d) for k in ks]


def _star(ks, npan, d, order=7):
    so = api.SolutionsOperator(api.BuilderData(geometry.polygon(*geometry.star_polygon(9, seed=5), npan), order=order))
    return [list(so._gen(k, 1.0, 9.0, d)) for k in ks]


def _device(Ts, d):
    nmat, n = len(Ts), Ts[0][0].shape[0]
    buf = np.zeros((nmat, d + 1, n, n), np.complex128)
    for m, mats in enumerate(Ts):
        for t in range(d + 1):
            buf[m, t] = np.asarray(mats[t]).T
    return torch.from_numpy(buf).cuda(), n, nmat


def _run_device(Ts, count, acc, d=0):
    X, n, nmat = _device(Ts, d)
    out = np.zeros((nmat, count, d + 1))
    status = (ctypes.c_int * nmat)()
    iters = (ctypes.c_int * nmat)()
    rc = C.lib().hbem_arnoldi_sv_batch_device(n, nmat, d, count, acc, ctypes.c_void_p(X.data_ptr()),
                                              (d + 1) * n * n, n * n, out.ctypes.data_as(C._dp), status, iters)
    return rc, out, list(status), list(iters)


@pytest.mark.parametrize("count", [1, 3])
def test_values_match_arpack_and_dense_small_path(count):
    ks = [1.1, 2.7, 4.05, 6.3, 9.7]
    mats = _circle(ks)
    rc, out, status, iters = _run_device(mats, count, 1e-12)
    check(rc)
    assert status == [0] * len(ks)
    for m, T in enumerate(mats):
        sv = np.sort(np.linalg.svd(T[0], compute_uv=False))[:count]
        arp = O.arnoldi_sv_arpack(T[0], count, 1e-12)
        got = out[m, :, 0]
        assert np.max(np.abs(got - sv)) <= 1e-11 * sv[-1]
        assert np.max(np.abs(got - arp)) <= 1e-11 * sv[-1]
        # same start block, same stopping test: the restated iteration stops within one step
        _, _, it_o, conv_o = O.arnoldi_block(T[0], count, 1e-12)
        assert conv_o and abs(iters[m] - it_o) <= 1


def test_derivatives_match_perturbation_theory():
    """Non-degenerate spectrum (star polygon): sigma_j' = Re u_j^H T' v_j and the
    bordered-system sigma_j'' against the dense perturbation formulas, j = 0, 1."""
    ks = [2.3, 3.9]
    mats = _star(ks, 40, d=2)
    rc, out, status, _ = _run_device(mats, 2, 1e-13, d=2)
    check(rc)
    for m, (T, T1, T2) in enumerate(mats):
        for j in range(2):
            ref = O.sv_derivs(T, T1, T2, which=j)
            assert abs(out[m, j, 0] - ref[0]) <= 1e-12 * ref[0] * 10
            assert abs(out[m, j, 1] - ref[1]) <= 1e-8 * max(abs(ref[1]), 1.0)
            assert abs(out[m, j, 2] - ref[2]) <= 1e-6 * max(abs(ref[2]), 1.0)


def test_global_path_matches_dense():
    """Order 240 (LU and blocks in global memory, lock-step iteration over the batch)."""
    ks = [3.1, 5.2, 7.7]
    mats = _star(ks, 120, d=1)
    rc, out, status, iters = _run_device(mats, 4, 1e-12, d=1)
    check(rc)
    assert status == [0] * 3 and min(iters) >= 1
    for m, (T, T1) in enumerate(mats):
        sv = np.sort(np.linalg.svd(T, compute_uv=False))[:4]
        assert np.max(np.abs(out[m, :, 0] - sv)) <= 1e-11 * sv[-1]
        ref = O.sv_derivs(T, T1, which=0)
        assert abs(out[m, 0, 1] - ref[1]) <= 1e-7 * max(abs(ref[1]), 1.0)


def test_batch_equals_single_calls():
    mats = _circle([2.7, 6.3, 9.7])
    _, out, _, it = _run_device(mats, 2, 1e-10)
    for m in range(3):
        _, o1, _, i1 = _run_device([mats[m]], 2, 1e-10)
        assert np.array_equal(o1[0], out[m]) and i1[0] == it[m]
    big = _star([3.1, 7.7], 120, d=0)
    _, out, _, it = _run_device(big, 2, 1e-10)
    for m in range(2):
        _, o1, _, i1 = _run_device([big[m]], 2, 1e-10)
        assert np.array_equal(o1[0], out[m]) and i1[0] == it[m]


def test_singular_and_iteration_cap_reported():
    mats = _circle([2.7, 4.05])
    T = mats[1][0].copy()
    T[:, 7] = 0.0
    rc, out, status, _ = _run_device([mats[0], [T]], 1, 1e-12)
    assert rc == 5                                          # HBEM_ERR_SINGULAR
    assert status == [0, 5] and np.isnan(out[1, 0, 0])
    assert abs(out[0, 0, 0] - np.linalg.svd(mats[0][0], compute_uv=False).min()) <= 1e-11
    check(C.lib().hbem_set_option(b"arnoldi_maxit", 1))
    try:
        rc, out, status, iters = _run_device(mats, 1, 1e-14)
    finally:
        check(C.lib().hbem_set_option(b"arnoldi_maxit", 1000))
    assert rc == 4 and status == [6, 6] and iters == [1, 1]  # HBEM_ERR_NOCONV, last iterate kept
    assert np.all(np.isfinite(out))


def test_many_values_take_the_dense_route():
    mats = _circle([4.05], npan=30, order=7)
    n = mats[0][0].shape[0]
    count = n - 1            # sv_circle_arnoldi: all but the largest singular value
    got = api.arnoldi_sv(mats, count, 1e-10, d=0)
    sv = np.sort(np.linalg.svd(mats[0][0], compute_uv=False))[:count]
    assert np.max(np.abs(got[0, :, 0] - sv)) <= 1e-12 * sv[-1] * 10
    with pytest.raises(HbemError):
        api.arnoldi_sv([[mats[0][0], mats[0][0]]], count, 1e-10, d=1)
