"""Batched LU with partial pivoting and its two solve forms (the Eigen::PartialPivLU
calls of randsvd.cpp) against numpy, through the C ABI on device buffers."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from helmholtzbem_gb300 import _capi as C  # noqa: E402
from helmholtzbem_gb300._capi import check  # noqa: E402


def _dev(mats):
    """list of n x n complex matrices -> (nmat, n, n) device tensor, each column-major."""
    a = np.stack([np.asarray(m).T for m in mats]).astype(np.complex128)
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _mats(n, nmat, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 2.0 * np.sqrt(n) * np.eye(n) *
            np.exp(1j * rng.uniform(0, 6.28)) for _ in range(nmat)]


def _factor(A, n, nmat):
    piv = torch.zeros(nmat * n, dtype=torch.int32, device="cuda")
    info = (ctypes.c_int * nmat)()
    st = C.lib().hbem_lu_factor_batch_device(n, nmat, ctypes.c_void_p(A.data_ptr()), n * n,
                                            ctypes.c_void_p(piv.data_ptr()), info)
    return st, piv, list(info)


@pytest.mark.parametrize("n", [5, 37, 100, 257])
def test_lu_solve_matches_numpy(n):
    nmat = 3
    mats = _mats(n, nmat, seed=n)
    A = _dev(mats)
    st, piv, info = _factor(A, n, nmat)
    check(st)
    assert info == [0] * nmat
    p = piv.cpu().numpy().reshape(nmat, n)
    assert np.all((p >= np.arange(n)) & (p < n))          # LAPACK ipiv convention, 0-based
    rng = np.random.default_rng(1)
    for nrhs in (1, 7, 20):                                # 20 > the 16-column register chunk
        B = [rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs)) for _ in range(nmat)]
        for trans in (0, 1):
            X = torch.from_numpy(np.ascontiguousarray(np.stack([b.T for b in B]))).cuda()   # column-major
            check(C.lib().hbem_lu_solve_batch_device(n, nmat, trans, ctypes.c_void_p(A.data_ptr()), n * n,
                                                     ctypes.c_void_p(piv.data_ptr()), nrhs,
                                                     ctypes.c_void_p(X.data_ptr()), n * nrhs))
            got = X.cpu().numpy()
            for m in range(nmat):
                M = mats[m].conj().T if trans else mats[m]
                ref = np.linalg.solve(M, B[m])
                assert np.linalg.norm(got[m].T - ref) <= 1e-12 * np.linalg.norm(ref)


def test_lu_reconstructs_pa():
    n, nmat = 70, 2
    mats = _mats(n, nmat, seed=5)
    A = _dev(mats)
    st, piv, _ = _factor(A, n, nmat)
    check(st)
    F = A.cpu().numpy()
    p = piv.cpu().numpy().reshape(nmat, n)
    for m in range(nmat):
        LU = F[m].T
        L = np.tril(LU, -1) + np.eye(n)
        U = np.triu(LU)
        PA = mats[m].copy()
        for k in range(n):
            PA[[k, p[m, k]]] = PA[[p[m, k], k]]
        assert np.linalg.norm(L @ U - PA) <= 1e-13 * np.linalg.norm(PA)
        # partial pivoting: |L| <= 1
        assert np.max(np.abs(L)) <= 1.0 + 1e-15


def test_lu_zero_pivot_reported():
    n, nmat = 40, 2
    mats = _mats(n, nmat, seed=9)
    mats[1][:, 17] = 0.0                                    # singular: zero column
    A = _dev(mats)
    st, _, info = _factor(A, n, nmat)
    assert st == 5 and info[0] == 0 and info[1] > 0


@pytest.mark.parametrize("n", [1000, 1500])
def test_cluster_panel_matches_global_panel(n):
    """Panels taller than one CTA's shared memory (FP64: > 440 rows): the cluster
    factorisation (rows spread over the CTAs' shared memory) gives the same pivots
    and factors as the in-place global-memory panel."""
    nmat = 2
    mats = _mats(n, nmat, seed=n + 1)
    res = []
    for on in (1, 0):
        check(C.lib().hbem_set_option(b"lu_cluster_panels", on))
        A = _dev(mats)
        st, piv, _ = _factor(A, n, nmat)
        check(st)
        res.append((A.cpu().numpy(), piv.cpu().numpy()))
    check(C.lib().hbem_set_option(b"lu_cluster_panels", 1))
    assert np.array_equal(res[0][1], res[1][1])
    assert np.max(np.abs(res[0][0] - res[1][0])) <= 1e-13 * np.max(np.abs(res[1][0]))
    b = np.random.default_rng(2).standard_normal((n, 3)) + 0j
    X = torch.from_numpy(np.ascontiguousarray(np.stack([b.T] * nmat))).cuda()
    A = _dev(mats)
    st, piv, _ = _factor(A, n, nmat)
    check(C.lib().hbem_lu_solve_batch_device(n, nmat, 0, ctypes.c_void_p(A.data_ptr()), n * n,
                                             ctypes.c_void_p(piv.data_ptr()), 3, ctypes.c_void_p(X.data_ptr()), 3 * n))
    for m in range(nmat):
        ref = np.linalg.solve(mats[m], b)
        assert np.linalg.norm(X.cpu().numpy()[m].T - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("n", [100, 256, 300, 513])
def test_lu_f32_reconstructs_pa_both_update_paths(n):
    """The complex-FP32 LU (from order 256: 128-column blocks with depth-128 tensor-core
    updates, 3xTF32) reconstructs P A to the FP32 rounding level, with |L| <= 1, and
    its pivots are those of the FP32 FMA path with 32-column panels."""
    nmat = 2
    mats = _mats(n, nmat, seed=3 * n)
    res = []
    for tc in (1, 0):
        check(C.lib().hbem_set_option(b"lu_tensor_cores", tc))
        try:
            A = torch.from_numpy(np.ascontiguousarray(np.stack([m.T for m in mats]).astype(np.complex64))).cuda()
            piv = torch.zeros(nmat * n, dtype=torch.int32, device="cuda")
            check(C.lib().hbem_lu_factor_batch_device_f32(n, nmat, ctypes.c_void_p(A.data_ptr()), n * n,
                                                          ctypes.c_void_p(piv.data_ptr()), None))
        finally:
            check(C.lib().hbem_set_option(b"lu_tensor_cores", 1))
        res.append((A.cpu().numpy(), piv.cpu().numpy().reshape(nmat, n)))
    for (F, p) in res:
        for m in range(nmat):
            LU = F[m].T.astype(np.complex128)
            L = np.tril(LU, -1) + np.eye(n)
            U = np.triu(LU)
            PA = mats[m].copy()
            for k in range(n):
                PA[[k, p[m, k]]] = PA[[p[m, k], k]]
            assert np.linalg.norm(L @ U - PA) <= 2e-6 * np.linalg.norm(PA)
            assert np.max(np.abs(L)) <= 1.0 + 1e-6
    assert np.array_equal(res[0][1], res[1][1])
