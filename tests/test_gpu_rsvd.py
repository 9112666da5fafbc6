"""Randomized smallest singular value on the GPU (randomized_svd::sv / sv_der)
against the oracle's restatement with the same sketch, and against dense SVD."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _mats(ks, npan=48, order=9, d=1):
    kinds, par = geometry.circle(0.25, npan)
    oso = O.SolutionsOperator(O.Builder(kinds, par, order))
    return [oso.gen_sol_op(k, 1.0, 23.4, d=d) for k in ks]


def test_rsvd_sv_matches_oracle_same_sketch():
    mats = _mats([1.1, 2.7, 4.05, 6.3], d=0)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 12, seed=7)
    for q in (0, 2):
        got = api.rsvd_sv(mats, R, q=q, d=0)[:, 0]
        ref = np.array([O.rsvd_sv(m[0], R, q) for m in mats])
        assert np.max(np.abs(got - ref) / ref) < 1e-10
    dense = np.array([np.linalg.svd(m[0], compute_uv=False).min() for m in mats])
    got = api.rsvd_sv(mats, R, q=2, d=0)[:, 0]
    assert np.all(got >= dense * (1 - 1e-12))           # the estimate is from above
    assert np.max((got - dense) / dense) < 1e-5         # 2.2e-6 at k = 1.1 (sigma_2 / sigma_min = 1.6)


def test_rsvd_sv_der_close_to_dense_derivative():
    mats = _mats([2.7, 4.05], d=1)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 16, seed=3)
    got = api.rsvd_sv(mats, R, q=3, d=1)
    for m, g in zip(mats, got):
        ref = O.sv_derivs(m[0], m[1])
        assert abs(g[0] - ref[0]) <= 1e-8 * ref[0]
        assert abs(g[1] - ref[1]) <= 1e-6 * max(abs(ref[1]), 1e-3)



def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_rsvd_sv_der2_small_path_vs_oracle():
    """sv_der2 (bordered 2n x 2n system) with the shared-memory LU path (n = 96)."""
    mats = _mats([2.7, 4.05, 6.3], d=2)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 16, seed=3)
    got = api.rsvd_sv(mats, R, q=3, d=2)
    for m, g in zip(mats, got):
        s, d1, d2 = O.rsvd_sv_der2(m[0], m[1], m[2], R, 3)
        assert _rel(g[0], s) < 1e-10
        assert abs(g[1] - d1) <= 1e-8 * max(abs(d1), 1e-2)
        assert abs(g[2] - d2) <= 1e-7 * max(abs(d2), 1e-1)


@pytest.mark.parametrize("q", [0, 2])
def test_rsvd_global_path_vs_oracle(q):
    """n = 160 (too large for one CTA's shared memory): batched global LU, solves,
    QR; sigma, sigma', sigma'' against the oracle with the same sketch."""
    mats = _mats([1.7, 3.9, 5.2], npan=80, order=7, d=2)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 12, seed=5)
    got0 = api.rsvd_sv(mats, R, q=q, d=0)[:, 0]
    got = api.rsvd_sv(mats, R, q=q, d=2)
    for m, g0, g in zip(mats, got0, got):
        s_ref = O.rsvd_sv(m[0], R, q)
        assert _rel(g0, s_ref) < 1e-10 and _rel(g[0], s_ref) < 1e-10
        if q == 2:
            s, d1, d2 = O.rsvd_sv_der2(m[0], m[1], m[2], R, q)
            assert abs(g[1] - d1) <= 1e-8 * max(abs(d1), 1e-2)
            assert abs(g[2] - d2) <= 1e-7 * max(abs(d2), 1e-1)


def test_rsvd_batched_scatterer_size():
    """Star polygon with N = 800 line panels (T of order 1600, the largest scatterer
    of the batching workload), sketch 12, two subspace steps, four wavenumbers in one
    batch: sigma equals the oracle's rSVD with the same sketch, and is an upper bound
    within 1e-6 of the dense sigma_min."""
    kinds, par = geometry.polygon(*geometry.star_polygon(24, seed=2), 800)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=11))
    ks = [3.0, 7.5, 12.25, 19.0]
    mats = [[so.gen_sol_op(k, 1.0, 9.0)] for k in ks]
    n = mats[0][0].shape[0]
    R = api.randGaussian(n, 12, seed=2024)
    got = api.rsvd_sv(mats, R, q=2, d=0)[:, 0]
    for m, g in zip(mats, got):
        ref = O.rsvd_sv(m[0], R, 2)
        assert _rel(g, ref) < 1e-10
    dense = np.linalg.svd(mats[1][0], compute_uv=False).min()
    assert got[1] >= dense * (1 - 1e-12) and (got[1] - dense) / dense < 1e-6
    # complex-FP32 LU (panels of more than 880 rows factored in global memory) with
    # FP64 refinement: the same sigma to 1e-9
    mixed = _rsvd_device(mats, R, 2, 0, 1, 3)[:, 0]
    assert np.max(np.abs(mixed - got) / got) < 1e-9
    # the same with the complex-FP32 LU's trailing updates in FP32 FMA instead of the
    # tensor cores (3xTF32): both refine to the FP64 result
    from helmholtzbem_gb300 import _capi as C
    C.check(C.lib().hbem_set_option(b"lu_tensor_cores", 0))
    try:
        mixed_fma = _rsvd_device(mats, R, 2, 0, 1, 3)[:, 0]
    finally:
        C.check(C.lib().hbem_set_option(b"lu_tensor_cores", 1))
    assert np.max(np.abs(mixed_fma - got) / got) < 1e-9


def _rsvd_device(mats, R, q, d, precision, refine):
    """hbem_rsvd_sv_batch_device_ex on device copies of [T, T', ...] (column-major)."""
    import ctypes
    torch = pytest.importorskip("torch")
    from helmholtzbem_gb300 import _capi as C
    nmat, n = len(mats), mats[0][0].shape[0]
    buf = np.stack([np.stack([np.asarray(m[t]).T for t in range(d + 1)]) for m in mats]).astype(np.complex128)
    Td = torch.from_numpy(np.ascontiguousarray(buf)).cuda()
    Rd = torch.from_numpy(np.ascontiguousarray(np.asarray(R, np.complex128).T)).cuda()
    out = np.zeros((nmat, d + 1))
    C.check(C.lib().hbem_rsvd_sv_batch_device_ex(n, nmat, d, ctypes.c_void_p(Td.data_ptr()), (d + 1) * n * n, n * n,
                                                 ctypes.c_void_p(Rd.data_ptr()), R.shape[1], q, precision, refine,
                                                 C.dptr(out)))
    return out


def test_rsvd_mixed_precision_matches_fp64():
    """Complex-FP32 LU + FP64 refinement against the FP64 path on the same sketch:
    n = 160 with sigma', sigma'' (bordered system in FP64), and the relative error of
    each result reported by the assertion."""
    mats = _mats([1.7, 3.9, 5.2], npan=80, order=7, d=2)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 12, seed=5)
    ref = _rsvd_device(mats, R, 2, 2, 0, 1)
    for refine in (3, 4):
        got = _rsvd_device(mats, R, 2, 2, 1, refine)
        assert np.max(np.abs(got[:, 0] - ref[:, 0]) / ref[:, 0]) < 1e-10
        assert np.max(np.abs(got[:, 1] - ref[:, 1]) / np.maximum(np.abs(ref[:, 1]), 1e-2)) < 1e-8
        assert np.max(np.abs(got[:, 2] - ref[:, 2]) / np.maximum(np.abs(ref[:, 2]), 1e-1)) < 1e-7


@pytest.mark.parametrize("n", [256, 300, 513])
def test_rsvd_mixed_two_level_lu_block_edges(n):
    """The complex-FP32 LU of order >= 256 runs in 128-column blocks with one depth-128
    tensor-core update per block (whole blocks, a ragged last block, a single extra
    column): with FP64 refinement its sigma equals the FP64 path's on the same sketch,
    with the trailing updates on the tensor cores and in FP32 FMA alike."""
    rng = np.random.default_rng(n)
    mats = []
    for _ in range(2):
        # a clear smallest singular value, so that the randomized estimate has converged
        # and only the LU's accuracy can move it
        U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        sv = np.linspace(1.0, 4.0, n)
        sv[0] = 1e-3
        mats.append([(U * sv) @ V.conj().T])
    R = O.rand_sketch(n, 12, seed=n)
    ref = _rsvd_device(mats, R, 2, 0, 0, 1)[:, 0]
    got = _rsvd_device(mats, R, 2, 0, 1, 3)[:, 0]
    # sigma_min = 1e-3 against sigma_max = 4: 1e-9 relative is 2.5e-13 of the norm
    assert np.max(np.abs(got - ref) / ref) < 1e-9
    from helmholtzbem_gb300 import _capi as C
    C.check(C.lib().hbem_set_option(b"lu_tensor_cores", 0))
    try:
        fma = _rsvd_device(mats, R, 2, 0, 1, 3)[:, 0]
    finally:
        C.check(C.lib().hbem_set_option(b"lu_tensor_cores", 1))
    assert np.max(np.abs(fma - ref) / ref) < 1e-9
