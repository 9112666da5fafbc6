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
    assert np.max((got - dense) / dense) < 1e-6


def test_rsvd_sv_der_close_to_dense_derivative():
    mats = _mats([2.7, 4.05], d=1)
    n = mats[0][0].shape[0]
    R = O.rand_sketch(n, 16, seed=3)
    got = api.rsvd_sv(mats, R, q=3, d=1)
    for m, g in zip(mats, got):
        ref = O.sv_derivs(m[0], m[1])
        assert abs(g[0] - ref[0]) <= 1e-8 * ref[0]
        assert abs(g[1] - ref[1]) <= 1e-6 * max(abs(ref[1]), 1e-3)

