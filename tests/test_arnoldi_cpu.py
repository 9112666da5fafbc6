"""arnoldi::sv oracle checks on the CPU (singular_values_arnoldi.cpp:19-246): the
ARPACK call of the reference (through scipy's ARPACK) and the block iteration
that stands in for it on the GPU both give the smallest singular values of the
dense SVD, and the block iteration's stopping test holds on its output."""
import math

import numpy as np
import pytest

from helmholtzbem_gb300 import geometry
from oracle import oracle as O


@pytest.fixture(scope="module")
def circle_ops():
    kinds, par = geometry.circle(0.25, 30)
    oso = O.SolutionsOperator(O.Builder(kinds, par, 7))
    return [oso.gen_sol_op(k, 1.0, 23.4)[0] for k in (1.1, 4.05, 9.7)]


def test_start_block_is_seeded_and_centred():
    a = O.arnoldi_start(50, 12, 0x5EED)
    b = O.arnoldi_start(50, 12, 0x5EED)
    c = O.arnoldi_start(50, 12, 1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.all(np.abs(a.real) <= 0.5) and np.all(np.abs(a.imag) <= 0.5)
    assert abs(a.real.mean()) < 0.1 and abs(a.imag.mean()) < 0.1


@pytest.mark.parametrize("count", [1, 3])
def test_arpack_and_block_match_dense(circle_ops, count):
    for T in circle_ops:
        sv = np.sort(np.linalg.svd(T, compute_uv=False))[:count]
        a = O.arnoldi_sv_arpack(T, count, 1e-12)
        b, V, it, conv = O.arnoldi_block(T, count, 1e-12)
        assert conv and it < 200
        assert np.max(np.abs(a - sv)) <= 1e-12 * sv[-1] * 100
        assert np.max(np.abs(b - sv)) <= 1e-12 * sv[-1] * 100
        # right vectors: |T v_j| = sigma_j
        for j in range(count):
            assert abs(np.linalg.norm(T @ V[:, j]) - sv[j]) <= 1e-6 * sv[j]


def test_block_residual_test_and_cap():
    rng = np.random.default_rng(4)
    n = 40
    T = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    sv = np.sort(np.linalg.svd(T, compute_uv=False))
    s, V, it, conv = O.arnoldi_block(T, 2, 1e-10)
    assert conv and np.max(np.abs(s - sv[:2]) / sv[:2]) < 1e-9
    # the residual test of the last iteration: |T^H T v - sigma^2 v| small relative to sigma^2
    for j in range(2):
        r = T.conj().T @ (T @ V[:, j]) - s[j] ** 2 * V[:, j]
        assert np.linalg.norm(r) <= 1e-6 * s[j] ** 2 * math.sqrt(n)
    s1, _, it1, conv1 = O.arnoldi_block(T, 2, 1e-14, maxit=1)
    assert it1 == 1 and not conv1


def test_block_size_rule():
    assert O.arnoldi_block_size(100, 1) == 12
    assert O.arnoldi_block_size(100, 10) == 20
    assert O.arnoldi_block_size(100, 28) == 32
    assert O.arnoldi_block_size(8, 3) == 8
