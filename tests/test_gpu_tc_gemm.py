"""Complex64 update C -= A B on the tensor cores (tcgen05, 3xTF32) against numpy
and against the FP32 FMA kernel, through the C ABI on device buffers."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from helmholtzbem_gb300 import _capi as C  # noqa: E402
from helmholtzbem_gb300._capi import check  # noqa: E402


def _colmajor(mats):
    """list of (r x c) complex matrices -> (nmat, c, r) complex64 device tensor (column-major)."""
    return torch.from_numpy(np.ascontiguousarray(np.stack([m.T for m in mats]).astype(np.complex64))).cuda()


def _update(A, B, Cm, tc):
    m, k = A[0].shape
    n = B[0].shape[1]
    nmat = len(A)
    dA, dB, dC = _colmajor(A), _colmajor(B), _colmajor(Cm)
    check(C.lib().hbem_cgemm_f32_batch_device(m, n, k, ctypes.c_void_p(dA.data_ptr()), m, m * k,
                                              ctypes.c_void_p(dB.data_ptr()), k, k * n,
                                              ctypes.c_void_p(dC.data_ptr()), m, m * n, nmat, tc))
    return [x.T for x in dC.cpu().numpy()]


def test_tc_update_exact_small_integers():
    """Small-integer operands are exact in TF32 (lo parts vanish) and all sums are
    exact in FP32: the tensor-core result must equal numpy's exactly; one full
    128 x 64 tile, K = 32."""
    rng = np.random.default_rng(1)
    m, n, k = 128, 64, 32
    A = [rng.integers(-4, 5, (m, k)) + 1j * rng.integers(-4, 5, (m, k))]
    B = [rng.integers(-4, 5, (k, n)) + 1j * rng.integers(-4, 5, (k, n))]
    C0 = [rng.integers(-50, 51, (m, n)) + 1j * rng.integers(-50, 51, (m, n))]
    got = _update(A, B, C0, 1)[0]
    ref = C0[0] - A[0] @ B[0]
    assert np.array_equal(got, ref.astype(np.complex64))
    # the same with K = 128 (four chunks accumulated in tensor memory)
    A = [rng.integers(-2, 3, (m, 128)) + 1j * rng.integers(-2, 3, (m, 128))]
    B = [rng.integers(-2, 3, (128, n)) + 1j * rng.integers(-2, 3, (128, n))]
    got = _update(A, B, C0, 1)[0]
    ref = C0[0] - A[0] @ B[0]
    assert np.array_equal(got, ref.astype(np.complex64))


@pytest.mark.parametrize("shape", [(300, 200, 32, 2), (130, 70, 17, 3), (1, 1, 1, 1), (257, 129, 32, 1),
                                   (300, 200, 128, 2), (190, 77, 77, 1), (256, 128, 96, 1), (129, 65, 33, 2)])
def test_tc_update_matches_fp32_and_numpy(shape):
    """Ragged tiles, K below, at and above the 32-column chunk (the LU's 128-wide
    blocks take four chunks into the same accumulator), batches: 3xTF32 products
    with FP32 accumulation agree with the FP32 FMA kernel and with numpy to the FP32
    rounding level."""
    m, n, k, nmat = shape
    rng = np.random.default_rng(m + n + k)
    A = [rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k)) for _ in range(nmat)]
    B = [rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n)) for _ in range(nmat)]
    C0 = [rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n)) for _ in range(nmat)]
    tc = _update(A, B, C0, 1)
    simt = _update(A, B, C0, 0)
    for q in range(nmat):
        ref = C0[q] - A[q] @ B[q]
        scale = np.abs(A[q]) @ np.abs(B[q]) + np.abs(C0[q])
        assert np.max(np.abs(tc[q] - ref) / scale) < 2e-6
        assert np.max(np.abs(simt[q] - ref) / scale) < 2e-6
