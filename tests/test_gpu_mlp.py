"""The proposal network on the GPU: the tcgen05 BF16 product kernel against numpy,
forward pass and gradients against the oracle (with the same bfloat16 roundings),
and Adam training reducing the loss."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from helmholtzbem_gb300 import _capi as C, api  # noqa: E402
from helmholtzbem_gb300._capi import check  # noqa: E402
from oracle import oracle as O  # noqa: E402


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (512, 128, 1024)])
def test_bf16_gemm_tensor_cores(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = O.bf16_round(rng.standard_normal((M, K)).astype(np.float32))
    B = O.bf16_round(rng.standard_normal((N, K)).astype(np.float32))
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    At = torch.from_numpy(A).to(torch.bfloat16).cuda()
    Bt = torch.from_numpy(B).to(torch.bfloat16).cuda()
    for tc in (1, 0):
        Ct = torch.zeros((M, N), dtype=torch.float32, device="cuda")
        check(C.lib().hbem_bf16_gemm_device(M, N, K, ctypes.c_void_p(At.data_ptr()), K, ctypes.c_void_p(Bt.data_ptr()),
                                            K, ctypes.c_void_p(Ct.data_ptr()), N, tc))
        got = Ct.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref)) * np.sqrt(K / 64)


def test_bf16_gemm_rejects_unpadded_shapes():
    t = torch.zeros(128 * 128, dtype=torch.bfloat16, device="cuda")
    c = torch.zeros(128 * 128, dtype=torch.float32, device="cuda")
    assert C.lib().hbem_bf16_gemm_device(100, 128, 64, ctypes.c_void_p(t.data_ptr()), 64, ctypes.c_void_p(t.data_ptr()),
                                         64, ctypes.c_void_p(c.data_ptr()), 128, 1) == 1


def _net(seed=3):
    return api.MLP(34, 512, 4, 128, seed=seed)


def test_forward_matches_oracle():
    net = _net()
    rng = np.random.default_rng(1)
    X = rng.standard_normal((200, 34)).astype(np.float32)
    Y = net.forward(X)
    ref = O.MLPOracle(net.get_params(), net.dims).forward(X)
    assert np.linalg.norm(Y - ref) <= 2e-3 * np.linalg.norm(ref)


def test_gradients_match_oracle():
    net = _net()
    rng = np.random.default_rng(2)
    X = rng.standard_normal((130, 34)).astype(np.float32)
    T = rng.standard_normal((130, 128)).astype(np.float32)
    loss, g = net.gradients(X, T)
    rloss, rg = O.MLPOracle(net.get_params(), net.dims).gradients(X, T)
    assert abs(loss - rloss) <= 1e-3 * rloss
    off = 0
    for i, o in zip(net.dims[:-1], net.dims[1:]):
        for size in (o * i, o):
            a, b = g[off:off + size], rg[off:off + size]
            assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-12, (off, size)
            off += size
    # the same network with FP32 FMA products gives the same gradients
    check(C.lib().hbem_set_option(b"mlp_tensor_cores", 0))
    try:
        loss2, g2 = net.gradients(X, T)
    finally:
        check(C.lib().hbem_set_option(b"mlp_tensor_cores", 1))
    assert np.linalg.norm(g2 - g) <= 1e-3 * np.linalg.norm(g)


def test_set_get_params_roundtrip():
    net = _net()
    p = net.get_params()
    q = (p * 0.5).astype(np.float32)
    net.set_params(q)
    assert np.array_equal(net.get_params(), q)


def test_adam_training_reduces_the_loss():
    """A smooth regression (sines of random projections): 300 Adam steps lower the
    mean squared error by more than an order of magnitude."""
    rng = np.random.default_rng(4)
    P = rng.standard_normal((34, 16))
    X = rng.standard_normal((512, 34)).astype(np.float32)
    T = np.sin(X @ P)[:, np.repeat(np.arange(16), 8)].astype(np.float32)
    net = _net(seed=7)
    first = net.train_step(X, T, 1e-3)
    for _ in range(299):
        last = net.train_step(X, T, 1e-3)
    assert last < first / 10, (first, last)
