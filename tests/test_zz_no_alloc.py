"""The allocation-free dense singular-value entry point.

Some callers cannot call cudaMalloc: code that runs while a memory pool is
locked, that lives inside another library's fixed memory budget, or that must
not let an allocation synchronise its stream.  hbem_sv_dense_batch_noalloc
serves them with a fixed 8 MiB working array compiled into the library.  This
file checks, through the C ABI, that it returns what the allocating entry point
returns, on two calls in a row (the second call reuses the array the first one
left behind), and that requests beyond its size limit are refused.

It is named so that pytest collects it last, and it runs alone as well as after
the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from helmholtzbem_gb300 import _capi as C
    from helmholtzbem_gb300 import api, geometry

    lib = C.lib()
    npan, nk, d = 24, 6, 2
    n = 2 * npan
    data = api.BuilderData(geometry.circle(0.25, npan), order=9)
    so = api.SolutionsOperator(data)
    ks = np.ascontiguousarray(np.linspace(1.0, 4.0, nk))
    # T, T', T'' for each k, column-major n x n each, on the device
    T = torch.empty((nk, d + 1, n, n), dtype=torch.complex128, device="cuda")
    C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), nk, 1.0, 23.4, d, ctypes.c_void_p(T.data_ptr())))

    ref = np.zeros((nk, 3))
    C.check(lib.hbem_sv_dense_batch_device(n, nk, d, ctypes.c_void_p(T.data_ptr()), (d + 1) * n * n, n * n,
                                           C.dptr(ref), None))

    out = torch.empty((nk, 3), dtype=torch.float64, device="cuda")
    status = torch.empty(nk, dtype=torch.int32, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        status.fill_(-1)
        C.check(lib.hbem_sv_dense_batch_noalloc(n, nk, d, ctypes.c_void_p(T.data_ptr()), (d + 1) * n * n, n * n,
                                                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(status.data_ptr()),
                                                None))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert (status.cpu().numpy() == 0).all()
        # same tolerances as the dense-SVD parity tests
        assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 1e-10 * ref[:, 0])
        assert np.all(np.abs(got[:, 1] - ref[:, 1]) <= 1e-8 * np.maximum(np.abs(ref[:, 1]), 1e-3))
        assert np.all(np.abs(got[:, 2] - ref[:, 2]) <= 1e-8 * np.maximum(np.abs(ref[:, 2]), 1e-3))


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    from helmholtzbem_gb300 import _capi as C

    lib = C.lib()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    st = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    ps = ctypes.c_void_p(st.data_ptr())
    HBEM_ERR_INVALID = 1
    # order above 116: the matrix would not fit in shared memory
    assert lib.hbem_sv_dense_batch_noalloc(117, 1, 0, p, 117 * 117, 0, p, ps, None) == HBEM_ERR_INVALID
    # nmat * n * n above 524288 complex elements (8 MiB)
    assert lib.hbem_sv_dense_batch_noalloc(100, 53, 0, p, 100 * 100, 0, p, ps, None) == HBEM_ERR_INVALID
    assert b"8 MiB" in lib.hbem_last_error()
