"""The allocation-free dense singular-value entry point.

Some callers cannot call cudaMalloc: code that runs while a memory pool is
locked, that lives inside another library's fixed memory budget, or that must
not let an allocation synchronise its stream.  hbem_sv_dense_batch_noalloc
serves them with a fixed 8 MiB working array compiled into the library.  This
file checks, through the C ABI, that it returns what the allocating entry point
returns, on two calls in a row (the second call reuses the array the first one
left behind), on the default stream and on a stream of the caller's, for every
derivative order; that the second call leaves the device's free memory as it
was; and that requests beyond its size limit or with host pointers are refused.

It is named so that pytest collects it last, and it runs alone as well as after
the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [2, 1, 0])
@pytest.mark.parametrize("own_stream", [False, True])
def test_noalloc_matches_allocating_entry_point(d, own_stream):
    torch = pytest.importorskip("torch")
    from helmholtzbem_gb300 import _capi as C
    from helmholtzbem_gb300 import api, geometry

    lib = C.lib()
    npan, nk = 24, 6
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
    stream = torch.cuda.Stream() if own_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    torch.cuda.synchronize()
    for call in range(2):
        out.fill_(float("nan"))
        status.fill_(-1)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        C.check(lib.hbem_sv_dense_batch_noalloc(n, nk, d, ctypes.c_void_p(T.data_ptr()), (d + 1) * n * n, n * n,
                                                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(status.data_ptr()),
                                                handle))
        torch.cuda.synchronize()
        if call == 1:   # the first call may load the module (lazy loading); the second allocates nothing
            assert torch.cuda.mem_get_info()[0] == free_before
        got = out.cpu().numpy()
        assert (status.cpu().numpy() == 0).all()
        # same tolerances as the dense-SVD parity tests
        assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 1e-10 * ref[:, 0])
        for t in range(1, d + 1):
            assert np.all(np.abs(got[:, t] - ref[:, t]) <= 1e-8 * np.maximum(np.abs(ref[:, t]), 1e-3))


def test_noalloc_rejects_sizes_beyond_its_limit_and_host_pointers():
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
    # host memory where device memory is expected: refused before any launch
    host = np.zeros(64, np.float64)
    hp = ctypes.c_void_p(host.ctypes.data)
    assert lib.hbem_sv_dense_batch_noalloc(2, 1, 0, hp, 4, 0, p, ps, None) == HBEM_ERR_INVALID
    assert lib.hbem_sv_dense_batch_noalloc(2, 1, 0, p, 4, 0, hp, ps, None) == HBEM_ERR_INVALID
    assert b"current device" in lib.hbem_last_error()
