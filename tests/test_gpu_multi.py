"""Many scatterers of uneven panel counts in one assembly launch
(hbem_gen_sol_op_multi_device) against each operator's own batched T(k)
(hbem_gen_sol_op_batch_device, checked against the oracle elsewhere): lines and
arcs, P1 and P0 spaces, with and without projection, d = 0 and 2, an operator
without wavenumbers."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import _capi as C, api, geometry  # noqa: E402


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _single(so, ks, c_o, c_i, d):
    import torch
    n = 2 * so.data.npanels
    T = torch.empty((len(ks), d + 1, n, n), dtype=torch.complex128, device="cuda")
    if len(ks):
        C.check(C.lib().hbem_gen_sol_op_batch_device(so._h, C.dptr(np.ascontiguousarray(ks, np.float64)), len(ks),
                                                     float(c_o), float(c_i), d, ctypes.c_void_p(T.data_ptr())))
    return T.cpu().numpy()


@pytest.mark.parametrize("d", [0, 2])
def test_multi_launch_matches_per_operator_batches(d):
    P0, P1 = C.SPACE_P0, C.SPACE_P1
    meshes = [
        (geometry.polygon(*geometry.star_polygon(11, seed=8), 40), P1, P1, True),
        (geometry.circle(0.25, 24), P1, P1, True),
        (geometry.fourier_curve(*geometry.random_fourier_coeffs(3005), 64), P1, P1, False),
        (geometry.polygon(*geometry.star_polygon(7, seed=9), 17), P0, P1, False),
        (geometry.circle(0.4, 9), P1, P1, True),
        (geometry.polygon(*geometry.star_polygon(9, seed=1), 30), P0, P0, True),
    ]
    ops = [api.SolutionsOperator(api.BuilderData(m, te, tr, 9), proj=pj) for m, te, tr, pj in meshes]
    rng = np.random.default_rng(5)
    ks = [np.sort(rng.uniform(0.5, 12.0, n)) for n in (5, 3, 7, 2, 0, 4)]
    ci = [9.0, 23.4, 4.0, 3.0, 2.0, 6.5]
    out = api.gen_sol_op_multi_device(ops, ks, 1.0, ci, d=d)
    for so, k, c, T in zip(ops, ks, ci, out):
        ref = _single(so, k, 1.0, c, d)
        got = T.cpu().numpy()
        assert got.shape == ref.shape
        for q in range(len(k)):
            for t in range(d + 1):
                assert rel(got[q, t], ref[q, t]) <= 1e-13, (q, t)


def test_multi_launch_refuses_bad_input():
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 8), order=5))
    with pytest.raises(C.HbemError):
        api.gen_sol_op_multi_device([so], [np.array([1.0, -2.0])], 1.0, [4.0])
    with pytest.raises(C.HbemError):
        api.gen_sol_op_multi_device([so], [np.array([1.0])], 1.0, [0.5])


def test_autotuned_layout_matches_and_persists(tmp_path, monkeypatch):
    """With the autotuner on, the first launch of a key times the general-pair layouts
    and records the fastest in HBEM_TUNE_CACHE; results equal the untuned ones to
    rounding."""
    import ctypes as ct
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("HBEM_TUNE_CACHE", str(cache))
    so = api.SolutionsOperator(api.BuilderData(geometry.polygon(*geometry.star_polygon(10, seed=2), 37), order=9))
    ks = [1.3, 4.4, 7.9]
    ref = [so.gen_sol_op_2nd_der(k, 1.0, 5.0) for k in ks]
    C.check(C.lib().hbem_set_option(b"autotune", 1))
    try:
        got = [so.gen_sol_op_2nd_der(k, 1.0, 5.0) for k in ks]
        v = ct.c_int()
        C.check(C.lib().hbem_get_option(b"autotune", ct.byref(v)))
        assert v.value == 1
    finally:
        C.check(C.lib().hbem_set_option(b"autotune", 0))
    for a, b in zip(got, ref):
        for x, y in zip(a, b):
            assert rel(x, y) <= 1e-13
    lines = cache.read_text().split("\n")
    rows = [list(map(int, l.split())) for l in lines if l.strip()]
    # one key per (panels, order, jobs, d, real k, kind) tuned: 37 panels, order 9, 2 jobs, d = 2
    assert any(r[:6] == [37, 9, 2, 2, 1, 0] and r[6] in (0, 1, 2, 4, 8, 16) for r in rows), rows
