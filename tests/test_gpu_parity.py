"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the
same inputs.  Tolerances: Hankel 1e-13 relative (2e-13 on the ascending-series
band 4 <= x < 8 where the series itself is only good to ~1e-13), operator
matrices and T(k) 1e-12 relative Frobenius, sigma_min 1e-10 relative, sigma'
and sigma'' 1e-8 relative, resonances |dk| <= 1e-8."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "hankel_mpmath.json")))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_hankel_real_device_vs_golden_and_oracle():
    xs = np.array([r["x"] for r in GOLD["real"]])
    r0 = np.array([complex(*r["h0"]) for r in GOLD["real"]])
    r1 = np.array([complex(*r["h1"]) for r in GOLD["real"]])
    h0, h1 = api.hankel01(xs)
    o0, o1 = O.hankel01(xs)
    band = (xs >= 4.0) & (xs < 8.0)
    big = xs > 1e6
    ok = ~band & ~big
    for h, r, o in ((h0, r0, o0), (h1, r1, o1)):
        e_ref = np.abs(h - r) / np.abs(r)
        e_orc = np.abs(h - o) / np.abs(o)
        assert e_ref[ok].max() < 1e-13 and e_orc[ok].max() < 1e-13
        assert e_orc[band].max() < 2e-13
        # 2 <= x < 8: Taylor polynomials, free of the series' cancellation
        assert e_ref[band].max() < 1e-15
        assert e_orc[big].max() < 1e-13       # same leading-order form as the reference
    kat = GOLD["reference_kats"]
    h0, h1 = api.hankel01(np.array([np.pi, 0.1]))
    assert abs(h0[0].real - kat["J0(pi)"]) <= 2.3e-16
    assert abs(-h1[0].real - kat["J0'(pi)"]) <= 2.3e-16


def test_hankel_complex_device_vs_golden():
    z = np.array([complex(*r["z"]) for r in GOLD["complex"]])
    r0 = np.array([complex(*r["h0"]) for r in GOLD["complex"]])
    r1 = np.array([complex(*r["h1"]) for r in GOLD["complex"]])
    h0, h1 = api.hankel01(z)
    o0, o1 = O.hankel01(z)
    tol = 4e-15 * np.exp(2.0 * z.imag)
    assert np.all(np.abs(h0 - r0) / np.abs(r0) < tol)
    assert np.all(np.abs(h1 - r1) / np.abs(r1) < tol)
    assert np.all(np.abs(h0 - o0) / np.abs(o0) < tol)


MESHES = {
    "circle": lambda: (geometry.circle(0.25, 24), 11),
    "polygon": lambda: (geometry.polygon(*geometry.star_polygon(9, seed=11), 40), 8),
}


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("k", [3.7, 2.0 + 0.4j])
def test_assemble_layers_vs_oracle(mesh, k):
    (kinds, par), order = MESHES[mesh]()
    data = api.BuilderData((kinds, par), order=order)
    gb = api.GalerkinBuilder(data)
    ob = O.Builder(kinds, par, order)
    c = 5.0
    gb.assembleDense(k, c, api.LayerType_ALL, 2)
    ref = ob.assemble(k, c, O.LAYER_ALL, 2)
    for t in range(3):
        assert rel(gb.getDoubleLayer(t), ref["K"][t]) < 1e-12
        assert rel(gb.getHypersingular(t), ref["W"][t]) < 1e-12
        assert rel(gb.getSingleLayer(t), ref["V"][t]) < 1e-12


@pytest.mark.parametrize("sub", [(3, 10, 12, 7), (0, 0, 5, 20), (8, 8, 9, 9), (17, 2, 7, 5)])
def test_assemble_submatrix_vs_oracle(sub):
    """assembleDense(k, c, layers, d, row, col, rows, cols): the reference's sub-matrix
    rule (panel pairs inside the row / column panel ranges only) against the oracle."""
    row, col, rows, cols = sub
    (kinds, par), order = MESHES[list(MESHES)[0]]()
    data = api.BuilderData((kinds, par), order=order)
    gb = api.GalerkinBuilder(data)
    ob = O.Builder(kinds, par, order)
    gb.assembleDense(2.9, 4.0, api.LayerType_ALL, 1, row, col, rows, cols)
    ref = ob.assemble(2.9, 4.0, O.LAYER_ALL, 1, row=row, col=col, rows=rows, cols=cols)
    for t in range(2):
        for got, name in ((gb.getDoubleLayer(t), "K"), (gb.getHypersingular(t), "W"), (gb.getSingleLayer(t), "V")):
            assert got.shape == (rows, cols)
            assert rel(got, ref[name][t]) < 1e-12


def test_geometry_matches_oracle_geometry():
    a = geometry.polygon(*geometry.star_polygon(24, seed=2), 1000)
    b = O.polygon_panels(*O.star_polygon(24, seed=2), 1000)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    a = geometry.circle(0.25, 50)
    b = O.circle_panels(0.25, 50)
    assert np.array_equal(a[1], b[1])


@pytest.mark.parametrize("mesh", list(MESHES))
def test_gen_sol_op_vs_oracle(mesh):
    (kinds, par), order = MESHES[mesh]()
    data = api.BuilderData((kinds, par), order=order)
    so = api.SolutionsOperator(data)
    oso = O.SolutionsOperator(O.Builder(kinds, par, order))
    assert rel(so.mass_matrix(), oso.M) < 1e-14
    k, c_o, c_i = 4.1, 1.0, 6.5
    got = so.gen_sol_op_2nd_der(k, c_o, c_i)
    ref = oso.gen_sol_op(k, c_o, c_i, d=2)
    for a, b in zip(got, ref):
        assert rel(a, b) < 1e-12
    # unprojected operator too
    so2 = api.SolutionsOperator(data, proj=False)
    T0 = so2.gen_sol_op(k, c_o, c_i)
    assert rel(T0, oso.blocks(k, c_o, c_i, 0)[0]) < 1e-12


def test_sv_dense_vs_oracle():
    kinds, par = geometry.circle(0.25, 20)
    oso = O.SolutionsOperator(O.Builder(kinds, par, 9))
    Ts, refs = [], []
    for k in (1.3, 2.9, 4.4):
        mats = oso.gen_sol_op(k, 1.0, 23.4, d=2)
        Ts.append(mats)
        refs.append(O.sv_derivs(*mats))
    out, sig = api.sv_dense(Ts, d=2, all_values=True)
    for m, ref in enumerate(refs):
        s_np = np.sort(np.linalg.svd(Ts[m][0], compute_uv=False))
        assert np.max(np.abs(np.sort(sig[m]) - s_np) / s_np.max()) < 1e-13
        assert abs(out[m, 0] - ref[0]) <= 1e-10 * ref[0]
        assert abs(out[m, 1] - ref[1]) <= 1e-8 * max(abs(ref[1]), 1e-3)
        assert abs(out[m, 2] - ref[2]) <= 1e-8 * max(abs(ref[2]), 1e-3)


def test_sweep_sigma_end_to_end():
    kinds, par = geometry.circle(0.25, 16)
    data = api.BuilderData((kinds, par), order=7)
    so = api.SolutionsOperator(data)
    oso = O.SolutionsOperator(O.Builder(kinds, par, 7))
    ks = np.linspace(0.5, 6.0, 9)
    out = so.sweep_sigma(ks, 1.0, 23.4, d=2)
    for i, k in enumerate(ks):
        ref = O.sv_derivs(*oso.gen_sol_op(k, 1.0, 23.4, d=2))
        assert abs(out[i, 0] - ref[0]) <= 1e-10 * ref[0]
        assert abs(out[i, 1] - ref[1]) <= 1e-8 * max(abs(ref[1]), 1e-3)


def test_find_resonances_plain_vs_oracle():
    """Plain sweep + Newton on a small circle: every GPU root within 1e-8 of the
    oracle's, and the sign of sigma' changes across [root - 1e-8, root + 1e-8]."""
    kinds, par = geometry.circle(0.25, 16)
    data = api.BuilderData((kinds, par), order=7)
    so = api.SolutionsOperator(data)
    oso = O.SolutionsOperator(O.Builder(kinds, par, 7))
    c_o, c_i = 1.0, 23.4
    roots, grid, nev = so.find_resonances_plain(0.5, 6.0, 60, c_o, c_i, tol=1e-8)

    def evald(klist, d):
        return np.array([O.sv_derivs(*oso.gen_sol_op(k, c_o, c_i, d=d)) for k in klist])

    oroots, osig = O.plain_sweep(evald, np.linspace(0.5, 6.0, 60), tol=1e-8)
    assert np.max(np.abs(grid[:, 0] - osig) / osig) < 1e-10
    assert len(roots) == len(oroots) and len(roots) > 0
    assert np.max(np.abs(np.sort(roots) - np.sort(oroots))) <= 1e-8
    lo = so.sweep_sigma(roots - 1e-8, c_o, c_i, d=1)[:, 1]
    hi = so.sweep_sigma(roots + 1e-8, c_o, c_i, d=1)[:, 1]
    assert np.all(lo <= 0) and np.all(hi >= 0)


def test_errors_like_reference():
    from helmholtzbem_gb300._capi import HbemError
    kinds, par = geometry.circle(0.25, 8)
    data = api.BuilderData((kinds, par), order=5)
    gb = api.GalerkinBuilder(data)
    with pytest.raises(HbemError):
        gb.assembleDense(1.0, 0.5)              # c < 1
    with pytest.raises(HbemError):
        gb.assembleDense(1.0 - 0.1j, 2.0)       # Im k < 0
    with pytest.raises(HbemError):
        gb.assembleDense(1.0, 2.0, api.LayerType_ALL, 3)
    gb.assembleDense(1.0, 2.0, api.LayerType_SINGLE, 0)
    with pytest.raises(HbemError):
        gb.getDoubleLayer(0)                    # layer not assembled
    with pytest.raises(HbemError):
        gb.getSingleLayer(1)                    # derivative not assembled


def _config2_mesh(N=1000):
    """Assembly-at-scale scatterer: seeded star polygon, 24 vertices, r = 1 + 0.3 u,
    N line panels split in proportion to edge length."""
    return geometry.polygon(*geometry.star_polygon(24, seed=2), N)


def test_config2_reduced_vs_oracle():
    """Same polygon family at N = 200, Gauss order 16, k = 20, c = 4, d <= 2."""
    kinds, par = _config2_mesh(200)
    data = api.BuilderData((kinds, par), order=16)
    gb = api.GalerkinBuilder(data)
    ob = O.Builder(kinds, par, 16)
    gb.assembleDense(20.0, 4.0, api.LayerType_ALL, 2)
    ref = ob.assemble(20.0, 4.0, O.LAYER_ALL, 2)
    for t in range(3):
        assert rel(gb.getDoubleLayer(t), ref["K"][t]) < 1e-12
        assert rel(gb.getHypersingular(t), ref["W"][t]) < 1e-12
        assert rel(gb.getSingleLayer(t), ref["V"][t]) < 1e-12


def test_config2_full_size_properties():
    """N = 1000, order 16, k = 20, both media: size-independent properties of the full
    T(k), T', T'': V, W symmetric, and T', T'' consistent with central differences of
    the GPU's own T at k +- h (the oracle checks the same family at N = 200 above)."""
    kinds, par = _config2_mesh(1000)
    data = api.BuilderData((kinds, par), order=16)
    gb = api.GalerkinBuilder(data)
    gb.assembleDense(20.0, 4.0, api.LayerType_ALL, 2)
    for t in range(3):
        V, W = gb.getSingleLayer(t), gb.getHypersingular(t)
        assert np.abs(V - V.T).max() <= 1e-13 * np.abs(V).max()
        assert np.abs(W - W.T).max() <= 1e-13 * np.abs(W).max()
    so = api.SolutionsOperator(data)
    h = 1e-4
    T, T1, T2 = so.gen_sol_op_2nd_der(20.0, 1.0, 4.0)
    Tp = so.gen_sol_op(20.0 + h, 1.0, 4.0)
    Tm = so.gen_sol_op(20.0 - h, 1.0, 4.0)
    assert rel((Tp - Tm) / (2 * h), T1) < 1e-6
    assert rel((Tp - 2 * T + Tm) / h ** 2, T2) < 1e-3


@pytest.mark.parametrize("curved", [True, False])
def test_singular_table_matches_on_the_fly(curved):
    """Singular pairs read their k-independent point data from the builder's table
    (default) or compute it in the kernel: the same T(k), T', T'' to rounding."""
    from helmholtzbem_gb300 import _capi as C
    mesh = geometry.circle(0.25, 24) if curved else geometry.polygon(*geometry.star_polygon(12, seed=3), 40)
    so = api.SolutionsOperator(api.BuilderData(mesh, order=9))
    ks = [0.7, 3.3, 9.1]
    C.check(C.lib().hbem_set_option(b"singular_table", 1))
    a = [so.gen_sol_op_2nd_der(k, 1.0, 23.4) for k in ks]
    C.check(C.lib().hbem_set_option(b"singular_table", 0))
    try:
        b = [so.gen_sol_op_2nd_der(k, 1.0, 23.4) for k in ks]
    finally:
        C.check(C.lib().hbem_set_option(b"singular_table", 1))
    for ta, tb in zip(a, b):
        for x, y in zip(ta, tb):
            assert rel(x, y) <= 1e-14


def test_general_pairs_thread_and_warp_layouts_agree():
    """General panel pairs go to a thread per pair in large launches (many pairs x
    media) and to a warp per pair in small ones: T(k) of a 40-wavenumber batch (thread
    layout) against the same wavenumbers one at a time (warp layout)."""
    import ctypes
    import torch
    from helmholtzbem_gb300 import _capi as C
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    n = 100
    ks = np.linspace(0.7, 9.3, 40)
    big = torch.empty(ks.size * 3 * n * n * 2, dtype=torch.float64, device="cuda")
    C.check(C.lib().hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), ks.size, 1.0, 23.4, 2,
                                                 ctypes.c_void_p(big.data_ptr())))
    big = big.cpu().numpy().view(np.complex128).reshape(ks.size, 3, n, n)
    for i in (0, 17, 39):
        one = so.gen_sol_op_2nd_der(ks[i], 1.0, 23.4)
        for t in range(3):
            assert rel(big[i, t].T, one[t]) <= 1e-12   # summation order of the 121 points differs
