"""Analytic checks of the restated Galerkin assembly (no reference fixtures exist
for these matrices): circle eigenvalues, symmetry, derivative consistency."""
import numpy as np
import pytest
import scipy.special as sp

from oracle import oracle as O


def _circle(N, order=11, R=0.25):
    k, p = O.circle_panels(R, N)
    return O.Builder(k, p, order)


def _rayleigh(B, L, M, n):
    N = B.n
    th = 2 * np.pi * np.arange(N) / N
    c = np.exp(1j * n * th)
    den = np.vdot(c, M @ c)
    return {name: np.vdot(c, L[name][0] @ c) / den for name in ("K", "W", "V")}


@pytest.mark.parametrize("n", [0, 1, 2])
def test_circle_eigenvalues_converge(n):
    R, k, c = 0.25, 3.0, 23.4
    kap = k * np.sqrt(c)
    J = lambda m: sp.jv(m, kap * R)
    H = lambda m: sp.hankel1(m, kap * R)
    ev = {"V": 1j * np.pi * R / 2 * J(n) * H(n),
          "W": 1j * np.pi * R / 2 * ((n / R) ** 2 * J(n) * H(n) - kap ** 2 / 2 * (J(n + 1) * H(n + 1) + J(n - 1) * H(n - 1))),
          "K": 1j * np.pi * kap * R / 4 * (J(n) * sp.h1vp(n, kap * R) + sp.jvp(n, kap * R) * H(n))}
    errs = []
    for N in (25, 50, 100):
        B = _circle(N)
        lam = _rayleigh(B, B.assemble(k, c, O.LAYER_ALL, 0), B.mass(), n)
        errs.append({m: abs(lam[m] - ev[m]) / abs(ev[m]) for m in ev})
    for m in ev:
        assert errs[-1][m] < 2e-5
        if errs[0][m] > 1e-6:   # clear of the quadrature floor: at least second order
            assert errs[0][m] / errs[-1][m] > 12.0


def test_symmetry_square_spaces():
    B = _circle(30)
    L = B.assemble(2.0, 4.0, O.LAYER_ALL, 2)
    for t in range(3):
        for name in ("V", "W"):
            A = L[name][t]
            assert np.abs(A - A.T).max() <= 1e-13 * np.abs(A).max()


@pytest.mark.parametrize("kind", ["circle", "polygon"])
def test_k_derivatives_match_finite_differences(kind):
    if kind == "circle":
        B = _circle(20)
    else:
        x, y = O.star_polygon(7, seed=5)
        B = O.Builder(*O.polygon_panels(x, y, 28), 8)
    k, c, h = 2.3, 4.0, 1e-4
    L = B.assemble(k, c, O.LAYER_ALL, 2)
    Lp = B.assemble(k + h, c, O.LAYER_ALL, 0)
    Lm = B.assemble(k - h, c, O.LAYER_ALL, 0)
    for name in ("K", "W", "V"):
        d1 = (Lp[name][0] - Lm[name][0]) / (2 * h)
        d2 = (Lp[name][0] - 2 * L[name][0] + Lm[name][0]) / h ** 2
        assert np.linalg.norm(L[name][1] - d1) <= 1e-7 * np.linalg.norm(L[name][1])
        assert np.linalg.norm(L[name][2] - d2) <= 1e-4 * np.linalg.norm(L[name][2])


def test_reference_single_layer_quirk_is_wrong():
    """galerkin_builder.cpp:749 copies the order-0 entry into the derivative blocks of
    the coincident single layer; with that quirk V' no longer matches d/dk V."""
    B = _circle(16)
    k, c, h = 2.0, 4.0, 1e-4
    d1 = (B.assemble(k + h, c, O.LAYER_SINGLE, 0)["V"][0] - B.assemble(k - h, c, O.LAYER_SINGLE, 0)["V"][0]) / (2 * h)
    good = B.assemble(k, c, O.LAYER_SINGLE, 1)["V"][1]
    B.set_quirks(1)
    bad = B.assemble(k, c, O.LAYER_SINGLE, 1)["V"][1]
    B.set_quirks(0)
    assert np.linalg.norm(good - d1) < 1e-7 * np.linalg.norm(d1)
    assert np.linalg.norm(bad - d1) > 1e-3 * np.linalg.norm(d1)


def test_submatrix_matches_full():
    """Sub-matrix assembly adds the interactions of a block of panels; with
    discontinuous P0 spaces (one dof per panel) that is exactly the full block."""
    k, p = O.circle_panels(0.25, 24)
    B = O.Builder(k, p, 11, qtest=1, qtrial=1)
    full = B.assemble(1.7, 3.0, O.LAYER_ALL, 1)
    sub = B.assemble(1.7, 3.0, O.LAYER_ALL, 1, row=5, col=9, rows=7, cols=11)
    for name in ("K", "W", "V"):
        for t in range(2):
            ref = full[name][t][5:12, 9:20]
            assert np.abs(sub[name][t] - ref).max() <= 1e-13 * np.abs(full[name][t]).max()


def test_pair_classification():
    B = _circle(10)
    assert B.is_adjacent(1, 0) == (True, True)
    assert B.is_adjacent(9, 0) == (True, False)
    assert B.is_adjacent(5, 2) == (False, False)


def test_polygon_panel_counts():
    x, y = O.star_polygon(24, seed=2)
    kinds, par = O.polygon_panels(x, y, 1000)
    assert kinds.size == 1000
    # panels chain end-to-start
    gaps = np.hypot(par[:, 2] - np.roll(par[:, 0], -1), par[:, 3] - np.roll(par[:, 1], -1))
    assert gaps.max() < 1e-14


def test_nonsquare_spaces():
    """P0 test / P1 trial (the operator unit tests' spaces): shapes and consistency of
    the double layer with the P1/P1 one summed over the two P1 functions of a panel."""
    k, p = O.circle_panels(0.25, 12)
    Bq = O.Builder(k, p, 7, qtest=1, qtrial=2)
    L = Bq.assemble(1.0, 5.0, O.LAYER_ALL, 0)
    assert L["K"][0].shape == (12, 12) and L["V"][0].shape == (12, 12)
    Bs = O.Builder(k, p, 7)
    Ls = Bs.assemble(1.0, 5.0, O.LAYER_DOUBLE, 0)
    # P0 indicator of panel i = hat_i + hat_{i+1} restricted to panel i
    assert np.isfinite(L["K"][0]).all() and np.isfinite(Ls["K"][0]).all()
