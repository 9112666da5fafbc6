"""Incoming waves, the transmission solve and the field on a grid on the GPU
(tp::direct_second_kind::solve / solve_in_rectangle, source/utilities/solvers.cpp,
incoming.cpp) against the oracle restatement."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402

WAVES = [api.wave("Plane", 1.0, (0.1, -0.2), angle=0.7),
         api.wave("CircularJ", 0.5, (0.05, 0.0), order=-2),
         api.wave("CircularJ", 0.5, (0.0, 0.0), order=1),
         api.wave("CircularY", 0.3, (1.5, 1.5), order=1),
         api.wave("FourierHankel1", 0.2, (-1.4, 0.3), order=3),
         api.wave("FourierHankel2", 0.2, (1.4, -0.3), order=0),
         api.wave("CircularJ", 1.0, (0.0, 0.0), order=25),
         api.wave("Herglotz", 1.0, (-0.2, 0.0), angle=0.85, eps=0.1)]


@pytest.mark.parametrize("w", range(len(WAVES)))
def test_incoming_waves_match_oracle(w):
    rng = np.random.default_rng(w)
    pts = rng.uniform(-1.2, 1.2, (40, 2))
    pts[0] = (0.0, 0.0)                 # the centre of the circular waves at the origin
    for k in (0.7, 3.3, 17.0):
        u, du = api.incoming_eval(WAVES[w], k, pts)
        for m, (x, y) in enumerate(pts):
            ru, rux, ruy = O.wave_eval(WAVES[w], k, x, y)
            if not np.isfinite(ru):
                continue
            sc = max(1.0, abs(ru))
            assert abs(u[m] - ru) <= 1e-11 * sc
            gs = max(1.0, abs(rux), abs(ruy))
            if np.isfinite(rux) and np.isfinite(ruy):
                assert abs(du[m, 0] - rux) <= 1e-10 * gs and abs(du[m, 1] - ruy) <= 1e-10 * gs


def test_complex_wavenumber_plane_and_herglotz():
    pts = np.array([[0.3, 0.1], [-0.5, 0.8]])
    for w in (WAVES[0], WAVES[-1]):
        u, du = api.incoming_eval(w, 2.0 + 0.3j, pts)
        for m, (x, y) in enumerate(pts):
            ru, rux, ruy = O.wave_eval(w, 2.0 + 0.3j, x, y)
            assert abs(u[m] - ru) <= 1e-12 * max(1, abs(ru)) and abs(du[m, 1] - ruy) <= 1e-11 * max(1, abs(ruy))


MESHES = {
    "square24": lambda: geometry.polygon([-0.5, 0.5, 0.5, -0.5], [-0.5, -0.5, 0.5, 0.5], 24),
    "circle20": lambda: geometry.circle(0.5, 20),
    "graded_L": lambda: geometry.polygon_graded([0.0, 1.0, 1.0, 0.5, 0.5, 0.0], [0.0, 0.0, 0.5, 0.5, 1.0, 1.0], 30,
                                                0.5),
}


@pytest.mark.parametrize("mesh", list(MESHES))
def test_tp_solve_matches_oracle(mesh):
    kinds, par = MESHES[mesh]()
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=9), proj=False)
    for w, k, c_o, c_i in ((WAVES[0], 3.1, 1.0, 4.0), (WAVES[-1], 2.2, 1.0, 9.0)):
        got = api.tp_solve(so, w, k, c_o, c_i)
        ref = O.tp_solve(kinds, par, 9, w, k, c_o, c_i)
        assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)


def test_tp_solve_needs_unprojected_operator():
    kinds, par = MESHES["square24"]()
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=7))
    with pytest.raises(api.C.HbemError):
        api.tp_solve(so, WAVES[0], 2.0, 1.0, 4.0)


@pytest.mark.parametrize("mesh,ll,ur,n", [
    ("square24", (-0.7, -0.7), (0.7, 0.7), 15),            # grid lines through the edges: on-boundary points
    ("square24", (-0.7 + 3e-4, -0.69), (0.7 + 3e-4, 0.71), 15),   # points 3e-4 from the edges: near panels
    ("circle20", (-0.8, -0.8), (0.8, 0.8), 13),
    ("graded_L", (-0.2, -0.2), (1.2, 1.2), 15),
])
def test_field_grid_matches_oracle(mesh, ll, ur, n):
    kinds, par = MESHES[mesh]()
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=9), proj=False)
    w, k, c_o, c_i = WAVES[0], 3.1, 1.0, 4.0
    tr = api.tp_solve(so, w, k, c_o, c_i)
    for total in (False, True):
        S, gx, gy = api.tp_field_grid(so, w, k, c_o, c_i, 8, ll, ur, n, n, total_field=total, traces=tr)
        pts = list(zip(gx.ravel(order="F"), gy.ravel(order="F")))
        ref = O.field_points(kinds, par, tr, w, k, c_o, c_i, 8, pts, total_field=total)
        got = S.ravel(order="F")
        scale = np.max(np.abs(ref))
        err = np.abs(got - ref)
        assert np.max(err) <= 1e-8 * scale, (np.argmax(err), np.max(err) / scale)


def test_field_grid_solves_when_no_traces_given_and_transparent_scatterer():
    kinds, par = geometry.circle(0.5, 40)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=9), proj=False)
    w, k = api.wave("Plane", 1.0, angle=0.4), 2.0
    S, gx, gy = api.tp_field_grid(so, w, k, 1.0, 1.0, 12, (-1.0, -1.0), (1.0, 1.0), 21, 21, total_field=True)
    u, _ = api.incoming_eval(w, k, np.c_[gx.ravel(), gy.ravel()])
    r = np.hypot(gx.ravel(), gy.ravel())
    away = np.abs(r - 0.5) > 0.1
    assert np.max(np.abs(S.ravel() - u)[away]) < 5e-3


def _analytic_circle(a, k, n_i, eps, x, y):
    """Transmission by a circle of radius eps (c_o = 1, c_i = n_i) of the incoming
    wave sum_n a_n J_n(k r) e^(i n theta): total field u_i + sum a_n R_n H_n(k r) e^(i n theta)
    outside, sum a_n T_n J_n(lambda k r) e^(i n theta) inside, lambda = sqrt(n_i)
    (source/utilities/gen_sol.cpp:29-110), with R_n, T_n from continuity of u and du/dr."""
    from scipy.special import jv, jvp, hankel1, h1vp
    lam = math.sqrt(n_i)
    r, th = math.hypot(x, y), math.atan2(y, x)
    u = 0j
    for n, an in a.items():
        ke = k * eps
        den = h1vp(n, ke) * jv(n, lam * ke) - lam * jvp(n, lam * ke) * hankel1(n, ke)
        R = (lam * jvp(n, lam * ke) * jv(n, ke) - jvp(n, ke) * jv(n, lam * ke)) / den
        T = (jv(n, ke) + R * hankel1(n, ke)) / jv(n, lam * ke)
        e = np.exp(1j * n * th)
        if r < eps:
            u += an * T * jv(n, lam * k * r) * e
        else:
            u += an * (jv(n, k * r) + R * hankel1(n, k * r)) * e
    return u


def test_field_converges_to_the_analytic_circle_solution():
    """The whole chain -- incoming circular waves, transmission solve, trace splines,
    Green representation on the grid -- against the Bessel-series solution of the
    circle, on two meshes: the error is small and falls with the panel size."""
    rng = np.random.default_rng(5)
    a = {n: float(rng.uniform(-1, 1)) for n in range(-3, 4)}
    waves = [api.wave("CircularJ", an, order=n) for n, an in a.items()]
    k, n_i, eps = 2.0, 4.0, 0.5
    errs = []
    for N in (40, 80):
        so = api.SolutionsOperator(api.BuilderData(geometry.circle(eps, N), order=11), proj=False)
        S, gx, gy = api.tp_field_grid(so, waves, k, 1.0, n_i, 16, (-1.2, -1.2), (1.2, 1.2), 25, 25, total_field=True)
        err, top = 0.0, 0.0
        for s, x, y in zip(S.ravel(), gx.ravel(), gy.ravel()):
            if abs(math.hypot(x, y) - eps) < 0.1:
                continue
            ref = _analytic_circle(a, k, n_i, eps, x, y)
            err = max(err, abs(s - ref))
            top = max(top, abs(ref))
        errs.append(err / top)
    assert errs[1] < 1e-5 and errs[1] < errs[0] / 4, errs   # 1.4e-5 -> 1.4e-6 in the oracle
