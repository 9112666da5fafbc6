"""Parity at the benchmark configurations themselves, at full size.

* The plain resonance search of the bench line (circle r = 0.25, N = 50 arcs,
  c_i = 23.4, Gauss order 11, 200 grid points on [0.5, 10], Newton to 1e-8) against
  the oracle's search on the same workload (committed fixture
  tests/golden/plain_search_circle_N50.json, made by tests/golden/gen_plain_roots.py):
  the same roots to |dk| <= 1e-8, sigma on the grid to 1e-10.
* A star polygon of lines (12 vertices, N = 48, c_i = 9, order 9, 200 points on
  [1, 12]; fixture tests/golden/plain_search_star12_N48.json with its panels): the
  same checks through the verified search (every pipeline feature: grid chunks,
  two-CTA dense sigma, Taylor-polynomial Newton steps and check points), 33 roots.
* The assembly-at-scale configuration (seeded star polygon, 24 vertices, N = 1000
  lines, Gauss order 16, k = 20, c_i = 4, c_o = 1, d <= 2): V, K, W and their k
  derivatives for both media and the projected T, T', T'' against the oracle's
  GalerkinBuilder / SolutionsOperator restatement at 1e-12 relative Frobenius.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_plain_search_circle_N50_matches_oracle_roots():
    with open(os.path.join(HERE, "golden", "plain_search_circle_N50.json")) as f:
        gold = json.load(f)
    cfg = gold["config"]
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(cfg["radius"], cfg["N"]), order=cfg["order"]))
    roots, grid, nev = so.find_resonances_plain(cfg["k_min"], cfg["k_max"], cfg["npoints"], cfg["c_o"], cfg["c_i"],
                                                tol=cfg["tol"])
    osig = np.array(gold["grid_sigma"])
    assert np.max(np.abs(grid[:, 0] - osig) / osig) <= 1e-10
    oroots = np.array(gold["roots"])
    assert len(roots) == len(oroots) == 10
    dk = np.abs(np.sort(roots) - np.sort(oroots))
    assert dk.max() <= 1e-8, dk
    # every GPU root brackets a sign change of sigma' within the tolerance
    lo = so.sweep_sigma(roots - cfg["tol"], cfg["c_o"], cfg["c_i"], d=1)[:, 1]
    hi = so.sweep_sigma(roots + cfg["tol"], cfg["c_o"], cfg["c_i"], d=1)[:, 1]
    assert np.all(lo <= 0) and np.all(hi >= 0)


def test_plain_search_star_polygon_matches_oracle_roots():
    with open(os.path.join(HERE, "golden", "plain_search_star12_N48.json")) as f:
        gold = json.load(f)
    cfg = gold["config"]
    kinds = np.array(gold["panel_kinds"], dtype=np.int32)
    par = np.array(gold["panel_params"], dtype=np.float64).reshape(len(kinds), -1)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=cfg["order"]))
    roots, grid, nev, chk = so.find_resonances_plain_verified(cfg["k_min"], cfg["k_max"], cfg["npoints"], cfg["c_o"],
                                                              cfg["c_i"], tol=cfg["tol"])
    osig = np.array(gold["grid_sigma"])
    assert np.max(np.abs(grid[:, 0] - osig) / osig) <= 1e-10
    oroots = np.array(gold["roots"])
    assert len(roots) == len(oroots) == 33
    assert np.abs(np.sort(roots) - np.sort(oroots)).max() <= 1e-8
    assert np.all(chk[:, 0] <= 0) and np.all(chk[:, 1] >= 0)


def test_assembly_star24_N1000_order16_full_size_vs_oracle():
    N, order, k, c_o, c_i = 1000, 16, 20.0, 1.0, 4.0
    kinds, par = geometry.polygon(*geometry.star_polygon(24, seed=2), N)
    data = api.BuilderData((kinds, par), order=order)
    gb = api.GalerkinBuilder(data)
    ob = O.Builder(kinds, par, order)
    for c in (c_i, c_o):
        gb.assembleDense(k, c, api.LayerType_ALL, 2)
        ref = ob.assemble(k, c, O.LAYER_ALL, 2)
        for t in range(3):
            assert rel(gb.getDoubleLayer(t), ref["K"][t]) <= 1e-12, ("K", c, t)
            assert rel(gb.getHypersingular(t), ref["W"][t]) <= 1e-12, ("W", c, t)
            assert rel(gb.getSingleLayer(t), ref["V"][t]) <= 1e-12, ("V", c, t)
        del ref
    so = api.SolutionsOperator(data)
    T = so.gen_sol_op_2nd_der(k, c_o, c_i)
    R = O.SolutionsOperator(ob).gen_sol_op(k, c_o, c_i, d=2)
    for t in range(3):
        assert rel(T[t], R[t]) <= 1e-12, ("T", t)
