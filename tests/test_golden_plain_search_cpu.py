"""The committed fixture of the oracle's plain search on the bench workload
(tests/golden/plain_search_circle_N50.json): its grid sigma at a few points,
recomputed by the oracle, and its roots, each of which the oracle's sigma'
brackets within 1e-8."""
import json
import os

import numpy as np

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def _gold():
    with open(os.path.join(HERE, "golden", "plain_search_circle_N50.json")) as f:
        return json.load(f)


def test_fixture_grid_and_roots_are_the_oracles():
    gold = _gold()
    cfg = gold["config"]
    kinds, par = O.circle_panels(cfg["radius"], cfg["N"])
    oso = O.SolutionsOperator(O.Builder(kinds, par, cfg["order"]))
    h = (cfg["k_max"] - cfg["k_min"]) / (cfg["npoints"] - 1)
    for i in (0, 57, 199):
        s = O.sv_derivs(oso.gen_sol_op(cfg["k_min"] + i * h, cfg["c_o"], cfg["c_i"])[0])[0]
        # the fixture's assembly ran single-threaded: summation order differs from here
        assert abs(s - gold["grid_sigma"][i]) <= 1e-11 * s
    assert len(gold["roots"]) == 10 and all(gold["verified"])
    r = gold["roots"][3]
    lo = O.sv_derivs(*oso.gen_sol_op(r - cfg["tol"], cfg["c_o"], cfg["c_i"], d=1))[1]
    hi = O.sv_derivs(*oso.gen_sol_op(r + cfg["tol"], cfg["c_o"], cfg["c_i"], d=1))[1]
    assert lo <= 0.0 <= hi
    # every root lies inside a bracket [k_i, k_i+2] around a grid minimum
    sig = np.array(gold["grid_sigma"])
    mins = [i for i in range(sig.size - 2) if sig[i] > sig[i + 1] < sig[i + 2]]
    for r in gold["roots"]:
        assert any(cfg["k_min"] + i * h <= r <= cfg["k_min"] + (i + 2) * h for i in mins)


def test_polygon_fixture_grid_and_roots_are_the_oracles():
    with open(os.path.join(HERE, "golden", "plain_search_star12_N48.json")) as f:
        gold = json.load(f)
    cfg = gold["config"]
    kinds = np.array(gold["panel_kinds"], dtype=np.int32)
    par = np.array(gold["panel_params"], dtype=np.float64).reshape(len(kinds), -1)
    oso = O.SolutionsOperator(O.Builder(kinds, par, cfg["order"]))
    h = (cfg["k_max"] - cfg["k_min"]) / (cfg["npoints"] - 1)
    for i in (0, 101, 199):
        s = O.sv_derivs(oso.gen_sol_op(cfg["k_min"] + i * h, cfg["c_o"], cfg["c_i"])[0])[0]
        assert abs(s - gold["grid_sigma"][i]) <= 1e-11 * s
    assert len(gold["roots"]) == 33 and all(gold["verified"])
    r = gold["roots"][17]
    lo = O.sv_derivs(*oso.gen_sol_op(r - cfg["tol"], cfg["c_o"], cfg["c_i"], d=1))[1]
    hi = O.sv_derivs(*oso.gen_sol_op(r + cfg["tol"], cfg["c_o"], cfg["c_i"], d=1))[1]
    assert lo <= 0.0 <= hi
