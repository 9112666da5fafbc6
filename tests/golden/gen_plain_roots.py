"""Generate the oracle's plain resonance searches used as golden fixtures:

* tests/golden/plain_search_circle_N50.json: the circle workload (radius 0.25, N = 50
  arc panels, c_i = 23.4, c_o = 1, Gauss order 11, P1/P1, grid k_i = 0.5 + i (10 -
  0.5) / 199, i = 0..199, Newton to |dk| <= 1e-8);
* tests/golden/plain_search_star12_N48.json: a star polygon (12 vertices, seed 5,
  geometry.star_polygon) split into N = 48 lines by the library's
  make_N_polygonal_panels (panel parameters stored in the file), c_i = 9, c_o = 1,
  Gauss order 9, 200 points on [1, 12], Newton to 1e-8.

The search is examples/roots_newton_polygon_rsvd.cpp:172-265 with dense sigma,
restated by oracle/oracle.py (``SweepPool.plain_sweep``; the same iterates as
``plain_sweep``).  Run from the repository root (the polygon case needs the built
library for its panels):

    python tests/golden/gen_plain_roots.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

CFG = dict(radius=0.25, N=50, c_i=23.4, c_o=1.0, order=11, k_min=0.5, k_max=10.0, npoints=200, tol=1e-8)


POLY = dict(vertices=12, seed=5, N=48, c_i=9.0, c_o=1.0, order=9, k_min=1.0, k_max=12.0, npoints=200, tol=1e-8)


def search(kinds, par, cfg, name, extra=None):
    from oracle import oracle as O
    h = (cfg["k_max"] - cfg["k_min"]) / (cfg["npoints"] - 1)
    ks = cfg["k_min"] + h * np.arange(cfg["npoints"])
    with O.SweepPool(kinds, par, cfg["order"], cfg["c_o"], cfg["c_i"]) as pool:
        roots, sig, nev = pool.plain_sweep(ks, tol=cfg["tol"])
        ok = pool.verify(roots, tol=cfg["tol"])
    out = {"config": cfg, "grid_sigma": [float(v) for v in sig], "roots": [float(r) for r in roots],
           "verified": [bool(v) for v in ok], "evaluations": int(nev),
           "generator": "tests/golden/gen_plain_roots.py (oracle/oracle.py SweepPool.plain_sweep)"}
    if extra:
        out.update(extra)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), name), "w") as f:
        json.dump(out, f, indent=1)
    print(name, len(roots), "roots,", int(ok.sum()), "verified")


def main():
    from oracle import oracle as O
    if "--polygon-only" not in sys.argv:
        kinds, par = O.circle_panels(CFG["radius"], CFG["N"])
        search(kinds, par, CFG, "plain_search_circle_N50.json")
    from helmholtzbem_gb300 import geometry
    kinds, par = geometry.polygon(*geometry.star_polygon(POLY["vertices"], seed=POLY["seed"]), POLY["N"])
    kinds = np.asarray(kinds, dtype=np.int32)
    par = np.asarray(par, dtype=np.float64)
    search(kinds, par, POLY, "plain_search_star12_N48.json",
           {"panel_kinds": [int(v) for v in kinds], "panel_params": [float(v) for v in par.ravel()]})


if __name__ == "__main__":
    main()
