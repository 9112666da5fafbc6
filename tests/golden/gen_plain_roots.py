"""Generate tests/golden/plain_search_circle_N50.json: the oracle's plain resonance
search on the circle workload (radius 0.25, N = 50 arc panels, c_i = 23.4, c_o = 1,
Gauss order 11, P1/P1, grid k_i = 0.5 + i (10 - 0.5) / 199, i = 0..199, Newton to
|dk| <= 1e-8).  The search is examples/roots_newton_polygon_rsvd.cpp:172-265 with
dense sigma, restated by oracle/oracle.py (``SweepPool.plain_sweep``; the same
iterates as ``plain_sweep``).  Run from the repository root:

    python tests/golden/gen_plain_roots.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

CFG = dict(radius=0.25, N=50, c_i=23.4, c_o=1.0, order=11, k_min=0.5, k_max=10.0, npoints=200, tol=1e-8)


def main():
    from oracle import oracle as O
    kinds, par = O.circle_panels(CFG["radius"], CFG["N"])
    h = (CFG["k_max"] - CFG["k_min"]) / (CFG["npoints"] - 1)
    ks = CFG["k_min"] + h * np.arange(CFG["npoints"])
    with O.SweepPool(kinds, par, CFG["order"], CFG["c_o"], CFG["c_i"]) as pool:
        roots, sig, nev = pool.plain_sweep(ks, tol=CFG["tol"])
        ok = pool.verify(roots, tol=CFG["tol"])
    out = {"config": CFG, "grid_sigma": [float(v) for v in sig], "roots": [float(r) for r in roots],
           "verified": [bool(v) for v in ok], "evaluations": int(nev),
           "generator": "tests/golden/gen_plain_roots.py (oracle/oracle.py SweepPool.plain_sweep)"}
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "plain_search_circle_N50.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(len(roots), "roots,", int(ok.sum()), "verified")


if __name__ == "__main__":
    main()
