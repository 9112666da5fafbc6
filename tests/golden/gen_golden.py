"""Generate the golden Hankel vectors in tests/golden/hankel_mpmath.json.

Values of H0^(1), H1^(1) at real and complex arguments, computed with mpmath at
40 significant digits.  The arguments cover every branch boundary of the
real-argument evaluator (1e-8, 8, 1e6) and a spread of complex arguments with
0 <= Im z <= 3.  Run from the repository root:

    python tests/golden/gen_golden.py
"""
import json
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 40


def main():
    rng = np.random.default_rng(20240611)
    xr = [1e-12, 3e-9, 9.99e-9, 1.0001e-8, 1e-6, 1e-3, 0.1, 0.5, 1.0, 2.0, 2.404825557695773, 3.0,
          3.831705970207512, 5.0, 7.0, 7.9999, 8.0, 8.0001, 8.5, 10.0, 12.5, 20.0, 40.0, 77.7, 123.456,
          400.0, 999.9, 1e4, 1e5, 9.99e5, 1.0001e6, 3e6]
    xr += list(rng.uniform(0.0, 8.0, 40)) + list(rng.uniform(8.0, 500.0, 40))
    zc = [complex(a, b) for a, b in zip(rng.uniform(0.05, 40.0, 60), rng.uniform(0.0, 3.0, 60))]
    zc += [1.5 + 0.5j, 2.0 + 0.01j, 19.99 + 1j, 20.01 + 1j, 0.3 + 0.001j, 12 + 1e-4j, 5 + 2j]
    real = [{"x": float(x), "h0": [float(mp.besselj(0, x)), float(mp.bessely(0, x))],
             "h1": [float(mp.besselj(1, x)), float(mp.bessely(1, x))]} for x in xr]
    cplx = []
    for z in zc:
        h0 = complex(mp.hankel1(0, mp.mpc(z.real, z.imag)))
        h1 = complex(mp.hankel1(1, mp.mpc(z.real, z.imag)))
        cplx.append({"z": [z.real, z.imag], "h0": [h0.real, h0.imag], "h1": [h1.real, h1.imag]})
    out = {
        "source": "mpmath %s at %d digits" % (mp.__version__, mp.mp.dps),
        "real": real,
        "complex": cplx,
        # Known answers from the reference's own tests (test/googletest/solutions_test.cpp:55-72)
        "reference_kats": {
            "J0(pi)": -0.304242177644093864202,
            "J0'(pi)": -0.284615343179752757345310599686,
            "H0'(0.1)": [-0.0499375, 6.45895],
            "H0'(0.1)_tol": 1.4901161193847656e-06,
        },
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hankel_mpmath.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
