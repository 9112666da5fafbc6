"""Generate the oracle's Chebyshev tables for the large-argument Bessel amplitudes.

For x >= 8 the oracle writes (DLMF 10.17 modulus/phase form)

    J_nu(x) + i Y_nu(x) = sqrt(2/(pi x)) (P_nu(x) + i Q_nu(x)) exp(i (x - (2 nu + 1) pi/4))

and approximates, in w = 64/x^2 on [0, 1],

    f0(w) = P_0(x) - 1,   g0(w) = x Q_0(x) + 1/8,
    f1(w) = P_1(x) - 1,   g1(w) = x Q_1(x) - 3/8

by Chebyshev series in (2w - 1), evaluated with Clenshaw's recurrence.  The
samples come from mpmath at 40 digits.  This is test infrastructure: the
product's tables are generated separately (monomial form, different degree).

Usage:  python oracle/gen_pq_cheb.py > oracle/pq_cheb.h
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40
DEG = 17
M = 80


def amplitudes(w):
    x = 8 / mp.sqrt(mp.mpf(w))
    out = []
    for nu in (0, 1):
        J, Y = mp.besselj(nu, x), mp.bessely(nu, x)
        chi = x - (2 * nu + 1) * mp.pi / 4
        s = mp.sqrt(mp.pi * x / 2)
        P = s * (J * mp.cos(chi) + Y * mp.sin(chi))
        Q = s * (Y * mp.cos(chi) - J * mp.sin(chi))
        out += [P - 1, x * Q + (mp.mpf(1) / 8 if nu == 0 else -mp.mpf(3) / 8)]
    return out


def main():
    k = np.arange(M)
    y = -np.cos(np.pi * (k + 0.5) / M)           # Chebyshev points in (-1, 1)
    vals = np.array([[float(v) for v in amplitudes((yy + 1) / 2)] for yy in y])
    names = ["ORC_F0", "ORC_G0", "ORC_F1", "ORC_G1"]
    print("/* generated by oracle/gen_pq_cheb.py; Chebyshev coefficients in (2w-1), w = 64/x^2 */")
    print("#pragma once")
    print("#define ORC_PQ_DEG %d" % DEG)
    for n, c in zip(names, range(4)):
        cf = np.polynomial.chebyshev.chebfit(y, vals[:, c], DEG)
        print("static const double %s[%d] = {" % (n, DEG + 1))
        print(",\n".join("  %.17e" % v for v in cf))
        print("};")


if __name__ == "__main__":
    main()
