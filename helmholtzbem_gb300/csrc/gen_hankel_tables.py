"""Generate hankel_tables.h: monomial coefficients for the large-argument Bessel
amplitudes used by the device Hankel routine.

For x >= 8 the device writes (DLMF 10.17)
    H_nu(x) = (x pi)^(-1/2) * [(P_nu + i Q_nu) (sin x +- cos x) combinations]
with, in w = 64/x^2 in (0, 1],
    P_0 = 1 + F0(w),  x Q_0 = -1/8 + G0(w),  P_1 = 1 + F1(w),  x Q_1 = 3/8 + G1(w),
F*, G* polynomials of degree DEG (least squares on Chebyshev points, samples from
mpmath at 40 digits), evaluated by Horner's rule.  Absolute error < 3e-18 on (0,1].
For x >= 16 (w <= 1/4) a second set of degree DEG_FAR reaches < 2e-18 there.

For 2 <= x < 8 the device evaluates J0, Y0, J1, Y1 by Taylor polynomials of degree
TAY_DEG about the centres 2.25, 2.75, ..., 7.75 (|x - centre| <= 1/4).  The
coefficients f^(m)(c)/m! come from the derivative rule
    Z_nu^(m)(x) = 2^-m sum_k (-1)^k C(m, k) Z_(nu - m + 2k)(x)
at 40 digits.  Truncation: below (1/4)^18/18! for J and (1/9)^18 relative for Y (whose
Taylor radius about c is c >= 2.25); the series' cancellation for 4 <= x < 8 is gone.

Usage (from the repository root):
    python helmholtzbem_gb300/csrc/gen_hankel_tables.py > helmholtzbem_gb300/csrc/hankel_tables.h
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40
DEG = 14
M = 64
DEG_FAR, W_FAR = 8, 0.25   # x >= 16: absolute error < 2e-18 on (0, 1/4]


def targets(w):
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
    y = -np.cos(np.pi * (k + 0.5) / M)
    wn = (y + 1) / 2
    vals = np.array([[float(v) for v in targets(w)] for w in wn])
    print("/* generated by gen_hankel_tables.py -- monomial coefficients in w = 64/x^2, lowest first */")
    print("#pragma once")
    print("#define HBEM_PQ_DEG %d" % DEG)
    for name, c in zip(["HBEM_F0", "HBEM_G0", "HBEM_F1", "HBEM_G1"], range(4)):
        cf = np.polynomial.chebyshev.chebfit(y, vals[:, c], DEG)
        mono = np.polynomial.chebyshev.cheb2poly(cf)
        P = np.polynomial.Polynomial(mono)(np.polynomial.Polynomial([-1.0, 2.0]))
        print("static __device__ __constant__ double %s[%d] = {" % (name, DEG + 1))
        print(",\n".join("  %.17e" % v for v in P.coef))
        print("};")
    # x >= 16 (w <= 1/4): the same amplitudes to the same accuracy with degree DEG_FAR
    wf = (y + 1) / 2 * W_FAR
    valsf = np.array([[float(v) for v in targets(w)] for w in wf])
    print("#define HBEM_PQ_DEG_FAR %d" % DEG_FAR)
    for name, c in zip(["HBEM_F0F", "HBEM_G0F", "HBEM_F1F", "HBEM_G1F"], range(4)):
        cf = np.polynomial.chebyshev.chebfit(y, valsf[:, c], DEG_FAR)
        mono = np.polynomial.chebyshev.cheb2poly(cf)
        P = np.polynomial.Polynomial(mono)(np.polynomial.Polynomial([-1.0, 2.0 / W_FAR]))
        print("static __device__ __constant__ double %s[%d] = {" % (name, DEG_FAR + 1))
        print(",\n".join("  %.17e" % v for v in P.coef))
        print("};")
    # ascending-series constants, index k = 1..SER_N (entry 0 unused):
    # 1/k^2, H_k, 1/(k+1), H_k/(k+1) -- exact rationals rounded once
    from fractions import Fraction
    ser_n = 48
    H = Fraction(0)
    rows = {"HBEM_SER_IK2": [0.0], "HBEM_SER_H": [0.0], "HBEM_SER_IK1": [0.0], "HBEM_SER_HK1": [0.0]}
    for k in range(1, ser_n + 1):
        H += Fraction(1, k)
        rows["HBEM_SER_IK2"].append(float(Fraction(1, k * k)))
        rows["HBEM_SER_H"].append(float(H))
        rows["HBEM_SER_IK1"].append(float(Fraction(1, k + 1)))
        rows["HBEM_SER_HK1"].append(float(H / (k + 1)))
    print("#define HBEM_SER_N %d" % ser_n)
    for name, vals_ in rows.items():
        print("static __device__ __constant__ double %s[%d] = {" % (name, ser_n + 1))
        print(",\n".join("  %.17e" % v for v in vals_))
        print("};")
    taylor_tables()


TAY_X0, TAY_W, TAY_N, TAY_DEG = 2, 0.5, 12, 17


def taylor_tables():
    """HBEM_TAY[i][m][f]: coefficient of (x - c_i)^m, c_i = 2.25 + i/2, for f = J0, Y0,
    J1, Y1 (global memory: the interval differs from lane to lane)."""
    print("#define HBEM_TAY_N %d" % TAY_N)
    print("#define HBEM_TAY_DEG %d" % TAY_DEG)
    print("static __device__ __align__(16) const double HBEM_TAY[%d][%d][4] = {" % (TAY_N, TAY_DEG + 1))
    blocks = []
    for i in range(TAY_N):
        c = mp.mpf(TAY_X0) + mp.mpf(TAY_W) * i + mp.mpf(TAY_W) / 2
        rows = []
        for m in range(TAY_DEG + 1):
            vals = []
            for fn, nu in ((mp.besselj, 0), (mp.bessely, 0), (mp.besselj, 1), (mp.bessely, 1)):
                d = mp.mpf(0)
                for k in range(m + 1):
                    d += (-1) ** k * mp.binomial(m, k) * fn(nu - m + 2 * k, c)
                vals.append(d / (mp.mpf(2) ** m * mp.factorial(m)))
            rows.append("  {" + ", ".join("%.17e" % float(v) for v in vals) + "}")
        blocks.append(" {\n" + ",\n".join(rows) + "}")
    print(",\n".join(blocks))
    print("};")


if __name__ == "__main__":
    main()
