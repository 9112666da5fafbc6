// Incoming waves on the device (namespace incoming, include/incoming.hpp,
// source/utilities/incoming.cpp:95-229): plane waves, circular waves J_l / Y_l,
// Fourier-Hankel waves J_l +- i Y_l and Herglotz waves, their values and gradients.
// A wave is a sum of records of 7 doubles: type, amplitude, x0, y0, angle, eps,
// order (the fields of incoming::wavespec_t).
#pragma once
#include "hbem_device.cuh"

namespace hbem {

enum WaveKind : int {
    WAVE_PLANE = 0,
    WAVE_CIRCULAR_J = 1,
    WAVE_CIRCULAR_Y = 2,
    WAVE_FOURIER_HANKEL1 = 3,
    WAVE_FOURIER_HANKEL2 = 4,
    WAVE_HERGLOTZ = 5
};
constexpr int kWaveDoubles = 7;
constexpr int kHerglotzNodes = 21;   // incoming.cpp:22, Gauss-Legendre on [0, 1]

// J_m(z), Y_m(z) for integer m and real z > 0.  J0, J1, Y0, Y1 from the real-argument
// Hankel evaluator; Y_m by upward recurrence (stable); J_m by upward recurrence while
// m <= z, otherwise by Miller's backward recurrence from an even start index well
// above max(m, z), normalised with J0 + 2 (J2 + J4 + ...) = 1.  Negative orders:
// J_-m = (-1)^m J_m, Y_-m = (-1)^m Y_m.  z = 0: J_0 = 1, J_m = 0, Y_m = -inf.
static __device__ void bessel_jy(int l, double z, double& J, double& Y) {
    const int m = l < 0 ? -l : l;
    const double sgn = (l < 0 && (m & 1)) ? -1. : 1.;
    if (!(z > 0.)) {
        J = m == 0 ? 1. : 0.;
        Y = -CUDART_INF;
        return;
    }
    cplx h0, h1;
    hankel01_real(z, h0, h1);
    if (m == 0) {
        J = h0.re;
        Y = h0.im;
        return;
    }
    if (m == 1) {
        J = sgn * h1.re;
        Y = sgn * h1.im;
        return;
    }
    double ya = h0.im, yb = h1.im;
    for (int j = 1; j < m; ++j) {
        const double yn = (2. * j / z) * yb - ya;
        ya = yb;
        yb = yn;
    }
    Y = sgn * yb;
    if (m <= z) {
        double ja = h0.re, jb = h1.re;
        for (int j = 1; j < m; ++j) {
            const double jn = (2. * j / z) * jb - ja;
            ja = jb;
            jb = jn;
        }
        J = sgn * jb;
        return;
    }
    const int top = 2 * ((m + (int)sqrt(160. * m) + 24) / 2);
    double bnext = 0., b = 1., sum = 0., bm = 0.;
    for (int j = top; j > 0; --j) {            // b holds b_j, bnext b_(j+1); make b_(j-1)
        const double bprev = (2. * j / z) * b - bnext;
        bnext = b;
        b = bprev;
        if (j - 1 == m) bm = b;
        if (j - 1 >= 2 && ((j - 1) & 1) == 0) sum += b;
        if (fabs(b) > 1e200) {
            b *= 1e-200;
            bnext *= 1e-200;
            sum *= 1e-200;
            bm *= 1e-200;
        }
    }
    J = sgn * bm / (b + 2. * sum);
}

// u = sum of the wave records at (x, y) and, if grad, its gradient (ux, uy).
// Circular and Fourier-Hankel records need a real wavenumber (the caller checks).
static __device__ void wave_eval(const double* W, int nw, const double* g21, double kre, double kim, double x,
                                 double y, bool grad, cplx& u, cplx& ux, cplx& uy) {
    u = mk(0.);
    ux = mk(0.);
    uy = mk(0.);
    const cplx ik = mk(-kim, kre);
    for (int q = 0; q < nw; ++q) {
        const double* w = W + q * kWaveDoubles;
        const int type = (int)w[0];
        const double amp = w[1], px = x - w[2], py = y - w[3];
        if (type == WAVE_PLANE) {
            double sa, ca;
            sincos(w[4], &sa, &ca);
            const double s = px * ca + py * sa;
            const cplx e = cexp(mk(-kim * s, kre * s));
            u += amp * e;
            if (grad) {
                const cplx g = amp * (ik * e);
                ux += ca * g;
                uy += sa * g;
            }
        } else if (type == WAVE_HERGLOTZ) {
            const double lb = w[4] - w[5], h = 2. * w[5];
            cplx su = mk(0.), sx = mk(0.), sy = mk(0.);
            for (int j = 0; j < kHerglotzNodes; ++j) {
                double st, ct;
                sincos(lb + h * g21[j], &st, &ct);
                const double s = px * ct + py * st;
                const cplx e = g21[kHerglotzNodes + j] * cexp(mk(-kim * s, kre * s));
                su += e;
                sx += ct * e;
                sy += st * e;
            }
            u += amp * su;
            if (grad) {
                ux += amp * (ik * sx);
                uy += amp * (ik * sy);
            }
        } else {
            // circular J / Y and Fourier-Hankel: F_l(k r) e^(i l theta)
            const int l = (int)w[6];
            const double r = sqrt(px * px + py * py), th = atan2(py, px);
            double st, ct;
            sincos(th, &st, &ct);
            const cplx eil = cexp_i(l * th);
            double J0, Y0, Jm, Ym, Jp, Yp;
            bessel_jy(l, kre * r, J0, Y0);
            cplx f = mk(0.);
            const bool needJ = type != WAVE_CIRCULAR_Y, needY = type != WAVE_CIRCULAR_J;
            const double ysg = type == WAVE_FOURIER_HANKEL2 ? -1. : 1.;
            if (grad) {
                bessel_jy(l - 1, kre * r, Jm, Ym);
                bessel_jy(l + 1, kre * r, Jp, Yp);
            } else {
                Jm = Ym = Jp = Yp = 0.;
            }
            if (needJ) f += mk(J0);
            if (needY) f += mk(0., ysg * Y0);
            u += amp * (f * eil);
            if (grad) {
                // incoming.cpp:166-200: df/dr = k (F_(l-1) - F_(l+1)) / 2, df/dtheta = i l F_l
                cplx gx = mk(0.), gy = mk(0.);
                if (needJ) {
                    const cplx dfdr = mk(kre * (Jm - Jp) / 2.), dfdt = mk(0., l * J0);
                    if (r == 0.) {
                        if (l == 1 || l == -1) {
                            gx += dfdr * ct - mk(0., st * kre * 0.5);
                            gy += dfdr * st + mk(0., ct * kre * 0.5);
                        } else {
                            gx += dfdr * ct;
                            gy += dfdr * st;
                        }
                    } else {
                        gx += dfdr * ct - (st / r) * dfdt;
                        gy += dfdr * st + (ct / r) * dfdt;
                    }
                }
                if (needY && r != 0.) {
                    const cplx dfdr = mk(0., ysg * kre * (Ym - Yp) / 2.), dfdt = mk(-ysg * l * Y0, 0.);
                    gx += dfdr * ct - (st / r) * dfdt;
                    gy += dfdr * st + (ct / r) * dfdt;
                }
                ux += amp * (gx * eil);
                uy += amp * (gy * eil);
            }
        }
    }
}

}  // namespace hbem
