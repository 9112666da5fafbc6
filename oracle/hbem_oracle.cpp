/*
 * hbem_oracle.cpp -- CPU restatement of HelmholtzBEM's assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls this
 * file; only the tests, the smoke check and the CPU-baseline leg of bench.py
 * use it, and only as the checker / the timed CPU baseline.
 *
 * It restates, formula by formula, the reference's CPU path (Eigen/TBB C++,
 * which cannot be compiled here: Eigen 3.3, TBB, GSL and H2Lib are absent):
 *   include/gauleg.hpp:35-168                   Gauss-Legendre + graded composite rule
 *   source/parametrizations/parametrized_line.cpp:20-144, parametrized_circular_arc.cpp:18-152
 *   include/continuous_space.hpp:33-152, include/discontinuous_space.hpp:33-127
 *   source/utilities/cbessel.cpp:1707-2017      real-argument H0/H1 branch structure
 *   source/utilities/cbessel.cpp:1210-1287      complex-argument H0/H1 (restated from the
 *                                               published methods, see hankel_cplx below)
 *   source/galerkin_builder.cpp:17-1018         BuilderData tables, pair classification,
 *                                               coincident/adjacent/general local matrices,
 *                                               scatter, x i/4
 *   source/mass_matrix.cpp:6-47                 mass matrix
 *   source/utilities/gen_sol_op.cpp:23-196      T(k) blocks and the mass projection
 *
 * Parity status: Hankel values are pinned against the reference's own known
 * answers (test/googletest/solutions_test.cpp:55-72) and against mpmath /
 * scipy (AMOS); operator matrices are NOT pinned by reference fixtures (the
 * reference's golden rows are absolute paths on the author's machine and are
 * absent), so at matrix level parity is unpinned and checked analytically
 * (circle eigenvalues, finite differences) instead.
 *
 * Deliberate divergences from the reference's literal behaviour (intended
 * semantics are restated; each has a switch where cheap):
 *   - gen_sol_op.cpp:151,194-195 write every derivative into T; here T' / T''
 *     receive the projected derivative blocks (no mass term).
 *   - galerkin_builder.cpp:749 copies res(j,i) of the order-0 block into every
 *     derivative order of the coincident single-layer block; here the matching
 *     derivative entry is copied (set quirk_sl_coinc=1 to reproduce literally).
 *   - galerkin_builder.cpp:984-1009 adds uninitialised SL/HY workspaces for
 *     j > i pairs when test != trial; here those pairs add nothing.
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "pq_cheb.h"

typedef std::complex<double> cd;
static const double EPS = 2.220446049250313e-16;
static const double PI = 3.14159265358979323846;
static const double EULER_GAMMA = 0.57721566490153286061;

/* ------------------------------------------------------------------ quadrature */

/* include/gauleg.hpp:35-79: Newton on the three-term Legendre recurrence. */
static void gauleg(double a, double b, int n, double eps, double *xq, double *wq) {
    int m = (n + 1) / 2;
    double xmid = 0.5 * (a + b), xlen = 0.5 * (b - a);
    for (int i = 0; i < m; ++i) {
        double z = std::cos(PI * (i + 1 - 0.25) / (n + 0.5)), z1, p1, p2, p3, dp1;
        int guard = 0;
        do {
            p1 = 1.; p2 = 0.;
            for (int j = 1; j <= n; ++j) {
                p3 = p2; p2 = p1;
                p1 = ((2. * j - 1.) * z * p2 - (j - 1.) * p3) / j;
            }
            dp1 = n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / dp1;
        } while (std::fabs(z - z1) > eps && ++guard < 100);
        xq[i] = xmid - xlen * z;
        xq[n - 1 - i] = xmid + xlen * z;
        double wqi = 2. * xlen / ((1. - z * z) * dp1 * dp1);
        wq[i] = wqi;
        wq[n - 1 - i] = wqi;
    }
}

/* include/gauleg.hpp:89-121: geometrically graded composite rule on [0,1],
 * levels [s^(l+1), s^l] with s = (sqrt2-1)^2 and orders n, n-1, ..., 2. */
static void cgauleg_redux(int n, double eps, double *pts, double *wts) {
    int N = n * (n + 1) / 2 - 1;
    double sigma = (std::sqrt(2.) - 1.) * (std::sqrt(2.) - 1.);
    double xl = sigma, xr = 1.;
    int ii = N - 1, qq = n;
    std::vector<double> xg(n), wg(n);
    for (int i = 1; i < n; ++i) {
        gauleg(0, 1, qq, eps, xg.data(), wg.data());
        for (int j = qq - 1; j >= 0; --j) {
            wts[ii] = (xr - xl) * wg[j];
            pts[ii] = (xr - xl) * xg[j] + xl;
            --ii;
        }
        --qq;
        xr = xl;
        xl = xl * sigma;
    }
}

/* ------------------------------------------------------------------ panels */

struct Panel {
    int kind;            /* 0 = line, 1 = circular arc */
    double p[5];         /* line: x1 y1 x2 y2 ; arc: cx cy r phi0 phi1 */
};

/* point on [0,1] (operator[]) */
static inline cd pan_op01(const Panel &P, double t) {
    if (P.kind == 0) {
        double x1 = P.p[0], y1 = P.p[1], x2 = P.p[2], y2 = P.p[3];
        return cd(x2 - x1, y2 - y1) * t + cd(x1, y1);
    }
    double d = P.p[4] - P.p[3];
    return cd(P.p[0], P.p[1]) + P.p[2] * std::exp(cd(0., t * d + P.p[3]));
}
/* reversed point on [0,1] (swapped_op) */
static inline cd pan_swapped(const Panel &P, double t) {
    if (P.kind == 0) {
        double x1 = P.p[0], y1 = P.p[1], x2 = P.p[2], y2 = P.p[3];
        return cd(x1 - x2, y1 - y2) * t + cd(x2, y2);
    }
    double d = P.p[3] - P.p[4];
    return cd(P.p[0], P.p[1]) + P.p[2] * std::exp(cd(0., t * d + P.p[4]));
}
/* point on [-1,1] (operator()) -- used for the adjacency test */
static inline cd pan_op11(const Panel &P, double t) {
    if (P.kind == 0) {
        double x1 = P.p[0], y1 = P.p[1], x2 = P.p[2], y2 = P.p[3];
        return cd(t * (x2 - x1) + (x2 + x1), t * (y2 - y1) + (y2 + y1)) * 0.5;
    }
    double mean = (P.p[3] + P.p[4]) / 2., diff = (P.p[4] - P.p[3]) / 2.;
    return cd(P.p[0] + P.p[2] * std::cos(t * diff + mean), P.p[1] + P.p[2] * std::sin(t * diff + mean));
}
/* tangent on [0,1] (Derivative_01) and its norm */
static inline cd pan_d01(const Panel &P, double t, double *nrm) {
    if (P.kind == 0) {
        cd z(P.p[2] - P.p[0], P.p[3] - P.p[1]);
        *nrm = std::abs(z);
        return z;
    }
    double d = P.p[4] - P.p[3];
    *nrm = P.p[2] * std::fabs(d);
    return cd(0., 1.) * P.p[2] * d * std::exp(cd(0., t * d + P.p[3]));
}
/* tangent of the reversed map (Derivative_01_swapped) */
static inline cd pan_d01_sw(const Panel &P, double t, bool neg, double *nrm) {
    double s = neg ? -1. : 1.;
    if (P.kind == 0) {
        cd z(P.p[0] - P.p[2], P.p[1] - P.p[3]);
        *nrm = std::abs(z);
        return s * z;
    }
    double d = P.p[3] - P.p[4];
    *nrm = P.p[2] * std::fabs(d);
    return s * cd(0., 1.) * P.p[2] * d * std::exp(cd(0., t * d + P.p[4]));
}

/* ------------------------------------------------------------------ spaces */

struct Space {
    int q;               /* 2 = continuous P1, 1 = discontinuous P0 */
    double f(int i, double t) const { return q == 1 ? 1. : (i == 0 ? t : 1. - t); }
    double fsw(int i, double t) const { return q == 1 ? 1. : (i == 0 ? 1. - t : t); }
    double df(int i) const { return q == 1 ? 0. : (i == 0 ? 1. : -1.); }
    double dfsw(int i) const { return q == 1 ? 0. : (i == 0 ? 1. : -1.); }
    /* LocGlobMap, 0-based in and out (continuous_space.hpp:38-47, discontinuous_space.hpp:38-45) */
    int map(int loc, int panel, int dim) const {
        if (q == 1) return panel;
        if (loc == 1) return panel;
        return ((panel + 1) % dim == 0) ? 0 : panel + 1;
    }
};

/* ------------------------------------------------------------------ Hankel, real argument */

static inline double cheb(const double *c, int deg, double y) {
    /* Clenshaw */
    double b1 = 0., b2 = 0.;
    for (int k = deg; k >= 1; --k) {
        double b0 = 2. * y * b1 - b2 + c[k];
        b2 = b1; b1 = b0;
    }
    return y * b1 - b2 + c[0];
}

/* Branch structure of Hankel1Real01::jy_01 (cbessel.cpp:1858-1997):
 *   x <= 0          : J0 = 1, J1 = Y0 = Y1 = 0
 *   x < 1e-8        : limiting forms (DLMF 10.7.2-10.7.4)
 *   x < 8           : ascending series (DLMF 10.8.1/10.8.2) with harmonic numbers
 *   8 <= x <= 1e6   : modulus/phase amplitudes P, Q (DLMF 10.17) -- here Chebyshev fits
 *   x > 1e6         : leading-order asymptotics (DLMF 10.17.3, first term)           */
static void hankel_real(double x, cd &h0, cd &h1) {
    double j0, j1, y0, y1;
    if (x <= 0.) {
        h0 = cd(1., 0.); h1 = cd(0., 0.);
        return;
    } else if (x < 1e-8) {
        j0 = 1.; j1 = .5 * x;
        y0 = (2. / PI) * (std::log(j1) + EULER_GAMMA);
        y1 = -(2. / PI) / x;
    } else if (x < 8.) {
        double x2_4 = x * x * 0.25, t = 1., Hk = 0., k = 1.;
        j0 = 1.; j1 = 1.; y0 = 0.; y1 = 0.;
        do {
            t *= -x2_4 / (k * k);
            Hk += 1.0 / k;
            j0 += t;
            y0 -= Hk * t;
            k += 1.0;
            j1 += t / k;
            y1 -= (Hk / k) * t;
        } while (Hk * std::fabs(t) > EPS && k <= 1000);
        j1 *= x * 0.5;
        double lg = std::log(x * 0.5) + EULER_GAMMA;
        y0 += lg * j0;
        y0 *= 2. / PI;
        y1 *= x;
        y1 += 2.0 * (lg * j1 + (j0 - 2.0) / x);
        y1 *= 1. / PI;
    } else if (x <= 1e6) {
        double w = 64. / (x * x), yv = 2. * w - 1.;
        double P0 = 1. + cheb(ORC_F0, ORC_PQ_DEG, yv);
        double Q0 = (cheb(ORC_G0, ORC_PQ_DEG, yv) - 0.125) / x;
        double P1 = 1. + cheb(ORC_F1, ORC_PQ_DEG, yv);
        double Q1 = (cheb(ORC_G1, ORC_PQ_DEG, yv) + 0.375) / x;
        /* phases x - pi/4, x - 3pi/4 through sin x +- cos x, exact in x */
        double r = 1. / std::sqrt(PI * x), sx = std::sin(x), cx = std::cos(x);
        double cc = sx + cx, ss = sx - cx;
        j0 = r * (P0 * cc - Q0 * ss);
        y0 = r * (P0 * ss + Q0 * cc);
        j1 = r * (P1 * ss + Q1 * cc);
        y1 = r * (Q1 * ss - P1 * cc);
    } else {
        double r = std::sqrt(2. / (PI * x));
        j0 = r * std::cos(x - PI / 4); y0 = r * std::sin(x - PI / 4);
        j1 = r * std::cos(x - 3 * PI / 4); y1 = r * std::sin(x - 3 * PI / 4);
    }
    h0 = cd(j0, y0);
    h1 = cd(j1, y1);
}

/* ------------------------------------------------------------------ Hankel, complex argument */

/* H0, H1 of the first kind for complex z (the reference calls HankelH1(0|1, z),
 * cbessel.cpp:1271-1287, an Amos-method routine).  Restated from the published
 * methods of that family:
 *   |z| <= 2        ascending series (DLMF 10.8.1/10.8.2), principal log
 *   2 < |z| < 20    Miller backward recurrence for J_n normalised by
 *                   J0 + 2 sum J_2k = 1 (DLMF 10.23.E? generating function at t=1,
 *                   10.12.E? ) and Neumann's series for Y0, Y1 (DLMF 10.23.E3 and its
 *                   derivative, using J_n' = (J_{n-1} - J_{n+1})/2)
 *   |z| >= 20       Hankel's asymptotic expansion (DLMF 10.17.5), terms until < eps
 * Non-finite results become 0 (galerkin_builder.cpp:216-235).                          */
static void hankel_cplx(cd z, cd &h0, cd &h1) {
    const cd I(0., 1.);
    double az = std::abs(z);
    cd j0, j1, y0, y1;
    if (az == 0.) {
        h0 = 0.; h1 = 0.;
        return;
    }
    if (az <= 2.) {
        cd x2_4 = z * z * 0.25, t = 1.;
        double Hk = 0., k = 1.;
        j0 = 1.; j1 = 1.; y0 = 0.; y1 = 0.;
        do {
            t *= -x2_4 / (k * k);
            Hk += 1.0 / k;
            j0 += t;
            y0 -= Hk * t;
            k += 1.0;
            j1 += t / k;
            y1 -= (Hk / k) * t;
        } while (Hk * std::abs(t) > 0.1 * EPS && k <= 1000);
        j1 *= z * 0.5;
        cd lg = std::log(z * 0.5) + EULER_GAMMA;
        y0 += lg * j0;
        y0 *= 2. / PI;
        y1 *= z;
        y1 += 2.0 * (lg * j1 + (j0 - 2.0) / z);
        y1 *= 1. / PI;
        h0 = j0 + I * y0;
        h1 = j1 + I * y1;
    } else if (az < 20.) {
        int nstart = 2 * (int)((az + 40.) / 2.);
        std::vector<cd> J(nstart + 2);
        J[nstart + 1] = 0.;
        J[nstart] = 1e-30;
        for (int n = nstart; n >= 1; --n) {
            J[n - 1] = (2. * n) / z * J[n] - J[n + 1];
            if (std::abs(J[n - 1]) > 1e200) {
                for (int m = n - 1; m <= nstart + 1; ++m) J[m] *= 1e-200;
            }
        }
        cd S = J[0];
        for (int n = 2; n <= nstart; n += 2) S += 2. * J[n];
        for (int n = 0; n <= nstart + 1; ++n) J[n] /= S;
        j0 = J[0]; j1 = J[1];
        cd sy0 = 0., sy1 = 0.;
        for (int k = 1; 2 * k + 1 <= nstart + 1; ++k) {
            double sg = (k & 1) ? -1. : 1.;
            sy0 += sg * J[2 * k] / (double)k;
            sy1 += sg * (J[2 * k - 1] - J[2 * k + 1]) / (double)k;
        }
        cd lg = std::log(z * 0.5) + EULER_GAMMA;
        y0 = (2. / PI) * lg * j0 - (4. / PI) * sy0;
        y1 = (2. / PI) * lg * j1 - (2. / PI) * j0 / z + (2. / PI) * sy1;
        h0 = j0 + I * y0;
        h1 = j1 + I * y1;
    } else {
        cd s[2];
        for (int nu = 0; nu < 2; ++nu) {
            double mu = 4. * nu * nu;
            cd sum = 1., term = 1.;
            for (int k = 1; k < 200; ++k) {
                double a = (mu - (2. * k - 1.) * (2. * k - 1.)) / (k * 8.);
                term *= I * a / z;
                sum += term;
                if (std::abs(term) < 0.25 * EPS) break;
            }
            s[nu] = sum;
        }
        cd r = std::sqrt(2. / (PI * z));
        h0 = r * std::exp(I * (z - PI / 4.)) * s[0];
        h1 = r * std::exp(I * (z - 3. * PI / 4.)) * s[1];
    }
    if (!std::isfinite(h0.real()) || !std::isfinite(h0.imag())) h0 = 0.;
    if (!std::isfinite(h1.real()) || !std::isfinite(h1.imag())) h1 = 0.;
}

/* ------------------------------------------------------------------ builder */

struct Builder {
    int npanels, p, nc;
    bool lines;
    Space test, trial;
    std::vector<Panel> pan;
    std::vector<double> xg, wg, xc, wc;
    /* k-dependent constants (initialize_constants, galerkin_builder.cpp:899-916) */
    cd k, ksqrtc, k2ch, ksqrtc_inv, ksqrtc_two;
    double c, sqrtc;
    bool k_rp;
    int quirk_sl_coinc;

    bool square() const { return test.q == trial.q; }

    /* BuilderData::is_adjacent (galerkin_builder.cpp:189-201) */
    bool is_adjacent(int i, int j, bool &swap) const {
        double e = EPS * 100.;
        if (std::abs(pan_op11(pan[i], 1) - pan_op11(pan[j], -1)) < e) { swap = false; return true; }
        if (std::abs(pan_op11(pan[i], -1) - pan_op11(pan[j], 1)) < e) { swap = true; return true; }
        return false;
    }
};

/* Per-pair geometry over an n x n node grid (column-major, index a + n*b). */
struct Geo {
    int n;
    std::vector<cd> v[2], tan[2], tanp[2], h0[2], h1[2];
    std::vector<double> vn[2], vn2[2], tn[2], tpn[2];
    void resize(int nn) {
        n = nn;
        for (int K = 0; K < 2; ++K) {
            v[K].resize(n * n); tan[K].resize(n * n); tanp[K].resize(n * n);
            h0[K].resize(n * n); h1[K].resize(n * n);
            vn[K].resize(n * n); vn2[K].resize(n * n); tn[K].resize(n * n); tpn[K].resize(n * n);
        }
    }
};

static inline void kernel_at(const Builder &B, double vnorm, cd &h0, cd &h1) {
    if (B.k_rp) hankel_real(B.ksqrtc.real() * vnorm, h0, h1);
    else hankel_cplx(B.ksqrtc * vnorm, h0, h1);
}

/* Node tables (BuilderData ctor, galerkin_builder.cpp:41-49):
 *   coincident: t = xc[b], s = t (1 - xc[a]), w = t wc[a] wc[b]
 *   adjacent:   t = xc[a], s = t xc[b],       w = t wc[a] wc[b]
 *   general:    s = xg[a], t = xg[b],         w = wg[a] wg[b]                        */
static inline void node_c(const Builder &B, int a, int b, double &s, double &t, double &w) {
    t = B.xc[b]; s = t * (1. - B.xc[a]); w = t * B.wc[a] * B.wc[b];
}
static inline void node_a(const Builder &B, int a, int b, double &s, double &t, double &w) {
    t = B.xc[a]; s = t * B.xc[b]; w = t * B.wc[a] * B.wc[b];
}
static inline void node_g(const Builder &B, int a, int b, double &s, double &t, double &w) {
    s = B.xg[a]; t = B.xg[b]; w = B.wg[a] * B.wg[b];
}

/* compute_coinciding (galerkin_builder.cpp:237-265) */
static void compute_coinciding(const Builder &B, int i, Geo &G) {
    int n = B.nc;
    G.resize(n);
    const Panel &P = B.pan[i];
    for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
        double s, t, w; node_c(B, a, b, s, t, w);
        int id = a + n * b;
        G.tanp[0][id] = pan_d01(P, t, &G.tpn[0][id]);
        G.tan[0][id] = pan_d01(P, s, &G.tn[0][id]);
        G.v[0][id] = pan_op01(P, s) - pan_op01(P, t);
        G.vn2[0][id] = std::norm(G.v[0][id]);
        G.vn[0][id] = std::sqrt(G.vn2[0][id]);
        kernel_at(B, G.vn[0][id], G.h0[0][id], G.h1[0][id]);
    }
}

/* compute_adjacent (galerkin_builder.cpp:267-306): both panels parametrised from
 * the shared vertex; K = 0 covers s < t, K = 1 the mirrored triangle.          */
static void compute_adjacent(const Builder &B, int i, int j, bool swap, Geo &G) {
    int n = B.nc;
    G.resize(n);
    const Panel &P = B.pan[i], &Q = B.pan[j];
    for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
        double sa, ta, w; node_a(B, a, b, sa, ta, w);
        int id = a + n * b;
        if (swap) {
            G.tanp[0][id] = pan_d01_sw(Q, ta, true, &G.tpn[0][id]);
            G.tanp[1][id] = pan_d01_sw(Q, sa, true, &G.tpn[1][id]);
            G.tan[0][id] = pan_d01(P, sa, &G.tn[0][id]);
            G.tan[1][id] = pan_d01(P, ta, &G.tn[1][id]);
            G.v[0][id] = pan_op01(P, sa) - pan_swapped(Q, ta);
            G.v[1][id] = pan_op01(P, ta) - pan_swapped(Q, sa);
        } else {
            G.tanp[0][id] = pan_d01(Q, ta, &G.tpn[0][id]);
            G.tanp[1][id] = pan_d01(Q, sa, &G.tpn[1][id]);
            G.tan[0][id] = pan_d01_sw(P, sa, true, &G.tn[0][id]);
            G.tan[1][id] = pan_d01_sw(P, ta, true, &G.tn[1][id]);
            G.v[0][id] = pan_swapped(P, sa) - pan_op01(Q, ta);
            G.v[1][id] = pan_swapped(P, ta) - pan_op01(Q, sa);
        }
        if (B.lines) {  /* line panels use a single (constant) tangent for both halves */
            G.tan[1][id] = G.tan[0][id]; G.tn[1][id] = G.tn[0][id];
            G.tanp[1][id] = G.tanp[0][id]; G.tpn[1][id] = G.tpn[0][id];
        }
        for (int K = 0; K < 2; ++K) {
            G.vn2[K][id] = std::norm(G.v[K][id]);
            G.vn[K][id] = std::sqrt(G.vn2[K][id]);
            kernel_at(B, G.vn[K][id], G.h0[K][id], G.h1[K][id]);
        }
    }
}

/* compute_general (galerkin_builder.cpp:308-327) */
static void compute_general(const Builder &B, int i, int j, Geo &G) {
    int n = B.p;
    G.resize(n);
    const Panel &P = B.pan[i], &Q = B.pan[j];
    for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
        double s, t, w; node_g(B, a, b, s, t, w);
        int id = a + n * b;
        G.tan[0][id] = pan_d01(P, s, &G.tn[0][id]);
        G.tanp[0][id] = pan_d01(Q, t, &G.tpn[0][id]);
        G.v[0][id] = pan_op01(P, s) - pan_op01(Q, t);
        G.vn2[0][id] = std::norm(G.v[0][id]);
        G.vn[0][id] = std::sqrt(G.vn2[0][id]);
        kernel_at(B, G.vn[0][id], G.h0[0][id], G.h1[0][id]);
    }
}

enum { CNC = 0, ADJ = 1, GEN = 2 };

/* Local result: res[layer] row-major Q x cols, cols = Q*(d+1) (x2 for DL transposed). */
struct Local {
    cd dl[2][12], hy[2][6], sl[2][6];
};

static inline double cross_vt(cd v, cd tau) { /* Im v Re tau - Re v Im tau */
    return v.imag() * tau.real() - v.real() * tau.imag();
}

/* double_layer_{coinciding,adjacent,general} (galerkin_builder.cpp:346-541).
 * The weighted shape products f_i(s) g_j(t) w are evaluated on the fly; the
 * "_t" variants evaluate test at t and trial at s.                             */
static void double_layer(const Builder &B, int kind, bool swap, int d, bool comp_t, const Geo &G, Local &L) {
    int Qte = B.test.q, Qtr = B.trial.q, step = (comp_t && kind != CNC) ? 2 : 1, n = G.n;
    for (int a = 0; a < 2; ++a) for (int b = 0; b < 12; ++b) L.dl[a][b] = 0.;
    int nK = (kind == GEN) ? 1 : 2;
    std::vector<double> vdn(n * n), vdnt(n * n);
    for (int K = 0; K < nK; ++K) {
        int gK = (kind == ADJ) ? K : 0;
        const std::vector<cd> &v = G.v[gK];
        const std::vector<double> &vn = G.vn[gK];
        /* orientation factors and the all-zero tests (isArrayZero) */
        bool zr = true, zr_t = true;
        for (int id = 0; id < n * n; ++id) {
            if (kind == CNC) {
                const cd &tau = (K == 0 ? G.tanp[0] : G.tan[0])[id];
                double tn = (K == 0 ? G.tn[0] : G.tpn[0])[id];
                vdn[id] = (K * 2 - 1.) * tn * cross_vt(v[id], tau);
            } else if (kind == ADJ) {
                vdn[id] = -cross_vt(v[id], G.tanp[K][id]) * G.tn[K][id];
                if (comp_t) vdnt[id] = cross_vt(v[id], G.tan[K][id]) * G.tpn[K][id];
            } else {
                vdn[id] = v[id].real() * G.tanp[0][id].imag() - v[id].imag() * G.tanp[0][id].real();
                if (comp_t) vdnt[id] = v[id].imag() * G.tan[0][id].real() - v[id].real() * G.tan[0][id].imag();
            }
            if (std::fabs(vdn[id]) >= EPS) zr = false;
            if (comp_t && kind != CNC && std::fabs(vdnt[id]) >= EPS) zr_t = false;
        }
        if (kind == GEN) {
            /* general: norm factors multiplied after the zero test */
            if (!zr) for (int id = 0; id < n * n; ++id) vdn[id] *= G.tn[0][id];
            if (comp_t && !zr_t) for (int id = 0; id < n * n; ++id) vdnt[id] *= G.tpn[0][id];
        }
        for (int pass = 0; pass < 2; ++pass) {
            if (pass == 0 && zr) continue;
            if (pass == 1 && (!comp_t || kind == CNC || zr_t)) continue;
            const std::vector<double> &vv = pass == 0 ? vdn : vdnt;
            for (int jj = 0; jj < Qtr; ++jj) for (int ii = 0; ii < Qte; ++ii) {
                cd s0 = 0., s1 = 0., s2 = 0.;
                for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
                    int id = a + n * b;
                    double s, t, w, fg;
                    if (kind == CNC) {
                        node_c(B, a, b, s, t, w);
                        fg = (K == 0 ? B.test.f(ii, s) * B.trial.f(jj, t) : B.test.f(ii, t) * B.trial.f(jj, s)) * w;
                    } else if (kind == ADJ) {
                        node_a(B, a, b, s, t, w);
                        /* K selects the triangle; pass selects normal / transposed block */
                        bool useT = (pass == 0) ? (K == 1) : (K == 0);
                        bool sw = (pass == 0) ? swap : !swap;
                        double x1 = useT ? t : s, x2 = useT ? s : t;
                        if (!sw) fg = B.test.fsw(ii, x1) * B.trial.f(jj, x2) * w;
                        else fg = B.test.f(ii, x1) * B.trial.fsw(jj, x2) * w;
                    } else {
                        node_g(B, a, b, s, t, w);
                        fg = (pass == 0 ? B.test.f(ii, s) * B.trial.f(jj, t) : B.test.f(ii, t) * B.trial.f(jj, s)) * w;
                    }
                    double cfr = vv[id] * fg;
                    cd m1 = vn[id] <= 0 ? cd(0.) : B.ksqrtc * G.h1[gK][id] / vn[id];
                    s0 += cfr * m1;
                    if (d) s1 += cfr * G.h0[gK][id];
                    if (d > 1) {
                        cd m3 = (kind == GEN) ? G.h0[gK][id] - m1 * G.vn2[gK][id]
                                              : G.h0[gK][id] - G.h1[gK][id] * B.ksqrtc * vn[id];
                        s2 += cfr * m3;
                    }
                }
                int off = pass == 0 ? 0 : Qtr;
                L.dl[ii][off + jj] += s0;
                if (d) L.dl[ii][step * Qtr + off + jj] += s1;
                if (d > 1) L.dl[ii][2 * step * Qtr + off + jj] += s2;
            }
        }
    }
    if (!d) return;
    for (int ii = 0; ii < Qte; ++ii) {
        for (int c = step * Qtr; c < 2 * step * Qtr; ++c) L.dl[ii][c] *= B.k * B.c;
        if (d > 1) for (int c = 2 * step * Qtr; c < 3 * step * Qtr; ++c) L.dl[ii][c] *= B.c;
    }
}

/* hypersingular_{coinciding,adjacent,general} (galerkin_builder.cpp:543-718) */
static void hypersingular(const Builder &B, int kind, bool swap, int d, const Geo &G, Local &L) {
    int Q = B.trial.q, n = G.n;
    for (int a = 0; a < 2; ++a) for (int b = 0; b < 6; ++b) L.hy[a][b] = 0.;
    int nK = (kind == GEN) ? 1 : 2;
    std::vector<double> tdt(n * n);
    bool tz = true;
    for (int K = 0; K < nK; ++K) {
        int gK = (kind == ADJ) ? K : 0;
        if (K == 0 || (kind == ADJ && !B.lines)) {   /* compute_tdottp / compute_tdottp_s */
            tz = true;
            if (B.lines) {
                const cd &z = G.tan[gK][0], &zp = G.tanp[gK][0];
                double vv = z.imag() * zp.imag() + z.real() * zp.real();
                tz = std::fabs(vv) < EPS;
                for (int id = 0; id < n * n; ++id) tdt[id] = 2. * vv;
            } else {
                for (int id = 0; id < n * n; ++id) {
                    const cd &z = G.tan[gK][id], &zp = G.tanp[gK][id];
                    tdt[id] = z.imag() * zp.imag() + z.real() * zp.real();
                    if (std::fabs(tdt[id]) >= EPS) tz = false;
                }
                for (int id = 0; id < n * n; ++id) tdt[id] *= 2.0;
            }
        }
        for (int jj = 0; jj < Q; ++jj) for (int ii = 0; ii < Q; ++ii) {
            if (kind == CNC && ii < jj) {   /* symmetry */
                for (int l = 0; l <= d; ++l) L.hy[ii][l * Q + jj] = L.hy[jj][l * Q + ii];
                continue;
            }
            cd r0 = 0., r1 = 0., r2 = 0.;
            for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
                int id = a + n * b;
                double s, t, w, arc, fg;
                if (kind == CNC) {
                    node_c(B, a, b, s, t, w);
                    int r = K > 0 ? jj : ii, cc = K > 0 ? ii : jj;
                    arc = B.trial.df(r) * B.trial.df(cc) * w;
                    fg = B.trial.f(r, s) * B.trial.f(cc, t) * w;
                } else if (kind == ADJ) {
                    node_a(B, a, b, s, t, w);
                    /* block (r, cc) of the table chosen by (swap, K) */
                    int r = K > 0 ? jj : ii, cc = K > 0 ? ii : jj;
                    bool use_swap_tab = swap ? (K == 0) : (K > 0);
                    if (!use_swap_tab) {  /* m_hyp_adj_fg(_arc): swapped(r, sa) * plain(cc, ta) */
                        arc = B.trial.dfsw(r) * B.trial.df(cc) * w;
                        fg = B.trial.fsw(r, s) * B.trial.f(cc, t) * w;
                    } else {              /* m_hyp_adj_fg_swap(_arc): plain(r, sa) * swapped(cc, ta) */
                        arc = B.trial.df(r) * B.trial.dfsw(cc) * w;
                        fg = B.trial.f(r, s) * B.trial.fsw(cc, t) * w;
                    }
                } else {
                    node_g(B, a, b, s, t, w);
                    arc = B.trial.df(ii) * B.trial.df(jj) * w;
                    fg = B.trial.f(ii, s) * B.trial.f(jj, t) * w;
                }
                const cd &h0 = G.h0[gK][id];
                cd hv = G.h1[gK][id] * G.vn[gK][id];
                double temp = tz ? 0. : fg * tdt[id];
                cd cf = tz ? cd(arc) : (B.k_rp ? cd(arc - B.k2ch.real() * temp) : arc - B.k2ch * temp);
                r0 += cf * h0;
                if (d) r1 += tz ? hv * cf : hv * cf + B.ksqrtc * h0 * temp;
                if (d > 1) {
                    cd base = (h0 * G.vn2[gK][id] - hv * B.ksqrtc_inv) * cf;
                    r2 += tz ? base : base - temp * (B.ksqrtc_two * hv - h0);
                }
            }
            L.hy[ii][jj] += r0;
            if (d) L.hy[ii][Q + jj] += r1;
            if (d > 1) L.hy[ii][2 * Q + jj] += r2;
        }
    }
    if (!d) return;
    for (int ii = 0; ii < Q; ++ii) {
        for (int c = Q; c < 2 * Q; ++c) L.hy[ii][c] *= -B.sqrtc;
        if (d > 1) for (int c = 2 * Q; c < 3 * Q; ++c) L.hy[ii][c] *= -B.c;
    }
}

/* single_layer_{coinciding,adjacent,general} (galerkin_builder.cpp:720-832) */
static void single_layer(const Builder &B, int kind, bool swap, int d, const Geo &G, Local &L) {
    int Q = B.test.q, n = G.n;
    for (int a = 0; a < 2; ++a) for (int b = 0; b < 6; ++b) L.sl[a][b] = 0.;
    int nK = (kind == GEN) ? 1 : 2;
    for (int K = 0; K < nK; ++K) {
        int gK = (kind == ADJ) ? K : 0;
        for (int jj = 0; jj < Q; ++jj) for (int ii = 0; ii < Q; ++ii) {
            if (kind == CNC && ii < jj) {   /* symmetry */
                for (int l = 0; l <= d; ++l)
                    L.sl[ii][l * Q + jj] = B.quirk_sl_coinc ? L.sl[jj][ii] : L.sl[jj][l * Q + ii];
                continue;
            }
            cd r0 = 0., r1 = 0., r2 = 0.;
            for (int b = 0; b < n; ++b) for (int a = 0; a < n; ++a) {
                int id = a + n * b;
                double s, t, w, fg;
                int KK = B.lines ? 0 : gK;
                double ttp = G.tn[KK][id] * G.tpn[KK][id];
                if (kind == CNC) {
                    node_c(B, a, b, s, t, w);
                    int r = K > 0 ? jj : ii, cc = K > 0 ? ii : jj;
                    fg = B.test.f(r, s) * B.test.f(cc, t) * w;
                } else if (kind == ADJ) {
                    node_a(B, a, b, s, t, w);
                    int r = K > 0 ? jj : ii, cc = K > 0 ? ii : jj;
                    bool use_swap_tab = swap ? (K == 0) : (K > 0);
                    if (!use_swap_tab) fg = B.test.fsw(r, s) * B.test.f(cc, t) * w;
                    else fg = B.test.f(r, s) * B.test.fsw(cc, t) * w;
                } else {
                    node_g(B, a, b, s, t, w);
                    fg = B.test.f(ii, s) * B.test.f(jj, t) * w;
                }
                double cfr = ttp * fg;
                const cd &h0 = G.h0[gK][id];
                cd m2 = G.h1[gK][id] * G.vn[gK][id];
                r0 += cfr * h0;
                if (d) r1 += cfr * m2;
                if (d > 1) r2 += cfr * (m2 * B.ksqrtc_inv - h0 * G.vn2[gK][id]);
            }
            L.sl[ii][jj] += r0;
            if (d) L.sl[ii][Q + jj] += r1;
            if (d > 1) L.sl[ii][2 * Q + jj] += r2;
        }
    }
    if (!d) return;
    for (int ii = 0; ii < Q; ++ii) {
        for (int c = Q; c < 2 * Q; ++c) L.sl[ii][c] *= -B.sqrtc;
        if (d > 1) for (int c = 2 * Q; c < 3 * Q; ++c) L.sl[ii][c] *= B.c;
    }
}

/* ------------------------------------------------------------------ assembleDense */

enum { L_DOUBLE = 1, L_SINGLE = 2, L_HYPER = 4 };

struct Dense {
    int dim_test, dim_trial;
    /* [layer 0=K,1=W,2=V][t] column-major */
    std::vector<cd> m[3][3];
    int rows[3], cols[3];
};

/* GalerkinBuilder::assembleDense (galerkin_builder.cpp:918-1018), full or
 * sub-matrix (row, col, rows, cols in panels).                                 */
static void assemble_dense(Builder &B, cd k_in, double c_in, int layers, int d,
                           int row, int col, int rows, int cols, Dense &D, int nthreads) {
    if (c_in < 1.) throw std::runtime_error("Refraction index must not be smaller than 1");
    if (k_in.imag() < 0.0) throw std::runtime_error("Wavenumber does not meet conditions for uniqueness of the solution (Im(k) >= 0)");
    if (d > 2) throw std::runtime_error("Invalid order of derivative");
    B.k = k_in; B.c = c_in; B.sqrtc = std::sqrt(c_in);
    B.ksqrtc = k_in * B.sqrtc;
    B.ksqrtc_inv = 1.0 / B.ksqrtc;
    B.ksqrtc_two = 2.0 * B.ksqrtc;
    B.k2ch = B.ksqrtc * B.ksqrtc * .5;
    B.k_rp = k_in.imag() == 0 && k_in.real() > 0;
    int np = B.npanels;
    if (rows == 0) rows = np;
    if (cols == 0) cols = np;
    bool is_full = rows == np && cols == np;
    /* getSpaceDim(n) is n for both P1 (q-1 per panel) and P0 (1 per panel) */
    int dim_test = rows, dim_trial = cols, m0 = row, n0 = col;
    int diag_start = std::max(row, col), diag_end = std::min(row + rows - 1, col + cols - 1);
    bool is_square = B.square();
    if (!(layers & L_DOUBLE)) is_square = true;
    int Qte = B.test.q, Qtr = B.trial.q;
    /* every layer's (sub)matrix is rows x cols panels' dofs; the reference sizes V as
     * rows x rows and W as cols x cols, which overruns when rows != cols          */
    int R[3] = {dim_test, dim_test, dim_test}, C[3] = {dim_trial, dim_trial, dim_trial};
    for (int L = 0; L < 3; ++L) {
        D.rows[L] = R[L]; D.cols[L] = C[L];
        for (int t = 0; t < 3; ++t) D.m[L][t].clear();
    }
    bool hasL[3] = {(layers & L_DOUBLE) != 0, (layers & L_HYPER) != 0, (layers & L_SINGLE) != 0};
    for (int L = 0; L < 3; ++L) if (hasL[L]) for (int t = 0; t <= d; ++t) D.m[L][t].assign((size_t)R[L] * C[L], 0.);
    D.dim_test = dim_test; D.dim_trial = dim_trial;
    int full_test = np, full_trial = np;   /* LocGlobMap dimension = full space dim */
    auto is_required = [&](int i, int j) {
        return i < diag_start || j < diag_start || i > diag_end || j > diag_end || j <= i;
    };
    auto within = [&](int &m, int &n) {
        if (is_full) return true;
        bool ret = m >= m0 && n >= n0 && m < m0 + dim_test && n < n0 + dim_trial;
        if (ret) { m -= m0; n -= n0; }
        return ret;
    };
    /* 4-colour pair lists (galerkin_builder.cpp:964-1013).  The colouring does not keep
     * concurrent scatters apart once square-case pairs are reordered to (max, min), nor
     * across the cyclic P1 wrap for odd N, so the pair blocks are computed in parallel
     * and scattered serially, in list order: deterministic sums.                  */
    int inits[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
    for (int sc = 0; sc < 4; ++sc) {
        std::vector<std::pair<int, int>> ind;
        for (int i = row + inits[sc][0]; i < row + rows; i += 2)
            for (int j = col + inits[sc][1]; j < col + cols; j += 2) {
                if (!is_square) ind.push_back({i, j});
                else if (is_required(i, j)) ind.push_back({std::max(i, j), std::min(i, j)});
            }
        std::vector<Local> locs(ind.size());
        std::vector<int> kinds(ind.size());
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
        for (long q = 0; q < (long)ind.size(); ++q) {
            int i = ind[q].first, j = ind[q].second;
            bool comp_hs = is_square || is_required(i, j);
            Geo G;
            Local &Lc = locs[q];
            std::memset((void *)&Lc, 0, sizeof(Lc));
            bool swap = false;
            int kind;
            if (i == j) { kind = CNC; compute_coinciding(B, i, G); }
            else if (B.is_adjacent(i, j, swap)) { kind = ADJ; compute_adjacent(B, i, j, swap, G); }
            else { kind = GEN; compute_general(B, i, j, G); }
            kinds[q] = kind;
            if (hasL[0]) double_layer(B, kind, swap, d, is_square, G, Lc);
            if (kind == CNC || comp_hs) {
                if (hasL[1]) hypersingular(B, kind, swap, d, G, Lc);
                if (hasL[2]) single_layer(B, kind, swap, d, G, Lc);
            }
        }
        for (long q = 0; q < (long)ind.size(); ++q) {
            int i = ind[q].first, j = ind[q].second;
            int step = (i != j && is_square) ? 2 : 1;
            bool comp_hs = is_square || is_required(i, j);
            const Local &Lc = locs[q];
            int kind = kinds[q];
            /* local -> global (map_local_to_global, galerkin_builder.cpp:334-344) */
            for (int L = 0; L < 3; ++L) {
                if (!hasL[L]) continue;
                if (L > 0 && !(kind == CNC || comp_hs)) continue;  /* see header: no uninitialised adds */
                bool ld = (L == 0);
                int nr = (L == 1) ? Qtr : Qte, nc = (L == 2) ? Qte : Qtr;
                bool write_t = i != j && (!ld || is_square);
                int alpha = ld ? step : 1, offset = ld ? 1 : 0;
                const Space &rs = (L == 1) ? B.trial : B.test, &cs = (L == 2) ? B.test : B.trial;
                int rdim = (L == 1) ? full_trial : full_test, cdim = (L == 2) ? full_test : full_trial;
                for (int l = 0; l < nc; ++l) for (int kk = 0; kk < nr; ++kk) {
                    int m = rs.map(kk, i, rdim), n = cs.map(l, j, cdim);
                    if (within(m, n)) for (int t = 0; t <= d; ++t) {
                        cd val = L == 0 ? Lc.dl[kk][t * alpha * nc + l] : (L == 1 ? Lc.hy[kk][t * nc + l] : Lc.sl[kk][t * nc + l]);
                        D.m[L][t][(size_t)m + (size_t)n * R[L]] += val;
                    }
                    if (write_t) {
                        int m2 = rs.map(kk, j, rdim), n2 = cs.map(l, i, cdim);
                        if (within(m2, n2)) for (int t = 0; t <= d; ++t) {
                            cd val = L == 0 ? Lc.dl[kk][(t * alpha + offset) * nc + l]
                                            : (L == 1 ? Lc.hy[l][t * nc + kk] : Lc.sl[l][t * nc + kk]);
                            D.m[L][t][(size_t)m2 + (size_t)n2 * R[L]] += val;
                        }
                    }
                }
            }
        }
    }
    for (int L = 0; L < 3; ++L) if (hasL[L])
        for (int t = 0; t <= d; ++t) for (auto &z : D.m[L][t]) z *= cd(0., 0.25);
}

/* ------------------------------------------------------------------ mass matrix */

/* mass_matrix::GalerkinMatrix (mass_matrix.cpp:6-47): M(II,JJ) += sum_k w_k g(s_k) f(s_k) |gamma'(s_k)| */
static void mass_matrix(const Builder &B, int order, std::vector<double> &M) {
    int np = B.npanels, rows = np, cols = np;
    std::vector<double> x(order), w(order);
    gauleg(0., 1., order, EPS, x.data(), w.data());
    M.assign((size_t)rows * cols, 0.);
    for (int i = 0; i < np; ++i)
        for (int ii = 0; ii < B.test.q; ++ii)
            for (int jj = 0; jj < B.trial.q; ++jj) {
                int II = B.test.map(ii, i, rows), JJ = B.trial.map(jj, i, cols);
                double sum = 0.;
                for (int k = 0; k < order; ++k) {
                    double s = x[k], nr;
                    pan_d01(B.pan[i], s, &nr);
                    double F = B.trial.f(jj, s) * nr, G = B.test.f(ii, s);
                    sum = sum + w[k] * F * G;
                }
                M[(size_t)II + (size_t)JJ * rows] += sum;
            }
}

/* ------------------------------------------------------------------ C API */

struct OracleBuilder {
    Builder B;
    int mass_order;
};

extern "C" {

int hbo_gauss(int n, double *x, double *w) {
    gauleg(0., 1., n, EPS, x, w);
    return 0;
}

int hbo_cgauss(int n, double *x, double *w) {
    cgauleg_redux(n, EPS, x, w);
    return n * (n + 1) / 2 - 1;
}

void hbo_hankel_real(int n, const double *x, double *h0, double *h1) {
    for (int i = 0; i < n; ++i) {
        cd a, b;
        hankel_real(x[i], a, b);
        h0[2 * i] = a.real(); h0[2 * i + 1] = a.imag();
        h1[2 * i] = b.real(); h1[2 * i + 1] = b.imag();
    }
}

void hbo_hankel_cplx(int n, const double *z, double *h0, double *h1) {
    for (int i = 0; i < n; ++i) {
        cd a, b;
        hankel_cplx(cd(z[2 * i], z[2 * i + 1]), a, b);
        h0[2 * i] = a.real(); h0[2 * i + 1] = a.imag();
        h1[2 * i] = b.real(); h1[2 * i + 1] = b.imag();
    }
}

/* kinds[i]: 0 line (x1 y1 x2 y2), 1 arc (cx cy r phi0 phi1); params 5 per panel. */
void *hbo_builder_create(int npanels, const int *kinds, const double *params, int order, int qtest, int qtrial) {
    OracleBuilder *ob = new OracleBuilder();
    Builder &B = ob->B;
    B.npanels = npanels;
    B.pan.resize(npanels);
    B.lines = true;
    for (int i = 0; i < npanels; ++i) {
        B.pan[i].kind = kinds[i];
        for (int k = 0; k < 5; ++k) B.pan[i].p[k] = params[5 * i + k];
        if (kinds[i] != 0) B.lines = false;
    }
    B.p = order;
    B.nc = order * (order + 1) / 2 - 1;
    B.xg.resize(order); B.wg.resize(order);
    gauleg(0., 1., order, EPS, B.xg.data(), B.wg.data());
    B.xc.resize(B.nc); B.wc.resize(B.nc);
    cgauleg_redux(order, EPS, B.xc.data(), B.wc.data());
    B.test.q = qtest; B.trial.q = qtrial;
    B.quirk_sl_coinc = 0;
    /* SolutionsOperator ctor: 2*max(Q) Gauss points for lines, the builder's order otherwise */
    ob->mass_order = B.lines ? 2 * std::max(qtest, qtrial) : order;
    return ob;
}

void hbo_builder_destroy(void *h) { delete (OracleBuilder *)h; }

void hbo_builder_set_quirks(void *h, int quirk_sl_coinc) { ((OracleBuilder *)h)->B.quirk_sl_coinc = quirk_sl_coinc; }

int hbo_builder_is_adjacent(void *h, int i, int j, int *swap) {
    bool s = false;
    bool r = ((OracleBuilder *)h)->B.is_adjacent(i, j, s);
    *swap = s;
    return r;
}

/* out: interleaved complex; for each present layer L in order K, W, V and each t <= d,
 * a column-major R_L x C_L block, written consecutively.  Returns 0 or -1 on error. */
int hbo_assemble(void *h, double k_re, double k_im, double c, int layers, int d,
                 int row, int col, int rows, int cols, double *out, int nthreads) {
    OracleBuilder *ob = (OracleBuilder *)h;
    Dense D;
    try {
        assemble_dense(ob->B, cd(k_re, k_im), c, layers, d, row, col, rows, cols, D, nthreads);
    } catch (std::exception &) {
        return -1;
    }
    size_t off = 0;
    for (int L = 0; L < 3; ++L) {
        if (D.m[L][0].empty()) continue;
        for (int t = 0; t <= d; ++t) {
            std::memcpy(out + 2 * off, D.m[L][t].data(), D.m[L][t].size() * sizeof(cd));
            off += D.m[L][t].size();
        }
    }
    return 0;
}

void hbo_mass(void *h, double *M) {
    OracleBuilder *ob = (OracleBuilder *)h;
    std::vector<double> m;
    mass_matrix(ob->B, ob->mass_order, m);
    std::memcpy(M, m.data(), m.size() * sizeof(double));
}

}  /* extern "C" */
