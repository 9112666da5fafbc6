// Host root finding and the plain resonance search.
//
// rtsafe  : safeguarded Newton (bisection when the Newton step leaves the bracket or
//           does not halve the step), as used at source/utilities/find_roots.cpp:117-217
// zbrent  : Brent's zero finder (inverse quadratic interpolation / bisection),
//           find_roots.cpp:19-115
// brent_min: Brent's localmin (golden section + parabolic steps), the algorithm of
//           BrentMinimizer::local_min_rc, find_roots.cpp:1003-1184
// The stopping rules are kept as in the reference so the iterates agree; the
// resonance search runs many rtsafe iterations in lock step so every Newton
// round is one batched GPU evaluation of sigma' and sigma''.
#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

#include "../../include/hbem.h"

namespace {

const double kEps = std::numeric_limits<double>::epsilon();
const int kMaxIt = 1000;

// rtsafe as a resumable state machine: request(x) -> feed(f, df) -> ...
struct Newton {
    double xl, xh, rts, dx, dxold, f, df, tol;
    int it = 0;
    bool first = true, done = false, found = false;
    void start(double x1, double x2, double guess, double tol_in) {
        // the reference's "initial guess" entry (fct(x1) is NaN): xl = x1, xh = x2
        xl = x1; xh = x2; rts = guess; tol = tol_in;
        dxold = std::fabs(x2 - x1);
        dx = dxold;
    }
    void finish(bool ok) { done = true; found = ok; if (!ok) rts = NAN; }
    void feed(double fv, double dfv) {
        f = fv; df = dfv;
        if (!first) {
            if (f < 0.0) xl = rts;
            else xh = rts;
        }
        first = false;
        if (++it > kMaxIt) { finish(false); return; }
        if ((((rts - xh) * df - f) * ((rts - xl) * df - f) > 0.0) || (std::fabs(2.0 * f) > std::fabs(dxold * df))) {
            dxold = dx;
            dx = 0.5 * (xh - xl);
            rts = xl + dx;
            if (std::fabs(xl - rts) < kEps) { finish(true); return; }
        } else {
            dxold = dx;
            dx = f / df;
            double temp = rts;
            rts -= dx;
            if (temp == rts) { finish(true); return; }
        }
        if (std::fabs(dx) < tol) { finish(true); return; }
    }
};

// Brent's localmin on [a, b] with tolerance tol (tol1 = sqrt(tol)|x| + tol/3, as the
// reference's wrapper sets eps = sqrt(tol))
template <class F>
double localmin(F&& f, double a, double b, double tol) {
    const double c = 0.5 * (3.0 - std::sqrt(5.0)), eps = std::sqrt(tol);
    double v = a + c * (b - a), w = v, x = v, e = 0.0, d = 0.0;
    double fx = f(x), fv = fx, fw = fx;
    for (int it = 0; it < 10000; ++it) {
        double mid = 0.5 * (a + b), tol1 = eps * std::fabs(x) + tol / 3.0, tol2 = 2.0 * tol1;
        if (std::fabs(x - mid) <= tol2 - 0.5 * (b - a)) return x;
        bool golden = std::fabs(e) <= tol1;
        if (!golden) {
            double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), p = (x - v) * q - (x - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) p = -p;
            q = std::fabs(q);
            r = e;
            e = d;
            if (std::fabs(0.5 * q * r) <= std::fabs(p) || p <= q * (a - x) || q * (b - x) <= p) {
                golden = true;
            } else {
                d = p / q;
                double u = x + d, sg = (mid - x) < 0. ? -1. : 1.;
                if ((u - a) < tol2 || (b - u) < tol2) d = tol1 * sg;
            }
        }
        if (golden) {
            e = (mid <= x) ? a - x : b - x;
            d = c * e;
        }
        double u = std::fabs(d) >= tol1 ? x + d : x + tol1 * (d < 0. ? -1. : 1.);
        double fu = f(u);
        if (fu <= fx) {
            if (x <= u) a = x; else b = x;
            v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
        } else {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) { v = w; fv = fw; w = u; fw = fu; }
            else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
        }
    }
    return x;
}

// quartic Hermite model through (a, f1, d1), (a+h, f0), (a+2h, f2, d2)
// (examples/roots_newton_polygon_rsvd.cpp:224-245), minimised by Brent
double quartic_guess(double a, double h, double f1, double f0, double f2, double d1, double d2, double tol) {
    double scale = 0.25 * std::pow(h, -4), a2 = a * a;
    double p1 = a2 * (h * (d2 - d1) - 2. * (f1 + f2 - 2. * f0));
    double p2 = a * h * (h * (3. * d2 - 5. * d1) - (9. * f1 + 7. * f2 - 16. * f0));
    double p3 = h * h * (2. * h * (d2 - 4. * d1) - (11. * f1 + 5. * f2 - 16. * f0));
    double A = scale * p1 / a2, B = -scale * (4. * p1 + p2) / a, C = scale * (6. * p1 + 3 * p2 + p3);
    double D = d1 - scale * a * (4. * p1 + 3. * p2 + 2. * p3), E = f1 - a * d1 + scale * a2 * (p1 + p2 + p3);
    return localmin([&](double t) { return (((A * t + B) * t + C) * t + D) * t + E; }, a, a + 2 * h, tol);
}

}  // namespace

extern "C" {

double hbem_rtsafe(hbem_fn fct, hbem_fn_both fboth, void* user, double x1, double x2, double tol, int* root_found,
                   unsigned* num_iter) {
    if (root_found) *root_found = 0;
    if (num_iter) *num_iter = 0;
    double fl = fct(x1, user), fh = fct(x2, user), rts, xl, xh;
    if (fl == fl && fh == fh) {
        if (fl * fh > 0.) return fl > fh ? x1 : x2;
        if (fl == 0.0) { if (root_found) *root_found = 1; return x1; }
        if (fh == 0.0) { if (root_found) *root_found = 1; return x2; }
        if (fl < 0.0) { xl = x1; xh = x2; } else { xh = x1; xl = x2; }
        rts = 0.5 * (x1 + x2);
    } else {
        rts = fct(NAN, user);
        xl = x1; xh = x2;
    }
    Newton nt;
    nt.start(x1, x2, rts, tol);
    nt.xl = xl; nt.xh = xh;
    while (!nt.done) {
        double f, df;
        fboth(nt.rts, &f, &df, user);
        nt.feed(f, df);
    }
    if (root_found) *root_found = nt.found;
    if (num_iter) *num_iter = (unsigned)nt.it;
    return nt.rts;
}

double hbem_zbrent(hbem_fn f, void* user, double x1, double x2, double tol, int* root_found, unsigned* num_iter) {
    double a = x1, b = x2, c = x2, d = 0., e = 0., fa = f(a, user), fb = f(b, user), fc;
    if (root_found) *root_found = 0;
    if (fa * fb > 0.) return 0.0;
    fc = fb;
    for (int it = 1; it <= kMaxIt; ++it) {
        if ((fb > 0.0 && fc > 0.0) || (fb < 0.0 && fc < 0.0)) { c = a; fc = fa; e = d = b - a; }
        if (std::fabs(fc) < std::fabs(fb)) { a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
        double tol1 = 2.0 * kEps * std::fabs(b) + 0.5 * tol, xm = 0.5 * (c - b);
        if (std::fabs(xm) <= tol1 || fb == 0.0) {
            if (root_found) *root_found = 1;
            if (num_iter) *num_iter = (unsigned)it;
            return b;
        }
        if (std::fabs(e) >= tol1 && std::fabs(fa) > std::fabs(fb)) {
            double s = fb / fa, p, q;
            if (a == c) { p = 2.0 * xm * s; q = 1.0 - s; }
            else {
                double qq = fa / fc, r = fb / fc;
                p = s * (2.0 * xm * qq * (qq - r) - (b - a) * (r - 1.0));
                q = (qq - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0.0) q = -q;
            p = std::fabs(p);
            double m1 = 3.0 * xm * q - std::fabs(tol1 * q), m2 = std::fabs(e * q);
            if (2.0 * p < std::min(m1, m2)) { e = d; d = p / q; }
            else { d = xm; e = d; }
        } else { d = xm; e = d; }
        a = b;
        fa = fb;
        b += std::fabs(d) > tol1 ? d : (xm >= 0 ? std::fabs(tol1) : -std::fabs(tol1));
        fb = f(b, user);
    }
    return 0.0;
}

double hbem_brent_min(hbem_fn f, void* user, double a, double b, double tol) {
    if (!(a < b)) return NAN;
    return localmin([&](double x) { return f(x, user); }, a, b, tol);
}

int hbem_find_resonances_plain(hbem_solop s, double k_min, double k_max, int npoints, double c_o, double c_i,
                               double tol, double* roots_host, int max_roots, int* nroots, double* grid_host,
                               int* n_evals) {
    if (!s || npoints < 3 || !(k_max > k_min) || !nroots) return HBEM_ERR_INVALID;
    std::vector<double> ks(npoints), g(3 * (size_t)npoints);
    const double h = (k_max - k_min) / (npoints - 1);
    for (int i = 0; i < npoints; ++i) ks[i] = k_min + i * h;
    int evals = npoints;
    // sigma on the grid (randomized_svd::sv / direct::sv at roots_newton_polygon_rsvd.cpp:172-177)
    if (int r = hbem_sweep_sigma(s, ks.data(), npoints, c_o, c_i, 0, g.data())) return r;
    for (int i = 0; i < npoints; ++i) g[3 * i + 1] = g[3 * i + 2] = NAN;
    // 3-point local minima (:185-194)
    std::vector<int> cidx;
    for (int i = 0; i + 2 < npoints; ++i) {
        const double L = g[3 * i], C = g[3 * (i + 1)], R = g[3 * (i + 2)];
        if (L - C > 0. && R - C > 0.) cidx.push_back(i);
    }
    // sigma' at both bracket ends of every candidate in one batch (sv_der, :204-208)
    std::vector<double> ends(2 * cidx.size()), der(6 * cidx.size());
    for (size_t c = 0; c < cidx.size(); ++c) {
        ends[2 * c] = ks[cidx[c]];
        ends[2 * c + 1] = ks[cidx[c] + 2];
    }
    if (!ends.empty()) {
        if (int r = hbem_sweep_sigma(s, ends.data(), (int)ends.size(), c_o, c_i, 1, der.data())) return r;
        evals += (int)ends.size();
    }
    // validation sigma'(left) < 0 < sigma'(right), quartic Hermite model + Brent (:209-245)
    struct Cand { double a, guess; };
    std::vector<Cand> cands;
    for (size_t c = 0; c < cidx.size(); ++c) {
        const int i = cidx[c];
        const double d1 = der[3 * (2 * c) + 1], d2 = der[3 * (2 * c + 1) + 1];
        g[3 * i + 1] = d1;
        g[3 * (i + 2) + 1] = d2;
        if (!(d1 < 0. && d2 > 0.)) continue;
        cands.push_back(Cand{ks[i], quartic_guess(ks[i], h, g[3 * i], g[3 * (i + 1)], g[3 * (i + 2)], d1, d2, tol)});
    }
    if (grid_host) std::copy(g.begin(), g.end(), grid_host);
    std::vector<Newton> nt(cands.size());
    for (size_t c = 0; c < cands.size(); ++c) nt[c].start(cands[c].a, cands[c].a + 2 * h, cands[c].guess, tol);
    // lock-step Newton rounds: one batched sigma', sigma'' evaluation per round
    for (int round = 0; round < kMaxIt; ++round) {
        std::vector<double> xs;
        std::vector<size_t> who;
        for (size_t c = 0; c < nt.size(); ++c)
            if (!nt[c].done) { xs.push_back(nt[c].rts); who.push_back(c); }
        if (xs.empty()) break;
        std::vector<double> out(3 * xs.size());
        if (int r = hbem_sweep_sigma(s, xs.data(), (int)xs.size(), c_o, c_i, 2, out.data())) return r;
        evals += (int)xs.size();
        for (size_t q = 0; q < who.size(); ++q) nt[who[q]].feed(out[3 * q + 1], out[3 * q + 2]);
    }
    int cnt = 0;
    for (auto& x : nt)
        if (x.done && x.found && x.rts == x.rts) {
            if (roots_host && cnt < max_roots) roots_host[cnt] = x.rts;
            ++cnt;
        }
    *nroots = cnt;
    if (n_evals) *n_evals = evals;
    return HBEM_OK;
}

}  // extern "C"
