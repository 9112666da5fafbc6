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
#include <array>
#include <cstdint>
#include <functional>
#include <cmath>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hbem.h"

namespace hbem {
int plain_speculate_ok(hbem_solop s);
int plain_warm_start_ok();
int plain_async_ok();
int plain_spec_limits(int* deep);
void svd_pair_hold(int on);
void singular_split_hold(int on);
int pipeline_setup(hbem_solop s, int npoints, int npool);
void pipeline_keep_uv(hbem_solop s, int npoints);
int lane_launch_grid(hbem_solop s, int lane, const double* k_host, int npts, int first, double c_o, double c_i,
                     int npool, int after);
int lane_launch_ends(hbem_solop s, int lane, const double* k_host, const int* gidx, double c_o, double c_i);
int lane_results_grid(hbem_solop s, int lane, double* sigma_host, int* all_fast);
int lane_results_ends(hbem_solop s, int lane, double* d1_host);
int lane_launch(hbem_solop s, int lane, const double* k_host, int npts, double c_o, double c_i, const int* wslot,
                const int* oslot, int npool, unsigned d);
int lane_wait(hbem_solop s, int lane, int block, int* finished);
int lane_results(hbem_solop s, int lane, double c_o, double c_i, double* out_host);
int lane_launch_near(hbem_solop s, int lane, const double* k_host, int npts, unsigned d, const int* wslot,
                     const int* oslot, int npool);
int sweep_sigma_warm(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d,
                     const int* warm_slot, const int* out_slot, int npool, double* out_host, int keep_uv = 0);
int sigma1_from_kept(hbem_solop s, const double* k_host, const int* idx, int ne, double c_o, double c_i,
                     double* d1_host);
}  // namespace hbem

namespace {

const double kEps = std::numeric_limits<double>::epsilon();
const int kMaxIt = 1000;

// rtsafe as a resumable state machine: request(x) -> feed(f, df) -> ...
struct Newton {
    double xl, xh, rts, dx, dxold, f, df, tol;
    int it = 0;
    bool first = true, done = false, found = false, bisected = false;
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
            bisected = true;
            if (std::fabs(xl - rts) < kEps) { finish(true); return; }
        } else {
            bisected = false;
            dxold = dx;
            dx = f / df;
            double temp = rts;
            rts -= dx;
            if (temp == rts) { finish(true); return; }
        }
        if (std::fabs(dx) < tol) { finish(true); return; }
    }
    // the points a bisection step could move to after the next feed (f < 0 moves xl
    // to rts, otherwise xh; the first feed, at the initial guess, moves neither),
    // computed with the same operations as feed() so that they compare equal
    int bisect_next(double* c) const {
        if (first) {
            c[0] = xl + 0.5 * (xh - xl);
            return 1;
        }
        c[0] = rts + 0.5 * (xh - rts);
        c[1] = xl + 0.5 * (rts - xl);
        return 2;
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

// ------------------------------------------------------------------ adaptive sampler pieces

// SplitMix64 (Steele, Lea and Flood 2014): seeded stand-in for the reference's
// std::random_device-seeded mt19937; uniform in [0, 1) from the top 53 bits, normal
// deviates by the Box-Muller transform.
struct SplitMix {
    uint64_t s;
    explicit SplitMix(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal(double mu, double sd) {
        double u1 = uniform(), u2 = uniform();
        if (u1 <= 0.) u1 = 1.0 / 9007199254740992.0;
        return mu + sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

// Monotone cubic interpolation of M. Steffen, A&A 239 (1990) 443-450: slopes
// (sign s_{i-1} + sign s_i) min(|s_{i-1}|, |s_i|, |p_i| / 2) at interior nodes, the
// parabola-through-three-points boundary slopes limited to [0, 2 s] (eqs. 26-27).
struct Steffen {
    std::vector<double> x, y, yp;
    bool init(const std::vector<std::pair<double, double>>& xy, size_t n) {
        if (n < 3) return false;
        x.resize(n); y.resize(n); yp.resize(n);
        for (size_t i = 0; i < n; ++i) { x[i] = xy[i].first; y[i] = xy[i].second; }
        std::vector<double> h(n - 1), sl(n - 1);
        for (size_t i = 0; i + 1 < n; ++i) {
            h[i] = x[i + 1] - x[i];
            if (!(h[i] > 0.)) return false;
            sl[i] = (y[i + 1] - y[i]) / h[i];
        }
        auto sgn = [](double v) { return (double)((v > 0.) - (v < 0.)); };
        for (size_t i = 1; i + 1 < n; ++i) {
            const double p = (sl[i - 1] * h[i] + sl[i] * h[i - 1]) / (h[i - 1] + h[i]);
            yp[i] = (sgn(sl[i - 1]) + sgn(sl[i])) * std::min(std::min(std::fabs(sl[i - 1]), std::fabs(sl[i])),
                                                              0.5 * std::fabs(p));
        }
        auto bound = [](double s0, double s1, double h0, double h1) {
            const double p = s0 * (1. + h0 / (h0 + h1)) - s1 * h0 / (h0 + h1);
            if (p * s0 <= 0.) return 0.;
            return std::fabs(p) > 2. * std::fabs(s0) ? 2. * s0 : p;
        };
        yp[0] = bound(sl[0], sl[1], h[0], h[1]);
        yp[n - 1] = bound(sl[n - 2], sl[n - 3], h[n - 2], h[n - 3]);
        return true;
    }
    // false outside [x_0, x_{n-1}]
    bool eval(double t, double& v) const {
        if (!(t >= x.front() && t <= x.back())) return false;
        size_t i = std::upper_bound(x.begin(), x.end(), t) - x.begin();
        i = i == 0 ? 0 : std::min(i - 1, x.size() - 2);
        const double h = x[i + 1] - x[i], sl = (y[i + 1] - y[i]) / h, dt = t - x[i];
        const double a = (yp[i] + yp[i + 1] - 2. * sl) / (h * h), b = (3. * sl - 2. * yp[i] - yp[i + 1]) / h;
        v = y[i] + dt * (yp[i] + dt * (b + dt * a));
        return true;
    }
};

// Barycentric rational interpolant of M. S. Floater and K. Hormann, Numer. Math. 107
// (2007) 315-331, blending order d (the reference uses order 5 through
// boost::math::barycentric_rational).
struct BaryRat {
    std::vector<double> x, y, w;
    void init(const double* xs, const double* ys, int n, int d) {
        x.assign(xs, xs + n);
        y.assign(ys, ys + n);
        w.assign(n, 0.);
        for (int k = 0; k < n; ++k)
            for (int i = std::max(0, k - d); i <= std::min(k, n - 1 - d); ++i) {
                double prod = 1.;
                for (int j = i; j <= i + d; ++j)
                    if (j != k) prod /= (x[k] - x[j]);
                w[k] += (i % 2 ? -1. : 1.) * prod;
            }
    }
    double operator()(double t) const {
        double num = 0., den = 0.;
        for (size_t k = 0; k < x.size(); ++k) {
            if (t == x[k]) return y[k];
            const double c = w[k] / (t - x[k]);
            num += c * y[k];
            den += c;
        }
        return num / den;
    }
};

// One proposal of Brent's minimiser: parabolic step through (x, w, v) when it is
// acceptable, else a golden-section step into the larger part of [a, b].
struct BrentState {
    double a, b, x, w, v, fx, fw, fv, d = 0., e = 0.;
    double propose(double tol1) {
        const double tol2 = 2. * tol1, xm = 0.5 * (a + b);
        bool golden = true;
        if (std::fabs(e) > tol1) {
            double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), p = (x - v) * q - (x - w) * r;
            q = 2. * (q - r);
            if (q > 0.) p = -p;
            q = std::fabs(q);
            const double et = e;
            e = d;
            if (!(std::fabs(p) >= std::fabs(0.5 * q * et) || p <= q * (a - x) || p >= q * (b - x))) {
                d = p / q;
                const double uu = x + d;
                if (uu - a < tol2 || b - uu < tol2) d = xm - x > 0. ? tol1 : -tol1;
                golden = false;
            }
        }
        if (golden) {
            e = x >= xm ? a - x : b - x;
            d = 0.3819660 * e;
        }
        return std::fabs(d) >= tol1 ? x + d : x + (d > 0. ? tol1 : -tol1);
    }
    void update(double u, double fu) {
        if (fu <= fx) {
            if (u >= x) a = x; else b = x;
            v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
        } else {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) { v = w; fv = fw; w = u; fw = fu; }
            else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
        }
    }
};

// brent_guess (find_roots.cpp:1233-1313): Brent's minimisation on [a, b] started from
// a guess with known value, tolerance max(tol, sqrt eps) |x| + 1e-10.
template <class F>
double brent_guess(double a, double b, double guess, double fguess, F&& f, double tol, unsigned* count = nullptr) {
    const double tolc = std::max(tol, std::sqrt(kEps));
    BrentState S{a, b, guess, guess, guess, fguess, fguess, fguess};
    unsigned ic = 0;
    for (; ic < 100; ++ic) {
        const double xm = 0.5 * (S.a + S.b), tol1 = tolc * std::fabs(S.x) + 1e-10;
        if (std::fabs(S.x - xm) <= 2. * tol1 - 0.5 * (S.b - S.a)) break;
        const double u = S.propose(tol1);
        S.update(u, f(u));
    }
    if (count) *count = ic;
    return S.x;
}

// Brent minimisation as a resumable state machine, for many candidates in lock step
// (brent_gsl, find_roots.cpp:1426-1473): the bracket must hold f(guess) < f(a), f(b)
// (the condition the reference's GSL minimiser sets); converged when |b - a| < tol
// min(|a|, |b|) (GSL's interval test with relative error tol), at most 100 steps.
struct BrentSearch {
    BrentState S;
    double tol = 0., u = 0.;
    int it = 0;
    bool done = false, ok = false;
    void start(double a0, double fa, double b0, double fb, double guess, double fg, double tol_in) {
        S = BrentState{a0, b0, guess, guess, guess, fg, fg, fg};
        tol = tol_in;
        if (!(fg < fa && fg < fb) || !(a0 < guess && guess < b0)) { done = true; ok = false; return; }
        u = S.propose(std::sqrt(kEps) * std::fabs(S.x) + 1e-10);
    }
    void feed(double fu) {
        ++it;
        S.update(u, fu);
        const double lo = std::min(std::fabs(S.a), std::fabs(S.b));
        if (std::fabs(S.b - S.a) < tol * lo || it >= 100) { done = true; ok = true; return; }
        u = S.propose(std::sqrt(kEps) * std::fabs(S.x) + 1e-10);
    }
};

typedef std::function<int(const double*, int, double*)> BatchEval;

// opt_subdiv (find_roots.cpp:1615-1726): batches of random abscissae -- uniform on
// odd iterations, normal about the centre of the spline error on even ones -- kept
// at least tol (x_max - x_min) away from earlier samples; stops when the number of
// interior local minima has not grown for `limit` batches.  Restated with its
// behaviour kept: the two end-point evaluations are overwritten by the first batch.
int opt_subdiv_impl(const BatchEval& f, double x_min, double x_max, int batch, int limit, double tol, uint64_t seed,
                    std::vector<std::pair<double, double>>& xy, std::vector<int>& p) {
    const double d = x_max - x_min;
    double ends[2] = {x_min, x_max}, fe[2];
    if (int r = f(ends, 2, fe)) return r;
    xy.assign({{x_min, fe[0]}, {x_max, fe[1]}});
    size_t n = 0, mc = 0;
    int count = 0;
    unsigned iter = 0;
    double sigma = -1., mu = 0.;
    SplitMix rng(seed);
    std::vector<double> xt(batch), yt(batch);
    p.clear();
    while (count < limit && ++iter < 1000) {
        Steffen sp;
        const bool have = n > 3 && sp.init(xy, n);
        for (int i = 0; i < batch; ++i) {
            double x0 = x_min;
            for (int tries = 0; tries < 100000; ++tries) {
                if (iter % 2 || sigma < 0. || sigma > 3. * d || !(sigma == sigma)) {
                    x0 = x_min + rng.uniform() * d;
                } else {
                    int g = 0;
                    do x0 = rng.normal(mu, sigma);
                    while ((x0 <= x_min || x0 >= x_max) && ++g < 1000);
                    if (x0 <= x_min || x0 >= x_max) x0 = x_min + rng.uniform() * d;
                }
                // xy holds the previous samples sorted by x: only the two neighbours of
                // x0 can be within tol d of it (same test as a scan of every sample)
                auto it = std::lower_bound(xy.begin(), xy.end(), x0,
                                           [](const std::pair<double, double>& q, double x) { return q.first < x; });
                bool near = (it != xy.end() && std::fabs(x0 - it->first) < tol * d) ||
                            (it != xy.begin() && std::fabs(x0 - (it - 1)->first) < tol * d);
                if (!near) break;
            }
            xt[i] = x0;
        }
        xy.resize(n + batch);
        if (int r = f(xt.data(), batch, yt.data())) return r;
        for (int i = 0; i < batch; ++i) xy[n + i] = {xt[i], yt[i]};
        if (have) {
            double erravg = 0., errmax = 0., m = 0.;
            int cnt = 0;
            for (size_t i = n; i < xy.size(); ++i) {
                double ys;
                if (sp.eval(xy[i].first, ys)) {
                    const double err = std::fabs(xy[i].second - ys);
                    erravg += err;
                    errmax = std::max(errmax, err);
                    m += err * xy[i].first;
                    ++cnt;
                }
            }
            if (cnt >= 2 && erravg > 0. && errmax > erravg / cnt) {
                erravg /= cnt;
                sigma = d * erravg * (cnt - 1.) / (6. * (errmax - erravg));
                mu = m / (erravg * cnt);
            } else {
                sigma = -1.;
            }
        }
        std::sort(xy.begin(), xy.end());
        n += batch;
        p.clear();
        for (size_t i = 1; i + 1 < n; ++i)
            if (xy[i].second < std::min(xy[i - 1].second, xy[i + 1].second)) p.push_back((int)i);
        if (p.size() > mc) { count = 0; mc = p.size(); }
        else ++count;
    }
    return HBEM_OK;
}

// ---------------------------------------------------------------- Newton rounds with speculation
//
// The Newton phase of the plain search (examples/roots_newton_polygon_rsvd.cpp:209-265)
// for candidates whose brackets have been validated.  Every round is one batched
// sigma', sigma'' evaluation; in a round with at most kSpecRound active candidates,
// a candidate at its first point or just after a bisection step also has the one or
// two points a further bisection step of rtsafe could move to evaluated
// (Newton::bisect_next).  When that step follows, its point is already known and costs
// no round of its own.  Each candidate is fed exactly the values it would be fed
// without speculation, so its iterates are unchanged.  A round's cost is a fixed part
// (one dense-sigma CTA per matrix runs for milliseconds) plus a part per point (the
// assembly of T, T', T''), so speculation pays where bisection steps run in series.
// evals counts the evaluations the search used (unused speculative points excluded).
constexpr int kSpecRound = 8;

// With warm starts (first_warm != null): candidate c's dense-sigma evaluations start
// their FP32 Jacobi from the V set of its previous evaluated point, the first from
// pool slot first_warm[c] (a grid point beside the guess); its main points alternate
// between its two own slots slot_base + 2c, slot_base + 2c + 1, speculative points
// only read.
int newton_rounds(hbem_solop s, std::vector<Newton>& nt, double c_o, double c_i, int& evals,
                  const std::vector<int>* first_warm = nullptr, int slot_base = 0) {
    std::vector<std::vector<std::array<double, 3>>> cache(nt.size());   // (k, sigma', sigma'')
    struct Req { size_t cand; bool spec; };
    std::vector<Req> who;
    std::vector<double> xs, out;
    std::vector<int> cur, wslot, oslot;
    if (first_warm) cur = *first_warm;
    const int npool = slot_base + 2 * (int)nt.size();
    for (int round = 0; round < kMaxIt; ++round) {
        // points already evaluated speculatively
        for (size_t c = 0; c < nt.size(); ++c)
            while (!nt[c].done) {
                auto it = std::find_if(cache[c].begin(), cache[c].end(),
                                       [&](const std::array<double, 3>& e) { return e[0] == nt[c].rts; });
                if (it == cache[c].end()) break;
                nt[c].feed((*it)[1], (*it)[2]);
                ++evals;
            }
        xs.clear();
        who.clear();
        for (size_t c = 0; c < nt.size(); ++c)
            if (!nt[c].done) {
                xs.push_back(nt[c].rts);
                who.push_back(Req{c, false});
            }
        if (xs.empty()) break;
        if (xs.size() <= (size_t)kSpecRound)
            for (size_t c = 0; c < nt.size(); ++c) {
                // bisection steps come in runs: speculate at the first point and after a
                // bisection, not after a Newton step (which usually converges on)
                if (nt[c].done || !(nt[c].first || nt[c].bisected)) continue;
                cache[c].clear();
                double sp[2];
                const int m = nt[c].bisect_next(sp);
                for (int j = 0; j < m; ++j)
                    if (sp[j] != nt[c].rts) {
                        xs.push_back(sp[j]);
                        who.push_back(Req{c, true});
                    }
            }
        out.assign(3 * xs.size(), 0.);
        if (first_warm) {
            wslot.assign(xs.size(), -1);
            oslot.assign(xs.size(), -1);
            for (size_t q = 0; q < who.size(); ++q) {
                const int c = (int)who[q].cand, own0 = slot_base + 2 * c;
                wslot[q] = cur[c];
                if (!who[q].spec) oslot[q] = cur[c] == own0 ? own0 + 1 : own0;
            }
            if (int r = hbem::sweep_sigma_warm(s, xs.data(), (int)xs.size(), c_o, c_i, 2, wslot.data(), oslot.data(),
                                               npool, out.data()))
                return r;
            for (size_t q = 0; q < who.size(); ++q)
                if (!who[q].spec) cur[who[q].cand] = oslot[q];
        } else if (int r = hbem_sweep_sigma(s, xs.data(), (int)xs.size(), c_o, c_i, 2, out.data())) {
            return r;
        }
        for (size_t q = 0; q < who.size(); ++q) {
            const double* o = &out[3 * q];
            if (who[q].spec) {
                cache[who[q].cand].push_back({xs[q], o[1], o[2]});
            } else {
                nt[who[q].cand].feed(o[1], o[2]);
                ++evals;
            }
        }
    }
    return HBEM_OK;
}

// The plain search as one pipeline on several streams ("lanes"): the grid in chunks
// whose assemblies run one after another (from the top of the range down) while each
// chunk's dense sigma overlaps the next chunk's assembly; a candidate's bracket ends
// (sigma' from the grid's kept singular vectors) as soon as the grid around it is
// known; its Newton steps as soon as its previous point is evaluated, one point per
// lane; and, when asked for, its root's sign-change check as soon as it converges.
// The FP64 assembly of one candidate runs while another's dense sigma does, and the
// grid's tail overlaps the first candidates' work.  Values are those of the lock-step
// search -- the same grid (chunks of at least the size below, so that their general
// pairs take the same layout as one batch), the same bracket ends, and the same Newton
// and bisection steps with the same warm-start slots for the Newton points -- except
// for points within 1e-6 of the point a candidate has just evaluated (a Newton step
// that small, the root's two check points): they take that point's T, T', T'' by
// Taylor polynomials (lane_launch_near), so their sigma' agrees with an assembled
// one to ~1e-11 rather than bit for bit.  Grid chunks run on the lowest-priority
// streams, candidates' evaluations above them (the long runs highest), and the host
// polls every lane so that each result is taken as soon as it is there.  Speculative
// bisection points run on lanes of their own once the grid is complete and at most
// "plain_spec_async" candidates (option, default 2) are unfinished
// ("plain_spec_deep": the bisection after next too); one may be evaluated from
// another warm start than in lock step, so its values agree to the dense kernel's
// accuracy (sigma' and sigma'' to ~1e-12 relative), not bit for bit.
constexpr int kSpecDeep = 2;
// lanes (streams) of the search: with the builder's and the runtime's own streams they
// stay within the 32 hardware work queues, so that no two lanes share one (a lane's
// launch that waits for its own stream's previous one would hold up the other's)
constexpr int kLanes = 24;
constexpr int kCandLane = 8;   // the first lane of candidates' evaluations (the grid's below)
constexpr int kUrgentEnd = 16; // lanes kCandLane .. kUrgentEnd - 1: highest stream priority
constexpr int kMain = 0, kSpec = 1, kVerify = 2, kGrid = 3, kEnds = 4, kVerify2 = 5;

// Returns HBEM_ERR_UNSUPPORTED, with nothing left in flight, when the grid cannot be
// chunked without changing its values or a grid matrix needs the polished kernel:
// the caller then runs the lock-step search.
int plain_pipelined(hbem_solop s, const std::vector<double>& ks, double h, double c_o, double c_i, double tol,
                    std::vector<double>& g, std::vector<Newton>& nt, std::vector<double>* vder, int& evals) {
    const int npoints = (int)ks.size();
    int npan = 0;
    if (int r = hbem_solop_info(s, &npan)) return r;
    // chunk size: general pairs x jobs of a chunk on the same side of the thread / warp
    // layout threshold (152 x 16 x 32) as the whole grid's
    const long long nlow = (long long)npan * (npan - 1) / 2;
    const long long thr = 152LL * 16 * 32;
    const bool whole_thread = nlow * 2 * npoints >= thr;
    int csize = std::max(32, (npoints + 4) / 5);
    if (whole_thread) csize = std::max<long long>(csize, (thr + 2 * nlow - 1) / (2 * nlow));
    if (csize > 64) return HBEM_ERR_UNSUPPORTED;
    const int nch = (npoints + csize - 1) / csize;
    if (nch > kCandLane) return HBEM_ERR_UNSUPPORTED;
    if (!whole_thread) {
        // every chunk, the smallest last one included, must stay below the threshold too
        // (it does: fewer jobs than the whole grid)
    } else if (nlow * 2 * (npoints - (nch - 1) * csize) < thr) {
        return HBEM_ERR_UNSUPPORTED;
    }
    const int npool = 2 * npoints;   // grid slots, then two per candidate (at most npoints / 2)
    if (int r = hbem::pipeline_setup(s, npoints, npool)) return r;
    int spec_deep = kSpecDeep;
    const int spec_lim = hbem::plain_spec_limits(&spec_deep);

    struct Flight { int cand; double x; int kind; int side; int rslot; };
    std::vector<Flight> fl(kLanes);
    std::vector<int> busy(kLanes, 0);
    std::vector<int> order;   // lanes in launch order
    // candidates (grid index, state 0: bracket ends to launch, 1: ends in flight,
    // 2: rejected, 3: Newton)
    std::vector<int> cgrid, cstate, cur, in_flight, vsent;
    // the lane of each candidate's last Newton point, that lane's launch count then and
    // the point: while the lane has had no launch since, it still holds T, T', T''
    std::vector<int> last_lane;
    std::vector<long long> last_gen;
    std::vector<double> last_x;
    std::vector<long long> lane_gen(kLanes, 0);
    std::vector<std::vector<std::array<double, 3>>> cache;
    std::vector<std::vector<double>> pend;
    nt.clear();
    std::vector<double> vd;   // sigma' at root -/+ tol per candidate (NaN: none)
    std::vector<char> gknown(npoints, 0), scanned(npoints, 0);
    int chunks_done = 0;
    bool grid_ok = true;
    for (int i = 0; i < npoints; ++i) g[3 * i] = g[3 * i + 1] = g[3 * i + 2] = NAN;

    auto has = [](const std::vector<double>& v, double x) { return std::find(v.begin(), v.end(), x) != v.end(); };
    auto cached = [&](size_t c, double x) {
        return std::find_if(cache[c].begin(), cache[c].end(),
                            [&](const std::array<double, 3>& e) { return e[0] == x; }) != cache[c].end();
    };
    // candidates' evaluations on lanes kCandLane .. (higher stream priority than the grid
    // chunks on lanes 0 .. nch - 1): a free lane of the highest priority for a candidate
    // deep into its Newton run (the runs with bisection steps, the longest, set the
    // search's end), else one of the next
    // busy[l]: 0 free, 1 in flight, 2 held for candidate fl[l].cand (the lane keeps that
    // candidate's last Newton point's T, T', T'' for its next step, lane_launch_near)
    auto free_lane = [&](bool urgent = false) {
        const int first = urgent ? kCandLane : kUrgentEnd, nl = kLanes - kCandLane;
        for (int q = 0; q < nl; ++q) {
            const int l = kCandLane + (first - kCandLane + q) % nl;
            if (!busy[l]) return l;
        }
        // none free: wait for a lane in flight; with none in flight, give up a held lane
        // (only then, so that while lanes suffice the Taylor steps, and with them the
        // values, do not depend on timing)
        if (order.empty())
            for (int l = kCandLane; l < kLanes; ++l)
                if (busy[l] == 2) {
                    busy[l] = 0;
                    return l;
                }
        return -1;
    };
    auto release = [&](size_t c) {
        const int ll = last_lane[c];
        if (ll >= 0 && busy[ll] == 2 && fl[ll].cand == (int)c) busy[ll] = 0;
    };
    auto urgent = [&](size_t c) { return cstate[c] == 3 && nt[c].it >= 3; };
    auto unfinished = [&]() {
        if (chunks_done < nch) return (size_t)1 << 30;   // candidates still to come
        size_t u = 0;
        for (size_t c = 0; c < cstate.size(); ++c) u += cstate[c] < 2 || (cstate[c] == 3 && !nt[c].done);
        return u;
    };
    double out[3 * 64];
    auto grid_left = [&]() {
        for (int j = 0; j < nch; ++j)
            if (busy[j] && fl[j].kind == kGrid) return true;
        return false;
    };
    auto finish = [&](int lane) -> int {
        order.erase(std::find(order.begin(), order.end(), lane));
        const Flight F = fl[lane];
        busy[lane] = 0;
        if (F.kind == kGrid) {
            int fast = 1;
            if (int r = hbem::lane_results_grid(s, lane, out, &fast)) return r;
            const int first = F.cand * csize, cnt = std::min(csize, npoints - first);
            for (int q = 0; q < cnt; ++q) g[3 * (first + q)] = out[q];
            if (!fast) grid_ok = false;
            ++chunks_done;
            for (int q = 0; q < cnt; ++q) gknown[first + q] = 1;
            // 3-point local minima (roots_newton_polygon_rsvd.cpp:185-194) of the grid
            // triples this chunk completes (candidates are put in grid order at the end)
            for (int i = std::max(0, first - 2); i <= std::min(npoints - 3, first + cnt - 1); ++i) {
                if (scanned[i] || !gknown[i] || !gknown[i + 1] || !gknown[i + 2]) continue;
                scanned[i] = 1;
                const double L = g[3 * i], C = g[3 * (i + 1)], R = g[3 * (i + 2)];
                if (L - C > 0. && R - C > 0.) {
                    cgrid.push_back(i);
                    cstate.push_back(0);
                    cur.push_back(-1);
                    last_lane.push_back(-1);
                    last_gen.push_back(0);
                    last_x.push_back(NAN);
                    in_flight.push_back(0);
                    vsent.push_back(0);
                    cache.emplace_back();
                    pend.emplace_back();
                    nt.emplace_back();
                    vd.push_back(NAN);
                    vd.push_back(NAN);
                }
            }
            return HBEM_OK;
        }
        if (F.kind == kEnds) {
            double d[2];
            if (int r = hbem::lane_results_ends(s, lane, d)) return r;
            const size_t c = (size_t)F.cand;
            const int i = cgrid[c];
            g[3 * i + 1] = d[0];
            g[3 * (i + 2) + 1] = d[1];
            evals += 2;
            // validation sigma'(left) < 0 < sigma'(right), quartic guess (:209-245)
            if (!(d[0] < 0. && d[1] > 0.)) {
                cstate[c] = 2;
                return HBEM_OK;
            }
            const double guess = quartic_guess(ks[i], h, g[3 * i], g[3 * (i + 1)], g[3 * (i + 2)], d[0], d[1], tol);
            cur[c] = guess - ks[i] < 0.5 * h ? i : (guess - ks[i] < 1.5 * h ? i + 1 : i + 2);
            nt[c].start(ks[i], ks[i] + 2 * h, guess, tol);
            cstate[c] = 3;
            return HBEM_OK;
        }
        if (int r = hbem::lane_results(s, lane, c_o, c_i, out)) return r;
        if (F.kind == kSpec) {
            cache[F.cand].push_back({F.x, out[1], out[2]});
            pend[F.cand].erase(std::find(pend[F.cand].begin(), pend[F.cand].end(), F.x));
        } else if (F.kind == kVerify) {
            vd[2 * (size_t)F.cand + F.side] = out[1];
        } else if (F.kind == kVerify2) {
            vd[2 * (size_t)F.cand] = out[1];
            vd[2 * (size_t)F.cand + 1] = out[4];
        } else {
            const size_t c = (size_t)F.cand;
            nt[c].feed(out[1], out[2]);
            ++evals;
            in_flight[c] = 0;
            last_lane[c] = lane;
            last_gen[c] = lane_gen[lane];
            last_x[c] = F.x;
            // a root that has just converged: its sign-change check at once, on this lane,
            // from this point's T, T', T'' (the check points lie within 2 tol of it)
            if (vder && vsent[c] == 0 && nt[c].done && nt[c].found && nt[c].rts == nt[c].rts) {
                const double xv[2] = {nt[c].rts - tol, nt[c].rts + tol};
                const int ws[2] = {cur[c], cur[c]}, os[2] = {-1, -1};
                hbem::svd_pair_hold(grid_left() ? 1 : 0);
                const int r = hbem::lane_launch_near(s, lane, xv, 2, 1u, ws, os, npool);
                if (r == HBEM_OK) {
                    fl[lane] = Flight{(int)c, nt[c].rts, kVerify2, 0, cur[c]};
                    ++lane_gen[lane];
                    busy[lane] = 1;
                    order.push_back(lane);
                    vsent[c] = 2;
                } else if (r != HBEM_ERR_UNSUPPORTED) {
                    return r;
                }
            }
            // a Newton step of at most 1e-6 next: keep this lane's matrices for it
            if (!busy[lane] && !nt[c].done && std::fabs(nt[c].dx) <= 1e-6) busy[lane] = 2;
        }
        return HBEM_OK;
    };
    auto launch = [&](int lane, size_t c, double x, int kind, int side, int ws, int os) -> int {
        // one-CTA dense sigma while grid chunks still fill the GPU (a two-CTA cluster
        // would wait for them to drain), the paired form afterwards
        hbem::svd_pair_hold(grid_left() ? 1 : 0);
        if (int r = hbem::lane_launch(s, lane, &x, 1, c_o, c_i, &ws, &os, npool, kind == kVerify ? 1u : 2u)) return r;
        fl[lane] = Flight{(int)c, x, kind, side, ws};
        ++lane_gen[lane];
        busy[lane] = 1;
        order.push_back(lane);
        return HBEM_OK;
    };
    // candidate c's next launch, if it needs one: -1 when no lane is free, a status code
    // on error, 0 otherwise
    auto advance = [&](size_t c) -> int {
        for (;;) {
            if (cstate[c] == 2 || cstate[c] == 1) return 0;
            if (cstate[c] == 0) {
                const int lane = free_lane();
                if (lane < 0) return -1;
                const int i = cgrid[c];
                const double e2[2] = {ks[i], ks[i + 2]};
                const int gi[2] = {i, i + 2};
                if (int r = hbem::lane_launch_ends(s, lane, e2, gi, c_o, c_i)) return r;
                fl[lane] = Flight{(int)c, 0., kEnds, 0, -1};
                ++lane_gen[lane];
                busy[lane] = 1;
                order.push_back(lane);
                cstate[c] = 1;
                return 0;
            }
            if (in_flight[c]) return 0;
            // values already at hand (speculative points evaluated earlier)
            while (!nt[c].done) {
                auto it = std::find_if(cache[c].begin(), cache[c].end(),
                                       [&](const std::array<double, 3>& e) { return e[0] == nt[c].rts; });
                if (it == cache[c].end()) break;
                nt[c].feed((*it)[1], (*it)[2]);
                ++evals;
            }
            if (nt[c].done) {
                release(c);
                // a converged candidate: its root's sign-change check beside the others' work
                if (vder && vsent[c] < 2 && nt[c].found && nt[c].rts == nt[c].rts) {
                    const int l = free_lane(urgent(c));
                    if (l < 0) return -1;
                    const int side = vsent[c];
                    if (int r = launch(l, c, nt[c].rts + (side ? tol : -tol), kVerify, side, cur[c], -1)) return r;
                    ++vsent[c];
                    continue;
                }
                return 0;
            }
            if (has(pend[c], nt[c].rts)) {   // its point is on its way
                release(c);
                return 0;
            }
            const int own0 = npoints + 2 * (int)c, wslot = cur[c], oslot = cur[c] == own0 ? own0 + 1 : own0;
            // the slot this point's V set goes to must not be read by a speculative point
            // still in flight (it started from the slot before)
            bool waited = false;
            for (size_t q = 0; q < order.size(); ++q) {
                const int l = order[q];
                if (fl[l].cand == (int)c && fl[l].kind == kSpec && fl[l].rslot == oslot) {
                    int fin = 0;
                    if (int r = hbem::lane_wait(s, l, 1, &fin)) return r;
                    if (int r = finish(l)) return r;
                    waited = true;
                    break;
                }
            }
            if (waited) continue;   // look again: the wait may have brought this point's value
            // a Newton step of at most 1e-6 from the point just evaluated: that point's T,
            // T', T'' by their Taylor polynomials on the lane that holds them (no assembly)
            int lane = -1;
            const int ll = last_lane[c];
            const bool held = ll >= 0 && busy[ll] == 2 && fl[ll].cand == (int)c;
            release(c);
            if (held && lane_gen[ll] == last_gen[c] && std::fabs(nt[c].rts - last_x[c]) <= 1e-6) {
                const double x = nt[c].rts;
                hbem::svd_pair_hold(grid_left() ? 1 : 0);
                const int r = hbem::lane_launch_near(s, ll, &x, 1, 2u, &wslot, &oslot, npool);
                if (r == HBEM_OK) {
                    fl[ll] = Flight{(int)c, x, kMain, 0, wslot};
                    ++lane_gen[ll];
                    busy[ll] = 1;
                    order.push_back(ll);
                    lane = ll;
                } else if (r != HBEM_ERR_UNSUPPORTED) {
                    return r;
                }
            }
            if (lane < 0) {
                lane = free_lane(urgent(c));
                if (lane < 0) return -1;
                if (int r = launch(lane, c, nt[c].rts, kMain, 0, wslot, oslot)) return r;
            }
            in_flight[c] = 1;
            cur[c] = oslot;
            // speculative bisection points (plus the next level when few candidates are left)
            const size_t left = unfinished();
            if (left <= (size_t)spec_lim && (nt[c].first || nt[c].bisected)) {
                double pts[6];
                int np = nt[c].bisect_next(pts);
                if (left <= (size_t)spec_deep && !nt[c].first) {
                    const int n1 = np;
                    for (int j = 0; j < n1; ++j) {
                        // the state after a bisection to pts[j] (feed()'s operations)
                        Newton t = nt[c];
                        if (j == 0) t.xl = t.rts;
                        else t.xh = t.rts;
                        t.dx = 0.5 * (t.xh - t.xl);
                        t.rts = t.xl + t.dx;
                        if (t.rts == pts[j]) np += t.bisect_next(pts + np);
                    }
                }
                for (int j = 0; j < np; ++j) {
                    const double x = pts[j];
                    if (x == nt[c].rts || cached(c, x) || has(pend[c], x)) continue;
                    const int l2 = free_lane(urgent(c));
                    if (l2 < 0) break;
                    if (int r = launch(l2, c, x, kSpec, 0, wslot, -1)) return r;
                    pend[c].push_back(x);
                }
            }
            return 0;
        }
    };
    auto drain = [&]() {
        for (int l : order) {
            int fin = 0;
            hbem::lane_wait(s, l, 1, &fin);
        }
    };
    // the grid chunks (chunk j on lane j), assembled one after another from the top of
    // the range down: the sharpest minima, whose Newton runs take the most steps (long
    // bisection runs), tend to lie at the higher wavenumbers, so their runs start first
    for (int q = 0; q < nch; ++q) {
        const int j = nch - 1 - q;
        const int first = j * csize, cnt = std::min(csize, npoints - first);
        if (int r = hbem::lane_launch_grid(s, j, ks.data() + first, cnt, first, c_o, c_i, npool, q ? j + 1 : -1)) {
            drain();
            return r;
        }
        fl[j] = Flight{j, 0., kGrid, 0, -1};
        ++lane_gen[j];
        busy[j] = 1;
        order.push_back(j);
    }
    for (;;) {
        if (!grid_ok) {   // a grid matrix the fast kernel could not finish: the lock-step path redoes it
            drain();
            return HBEM_ERR_UNSUPPORTED;
        }
        for (size_t c = 0; c < cstate.size(); ++c) {
            const int r = advance(c);
            if (r == -1) break;
            if (r) {
                drain();
                return r;
            }
        }
        if (order.empty()) break;
        // the first lane to finish, whichever it is: poll them all (blocking on one lane
        // would hold up the results of lanes that finish before it)
        int pick = -1;
        for (long long spin = 0; pick < 0; ++spin) {
            for (size_t q = 0; q < order.size() && pick < 0; ++q) {
                int fin = 0;
                if (int r = hbem::lane_wait(s, order[q], 0, &fin)) {
                    drain();
                    return r;
                }
                if (fin) pick = order[q];
            }
            if (pick < 0 && spin > 64) std::this_thread::yield();
        }
        if (int r = finish(pick)) {
            drain();
            return r;
        }
    }
    // candidates in grid order, the order the lock-step search finds them in
    std::vector<size_t> by_k(cgrid.size());
    for (size_t c = 0; c < by_k.size(); ++c) by_k[c] = c;
    std::sort(by_k.begin(), by_k.end(), [&](size_t a, size_t b) { return cgrid[a] < cgrid[b]; });
    std::vector<Newton> nt_k;
    std::vector<double> vd_k;
    for (size_t c : by_k) {
        nt_k.push_back(nt[c]);
        vd_k.push_back(vd[2 * c]);
        vd_k.push_back(vd[2 * c + 1]);
    }
    nt.swap(nt_k);
    vd.swap(vd_k);
    if (vder) *vder = vd;
    hbem::pipeline_keep_uv(s, npoints);
    return HBEM_OK;
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

// BrentMinimizer::local_min_rc (find_roots.cpp:1003-1184): localmin above as a
// reverse-communication state machine; the caller evaluates f at the returned point
// while *status > 0 (the iterates are those of hbem_brent_min).
namespace {
struct BrentRC {
    double A, B, tol, eps, a = 0., b = 0., d = 0., e = 0., fu = 0., fv = 0., fw = 0., fx = 0., u = 0., v = 0., w = 0.,
                                    x = 0.;
};
}  // namespace

int hbem_brent_rc_create(double a, double b, double tol, void** handle) {
    if (!handle || !(a < b) || !(tol > 0.)) return HBEM_ERR_INVALID;
    *handle = new BrentRC{a, b, tol, std::sqrt(tol)};
    return HBEM_OK;
}

int hbem_brent_rc_destroy(void* handle) {
    delete static_cast<BrentRC*>(handle);
    return HBEM_OK;
}

double hbem_brent_rc_step(void* handle, int* status, double value) {
    BrentRC* R = static_cast<BrentRC*>(handle);
    if (!R || !status) return NAN;
    const double c = 0.5 * (3.0 - std::sqrt(5.0));
    if (*status == 0) {
        R->a = R->A;
        R->b = R->B;
        R->v = R->a + c * (R->b - R->a);
        R->w = R->x = R->v;
        R->e = R->d = 0.;
        *status = 1;
        return R->x;
    }
    if (*status == 1) {
        R->fx = R->fv = R->fw = value;
    } else {
        const double u = R->u, fu = value;
        if (fu <= R->fx) {
            if (R->x <= u) R->a = R->x; else R->b = R->x;
            R->v = R->w; R->fv = R->fw; R->w = R->x; R->fw = R->fx; R->x = u; R->fx = fu;
        } else {
            if (u < R->x) R->a = u; else R->b = u;
            if (fu <= R->fw || R->w == R->x) { R->v = R->w; R->fv = R->fw; R->w = u; R->fw = fu; }
            else if (fu <= R->fv || R->v == R->x || R->v == R->w) { R->v = u; R->fv = fu; }
        }
    }
    const double mid = 0.5 * (R->a + R->b), tol1 = R->eps * std::fabs(R->x) + R->tol / 3.0, tol2 = 2.0 * tol1;
    if (std::fabs(R->x - mid) <= tol2 - 0.5 * (R->b - R->a)) {
        *status = 0;
        return R->x;
    }
    bool golden = std::fabs(R->e) <= tol1;
    if (!golden) {
        double r = (R->x - R->w) * (R->fx - R->fv), q = (R->x - R->v) * (R->fx - R->fw),
               p = (R->x - R->v) * q - (R->x - R->w) * r;
        q = 2.0 * (q - r);
        if (q > 0.0) p = -p;
        q = std::fabs(q);
        r = R->e;
        R->e = R->d;
        if (std::fabs(0.5 * q * r) <= std::fabs(p) || p <= q * (R->a - R->x) || q * (R->b - R->x) <= p) {
            golden = true;
        } else {
            R->d = p / q;
            const double uu = R->x + R->d, sg = (mid - R->x) < 0. ? -1. : 1.;
            if ((uu - R->a) < tol2 || (R->b - uu) < tol2) R->d = tol1 * sg;
        }
    }
    if (golden) {
        R->e = (mid <= R->x) ? R->a - R->x : R->b - R->x;
        R->d = c * R->e;
    }
    R->u = std::fabs(R->d) >= tol1 ? R->x + R->d : R->x + tol1 * (R->d < 0. ? -1. : 1.);
    *status = 2;
    return R->u;
}

double hbem_brent_guess(hbem_fn f, void* user, double a, double b, double guess, double fguess, double tol,
                        unsigned* num_iter) {
    if (!f || !(a < b)) return NAN;
    return brent_guess(a, b, guess, fguess, [&](double x) { return f(x, user); }, tol, num_iter);
}

double hbem_brent_gsl_with_values(hbem_fn f, void* user, double a, double fa, double b, double fb, double guess,
                                  double fguess, double tol, unsigned* num_iter) {
    if (!f) return NAN;
    BrentSearch bs;
    bs.start(a, fa, b, fb, guess, fguess, tol);
    while (!bs.done) bs.feed(f(bs.u, user));
    if (num_iter) *num_iter = (unsigned)bs.it;
    return bs.ok ? bs.S.x : NAN;
}

double hbem_brent_gsl(hbem_fn f, void* user, double a, double b, double guess, double tol, unsigned* num_iter) {
    if (!f) return NAN;
    return hbem_brent_gsl_with_values(f, user, a, f(a, user), b, f(b, user), guess, f(guess, user), tol, num_iter);
}

double hbem_brent_min(hbem_fn f, void* user, double a, double b, double tol) {
    if (!(a < b)) return NAN;
    return localmin([&](double x) { return f(x, user); }, a, b, tol);
}

int hbem_find_resonances_plain(hbem_solop s, double k_min, double k_max, int npoints, double c_o, double c_i,
                               double tol, double* roots_host, int max_roots, int* nroots, double* grid_host,
                               int* n_evals) {
    return hbem_find_resonances_plain_verified(s, k_min, k_max, npoints, c_o, c_i, tol, roots_host, max_roots, nroots,
                                               grid_host, n_evals, nullptr);
}

int hbem_find_resonances_plain_verified(hbem_solop s, double k_min, double k_max, int npoints, double c_o, double c_i,
                                        double tol, double* roots_host, int max_roots, int* nroots, double* grid_host,
                                        int* n_evals, double* check_host) {
    if (!s || npoints < 3 || !(k_max > k_min) || !nroots) return HBEM_ERR_INVALID;
    std::vector<double> ks(npoints), g(3 * (size_t)npoints);
    const double h = (k_max - k_min) / (npoints - 1);
    for (int i = 0; i < npoints; ++i) ks[i] = k_min + i * h;
    int evals = npoints;
    std::vector<Newton> nt;
    std::vector<double> vder;
    bool checked = false, piped = false;
    // the whole search as one pipeline of streams (option "plain_async") where the
    // one-CTA dense kernel takes the order; else grid, bracket ends and lock-step
    // Newton rounds one after another
    if (hbem::plain_speculate_ok(s) && hbem::plain_warm_start_ok() && hbem::plain_async_ok()) {
        // its launches share the GPU with each other: the split singular launch of few
        // jobs (lower latency alone, more launches and CTAs) measured no faster there
        hbem::singular_split_hold(1);
        const int r = plain_pipelined(s, ks, h, c_o, c_i, tol, g, nt, check_host ? &vder : nullptr, evals);
        hbem::svd_pair_hold(0);
        hbem::singular_split_hold(0);
        if (r == HBEM_OK) {
            piped = true;
            checked = check_host != nullptr;
        } else if (r != HBEM_ERR_UNSUPPORTED) {
            return r;
        } else {
            evals = npoints;
        }
    }
    if (!piped) {
        // where sigma comes from the one-CTA dense kernel, every evaluation leaves its FP32
        // V set in a pool slot (grid point i: slot i) and later evaluations near it start
        // their Jacobi sweeps there
        bool warm = hbem::plain_speculate_ok(s) && hbem::plain_warm_start_ok();
        std::vector<int> wslot, oslot;
        // sigma on the grid (randomized_svd::sv / direct::sv at roots_newton_polygon_rsvd.cpp:172-177)
        if (warm) {
            wslot.assign(npoints, -1);
            oslot.resize(npoints);
            for (int i = 0; i < npoints; ++i) oslot[i] = i;
            const int r = hbem::sweep_sigma_warm(s, ks.data(), npoints, c_o, c_i, 0, wslot.data(), oslot.data(),
                                                 npoints, g.data(), 1);
            if (r == HBEM_ERR_UNSUPPORTED) warm = false;
            else if (r) return r;
        }
        if (!warm)
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
            // the bracket ends are grid points: sigma' from the grid's own singular vectors
            // (sv_der there would redo the same SVD), else their V sets start the Jacobi
            std::vector<int> gidx(ends.size());
            for (size_t c = 0; c < cidx.size(); ++c) {
                gidx[2 * c] = cidx[c];
                gidx[2 * c + 1] = cidx[c] + 2;
            }
            std::vector<double> d1v(ends.size());
            const int kept = warm ? hbem::sigma1_from_kept(s, ends.data(), gidx.data(), (int)ends.size(), c_o, c_i,
                                                           d1v.data())
                                  : (int)HBEM_ERR_UNSUPPORTED;
            if (kept == HBEM_OK) {
                for (size_t e = 0; e < ends.size(); ++e) {
                    der[3 * e] = g[3 * (size_t)gidx[e]];
                    der[3 * e + 1] = d1v[e];
                    der[3 * e + 2] = 0.;
                }
            } else if (kept != HBEM_ERR_UNSUPPORTED) {
                return kept;
            } else if (warm) {
                oslot.assign(ends.size(), -1);
                if (int r = hbem::sweep_sigma_warm(s, ends.data(), (int)ends.size(), c_o, c_i, 1, gidx.data(),
                                                   oslot.data(), npoints, der.data()))
                    return r;
            } else if (int r = hbem_sweep_sigma(s, ends.data(), (int)ends.size(), c_o, c_i, 1, der.data())) {
                return r;
            }
            evals += (int)ends.size();
        }
        // validation sigma'(left) < 0 < sigma'(right), quartic Hermite model + Brent (:209-245)
        struct Cand { double a, guess; };
        std::vector<Cand> cands;
        std::vector<int> first_warm;   // grid point beside the guess (its V set starts the first Newton point)
        for (size_t c = 0; c < cidx.size(); ++c) {
            const int i = cidx[c];
            const double d1 = der[3 * (2 * c) + 1], d2 = der[3 * (2 * c + 1) + 1];
            g[3 * i + 1] = d1;
            g[3 * (i + 2) + 1] = d2;
            if (!(d1 < 0. && d2 > 0.)) continue;
            cands.push_back(
                Cand{ks[i], quartic_guess(ks[i], h, g[3 * i], g[3 * (i + 1)], g[3 * (i + 2)], d1, d2, tol)});
            const double gs = cands.back().guess;
            first_warm.push_back(gs - ks[i] < 0.5 * h ? i : (gs - ks[i] < 1.5 * h ? i + 1 : i + 2));
        }
        nt.assign(cands.size(), Newton());
        for (size_t c = 0; c < cands.size(); ++c) nt[c].start(cands[c].a, cands[c].a + 2 * h, cands[c].guess, tol);
        // lock-step Newton rounds: one batched sigma', sigma'' evaluation per round (with
        // speculative bisection points where the dense sigma is latency bound)
        if (hbem::plain_speculate_ok(s)) {
            if (int r = newton_rounds(s, nt, c_o, c_i, evals, warm ? &first_warm : nullptr, npoints)) return r;
        } else {
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
        }
    }   // !piped
    if (grid_host) std::copy(g.begin(), g.end(), grid_host);
    int cnt = 0;
    std::vector<double> vpts;   // sign-change check points evaluated after the search
    for (size_t c = 0; c < nt.size(); ++c) {
        const Newton& x = nt[c];
        if (x.done && x.found && x.rts == x.rts) {
            if (roots_host && cnt < max_roots) roots_host[cnt] = x.rts;
            if (check_host && cnt < max_roots) {
                if (checked) {
                    check_host[2 * cnt] = vder[2 * c];
                    check_host[2 * cnt + 1] = vder[2 * c + 1];
                } else {
                    vpts.push_back(x.rts - tol);
                    vpts.push_back(x.rts + tol);
                }
            }
            ++cnt;
        }
    }
    if (check_host && !checked && !vpts.empty()) {
        // sigma' at both ends of every root in one batch after the search
        std::vector<double> o(3 * vpts.size());
        if (int r = hbem_sweep_sigma(s, vpts.data(), (int)vpts.size(), c_o, c_i, 1, o.data())) return r;
        for (size_t e = 0; e < vpts.size(); ++e) check_host[e] = o[3 * e + 1];
    }
    *nroots = cnt;
    if (n_evals) *n_evals = evals;
    return HBEM_OK;
}

// Local minima of sigma_min from candidate brackets (the confirmation step of the
// learned proposal; the Newton phase of the plain search above): sigma' at both ends
// of every bracket in one batch; a bracket with sigma'(a) < 0 < sigma'(b) goes to
// Newton from the secant zero of sigma'; one whose ends both rise (fall) is moved one
// width to the left (right), at most max_shift times; brackets that hold a maximum are
// dropped.  Newton rounds run in lock step (one batched sigma', sigma'' evaluation per
// round); roots closer than tol to an earlier one are merged.
int hbem_refine_brackets(hbem_solop s, const double* a_host, const double* b_host, int ncand, double c_o, double c_i,
                         double tol, int max_shift, double* roots_host, int max_roots, int* nroots, int* n_evals) {
    if (!s || ncand < 0 || (ncand > 0 && (!a_host || !b_host)) || !(tol > 0.) || max_shift < 0 || !nroots)
        return HBEM_ERR_INVALID;
    struct Br { double a, b, da, db; };
    std::vector<Br> live, valid;
    for (int c = 0; c < ncand; ++c)
        if (b_host[c] > a_host[c]) live.push_back(Br{a_host[c], b_host[c], 0., 0.});
    int evals = 0;
    for (int round = 0; round <= max_shift && !live.empty(); ++round) {
        std::vector<double> ends(2 * live.size()), der(6 * live.size());
        for (size_t c = 0; c < live.size(); ++c) {
            ends[2 * c] = live[c].a;
            ends[2 * c + 1] = live[c].b;
        }
        if (int r = hbem_sweep_sigma(s, ends.data(), (int)ends.size(), c_o, c_i, 1, der.data())) return r;
        evals += (int)ends.size();
        std::vector<Br> next;
        for (size_t c = 0; c < live.size(); ++c) {
            Br br = live[c];
            br.da = der[6 * c + 1];
            br.db = der[6 * c + 4];
            const double w = br.b - br.a;
            if (br.da < 0. && br.db > 0.) valid.push_back(br);
            else if (br.da >= 0. && br.db > 0.) next.push_back(Br{br.a - w, br.a, 0., 0.});
            else if (br.da < 0. && br.db <= 0.) next.push_back(Br{br.b, br.b + w, 0., 0.});
        }
        live.swap(next);
    }
    std::vector<Newton> nt(valid.size());
    for (size_t c = 0; c < valid.size(); ++c) {
        const Br& br = valid[c];
        const double guess = br.a - br.da * (br.b - br.a) / (br.db - br.da);
        nt[c].start(br.a, br.b, guess, tol);
    }
    // lock-step Newton rounds, with speculative bisection points where the dense sigma
    // is latency bound (the plain search's rounds)
    if (hbem::plain_speculate_ok(s)) {
        if (int r = newton_rounds(s, nt, c_o, c_i, evals)) return r;
    } else {
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
    }
    std::vector<double> roots;
    for (auto& x : nt)
        if (x.done && x.found && x.rts == x.rts) {
            bool dup = false;
            for (double r : roots) dup |= std::fabs(r - x.rts) <= tol;
            if (!dup) roots.push_back(x.rts);
        }
    std::sort(roots.begin(), roots.end());
    *nroots = (int)roots.size();
    for (size_t i = 0; i < roots.size() && (int)i < max_roots; ++i)
        if (roots_host) roots_host[i] = roots[i];
    if (n_evals) *n_evals = evals;
    return HBEM_OK;
}

// ---------------------------------------------------------------- many scatterers in lock step
//
// The plain search and the bracket refinement above, run for many (scatterer,
// k-window) pairs at once: every phase (grid, bracket ends, each Newton round) is one
// hbem_sweep_sigma_multi call over all pairs, so the per-scatterer launches overlap.

namespace {

struct MultiSigma {
    const hbem_solop* ops;
    int nops;
    double c_o;
    const double* c_i;
    int evals = 0;
    // ks[i]: the points of operator i; out[i]: 3 values per point
    int operator()(const std::vector<std::vector<double>>& ks, unsigned d, std::vector<std::vector<double>>& out) {
        std::vector<int> counts(nops);
        std::vector<double> flat;
        for (int i = 0; i < nops; ++i) {
            counts[i] = (int)ks[i].size();
            flat.insert(flat.end(), ks[i].begin(), ks[i].end());
        }
        out.assign(nops, {});
        if (flat.empty()) return HBEM_OK;
        std::vector<double> res(3 * flat.size());
        if (int r = hbem_sweep_sigma_multi(ops, nops, counts.data(), flat.data(), c_i, c_o, d, res.data())) return r;
        evals += (int)flat.size();
        size_t off = 0;
        for (int i = 0; i < nops; ++i) {
            out[i].assign(res.begin() + 3 * off, res.begin() + 3 * (off + counts[i]));
            off += counts[i];
        }
        return HBEM_OK;
    }
};

struct Job1 {
    int op;
    Newton nt;
};

// lock-step Newton over all (operator, candidate) states; the speculative bisection
// points of newton_rounds once at most kSpecRound candidates are left (the late,
// latency-bound rounds), with the same feeding rule, so the iterates are unchanged
int newton_multi(MultiSigma& ev, std::vector<Job1>& jobs) {
    std::vector<std::vector<std::array<double, 3>>> cache(jobs.size());   // (k, sigma', sigma'')
    bool spec_ok = true;   // every operator's sigma from the latency-bound dense kernel
    for (int i = 0; i < ev.nops; ++i) spec_ok &= hbem::plain_speculate_ok(ev.ops[i]) != 0;
    for (int round = 0; round < kMaxIt; ++round) {
        size_t active = 0;
        for (size_t c = 0; c < jobs.size(); ++c) {
            Newton& nt = jobs[c].nt;
            while (!nt.done) {
                auto it = std::find_if(cache[c].begin(), cache[c].end(),
                                       [&](const std::array<double, 3>& e) { return e[0] == nt.rts; });
                if (it == cache[c].end()) break;
                nt.feed((*it)[1], (*it)[2]);
                ++ev.evals;
            }
            active += nt.done ? 0 : 1;
        }
        if (!active) break;
        std::vector<std::vector<double>> xs(ev.nops);
        std::vector<std::vector<std::pair<size_t, bool>>> who(ev.nops);   // (job, speculative)
        for (size_t c = 0; c < jobs.size(); ++c) {
            Newton& nt = jobs[c].nt;
            if (nt.done) continue;
            xs[jobs[c].op].push_back(nt.rts);
            who[jobs[c].op].push_back({c, false});
            if (spec_ok && active <= (size_t)kSpecRound && (nt.first || nt.bisected)) {
                cache[c].clear();
                double sp[2];
                const int m = nt.bisect_next(sp);
                for (int j = 0; j < m; ++j)
                    if (sp[j] != nt.rts) {
                        xs[jobs[c].op].push_back(sp[j]);
                        who[jobs[c].op].push_back({c, true});
                    }
            }
        }
        std::vector<std::vector<double>> out;
        const int before = ev.evals;
        if (int r = ev(xs, 2, out)) return r;
        ev.evals = before;   // counted below: only the points the iterations use
        for (int i = 0; i < ev.nops; ++i)
            for (size_t q = 0; q < who[i].size(); ++q) {
                const size_t c = who[i][q].first;
                if (who[i][q].second) {
                    cache[c].push_back({xs[i][q], out[i][3 * q + 1], out[i][3 * q + 2]});
                } else {
                    jobs[c].nt.feed(out[i][3 * q + 1], out[i][3 * q + 2]);
                    ++ev.evals;
                }
            }
    }
    return HBEM_OK;
}

int collect_roots(int nops, const std::vector<Job1>& jobs, double tol, double* roots_host, int max_roots,
                  int* root_counts) {
    int total = 0;
    for (int i = 0; i < nops; ++i) {
        std::vector<double> r;
        for (const auto& j : jobs)
            if (j.op == i && j.nt.done && j.nt.found && j.nt.rts == j.nt.rts) {
                bool dup = false;
                for (double x : r) dup |= std::fabs(x - j.nt.rts) <= tol;
                if (!dup) r.push_back(j.nt.rts);
            }
        std::sort(r.begin(), r.end());
        if (root_counts) root_counts[i] = (int)r.size();
        for (double x : r) {
            if (roots_host && total < max_roots) roots_host[total] = x;
            ++total;
        }
    }
    return total;
}

}  // namespace

int hbem_find_resonances_plain_multi(const hbem_solop* ops, int nops, const double* k_min, const double* k_max,
                                     int npoints, double c_o, const double* c_i, double tol, double* roots_host,
                                     int max_roots, int* root_counts, int* n_evals) {
    if (!ops || nops < 1 || !k_min || !k_max || !c_i || npoints < 3 || !(tol > 0.)) return HBEM_ERR_INVALID;
    MultiSigma ev{ops, nops, c_o, c_i};
    std::vector<std::vector<double>> grid(nops), g;
    std::vector<double> h(nops);
    for (int i = 0; i < nops; ++i) {
        if (!(k_max[i] > k_min[i])) return HBEM_ERR_INVALID;
        h[i] = (k_max[i] - k_min[i]) / (npoints - 1);
        for (int j = 0; j < npoints; ++j) grid[i].push_back(k_min[i] + j * h[i]);
    }
    if (int r = ev(grid, 0, g)) return r;
    // 3-point minima, then sigma' at both bracket ends of all of them
    std::vector<std::vector<int>> cidx(nops);
    std::vector<std::vector<double>> ends(nops), der;
    for (int i = 0; i < nops; ++i)
        for (int j = 0; j + 2 < npoints; ++j) {
            const double L = g[i][3 * j], Cc = g[i][3 * (j + 1)], R = g[i][3 * (j + 2)];
            if (L - Cc > 0. && R - Cc > 0.) {
                cidx[i].push_back(j);
                ends[i].push_back(grid[i][j]);
                ends[i].push_back(grid[i][j + 2]);
            }
        }
    if (int r = ev(ends, 1, der)) return r;
    std::vector<Job1> jobs;
    for (int i = 0; i < nops; ++i)
        for (size_t c = 0; c < cidx[i].size(); ++c) {
            const int j = cidx[i][c];
            const double d1 = der[i][3 * (2 * c) + 1], d2 = der[i][3 * (2 * c + 1) + 1];
            if (!(d1 < 0. && d2 > 0.)) continue;
            Job1 jb;
            jb.op = i;
            jb.nt.start(grid[i][j], grid[i][j] + 2 * h[i],
                        quartic_guess(grid[i][j], h[i], g[i][3 * j], g[i][3 * (j + 1)], g[i][3 * (j + 2)], d1, d2, tol),
                        tol);
            jobs.push_back(jb);
        }
    if (int r = newton_multi(ev, jobs)) return r;
    collect_roots(nops, jobs, 0., roots_host, max_roots, root_counts);
    if (n_evals) *n_evals = ev.evals;
    return HBEM_OK;
}

int hbem_refine_brackets_multi(const hbem_solop* ops, int nops, const int* counts, const double* a_host,
                               const double* b_host, double c_o, const double* c_i, double tol, int max_shift,
                               double* roots_host, int max_roots, int* root_counts, int* n_evals) {
    if (!ops || nops < 1 || !counts || !c_i || !(tol > 0.) || max_shift < 0) return HBEM_ERR_INVALID;
    MultiSigma ev{ops, nops, c_o, c_i};
    struct Br { int op; double a, b, da, db; };
    std::vector<Br> live, valid;
    size_t off = 0;
    for (int i = 0; i < nops; ++i) {
        for (int c = 0; c < counts[i]; ++c)
            if (b_host[off + c] > a_host[off + c]) live.push_back(Br{i, a_host[off + c], b_host[off + c], 0., 0.});
        off += (size_t)counts[i];
    }
    for (int round = 0; round <= max_shift && !live.empty(); ++round) {
        std::vector<std::vector<double>> ends(nops), der;
        std::vector<std::vector<size_t>> who(nops);
        for (size_t c = 0; c < live.size(); ++c) {
            ends[live[c].op].push_back(live[c].a);
            ends[live[c].op].push_back(live[c].b);
            who[live[c].op].push_back(c);
        }
        if (int r = ev(ends, 1, der)) return r;
        std::vector<Br> next;
        for (int i = 0; i < nops; ++i)
            for (size_t q = 0; q < who[i].size(); ++q) {
                Br br = live[who[i][q]];
                br.da = der[i][6 * q + 1];
                br.db = der[i][6 * q + 4];
                const double w = br.b - br.a;
                if (br.da < 0. && br.db > 0.) valid.push_back(br);
                else if (br.da >= 0. && br.db > 0.) next.push_back(Br{br.op, br.a - w, br.a, 0., 0.});
                else if (br.da < 0. && br.db <= 0.) next.push_back(Br{br.op, br.b, br.b + w, 0., 0.});
            }
        live.swap(next);
    }
    std::vector<Job1> jobs;
    for (const Br& br : valid) {
        Job1 jb;
        jb.op = br.op;
        jb.nt.start(br.a, br.b, br.a - br.da * (br.b - br.a) / (br.db - br.da), tol);
        jobs.push_back(jb);
    }
    if (int r = newton_multi(ev, jobs)) return r;
    collect_roots(nops, jobs, tol, roots_host, max_roots, root_counts);
    if (n_evals) *n_evals = ev.evals;
    return HBEM_OK;
}

int hbem_opt_subdiv(hbem_fn_batch f, void* user, double x_min, double x_max, int batch_size, int limit, double tol,
                    unsigned long long seed, double* x_out, double* y_out, int max_points, int* n_points,
                    int* minima_out, int max_minima, int* n_minima) {
    if (!f || !(x_max > x_min) || batch_size < 1 || limit < 1 || !(tol >= 0.) || !n_points || !n_minima)
        return HBEM_ERR_INVALID;
    std::vector<std::pair<double, double>> xy;
    std::vector<int> p;
    BatchEval ev = [&](const double* xs, int n, double* ys) {
        f(xs, n, ys, user);
        return (int)HBEM_OK;
    };
    if (int r = opt_subdiv_impl(ev, x_min, x_max, batch_size, limit, tol, seed, xy, p)) return r;
    *n_points = (int)xy.size();
    for (size_t i = 0; i < xy.size() && (int)i < max_points; ++i) {
        if (x_out) x_out[i] = xy[i].first;
        if (y_out) y_out[i] = xy[i].second;
    }
    *n_minima = (int)p.size();
    for (size_t i = 0; i < p.size() && (int)i < max_minima; ++i)
        if (minima_out) minima_out[i] = p[i];
    return HBEM_OK;
}

int hbem_find_resonances_adaptive(hbem_solop s, double k_min, double k_max, double c_o, double c_i, int batch_size,
                                  int limit, double sample_tol, double tol, unsigned long long seed, int sketch,
                                  int q, double* roots_host, int max_roots, int* nroots, int* n_samples,
                                  int* n_evals) {
    if (!s || !(k_max > k_min) || batch_size < 1 || limit < 1 || !(tol > 0.) || sketch < 1 || q < 0 || !nroots)
        return HBEM_ERR_INVALID;
    int N = 0;
    if (int r = hbem_solop_info(s, &N)) return r;
    const int n = 2 * N;
    if (sketch > n) return HBEM_ERR_INVALID;
    int evals = 0;
    // sampling evaluator: randomized_svd::sv on a sketch of width `sketch`
    // (examples/find_resonances.cpp:135-139)
    BatchEval f_sample = [&](const double* ks, int nk, double* ys) {
        evals += nk;
        return hbem_sigma_rsvd_sweep(s, ks, nk, c_o, c_i, sketch, q, 0, seed, ys);
    };
    // local-search evaluator (the reference: arnoldi::sv): dense sigma_min for T up to
    // order 100, else the randomized estimate on a 16-wide sketch with q + 1 steps
    BatchEval f_fine = [&](const double* ks, int nk, double* ys) {
        evals += nk;
        if (n <= 100) {
            std::vector<double> out(3 * (size_t)nk);
            if (int r = hbem_sweep_sigma(s, ks, nk, c_o, c_i, 0, out.data())) return r;
            for (int i = 0; i < nk; ++i) ys[i] = out[3 * (size_t)i];
            return (int)HBEM_OK;
        }
        return hbem_sigma_rsvd_sweep(s, ks, nk, c_o, c_i, std::min(n, std::max(16, sketch)), q + 1, 0, seed + 1, ys);
    };
    std::vector<std::pair<double, double>> xy;
    std::vector<int> loc;
    if (int r = opt_subdiv_impl(f_sample, k_min, k_max, batch_size, limit, sample_tol, seed, xy, loc)) return r;
    const int np = (int)xy.size();
    if (n_samples) *n_samples = np;
    std::vector<double> kv(np), rsv(np);
    for (int i = 0; i < np; ++i) { kv[i] = xy[i].first; rsv[i] = xy[i].second; }
    // improve each candidate on a barycentric rational interpolant of its convex
    // neighbourhood (find_resonances.cpp:179-208)
    const size_t nc = loc.size();
    std::vector<double> A(nc), B(nc), G(nc);
    for (size_t c = 0; c < nc; ++c) {
        const int pos = loc[c];
        int il = pos, ir = pos;
        while (ir + 1 < np && rsv[ir - 1] + rsv[ir + 1] > 2. * rsv[ir]) ++ir;
        while (il > 0 && rsv[il - 1] + rsv[il + 1] > 2. * rsv[il]) --il;
        const int cnt = ir - il + 1;
        BaryRat interp;
        interp.init(&kv[il], &rsv[il], cnt, std::min(5, cnt - 1));
        A[c] = kv[pos - 1];
        B[c] = kv[pos + 1];
        double g = brent_guess(A[c], B[c], kv[pos], interp(kv[pos]), interp, tol);
        if (!(g > A[c] && g < B[c])) g = kv[pos];
        G[c] = g;
    }
    // lock-step Brent searches, one batched evaluation per round (find_resonances.cpp:225-237).
    // With the dense kernel, each candidate's evaluations start the FP32 Jacobi from the
    // V set of its previous one (pool slots 2c, 2c + 1 alternate; the guess G starts it).
    const bool warm = n <= 100 && hbem::plain_speculate_ok(s) && hbem::plain_warm_start_ok();
    std::vector<int> cur(nc, -1), wslot, oslot;
    const int npool = std::max(1, 2 * (int)nc);
    auto fine = [&](const std::vector<double>& xs, const std::vector<size_t>& who, bool first, double* ys) {
        if (!warm) return f_fine(xs.data(), (int)xs.size(), ys);
        evals += (int)xs.size();
        wslot.assign(xs.size(), -1);
        oslot.assign(xs.size(), -1);
        for (size_t q = 0; q < xs.size(); ++q) {
            const int c = (int)who[q];
            if (first) {
                if (q % 3 == 2) oslot[q] = 2 * c;   // the guess G
            } else {
                wslot[q] = cur[c];
                oslot[q] = cur[c] == 2 * c ? 2 * c + 1 : 2 * c;
            }
        }
        std::vector<double> out(3 * xs.size());
        if (int r = hbem::sweep_sigma_warm(s, xs.data(), (int)xs.size(), c_o, c_i, 0, wslot.data(), oslot.data(), npool,
                                           out.data()))
            return r;
        for (size_t q = 0; q < xs.size(); ++q) {
            ys[q] = out[3 * q];
            if (oslot[q] >= 0) cur[who[q]] = oslot[q];
        }
        return (int)HBEM_OK;
    };
    std::vector<BrentSearch> bs(nc);
    if (nc) {
        std::vector<double> xs(3 * nc), ys(3 * nc);
        std::vector<size_t> who(3 * nc);
        for (size_t c = 0; c < nc; ++c) {
            xs[3 * c] = A[c]; xs[3 * c + 1] = B[c]; xs[3 * c + 2] = G[c];
            who[3 * c] = who[3 * c + 1] = who[3 * c + 2] = c;
        }
        if (int r = fine(xs, who, true, ys.data())) return r;
        for (size_t c = 0; c < nc; ++c) bs[c].start(A[c], ys[3 * c], B[c], ys[3 * c + 1], G[c], ys[3 * c + 2], tol);
    }
    for (int round = 0; round < 200; ++round) {
        std::vector<double> xs;
        std::vector<size_t> who;
        for (size_t c = 0; c < nc; ++c)
            if (!bs[c].done) { xs.push_back(bs[c].u); who.push_back(c); }
        if (xs.empty()) break;
        std::vector<double> ys(xs.size());
        if (int r = fine(xs, who, false, ys.data())) return r;
        for (size_t w = 0; w < who.size(); ++w) bs[who[w]].feed(ys[w]);
    }
    std::vector<double> roots;
    for (auto& b : bs)
        if (b.ok && std::isfinite(b.S.x)) roots.push_back(b.S.x);
    std::sort(roots.begin(), roots.end());
    *nroots = (int)roots.size();
    for (size_t i = 0; i < roots.size() && (int)i < max_roots; ++i)
        if (roots_host) roots_host[i] = roots[i];
    if (n_evals) *n_evals = evals;
    return HBEM_OK;
}

}  // extern "C"
