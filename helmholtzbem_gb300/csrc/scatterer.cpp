// Scatterer input and polygonal panelisation (host code): the vertex-file reader,
// polygon length, automatic and Brent-chosen panel counts, and the uniform and
// corner-graded line-panel meshes of source/utilities/scatterer.cpp and
// examples/find_resonances.cpp.  Panels come out in the C-ABI layout (5 doubles per
// panel: x1 y1 x2 y2 0, kind HBEM_PANEL_LINE).
//
// Sums run in index order and vector norms are sqrt(x^2 + y^2), as the reference
// writes them; the library is built without floating-point contraction, so these
// results are the same on every host.
#include <cerrno>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <utility>
#include <vector>
#include <algorithm>

#include "../../include/hbem.h"

namespace {

struct V2 {
    double x, y;
};
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator*(V2 a, double s) { return {a.x * s, a.y * s}; }
inline V2 operator/(V2 a, double s) { return {a.x / s, a.y / s}; }
inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
inline double norm(V2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }

// std::stod: strtod on the token, no conversion -> invalid, ERANGE -> out of range
bool parse_double(const std::string& s, double& v) {
    if (s.empty()) return false;
    const char* b = s.c_str();
    char* e = nullptr;
    errno = 0;
    v = std::strtod(b, &e);
    if (e == b) return false;
    if (errno == ERANGE) return false;
    return true;
}

struct Panels {
    std::vector<double>* out;
    void line(V2 a, V2 b) { out->insert(out->end(), {a.x, a.y, b.x, b.y, 0.}); }
};

// ParametrizedLine(p, q).split(m): endpoints through the [-1, 1] parameter map
// (source/parametrizations/parametrized_line.cpp:23-29,112-131)
void split_line(V2 p, V2 q, int m, Panels& P) {
    for (int i = 0; i < m; ++i) {
        const double t1 = -1.0 + i * 2.0 / m;
        double t2 = -1.0 + (i + 1) * 2.0 / m;
        if (i == m - 1) t2 = 1.0;
        const V2 a{(t1 * (q.x - p.x) + (q.x + p.x)) * 0.5, (t1 * (q.y - p.y) + (q.y + p.y)) * 0.5};
        const V2 b{(t2 * (q.x - p.x) + (q.x + p.x)) * 0.5, (t2 * (q.y - p.y) + (q.y + p.y)) * 0.5};
        P.line(a, b);
    }
}

double polygon_length(const double* x, const double* y, int n) {
    double L = 0.;
    for (int i = 0; i < n; ++i) L += norm(V2{x[(i + 1) % n] - x[i], y[(i + 1) % n] - y[i]});
    return L;
}

// mean and population variance of d / k, index-order sums
void mean_var(const std::vector<double>& d, const std::vector<double>& k, double& mu, double& var) {
    const size_t n = d.size();
    double s = 0.;
    for (size_t i = 0; i < n; ++i) s += d[i] / k[i];
    mu = s / double(n);
    double q = 0.;
    for (size_t i = 0; i < n; ++i) {
        const double a = d[i] / k[i] - mu;
        q += a * a;
    }
    var = q / double(n);
}

// scatterer::make_N_polygonal_panels (source/utilities/scatterer.cpp:114-155)
void uniform_panels(const double* x, const double* y, int n, unsigned N, std::vector<double>& out) {
    std::vector<double> m(n), d(n);
    const double alpha = double(N) / polygon_length(x, y, n);
    long cs = 0;
    for (int i = 0; i < n; ++i) {
        const int j = i == n - 1 ? 0 : i + 1;
        d[i] = norm(V2{x[i] - x[j], y[i] - y[j]});
        m[i] = std::round(alpha * d[i]);
        cs += (long)m[i];
    }
    while (cs != (long)N) {
        const int k = cs > (long)N ? -1 : 1;
        double min_var = std::numeric_limits<double>::max(), mu, var;
        int i_min = 0;
        for (int i = 0; i < n; ++i) {
            m[i] += k;
            mean_var(d, m, mu, var);
            if (var < min_var) {
                min_var = var;
                i_min = i;
            }
            m[i] -= k;
        }
        m[i_min] += k;
        cs += k;
    }
    Panels P{&out};
    for (int i = 0; i < n; ++i) {
        const int j = i == n - 1 ? 0 : i + 1;
        split_line(V2{x[i], y[i]}, V2{x[j], y[j]}, (int)m[i], P);
    }
}

// scatterer::make_polygonal_panels (source/utilities/scatterer.cpp:157-277): edge
// panel counts proportional to the edge lengths, rounded one edge at a time (largest
// share first) to whichever of floor / floor + 1 keeps the panel lengths more even;
// on each edge with three or more panels the lengths grow geometrically from both
// corners, starting at f times the uniform length, f = rf + (1 - rf)(1 - cos angle)/2.
// The edge shares k_i = N d_i / L are the solution the reference obtains from a
// full-pivot LU of its proportionality system.
void graded_panels(const double* x, const double* y, int n, unsigned N, double rf, std::vector<double>& out) {
    const double eps = std::numeric_limits<double>::epsilon(), eps2 = 1e-3;
    const int kMaxIterAlpha = 5000;
    std::vector<double> d(n), k(n);
    for (int i = 0; i < n; ++i) {
        const int j = i < n - 1 ? i + 1 : 0;
        d[i] = norm(V2{x[j] - x[i], y[j] - y[i]});
    }
    double L = 0.;
    for (int i = 0; i < n; ++i) L += d[i];
    for (int i = 0; i < n; ++i) k[i] = double(N) * d[i] / L;
    // largest share first; equal shares: larger index first (descending pair order)
    std::vector<std::pair<double, int>> dd(n);
    for (int i = 0; i < n; ++i) dd[i] = {k[i], i};
    std::sort(dd.begin(), dd.end());
    std::reverse(dd.begin(), dd.end());
    auto obj = [&](double send) {
        double mu, var;
        mean_var(d, k, mu, var);
        double ks = 0.;
        for (int i = 0; i < n; ++i) ks += k[i];
        return std::sqrt(var) / mu + send * std::fabs(double(N) / ks - 1.0);
    };
    for (int i = 0; i < n; ++i) {
        const int j = dd[i].second;
        k[j] = std::floor(k[j]);
        const double f1 = obj(1.0);
        k[j] += 1.0;
        const double f2 = obj(1.0);
        if (f1 == f1 && f1 < f2) k[j] -= 1.0;
    }
    Panels P{&out};
    for (int i = 0; i < n; ++i) {
        const V2 p0{i == 0 ? x[n - 1] : x[i - 1], i == 0 ? y[n - 1] : y[i - 1]};
        const V2 p1{x[i], y[i]};
        const V2 p2{x[i < n - 1 ? i + 1 : 0], y[i < n - 1 ? i + 1 : 0]};
        const int i3 = i < n - 2 ? i + 2 : i - n + 2;
        const V2 p3{x[i3], y[i3]};
        const V2 D = (p2 - p1) / k[i];
        const int n_i = (int)k[i];
        double f1 = (1. - dot(p0 - p1, p2 - p1) / (norm(p0 - p1) * norm(p2 - p1))) / 2.;
        double f2 = (1. - dot(p1 - p2, p3 - p2) / (norm(p1 - p2) * norm(p3 - p2))) / 2.;
        f1 = rf + (1. - rf) * f1;
        f2 = rf + (1. - rf) * f2;
        if (rf >= 1. || n_i < 3) {
            for (int j = 0; j < n_i; ++j) P.line(p1 + D * double(j), j + 1 < n_i ? p1 + D * double(j + 1) : p2);
            continue;
        }
        // split panel j_best: lengths f1 D, f1 D / alpha, ... up to it and f2 D, f2 D / alpha,
        // ... back from p2, alpha the root (Newton from rf) that makes them add up to the edge
        int j_best = 0;
        double alpha_best = 0., d1_best = 0., d2_best = 0.;
        for (int j = 1; j < n_i; ++j) {
            double alpha, alpha_next = rf;
            auto f = [&](double t) {
                return f1 * std::pow(t, double(1 - j)) + f2 * std::pow(t, double(j + 1 - n_i)) - t * (f1 + f2) -
                       double(n_i) * (1. - t);
            };
            auto f_der = [&](double t) {
                return double(n_i) - f1 - f2 - f1 * (j - 1.) * std::pow(t, double(-j)) -
                       f2 * (n_i - j - 1.) * std::pow(t, double(j - n_i));
            };
            int iter_count = 0;
            do {
                alpha = alpha_next;
                alpha_next = alpha - f(alpha) / f_der(alpha);
                ++iter_count;
            } while (std::fabs(alpha_next - alpha) > eps && iter_count <= kMaxIterAlpha);
            const double d1 = f1 / std::pow(alpha, double(j - 1)), d2 = f2 / std::pow(alpha, double(n_i - j - 1));
            if (!j_best || std::fabs(d1 - d2) < std::fabs(d1_best - d2_best)) {
                d1_best = d1;
                d2_best = d2;
                j_best = j;
                alpha_best = alpha;
            }
        }
        const size_t mark = out.size();
        V2 pos = p1;
        for (int j = 0; j < n_i; ++j) {
            const V2 step = j < j_best ? D * d1_best * std::pow(alpha_best, double(j_best - 1 - j))
                                       : D * d2_best * std::pow(alpha_best, double(j - j_best));
            P.line(pos, j + 1 < n_i ? pos + step : p2);
            pos = pos + step;
        }
        if (norm(pos - p2) / norm(D) > eps2) {   // the grading missed p2: uniform panels instead
            out.resize(mark);
            pos = p1;
            for (int j = 0; j < n_i; ++j) {
                P.line(pos, j + 1 < n_i ? pos + D : p2);
                pos = pos + D;
            }
        }
    }
}

int copy_out(const std::vector<double>& v, double* params, int cap, int* npanels) {
    const int np = (int)(v.size() / 5);
    if (npanels) *npanels = np;
    if (!params) return HBEM_OK;
    if (np > cap) return HBEM_ERR_INVALID;
    std::copy(v.begin(), v.end(), params);
    return HBEM_OK;
}

bool valid_polygon(const double* x, const double* y, int n) { return x && y && n >= 3; }

struct ChooseCtx {
    const double *x, *y;
    int n;
    double target, rfac;
};

double max_panel_length(const std::vector<double>& v) {
    double r = 0.;
    for (size_t p = 0; p + 4 < v.size(); p += 5) {
        const double L = norm(V2{v[p + 2] - v[p], v[p + 3] - v[p + 1]});
        if (L > r) r = L;
    }
    return r;
}

double choose_objective(double Np, void* u) {
    const ChooseCtx* c = static_cast<const ChooseCtx*>(u);
    std::vector<double> v;
    graded_panels(c->x, c->y, c->n, (unsigned)std::round(Np), c->rfac, v);
    return std::fabs(c->target - max_panel_length(v));
}

}  // namespace

extern "C" {

int hbem_scatterer_read(const char* fname, double scale, double* x_host, double* y_host, int cap, int* nvert) {
    if (!fname || !nvert) return HBEM_ERR_INVALID;
    *nvert = 0;
    std::ifstream input(fname);
    if (!input) return HBEM_ERR_INVALID;
    std::vector<std::vector<double>> rows;
    std::string s, tok;
    size_t m = 0;
    while (std::getline(input, s)) {
        s.erase(std::remove_if(s.begin(), s.end(), [](unsigned char c) { return std::isspace(c) != 0; }), s.end());
        if (s.empty()) continue;
        std::vector<double> row;
        std::istringstream iss(s);
        while (std::getline(iss, tok, ',')) {
            double v;
            if (!parse_double(tok, v)) return HBEM_ERR_INVALID;
            row.push_back(v);
        }
        if (m == 0 || row.size() > m) m = row.size();
        rows.push_back(std::move(row));
    }
    if (rows.empty() || m != 2) return HBEM_ERR_INVALID;
    *nvert = (int)rows.size();
    if (!x_host || !y_host) return HBEM_OK;
    if ((int)rows.size() > cap) return HBEM_ERR_INVALID;
    for (size_t i = 0; i < rows.size(); ++i) {
        x_host[i] = scale * (rows[i].size() > 0 ? rows[i][0] : 0.);
        y_host[i] = scale * (rows[i].size() > 1 ? rows[i][1] : 0.);
    }
    return HBEM_OK;
}

double hbem_polygon_length(const double* x, const double* y, int n) {
    if (!x || !y || n < 1) return 0.;
    return polygon_length(x, y, n);
}

unsigned hbem_auto_num_panels(const double* x, const double* y, int n, double f) {
    if (!x || !y || n < 1) return 0;
    double min_s = std::numeric_limits<double>::max(), d = 0.;
    for (int i = 0; i < n; ++i) {
        const int j = i < n - 1 ? i + 1 : 0;
        const double l = norm(V2{x[j] - x[i], y[j] - y[i]});
        d += l;
        if (l < min_s) min_s = l;
    }
    return (unsigned)std::round(d / (min_s * f));
}

int hbem_polygon_panels(const double* x, const double* y, int n, unsigned N, double* params, int cap,
                        int* npanels) {
    if (!valid_polygon(x, y, n) || N < 1) return HBEM_ERR_INVALID;
    std::vector<double> v;
    uniform_panels(x, y, n, N, v);
    return copy_out(v, params, cap, npanels);
}

int hbem_polygon_panels_graded(const double* x, const double* y, int n, unsigned N, double refinement_factor,
                               double* params, int cap, int* npanels) {
    if (!valid_polygon(x, y, n) || N < 1 || !(refinement_factor > 0.)) return HBEM_ERR_INVALID;
    std::vector<double> v;
    graded_panels(x, y, n, N, refinement_factor, v);
    return copy_out(v, params, cap, npanels);
}

int hbem_choose_num_panels(const double* x, const double* y, int n, double k_max, double degf, double rfac,
                           unsigned* npanels) {
    if (!valid_polygon(x, y, n) || !npanels || !(k_max > 0.) || !(degf > 0.) || !(rfac > 0. && rfac < 1.))
        return HBEM_ERR_INVALID;
    const double pi = 3.14159265358979323846;
    const double inv_pi = 0.31830988618379067154;   // M_1_PI
    const double L = polygon_length(x, y, n), Np0 = degf * L * k_max * .5 * inv_pi;
    ChooseCtx c{x, y, n, 2. * pi / (degf * k_max), rfac};
    const double Np = hbem_brent_min(choose_objective, &c, Np0, Np0 / rfac, 1e-3);
    if (!(Np == Np)) return HBEM_ERR_INVALID;
    *npanels = (unsigned)std::round(Np);
    return HBEM_OK;
}

}  // extern "C"
