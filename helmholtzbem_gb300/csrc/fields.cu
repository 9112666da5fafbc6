// The Helmholtz transmission problem for an incoming wave and its field on a grid
// (tp::direct_second_kind::solve / solve_in_rectangle, include/solvers.hpp:65-200,
// source/utilities/solvers.cpp:116-391; incoming waves, source/utilities/incoming.cpp).
//
// Traces: T(k) of the unprojected solutions operator, the right-hand side
// [-K_o + M/2, V_o; W_o, K_o^T + M/2] (u_inc, du_inc/dn) at the panel start points,
// T x = rhs by the batched LU.
//
// Field: the traces become two periodic Akima splines over arc length; at every grid
// point x the Green representation
//   u(x) = s sum_{panels, Gauss nodes} w |gamma'| [H0(kappa r) t_N - kappa H1(kappa r) t_D (x - y).n / r],
// s = i/4 inside and -i/4 outside, kappa = k sqrt(c_i) or k sqrt(c_o), with the
// outside traces minus the incoming wave, is summed on the GPU (one thread per grid
// point, boundary nodes staged through shared memory).  Grid points on the boundary
// take the Dirichlet trace; for panels within 1e-2 / |kappa| of the point the
// panel's Gauss sum is replaced by a geometrically graded composite Gauss rule
// around the nearest point (one warp per such pair).
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/hbem.h"
#include "hbem_device.cuh"
#include "waves.cuh"

namespace hbem {

int set_error(int code, const char* msg);
int solop_mesh(hbem_solop s, int* n, const int** kinds, const double** par, int* proj, int* device);
int solop_gen_T(hbem_solop s, double k_re, double k_im, double c_o, double c_i, void* T_dev);
hbem_builder solop_builder(hbem_solop s);
void gauss_rule(double a, double b, int n, double* x, double* w);
void count_launches(long long n);
cudaError_t lu_factor_batched(int n, int nmat, cplx* A, long long stride, int* piv, int* perm, int* info,
                              cudaStream_t st, long long* launches);
cudaError_t lu_solve_batched(int n, int nmat, int trans, const cplx* LU, long long stride, const int* perm, int s,
                             cplx* X, long long xstride, cudaStream_t st);

namespace {

constexpr int kFieldSlices = 4;               // warps per CTA, each a share of panels / nodes
constexpr int kFieldThreads = 32 * kFieldSlices;
constexpr int kNodeTile = 128;
constexpr int kNearOrder = 12;        // Gauss points per graded sub-interval
constexpr int kNearLevels = 60;       // cap on the geometric levels per side
constexpr double kMachEpsF = 2.220446049250313e-16;

struct FNode {
    double yx, yy, nx, ny, D, pad;
    cplx tdi, tni, tdo, tno;          // Dirichlet / Neumann traces, inside and outside
};

struct NearEntry {
    int g, panel;
    double t;
};

// growable device buffer
struct Buf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

#define FD_CK(x)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return set_error(HBEM_ERR_CUDA, (std::string(#x) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

// ------------------------------------------------------------------ panels (device)

// point, tangent and tangent norm on [0, 1] (operator[] and Derivative_01 of
// ParametrizedLine / ParametrizedCircularArc)
__device__ __forceinline__ void fpan(const double* P, int kind, double t, double& px, double& py, double& tx,
                                     double& ty, double& tn) {
    if (kind == HBEM_PANEL_LINE) {
        tx = P[2] - P[0];
        ty = P[3] - P[1];
        px = t * tx + P[0];
        py = t * ty + P[1];
        tn = sqrt(tx * tx + ty * ty);
        return;
    }
    const double d = P[4] - P[3];
    double s, c;
    sincos(t * d + P[3], &s, &c);
    px = P[0] + P[2] * c;
    py = P[1] + P[2] * s;
    tx = -P[2] * d * s;
    ty = P[2] * d * c;
    tn = P[2] * fabs(d);
}

// distance from (x, y) to the panel and the parameter of the nearest point
// (scatterer::panel_distance, scatterer.cpp:279-341: the projection on a line; on an
// arc the nearest of the end points and the radial foot point when it lies on the arc)
__device__ double fpan_dist(const double* P, int kind, double x, double y, double& t) {
    if (kind == HBEM_PANEL_LINE) {
        const double hx = P[2] - P[0], hy = P[3] - P[1];
        double u = ((x - P[0]) * hx + (y - P[1]) * hy) / (hx * hx + hy * hy);
        u = fmax(0., fmin(1., u));
        t = u;
        const double dx = x - (P[0] + u * hx), dy = y - (P[1] + u * hy);
        return sqrt(dx * dx + dy * dy);
    }
    double px, py, tx, ty, tn;
    fpan(P, kind, 0., px, py, tx, ty, tn);
    double best = sqrt((x - px) * (x - px) + (y - py) * (y - py));
    t = 0.;
    fpan(P, kind, 1., px, py, tx, ty, tn);
    const double d1 = sqrt((x - px) * (x - px) + (y - py) * (y - py));
    if (d1 < best) {
        best = d1;
        t = 1.;
    }
    const double rx = x - P[0], ry = y - P[1], rho = sqrt(rx * rx + ry * ry), D = P[4] - P[3];
    if (rho > 0. && D != 0.) {
        const double th = atan2(ry, rx);
        for (int s = -2; s <= 2; ++s) {
            const double u = (th + s * 2. * kPi - P[3]) / D;
            if (u >= 0. && u <= 1.) {
                const double dd = fabs(rho - P[2]);
                if (dd < best) {
                    best = dd;
                    t = u;
                }
            }
        }
    }
    return best;
}

// scatterer::inside_mesh (scatterer.cpp:287-315), one panel's share: whether the
// leftward ray from the point crosses the chord between the panel's end points
// (half-open in y), and, for an arc, whether the point lies in the circular segment
// between chord and arc (tested only where the reference tests it: foot point inside
// the chord, chord distance <= 2 x signed length).  The point is inside when the
// crossings and the segments are odd in number together (crossings parity, flipped by
// an odd segment count).
__device__ __forceinline__ void inside_share(const double* P, int kind, double x, double y, int& cross, int& seg) {
    double x1, y1, x2, y2, tx, ty, tn;
    fpan(P, kind, 0., x1, y1, tx, ty, tn);
    fpan(P, kind, 1., x2, y2, tx, ty, tn);
    cross = ((((y1 <= y) && (y < y2)) || ((y2 <= y) && (y < y1))) && (x < (x2 - x1) * (y - y1) / (y2 - y1) + x1)) ? 1
                                                                                                                 : 0;
    seg = 0;
    if (kind == HBEM_PANEL_LINE) return;
    if ((x2 - x1) * (x - x1) + (y2 - y1) * (y - y1) <= 0. || (x1 - x2) * (x - x2) + (y1 - y2) * (y - y2) <= 0.)
        return;
    const double hx = x2 - x1, hy = y2 - y1;
    const double u = fmax(0., fmin(1., ((x - x1) * hx + (y - y1) * hy) / (hx * hx + hy * hy)));
    const double cdx = x - (x1 + u * hx), cdy = y - (y1 + u * hy);
    const double len = P[2] * (P[4] - P[3]);             // ParametrizedCircularArc::length (signed)
    if (sqrt(cdx * cdx + cdy * cdy) > 2. * len) return;
    const double rx = x - P[0], ry = y - P[1], half = 0.5 * (P[4] - P[3]);
    double sm, cm;
    sincos(P[3] + half, &sm, &cm);
    if (rx * rx + ry * ry < P[2] * P[2] && rx * cm + ry * sm > P[2] * cos(half)) seg = 1;
}

// ------------------------------------------------------------------ trace splines (device)

// interval of arc length s among the knots t[0..n] (clamped)
__device__ __forceinline__ int knot_interval(const double* t, int n, double s) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t[mid] <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

// spline coefficients per interval: [y, b, c, d] for the Dirichlet then the Neumann trace
__device__ __forceinline__ void trace_eval(const double* knots, const cplx* C, int n, double s, cplx& tD, cplx& tN) {
    const int i = knot_interval(knots, n, s);
    const double h = s - knots[i];
    const cplx* c = C + 8 * i;
    tD = c[0] + h * (c[1] + h * (c[2] + h * c[3]));
    tN = c[4] + h * (c[5] + h * (c[6] + h * c[7]));
}

struct FieldJob {
    int npan, nq, nx, ny, real_k, nw, total;
    double llx, lly, hx, hy;
    double kire, kiim, kore, koim;        // kappa inside / outside
    double abs_ki, abs_ko;
    double kre, kim;
    const int* kind;
    const double* par;
    const double* csum;                    // arc length at each panel's start
    const double* plen;                    // signed panel lengths
    const double* knots;                   // npan + 1 spline knots
    const cplx* spl;                       // npan x 8 spline coefficients
    const double* waves;
    const double* g21;
    const FNode* nodes;                    // npan x nq
    cplx* acc;                             // per grid point: the Green sum (unscaled)
    int* flag;                             // 0 outside, 1 inside, 2 | 4 x panel on the boundary
    double* bnd_t;
    NearEntry* near;
    int* near_count;
    int near_cap;
};

// grid point g: x = ll_x + i h_x, y = ll_y + j h_y, rounded as the host (and the
// reference) round them -- no fused multiply-add, so points on a coordinate line
// through a mesh vertex fall on the same side of it everywhere
__device__ __forceinline__ void grid_xy(const FieldJob& J, int g, double& x, double& y) {
    x = __dadd_rn(J.llx, __dmul_rn((double)(g % J.nx), J.hx));
    y = __dadd_rn(J.lly, __dmul_rn((double)(g / J.nx), J.hy));
}

__device__ __forceinline__ void hankel_pair(bool real_k, double kre, double kim, double r, cplx& h0, cplx& h1) {
    if (real_k) hankel01_real(kre * r, h0, h1);
    else hankel01_cplx(kre * r, kim * r, h0, h1);
}

// ------------------------------------------------------------------ kernels

// Green quadrature nodes: points, normals, weights x |gamma'|, splined traces and the
// outside traces (minus the incoming wave) -- in_solve, solvers.cpp:198-223
__global__ void k_field_nodes(FieldJob J, const double* xg, const double* wg, FNode* out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= J.npan * J.nq) return;
    const int i = q / J.nq, j = q % J.nq;
    const double* P = J.par + 5 * i;
    double px, py, tx, ty, tn;
    fpan(P, J.kind[i], xg[j], px, py, tx, ty, tn);
    FNode n;
    n.yx = px;
    n.yy = py;
    n.D = tn * wg[j];
    n.pad = 0.;
    n.nx = ty / tn;
    n.ny = -tx / tn;
    trace_eval(J.knots, J.spl, J.npan, J.csum[i] + xg[j] * J.plen[i], n.tdi, n.tni);
    cplx u, ux, uy;
    wave_eval(J.waves, J.nw, J.g21, J.kre, J.kim, px, py, true, u, ux, uy);
    n.tdo = n.tdi - u;
    n.tno = n.tni - (n.nx * ux + n.ny * uy);
    out[q] = n;
}

// 32 grid points per CTA, one per lane; the CTA's four warps split the panels for the
// inside / boundary / near tests and the boundary nodes of every shared-memory tile
// for the Green sum, then combine through shared memory.
__global__ void __launch_bounds__(kFieldThreads) k_field_grid(FieldJob J) {
    __shared__ FNode tile[kNodeTile];
    __shared__ int s_cross[kFieldSlices][32], s_seg[kFieldSlices][32], s_onb[kFieldSlices][32];
    __shared__ double s_bt[kFieldSlices][32];
    __shared__ cplx s_part[kFieldSlices][32];
    const int G = J.nx * J.ny, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = blockIdx.x * 32 + lane;
    double x = 0., y = 0.;
    int cross = 0, seg = 0, onb = 0x7fffffff;
    double bt = 0.;
    if (g < G) {
        grid_xy(J, g, x, y);
        for (int i = w; i < J.npan; i += kFieldSlices) {
            int c, sg;
            inside_share(J.par + 5 * i, J.kind[i], x, y, c, sg);
            cross ^= c;
            seg += sg;
        }
    }
    s_cross[w][lane] = cross;
    s_seg[w][lane] = seg;
    __syncthreads();
    for (int q = 0; q < kFieldSlices; ++q)
        if (q != w) {
            cross ^= s_cross[q][lane];
            seg += s_seg[q][lane];
        }
    const bool inside = (seg & 1) ? !cross : (cross != 0);
    if (g < G) {
        const double akap = inside ? J.abs_ki : J.abs_ko;
        for (int i = w; i < J.npan; i += kFieldSlices) {
            double t;
            const double d = fpan_dist(J.par + 5 * i, J.kind[i], x, y, t);
            if (d < 1e2 * kMachEpsF) {            // on the boundary: the Dirichlet trace
                onb = i;
                bt = t;
                break;
            }
            if (d * akap < 1e-2) {
                const int slot = atomicAdd(J.near_count, 1);
                if (slot < J.near_cap) J.near[slot] = NearEntry{g, i, t};
            }
        }
    }
    s_onb[w][lane] = onb;
    s_bt[w][lane] = bt;
    __syncthreads();
    for (int q = 0; q < kFieldSlices; ++q)       // the first panel in index order
        if (s_onb[q][lane] < onb) {
            onb = s_onb[q][lane];
            bt = s_bt[q][lane];
        }
    const bool active = g < G && onb == 0x7fffffff;
    if (g < G && w == 0) {
        J.flag[g] = onb != 0x7fffffff ? (2 | (onb << 2)) : (inside ? 1 : 0);
        if (onb != 0x7fffffff) J.bnd_t[g] = bt;
    }
    const double kr = inside ? J.kire : J.kore, ki = inside ? J.kiim : J.koim;
    const double ikr = kr > 0. ? 1.0 / kr : 0.;
    cplx sum = mk(0.);
    const int M = J.npan * J.nq;
    constexpr int kPerWarp = kNodeTile / kFieldSlices;
    for (int base = 0; base < M; base += kNodeTile) {
        const int cnt = min(kNodeTile, M - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kFieldThreads) tile[e] = J.nodes[base + e];
        __syncthreads();
        if (!active) continue;
        const int e1 = min(cnt, (w + 1) * kPerWarp);
        for (int e = w * kPerWarp; e < e1; ++e) {
            const FNode& nd = tile[e];
            const double zx = x - nd.yx, zy = y - nd.yy, r2 = zx * zx + zy * zy;
            if (!(r2 > 0.)) continue;
            // 1/r once: the normal projection and (real k) the Hankel pair's 1/x use it
            const double ir = rsqrt(r2), r = r2 * ir;
            cplx h0, h1;
            if (J.real_k) hankel01_real_ix(kr * r, ikr * ir, h0, h1);
            else hankel01_cplx(kr * r, ki * r, h0, h1);
            const double zn = (zx * nd.nx + zy * nd.ny) * ir;
            const cplx tD = inside ? nd.tdi : nd.tdo, tN = inside ? nd.tni : nd.tno;
            cplx term = h0 * tN - (mk(kr, ki) * zn) * (h1 * tD);
            sum += nd.D * term;
        }
    }
    s_part[w][lane] = sum;
    __syncthreads();
    if (w == 0 && g < G) {
        cplx tot = s_part[0][lane];
        for (int q = 1; q < kFieldSlices; ++q) tot += s_part[q][lane];
        J.acc[g] = tot;
    }
}

// f(t) of the near-panel integral (the integrand of solvers.cpp:275-293)
__device__ cplx near_integrand(const FieldJob& J, int i, double t, double x, double y, bool inside, double kr,
                               double ki) {
    const double* P = J.par + 5 * i;
    double px, py, tx, ty, tn;
    fpan(P, J.kind[i], t, px, py, tx, ty, tn);
    const double zx = x - px, zy = y - py, d = sqrt(zx * zx + zy * zy);
    if (d == 0.) return mk(0.);
    cplx h0, h1, tD, tN;
    hankel_pair(J.real_k, kr, ki, d, h0, h1);
    trace_eval(J.knots, J.spl, J.npan, J.csum[i] + t * J.plen[i], tD, tN);
    const double nx = ty / tn, ny = -tx / tn;
    if (!inside) {
        cplx u, ux, uy;
        wave_eval(J.waves, J.nw, J.g21, J.kre, J.kim, px, py, true, u, ux, uy);
        tD = tD - u;
        tN = tN - (nx * ux + ny * uy);
    }
    return tn * (h0 * tN - (mk(kr, ki) * ((nx * zx + ny * zy) / d)) * (h1 * tD));
}

// one warp per near (grid point, panel) pair: out[e] = graded integral - Gauss sum
__global__ void __launch_bounds__(256) k_field_near(FieldJob J, const NearEntry* ent, int nent, const double* xq,
                                                    const double* wq, cplx* out) {
    const int lane = threadIdx.x & 31;
    const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (e >= nent) return;
    const NearEntry E = ent[e];
    const int g = E.g, i = E.panel;
    double x, y;
    grid_xy(J, g, x, y);
    const bool inside = (J.flag[g] & 3) == 1;
    const double kr = inside ? J.kire : J.kore, ki = inside ? J.kiim : J.koim;
    // regular Gauss sum of the panel (what the grid kernel added)
    cplx reg = mk(0.);
    for (int j = lane; j < J.nq; j += 32) {
        const FNode& nd = J.nodes[i * J.nq + j];
        const double zx = x - nd.yx, zy = y - nd.yy, r = sqrt(zx * zx + zy * zy);
        if (!(r > 0.)) continue;
        cplx h0, h1;
        hankel_pair(J.real_k, kr, ki, r, h0, h1);
        const double zn = (zx * nd.nx + zy * nd.ny) / r;
        const cplx tD = inside ? nd.tdi : nd.tdo, tN = inside ? nd.tni : nd.tno;
        reg += nd.D * (h0 * tN - (mk(kr, ki) * zn) * (h1 * tD));
    }
    // graded composite rule on [0, t] and [t, 1]: sub-intervals halve towards t down
    // to the scale of the distance (in parameter units), then one last interval
    const double* P = J.par + 5 * i;
    double px, py, tx, ty, tn;
    fpan(P, J.kind[i], E.t, px, py, tx, ty, tn);
    const double dist = sqrt((x - px) * (x - px) + (y - py) * (y - py));
    const double delta = fmax(dist / fmax(fabs(J.plen[i]), 1e-300), 1e-15);
    cplx acc = mk(0.);
    for (int side = 0; side < 2; ++side) {
        const double span = side == 0 ? E.t : 1. - E.t;
        if (!(span > 0.)) continue;
        int L = (int)ceil(log2(span / delta)) + 1;
        L = max(1, min(kNearLevels, L));
        const int npts = (L + 1) * kNearOrder;
        for (int idx = lane; idx < npts; idx += 32) {
            const int l = idx / kNearOrder, q = idx % kNearOrder;
            // interval l < L: distances from t in [span 2^-(l+1), span 2^-l]; l = L: [0, span 2^-L]
            const double far = l < L ? span * ldexp(1., -l) : span * ldexp(1., -L);
            const double near = l < L ? span * ldexp(1., -(l + 1)) : 0.;
            const double dd = near + (far - near) * xq[q], w = (far - near) * wq[q];
            const double tt = side == 0 ? E.t - dd : E.t + dd;
            acc += w * near_integrand(J, i, tt, x, y, inside, kr, ki);
        }
    }
    cplx v = acc - reg;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
        v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
    }
    if (lane == 0) out[e] = v;
}

__global__ void k_field_add(const int* idx, const cplx* val, int n, cplx* acc) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) acc[idx[e]] += val[e];
}

// S = s (sum + excess) (+ u_inc outside), or the Dirichlet trace on the boundary
__global__ void k_field_finalize(FieldJob J, cplx* S) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= J.nx * J.ny) return;
    const int fl = J.flag[g];
    if (fl & 2) {
        const int i = fl >> 2;
        cplx tD, tN;
        trace_eval(J.knots, J.spl, J.npan, J.csum[i] + J.bnd_t[g] * J.plen[i], tD, tN);
        S[g] = tD;
        return;
    }
    const bool inside = fl == 1;
    const cplx a = J.acc[g];
    cplx v = inside ? mk(-0.25 * a.im, 0.25 * a.re) : mk(0.25 * a.im, -0.25 * a.re);
    if (J.total && !inside) {
        cplx u, ux, uy;
        double x, y;
        grid_xy(J, g, x, y);
        wave_eval(J.waves, J.nw, J.g21, J.kre, J.kim, x, y, false, u, ux, uy);
        v += u;
    }
    S[g] = v;
}

// u_inc and du_inc/dn at the panel start points (Interpolate_helmholtz / _neu of
// ContinuousSpace<1>, include/continuous_space.hpp:67-101)
__global__ void k_tp_inc(int npan, const int* kind, const double* par, const double* waves, int nw, const double* g21,
                         double kre, double kim, cplx* uD, cplx* uN) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npan) return;
    double px, py, tx, ty, tn;
    fpan(par + 5 * i, kind[i], 0., px, py, tx, ty, tn);
    cplx u, ux, uy;
    wave_eval(waves, nw, g21, kre, kim, px, py, true, u, ux, uy);
    uD[i] = u;
    const double nx = ty / tn, ny = -tx / tn;
    uN[i] = nx * ux + ny * uy;
}

// rhs = [-K_o + M/2, V_o; W_o, K_o^T + M/2] [uD; uN] (A_rhs, solvers.cpp:116-141)
__global__ void k_tp_rhs(int N, const cplx* K, const cplx* V, const cplx* W, const double* M, const cplx* uD,
                         const cplx* uN, cplx* rhs) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= 2 * N) return;
    cplx s = mk(0.);
    if (row < N) {
        const int i = row;
        for (int j = 0; j < N; ++j) {
            const size_t e = i + (size_t)j * N;
            s += (mk(0.5 * M[e]) - K[e]) * uD[j];
            s += V[e] * uN[j];
        }
    } else {
        const int i = row - N;
        for (int j = 0; j < N; ++j) {
            const size_t e = i + (size_t)j * N;
            s += W[e] * uD[j];
            s += (K[j + (size_t)i * N] + mk(0.5 * M[e])) * uN[j];
        }
    }
    rhs[row] = s;
}

__global__ void k_nonfinite(const cplx* a, long long n, int* flag) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        if (!isfinite(a[e].re) || !isfinite(a[e].im)) *flag = 1;
}

__global__ void k_wave_points(const double* waves, int nw, const double* g21, double kre, double kim, const double* xy,
                              int n, cplx* u, cplx* du) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    cplx a, b, c;
    wave_eval(waves, nw, g21, kre, kim, xy[2 * e], xy[2 * e + 1], du != nullptr, a, b, c);
    u[e] = a;
    if (du) {
        du[2 * e] = b;
        du[2 * e + 1] = c;
    }
}

// ------------------------------------------------------------------ host helpers

// Akima's slopes (Akima 1970) on a periodic knot sequence t[0..n] with y[n] = y[0],
// interval slopes m_j extended periodically; where both weights vanish the corner is
// left unrounded (Wodicka): the interval to the left ends with slope m_(i-1), the
// interval to the right starts with m_i.  Cubic Hermite pieces per interval:
// y_i + b h + c h^2 + d h^3.
void akima_periodic(const std::vector<double>& t, const std::vector<double>& y, std::vector<double>& b,
                    std::vector<double>& c, std::vector<double>& d) {
    const int n = (int)t.size() - 1;
    std::vector<double> m(n), tl(n + 1), tr(n + 1);
    for (int j = 0; j < n; ++j) m[j] = (y[j + 1] - y[j]) / (t[j + 1] - t[j]);
    auto M = [&](int j) { return m[((j % n) + n) % n]; };
    for (int i = 0; i <= n; ++i) {
        const double w1 = std::fabs(M(i + 1) - M(i)), w2 = std::fabs(M(i - 1) - M(i - 2));
        if (w1 + w2 == 0.) {
            tl[i] = M(i - 1);
            tr[i] = M(i);
        } else {
            tl[i] = tr[i] = (w1 * M(i - 1) + w2 * M(i)) / (w1 + w2);
        }
    }
    b.assign(n, 0.);
    c.assign(n, 0.);
    d.assign(n, 0.);
    for (int i = 0; i < n; ++i) {
        const double h = t[i + 1] - t[i];
        b[i] = tr[i];
        c[i] = (3. * m[i] - 2. * tr[i] - tl[i + 1]) / h;
        d[i] = (tr[i] + tl[i + 1] - 2. * m[i]) / (h * h);
    }
}

// incoming::load field parsers (std::stod / std::stoi on one comma-separated field)
bool field_double(std::istringstream& iss, double& v) {
    std::string tok;
    if (!std::getline(iss, tok, ',')) return false;
    if (tok.empty()) return false;
    const char* b = tok.c_str();
    char* e = nullptr;
    errno = 0;
    v = std::strtod(b, &e);
    return e != b && errno != ERANGE;
}

bool field_int(std::istringstream& iss, int& v) {
    std::string tok;
    if (!std::getline(iss, tok, ',')) return false;
    if (tok.empty()) return false;
    const char* b = tok.c_str();
    char* e = nullptr;
    errno = 0;
    const long r = std::strtol(b, &e, 10);
    if (e == b || errno == ERANGE || r < -2147483648L || r > 2147483647L) return false;
    v = (int)r;
    return true;
}

int check_waves(const double* waves, int nw, double k_im) {
    if (nw < 0 || (nw > 0 && !waves)) return set_error(HBEM_ERR_INVALID, "incoming wave: bad argument");
    for (int q = 0; q < nw; ++q) {
        const int type = (int)waves[kWaveDoubles * q];
        if (type < WAVE_PLANE || type > WAVE_HERGLOTZ || (double)type != waves[kWaveDoubles * q])
            return set_error(HBEM_ERR_INVALID, "incoming wave: unknown wave type");
        if (type != WAVE_PLANE && type != WAVE_HERGLOTZ && k_im != 0.)
            return set_error(HBEM_ERR_UNSUPPORTED,
                             "incoming wave: circular and Fourier-Hankel waves need a real wavenumber here");
        if (std::fabs(waves[kWaveDoubles * q + 6]) > 10000.)
            return set_error(HBEM_ERR_INVALID, "incoming wave: order above 10000");
    }
    return HBEM_OK;
}

struct FieldState {
    Buf waves, g21, T, piv, perm, info, uD, uN, rhs, M, flagbuf;
    Buf kind, par, csum, plen, knots, spl, nodes, xg, wg, acc, flag, bndt, near, nearcnt, xq, wq, nearout, addidx,
        addval, S;
    double last_grid_ms = 0.;
    long long last_units = 0, last_near = 0;
};

FieldState& state() {
    static thread_local FieldState s;
    return s;
}

template <class T>
cudaError_t put(Buf& b, const T* src, size_t n) {
    cudaError_t e = b.ensure(std::max<size_t>(1, n * sizeof(T)));
    if (e != cudaSuccess || n == 0) return e;
    return cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

int upload_waves(FieldState& F, const double* waves, int nw) {
    std::vector<double> g(2 * kHerglotzNodes);
    gauss_rule(0., 1., kHerglotzNodes, g.data(), g.data() + kHerglotzNodes);
    FD_CK(put(F.g21, g.data(), g.size()));
    FD_CK(put(F.waves, waves, (size_t)nw * kWaveDoubles));
    return HBEM_OK;
}

// traces of the transmission problem into F.rhs (2N complex, device)
int tp_solve_device(hbem_solop s, const double* waves, int nw, double k_re, double k_im, double c_o, double c_i, int& N) {
    FieldState& F = state();
    const int* kinds;
    const double* par;
    int proj, device;
    if (int r = solop_mesh(s, &N, &kinds, &par, &proj, &device)) return r;
    if (proj) return set_error(HBEM_ERR_INVALID, "tp solve: the solutions operator must be created without projection");
    if (int r = check_waves(waves, nw, k_im)) return r;
    FD_CK(cudaSetDevice(device));
    const size_t n2 = 2 * (size_t)N;
    FD_CK(F.T.ensure(n2 * n2 * sizeof(cplx)));
    if (int r = solop_gen_T(s, k_re, k_im, c_o, c_i, F.T.p)) return r;
    hbem_builder b = solop_builder(s);
    if (int r = hbem_assemble_dense(b, k_re, k_im, c_o, HBEM_LAYER_ALL, 0)) return r;
    const void *K, *V, *W;
    if (int r = hbem_get_layer_device(b, HBEM_LAYER_DOUBLE, 0, &K)) return r;
    if (int r = hbem_get_layer_device(b, HBEM_LAYER_SINGLE, 0, &V)) return r;
    if (int r = hbem_get_layer_device(b, HBEM_LAYER_HYPERSINGULAR, 0, &W)) return r;
    std::vector<double> M((size_t)N * N);
    if (int r = hbem_mass_matrix(s, M.data())) return r;
    FD_CK(put(F.M, M.data(), M.size()));
    if (int r = upload_waves(F, waves, nw)) return r;
    FD_CK(put(F.kind, kinds, (size_t)N));
    FD_CK(put(F.par, par, (size_t)N * 5));
    FD_CK(F.uD.ensure(N * sizeof(cplx)));
    FD_CK(F.uN.ensure(N * sizeof(cplx)));
    FD_CK(F.rhs.ensure(n2 * sizeof(cplx)));
    k_tp_inc<<<(N + 127) / 128, 128>>>(N, F.kind.as<int>(), F.par.as<double>(), F.waves.as<double>(), nw,
                                       F.g21.as<double>(), k_re, k_im, F.uD.as<cplx>(), F.uN.as<cplx>());
    k_tp_rhs<<<(unsigned)((n2 + 127) / 128), 128>>>(N, static_cast<const cplx*>(K), static_cast<const cplx*>(V),
                                                    static_cast<const cplx*>(W), F.M.as<double>(), F.uD.as<cplx>(),
                                                    F.uN.as<cplx>(), F.rhs.as<cplx>());
    FD_CK(cudaGetLastError());
    FD_CK(F.flagbuf.ensure(2 * sizeof(int)));
    FD_CK(cudaMemset(F.flagbuf.p, 0, 2 * sizeof(int)));
    k_nonfinite<<<64, 256>>>(F.rhs.as<cplx>(), (long long)n2, F.flagbuf.as<int>());
    k_nonfinite<<<1024, 256>>>(F.T.as<cplx>(), (long long)(n2 * n2), F.flagbuf.as<int>() + 1);
    count_launches(4);
    int fl[2];
    FD_CK(cudaMemcpy(fl, F.flagbuf.p, sizeof(fl), cudaMemcpyDeviceToHost));
    if (fl[0]) return set_error(HBEM_ERR_NONFINITE, "Failed to solve for traces, right-hand side is undefined");
    if (fl[1]) return set_error(HBEM_ERR_NONFINITE, "Failed to solve for traces, solutions operator is undefined");
    FD_CK(F.piv.ensure(n2 * sizeof(int)));
    FD_CK(F.perm.ensure(n2 * sizeof(int)));
    FD_CK(F.info.ensure(sizeof(int)));
    long long nl = 0;
    FD_CK(lu_factor_batched((int)n2, 1, F.T.as<cplx>(), (long long)(n2 * n2), F.piv.as<int>(), F.perm.as<int>(),
                            F.info.as<int>(), 0, &nl));
    int info = 0;
    FD_CK(cudaMemcpy(&info, F.info.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (info) return set_error(HBEM_ERR_SINGULAR, "zgesv: LU is singular");
    FD_CK(lu_solve_batched((int)n2, 1, 0, F.T.as<cplx>(), (long long)(n2 * n2), F.perm.as<int>(), 1, F.rhs.as<cplx>(),
                           (long long)n2, 0));
    count_launches(nl + 1);
    FD_CK(cudaDeviceSynchronize());
    return HBEM_OK;
}

}  // namespace
}  // namespace hbem

using namespace hbem;

extern "C" {

int hbem_incoming_load(const char* fname, double* waves, int cap, int* nwaves) {
    if (!fname || !nwaves) return set_error(HBEM_ERR_INVALID, "incoming::load: bad argument");
    *nwaves = 0;
    std::ifstream input(fname);
    if (!input) return set_error(HBEM_ERR_INVALID, "incoming::load: cannot open the file");
    std::vector<double> out;
    std::string s, param;
    while (std::getline(input, s)) {
        s.erase(std::remove_if(s.begin(), s.end(), [](unsigned char c) { return std::isspace(c) != 0; }), s.end());
        if (s.empty() || s[0] == '#') continue;
        std::istringstream iss(s);
        std::getline(iss, param, ',');
        double rec[kWaveDoubles] = {0., 0., 0., 0., 0., 0., 0.};
        if (param == "Plane") rec[0] = WAVE_PLANE;
        else if (param == "CircularJ") rec[0] = WAVE_CIRCULAR_J;
        else if (param == "CircularY") rec[0] = WAVE_CIRCULAR_Y;
        else if (param == "FourierHankel1") rec[0] = WAVE_FOURIER_HANKEL1;
        else if (param == "FourierHankel2") rec[0] = WAVE_FOURIER_HANKEL2;
        else if (param == "Herglotz") rec[0] = WAVE_HERGLOTZ;
        else return set_error(HBEM_ERR_INVALID, "incoming::load: unknown wave type");
        bool ok = field_double(iss, rec[1]) && field_double(iss, rec[2]) && field_double(iss, rec[3]);
        const int type = (int)rec[0];
        if (ok && (type == WAVE_PLANE || type == WAVE_HERGLOTZ)) {
            ok = field_double(iss, rec[4]);
            if (ok && type == WAVE_HERGLOTZ) ok = field_double(iss, rec[5]);
        } else if (ok) {
            int order = 0;
            ok = field_int(iss, order);
            rec[6] = order;
        }
        std::string extra;
        if (ok && std::getline(iss, extra, ',')) ok = false;
        if (!ok) return set_error(HBEM_ERR_INVALID, "incoming::load: malformed wave record");
        out.insert(out.end(), rec, rec + kWaveDoubles);
    }
    *nwaves = (int)(out.size() / kWaveDoubles);
    if (!waves) return HBEM_OK;
    if (*nwaves > cap) return set_error(HBEM_ERR_INVALID, "incoming::load: more records than cap");
    std::copy(out.begin(), out.end(), waves);
    return HBEM_OK;
}

int hbem_incoming_eval(const double* waves, int nwaves, double k_re, double k_im, const double* xy_host, int npts,
                       double* u_host, double* du_host) {
    if (npts < 0 || (npts > 0 && (!xy_host || !u_host))) return set_error(HBEM_ERR_INVALID, "incoming eval: bad argument");
    if (int r = check_waves(waves, nwaves, k_im)) return r;
    if (npts == 0) return HBEM_OK;
    FieldState& F = state();
    if (int r = upload_waves(F, waves, nwaves)) return r;
    Buf xy, u, du;
    FD_CK(put(xy, xy_host, 2 * (size_t)npts));
    FD_CK(u.ensure(npts * sizeof(cplx)));
    if (du_host) FD_CK(du.ensure(2 * npts * sizeof(cplx)));
    k_wave_points<<<(npts + 127) / 128, 128>>>(F.waves.as<double>(), nwaves, F.g21.as<double>(), k_re, k_im,
                                               xy.as<double>(), npts, u.as<cplx>(), du_host ? du.as<cplx>() : nullptr);
    count_launches(1);
    FD_CK(cudaGetLastError());
    FD_CK(cudaMemcpy(u_host, u.p, npts * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (du_host) FD_CK(cudaMemcpy(du_host, du.p, 2 * npts * sizeof(cplx), cudaMemcpyDeviceToHost));
    cudaFree(xy.p);
    cudaFree(u.p);
    if (du.p) cudaFree(du.p);
    return HBEM_OK;
}

int hbem_tp_solve(hbem_solop s, const double* waves, int nwaves, double k_re, double k_im, double c_o, double c_i,
                  double* traces_host) {
    if (!s || !traces_host) return set_error(HBEM_ERR_INVALID, "tp solve: bad argument");
    int N = 0;
    if (int r = tp_solve_device(s, waves, nwaves, k_re, k_im, c_o, c_i, N)) return r;
    FD_CK(cudaMemcpy(traces_host, state().rhs.p, 2 * (size_t)N * sizeof(cplx), cudaMemcpyDeviceToHost));
    return HBEM_OK;
}

int hbem_tp_field_grid(hbem_solop s, const double* waves, int nwaves, double k_re, double k_im, double c_o,
                       double c_i, unsigned order_green, double ll_x, double ll_y, double ur_x, double ur_y, int nx,
                       int ny, int total_field, const double* traces_host, double* field_host, double* grid_x_host,
                       double* grid_y_host) {
    if (!s || !field_host || order_green < 1 || order_green > 64 || nx < 2 || ny < 2 ||
        (long long)nx * ny > (1LL << 28))
        return set_error(HBEM_ERR_INVALID, "tp field: bad argument");
    if (!(c_o >= 1.) || !(c_i >= 1.)) return set_error(HBEM_ERR_INVALID, "Refraction index must not be smaller than 1");
    if (int r = check_waves(waves, nwaves, k_im)) return r;
    FieldState& F = state();
    int N = 0;
    const int* kinds;
    const double* par;
    int proj, device;
    if (int r = solop_mesh(s, &N, &kinds, &par, &proj, &device)) return r;
    FD_CK(cudaSetDevice(device));
    std::vector<cplx> tr(2 * (size_t)N);
    if (traces_host) {
        std::copy(traces_host, traces_host + 4 * (size_t)N, reinterpret_cast<double*>(tr.data()));
    } else {
        int n2 = 0;
        if (int r = tp_solve_device(s, waves, nwaves, k_re, k_im, c_o, c_i, n2)) return r;
        FD_CK(cudaMemcpy(tr.data(), F.rhs.p, 2 * (size_t)N * sizeof(cplx), cudaMemcpyDeviceToHost));
    }
    for (const cplx& v : tr)
        if (!std::isfinite(v.re) || !std::isfinite(v.im))
            return set_error(HBEM_ERR_NONFINITE, "Traces are undefined, aborting solution lifting");
    // panel lengths (ParametrizedLine / ParametrizedCircularArc::length) and their running sums
    std::vector<double> plen(N), csum(N), knots(N + 1);
    double acc = 0.;
    for (int i = 0; i < N; ++i) {
        const double* P = par + 5 * i;
        if (kinds[i] == HBEM_PANEL_LINE) {
            const double ax = (-1. * (P[2] - P[0]) + (P[2] + P[0])) * 0.5, ay = (-1. * (P[3] - P[1]) + (P[3] + P[1])) * 0.5;
            const double bx = (1. * (P[2] - P[0]) + (P[2] + P[0])) * 0.5, by = (1. * (P[3] - P[1]) + (P[3] + P[1])) * 0.5;
            plen[i] = std::sqrt((bx - ax) * (bx - ax) + (by - ay) * (by - ay));
        } else {
            plen[i] = P[2] * (P[4] - P[3]);
        }
        csum[i] = acc;
        knots[i] = acc;
        acc += plen[i];
    }
    knots[N] = acc;
    // trace splines over arc length (ComplexSpline(mesh, traces), cspline.cpp:30-53)
    std::vector<cplx> spl(8 * (size_t)N);
    for (int half = 0; half < 2; ++half) {
        for (int part = 0; part < 2; ++part) {
            std::vector<double> yv(N + 1), bb, cc, dd;
            for (int i = 0; i < N; ++i) yv[i] = part ? tr[half * N + i].im : tr[half * N + i].re;
            yv[N] = yv[0];
            akima_periodic(knots, yv, bb, cc, dd);
            for (int i = 0; i < N; ++i) {
                double* c = reinterpret_cast<double*>(&spl[8 * (size_t)i + 4 * half]);
                c[0 + part] = yv[i];
                c[2 + part] = bb[i];
                c[4 + part] = cc[i];
                c[6 + part] = dd[i];
            }
        }
    }
    std::vector<double> xg(order_green), wg(order_green), xq(kNearOrder), wq(kNearOrder);
    gauss_rule(0., 1., (int)order_green, xg.data(), wg.data());
    gauss_rule(0., 1., kNearOrder, xq.data(), wq.data());
    if (int r = upload_waves(F, waves, nwaves)) return r;
    FD_CK(put(F.kind, kinds, (size_t)N));
    FD_CK(put(F.par, par, (size_t)N * 5));
    FD_CK(put(F.csum, csum.data(), csum.size()));
    FD_CK(put(F.plen, plen.data(), plen.size()));
    FD_CK(put(F.knots, knots.data(), knots.size()));
    FD_CK(put(F.spl, spl.data(), spl.size()));
    FD_CK(put(F.xg, xg.data(), xg.size()));
    FD_CK(put(F.wg, wg.data(), wg.size()));
    FD_CK(put(F.xq, xq.data(), xq.size()));
    FD_CK(put(F.wq, wq.data(), wq.size()));
    const long long G = (long long)nx * ny;
    const int M = N * (int)order_green;
    FD_CK(F.nodes.ensure((size_t)M * sizeof(FNode)));
    FD_CK(F.acc.ensure(G * sizeof(cplx)));
    FD_CK(F.flag.ensure(G * sizeof(int)));
    FD_CK(F.bndt.ensure(G * sizeof(double)));
    FD_CK(F.nearcnt.ensure(sizeof(int)));
    FD_CK(F.S.ensure(G * sizeof(cplx)));

    FieldJob J{};
    J.npan = N;
    J.nq = (int)order_green;
    J.nx = nx;
    J.ny = ny;
    const cplx ki = mk(k_re * std::sqrt(c_i), k_im * std::sqrt(c_i)), ko = mk(k_re * std::sqrt(c_o), k_im * std::sqrt(c_o));
    J.real_k = (k_im == 0. && k_re > 0.) ? 1 : 0;
    J.nw = nwaves;
    J.total = total_field ? 1 : 0;
    J.llx = ll_x;
    J.lly = ll_y;
    J.hx = (ur_x - ll_x) / (nx - 1.);
    J.hy = (ur_y - ll_y) / (ny - 1.);
    J.kire = ki.re;
    J.kiim = ki.im;
    J.kore = ko.re;
    J.koim = ko.im;
    J.abs_ki = std::hypot(ki.re, ki.im);
    J.abs_ko = std::hypot(ko.re, ko.im);
    J.kre = k_re;
    J.kim = k_im;
    J.kind = F.kind.as<int>();
    J.par = F.par.as<double>();
    J.csum = F.csum.as<double>();
    J.plen = F.plen.as<double>();
    J.knots = F.knots.as<double>();
    J.spl = F.spl.as<cplx>();
    J.waves = F.waves.as<double>();
    J.g21 = F.g21.as<double>();
    J.nodes = F.nodes.as<FNode>();
    J.acc = F.acc.as<cplx>();
    J.flag = F.flag.as<int>();
    J.bnd_t = F.bndt.as<double>();
    J.near_count = F.nearcnt.as<int>();

    k_field_nodes<<<(M + 127) / 128, 128>>>(J, F.xg.as<double>(), F.wg.as<double>(), F.nodes.as<FNode>());
    FD_CK(cudaGetLastError());
    int cap = (int)std::max<long long>(4096, G / 8);
    int nnear = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int pass = 0; pass < 2; ++pass) {
        FD_CK(F.near.ensure((size_t)cap * sizeof(NearEntry)));
        J.near = F.near.as<NearEntry>();
        J.near_cap = cap;
        FD_CK(cudaMemset(F.nearcnt.p, 0, sizeof(int)));
        cudaEventRecord(e0, 0);
        k_field_grid<<<(unsigned)((G + 31) / 32), kFieldThreads>>>(J);
        cudaEventRecord(e1, 0);
        FD_CK(cudaGetLastError());
        FD_CK(cudaMemcpy(&nnear, F.nearcnt.p, sizeof(int), cudaMemcpyDeviceToHost));
        count_launches(1);
        if (nnear <= cap) break;
        cap = nnear;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // near pairs of points not on the boundary, in (point, panel) order
    std::vector<NearEntry> ent(nnear);
    std::vector<int> flag(G);
    if (nnear) FD_CK(cudaMemcpy(ent.data(), F.near.p, nnear * sizeof(NearEntry), cudaMemcpyDeviceToHost));
    FD_CK(cudaMemcpy(flag.data(), F.flag.p, G * sizeof(int), cudaMemcpyDeviceToHost));
    long long onb = 0;
    for (int v : flag) onb += (v & 2) ? 1 : 0;
    ent.erase(std::remove_if(ent.begin(), ent.end(), [&](const NearEntry& a) { return (flag[a.g] & 2) != 0; }),
              ent.end());
    std::sort(ent.begin(), ent.end(),
              [](const NearEntry& a, const NearEntry& b) { return a.g != b.g ? a.g < b.g : a.panel < b.panel; });
    const int ne = (int)ent.size();
    if (ne) {
        FD_CK(put(F.near, ent.data(), ent.size()));
        FD_CK(F.nearout.ensure(ne * sizeof(cplx)));
        k_field_near<<<(ne + 7) / 8, 256>>>(J, F.near.as<NearEntry>(), ne, F.xq.as<double>(), F.wq.as<double>(),
                                            F.nearout.as<cplx>());
        FD_CK(cudaGetLastError());
        std::vector<cplx> ex(ne);
        FD_CK(cudaMemcpy(ex.data(), F.nearout.p, ne * sizeof(cplx), cudaMemcpyDeviceToHost));
        std::vector<int> ai;
        std::vector<cplx> av;
        for (int e = 0; e < ne; ++e) {
            if (ai.empty() || ai.back() != ent[e].g) {
                ai.push_back(ent[e].g);
                av.push_back(mk(0.));
            }
            av.back() += ex[e];
        }
        FD_CK(put(F.addidx, ai.data(), ai.size()));
        FD_CK(put(F.addval, av.data(), av.size()));
        k_field_add<<<(unsigned)((ai.size() + 127) / 128), 128>>>(F.addidx.as<int>(), F.addval.as<cplx>(),
                                                                 (int)ai.size(), F.acc.as<cplx>());
        FD_CK(cudaGetLastError());
        count_launches(2);
    }
    k_field_finalize<<<(unsigned)((G + 127) / 128), 128>>>(J, F.S.as<cplx>());
    FD_CK(cudaGetLastError());
    count_launches(2);
    FD_CK(cudaMemcpy(field_host, F.S.p, G * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (grid_x_host && grid_y_host)
        for (long long g = 0; g < G; ++g) {
            grid_x_host[g] = ll_x + (g % nx) * J.hx;
            grid_y_host[g] = ll_y + (g / nx) * J.hy;
        }
    F.last_grid_ms = ms;
    F.last_units = (G - onb) * (long long)M;
    F.last_near = ne;
    return HBEM_OK;
}

void hbem_field_stats(double* grid_kernel_ms, long long* point_node_pairs, long long* near_pairs) {
    const FieldState& F = state();
    if (grid_kernel_ms) *grid_kernel_ms = F.last_grid_ms;
    if (point_node_pairs) *point_node_pairs = F.last_units;
    if (near_pairs) *near_pairs = F.last_near;
}

}  // extern "C"
