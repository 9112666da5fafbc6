"""Second, independent CPU restatement of the Galerkin operators: the reference's
per-operator assembly files.

TEST INFRASTRUCTURE ONLY (like oracle.py): it cross-checks the oracle's
restatement of GalerkinBuilder (hbem_oracle.cpp) so that matrix parity does not
rest on one reading of the reference.  Nothing in the product imports it.

The reference keeps, besides GalerkinBuilder, an older point-by-point assembly per
operator and derivative order:

* source/single_layer.cpp:9-240, single_layer_der.cpp, single_layer_der2.cpp
* source/double_layer.cpp:9-284, double_layer_der.cpp, double_layer_der2.cpp
* source/hypersingular.cpp:9-299, hypersingular_der.cpp, hypersingular_der2.cpp

Each evaluates, for every ordered panel pair (i, j), the double integral of a
kernel times shape functions with one of three tensor rules -- coincident
(s = x_l (1 - x_k), t = x_l, w = x_l w_k w_l, both (s, t) and (t, s)), adjacent
(s = x_k x_l, t = x_k, w = x_k w_k w_l, both orders, each panel parametrised from
the shared vertex) and general (Gauss x Gauss) -- and scatters the Q x Q block by
the spaces' LocGlobMap.  The kernel is evaluated at every point with the complex
Hankel function (HankelH1 / HankelH1p), with the log fallbacks for arguments below
machine epsilon.  Here every point is written in each panel's own parameter sigma
in [0, 1] (the swapped maps of the reference are gamma(1 - t)); kernels:

  single layer   d0  i/4 H0(x)               [x <= eps: -log(r) / (2 pi)]
                 d1  -i sqrt(c)/4 H1(x) r
                 d2  i c/4 H0''(x) r^2
  double layer   d0  i ks/4 H1(x) (v/r . n_j) [x <= eps: (v . n_j) / (2 pi r^2)]
                 d1  i sqrt(c)/4 (x H1'(x) + H1(x)) (v/r . n_j)
                 d2  i c/4 (x H1''(x) + 2 H1'(x)) (v . n_j)
  hypersingular  A = b_i' b_j' - ks^2 b_i b_j |g_i'| |g_j'| (n_i . n_j)
                 d0  i/4 H0(x) A              [x <= eps: -log(r) / (2 pi) A]
                 d1  -i sqrt(c)/4 (H1(x) r A + 2 ks H0(x) B)
                 d2  -i c/4 (H1'(x) r^2 A - 4 ks H1(x) r B + 2 H0(x) B)

with v = g_i(s) - g_j(t), r = |v|, ks = k sqrt(c), x = ks r, B = b_i b_j |g_i'|
|g_j'| (n_i . n_j), the single and double layer's shape products b_i b_j |g_i'|
|g_j'|, and n = (t_y, -t_x) / |t| from each panel's own tangent.  Quadrature nodes
come from numpy's Gauss-Legendre rule (not from the oracle's C++ gauleg), mapped
into the reference's reduced composite rule (include/gauleg.hpp:89-121).  The
Hankel functions are scipy's (AMOS zbesh), not the oracle's.

``galerkin_matrix`` returns one layer and derivative order for P1 or P0 spaces:
the single layer on the test space, the hypersingular on the trial space, the
double layer test x trial -- the spaces GalerkinBuilder gives each layer.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.special as sp

EPS = np.finfo(float).eps
LINE, ARC = 0, 1
SINGLE, DOUBLE, HYPERSINGULAR = "V", "K", "W"


def gauss01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def cgauss01(n):
    """Reduced composite rule of order n: n(n+1)/2 - 1 nodes on [sigma^(n-1), 1] in
    geometrically graded intervals [sigma^(l+1), sigma^l] with n - l nodes,
    sigma = (sqrt2 - 1)^2."""
    sig = (math.sqrt(2.0) - 1.0) ** 2
    xl, xr = sig, 1.0
    xs, ws = [], []
    for q in range(n, 1, -1):
        x, w = gauss01(q)
        xs.append((xr - xl) * x + xl)
        ws.append((xr - xl) * w)
        xr, xl = xl, xl * sig
    return np.concatenate(xs[::-1]), np.concatenate(ws[::-1])


def panel_eval(kind, P, sig):
    """Point and tangent d/dsigma (complex x + iy) of a panel at sigma in [0, 1]:
    line a + sigma (b - a); arc c + r exp(i (phi0 + sigma (phi1 - phi0)))."""
    sig = np.asarray(sig, float)
    if kind == LINE:
        a, b = complex(P[0], P[1]), complex(P[2], P[3])
        return a + sig * (b - a), np.full(sig.shape, b - a, complex)
    c, r, p0, p1 = complex(P[0], P[1]), P[2], P[3], P[4]
    e = np.exp(1j * (p0 + sig * (p1 - p0)))
    return c + r * e, 1j * r * (p1 - p0) * e


def _dot(a, b):
    return (a * np.conj(b)).real


def _nodes(kinds, params, order, i, j):
    """(sigma_i, sigma_j, w) of the rule the reference picks for the ordered pair."""
    if i == j:
        x, w = cgauss01(order)
        xk, xl = np.meshgrid(x, x, indexing="ij")
        wk, wl = np.meshgrid(w, w, indexing="ij")
        s, t, ww = (xl * (1.0 - xk)).ravel(), xl.ravel(), (xl * wk * wl).ravel()
        return np.concatenate([s, t]), np.concatenate([t, s]), np.concatenate([ww, ww])
    gi_end = panel_eval(kinds[i], params[i], 1.0)[0]
    gi_start = panel_eval(kinds[i], params[i], 0.0)[0]
    gj_start = panel_eval(kinds[j], params[j], 0.0)[0]
    gj_end = panel_eval(kinds[j], params[j], 1.0)[0]
    noswap = abs(gi_end - gj_start) / 100.0 < EPS
    swap = abs(gi_start - gj_end) / 100.0 < EPS
    if noswap or swap:
        x, w = cgauss01(order)
        xk, xl = np.meshgrid(x, x, indexing="ij")
        wk, wl = np.meshgrid(w, w, indexing="ij")
        s, t, ww = (xk * xl).ravel(), xk.ravel(), (xk * wk * wl).ravel()
        a, b = np.concatenate([s, t]), np.concatenate([t, s])
        if noswap:   # panel i from its end, panel j from its start
            return 1.0 - a, b, np.concatenate([ww, ww])
        return a, 1.0 - b, np.concatenate([ww, ww])
    x, w = gauss01(order)
    a, b = np.meshgrid(x, x, indexing="ij")
    wa, wb = np.meshgrid(w, w, indexing="ij")
    return a.ravel(), b.ravel(), (wa * wb).ravel()


def _shape(q):
    """Local functions (value, d/dsigma) of a space: P1 -> [sigma, 1 - sigma] with
    derivatives [1, -1] (continuous_space.hpp:38-47 and the _01 variants); P0 -> [1]."""
    if q == 1:
        return [(lambda s: np.ones_like(s), 0.0)]
    return [(lambda s: s, 1.0), (lambda s: 1.0 - s, -1.0)]


def _dof(q, a, i, n):
    """LocGlobMap, 0-based: P1 local 0 on panel i -> dof i + 1 (cyclic), local 1 -> i;
    P0 -> i."""
    if q == 1:
        return i
    return (i + 1) % n if a == 0 else i


def _kernel(layer, d, k, c, v, r, Ti, Tj):
    """Kernel pieces at the points of one pair: returns (coefficient of the shape
    product, coefficient of the shape-derivative product) with the scale factor of
    the operator and derivative order included."""
    sc = math.sqrt(c)
    ks = k * sc
    x = ks * r
    big = abs(ks) * r > EPS
    small = (~big) & (r > EPS)
    xs = np.where(big, x, 1.0)
    H0 = np.where(big, sp.hankel1(0, xs), 0.0)
    H1 = np.where(big, sp.hankel1(1, xs), 0.0)
    ni, nj = -1j * Ti / np.abs(Ti), -1j * Tj / np.abs(Tj)
    meas = np.abs(Ti) * np.abs(Tj)
    zero = np.zeros(r.shape, complex)
    rs = np.where(r > 0, r, 1.0)
    logf = np.where(small, -np.log(rs) / (2.0 * math.pi), 0.0)
    if layer == SINGLE:
        if d == 0:
            return (0.25j * H0 + logf) * meas, zero
        if d == 1:
            return -0.25j * sc * H1 * r * meas, zero
        H0pp = np.where(big, sp.h1vp(0, xs, 2), 0.0)
        return 0.25j * c * H0pp * r * r * meas, zero
    if layer == DOUBLE:
        vn = _dot(v, nj)
        if d == 0:
            val = np.where(big, 0.25j * ks * H1 * vn / rs, 0.0) + np.where(small, vn / (2 * math.pi * rs * rs), 0.0)
            return val * meas, zero
        H1p = np.where(big, sp.h1vp(1, xs, 1), 0.0)
        if d == 1:
            return 0.25j * sc * (x * H1p + H1) * vn / rs * meas, zero
        H1pp = np.where(big, sp.h1vp(1, xs, 2), 0.0)
        return 0.25j * c * (x * H1pp + 2.0 * H1p) * vn * meas, zero
    nn = _dot(ni, nj)
    B = meas * nn
    if d == 0:
        g = 0.25j * H0 + logf
        return -ks * ks * g * B, g
    if d == 1:
        return -0.25j * sc * (-H1 * r * ks * ks * B + 2.0 * ks * H0 * B), -0.25j * sc * H1 * r
    H1p = np.where(big, sp.h1vp(1, xs, 1), 0.0)
    return (-0.25j * c * (-H1p * r * r * ks * ks * B - 4.0 * ks * H1 * r * B + 2.0 * H0 * B),
            -0.25j * c * H1p * r * r)


def galerkin_matrix(kinds, params, order, k, c, layer, d=0, test=2, trial=2):
    """One layer matrix (V on test x test, K on test x trial, W on trial x trial) of
    derivative order d, assembled over every ordered panel pair as the per-operator
    files do."""
    kinds = np.asarray(kinds)
    params = np.asarray(params, float)
    n = kinds.size
    qr = {SINGLE: test, DOUBLE: test, HYPERSINGULAR: trial}[layer]
    qc = {SINGLE: test, DOUBLE: trial, HYPERSINGULAR: trial}[layer]
    shr, shc = _shape(qr), _shape(qc)
    out = np.zeros((n, n), complex)
    for i in range(n):
        for j in range(n):
            si, sj, w = _nodes(kinds, params, order, i, j)
            Pi, Ti = panel_eval(kinds[i], params[i], si)
            Pj, Tj = panel_eval(kinds[j], params[j], sj)
            v = Pi - Pj
            r = np.abs(v)
            kv, kd = _kernel(layer, d, complex(k) if np.iscomplexobj(k) else float(k), float(c), v, r, Ti, Tj)
            kv, kd = w * kv, w * kd
            for a, (fa, da) in enumerate(shr):
                ga = fa(si)
                for b, (fb, db) in enumerate(shc):
                    val = np.sum(kv * ga * fb(sj))
                    if layer == HYPERSINGULAR and da * db != 0.0:
                        val += da * db * np.sum(kd)
                    out[_dof(qr, a, i, n), _dof(qc, b, j, n)] += val
    return out
