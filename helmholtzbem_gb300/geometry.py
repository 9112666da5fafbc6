"""Panel meshes in the layout of the C ABI (kinds[n], params[n][5]).

Restates the reference's mesh constructors:
* ``ParametrizedCircularArc(center, r, phi0, phi1).split(N)``
  (source/parametrizations/parametrized_circular_arc.cpp:141-152)
* ``ParametrizedLine(p, q).split(m)`` (source/parametrizations/parametrized_line.cpp:112-131)
* ``scatterer::make_N_polygonal_panels(x, y, N)`` (source/utilities/scatterer.cpp:114-156)
plus the synthetic scatterers of the benchmark configurations (seeded star
polygons; Fourier-sum curves sampled into line panels).
"""
import math

import numpy as np

from ._capi import PANEL_ARC, PANEL_LINE


def circle(radius, n, center=(0.0, 0.0)):
    kinds = np.full(n, PANEL_ARC, np.int32)
    par = np.zeros((n, 5))
    phi_s, phi_e = 0.0, 2 * math.pi
    for i in range(n):
        a = phi_s + i * (phi_e - phi_s) / n
        b = phi_s + (i + 1) * (phi_e - phi_s) / n
        if i == n - 1:
            b = phi_e
        par[i] = (center[0], center[1], radius, a, b)
    return kinds, par


def split_line(p, q, m):
    x1, y1 = p
    x2, y2 = q
    out = []
    for i in range(m):
        t1 = -1.0 + i * 2.0 / m
        t2 = 1.0 if i == m - 1 else -1.0 + (i + 1) * 2.0 / m
        out.append(((t1 * (x2 - x1) + (x2 + x1)) * 0.5, (t1 * (y2 - y1) + (y2 + y1)) * 0.5,
                    (t2 * (x2 - x1) + (x2 + x1)) * 0.5, (t2 * (y2 - y1) + (y2 + y1)) * 0.5, 0.0))
    return out


def polygon(x, y, N):
    """Edge panel counts proportional to edge length, corrected one panel at a time
    on the edge that minimises the variance of the panel lengths."""
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    n = x.size
    d = np.array([math.hypot(x[(i + 1) % n] - x[i], y[(i + 1) % n] - y[i]) for i in range(n)])
    alpha = N / float(np.sum(d))
    m = np.array([float(np.round(alpha * di)) for di in d])
    cs = int(np.sum(m))
    while cs != N:
        step = -1 if cs > N else 1
        best, i_best = np.inf, 0
        for i in range(n):
            m[i] += step
            a = d / m
            var = float(np.mean((a - np.mean(a)) ** 2))
            if var < best:
                best, i_best = var, i
            m[i] -= step
        m[i_best] += step
        cs += step
    panels = []
    for i in range(n):
        panels += split_line((x[i], y[i]), (x[(i + 1) % n], y[(i + 1) % n]), int(m[i]))
    return np.full(len(panels), PANEL_LINE, np.int32), np.array(panels)


def star_polygon(nvert, seed, amp=0.3):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, nvert)
    th = 2 * np.pi * np.arange(nvert) / nvert
    r = 1.0 + amp * u
    return r * np.cos(th), r * np.sin(th)


def fourier_curve(a, b, N):
    th = 2 * np.pi * np.arange(N) / N
    m = np.arange(1, len(a) + 1)
    r = 1.0 + np.cos(np.outer(th, m)) @ np.asarray(a) + np.sin(np.outer(th, m)) @ np.asarray(b)
    xs, ys = r * np.cos(th), r * np.sin(th)
    panels = [(xs[i], ys[i], xs[(i + 1) % N], ys[(i + 1) % N], 0.0) for i in range(N)]
    return np.full(N, PANEL_LINE, np.int32), np.array(panels)


def random_fourier_coeffs(seed, modes=8, scale=0.05, rmin=0.3):
    """Seeded Fourier-sum radius r(t) = 1 + sum_m a_m cos mt + b_m sin mt with
    a_m, b_m ~ N(0, scale / m), redrawn until min r >= rmin."""
    rng = np.random.default_rng(seed)
    while True:
        sd = scale / np.arange(1, modes + 1)
        a = rng.normal(0.0, sd)
        b = rng.normal(0.0, sd)
        th = np.linspace(0, 2 * np.pi, 2048, endpoint=False)
        m = np.arange(1, modes + 1)
        r = 1 + np.cos(np.outer(th, m)) @ a + np.sin(np.outer(th, m)) @ b
        if r.min() >= rmin:
            return a, b
