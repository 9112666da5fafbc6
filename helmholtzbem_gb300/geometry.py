"""Panel meshes in the layout of the C ABI (kinds[n], params[n][5]).

Restates the reference's mesh constructors:
* ``ParametrizedCircularArc(center, r, phi0, phi1).split(N)``
  (source/parametrizations/parametrized_circular_arc.cpp:141-152)
* ``ParametrizedLine(p, q).split(m)`` (source/parametrizations/parametrized_line.cpp:112-131)
* ``scatterer::read``, ``length``, ``auto_num_panels``, ``make_N_polygonal_panels``,
  ``make_polygonal_panels`` (source/utilities/scatterer.cpp:30-277) and the panel
  count of examples/find_resonances.cpp:111-124, through the host code of libhbem
plus the synthetic scatterers of the benchmark configurations (seeded star
polygons; Fourier-sum curves sampled into line panels).
"""
import ctypes
import math
import os

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


def _poly_arrays(x, y):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    if x.shape != y.shape or x.ndim != 1:
        raise ValueError("x and y must be 1-D arrays of equal length")
    return x, y


def _panels_from(fn, x, y, *args):
    from . import _capi as C
    x, y = _poly_arrays(x, y)
    n = ctypes.c_int()
    C.check(fn(C.dptr(x), C.dptr(y), int(x.size), *args, None, 0, ctypes.byref(n)))
    par = np.zeros((n.value, 5))
    C.check(fn(C.dptr(x), C.dptr(y), int(x.size), *args, C.dptr(par), n.value, ctypes.byref(n)))
    return np.full(n.value, PANEL_LINE, np.int32), par


def polygon(x, y, N):
    """scatterer::make_N_polygonal_panels: exactly N line panels, edge counts
    proportional to the edge lengths and corrected one panel at a time on the edge
    that minimises the variance of the panel lengths (host code of libhbem)."""
    from . import _capi as C
    return _panels_from(C.lib().hbem_polygon_panels, x, y, ctypes.c_uint(int(N)))


def polygon_graded(x, y, N, refinement_factor=0.5):
    """scatterer::make_polygonal_panels: about N line panels graded geometrically
    towards the corners (host code of libhbem)."""
    from . import _capi as C
    return _panels_from(C.lib().hbem_polygon_panels_graded, x, y, ctypes.c_uint(int(N)),
                        ctypes.c_double(float(refinement_factor)))


def read_scatterer(fname, scale=1.0):
    """scatterer::read: vertices (x, y) of a polygon file with one "x,y" per line;
    raises ValueError where the reference returns false."""
    from . import _capi as C
    n = ctypes.c_int()
    if C.lib().hbem_scatterer_read(os.fsencode(fname), float(scale), None, None, 0, ctypes.byref(n)) != 0:
        raise ValueError("failed to read scatterer from file " + str(fname))
    x = np.zeros(n.value)
    y = np.zeros(n.value)
    C.check(C.lib().hbem_scatterer_read(os.fsencode(fname), float(scale), C.dptr(x), C.dptr(y), n.value,
                                        ctypes.byref(n)))
    return x, y


def polygon_length(x, y):
    """scatterer::length: perimeter of the closed polygon."""
    from . import _capi as C
    x, y = _poly_arrays(x, y)
    return float(C.lib().hbem_polygon_length(C.dptr(x), C.dptr(y), int(x.size)))


def auto_num_panels(x, y, f):
    """scatterer::auto_num_panels: round(perimeter / (f * shortest side))."""
    from . import _capi as C
    x, y = _poly_arrays(x, y)
    return int(C.lib().hbem_auto_num_panels(C.dptr(x), C.dptr(y), int(x.size), float(f)))


def choose_num_panels(x, y, k_max, degf=10.0, rfac=0.5):
    """The panel count of examples/find_resonances.cpp:111-124 (Brent's minimiser
    matching the longest graded panel to 2 pi / (degf k_max))."""
    from . import _capi as C
    x, y = _poly_arrays(x, y)
    out = ctypes.c_uint()
    C.check(C.lib().hbem_choose_num_panels(C.dptr(x), C.dptr(y), int(x.size), float(k_max), float(degf),
                                           float(rfac), ctypes.byref(out)))
    return int(out.value)


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
