"""Incoming waves, the transmission solve and the field lifting on the CPU
(source/utilities/incoming.cpp, solvers.cpp:116-391): the wave-file parser of
libhbem against the oracle's, and checks of the oracle restatement itself --
wave gradients by finite differences, the periodic Akima spline, and a scatterer
with no contrast (c_i = c_o), whose total field is the incoming wave."""
import math
import os

import numpy as np
import pytest

from helmholtzbem_gb300 import _capi
from oracle import oracle as O

if not os.path.exists(_capi.LIB_PATH):
    pytest.skip("libhbem.so not built", allow_module_level=True)

from helmholtzbem_gb300 import api, geometry  # noqa: E402


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_incoming_load_formats(tmp_path):
    f = _write(tmp_path, "w.dat", "# comment\nPlane, 1.0, 0, 0, 1.047\n\n CircularJ, 1.0, 0.0, 0.0, -1\n"
               "Herglotz, 1.0, -0.2, 0, 0.85, 0.1\nFourierHankel2,0.5,1,2,3\nCircularY, 2, 0, 0, 4\n")
    got = api.incoming_load(f)
    ref = O.incoming_load(f)
    assert got.shape == (5, 7) and np.array_equal(got, ref)
    assert list(got[:, 0]) == [0, 1, 5, 4, 2]
    assert got[1, 6] == -1 and got[2, 5] == 0.1 and got[3, 6] == 3


@pytest.mark.parametrize("text", ["Wave, 1, 0, 0, 1\n", "Plane, 1, 0, 0\n", "Plane, 1, 0, 0, 1, 2\n",
                                  "CircularJ, 1, 0, 0, x\n", "Herglotz, 1, 0, 0, 1\n", "Plane, a, 0, 0, 1\n"])
def test_incoming_load_rejects(tmp_path, text):
    f = _write(tmp_path, "bad.dat", text)
    with pytest.raises(ValueError):
        api.incoming_load(f)
    assert O.incoming_load(f) is None


WAVES = [api.wave("Plane", 1.0, (0.1, -0.2), angle=0.7),
         api.wave("CircularJ", 0.5, (0.05, 0.0), order=-2),
         api.wave("CircularY", 0.3, (1.5, 1.5), order=1),
         api.wave("FourierHankel1", 0.2, (-1.4, 0.3), order=3),
         api.wave("FourierHankel2", 0.2, (1.4, -0.3), order=0),
         api.wave("Herglotz", 1.0, (-0.2, 0.0), angle=0.85, eps=0.1)]


@pytest.mark.parametrize("w", range(len(WAVES)))
def test_oracle_wave_gradient_by_finite_differences(w):
    k = 3.3
    for (x, y) in [(0.3, 0.4), (-0.7, 0.2), (0.05, -0.9)]:
        u, ux, uy = O.wave_eval(WAVES[w], k, x, y)
        h = 1e-6
        fx = (O.wave_eval(WAVES[w], k, x + h, y)[0] - O.wave_eval(WAVES[w], k, x - h, y)[0]) / (2 * h)
        fy = (O.wave_eval(WAVES[w], k, x, y + h)[0] - O.wave_eval(WAVES[w], k, x, y - h)[0]) / (2 * h)
        scale = max(1.0, abs(ux), abs(uy))
        assert abs(fx - ux) < 1e-6 * scale and abs(fy - uy) < 1e-6 * scale


def test_akima_periodic_interpolates_and_is_smooth():
    t = np.cumsum(np.r_[0.0, np.random.default_rng(1).uniform(0.5, 1.5, 20)])
    y = list(np.sin(2 * np.pi * t / t[-1]))
    y[-1] = y[0]
    b, c, d = O.akima_periodic(list(t), y)
    for i in range(len(t) - 1):
        h = t[i + 1] - t[i]
        assert abs(y[i] + h * (b[i] + h * (c[i] + h * d[i])) - y[i + 1]) < 1e-12
        # C1: slope at the right end of interval i equals b[i+1] (periodic)
        right = b[i] + h * (2 * c[i] + 3 * h * d[i])
        assert abs(right - b[(i + 1) % (len(t) - 1)]) < 1e-12
    # smooth data: close to the function between knots
    s = 0.37 * t[5] + 0.63 * t[6]
    i = 5
    h = s - t[i]
    assert abs(y[i] + h * (b[i] + h * (c[i] + h * d[i])) - math.sin(2 * math.pi * s / t[-1])) < 1e-2


def test_oracle_no_contrast_reproduces_the_incoming_wave():
    """c_i = c_o = 1: the scatterer is transparent; the field equals u_inc inside and
    the total field equals it outside (up to the P1 discretisation error)."""
    kinds, par = geometry.circle(0.5, 40)
    w = api.wave("Plane", 1.0, angle=0.4)
    k = 2.0
    tr = O.tp_solve(kinds, par, 9, w, k, 1.0, 1.0)
    pts = [(0.1, 0.2), (-0.2, -0.1), (0.9, 0.3), (-1.0, 0.6)]
    S = O.field_points(kinds, par, tr, w, k, 1.0, 1.0, 12, pts, total_field=True)
    for (x, y), s in zip(pts, S):
        assert abs(s - O.wave_eval(w, k, x, y)[0]) < 5e-3
