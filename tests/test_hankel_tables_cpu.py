"""The device Hankel tables (csrc/hankel_tables.h): regenerated bit for bit by their
generator, and the Taylor band (2 <= x < 8) and the far-field amplitudes (x >= 16)
evaluated here the way the device evaluates them, against mpmath."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

CSRC = os.path.join(os.path.dirname(__file__), "..", "helmholtzbem_gb300", "csrc")
HEADER = os.path.join(CSRC, "hankel_tables.h")


def _array(text, name):
    m = re.search(r"%s\[[^=]*=\s*\{(.*?)\};" % re.escape(name), text, re.S)
    assert m, name
    return np.array([float(v) for v in re.findall(r"[-+]?\d\.\d+e[-+]\d+", m.group(1))])


def test_generator_reproduces_the_header():
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_hankel_tables.py")], capture_output=True, text=True,
                         check=True).stdout
    assert out == open(HEADER).read()


def test_taylor_band_against_mpmath():
    txt = open(HEADER).read()
    T = _array(txt, "HBEM_TAY").reshape(12, 18, 4)
    rng = np.random.default_rng(3)
    worst = 0.0
    for x in np.concatenate([rng.uniform(2.0, 8.0, 200), [2.0, 4.75, 7.999999]]):
        i = min(11, int((x - 2.0) * 2.0))
        h = x - (2.25 + 0.5 * i)
        a = T[i, 17].copy()
        for m in range(16, -1, -1):
            a = a * h + T[i, m]
        ref = [float(mp.besselj(0, x)), float(mp.bessely(0, x)), float(mp.besselj(1, x)), float(mp.bessely(1, x))]
        h0, h1 = abs(complex(ref[0], ref[1])), abs(complex(ref[2], ref[3]))
        worst = max(worst, abs(a[0] - ref[0]) / h0, abs(a[1] - ref[1]) / h0, abs(a[2] - ref[2]) / h1,
                    abs(a[3] - ref[3]) / h1)
    assert worst < 1e-15


def test_far_field_amplitudes_against_mpmath():
    txt = open(HEADER).read()
    F0, G0, F1, G1 = (_array(txt, n) for n in ("HBEM_F0F", "HBEM_G0F", "HBEM_F1F", "HBEM_G1F"))
    mp.mp.dps = 30
    for x in (16.0, 17.3, 25.0, 60.0, 400.0):
        w = 64.0 / (x * x)
        P0 = 1.0 + np.polyval(F0[::-1], w)
        Q0 = (np.polyval(G0[::-1], w) - 0.125) / x
        P1 = 1.0 + np.polyval(F1[::-1], w)
        Q1 = (np.polyval(G1[::-1], w) + 0.375) / x
        s, c = np.sin(x), np.cos(x)
        r = 1.0 / np.sqrt(np.pi * x)
        cc, ss = (s + c) * r, (s - c) * r
        j0, y0 = P0 * cc - Q0 * ss, P0 * ss + Q0 * cc
        j1, y1 = P1 * ss + Q1 * cc, Q1 * ss - P1 * cc
        ref = [float(mp.besselj(0, x)), float(mp.bessely(0, x)), float(mp.besselj(1, x)), float(mp.bessely(1, x))]
        scale = np.sqrt(2.0 / (np.pi * x))
        for a, b in zip((j0, y0, j1, y1), ref):
            assert abs(a - b) <= 2e-15 * scale
