"""The oracle's Hankel functions against the reference's own known answers
(test/googletest/solutions_test.cpp:55-72) and mpmath golden vectors."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "hankel_mpmath.json")))
EPS = np.finfo(float).eps


def test_reference_kats():
    kat = GOLD["reference_kats"]
    h0, h1 = O.hankel01(np.array([np.pi, 0.1]))
    # J0(pi) and J0'(pi) = -J1(pi) at tolerance eps (solutions_test.cpp:55-65)
    assert abs(h0[0].real - kat["J0(pi)"]) <= EPS
    assert abs(-h1[0].real - kat["J0'(pi)"]) <= EPS
    # H0'(0.1) = -H1(0.1) at tolerance 100 sqrt(eps) (solutions_test.cpp:69-72)
    dh = -h1[1]
    assert abs(dh.real - kat["H0'(0.1)"][0]) <= kat["H0'(0.1)_tol"]
    assert abs(dh.imag - kat["H0'(0.1)"][1]) <= kat["H0'(0.1)_tol"]


def test_zero_argument():
    h0, h1 = O.hankel01(np.array([0.0]))
    assert h0[0] == 1.0 and h1[0] == 0.0


def test_real_against_mpmath():
    xs = np.array([r["x"] for r in GOLD["real"]])
    r0 = np.array([complex(*r["h0"]) for r in GOLD["real"]])
    r1 = np.array([complex(*r["h1"]) for r in GOLD["real"]])
    h0, h1 = O.hankel01(xs)
    e0 = np.abs(h0 - r0) / np.abs(r0)
    e1 = np.abs(h1 - r1) / np.abs(r1)
    big = xs > 1e6      # leading-order asymptotics, as in the reference (error ~ 1/(8x))
    small_series = (xs > 4.0) & (xs < 8.0)   # ascending series near its switch point loses ~3 digits
    ok = ~big & ~small_series
    assert e0[ok].max() < 2e-15 and e1[ok].max() < 2e-15
    assert e0[small_series].max() < 3e-13 and e1[small_series].max() < 3e-13
    assert e0[big].max() < 5e-7 and e1[big].max() < 5e-7


def test_complex_against_mpmath():
    z = np.array([complex(*r["z"]) for r in GOLD["complex"]])
    r0 = np.array([complex(*r["h0"]) for r in GOLD["complex"]])
    r1 = np.array([complex(*r["h1"]) for r in GOLD["complex"]])
    h0, h1 = O.hankel01(z)
    e0 = np.abs(h0 - r0) / np.abs(r0)
    e1 = np.abs(h1 - r1) / np.abs(r1)
    # accuracy envelope of the Miller/Neumann region grows like eps*exp(2 Im z)
    tol = 4e-15 * np.exp(2.0 * z.imag)
    assert np.all(e0 < tol) and np.all(e1 < tol)
