"""CPU-side checks of the C ABI library: it loads, exports exactly what
include/hbem.h declares, and its host-only root finders agree with the oracle's
restatement (no GPU call is made here)."""
import math
import os
import re

import numpy as np
import pytest

from helmholtzbem_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib_or_skip():
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("libhbem.so not built")
    return _capi.load()


def test_header_matches_exports():
    src = open(os.path.join(ROOT, "include", "hbem.h")).read()
    declared = set(re.findall(r"^\s*(?:const char\*|double|int|unsigned|void)\s+(hbem_\w+)\s*\(", src, re.M))
    assert declared == set(_capi.EXPORTS)


def test_library_exports_every_symbol():
    L = _lib_or_skip()
    for name in _capi.EXPORTS:
        assert hasattr(L, name), name
    assert L.hbem_version() >= 100
    assert L.hbem_status_string(1).decode() == "invalid argument"


def _api():
    _lib_or_skip()
    from helmholtzbem_gb300 import api
    return api


def test_rtsafe_matches_oracle():
    """d/dx of min(cos x, sin x)-like smooth function: the Newton iterates of the
    library and the oracle restatement coincide."""
    api = _api()
    from oracle import oracle as O
    f = lambda x: math.sin(x) - 0.3 * x
    fb = lambda x: (math.sin(x) - 0.3 * x, math.cos(x) - 0.3)
    r1, ok1, n1 = api.rtsafe(f, fb, 1.0, 3.5, 1e-12)
    r2, ok2, n2 = O.rtsafe(f, fb, 1.0, 3.5, 1e-12)
    assert ok1 and ok2 and n1 == n2 and r1 == r2
    assert abs(math.sin(r1) - 0.3 * r1) < 1e-12


def test_rtsafe_not_bracketed():
    api = _api()
    # f(x1) = 2 and f(x2) = 5 do not bracket a root: the end with the larger value returns
    r, ok, _ = api.rtsafe(lambda x: x * x + 1, lambda x: (x * x + 1, 2 * x), -1.0, 2.0, 1e-10)
    assert (not ok) and r == 2.0


def test_zbrent_and_brent_min():
    api = _api()
    r, ok, _ = api.zbrent(lambda x: math.cos(x) - x, 0.0, 1.0, 1e-14)
    assert ok and abs(math.cos(r) - r) < 1e-13
    r, ok, _ = api.zbrent(lambda x: x * x + 1, 0.0, 1.0, 1e-14)
    assert not ok
    from oracle import oracle as O
    g = lambda x: (x - 0.7) ** 2 * (x + 2.0) + 0.1 * math.sin(5 * x)
    m1 = api.brent_min(g, 0.0, 2.0, 1e-10)
    m2 = O.BrentMin(0.0, 2.0, 1e-10).minimize(g)
    assert m1 == m2


def test_reference_root_test_functions():
    """The reference's find_roots_test.cpp functions (min(cos x, sin x) family, tol 1e-5):
    zeros of the derivative found by rtsafe inside each bracket."""
    api = _api()
    for fn, a, b, root in [(math.cos, 1.0, 2.0, math.pi / 2), (math.sin, 3.0, 4.5, math.pi)]:
        r, ok, _ = api.zbrent(fn, a, b, 1e-10)
        assert ok and abs(r - root) < 1e-5
        r, ok, _ = api.rtsafe(fn, lambda x, g=fn: (g(x), (-math.sin(x) if g is math.cos else math.cos(x))),
                              a, b, 1e-10)
        assert ok and abs(r - root) < 1e-5


def test_rand_sketch_distribution():
    """randGaussian stand-in: (U[0,1] + i U[0,1])/sqrt2 entries, reproducible by seed."""
    api = _api()
    R = api.randGaussian(400, 50, seed=11)
    assert R.shape == (400, 50)
    s = np.sqrt(0.5)
    assert R.real.min() >= 0 and R.real.max() <= s and R.imag.min() >= 0 and R.imag.max() <= s
    assert abs(R.real.mean() - 0.5 * s) < 0.02 and abs(R.imag.mean() - 0.5 * s) < 0.02
    assert np.array_equal(R, api.randGaussian(400, 50, seed=11))


def test_brent_reverse_communication_matches_callback_and_oracle():
    """BrentMinimizer::local_min_rc driven by hand gives the iterates of the callback
    form and of the oracle's restatement (the panel-count loop of find_resonances)."""
    api = _api()
    from oracle import oracle as O
    f = lambda x: (x - 1.3) ** 2 * (1 + 0.3 * math.sin(5 * x)) + 0.1 * x
    br = api.BrentMinimizer(0.2, 3.0, 1e-3)
    arg, st = br.local_min_rc(0)
    n = 0
    while st:
        arg, st = br.local_min_rc(st, f(arg))
        n += 1
    assert n > 3
    assert arg == api.brent_min(f, 0.2, 3.0, 1e-3) == O.BrentMin(0.2, 3.0, 1e-3).minimize(f)


def test_brent_guess_and_gsl_with_values_match_oracle():
    api = _api()
    from oracle import oracle as O
    f = lambda x: math.cos(3 * x) + 0.1 * x * x
    g, _ = api.brent_guess(0.5, 1.6, 1.0, f(1.0), f, 1e-10)
    assert g == O.brent_guess(0.5, 1.6, 1.0, f(1.0), f, 1e-10)
    h, it = api.brent_gsl_with_values(0.5, f(0.5), 1.6, f(1.6), 1.0, f(1.0), f, 1e-9)
    assert h == O.brent_search(0.5, f(0.5), 1.6, f(1.6), 1.0, f(1.0), f, 1e-9) and it > 0
    # a bracket the GSL minimiser refuses: NaN
    r, _ = api.brent_gsl_with_values(0.5, f(0.5), 1.6, f(1.6), 0.6, f(0.6) + 10, f, 1e-9)
    assert math.isnan(r)


def test_every_documented_option_is_accepted():
    """The switches hbem.h documents for hbem_set_option: each accepts its default
    (no GPU involved), an unknown name is refused with a message."""
    L = _lib_or_skip()
    src = open(os.path.join(ROOT, "include", "hbem.h")).read()
    block = src[src.index("Process-wide switches"):src.index("int hbem_set_option")]
    documented = re.findall(r'"(\w+)" \(default (\d+)', block)
    assert {"svd_fast", "singular_table", "plain_speculate", "plain_warm_start", "svd_pair_max",
            "singular_split", "plain_async"} <= {n for n, _ in documented}
    import ctypes
    v = ctypes.c_int(-1)
    for name, default in documented:
        assert L.hbem_set_option(name.encode(), int(default)) == 0, name
        assert L.hbem_get_option(name.encode(), ctypes.byref(v)) == 0 and v.value == int(default), name
    assert L.hbem_set_option(b"no_such_switch", 1) == 1
    assert L.hbem_get_option(b"no_such_switch", ctypes.byref(v)) == 1
    assert b"unknown option" in L.hbem_last_error()
