"""The adaptive sampler (opt_subdiv) of the C ABI -- host code, no GPU -- against the
oracle's restatement on the same seeded generator, and the pieces it is built from."""
import math
import os

import numpy as np
import pytest

from helmholtzbem_gb300 import _capi
from oracle import oracle as O


def _api():
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("libhbem.so not built")
    from helmholtzbem_gb300 import api
    return api


def _f(xs):
    xs = np.asarray(xs, float)
    return np.cos(2.0 * xs) + 0.05 * (xs - 4.0) ** 2


@pytest.mark.parametrize("seed", [1, 7, 2024])
def test_opt_subdiv_matches_oracle(seed):
    api = _api()
    x, y, p = api.opt_subdiv(_f, 0.5, 9.5, 8, 4, 1e-4 * 9.0, seed=seed)
    ox, oy, op = O.opt_subdiv(lambda xs: list(_f(xs)), 0.5, 9.5, 8, 4, 1e-4 * 9.0, seed)
    assert len(x) == len(ox) and list(p) == list(op)
    assert np.max(np.abs(x - ox)) <= 1e-9 * 9.0
    assert np.all(np.diff(x) >= 0) and len(p) > 0
    # the reported minima are local minima of the samples, one per well of cos 2x
    assert np.all(y[p] < y[np.asarray(p) - 1]) and np.all(y[p] < y[np.asarray(p) + 1])
    wells = [m * math.pi + math.pi / 2 for m in range(0, 4) if 0.6 < m * math.pi + math.pi / 2 < 9.4]
    assert len(p) >= len(wells) - 1


def test_oracle_pieces():
    """Steffen's spline stays monotone on monotone data; the Floater-Hormann
    interpolant of order 5 reproduces a degree-5 polynomial; the two Brent variants
    find a parabola's minimum, and the bracketed one refuses a bad bracket."""
    x = np.linspace(0.0, 2.0, 9)
    y = x ** 3
    yp = O.steffen_slopes(x, y)
    vals = [O.steffen_eval(x, y, yp, t) for t in np.linspace(0.0, 2.0, 101)]
    assert np.all(np.diff(vals) >= -1e-15)
    r = O.floater_hormann(x, 1.0 + x - 2.0 * x ** 5, 5)
    for t in (0.13, 0.77, 1.91):
        assert abs(r(t) - (1.0 + t - 2.0 * t ** 5)) < 1e-10
    f = lambda t: (t - 0.7) ** 2 + 0.1   # noqa: E731
    assert abs(O.brent_guess(0.0, 2.0, 1.5, f(1.5), f, 1e-10) - 0.7) < 1e-6
    assert abs(O.brent_search(0.0, f(0.0), 2.0, f(2.0), 0.9, f(0.9), f, 1e-10) - 0.7) < 1e-6
    assert O.brent_search(0.0, f(0.0), 2.0, f(2.0), 1.99, f(1.99), f, 1e-10) is None
