"""Scatterer files and polygonal meshes (source/utilities/scatterer.cpp:30-277,
examples/find_resonances.cpp:111-124): the host code of libhbem against the oracle
restatement, bit for bit, plus the geometric properties of the graded meshes."""
import math
import os

import numpy as np
import pytest

from helmholtzbem_gb300 import _capi
from oracle import oracle as O

if not os.path.exists(_capi.LIB_PATH):
    pytest.skip("libhbem.so not built", allow_module_level=True)

from helmholtzbem_gb300 import geometry as G  # noqa: E402


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode())
    return str(p)


POLYGONS = {
    "square": ([0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 1.0]),
    "L": ([0.0, 2.0, 2.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 1.0, 2.0, 2.0]),
    "star24": G.star_polygon(24, seed=2),
    "star9": G.star_polygon(9, seed=5),
    "thin": ([0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 0.05, 0.05]),
}


def test_read_formats(tmp_path):
    good = _write(tmp_path, "a.dat", "0.5,0\n  0.25 , 0.75\r\n\n\t-1e-1,2.5E0\n0,1,\n")
    x, y = G.read_scatterer(good, scale=2.0)
    assert np.array_equal(x, [1.0, 0.5, -0.2, 0.0]) and np.array_equal(y, [0.0, 1.5, 5.0, 2.0])
    ox, oy = O.read_scatterer(good, 2.0)
    assert np.array_equal(x, ox) and np.array_equal(y, oy)
    # a one-field row among two-field rows is padded with 0
    x, y = G.read_scatterer(_write(tmp_path, "b.dat", "1,2\n3\n4,5\n"))
    assert np.array_equal(x, [1, 3, 4]) and np.array_equal(y, [2, 0, 5])
    assert np.array_equal(O.read_scatterer(str(tmp_path / "b.dat"))[1], y)


@pytest.mark.parametrize("text", ["# vertices\n0,0\n1,0\n", "0,0,0\n1,0,0\n", "1,,2\n", "abc,1\n", "", "\n\n",
                                  "1e999,0\n", ",1\n"])
def test_read_rejects(tmp_path, text):
    f = _write(tmp_path, "bad.dat", text)
    with pytest.raises(ValueError):
        G.read_scatterer(f)
    assert O.read_scatterer(f) is None


def test_read_missing_file(tmp_path):
    with pytest.raises(ValueError):
        G.read_scatterer(str(tmp_path / "none.dat"))


@pytest.mark.parametrize("name", list(POLYGONS))
def test_length_and_auto_count(name):
    x, y = POLYGONS[name]
    assert G.polygon_length(x, y) == O.polygon_length(list(x), list(y))
    for f in (0.1, 0.25, 0.5):
        assert G.auto_num_panels(x, y, f) == O.auto_num_panels(list(x), list(y), f)


@pytest.mark.parametrize("name", list(POLYGONS))
@pytest.mark.parametrize("N", [4, 37, 100, 1000])
def test_uniform_panels_bit_exact(name, N):
    x, y = POLYGONS[name]
    if N < len(x):
        N = len(x)
    k, p = G.polygon(x, y, N)
    ko, po = O.polygon_panels(x, y, N)
    assert len(k) == N and np.array_equal(k, ko) and np.array_equal(p, po)


def _chain_closed(par, x, y):
    n = par.shape[0]
    for i in range(n):
        assert par[i, 2] == par[(i + 1) % n, 0] or abs(par[i, 2] - par[(i + 1) % n, 0]) < 1e-12
        assert abs(par[i, 3] - par[(i + 1) % n, 1]) < 1e-12
    ends = {(a, b) for a, b in zip(par[:, 0], par[:, 1])}
    for vx, vy in zip(x, y):
        assert (vx, vy) in ends                # every corner is a panel endpoint, exactly


@pytest.mark.parametrize("name", list(POLYGONS))
@pytest.mark.parametrize("N", [12, 40, 97, 400])
@pytest.mark.parametrize("rf", [0.25, 0.5, 1.0])
def test_graded_panels_bit_exact_and_closed(name, N, rf):
    x, y = POLYGONS[name]
    k, p = G.polygon_graded(x, y, N, rf)
    ko, po = O.polygon_panels_graded(x, y, N, rf)
    assert np.array_equal(k, ko) and np.array_equal(p, po)
    _chain_closed(p, x, y)
    assert abs(len(k) - N) <= len(x)


def test_graded_square_shrinks_towards_corners():
    """Right angles: f = rf + (1 - rf)/2; the first and last panel of each edge are f
    times the uniform length and the panels grow towards the middle of the edge."""
    x, y = POLYGONS["square"]
    rf = 0.5
    _, p = G.polygon_graded(x, y, 40, rf)
    lens = np.hypot(p[:, 2] - p[:, 0], p[:, 3] - p[:, 1])
    per_edge = np.split(lens, 4)
    f = rf + (1 - rf) * 0.5
    for e in per_edge:
        uniform = 1.0 / len(e)
        assert abs(e[0] - f * uniform) < 1e-9 and abs(e[-1] - f * uniform) < 1e-9
        mid = len(e) // 2
        assert np.all(np.diff(e[:mid]) > 0) and np.all(np.diff(e[mid + 1:]) < 0)
        assert abs(e.sum() - 1.0) < 1e-12


def test_choose_num_panels_matches_oracle_and_target():
    for name in ("star24", "L"):
        x, y = POLYGONS[name]
        for kmax in (5.0, 12.0):
            n = G.choose_num_panels(x, y, kmax, degf=10.0, rfac=0.5)
            assert n == O.choose_num_panels(list(x), list(y), kmax, 10.0, 0.5)
            _, p = G.polygon_graded(x, y, n, 0.5)
            longest = np.hypot(p[:, 2] - p[:, 0], p[:, 3] - p[:, 1]).max()
            assert abs(longest - 2 * math.pi / (10.0 * kmax)) < 0.2 * 2 * math.pi / (10.0 * kmax)
