"""The C++ facade (include/hbem.hpp) compiles against the C ABI; on a GPU it runs
the reference's call sequence and agrees with the Python mirror."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_smoke.cpp")
LIBDIR = os.path.join(ROOT, "helmholtzbem_gb300", "_lib")


def _compile(tmp_path):
    exe = str(tmp_path / "facade_smoke")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-Wl,-rpath," + LIBDIR, "-lhbem"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libhbem.so")):
        pytest.skip("libhbem.so not built")
    _compile(tmp_path)


@pytest.mark.gpu
def test_facade_runs_and_matches_python(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, str(tmp_path / "square.dat")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = [float(v) for v in r.stdout.split()]
    from helmholtzbem_gb300 import api, geometry
    data = api.BuilderData(geometry.circle(0.25, 16), order=7)
    so = api.SolutionsOperator(data)
    ref = api.sv_dense([so.gen_sol_op_2nd_der(2.5, 1.0, 23.4)], d=2)[0]
    assert np.allclose(vals[:3], ref, rtol=1e-12, atol=0)
    assert abs(vals[4] - np.pi / 2) < 1e-12 and vals[5] == 1 and vals[6] == 1
    assert abs(vals[7] - ref[0]) <= 1e-11 * ref[0] and abs(vals[8] - ref[0]) <= 1e-11 * ref[0]
    # scatterer::read + make_polygonal_panels + SolutionsOperator on the graded square
    sq = geometry.polygon_graded([0.0, 0.5, 0.5, 0.0], [0.0, 0.0, 0.5, 0.5], 24, 0.5)
    assert int(vals[9]) == len(sq[0])
    ssq = api.sv_dense([[api.SolutionsOperator(api.BuilderData(sq, order=7)).gen_sol_op(3.0, 1.0, 4.0)]])[0][0]
    assert abs(vals[10] - ssq) <= 1e-12 * ssq
    # tp::direct_second_kind::solve_in_rectangle on the circle mesh, total field
    so_u = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 16), order=7), proj=False)
    S, gx, gy = api.tp_field_grid(so_u, api.wave("Plane", angle=0.5), 2.5, 1.0, 4.0, 10, (-0.5, -0.5), (0.5, 0.5),
                                  9, 7, total_field=True)
    assert abs(complex(vals[11], vals[12]) - S[2, 5]) <= 1e-12 * abs(S[2, 5]) and vals[13] == gy[2, 5]
    # randomized sigma: an estimate from above, close on the 12-wide sketch with 2 subspace steps
    assert ref[0] * (1 - 1e-12) <= vals[14] <= ref[0] * (1 + 1e-3)
    # reverse communication: the same iterates as the callback form (Brent's tolerance sqrt(tol) |x|)
    assert vals[15] == api.brent_min(np.cos, 2.0, 4.0, 1e-8) and abs(vals[15] - np.pi) < 1e-3
