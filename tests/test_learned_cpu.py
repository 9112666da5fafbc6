"""Host logic of the learned proposal: seeded scatterers, input features, mesh
scale, window grid and the local-minimum rule."""
import os

import numpy as np
import pytest

from helmholtzbem_gb300 import _capi

if not os.path.exists(_capi.LIB_PATH):
    pytest.skip("libhbem.so not built", allow_module_level=True)

from helmholtzbem_gb300 import learned as L  # noqa: E402


def test_draw_is_seeded_and_in_range():
    a1, b1, c1, k1 = L.draw(10001)
    a2, b2, c2, k2 = L.draw(10001)
    assert np.array_equal(a1, a2) and c1 == c2 and k1 == k2
    assert L.FAMILY["c_lo"] <= c1 <= L.FAMILY["c_hi"] and L.FAMILY["k_lo"] <= k1 <= L.FAMILY["k_hi"]
    assert L.draw(10002)[2] != c1


def test_features_layout():
    a, b, c, k0 = L.draw(7)
    x = L.features(a, b, c, k0)
    assert x.shape == (34,) and x.dtype == np.float32
    assert np.allclose(x[:8], 20 * a) and np.all(x[8:16] == 0) and np.allclose(x[16:24], 20 * b)
    assert np.isclose(x[32], np.sqrt(c) / 5) and np.isclose(x[33], k0 * np.sqrt(c) * 0.25 / 12.5)
    assert L.draw(7, 2)[2] == c and L.draw(7, 2)[3] != k0 and L.draw(7, 0)[3] == k0


def test_mesh_is_scaled_and_closed():
    a, b, _, _ = L.draw(3)
    kinds, par = L.mesh(a, b)
    assert len(kinds) == L.FAMILY["N"]
    r = np.hypot(par[:, 0], par[:, 1])
    assert 0.3 * 0.25 <= r.min() and r.max() < 0.6
    assert np.allclose(par[:-1, 2:4], par[1:, 0:2]) and np.allclose(par[-1, 2:4], par[0, 0:2])


def test_window_and_local_minima():
    ks = L.window(1.5)
    assert ks.size == 128 and ks[0] == 1.5 and abs(ks[-1] - 3.5) < 1e-12
    c = np.array([3.0, 2.0, 2.5, 1.0, 1.0, 4.0, 3.0])
    assert L.local_minima(c) == [1, 3]
