"""The proposal network's oracle on the CPU: exact (float64) gradients against
central finite differences, and the bfloat16 rounding helper."""
import numpy as np

from oracle import oracle as O


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -3.14159, 65504.0], np.float32)
    r = O.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == 1.0 + 2 ** -6
    assert abs(r[4] + 3.140625) < 1e-6
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(0)
    dims = [5, 7, 6, 3]
    nparam = sum(o * i + o for i, o in zip(dims[:-1], dims[1:]))
    p = rng.standard_normal(nparam) * 0.5
    X = rng.standard_normal((4, 5))
    T = rng.standard_normal((4, 3))
    loss, g = O.MLPOracle(p, dims, bf16=False).gradients(X, T)
    h = 1e-6
    for j in rng.choice(nparam, 25, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[j] += h
        pm[j] -= h
        lp = O.MLPOracle(pp, dims, bf16=False).gradients(X, T)[0]
        lm = O.MLPOracle(pm, dims, bf16=False).gradients(X, T)[0]
        assert abs((lp - lm) / (2 * h) - g[j]) <= 1e-6 * max(1.0, abs(g[j]))
