"""The learned proposal's GPU pieces: bracket refinement (Newton on sigma_min' from
candidate brackets) against the plain search's roots, and a small end-to-end
training run and evaluation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry, learned as L  # noqa: E402


def test_refine_brackets_recovers_the_plain_roots():
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(0.25, 50), order=11))
    roots, _, _ = so.find_resonances_plain(0.5, 10.0, 200, 1.0, 23.4, tol=1e-8)
    assert roots.size >= 5
    got, ne = so.refine_brackets(roots - 0.01, roots + 0.01, 1.0, 23.4)
    assert got.size == roots.size and np.max(np.abs(got - roots)) <= 1e-8
    # brackets one width off to the right: both ends rise, the bracket moves left once
    got2, _ = so.refine_brackets(roots + 0.011, roots + 0.031, 1.0, 23.4)
    assert got2.size == roots.size and np.max(np.abs(got2 - roots)) <= 1e-8
    # a bracket around a maximum of sigma (between two minima) gives nothing
    mid = 0.5 * (roots[0] + roots[1])
    got3, _ = so.refine_brackets(np.array([mid - 1e-3]), np.array([mid + 1e-3]), 1.0, 23.4, max_shift=0)
    assert got3.size == 0 or np.min(np.abs(got3[:, None] - roots[None, :])) <= 1e-8


def test_small_training_run_and_evaluation():
    X, Y = L.dataset(list(range(10000, 10064)))
    assert np.all(np.isfinite(Y)) and Y.min() < -1.0
    net, losses = L.train(X, Y, epochs=40, batch=64, lr=1e-3, seed=1)
    assert np.mean(losses[-4:]) < np.mean(losses[:4]) / 5
    res = L.evaluate(net, list(range(20000, 20004)), plain_points=105)
    assert res["windows"] == 4 and 0.0 <= (res["recall"] or 0.0) <= 1.0
    assert res["learned_evals"] > 0 and res["plain_evals"] > 0
