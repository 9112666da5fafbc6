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
    res = L.evaluate(net, list(range(20000, 20004)), plain_points=105, coarse_points=25)
    assert res["windows"] == 4
    # the batched plain search is the same search: the same roots
    assert res["plain_batched"]["roots"] == res["plain"]["roots"] and res["plain_batched"]["recall"] == 1.0
    for m in ("learned_batched", "coarse_batched", "learned_coarse_batched"):
        assert 0.0 <= res[m]["recall"] <= 1.0 and res[m]["evals"] > 0


def test_sweep_sigma_multi_matches_single_operator_sweeps():
    cases = [L.draw(s) for s in (20010, 20011, 20012)]
    ops = [L.operator(a, b) for (a, b, _, _) in cases]
    ks = [L.window(c[3])[::16] for c in cases]
    ci = [c[2] for c in cases]
    multi = api.sweep_sigma_multi(ops, ks, 1.0, ci, d=2)
    for so, k, c, m in zip(ops, ks, ci, multi):
        single = so.sweep_sigma(k, 1.0, c, d=2)
        assert np.array_equal(single, m)


def test_shipped_network_proposes_most_resonances():
    """The packaged network on the 40 held-out windows of the benchmark (seeds
    20000..20039): 75 of the plain search's 91 roots are found from its proposals
    alone (recall 0.824 measured), and the network adds recall to a coarse grid."""
    net = L.default_network()
    res = L.evaluate(net, list(range(20000, 20040)), plain_points=210, coarse_points=43)
    assert res["plain"]["roots"] == 91
    assert res["learned_batched"]["recall"] >= 0.82
    # resonances per second count only roots that match a plain root
    lb = res["learned_batched"]
    assert abs(lb["res_per_s"] * lb["seconds"] - lb["matched"]) < 1e-6 * lb["matched"]
    assert res["learned_coarse_batched"]["recall"] >= res["coarse_batched"]["recall"]
