"""The adaptive resonance search (examples/find_resonances.cpp with opt_subdiv) on the
GPU against the oracle's restatement with the oracle's sigma on the same sketch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from helmholtzbem_gb300 import api, geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402


def test_adaptive_search_vs_oracle():
    kinds, par = geometry.circle(0.25, 16)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=7))
    oso = O.SolutionsOperator(O.Builder(kinds, par, 7))
    c_o, c_i, k_min, k_max = 1.0, 23.4, 1.0, 6.0
    seed, sketch, q, batch, limit, tol = 11, 2, 2, 16, 4, 1e-8
    roots, ns, ne = so.find_resonances_adaptive(k_min, k_max, c_o, c_i, batch_size=batch, limit=limit, tol=tol,
                                                seed=seed, sketch=sketch, q=q)
    n = 2 * len(kinds)
    R = api.randGaussian(n, sketch, seed=seed)

    def f_sample(ks):
        return [O.rsvd_sv(oso.gen_sol_op(k, c_o, c_i)[0], R, q) for k in ks]

    def f_fine(ks):
        return [O.sv_derivs(oso.gen_sol_op(k, c_o, c_i)[0])[0] for k in ks]

    oroots, ons = O.find_resonances_adaptive(f_sample, f_fine, k_min, k_max, batch, limit, 1e-4 * (k_max - k_min),
                                             tol, seed)
    assert ns == ons
    assert len(roots) == len(oroots) and len(roots) > 0
    assert np.max(np.abs(roots - oroots)) <= 1e-6
    # every minimum found is a minimum of the dense sigma_min: sigma at root +- 1e-5 is larger
    s0 = so.sweep_sigma(roots, c_o, c_i, d=0)[:, 0]
    sl = so.sweep_sigma(roots - 1e-5, c_o, c_i, d=0)[:, 0]
    sr = so.sweep_sigma(roots + 1e-5, c_o, c_i, d=0)[:, 0]
    assert np.all(s0 <= sl) and np.all(s0 <= sr)
