"""The oracle against the reference's own regression data: the Mg24 / USDB
examples of examples/gradient_mg24 (stored tables copied to tests/golden/)."""

import numpy as np
import pytest

from conftest import golden_table

import oracle as O


def run_oracle(model, U, V, cons, M, eta, mu, iters=3000):
    om = O.OracleModel(model)
    ops, vals = cons
    vap = O.OracleVAP(om, U, V, M, M, 2 * np.pi, 4.0, 4.0, eta, mu, 1e-4, np.stack(ops), np.array(vals), nthreads=1)
    assert vap.initial_adjust() == 0
    for it in range(1, iters + 1):
        st, info = vap.iterate()
        assert st in (0, 1), st
        if st == 1:
            return it, info
    return iters, info


@pytest.mark.parametrize("eta,mu", [(0.05, 0.6), (0.1, 0.3), (0.05, 0.0)])
def test_mg24_pnvap_m5(usdb_model, mg24_seed, mg24_constraints, eta, mu):
    table = golden_table("mg24_results_vap_benchmark")
    it_ref, e_ref = table[(eta, mu)]
    it, info = run_oracle(usdb_model, *mg24_seed, mg24_constraints, 5, eta, mu)
    assert abs(info[1] - e_ref) < 1e-6  # printed with 6 decimals
    assert it == it_ref


@pytest.mark.parametrize("eta,mu", [(0.025, 0.6), (0.1, 0.0)])
def test_mg24_hfb(usdb_model, mg24_seed, mg24_constraints, eta, mu):
    table = golden_table("mg24_results_hfb_benchmark")
    it_ref, e_ref = table[(eta, mu)]
    it, info = run_oracle(usdb_model, *mg24_seed, mg24_constraints, 1, eta, mu)
    assert abs(info[1] - e_ref) < 1e-6
    assert it == it_ref
