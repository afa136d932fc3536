"""The device path reproduces the reference's Mg24 / USDB PNVAP regression
(examples/gradient_mg24): same iteration count, converged energy within 1e-6."""

import numpy as np
import pytest

from conftest import golden_table
from taurus_vap_gb300.native import Context
from taurus_vap_gb300.vap import VAP, Constraints

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("eta,mu", [(0.05, 0.6)])
def test_mg24_pnvap_on_device(usdb_model, mg24_seed, mg24_constraints, eta, mu):
    it_ref, e_ref = golden_table("mg24_results_vap_benchmark")[(eta, mu)]
    ctx = Context(usdb_model.basis, usdb_model.ham)
    ops, vals = mg24_constraints
    vap = VAP(ctx, *mg24_seed, 5, 5, 4.0, 4.0, eta, mu, constraints=Constraints(ops, vals))
    it, info = vap.run(iter_max=3000)
    assert abs(info[1] - e_ref) < 1e-6
    assert it == it_ref
