"""adjust_constraints (module_constraints.f90:270-373) on the device
(tvap_adjust_constraints) against the oracle's restatement: the adjusted
state from the same seed and targets, on the Mg24 / USDB example's
constraints (Z, N, Q21 = 0) and on the emax=4 basis with a quadrupole Q20
target moved away from the seed's value (several Newton steps, products on
the tensor cores).

Tolerances: U1, V1 to 1e-11; the constraint expectation values of the
adjusted state within the loop's own tolerance (1e-6) of the targets."""

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context
from taurus_vap_gb300.vap import particle_number_ops

import oracle as O

pytestmark = pytest.mark.gpu


def expectation(U, V, op, n):
    rho = V @ V.T
    return float(np.sum(np.reshape(op, (n, n), order="F") * rho.T))


def check_adjust(model, U, V, ops, vals):
    n = model.n
    ctx = Context(model.basis, model.ham)
    U1, V1, Zi, C20, steps = ctx.adjust_constraints(U, V, np.zeros(n * n), np.stack(ops), vals)
    om = O.OracleModel(model)
    ovap = O.OracleVAP(om, U, V, 1, 1, 2 * np.pi, 4.0, 4.0, 0.05, 0.0, 1e-4, np.stack(ops), np.array(vals), nthreads=0)
    assert ovap.initial_adjust() == 0
    Ur, Vr, Zr, _ = ovap.state()
    assert np.abs(U1 - Ur).max() < 1e-11 and np.abs(V1 - Vr).max() < 1e-11
    for op, val in zip(ops, vals):
        assert abs(expectation(U1, V1, op, n) - val) < 1e-6
    return steps


def test_adjust_mg24(usdb_model, mg24_seed, mg24_constraints):
    ops, vals = mg24_constraints
    steps = check_adjust(usdb_model, *mg24_seed, ops, vals)
    assert steps >= 1


def test_adjust_emax4_q20():
    mdl = M.noncore_model(4, seed=1, valence_Z=8, valence_N=8)
    U, V = M.random_bogoliubov(mdl.basis, 8, 8, seed=2)
    n = mdl.n
    q = mdl.multipoles()
    Qz, Qn = particle_number_ops(n)
    q20 = q[1, 0, 0] + q[1, 1, 0]
    target = expectation(U, V, q20, n) + 5.0
    steps = check_adjust(mdl, U, V, [Qz, Qn, q20], [8.0, 8.0, target])
    assert steps >= 2
