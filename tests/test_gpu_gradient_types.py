"""Gradient types 1 and 2 on the device: diagonalize_hsp_and_H11(0)
(module_gradient.f90:158-453) through tvap_diagonalize_hsp_and_H11 against
the oracle's DSYEV of the same matrices, and the device gradient loop with
the automatic step sizes against the reference's Mg24 'Recipe' rows
(examples/gradient_mg24: gradient_type 1 and 2, PNVAP M = 5).

Tolerance of the spectra: 1e-12 of the largest |eigenvalue| (both are
backward-stable FP64 reductions of the same matrices)."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context, gradient_parameters
from taurus_vap_gb300.vap import VAP, Constraints

import oracle as O

pytestmark = pytest.mark.gpu


def spectra_close(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= 1e-12 * max(np.abs(b).max(), 1e-300)


def test_diagonalize_mg24_with_constraints(usdb_model, mg24_seed, mg24_constraints):
    U, V = mg24_seed
    ops, _ = mg24_constraints
    lam = np.array([-7.3, -6.1, 0.42])
    ctx = Context(usdb_model.basis, usdb_model.ham)
    eh, e11, info = ctx.diagonalize_hsp_and_H11(U, V, lam, np.stack(ops))
    rh, r11, rinfo = O.diagonalize_hsp_and_H11(O.OracleModel(usdb_model), U, V, lam, np.stack(ops))
    assert info == (0, 0) and rinfo == (0, 0)
    assert spectra_close(eh, rh) and spectra_close(e11, r11)
    for t in (1, 2):
        assert np.allclose(gradient_parameters(t, eh, e11, info, 0.0, 0.0),
                           gradient_parameters(t, rh, r11, rinfo, 0.0, 0.0), rtol=1e-12, atol=0)


@pytest.mark.parametrize("emax,Z", [(2, 4), (4, 8)])
def test_diagonalize_noncore(emax, Z):
    # n = 40 and 140 (products on the tensor cores at n = 140), with a pair
    # constraint among the constraints (its H11 term is zero)
    mdl = M.noncore_model(emax, seed=1, valence_Z=Z, valence_N=Z)
    U, V = M.random_bogoliubov(mdl.basis, Z, Z, seed=2)
    n = mdl.n
    rng = np.random.default_rng(emax)
    A = rng.normal(size=(n, n))
    ops = np.stack([np.eye(n).reshape(-1), (A + A.T).reshape(-1), (A - A.T).reshape(-1)])
    lam = np.array([-3.0, 0.2, 0.7])
    ctx = Context(mdl.basis, mdl.ham)
    eh, e11, info = ctx.diagonalize_hsp_and_H11(U, V, lam, ops, cpair=1)
    rh, r11, rinfo = O.diagonalize_hsp_and_H11(O.OracleModel(mdl), U, V, lam, ops, cpair=1)
    assert info == (0, 0) and rinfo == (0, 0)
    assert spectra_close(eh, rh) and spectra_close(e11, r11)


def test_diagonalize_reports_nonfinite(usdb_model, mg24_seed):
    # a non-finite state (n = 24: every product on the FP64 pipe, which
    # carries the NaN).  A NaN in U reaches kappa and H11 but not
    # rho = V V^T and h; one in V reaches both.  The step sizes then fall back
    # to the input eta and mu, as the reference does for a failed DSYEV
    U, V = mg24_seed
    ctx = Context(usdb_model.basis, usdb_model.ham)
    U2 = U.copy(order="F")
    U2[3, 3] = np.nan
    eh, e11, info = ctx.diagonalize_hsp_and_H11(U2, V)
    assert info == (0, 1)
    assert gradient_parameters(1, eh, e11, info, 0.05, 0.6) == (0.05, 0.6)
    assert gradient_parameters(2, eh, e11, info, 0.05, 0.6) != (0.05, 0.6)
    V2 = V.copy(order="F")
    V2[3, 3] = np.nan
    eh, e11, info = ctx.diagonalize_hsp_and_H11(U, V2)
    assert info == (1, 1)
    assert gradient_parameters(2, eh, e11, info, 0.05, 0.6) == (0.05, 0.6)


@pytest.mark.parametrize("recipe", [1, 2])
def test_mg24_gradient_types_on_device(usdb_model, mg24_seed, mg24_constraints, recipe):
    from test_oracle_golden import recipe_rows

    it_ref, e_ref = recipe_rows("mg24_results_vap_benchmark")[recipe]
    ctx = Context(usdb_model.basis, usdb_model.ham)
    ops, vals = mg24_constraints
    vap = VAP(ctx, *mg24_seed, 5, 5, 4.0, 4.0, 0.0, 0.0, constraints=Constraints(ops, vals), gradient_type=recipe)
    it, info = vap.run(iter_max=3000)
    assert abs(info[1] - e_ref) < 1e-6
    assert it == it_ref
    assert math.isfinite(vap.step_sizes[0]) and vap.step_sizes[0] > 0
