"""The host side of the gradient loop (taurus_vap_gb300/vap.py: the constraint
algebra, the Lagrange multipliers, the adjust_constraints Newton loop, the
convergence test) on the CPU.

vap.VAP drives a context object; here the context's three calls come from the
oracle instead of the device library, so the loop's own logic is checked
against the reference's Mg24 / USDB regression tables without a GPU.
"""

import numpy as np
import pytest

from conftest import golden_table

import oracle as O
from taurus_vap_gb300.vap import VAP, Constraints


class OracleBackedContext:
    """The three calls vap.VAP makes, answered by the oracle: the projection
    and the Thouless evolution from liboracle, the type-0 gradient step
    Z_i = -eta (H20v - sum_j lambda_j C20_j) + mu Z_{i-1} with norm
    |Z_i|_F / eta (module_gradient.f90:124-141)."""

    def __init__(self, model):
        self.n = model.n
        self.om = O.OracleModel(model)

    def project(self, U0, V0, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=1.0, seed_occeps=0.0,
                seed_allemp=0, mode=0):
        r = self.om.project(U0, V0, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=factor_delta,
                            occeps=seed_occeps, allemp=seed_allemp, nthreads=1)
        assert r["status"] == 0, r["status"]
        return r["pnp"], r["H20v"]

    def calculate_gradient(self, H20v, lambdas, C20, Zim1, eta, mu):
        g = np.array(H20v, dtype=np.float64)
        if lambdas is not None:
            g -= np.asarray(lambdas) @ np.asarray(C20)
        Zi = -eta * g + mu * np.asarray(Zim1, dtype=np.float64).reshape(-1)
        return Zi, float(np.sqrt(np.sum(Zi * Zi)) / eta)

    def evolve(self, U0, V0, Z):
        st, U1, V1 = O.thouless_evolve(U0, V0, np.reshape(Z, (self.n, self.n), order="F"))
        assert st == 0, st
        return U1, V1

    def diagonalize_hsp_and_H11(self, U0, V0, lambdas=None, constraints_HO=None, cpair=0, factor_delta=1.0):
        return O.diagonalize_hsp_and_H11(self.om, U0, V0, () if lambdas is None else lambdas, constraints_HO,
                                         cpair=cpair, factor_delta=factor_delta, nthreads=1)


@pytest.mark.parametrize("M,table,eta,mu", [(5, "mg24_results_vap_benchmark", 0.05, 0.6),
                                            (1, "mg24_results_hfb_benchmark", 0.025, 0.6)])
def test_host_loop_reproduces_mg24(usdb_model, mg24_seed, mg24_constraints, M, table, eta, mu):
    it_ref, e_ref = golden_table(table)[(eta, mu)]
    ops, vals = mg24_constraints
    vap = VAP(OracleBackedContext(usdb_model), *mg24_seed, M, M, 4.0, 4.0, eta, mu,
              constraints=Constraints(ops, vals))
    it, info = vap.run(iter_max=3000)
    assert abs(info[1] - e_ref) < 1e-6
    assert it == it_ref


@pytest.mark.parametrize("recipe", [1, 2])
def test_host_loop_gradient_types(usdb_model, mg24_seed, mg24_constraints, recipe):
    # vap.VAP with gradient_type 1 / 2: the spectra from the context, the step
    # sizes from tvap_gradient_parameters (host arithmetic of the library);
    # the reference's PNVAP recipe rows (M = 5)
    from test_oracle_golden import recipe_rows

    it_ref, e_ref = recipe_rows("mg24_results_vap_benchmark")[recipe]
    ops, vals = mg24_constraints
    vap = VAP(OracleBackedContext(usdb_model), *mg24_seed, 5, 5, 4.0, 4.0, 0.0, 0.0,
              constraints=Constraints(ops, vals), gradient_type=recipe)
    it, info = vap.run(iter_max=3000)
    assert abs(info[1] - e_ref) < 1e-6
    assert it == it_ref


def test_constraints_hold_after_adjustment(usdb_model, mg24_seed, mg24_constraints):
    """After adjust_constraints the expectation values of the constraint
    operators (Z, N, Q21) sit at their targets within the tolerance
    (module_constraints.f90:270-373)."""
    from taurus_vap_gb300.vap import expectval_obo

    ops, vals = mg24_constraints
    vap = VAP(OracleBackedContext(usdb_model), *mg24_seed, 5, 5, 4.0, 4.0, 0.05, 0.6,
              constraints=Constraints(ops, vals))
    vap.adjust_constraints()
    for _ in range(3):
        st, _ = vap.iterate()
        assert st == 0
    n = usdb_model.n
    rho = vap.V0 @ vap.V0.T
    for op, val in zip(ops, vals):
        got = expectval_obo(rho, np.reshape(op, (n, n), order="F"))
        assert abs(got - val) < 1e-6, (got, val)


class OracleAdjointContext:
    """energy_adjoint answered by the oracle: E of the evolved state and
    dE/dZ = L^-T H20v L^-1 with L L^T = 1 + Z^T Z, the relation the device
    adjoint uses (checked against finite differences in
    test_oracle_identities)."""

    def __init__(self, model):
        self.n = model.n
        self.om = O.OracleModel(model)
        self.calls = 0

    def energy_adjoint(self, U0, V0, Z, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=1.0, mode=0):
        self.calls += 1
        n = self.n
        Z = np.reshape(Z, (n, n), order="F")
        st, U1, V1 = O.thouless_evolve(U0, V0, Z)
        assert st == 0
        r = self.om.project(U1, V1, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=factor_delta, nthreads=1)
        p = r["pnp"]
        H = r["H20v"].reshape(n, n, order="F")
        Li = np.linalg.inv(np.linalg.cholesky(np.eye(n) + Z.T @ Z))
        return (p.c("ener") / p.c("over")).real, np.asfortranarray(Li.T @ H @ Li)


def test_autograd_function_on_the_cpu():
    """taurus_vap_gb300.autograd: one adjoint call per forward, none in
    backward, the gradient scaled by the incoming one, and central finite
    differences of E(Z) matched."""
    torch = pytest.importorskip("torch")
    from taurus_vap_gb300 import model as M
    from taurus_vap_gb300.autograd import projected_energy

    mdl = M.sd_model(seed=3)
    n = mdl.n
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=7)
    ctx = OracleAdjointContext(mdl)
    rng = np.random.default_rng(4)
    Z0 = 0.1 * rng.normal(size=(n, n))
    Z0 = Z0 - Z0.T
    Z = torch.tensor(Z0, dtype=torch.float64, requires_grad=True)
    E = projected_energy(Z, ctx, U, V, 5, 5, 4, 4)
    (3.0 * E).backward()
    assert ctx.calls == 1
    D = rng.normal(size=(n, n))
    D = D - D.T
    h = 1e-5
    Ep = projected_energy(torch.tensor(Z0 + h * D), ctx, U, V, 5, 5, 4, 4).item()
    Em = projected_energy(torch.tensor(Z0 - h * D), ctx, U, V, 5, 5, 4, 4).item()
    fd = 3.0 * (Ep - Em) / (2 * h)
    assert abs(fd - float((Z.grad.numpy() * D).sum())) < 1e-6 * max(1.0, abs(fd))



def test_c20_follows_the_state(usdb_model, mg24_seed, mg24_constraints):
    """The loop takes C20 from the constraint loop that produced the state and
    recomputes it (update_constraints_qpbasis, module_constraints.f90:381-397)
    only for a state set from outside: after every iteration C20 is that of
    the current state (set_operator_qpbasis, module_operators.f90:49-97)."""
    from taurus_vap_gb300.vap import set_operator_qpbasis

    ops, vals = mg24_constraints
    vap = VAP(OracleBackedContext(usdb_model), *mg24_seed, 5, 5, 4.0, 4.0, 0.05, 0.6,
              constraints=Constraints(ops, vals))
    n = usdb_model.n
    calls = []  # the U of every C20 update
    update = vap.update_constraints_qpbasis

    def recording_update(U, V):
        calls.append(U)
        update(U, V)

    vap.update_constraints_qpbasis = recording_update

    def c20_is_of_state():
        for i, op in enumerate(ops):
            want = set_operator_qpbasis(vap._part(i), vap.U0, vap.V0, np.reshape(op, (n, n), order="F"))
            assert np.allclose(vap.C20[i].reshape((n, n), order="F"), want, rtol=0, atol=1e-13)

    seed = vap.U0
    vap.iterate()
    assert calls[0] is seed  # the seed's C20, before the first projection
    c20_is_of_state()
    state, n_calls = vap.U0, len(calls)
    vap.iterate()
    # no recompute for the constraint loop's own state: the next update is of
    # the loop's first evolved state
    assert len(calls) > n_calls and calls[n_calls] is not state
    c20_is_of_state()
    # a state set from outside is recomputed before it is used
    outside = np.asfortranarray(mg24_seed[0])
    vap.U0, vap.V0 = outside, np.asfortranarray(mg24_seed[1])
    n_calls = len(calls)
    vap.iterate()
    assert calls[n_calls] is outside
    c20_is_of_state()
