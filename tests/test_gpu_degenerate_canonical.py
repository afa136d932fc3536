"""Canonical bases with degenerate subspaces larger than 2 against the oracle.

A spherical state has one occupation per j-shell, so each shell is a
(2j+1)-fold degenerate level of rho; kappa is not in canonical form on such a
subspace until it is reduced (the reference uses the real Schur form, DGEES,
module_wavefunctions.f90:873-906).  These projections failed with
TVAP_ERR_CANONICAL before the device reduced the subspaces.

Tolerances as in test_gpu_parity: projected energy 1e-9 MeV, particle
numbers 1e-10, pnp_over 1e-10 relative, field_H20v 1e-9 of its largest entry.
"""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu


def check(mdl, U, V, Mphi, Z, N, gemm_mode=2, ctx=None):
    om = O.OracleModel(mdl)
    ref = om.project(U, V, Mphi, Mphi, 2 * math.pi, Z, N)
    assert ref["status"] == 0
    if ctx is None:
        ctx = Context(mdl.basis, mdl.ham)
    ctx.set_gemm_mode(gemm_mode)
    p, H = ctx.project(U, V, Mphi, Mphi, 2 * math.pi, Z, N)
    rp = ref["pnp"]
    assert (p.nocc, p.nemp) == (rp.nocc, rp.nemp)
    assert abs((p.c("ener") / p.c("over")).real - (rp.c("ener") / rp.c("over")).real) < 1e-9
    for k in ("prot", "neut", "prot2", "neut2"):
        assert abs((p.c(k) / p.c("over")).real - (rp.c(k) / rp.c("over")).real) < 1e-10, k
    assert abs(p.c("over") - rp.c("over")) < 1e-10 * abs(rp.c("over"))
    assert np.abs(H - ref["H20v"]).max() < 1e-9 * np.abs(ref["H20v"]).max()
    return ctx


@pytest.mark.parametrize("gemm_mode", [0, 2])
def test_spherical_bcs_sd(gemm_mode):
    mdl = M.sd_model(seed=2)
    U, V = M.spherical_seed(mdl.basis, 4, 4, seed=1)
    check(mdl, U, V, 9, 4, 4, gemm_mode)


@pytest.fixture(scope="module")
def emax4():
    return M.noncore_model(4, seed=1)


def test_spherical_bcs_emax4(emax4):
    U, V = M.spherical_seed(emax4.basis, 8, 8, seed=4)
    check(emax4, U, V, 7, 8, 8)


def test_slater_determinant_emax4(emax4):
    # closed 0s and 0p shells: every state occupied or empty (nocc = 16)
    U, V = M.spherical_seed(emax4.basis, 8, 8, slater=True)
    check(emax4, U, V, 5, 8, 8)


def test_spherical_iterations_sd():
    # the gradient of a rotation-invariant Hamiltonian keeps the state
    # spherical: the degenerate subspaces stay, iteration after iteration
    # (the canonical basis is warm-started from the previous one)
    mdl = M.sd_model(seed=2)
    n = mdl.n
    U, V = M.spherical_seed(mdl.basis, 4, 4, seed=1)
    om = O.OracleModel(mdl)
    eta, mu = 0.05, 0.3
    ovap = O.OracleVAP(om, U, V, 9, 9, 2 * math.pi, 4, 4, eta, mu, 0.0, np.zeros((0, n * n)), np.zeros(0))
    ctx = Context(mdl.basis, mdl.ham)
    Zim1 = np.zeros(n * n)
    for it in range(4):
        st, info = ovap.iterate()
        assert st == 0
        p, H = ctx.project(U, V, 9, 9, 2 * math.pi, 4, 4)
        assert abs((p.c("ener") / p.c("over")).real - info[1]) < 1e-9, it
        Zi, _ = ctx.calculate_gradient(H, None, None, Zim1, eta, mu)
        U, V = ctx.evolve(U, V, Zi)
        Zim1 = Zi
