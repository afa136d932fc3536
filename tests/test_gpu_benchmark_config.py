"""Device path against the oracle at the benchmark's own workload: the emax=4
no-core basis (n = 140), Z = N = 8, 15 x 15 gauge angles, FP64.

- iterated parity: five full gradient iterations (projection, gradient,
  Thouless evolution) of the device loop and of the oracle's loop
  (taurus_vap.f90:77-123) from the same seed with the bench's eta and mu:
  projected energy to 1e-9 MeV and the projected gradient field_H20v to 1e-9
  of its largest entry after every iteration, and the device evolution of the
  oracle's own (U, V, Z_i) at n = 140 to 1e-12 against the oracle's
  cholesky_factorization + evolve_wavefunction (module_constraints.f90:497-590);
- the adjoint of E(Z) at a random skew Thouless matrix Z with entries
  ~ N(0, 0.1): against the reference's own analytic gradient at that point
  (field_H20v of the evolved state from the oracle, carried back by
  L^-T . L^-1) to 1e-9, against central finite differences with h = 1e-6
  along random skew directions and single skew pairs, and at Z = 0 against
  the oracle's field_H20v.
"""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu

ETA, MU = 0.005, 0.3  # the bench's gradient step
MPHI = 15


def relerr(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def emax4():
    mdl = M.noncore_model(4, seed=1)
    U, V = M.random_bogoliubov(mdl.basis, 8, 8, seed=2)
    return mdl, U, V


def test_five_iterations_match_oracle(emax4):
    mdl, U0, V0 = emax4
    n = mdl.n
    om = O.OracleModel(mdl)
    ovap = O.OracleVAP(om, U0, V0, MPHI, MPHI, 2 * math.pi, 8, 8, ETA, MU, 0.0, np.zeros((0, n * n)), np.zeros(0))
    ctx = Context(mdl.basis, mdl.ham)
    U, V = np.asfortranarray(U0), np.asfortranarray(V0)
    Zim1 = np.zeros(n * n)
    for it in range(5):
        Ur, Vr, _, _ = ovap.state()
        st, info = ovap.iterate()
        assert st == 0, st
        Un, Vn, Zr, Hr = ovap.state()
        pnp, H20v = ctx.project(U, V, MPHI, MPHI, 2 * math.pi, 8, 8)
        e_dev = (pnp.c("ener") / pnp.c("over")).real
        assert abs(e_dev - info[1]) < 1e-9, (it, e_dev, info[1])
        assert relerr(H20v, Hr) < 1e-9, it
        Zi, gnorm = ctx.calculate_gradient(H20v, None, None, Zim1, ETA, MU)
        assert abs(gnorm - info[0]) < 1e-9 * info[0], it
        # the device evolution of the oracle's own state and step against the
        # oracle's next state
        U1o, V1o = ctx.evolve(Ur, Vr, Zr)
        assert np.abs(U1o - Un).max() < 1e-12 and np.abs(V1o - Vn).max() < 1e-12, it
        U, V = ctx.evolve(U, V, Zi)
        Zim1 = Zi


def _skew(rng, n, scale):
    Z = scale * rng.normal(size=(n, n))
    return Z - Z.T


def test_adjoint_at_random_thouless_matrix(emax4):
    mdl, U, V = emax4
    n = mdl.n
    rng = np.random.default_rng(40)
    Z = _skew(rng, n, 0.1)
    ctx = Context(mdl.basis, mdl.ham)
    args = (MPHI, MPHI, 2 * math.pi, 8, 8)
    E, G = ctx.energy_adjoint(U, V, Z, *args)

    # the reference's analytic gradient at Z: field_H20v of the evolved state
    # (oracle), carried back to Z by dE/dZ = L^-T H20v L^-1, L L^T = 1 + Z^T Z
    om = O.OracleModel(mdl)
    st, U1, V1 = O.thouless_evolve(U, V, Z)
    assert st == 0
    ref = om.project(U1, V1, *args)
    assert ref["status"] == 0
    e_ref = (ref["pnp"].c("ener") / ref["pnp"].c("over")).real
    assert abs(E - e_ref) < 1e-9, (E, e_ref)
    L = np.linalg.cholesky(np.eye(n) + Z.T @ Z)
    Linv = np.linalg.inv(L)
    G_ref = Linv.T @ ref["H20v"].reshape(n, n, order="F") @ Linv
    assert relerr(G, G_ref) < 1e-9

    # central finite differences, h = 1e-6, along skew directions of unit
    # Frobenius norm: three random ones and three single pairs e_ij - e_ji.
    # At this point E is about 3.4e3 MeV and |dE/dZ . D| about 0.2; the
    # oracle's own difference quotient along the first direction agrees with
    # the analytic value to 5e-8, so 2e-5 leaves room for the rounding of E
    # (1e-14 |E| / h = 3e-5 at worst) while still resolving 1e-4 of the slope.
    h = 1e-6
    dirs = []
    for _ in range(3):
        D = _skew(rng, n, 1.0)
        dirs.append(D / np.linalg.norm(D))
    for i, j in ((0, 1), (5, 77), (139, 70)):
        D = np.zeros((n, n))
        D[i, j], D[j, i] = 1.0, -1.0
        dirs.append(D / math.sqrt(2.0))
    tol = 2e-5
    for D in dirs:
        Ep, _ = ctx.energy_adjoint(U, V, Z + h * D, *args)
        Em, _ = ctx.energy_adjoint(U, V, Z - h * D, *args)
        fd = (Ep - Em) / (2 * h)
        an = float((G * D).sum())
        assert abs(fd - an) < tol, (fd, an, tol)

    # one direction also through the oracle's own E(Z)
    D = dirs[0]
    eo = []
    for sgn in (1.0, -1.0):
        st, U1, V1 = O.thouless_evolve(U, V, Z + sgn * h * D)
        r = om.project(U1, V1, *args)
        eo.append((r["pnp"].c("ener") / r["pnp"].c("over")).real)
    assert abs((eo[0] - eo[1]) / (2 * h) - float((G * D).sum())) < tol

    # at Z = 0 the adjoint is module_gradient's gradient field_H20v itself
    E0, G0 = ctx.energy_adjoint(U, V, np.zeros((n, n)), *args)
    ref0 = om.project(U, V, *args)
    assert relerr(G0.reshape(-1, order="F"), ref0["H20v"]) < 1e-9


def test_iterate_matches_oracle_and_three_calls(emax4):
    # tvap_iterate (one host round trip per iteration) against the oracle's
    # loop, and against the same iteration made of tvap_project,
    # tvap_calculate_gradient and tvap_evolve
    mdl, U0, V0 = emax4
    n = mdl.n
    om = O.OracleModel(mdl)
    ovap = O.OracleVAP(om, U0, V0, MPHI, MPHI, 2 * math.pi, 8, 8, ETA, MU, 0.0, np.zeros((0, n * n)), np.zeros(0))
    ctx = Context(mdl.basis, mdl.ham)
    U, V = np.asfortranarray(U0), np.asfortranarray(V0)
    Zim1 = np.zeros(n * n)
    for it in range(3):
        st, info = ovap.iterate()
        assert st == 0
        Un, Vn, Zr, Hr = ovap.state()
        pnp, Zi, gnorm, U1, V1, H = ctx.iterate(U, V, Zim1, MPHI, MPHI, 2 * math.pi, 8, 8, ETA, MU, want_H20v=True)
        assert abs((pnp.c("ener") / pnp.c("over")).real - info[1]) < 1e-9, it
        assert relerr(H, Hr) < 1e-9, it
        assert abs(gnorm - info[0]) < 1e-9 * info[0], it
        assert relerr(Zi, Zr) < 1e-9, it
        assert np.abs(U1 - Un).max() < 1e-11 and np.abs(V1 - Vn).max() < 1e-11, it
        p2, H2 = ctx.project(U, V, MPHI, MPHI, 2 * math.pi, 8, 8)
        Zi2, g2 = ctx.calculate_gradient(H2, None, None, Zim1, ETA, MU)
        U2, V2 = ctx.evolve(U, V, Zi2)
        assert abs(p2.c("ener") - pnp.c("ener")) < 1e-12 * abs(pnp.c("ener"))
        assert np.abs(U2 - U1).max() < 1e-13 and np.abs(V2 - V1).max() < 1e-13, it
        U, V, Zim1 = U1, V1, Zi
