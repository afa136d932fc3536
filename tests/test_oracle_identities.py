"""Identities the reference relies on, checked on the oracle."""

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
import oracle as O


def random_skew(n, rng):
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return A - A.T


@pytest.mark.parametrize("n", [2, 4, 10, 30, 64])
def test_pfaffian_squared_is_det(n):
    rng = np.random.default_rng(n)
    A = random_skew(n, rng)
    pf, info = O.pfaffian(A)
    assert info == 0
    d = np.linalg.det(A)
    assert abs(pf * pf - d) <= 1e-10 * abs(d)


def test_pfaffian_block_diagonal_sign():
    # Pf of diag blocks [[0, a],[-a, 0]] is the product of the a's
    a = [1.5, -2.0, 0.25]
    n = 2 * len(a)
    A = np.zeros((n, n), dtype=complex)
    for k, x in enumerate(a):
        A[2 * k, 2 * k + 1] = x
        A[2 * k + 1, 2 * k] = -x
    pf, _ = O.pfaffian(A)
    assert abs(pf - np.prod(a)) < 1e-15
    # a single exchange of two rows/columns flips the sign
    P = np.eye(n)[[0, 2, 1, 3, 4, 5]]
    pf2, _ = O.pfaffian(P @ A @ P.T)
    assert abs(pf2 + np.prod(a)) < 1e-15


def test_pfaffian_odd_is_zero():
    rng = np.random.default_rng(1)
    pf, _ = O.pfaffian(random_skew(5, rng))
    assert pf == 0


def test_fields_equal_fields_diag_for_same_state():
    # module_projection.f90:267-275: L = R -> calculate_fields == calculate_fields_diag
    mdl = M.sd_model(seed=2)
    om = O.OracleModel(mdl)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    rho = (V @ V.T).astype(complex)
    kap = (V @ U.T).astype(complex)
    g1, h1, d1, dr1 = om.calculate_fields(rho, kap, kap)
    g2, h2, d2, dr2 = om.calculate_fields_diag(rho, kap)
    scale = abs(g1).max()
    assert np.allclose(g1, g2, atol=1e-12 * scale)
    assert np.allclose(d1, d2, atol=1e-12 * abs(d1).max())
    assert np.allclose(d1, -d1.T)


def test_overlap_modulus_matches_onishi():
    # |<Phi|R|Phi>| from the Pfaffian vs sqrt|det(U_phi)| (calculate_norm)
    mdl = M.sd_model(seed=2)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=11)
    n = mdl.n
    for php, phn in [(0.3, 1.1), (2.0, 0.0), (np.pi / 2, np.pi / 3)]:
        o, st = O.overlap(U, V, php, phn)
        assert st == 0
        R = np.diag(np.r_[np.full(n // 2, np.exp(1j * php)), np.full(n // 2, np.exp(1j * phn))])
        Ur, Vr = R @ U, R.conj() @ V
        Uphi = Ur.conj().T @ U + Vr.conj().T @ V
        assert abs(abs(o) - np.sqrt(abs(np.linalg.det(Uphi)))) < 1e-12


def test_projection_particle_number_exact():
    # the projected <Z>, <N> of a number-parity-even state are the valence numbers
    mdl = M.sd_model(seed=2)
    om = O.OracleModel(mdl)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    r = om.project(U, V, 9, 9, 2 * np.pi, 4, 4, nthreads=1)
    p = r["pnp"]
    over = p.c("over")
    assert abs(p.c("prot") / over - 4) < 1e-10
    assert abs(p.c("neut") / over - 4) < 1e-10
    assert abs((p.c("prot2") / over).real - 16) < 1e-9


def test_adjoint_formula_against_finite_differences():
    # dE/dZ = L^-T H20v(Phi(Z)) L^-1  (the relation the device adjoint uses)
    mdl = M.sd_model(seed=3)
    n = mdl.n
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=7)
    om = O.OracleModel(mdl)

    def E(Z):
        st, U1, V1 = O.thouless_evolve(U, V, Z)
        r = om.project(U1, V1, 5, 5, 2 * np.pi, 4, 4, nthreads=1)
        p = r["pnp"]
        return (p.c("ener") / p.c("over")).real, r["H20v"].reshape(n, n, order="F")

    rng = np.random.default_rng(4)
    Z = 0.1 * rng.normal(size=(n, n))
    Z = Z - Z.T
    E0, H = E(Z)
    L = np.linalg.cholesky(np.eye(n) + Z.T @ Z)
    Li = np.linalg.inv(L)
    G = Li.T @ H @ Li
    D = rng.normal(size=(n, n))
    D = D - D.T
    h = 1e-5
    fd = (E(Z + h * D)[0] - E(Z - h * D)[0]) / (2 * h)
    assert abs(fd - (G * D).sum()) < 1e-6 * max(1.0, abs(fd))


# ---------------------------------------------------------------------------
# project_wavefunction with iopt = 1 (the printed observables)
# ---------------------------------------------------------------------------
def _obs_state(emax, Z, N, seed):
    mdl = M.noncore_model(emax, seed=1, valence_Z=Z, valence_N=N)
    U, V = M.random_bogoliubov(mdl.basis, Z, N, seed=seed)
    return mdl, U, V


def test_observables_unprojected_are_plain_traces():
    # M = 1: rho^LR = V V^T, the sums are the expectation values; |<P>| is
    # the Onishi overlap of the state with its parity image (U, V) -> (P U, P V)
    mdl, U, V = _obs_state(2, 4, 4, seed=3)
    ops = mdl.observable_operators()
    om = O.OracleModel(mdl)
    r = om.project_observables(U, V, 1, 1, 2 * np.pi, 4, 4, ops)
    assert r["status"] == 0
    n, h = mdl.n, mdl.n // 2
    rho = V @ V.T
    for k, B in enumerate(ops["obo"]):
        A = B @ rho
        assert abs(r["obo"][k, 0] - np.trace(A[:h, :h])) < 1e-12 * (1 + np.abs(A).max())
        assert abs(r["obo"][k, 1] - np.trace(A[h:, h:])) < 1e-12 * (1 + np.abs(A).max())
    P = np.diag(ops["parity"].astype(float))
    onishi = np.sqrt(abs(np.linalg.det(U.T @ P @ U + V.T @ P @ V)))
    assert abs(abs(r["scal"][6]) - onishi) < 1e-10
    occ = r["occnum"]
    assert abs(occ[:, 0].sum() - np.trace(rho[:h, :h])) < 1e-12
    # <J^2> = sum of its components is j-weighted: positive and at least <J>^2
    J2 = r["sq"].sum().real
    Jv = r["obo"][:3].sum(axis=1)
    assert J2 > 0 and J2 >= np.sum(np.abs(Jv) ** 2) - 1e-9


@pytest.mark.parametrize("emax,M_", [(0, 5), (2, 5)])
def test_observables_projected_identities(emax, M_):
    # the energy of the components equals the projection's energy (two code
    # paths over the same densities and fields), the shell occupations and
    # the trace of pnp_rho add up to the proton number, and with only even-l
    # states (the sd space) the parity-rotated overlaps are the overlaps
    if emax == 0:
        mdl = M.sd_model(seed=2)
        U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=5)
        Z = N = 4
    else:
        mdl, U, V = _obs_state(emax, 4, 4, seed=3)
        Z = N = 4
    ops = mdl.observable_operators()
    om = O.OracleModel(mdl)
    r = om.project_observables(U, V, M_, M_, 2 * np.pi, Z, N, ops)
    ref = om.project(U, V, M_, M_, 2 * np.pi, Z, N)
    assert r["status"] == 0 and ref["status"] == 0
    p = ref["pnp"]
    over = p.c("over")
    s = r["scal"]
    assert abs(s[0] - over) < 1e-12 * abs(over)
    assert abs(s[1] / s[0] - p.c("ener") / over) < 1e-9
    assert abs(s[2] / s[0] - p.c("prot") / over) < 1e-10
    h = mdl.n // 2
    assert abs(r["occnum"][:, 0].sum() - s[2]) < 1e-10 * abs(s[0])
    assert abs(np.trace(r["rho"][:h, :h]) - s[2]) < 1e-10 * abs(s[0])
    if np.all(ops["parity"] == 1):
        assert abs(s[6] - s[0]) < 1e-10 * abs(s[0])
    # the components: energy_p + energy_n = 1b + PH + PP over the blocks
    e = s[7:] / s[0]
    assert abs(e[10] + e[11] - (e[0] + e[1] + e[2:6].sum() + e[6:10].sum())) < 1e-9
