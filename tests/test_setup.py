"""Host setup library: basis conventions, interaction build, .red format."""

import os

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.model import _setup_lib


def test_basis_conventions(usdb_model):
    b = usdb_model.basis
    n = b.n
    assert n == 24
    assert list(b.sp_2mt[: n // 2]) == [-1] * (n // 2) and list(b.sp_2mt[n // 2:]) == [1] * (n // 2)
    # within a shell 2m runs from +2j down to -2j (module_basis.f90:209-238)
    assert list(b.sp_2mj[:6]) == [5, 3, 1, -1, -3, -5]
    # time-reversal partner k + 2m carries -m
    for k in range(n):
        t = b.sp_tr[k] - 1
        assert b.sp_2mj[t] == -b.sp_2mj[k] and b.sp_sh[t] == b.sp_sh[k] and b.sp_2mt[t] == b.sp_2mt[k]


def test_clebsch_values():
    L = _setup_lib()
    assert abs(L.tvs_clebsch(1, 1, 2, 1, -1, 0) - np.sqrt(0.5)) < 1e-15
    assert abs(L.tvs_clebsch(1, 1, 0, 1, -1, 0) - np.sqrt(0.5)) < 1e-15
    assert abs(L.tvs_clebsch(5, 5, 0, 5, -5, 0) - 1 / np.sqrt(6)) < 1e-15
    # orthogonality over m1 for fixed j1 j2 J M
    s = sum(L.tvs_clebsch(3, 1, 4, m1, 2 - m1, 2) ** 2 for m1 in (-3, -1, 1, 3))
    assert abs(s - 1.0) < 1e-14


def test_usdb_elements(usdb_model):
    h = usdb_model.ham
    S = h.S
    assert S == 1396
    abcd = h.abcd.reshape(-1, 4).astype(int)
    # storage filters of module_hamiltonian.f90:330-352
    assert np.all(abcd[:, 0] < abcd[:, 1]) and np.all(abcd[:, 2] < abcd[:, 3])
    assert np.all(abcd[:, 0] <= abcd[:, 2])
    b = usdb_model.basis
    m = b.sp_2mj
    assert np.all(m[abcd[:, 0] - 1] + m[abcd[:, 1] - 1] == m[abcd[:, 2] - 1] + m[abcd[:, 3] - 1])
    assert np.all(m[abcd[:, 0] - 1] + m[abcd[:, 1] - 1] >= 0)
    assert set(np.unique(h.trperm)).issubset(set(range(-8, 8)))


def test_red_roundtrip(tmp_path, usdb_model):
    path = str(tmp_path / "usdb.red")
    usdb_model.write_red(path)
    L = _setup_lib()
    h = L.tvs_load_antoine(os.path.join(os.path.dirname(__file__), "golden", "usdb.sho").encode(), 4.0, 4.0)
    assert L.tvs_read_red(h, path.encode()) == 0
    m2 = M._extract(h, 4.0, 4.0)
    assert np.array_equal(m2.ham.abcd, usdb_model.ham.abcd)
    assert np.array_equal(m2.ham.h2, usdb_model.ham.h2)
    assert np.array_equal(m2.ham.trperm, usdb_model.ham.trperm)
    assert np.array_equal(m2.ham.H1, usdb_model.ham.H1)
    size = os.path.getsize(path)
    n, S = usdb_model.n, usdb_model.ham.S
    assert size == 100 + 4 + 16 + 16 * n * n + 8 + 8 * S + 4 * S + S


def test_synthetic_sd_is_hermitian():
    mdl = M.sd_model(seed=5)
    n = mdl.n
    # reconstruct the dense antisymmetrised V_abcd from the stored list and
    # check hermiticity V_abcd = V_cdab through the field contraction: the
    # Gamma field of a hermitian density must be hermitian.
    import oracle as O
    om = O.OracleModel(mdl)
    rng = np.random.default_rng(0)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    rho = A + A.conj().T
    K = rng.normal(size=(n, n)); K = K - K.T
    g, h, dl, dr = om.calculate_fields(rho, K, K)
    assert np.allclose(g, g.conj().T, atol=1e-12 * abs(g).max())


def test_emax_shell_list():
    assert M.shells_up_to(1) == [1, 103, 101]
    assert len(M.shells_up_to(4)) == 15


def test_multipoles_symmetric(usdb_model):
    q = usdb_model.multipoles()
    n = usdb_model.n
    for lam in range(2):
        for t in range(2):
            Q = q[lam, t, 0].reshape(n, n)
            assert np.allclose(Q, Q.T, atol=1e-12)


def test_synthetic_emax4_is_hermitian():
    # the same field check on the emax=4 list of the benchmark (n = 140)
    mdl = M.noncore_model(4, seed=1)
    n = mdl.n
    import oracle as O
    om = O.OracleModel(mdl)
    rng = np.random.default_rng(1)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    rho = A + A.conj().T
    K = rng.normal(size=(n, n)); K = K - K.T
    g, h, dl, dr = om.calculate_fields(rho, K, K)
    assert np.allclose(g, g.conj().T, atol=1e-12 * abs(g).max())


@pytest.mark.parametrize("emax", [2, 4])
def test_synthetic_interaction_is_rotation_and_isospin_invariant(emax):
    # the JT-coupled synthetic interaction is a scalar in angular momentum and
    # isospin: the HFB energy (M = 1) of a state equals that of the state
    # rotated about y, c' = exp(beta Jy) c with the real antisymmetric table
    # of i Jy (set_angular_momentum), and that of the state with protons and
    # neutrons exchanged
    from scipy.linalg import expm

    import oracle as O
    mdl = M.noncore_model(emax, seed=1, valence_Z=4, valence_N=4)
    n, h = mdl.n, mdl.n // 2
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=7)
    om = O.OracleModel(mdl)

    def energy(U_, V_):
        r = om.project(U_, V_, 1, 1, 2 * np.pi, 4, 4)
        assert r["status"] == 0
        p = r["pnp"]
        return (p.c("ener") / p.c("over")).real

    e0 = energy(U, V)
    Jy = np.imag(mdl.observable_operators()["obo"][1])  # the real table: the operator is i Jy
    D = expm(0.7 * Jy)
    assert np.allclose(D.T @ D, np.eye(n), atol=1e-12)
    assert abs(energy(D @ U, D @ V) - e0) < 1e-9 * (1 + abs(e0))
    P = np.zeros((n, n))
    P[np.arange(h), np.arange(h) + h] = 1.0
    P[np.arange(h) + h, np.arange(h)] = 1.0
    assert abs(energy(P @ U, P @ V) - e0) < 1e-9 * (1 + abs(e0))
