"""Device path (libtvap_gpu.so through the C ABI) against the oracle.

Tolerances (the FP64 accuracy the path must keep): fields 1e-12 relative to the largest entry;
projected energy 1e-9 MeV; projected particle numbers 1e-10; the projected
gradient field_H20v 1e-9 relative to its largest entry."""

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-12


def relerr(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def sd():
    mdl = M.sd_model(seed=2)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    return mdl, U, V


@pytest.fixture(scope="module")
def emax2():
    mdl = M.noncore_model(2, seed=5, valence_Z=4, valence_N=4)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=6)
    return mdl, U, V


@pytest.fixture(scope="module")
def emax4():
    mdl = M.noncore_model(4, seed=1)
    U, V = M.random_bogoliubov(mdl.basis, 8, 8, seed=2)
    return mdl, U, V


@pytest.mark.parametrize("case", ["sd", "emax2", "emax4"])
def test_calculate_fields(case, request):
    mdl, U, V = request.getfixturevalue(case)
    om = O.OracleModel(mdl)
    st, (rho, kLR, kRL, _) = om.angle_densities(U, V, 0.7, 2.1)
    assert st == 0
    ref = om.calculate_fields(rho, kLR, kRL, nthreads=1)
    ctx = Context(mdl.basis, mdl.ham)
    got = ctx.calculate_fields(rho, kLR, kRL)
    for g, r, name in zip(got, ref, ("gamma", "h", "deltaLR", "deltaRL")):
        assert relerr(g, r) < FIELD_TOL, name


@pytest.mark.parametrize("case", ["sd", "emax2", "emax4"])
def test_calculate_fields_of_a_real_state_is_fields_diag(case, request):
    # calculate_fields_diag (module_fields.f90:204-317) is the L = R case:
    # the device's general contraction with kappa^RL = kappa^LR = V U^T and
    # rho = V V^T against the oracle's restatement of calculate_fields_diag
    mdl, U, V = request.getfixturevalue(case)
    rho = (V @ V.T).astype(complex)
    kap = (V @ U.T).astype(complex)
    ref = O.OracleModel(mdl).calculate_fields_diag(rho, kap, nthreads=1)
    got = Context(mdl.basis, mdl.ham).calculate_fields(rho, kap, kap)
    for g, r, name in zip(got, ref, ("gamma", "h", "deltaLR", "deltaRL")):
        assert relerr(g, r) < FIELD_TOL, name


def test_calculate_fields_edge_cases(sd):
    mdl, U, V = sd
    ctx = Context(mdl.basis, mdl.ham)
    n = mdl.n
    z = np.zeros((n, n), dtype=complex)
    g, h, dl, dr = ctx.calculate_fields(z, z, z)
    assert np.all(g == 0) and np.all(dl == 0) and np.all(dr == 0)
    assert np.array_equal(h, mdl.ham.H1)
    # an empty element list: fields vanish, h = H1
    empty = M.Hamiltonian(mdl.ham.H0, mdl.ham.H1, np.zeros(0, np.int16), np.zeros(0, np.float32),
                          np.zeros(0, np.int8))
    ctx2 = Context(mdl.basis, empty)
    rng = np.random.default_rng(0)
    r = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    g, h, dl, dr = ctx2.calculate_fields(r, r, r)
    assert np.all(g == 0) and np.all(dl == 0)


def test_calculate_fields_batched(emax2):
    mdl, U, V = emax2
    om = O.OracleModel(mdl)
    angles = [(0.1 * k, 0.37 * k) for k in range(7)]
    sets = [om.angle_densities(U, V, a, b)[1][:3] for a, b in angles]
    rho, kLR, kRL = (np.stack([s[q] for s in sets]) for q in range(3))
    ctx = Context(mdl.basis, mdl.ham)
    got = ctx.calculate_fields_batched(rho, kLR, kRL)
    for c in range(len(angles)):
        ref = om.calculate_fields(rho[c], kLR[c], kRL[c], nthreads=1)
        for q in range(4):
            assert relerr(got[q][c], ref[q]) < FIELD_TOL


@pytest.mark.parametrize("case,ncol", [("emax2", 20), ("emax4", 37)])
def test_calculate_fields_dense_blocks(case, ncol, request):
    # many angle columns take the dense symmetry-block path (FP64 emulated on
    # the tensor cores): against the oracle, and against the gather kernels
    # (FP64 pipe) on every column
    mdl, U, V = request.getfixturevalue(case)
    om = O.OracleModel(mdl)
    angles = [(0.13 * k, 0.29 * k + 0.05) for k in range(ncol)]
    sets = [om.angle_densities(U, V, a, b)[1][:3] for a, b in angles]
    rho, kLR, kRL = (np.stack([s[q] for s in sets]) for q in range(3))
    ctx = Context(mdl.basis, mdl.ham)
    got = ctx.calculate_fields_batched(rho, kLR, kRL)
    ctx.set_gemm_mode(0)
    gathered = ctx.calculate_fields_batched(rho, kLR, kRL)
    for c in range(0, ncol, 6):
        ref = om.calculate_fields(rho[c], kLR[c], kRL[c], nthreads=0)
        for q, name in enumerate(("gamma", "h", "deltaLR", "deltaRL")):
            assert relerr(got[q][c], ref[q]) < FIELD_TOL, (c, name)
    for c in range(ncol):
        for q in range(4):
            assert relerr(got[q][c], gathered[q][c]) < FIELD_TOL, (c, q)


def check_projection(mdl, U, V, Mp, Mn, Z, N, mode, nthreads=0, gemm_mode=2, pairs=None):
    om = O.OracleModel(mdl)
    ref = om.project(U, V, Mp, Mn, 2 * np.pi, Z, N, nthreads=nthreads)
    assert ref["status"] == 0
    ctx = Context(mdl.basis, mdl.ham)
    ctx.set_gemm_mode(gemm_mode)
    if pairs is not None:
        ctx.set_option(Context.OPT_COMPLEX_PAIRS, pairs)
    pnp, H20v = ctx.project(U, V, Mp, Mn, 2 * np.pi, Z, N, mode=mode)
    rp = ref["pnp"]
    e_ref = (rp.c("ener") / rp.c("over")).real
    e_got = (pnp.c("ener") / pnp.c("over")).real
    assert abs(e_got - e_ref) < 1e-9
    for k in ("prot", "neut", "prot2", "neut2"):
        assert abs((pnp.c(k) / pnp.c("over")).real - (rp.c(k) / rp.c("over")).real) < 1e-10, k
    assert abs(pnp.c("over") - rp.c("over")) < 1e-10 * abs(rp.c("over")) + 1e-14
    assert relerr(H20v, ref["H20v"]) < 1e-9
    return pnp, H20v


@pytest.mark.parametrize("gemm_mode", [0, 1, 2])
@pytest.mark.parametrize("mode", [0, 1])
def test_project_sd(sd, mode, gemm_mode):
    mdl, U, V = sd
    check_projection(mdl, U, V, 9, 9, 4, 4, mode, gemm_mode=gemm_mode)


@pytest.mark.parametrize("pairs", [0, 1])
def test_project_sd_complex_forms(sd, pairs):
    # both forms of the complex x complex tcgen05 products
    mdl, U, V = sd
    check_projection(mdl, U, V, 9, 9, 4, 4, 0, pairs=pairs)


@pytest.mark.parametrize("gemm_mode", [0, 1, 2])
def test_project_mg24_usdb(usdb_model, mg24_seed, gemm_mode):
    check_projection(usdb_model, *mg24_seed, 5, 5, 4, 4, 0, gemm_mode=gemm_mode)


def test_project_even_angles(sd):
    mdl, U, V = sd
    check_projection(mdl, U, V, 4, 6, 4, 4, 0)


@pytest.mark.parametrize("grid", [5, 7])
def test_project_emax2(emax2, grid):
    # 7 x 7 angles (25 folded columns) runs the fields on the dense blocks
    mdl, U, V = emax2
    check_projection(mdl, U, V, grid, grid, 4, 4, 0)


@pytest.mark.parametrize("gemm_mode", [0, 1, 2])
def test_project_emax4_small_grid(emax4, gemm_mode):
    mdl, U, V = emax4
    check_projection(mdl, U, V, 3, 3, 8, 8, 0, gemm_mode=gemm_mode)


@pytest.mark.parametrize("pairs", [0, 1])
def test_project_emax4_full_grid(emax4, pairs):
    # the benchmark's workload (n = 140, 15 x 15 angles, 113 folded pairs): the
    # staggered groups of the solve, the reused digit planes and the traces
    # beside H20 all run here, with both forms of the complex products
    mdl, U, V = emax4
    check_projection(mdl, U, V, 15, 15, 8, 8, 0, pairs=pairs)


def test_emulated_gemm_matches_fp64_pipe(emax4):
    # the two arithmetic modes of the dense products agree to FP64 rounding
    mdl, U, V = emax4
    ctx = Context(mdl.basis, mdl.ham)
    res = []
    for gm, pairs in ((0, 0), (1, 0), (2, 0), (2, 1)):
        ctx.set_gemm_mode(gm)
        ctx.set_option(Context.OPT_COMPLEX_PAIRS, pairs)
        res.append(ctx.project(U, V, 5, 5, 2 * np.pi, 8, 8))
    p0, h0 = res[0]
    e0 = (p0.c("ener") / p0.c("over")).real
    for p1, h1 in res[1:]:
        e1 = (p1.c("ener") / p1.c("over")).real
        assert abs(e0 - e1) < 1e-10 * max(1.0, abs(e0))
        assert relerr(h1, h0) < 1e-11


def test_plain_equals_batched(emax2):
    mdl, U, V = emax2
    ctx = Context(mdl.basis, mdl.ham)
    p0, h0 = ctx.project(U, V, 7, 7, 2 * np.pi, 4, 4, mode=0)
    p1, h1 = ctx.project(U, V, 7, 7, 2 * np.pi, 4, 4, mode=1)
    assert abs(p0.c("ener") / p0.c("over") - p1.c("ener") / p1.c("over")) < 1e-10
    assert relerr(h0, h1) < 1e-10


def test_gradient_and_evolve(sd):
    mdl, U, V = sd
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    rng = np.random.default_rng(3)
    H = rng.normal(size=n * n)
    Zm = rng.normal(size=n * n)
    C = rng.normal(size=(2, n * n))
    lam = np.array([0.3, -1.2])
    Zi, norm = ctx.calculate_gradient(H, lam, C, Zm, 0.05, 0.6)
    ref = -0.05 * (H - lam @ C) + 0.6 * Zm
    assert np.abs(Zi - ref).max() < 1e-14 * np.abs(ref).max() * 10
    assert abs(norm - np.linalg.norm(ref) / 0.05) < 1e-12 * norm
    Z = 0.1 * rng.normal(size=(n, n))
    Z = Z - Z.T
    U1, V1 = ctx.evolve(U, V, Z)
    st, U1r, V1r = O.thouless_evolve(U, V, Z)
    assert st == 0
    assert np.abs(U1 - U1r).max() < 1e-12 and np.abs(V1 - V1r).max() < 1e-12


def test_energy_adjoint(sd):
    mdl, U, V = sd
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    rng = np.random.default_rng(4)
    Z = 0.1 * rng.normal(size=(n, n))
    Z = Z - Z.T
    E, G = ctx.energy_adjoint(U, V, Z, 5, 5, 2 * np.pi, 4, 4)
    D = rng.normal(size=(n, n))
    D = D - D.T
    h = 1e-5
    Ep, _ = ctx.energy_adjoint(U, V, Z + h * D, 5, 5, 2 * np.pi, 4, 4)
    Em, _ = ctx.energy_adjoint(U, V, Z - h * D, 5, 5, 2 * np.pi, 4, 4)
    fd = (Ep - Em) / (2 * h)
    assert abs(fd - (G * D).sum()) < 1e-6 * max(1.0, abs(fd))
    # at Z = 0 the adjoint is module_gradient's analytic gradient field_H20v
    E0, G0 = ctx.energy_adjoint(U, V, np.zeros((n, n)), 5, 5, 2 * np.pi, 4, 4)
    om = O.OracleModel(mdl)
    ref = om.project(U, V, 5, 5, 2 * np.pi, 4, 4, nthreads=1)
    assert relerr(G0.reshape(-1, order="F"), ref["H20v"]) < 1e-9


def test_warm_started_canonical_basis(emax4):
    # successive projections in one context refine the previous canonical
    # basis instead of re-diagonalising; results must still match the oracle
    mdl, U, V = emax4
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    om = O.OracleModel(mdl)
    rng = np.random.default_rng(9)
    for step in range(3):
        pnp, H20v = ctx.project(U, V, 3, 3, 2 * np.pi, 8, 8)
        ref = om.project(U, V, 3, 3, 2 * np.pi, 8, 8)
        e_got = (pnp.c("ener") / pnp.c("over")).real
        e_ref = (ref["pnp"].c("ener") / ref["pnp"].c("over")).real
        assert abs(e_got - e_ref) < 1e-9, step
        assert relerr(H20v, ref["H20v"]) < 1e-9, step
        Z = 1e-3 * rng.normal(size=(n, n))
        Z = Z - Z.T
        U, V = ctx.evolve(U, V, Z)


def test_autograd_function_matches_finite_differences(sd):
    torch = pytest.importorskip("torch")
    from taurus_vap_gb300.autograd import projected_energy

    mdl, U, V = sd
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    rng = np.random.default_rng(12)
    Z0 = 0.05 * rng.normal(size=(n, n))
    Z0 = Z0 - Z0.T
    # the Thouless matrix enters in Fortran order: pass Z as the (n, n) array
    # whose [i, j] is Z(i, j)
    Z = torch.tensor(Z0, dtype=torch.float64, requires_grad=True)
    E = projected_energy(Z, ctx, U, V, 5, 5, 4, 4)
    E.backward()
    D = rng.normal(size=(n, n))
    D = D - D.T
    h = 1e-5
    Ep = projected_energy(torch.tensor(Z0 + h * D), ctx, U, V, 5, 5, 4, 4).item()
    Em = projected_energy(torch.tensor(Z0 - h * D), ctx, U, V, 5, 5, 4, 4).item()
    fd = (Ep - Em) / (2 * h)
    assert abs(fd - float((Z.grad.numpy() * D).sum())) < 1e-6 * max(1.0, abs(fd))


def test_project_batched_states(sd):
    # several states of one basis in one call: each agrees with its own
    # single projection (to rounding: the canonical basis is warm-started
    # from the previous state's), and with the oracle for one of them
    mdl, U, V = sd
    states = [(U, V)] + [M.random_bogoliubov(mdl.basis, 4, 4, seed=s) for s in (11, 12)]
    opts = [dict(Mphip=9, Mphin=9, facpi=2 * np.pi, valence_Z=4, valence_N=4),
            dict(Mphip=7, Mphin=5, facpi=2 * np.pi, valence_Z=4, valence_N=4),
            dict(Mphip=9, Mphin=9, facpi=2 * np.pi, valence_Z=4, valence_N=4, mode=1)]
    ctx = Context(mdl.basis, mdl.ham)
    got = ctx.project_batched([s[0] for s in states], [s[1] for s in states], opts)
    for (Us, Vs), o, (pnp, H20v) in zip(states, opts, got):
        p1, h1 = ctx.project(Us, Vs, o["Mphip"], o["Mphin"], o["facpi"], o["valence_Z"], o["valence_N"],
                             mode=o.get("mode", 0))
        assert abs(pnp.c("ener") / pnp.c("over") - p1.c("ener") / p1.c("over")) < 1e-12
        assert abs(pnp.c("over") - p1.c("over")) < 1e-12 * abs(p1.c("over"))
        assert relerr(H20v, h1) < 1e-12
    om = O.OracleModel(mdl)
    ref = om.project(states[1][0], states[1][1], 7, 5, 2 * np.pi, 4, 4)
    e_ref = (ref["pnp"].c("ener") / ref["pnp"].c("over")).real
    assert abs((got[1][0].c("ener") / got[1][0].c("over")).real - e_ref) < 1e-9
    assert relerr(got[1][1], ref["H20v"]) < 1e-9
