"""Failure paths, the Pfaffian and the emulated products on the device, each
against the oracle through the C ABI.

- failures made on the host: a canonical pair with u = v = 0 (U_phi exactly
  singular at every angle, module_projection.f90:700-702), a non-integer
  valence number (the projected gradient gets an imaginary part and the
  reference stops, module_projection.f90:751-755), non-finite entries in the
  state, a grid-wide wait that is never released;
- the half-circle projection (proj_facpi = pi) of a state with good proton
  and neutron number parities, and a strongly cancelling Fomenko sum
  (projection on Z = 3 of a state with <Z> = 4: pnp_over ~ 1e-5 of the
  summed magnitudes), in all three arithmetic modes;
- ZSKPFA (subroutines_pfaffian.f:12-258) directly: random complex skew
  matrices in both kernels (packed upper triangle in shared memory up to
  n = 164, global memory above), odd order, a zero column, the sign under a
  row/column exchange, Pf^2 = det;
- the emulated products against their documented bound
  |C - AB|_ij <= 2^-49 K a_i b_j (real), 2^-46 K a_i b_j (complex), with rows
  whose entries span twelve orders of magnitude.
"""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context, TvapError

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sd():
    mdl = M.sd_model(seed=2)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    return mdl, U, V


def energy(p):
    return (p.c("ener") / p.c("over")).real


# ---------------------------------------------------------------------------
# failures
# ---------------------------------------------------------------------------
def test_singular_uphi_is_reported(sd):
    # one canonical pair zeroed in U and V (no quasiparticle mixing after it):
    # rho and kappa are those of a valid state with that pair empty, so the
    # canonical basis and the overlap are regular, while U_phi has two zero
    # rows at every angle.  The oracle's zgetrf in calculate_thouless
    # (module_projection.f90:700-702) reports the zero pivot (its status 20;
    # the reference itself does not check that info); the device reports the
    # singular U_phi.
    mdl, U, V = sd
    U2, V2 = M.random_bogoliubov(mdl.basis, 4, 4, seed=3, zero_pair=3)
    ref = O.OracleModel(mdl).project(U2, V2, 9, 9, 2 * math.pi, 4, 4)
    assert ref["status"] == 20
    ctx = Context(mdl.basis, mdl.ham)
    with pytest.raises(TvapError) as e:
        ctx.project(U2, V2, 9, 9, 2 * math.pi, 4, 4)
    assert e.value.code == 10
    # the context stays usable
    p, _ = ctx.project(U, V, 9, 9, 2 * math.pi, 4, 4)
    assert abs(energy(p) - energy(O.OracleModel(mdl).project(U, V, 9, 9, 2 * math.pi, 4, 4)["pnp"])) < 1e-9


def test_imaginary_gradient_is_reported(sd):
    mdl, U, V = sd
    ref = O.OracleModel(mdl).project(U, V, 9, 9, 2 * math.pi, 4.5, 4)
    assert ref["status"] == 30  # the oracle's code for the reference's stop
    ctx = Context(mdl.basis, mdl.ham)
    with pytest.raises(TvapError) as e:
        ctx.project(U, V, 9, 9, 2 * math.pi, 4.5, 4)
    assert e.value.code == 13


def test_nonfinite_state_is_rejected(sd):
    torch = pytest.importorskip("torch")
    mdl, U, V = sd
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    U2 = U.copy(order="F")
    U2[5, 7] = np.nan
    with pytest.raises(TvapError) as e:
        ctx.project(U2, V, 9, 9, 2 * math.pi, 4, 4)
    assert e.value.code == 1 and "U0" in str(e.value)
    # device memory: an infinity in V0
    V2 = V.copy(order="F")
    V2[0, 11] = np.inf
    dU = torch.tensor(U.reshape(-1, order="F"), device="cuda")
    dV = torch.tensor(V2.reshape(-1, order="F"), device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(TvapError) as e:
        ctx.project(dU, dV, 9, 9, 2 * math.pi, 4, 4)
    assert e.value.code == 1 and "V0" in str(e.value)
    p, _ = ctx.project(U, V, 9, 9, 2 * math.pi, 4, 4)
    assert np.isfinite(energy(p))
    assert n == 24


def test_bounded_wait_runs_out_and_context_stays_usable(sd):
    # one CTA of the cooperative evolution leaves before the first grid
    # barrier; the others' bounded waits run out, the call reports the
    # timeout, and the next calls on the same context are correct
    from taurus_vap_gb300 import native as N

    mdl, U, V = sd
    n = mdl.n
    ctx = Context(mdl.basis, mdl.ham)
    rng = np.random.default_rng(8)
    Z = 0.1 * rng.normal(size=(n, n))
    Z = Z - Z.T
    U1, V1 = ctx.evolve(U, V, Z)
    assert N.lib().tvap_test_wait_timeout(ctx.h) == 0
    with pytest.raises(TvapError) as e:
        ctx.evolve(U, V, Z)
    assert e.value.code == 19
    U2, V2 = ctx.evolve(U, V, Z)
    assert np.array_equal(U1, U2) and np.array_equal(V1, V2)
    st, U1r, V1r = O.thouless_evolve(U, V, Z)
    assert np.abs(U2 - U1r).max() < 1e-12 and np.abs(V2 - V1r).max() < 1e-12
    p, _ = ctx.project(U, V, 9, 9, 2 * math.pi, 4, 4)
    assert abs(energy(p) - energy(O.OracleModel(mdl).project(U, V, 9, 9, 2 * math.pi, 4, 4)["pnp"])) < 1e-9


# ---------------------------------------------------------------------------
# projections that stress the FP64 accuracy
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("gemm_mode", [0, 1, 2])
def test_half_circle_projection(gemm_mode):
    mdl = M.sd_model(seed=2)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3, mix_isospin=False)
    ref = O.OracleModel(mdl).project(U, V, 9, 9, math.pi, 4, 4)
    assert ref["status"] == 0
    ctx = Context(mdl.basis, mdl.ham)
    ctx.set_gemm_mode(gemm_mode)
    p, H = ctx.project(U, V, 9, 9, math.pi, 4, 4)
    assert abs(energy(p) - energy(ref["pnp"])) < 1e-9
    assert np.abs(H - ref["H20v"]).max() < 1e-9 * np.abs(ref["H20v"]).max()


@pytest.mark.parametrize("gemm_mode", [0, 1, 2])
def test_strongly_cancelling_fomenko_sum(sd, gemm_mode):
    # projection on Z = 3 of a state with <Z> = 4: the weighted per-angle
    # overlaps cancel to ~2e-6 of their summed magnitude.  The error allowed
    # in E is the FP64 error carried through that cancellation:
    # 1e-12 sum_phi |w||o_phi| (|E_phi| + |E|) / |pnp_over|.
    mdl, U, V = sd
    om = O.OracleModel(mdl)
    ref = om.project(U, V, 9, 9, 2 * math.pi, 3, 4, want_angles=True)
    assert ref["status"] == 0
    rp = ref["pnp"]
    E = energy(rp)
    scale = sum(abs(complex(*a.over)) * (abs(complex(*a.ener)) + abs(E)) for a in ref["angles"]) / 81.0
    over_scale = sum(abs(complex(*a.over)) for a in ref["angles"]) / 81.0
    assert scale / abs(rp.c("over")) > 1e5  # the case is strongly cancelling
    ctx = Context(mdl.basis, mdl.ham)
    ctx.set_gemm_mode(gemm_mode)
    p, H = ctx.project(U, V, 9, 9, 2 * math.pi, 3, 4)
    assert abs(p.c("over") - rp.c("over")) < 1e-12 * over_scale
    assert abs(energy(p) - E) < 1e-12 * scale / abs(rp.c("over")) + 1e-9


# ---------------------------------------------------------------------------
# ZSKPFA
# ---------------------------------------------------------------------------
def _skew(rng, m):
    A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    return A - A.T


@pytest.mark.parametrize("m", [2, 8, 64, 140, 200, 282])
def test_zskpfa_matches_oracle(sd, m):
    mdl, _, _ = sd
    ctx = Context(mdl.basis)
    rng = np.random.default_rng(m)
    A = np.stack([_skew(rng, m) / math.sqrt(m) for _ in range(3)])
    got = ctx.zskpfa_batched(A)
    for q in range(3):
        ref, info = O.pfaffian(A[q])
        assert info == 0
        assert abs(got[q] - ref) < 1e-11 * abs(ref), (m, q)
        # Pf^2 = det
        sign, logdet = np.linalg.slogdet(A[q])
        assert abs(got[q] ** 2 / (sign * np.exp(logdet)) - 1.0) < 1e-9


@pytest.mark.parametrize("m", [40, 200])  # the unblocked and the blocked form
def test_zskpfa_identities(sd, m):
    mdl, _, _ = sd
    ctx = Context(mdl.basis)
    rng = np.random.default_rng(5)
    A = _skew(rng, m) / math.sqrt(m)
    # a row/column exchange flips the sign
    P = np.eye(m)
    P[[3, 29]] = P[[29, 3]]
    B = P @ A @ P.T
    # a zero column (and row): Pf = 0 from the zero pivot, status OK
    Z = A.copy()
    Z[:, 17] = 0
    Z[17, :] = 0
    # Pf(C A C^T) = det(C) Pf(A)
    C = np.eye(m) + (0.1 / math.sqrt(m / 40)) * (rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m)))
    D = C @ A @ C.T
    pa, pb, pz, pd = ctx.zskpfa_batched(np.stack([A, B, Z, D]))
    assert abs(pb + pa) < 1e-11 * abs(pa)
    assert pz == 0
    assert abs(pd - np.linalg.det(C) * pa) < 1e-10 * abs(pd)
    # odd order: 0 (A not referenced); order 0: 1
    assert ctx.zskpfa_batched(_skew(rng, 7)[None])[0] == 0
    assert ctx.zskpfa_batched(np.zeros((2, 0, 0)))[0] == 1


# ---------------------------------------------------------------------------
# emulated products against their documented bound
# ---------------------------------------------------------------------------
def _wide_rows(rng, m, k, cplx):
    # entries of each row spread over 12 decades, rows scaled over 12 more
    mag = 10.0 ** (-12.0 * rng.random((m, k))) * 10.0 ** (-12.0 * rng.random((m, 1)))
    X = rng.normal(size=(m, k)) * mag
    if cplx:
        X = X + 1j * rng.normal(size=(m, k)) * mag
    return X


@pytest.mark.parametrize("cplx,pairs", [(False, 0), (True, 0), (True, 1)])
@pytest.mark.parametrize("gemm_mode", [1, 2])
def test_emulated_product_bound(sd, cplx, pairs, gemm_mode):
    mdl, _, _ = sd
    ctx = Context(mdl.basis)
    ctx.set_gemm_mode(gemm_mode)
    ctx.set_option(Context.OPT_COMPLEX_PAIRS, pairs)
    rng = np.random.default_rng(17 + gemm_mode)
    m, n, k = 2048, 2048, 256  # 512 output tiles: the tcgen05 kernel in mode 2
    A = _wide_rows(rng, m, k, cplx)
    B = _wide_rows(rng, n, k, cplx).T.copy()  # columns of B spread likewise
    C = ctx.gemm(A, B)
    ref = A @ B
    part = lambda X: np.maximum(np.abs(X.real), np.abs(X.imag)) if cplx else np.abs(X)
    a = part(A).max(axis=1)
    b = part(B).max(axis=0)
    bound = (2.0 ** -46 if cplx else 2.0 ** -49) * k * np.outer(a, b)
    # the FP64 reference's own error, and the final rounding of C
    slack = 2.0 ** -50 * k * (np.abs(A) @ np.abs(B)) + 2.0 ** -52 * np.abs(ref)
    err = np.abs(C - ref)
    assert np.all(err <= bound + slack), float((err / (bound + slack)).max())
    # the FP64 pipe (mode 0) meets the per-term FP64 bound
    ctx.set_gemm_mode(0)
    C0 = ctx.gemm(A, B)
    assert np.all(np.abs(C0 - ref) <= 2.0 ** -49 * k * (np.abs(A) @ np.abs(B)) + 1e-300)


@pytest.mark.parametrize("shape,ta,tb,alpha,beta", [((1533, 1037, 141), "C", "T", -1.0, 0.5),
                                                    ((999, 1501, 77), "N", "C", 0.75, -2.0),
                                                    ((1200, 640, 300), "T", "N", 1.0, 1.0)])
def test_complex_product_forms(sd, shape, ta, tb, alpha, beta):
    # odd sizes, transposed and conjugated operands, alpha = -1 (the sign in the
    # integer conversion), a general alpha and beta (each product > 152
    # tiles): the paired form of the complex x complex tcgen05 products gives
    # the bits of the real representation, within the bound
    mdl, _, _ = sd
    ctx = Context(mdl.basis)
    rng = np.random.default_rng(41)
    m, n, k = shape
    A = _wide_rows(rng, m, k, True)
    B = _wide_rows(rng, n, k, True).T.copy()
    # op(Ain) = A, op(Bin) = B
    Ain = {"N": A, "T": A.T.copy(), "C": A.conj().T.copy()}[ta]
    Bin = {"N": B, "T": B.T.copy(), "C": B.conj().T.copy()}[tb]
    C0 = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
    got = []
    for min_k in (0, 1, k, k + 1):  # none, every product, this K, above this K
        ctx.set_option(Context.OPT_COMPLEX_PAIRS, min_k)
        assert ctx.option(Context.OPT_COMPLEX_PAIRS) == min_k
        got.append(ctx.gemm(Ain, Bin, ta, tb, alpha, beta, C0))
    for C in got[1:]:
        assert np.array_equal(C, got[0])
    ref = alpha * (A @ B) + beta * C0
    part = lambda X: np.maximum(np.abs(X.real), np.abs(X.imag))
    bound = abs(alpha) * 2.0 ** -46 * k * np.outer(part(A).max(axis=1), part(B).max(axis=0))
    slack = 2.0 ** -50 * k * abs(alpha) * (np.abs(A) @ np.abs(B)) + 2.0 ** -51 * (np.abs(ref) + abs(beta * C0))
    err = np.abs(got[0] - ref)
    assert np.all(err <= bound + slack), float((err / (bound + slack)).max())
