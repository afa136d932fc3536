"""tvap_evolve_noalloc: the Thouless evolution for callers that cannot
allocate device memory (its buffers live in a fixed array inside the library).
Its results must equal those of tvap_evolve, call after call.  This file is
collected last so that a failure here leaves every other test already run."""

import ctypes

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300 import native as N

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.tensor(np.asarray(a, dtype=np.float64).reshape(-1, order="F"), device="cuda")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_evolve_noalloc_matches_evolve_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    mdl = M.sd_model(seed=2)
    n = mdl.n
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    ctx = N.Context(mdl.basis, mdl.ham)
    rng = np.random.default_rng(21)
    dU, dV = _dev(torch, U), _dev(torch, V)
    for call in range(2):  # the shared array keeps the previous call's contents
        Z = 0.1 * rng.normal(size=(n, n))
        Z = Z - Z.T
        U1_ref, V1_ref = ctx.evolve(U, V, Z)
        dZ = _dev(torch, Z)
        dU1 = torch.empty(n * n, dtype=torch.float64, device="cuda")
        dV1 = torch.empty_like(dU1)
        torch.cuda.synchronize()
        rc = N.lib().tvap_evolve_noalloc(ctx.h, _ptr(dU), _ptr(dV), _ptr(dZ), _ptr(dU1), _ptr(dV1))
        assert rc == 0, N.lib().tvap_last_error()
        torch.cuda.synchronize()
        U1 = dU1.cpu().numpy().reshape(n, n, order="F")
        V1 = dV1.cpu().numpy().reshape(n, n, order="F")
        assert np.abs(U1 - U1_ref).max() < 1e-12, call
        assert np.abs(V1 - V1_ref).max() < 1e-12, call


def _basis_of_size(n):
    # the evolution reads no single-particle table: a basis of the right size
    return M.Basis(np.zeros(1, np.int32), *[np.zeros(n, np.int32) for _ in range(5)],
                   np.ones(n, np.int32), np.arange(1, n + 1, dtype=np.int32), 0.0, 0.0)


@pytest.mark.parametrize("n", [224, 336])
def test_evolve_noalloc_large_bases(n):
    # n = 224 (emax=5) and n = 336 (emax=6, the array's limit): the Cholesky
    # factor no longer fits shared memory, so the global-memory factorisation
    # runs.  Against tvap_evolve and the closed form (U0 + V0 Z) L^-T,
    # (V0 + U0 Z) L^-T with L L^T = 1 + Z^T Z, two calls in a row.
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    ctx = N.Context(_basis_of_size(n))
    rng = np.random.default_rng(n)
    U = np.linalg.qr(rng.normal(size=(n, n)))[0]
    V = 0.3 * np.linalg.qr(rng.normal(size=(n, n)))[0]
    dU, dV = _dev(torch, U), _dev(torch, V)
    for call in range(2):
        Z = 0.1 * rng.normal(size=(n, n))
        Z = Z - Z.T
        L = np.linalg.cholesky(np.eye(n) + Z.T @ Z)
        U1_cf = np.linalg.solve(L, (U + V @ Z).T).T
        V1_cf = np.linalg.solve(L, (V + U @ Z).T).T
        U1_ref, V1_ref = ctx.evolve(U, V, Z)
        dZ = _dev(torch, Z)
        dU1 = torch.empty(n * n, dtype=torch.float64, device="cuda")
        dV1 = torch.empty_like(dU1)
        torch.cuda.synchronize()
        rc = N.lib().tvap_evolve_noalloc(ctx.h, _ptr(dU), _ptr(dV), _ptr(dZ), _ptr(dU1), _ptr(dV1))
        assert rc == 0, N.lib().tvap_last_error()
        torch.cuda.synchronize()
        U1 = dU1.cpu().numpy().reshape(n, n, order="F")
        V1 = dV1.cpu().numpy().reshape(n, n, order="F")
        for got in ((U1, V1), (U1_ref, V1_ref)):
            assert np.abs(got[0] - U1_cf).max() < 1e-12, (call, n)
            assert np.abs(got[1] - V1_cf).max() < 1e-12, (call, n)
        assert np.abs(U1 - U1_ref).max() < 1e-12 and np.abs(V1 - V1_ref).max() < 1e-12


def test_evolve_noalloc_rejects_host_memory_and_large_bases():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    mdl = M.sd_model(seed=2)
    n = mdl.n
    ctx = N.Context(mdl.basis, mdl.ham)
    host = np.zeros(n * n)
    p = host.ctypes.data_as(ctypes.c_void_p)
    rc = N.lib().tvap_evolve_noalloc(ctx.h, p, p, p, p, p)
    assert rc == 1 and b"device memory" in N.lib().tvap_last_error()
    # a basis above the array's limit (n = 400) is refused before any work
    big = 400
    ctx_big = N.Context(_basis_of_size(big))
    d = torch.zeros(big * big, dtype=torch.float64, device="cuda")
    rc = N.lib().tvap_evolve_noalloc(ctx_big.h, _ptr(d), _ptr(d), _ptr(d), _ptr(d), _ptr(d))
    assert rc == 1 and b"n > 336" in N.lib().tvap_last_error()
