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
    b = M.Basis(np.zeros(1, np.int32), *[np.zeros(big, np.int32) for _ in range(5)],
                np.ones(big, np.int32), np.arange(1, big + 1, dtype=np.int32), 0.0, 0.0)
    ctx_big = N.Context(b)
    d = torch.zeros(big * big, dtype=torch.float64, device="cuda")
    rc = N.lib().tvap_evolve_noalloc(ctx_big.h, _ptr(d), _ptr(d), _ptr(d), _ptr(d), _ptr(d))
    assert rc == 1 and b"n > 336" in N.lib().tvap_last_error()
