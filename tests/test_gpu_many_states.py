"""Many independent states: odd number parity (one blocked quasiparticle,
block_quasiparticle, module_wavefunctions.f90:959-984) against the oracle,
and tvap_iterate_many (states of several contexts, bases of different sizes,
running concurrently) against the same iterations made one state at a time.

Tolerances: projected energy 1e-9 MeV and field_H20v 1e-9 of its largest
entry against the oracle; 1e-11 between the concurrent and the single-state
iterations (the same arithmetic; only the warm start of the canonical basis
differs)."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context, iterate_many

import oracle as O

pytestmark = pytest.mark.gpu


def energy(p):
    return (p.c("ener") / p.c("over")).real


@pytest.mark.parametrize("case", ["sd", "emax2", "emax4"])
def test_blocked_odd_state(case):
    if case == "sd":
        mdl, Z, N, Mp = M.sd_model(seed=2), 5, 4, 9
    elif case == "emax2":
        mdl, Z, N, Mp = M.noncore_model(2, seed=5, valence_Z=5, valence_N=4), 5, 4, 7
    else:
        mdl, Z, N, Mp = M.noncore_model(4, seed=1, valence_Z=9, valence_N=8), 9, 8, 5
    U, V = M.random_bogoliubov(mdl.basis, Z, N, seed=3, block=3)
    ref = O.OracleModel(mdl).project(U, V, Mp, Mp, 2 * math.pi, Z, N)
    assert ref["status"] == 0
    ctx = Context(mdl.basis, mdl.ham)
    p, H = ctx.project(U, V, Mp, Mp, 2 * math.pi, Z, N)
    assert (p.nocc, p.nemp) == (ref["pnp"].nocc, ref["pnp"].nemp)
    assert abs(energy(p) - energy(ref["pnp"])) < 1e-9
    assert np.abs(H - ref["H20v"]).max() < 1e-9 * np.abs(ref["H20v"]).max()


def test_iterate_many_uneven_bases():
    sd = M.sd_model(seed=2)
    e2 = M.noncore_model(2, seed=5, valence_Z=4, valence_N=4)
    sd_ctx = [Context(sd.basis, sd.ham) for _ in range(3)]
    e2_ctx = Context(e2.basis, e2.ham)
    states, ctxs, opts = [], [], []
    for k in range(6):  # mixed number parity on the sd space
        odd = k % 2 == 1
        Z = 5 if odd else 4
        states.append(M.random_bogoliubov(sd.basis, Z, 4, seed=10 + k, block=3 if odd else 0))
        ctxs.append(sd_ctx[k % 3])
        opts.append(dict(Mphip=9, Mphin=9, facpi=2 * math.pi, valence_Z=Z, valence_N=4))
    for k in range(3):
        states.append(M.random_bogoliubov(e2.basis, 4, 4, seed=20 + k))
        ctxs.append(e2_ctx)
        opts.append(dict(Mphip=7, Mphin=7, facpi=2 * math.pi, valence_Z=4, valence_N=4))
    ns = len(states)
    eta, mu = [0.02] * ns, [0.3] * ns
    U = [s[0] for s in states]
    V = [s[1] for s in states]
    Zm = [np.zeros(c.n * c.n) for c in ctxs]
    # the same iterations one state at a time, each on a context of its own
    single = [Context(sd.basis, sd.ham) if c is not e2_ctx else Context(e2.basis, e2.ham) for c in ctxs]
    Us, Vs, Zs = list(U), list(V), list(Zm)
    for it in range(2):
        res = iterate_many(ctxs, U, V, Zm, opts, eta, mu)
        for s in range(ns):
            o = opts[s]
            p1, Z1, g1, U1, V1 = single[s].iterate(Us[s], Vs[s], Zs[s], o["Mphip"], o["Mphin"], o["facpi"],
                                                  o["valence_Z"], o["valence_N"], eta[s], mu[s])
            p, Zi, g, Un, Vn = res[s]
            assert abs(energy(p) - energy(p1)) < 1e-11, (it, s)
            assert np.abs(Un - U1).max() < 1e-11 and np.abs(Vn - V1).max() < 1e-11, (it, s)
            assert abs(g - g1) < 1e-11 * g1
            U[s], V[s], Zm[s] = Un, Vn, Zi
            Us[s], Vs[s], Zs[s] = U1, V1, Z1
    # one odd state of the batch against the oracle
    s = 1
    ref = O.OracleModel(sd).project(U[s], V[s], 9, 9, 2 * math.pi, 5, 4)
    p, _ = single[s].project(U[s], V[s], 9, 9, 2 * math.pi, 5, 4)
    assert abs(energy(p) - energy(ref["pnp"])) < 1e-9
