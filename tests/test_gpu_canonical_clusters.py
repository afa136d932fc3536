"""Canonical basis of nearly closed-shell states (construct_canonical_basis,
module_wavefunctions.f90:777-945): five proton and five neutron pairs
occupied to within 1e-7 .. 1e-12 of 1, every other pair within 1e-7 ..
1e-12 of 0, turned by random orthogonal transformations.  The FP32 stage
cannot separate such levels (1 - 1e-9 and 1 - 1e-10 are the same FP32
number), so they form clusters (ten levels near 1, more than the in-kernel
limit of 8) that the FP64 refinement leaves to an exact diagonalisation,
and an FP32 start leaves the first three refinement steps short of the
orthonormality check.  The projection must match the oracle's, with the
refined path accepted (no FP64 Jacobi of the whole matrix).

Tolerances: projected energy 1e-9 MeV, field_H20v 1e-9 of its largest
entry, the projected proton number 1e-10."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu


def nearly_closed_shell_state(emax, seed):
    mdl = M.noncore_model(emax, seed=1, valence_Z=10, valence_N=10)
    n = mdl.n
    rng = np.random.default_rng(seed)
    v2 = []
    for _ in range(2):  # protons, neutrons
        x = 10.0 ** (-rng.uniform(7, 12, n // 4))
        x[:5] = 1.0 - x[:5]
        v2.append(x)
    U, V = M.random_bogoliubov(mdl.basis, 10, 10, seed=seed, v2=np.concatenate(v2))
    return mdl, U, V


@pytest.mark.parametrize("emax", [2, 4])
def test_nearly_closed_shell_projection(emax):
    mdl, U, V = nearly_closed_shell_state(emax, seed=emax)
    w = np.linalg.eigvalsh(V @ V.T)
    assert (w > 1 - 1e-6).sum() == 20 and (w < 1e-6).sum() == mdl.n - 20
    ref = O.OracleModel(mdl).project(U, V, 15, 15, 2 * math.pi, 10, 10)
    assert ref["status"] == 0
    ctx = Context(mdl.basis, mdl.ham)
    ctx.set_timing(False)  # resets the counters
    p, H = ctx.project(U, V, 15, 15, 2 * math.pi, 10, 10)
    r = ref["pnp"]
    assert abs((p.c("ener") / p.c("over")).real - (r.c("ener") / r.c("over")).real) < 1e-9
    # the 1e-8 occupancy cutoff moves <Z> off its projected value by ~1e-7 in
    # the reference's algorithm as well: compared with the oracle's
    assert abs((p.c("prot") / p.c("over")).real - (r.c("prot") / r.c("over")).real) < 1e-10
    assert np.abs(H - ref["H20v"]).max() < 1e-9 * np.abs(ref["H20v"]).max()
    paths = ctx.canonical_paths()
    assert paths[1] >= 1 and paths[2] == 0, paths  # accepted, no FP64 Jacobi of the whole matrix
