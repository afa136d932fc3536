"""The emax=6 no-core basis (n = 336, 12.9 million stored m-scheme elements,
the size of the uneven-basis configurations' largest member) against the
oracle.  At this n every stage takes its large-basis form: the gather or
dense-block fields over a 52 MB element list, the blocked LU of the Thouless
solve with inverted diagonal blocks (more than 192 rows per panel), the
FP64 Jacobi of the canonical basis, the Pfaffian in global memory and the
Cholesky of the evolution in global memory.

Tolerances as in test_gpu_parity: fields 1e-12 of the largest entry,
projected energy 1e-9 MeV, particle numbers 1e-10, pnp_over 1e-10
relative, field_H20v 1e-9 of its largest entry; evolution 1e-12."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def emax6():
    mdl = M.noncore_model(6, seed=1, valence_Z=10, valence_N=10)
    U, V = M.random_bogoliubov(mdl.basis, 10, 10, seed=7)
    return mdl, U, V, O.OracleModel(mdl), Context(mdl.basis, mdl.ham)


def test_calculate_fields_emax6(emax6):
    mdl, U, V, om, ctx = emax6
    st, (rho, kLR, kRL, _) = om.angle_densities(U, V, 0.7, 2.1)
    assert st == 0
    ref = om.calculate_fields(rho, kLR, kRL, nthreads=0)
    got = ctx.calculate_fields(rho, kLR, kRL)
    for g, r, name in zip(got, ref, ("gamma", "h", "deltaLR", "deltaRL")):
        assert relerr(g, r) < 1e-12, name


@pytest.mark.parametrize("grid", [3, 7])
def test_project_emax6(emax6, grid):
    # 3 x 3: 5 folded angle columns (gather fields); 7 x 7: 25 (dense blocks
    # on the tensor cores when the operator is block-dense)
    mdl, U, V, om, ctx = emax6
    ref = om.project(U, V, grid, grid, 2 * math.pi, 10, 10)
    assert ref["status"] == 0
    p, H = ctx.project(U, V, grid, grid, 2 * math.pi, 10, 10)
    rp = ref["pnp"]
    assert (p.nocc, p.nemp) == (rp.nocc, rp.nemp)
    assert abs((p.c("ener") / p.c("over")).real - (rp.c("ener") / rp.c("over")).real) < 1e-9
    for k in ("prot", "neut", "prot2", "neut2"):
        assert abs((p.c(k) / p.c("over")).real - (rp.c(k) / rp.c("over")).real) < 1e-10, k
    assert abs(p.c("over") - rp.c("over")) < 1e-10 * abs(rp.c("over"))
    assert relerr(H, ref["H20v"]) < 1e-9


def test_evolve_emax6(emax6):
    mdl, U, V, om, ctx = emax6
    n = mdl.n
    rng = np.random.default_rng(6)
    Z = 0.05 * rng.normal(size=(n, n))
    Z = Z - Z.T
    U1, V1 = ctx.evolve(U, V, Z)
    st, U1r, V1r = O.thouless_evolve(U, V, Z)
    assert st == 0
    assert np.abs(U1 - U1r).max() < 1e-12 and np.abs(V1 - V1r).max() < 1e-12
