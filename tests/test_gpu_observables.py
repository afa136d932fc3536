"""project_wavefunction with iopt = 1 on the device (tvap_project_observables):
the gauge sums of the observables print_results prints (module_projection.f90:
990-1322) against the oracle's restatement of the same branch (:279-354) and
of sum_gauge (:425-458): the energy decomposition, the one-body traces (J,
spin-orbit, Q_lm, r^2), <J_i^2>, the shell occupations, the parity overlap
and pnp_rho.  States: the Mg24 / USDB seed (sd, every l even: the parity
overlaps are the overlaps), emax=2 with M = 7 and M = 1 (p shells: a
non-trivial parity), and the benchmark's emax=4 state with 15 x 15 angles.

Tolerance: every sum divided by the projected overlap within 1e-9 of the
oracle's (relative to 1 + its size); pnp_rho / overlap within 1e-10."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

import oracle as O

pytestmark = pytest.mark.gpu


def compare(mdl, U, V, Mp, Z, N, with_parity=True):
    ops = mdl.observable_operators()
    ref = O.OracleModel(mdl).project_observables(U, V, Mp, Mp, 2 * math.pi, Z, N, ops, with_parity=with_parity)
    assert ref["status"] == 0
    got = Context(mdl.basis, mdl.ham).project_observables(U, V, Mp, Mp, 2 * math.pi, Z, N, ops,
                                                          with_parity=with_parity)
    ov_r, ov_g = ref["scal"][0], got["scal"][0]
    assert abs(ov_g - ov_r) <= 1e-10 * abs(ov_r)

    def close(a, b, tol=1e-9):
        x, y = np.asarray(a) / ov_g, np.asarray(b) / ov_r
        return np.all(np.abs(x - y) <= tol * (1.0 + np.abs(y)))

    assert close(got["scal"][1:], ref["scal"][1:])
    assert close(got["obo"], ref["obo"])
    assert close(got["sq"], ref["sq"])
    assert close(got["occnum"], ref["occnum"])
    assert close(got["rho"], ref["rho"], 1e-10)
    return got, ref


def test_observables_mg24(usdb_model, mg24_seed):
    got, _ = compare(usdb_model, *mg24_seed, 5, 4, 4)
    s = got["scal"]
    assert abs(s[6] - s[0]) <= 1e-10 * abs(s[0])  # sd: parity +1 throughout
    # the components add up to the projected energy
    e = s[7:] / s[0]
    assert abs((e[10] + e[11]).real + usdb_model.ham.H0.real - (s[1] / s[0]).real) < 1e-8


@pytest.mark.parametrize("Mp", [7, 1])
def test_observables_emax2(Mp):
    mdl = M.noncore_model(2, seed=1, valence_Z=4, valence_N=4)
    U, V = M.random_bogoliubov(mdl.basis, 4, 4, seed=3)
    got, _ = compare(mdl, U, V, Mp, 4, 4)
    assert abs(got["scal"][6]) > 0  # a non-trivial parity overlap
    got2, _ = compare(mdl, U, V, Mp, 4, 4, with_parity=False)
    assert got2["scal"][6] == 0


def test_observables_benchmark_state():
    mdl = M.noncore_model(4, seed=1)
    U, V = M.random_bogoliubov(mdl.basis, 8, 8, seed=2)
    compare(mdl, U, V, 15, 8, 8)
