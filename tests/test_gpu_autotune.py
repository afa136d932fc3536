"""tvap_autotune: the launch-shape candidates of the projection (B' tile
policy of the tcgen05 products, staggered groups of the Thouless solve, the
CTA cap beside the panel factorisations, the look-ahead of the solve's
panels, the form of the Pfaffian) give the same results -- the
emulated products sum exact integers whatever the tiling -- and the tuner
keeps the fastest one.  Workload: emax=4 (n = 140), 15 x 15 angles."""

import math

import numpy as np
import pytest

from taurus_vap_gb300 import model as M
from taurus_vap_gb300.native import Context

pytestmark = pytest.mark.gpu


def test_autotune_candidates_agree_and_fastest_is_kept():
    mdl = M.noncore_model(4, seed=1)
    U, V = M.random_bogoliubov(mdl.basis, 8, 8, seed=2)
    ctx = Context(mdl.basis, mdl.ham)
    args = (15, 15, 2 * math.pi, 8, 8)
    ref, Href = ctx.project(U, V, *args)
    for bn, groups, cap, la, pf in Context.TUNE_CANDIDATES:
        ctx.set_tuning(bn, groups, cap, la, pf)
        p, H = ctx.project(U, V, *args)
        # the shapes give the same sums to rounding; the blocked Pfaffian
        # only another order of the overlap's rounding
        tol = 1e-13 if pf == 0 else 1e-11
        assert abs(p.c("ener") - ref.c("ener")) <= tol * abs(ref.c("ener")), (bn, groups, cap, la, pf)
        assert np.abs(H - Href).max() <= tol * np.abs(Href).max(), (bn, groups, cap, la, pf)
    table = ctx.autotune(U, V, *args, reps=2)
    assert len(table) == 48 and all(v > 0 for v in table.values())
    assert ctx.tuning() == min(table, key=table.get)
