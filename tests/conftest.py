import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a) and the built device library")


@pytest.fixture(scope="session")
def usdb_model():
    from taurus_vap_gb300 import model as M
    return M.load_antoine(os.path.join(GOLDEN, "usdb.sho"), 4, 4)


@pytest.fixture(scope="session")
def mg24_seed(usdb_model):
    from taurus_vap_gb300 import model as M
    return M.read_wavefunction_text(os.path.join(GOLDEN, "mg24_initial_wf.txt"), usdb_model.n)


@pytest.fixture(scope="session")
def mg24_constraints(usdb_model):
    """Z, N and Q21 = 0 (examples/gradient_mg24/data/template_input.txt)."""
    import numpy as np
    from taurus_vap_gb300.vap import particle_number_ops
    n = usdb_model.n
    q = usdb_model.multipoles()
    Qz, Qn = particle_number_ops(n)
    return [Qz, Qn, q[1, 0, 1] + q[1, 1, 1]], [4.0, 4.0, 0.0]


def golden_table(name):
    """Parse the reference's results_*_benchmark tables: recipes and the
    eta/mu grid -> {(eta, mu): (iterations, energy)}."""
    rows = {}
    mus = [0.0, 0.3, 0.6, 0.9]
    for line in open(os.path.join(GOLDEN, name)):
        w = line.split()
        if len(w) == 9 and w[0].startswith("0."):
            eta = float(w[0])
            for k, mu in enumerate(mus):
                rows[(eta, mu)] = (int(w[1 + 2 * k]), float(w[2 + 2 * k]))
    return rows
