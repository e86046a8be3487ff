import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "big: full-size workload (minutes, tens of GB)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "digests.json")) as f:
        return json.load(f)


def load_kat(system):
    r"""Integrals of a known-answer-test system, rebuilt from the unique 8-fold elements."""
    z = np.load(os.path.join(GOLDEN, "kat_%s.npz" % system))
    one = z["one_mo"]
    n = one.shape[0]
    g = np.zeros((n, n, n, n))
    for (p, q, r, s), v in zip(z["keys"].astype(np.int64), z["vals"]):
        for (a, b, c, d) in ((p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                             (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)):
            g[a, b, c, d] = v
    two = np.ascontiguousarray(g.transpose(0, 2, 1, 3))
    return float(z["ecore"]), np.ascontiguousarray(one), two


def load_csr_case(name):
    z = np.load(os.path.join(GOLDEN, "csr_%s.npz" % name))
    return {k: z[k] for k in z.files}
