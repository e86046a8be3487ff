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


def unpack_8fold(one, keys, vals):
    r"""Physicist's two_mo from the unique chemist's (pq|rs) elements (p>=q, r>=s, pq>=rs)."""
    n = one.shape[0]
    g = np.zeros((n, n, n, n))
    k = keys.astype(np.int64)
    p, q, r, s = k[:, 0], k[:, 1], k[:, 2], k[:, 3]
    for (a, b, c, d) in ((p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                         (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)):
        g[a, b, c, d] = vals
    return np.ascontiguousarray(g.transpose(0, 2, 1, 3))


def load_kat(system):
    r"""Integrals of a known-answer-test system (ecore, one_mo, two_mo)."""
    z = np.load(os.path.join(GOLDEN, "kat_%s.npz" % system))
    one = np.ascontiguousarray(z["one_mo"])
    return float(z["ecore"]), one, unpack_8fold(one, z["keys"], z["vals"])


def load_csr_case(name):
    r"""A reference CSR fixture; its integrals are under "ecore", "one_mo", "two_mo"."""
    z = np.load(os.path.join(GOLDEN, "csr_%s.npz" % name))
    d = {k: z[k] for k in z.files}
    d["ecore"] = float(d["ecore"])
    d["two_mo"] = unpack_8fold(d["one_mo"], d.pop("keys"), d.pop("vals"))
    return d
