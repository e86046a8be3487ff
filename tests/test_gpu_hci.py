r"""Heat-bath CI selection (add_hci) on the GPU: one step against the C oracle
(same determinants, same first-occurrence order) and against the reference's
own step (same set), and the reference's HCI loop (pyci/test/test_routines.py
test_run_hci) through the drop-in API, converging to the known-answer
energies."""

import numpy as np
import numpy.testing as npt
import pytest

import oracle as O
import pyci_gb300 as pyci
from conftest import load_kat, unpack_8fold
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

ORC = {"doci": O.DOCI, "fullci": O.FULLCI, "genci": O.GENCI_REF}
GPU = {"doci": capi.WFN_DOCI, "fullci": capi.WFN_FULLCI, "genci": capi.WFN_GENCI}


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def load_hci(name):
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "hci_%s.npz" % name))
    one = np.ascontiguousarray(z["one_mo"])
    return z["dets"], z["coeffs"], z["added"], one, unpack_8fold(one, z["keys"], z["vals"])


def sorted_rows(a):
    return a[np.lexsort(a.T[::-1])] if len(a) else a


def test_add_hci_step_matches_oracle_and_reference(ctx, golden):
    for m in golden["hci_cases"]:
        dets, coeffs, added, one, two = load_hci(m["name"])
        n = one.shape[0]
        gpu = ctx.add_hci(GPU[m["wfn"]], n, m["nocc_up"], m["nocc_dn"], dets, coeffs, one, two, m["eps"])
        ref = O.add_hci(ORC[m["wfn"]], n, m["nocc_up"], m["nocc_dn"], dets, coeffs, one, two, m["eps"])
        assert np.array_equal(gpu, ref), m["name"]  # same determinants, same order
        assert np.array_equal(sorted_rows(gpu), added), m["name"]  # the reference's set
        assert gpu.shape[0] == m["nadded"]


@pytest.mark.parametrize("eps", [0.0, 1e-3, 1e-2])
def test_add_hci_genci_exact_rules(ctx, eps):
    # GenCI over the true virtual spin-orbitals: every added determinant keeps
    # the electron count.
    ecore, one, two = synthetic_integrals(10, 31)
    dets = O.all_dets(O.GENCI, 10, 4, 0)[::17]
    coeffs = np.random.default_rng(5).normal(size=dets.shape[0])
    gpu = ctx.add_hci(capi.WFN_GENCI, 10, 4, 0, dets, coeffs, one, two, eps, flags=capi.BUILD_GENCI_EXACT)
    ref = O.add_hci(O.GENCI, 10, 4, 0, dets, coeffs, one, two, eps)
    assert np.array_equal(gpu, ref)
    assert all(bin(int(d)).count("1") == 4 for d in gpu[:, 0])


@pytest.mark.parametrize("kind,n,nu,nd,eps", [("fullci", 9, 3, 3, 1e-3), ("doci", 14, 5, 5, 1e-4),
                                              ("fullci", 70, 2, 1, 1e-2), ("doci", 70, 2, 2, 1e-2)])
def test_add_hci_random_sets(ctx, kind, n, nu, nd, eps):
    # Random subsets of the full space, random coefficients (some zero), and
    # wave functions wider than one 64-bit word per string.
    ecore, one, two = synthetic_integrals(n, 40 + n)
    full = O.all_dets(ORC[kind], n, nu, nd)
    rng = np.random.default_rng(n)
    dets = full[np.sort(rng.choice(full.shape[0], size=min(300, full.shape[0] // 3), replace=False))]
    coeffs = rng.normal(size=dets.shape[0])
    coeffs[::7] = 0.0
    gpu = ctx.add_hci(GPU[kind], n, nu, nd, dets, coeffs, one, two, eps)
    ref = O.add_hci(ORC[kind], n, nu, nd, dets, coeffs, one, two, eps)
    assert gpu.shape[0] > 0
    assert np.array_equal(gpu, ref)


def test_add_hci_edge_cases(ctx):
    ecore, one, two = synthetic_integrals(6, 5)
    hf = O.all_dets(O.FULLCI, 6, 2, 2)[:1]
    assert ctx.add_hci(capi.WFN_FULLCI, 6, 2, 2, hf, np.array([0.0]), one, two, 1e-9).shape[0] == 0
    assert ctx.add_hci(capi.WFN_FULLCI, 6, 2, 2, hf, np.array([1.0]), one, two, 1e9).shape[0] == 0
    assert ctx.add_hci(capi.WFN_FULLCI, 6, 2, 2, hf[:0], np.zeros(0), one, two, 0.0).shape[0] == 0
    # The full space gains nothing.
    full = O.all_dets(O.FULLCI, 6, 2, 2)
    assert ctx.add_hci(capi.WFN_FULLCI, 6, 2, 2, full, np.ones(full.shape[0]), one, two, 0.0).shape[0] == 0


@pytest.mark.parametrize("kat", [0, 1, 2, 3])
def test_run_hci(golden, kat):
    # pyci/test/test_routines.py:431-470: HCI from the Hartree-Fock determinant
    # until no determinant is added (eps = 1e-4), then with eps = 0 until the
    # full space; the final energy is the known answer.
    from math import comb
    k = golden["kats"][kat]
    ham = pyci.secondquant_op(*load_kat(k["system"]))
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[k["wfn"]](ham.nbasis, *k["occs"])
    wfn.add_hartreefock_det()
    op = pyci.sparse_op(ham, wfn)
    es, cs = op.solve(n=1, tol=1.0e-6)
    dets_added, niter = 1, 0
    while dets_added:
        dets_added = pyci.add_hci(ham, wfn, cs[0], eps=1.0e-4)
        op.update(ham, wfn)
        es, cs = op.solve(n=1, tol=1.0e-6)
        niter += 1
    assert niter > 1
    full = comb(ham.nbasis, k["occs"][0]) * (comb(ham.nbasis, k["occs"][1]) if k["wfn"] == "fullci" else 1)
    assert len(wfn) <= full
    dets_added = 1
    while dets_added:
        dets_added = pyci.add_hci(ham, wfn, cs[0], eps=0.0)
        op.update(ham, wfn)
        es, cs = op.solve(n=1, tol=1.0e-6)
    assert len(wfn) == full
    npt.assert_allclose(es[0], k["energy"], rtol=0.0, atol=2.0e-9)
