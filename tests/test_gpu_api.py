r"""The drop-in Python API on the GPU, mirroring the reference's own tests of
sparse_op (pyci/test/test_routines.py:37-80, pyci/test/test_odometer.py)."""

import numpy as np
import numpy.testing as npt
import pytest

import pyci_gb300 as pyci
from conftest import load_csr_case, load_kat

pytestmark = pytest.mark.gpu


def ham_of(system):
    return pyci.secondquant_op(*load_kat(system))


@pytest.mark.parametrize("kat", [0, 1, 2, 3])
def test_solve_sparse(golden, kat):
    k = golden["kats"][kat]
    ham = ham_of(k["system"])
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[k["wfn"]](ham.nbasis, *k["occs"])
    wfn.add_all_dets()
    op = pyci.sparse_op(ham, wfn)
    es, cs = op.solve(n=1, ncv=30, tol=1.0e-6)
    npt.assert_allclose(es[0], k["energy"], rtol=0.0, atol=1.0e-9)
    assert cs.shape == (1, len(wfn))


@pytest.mark.parametrize("system, wfn_type, occs", [
    ("li2_ccpvdz", "doci", (3, 3)), ("h2o_ccpvdz", "doci", (5, 5)), ("be_ccpvdz", "fullci", (2, 2))])
def test_sparse_rectangular(system, wfn_type, occs):
    ham = ham_of(system)
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[wfn_type](ham.nbasis, *occs)
    pyci.add_excitations(wfn, 0, 1, 2)
    nrow = len(wfn) - 10
    op = pyci.sparse_op(ham, wfn, nrow, symmetric=False)
    assert op.shape == (nrow, len(wfn))
    y = op(np.ones(op.shape[1], dtype=pyci.c_double))
    assert y.ndim == 1 and y.shape[0] == op.shape[0]
    # Row sums of the stored matrix (the reference test sums get_element over all j).
    data, indices, indptr = op.data(), op.indices(), op.indptr()
    rows = np.repeat(np.arange(nrow), np.diff(indptr))
    z = np.bincount(rows, weights=data, minlength=nrow)
    npt.assert_allclose(y, z, rtol=1e-12, atol=1e-12)
    for i in range(0, nrow, max(1, nrow // 5)):
        assert sum(op.get_element(i, j) for j in indices[indptr[i]:indptr[i + 1]]) == pytest.approx(z[i], abs=1e-12)
    out = np.zeros(nrow)
    assert op(np.ones(op.shape[1]), out) is not None
    npt.assert_allclose(out, y)


@pytest.mark.parametrize("case", ["fci_6_3_2", "doci_10_4", "fci_7_3_3_cisd", "genci_10_4"])
def test_arrays_match_reference(golden, case):
    meta = {m["name"]: m for m in golden["csr_cases"]}[case]
    ref = load_csr_case(case)
    ham = pyci.secondquant_op(ref["ecore"], ref["one_mo"], ref["two_mo"])
    W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn, "genci": pyci.genci_wfn}[meta["wfn"]]
    wfn = W(meta["nbasis"], meta["nocc_up"], meta["nocc_dn"])
    if meta["excitations"] is None:
        wfn.add_all_dets()
    else:
        pyci.add_excitations(wfn, *meta["excitations"])
    op = pyci.sparse_op(ham, wfn, meta["nrow"], meta["ncol"], meta["symmetric"])
    assert op.size == meta["size"] and op.shape == tuple(meta["shape"])
    npt.assert_array_equal(op.indptr(), ref["indptr"])
    npt.assert_array_equal(op.indices(), ref["indices"])
    if meta["wfn"] != "genci":
        npt.assert_array_equal(op.data(), ref["data"])
    npt.assert_allclose(op(ref["x"]), ref["y"], rtol=1e-12, atol=1e-11)
    assert op.dtype == np.float64 and op.symmetric == meta["symmetric"]


@pytest.mark.parametrize("wfn_type, occs", [("doci", (2, 2)), ("fullci", (1, 1)), ("fullci", (2, 2))])
def test_nearly_all_roots_in_decreasing_order(wfn_type, occs):
    # test_odometer solves for n = len(wfn) - 1 roots of tiny problems and
    # relies on the reference's decreasing order.
    from pyci_gb300.synth import synthetic_integrals
    nb = 4 if occs != (1, 1) else 2
    ham = pyci.secondquant_op(*synthetic_integrals(nb, 3))
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[wfn_type](nb, *occs)
    wfn.add_all_dets()
    op = pyci.sparse_op(ham, wfn)
    n = len(wfn) - 1
    es, cs = op.solve(n=n, tol=1.0e-9)
    d, i, p = op.data(), op.indices(), op.indptr()
    low = np.zeros((len(wfn), len(wfn)))
    for r in range(len(wfn)):
        low[r, i[p[r]:p[r + 1]]] = d[p[r]:p[r + 1]]
    full = low + low.T - np.diag(np.diag(low))
    w = np.linalg.eigvalsh(full)[:n]
    npt.assert_allclose(es, w[::-1] + ham.ecore, atol=1e-10)
    for k in range(n):
        npt.assert_allclose(full @ cs[k], (es[k] - ham.ecore) * cs[k], atol=1e-8)


def test_solve_with_c0_and_mixed_mode():
    from pyci_gb300.synth import synthetic_integrals
    ham = pyci.secondquant_op(*synthetic_integrals(8, 1001))
    wfn = pyci.fullci_wfn(8, 4, 4)
    wfn.add_all_dets()
    op = pyci.sparse_op(ham, wfn)
    e64, c64 = op.solve(n=2, tol=1e-10)
    e2, c2 = op.solve(n=1, c0=c64[1], tol=1e-10)
    assert e2[0] == pytest.approx(e64[1], abs=1e-9)
    em, cm = op.solve(n=2, tol=1e-6, mode="mixed")
    npt.assert_allclose(em, e64, atol=1e-6)
    assert op.solve_stats["mode"] == "mixed"


def test_update_after_growth():
    ham = ham_of("be_ccpvdz")
    wfn = pyci.fullci_wfn(ham.nbasis, 2, 2)
    wfn.add_hartreefock_det()
    op = pyci.sparse_op(ham, wfn)
    pyci.add_excitations(wfn, 1, 2)
    op.update(ham, wfn)
    assert op.shape == (len(wfn), len(wfn))
    fresh = pyci.sparse_op(ham, wfn)
    npt.assert_array_equal(op.indptr(), fresh.indptr())
    npt.assert_array_equal(op.indices(), fresh.indices())
    npt.assert_array_equal(op.data(), fresh.data())
