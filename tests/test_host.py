r"""Host-side API of pyci_gb300 (no GPU needed): the reference's wave-function and
Hamiltonian behaviour (pyci/test/test_wavefunction.py, test_hamiltonian.py)."""

import os
import tempfile
from filecmp import cmp as compare
from math import comb

import numpy as np
import numpy.testing as npt
import pytest

import pyci_gb300 as pyci
from conftest import load_csr_case, load_kat


def test_module_surface():
    for name in ["secondquant_op", "hamiltonian", "doci_wfn", "fullci_wfn", "genci_wfn", "sparse_op",
                 "popcnt", "ctz", "get_num_threads", "set_num_threads", "add_excitations",
                 "c_long", "c_ulong", "c_double", "wavefunction", "one_spin_wfn", "two_spin_wfn"]:
        assert hasattr(pyci, name), name
    assert pyci.hamiltonian is pyci.secondquant_op


def test_doci_raises():
    npt.assert_raises(ValueError, pyci.doci_wfn, 10, 11, 11)
    wfn = pyci.doci_wfn(5, 3, 3)
    wfn.add_hartreefock_det()
    assert wfn[0].flags["OWNDATA"]


def test_fullci_raises():
    npt.assert_raises(ValueError, pyci.fullci_wfn, 10, 11, 1)
    npt.assert_raises(ValueError, pyci.fullci_wfn, 10, 11, 11)
    npt.assert_raises(ValueError, pyci.fullci_wfn, 10, 0, 1)
    npt.assert_raises(ValueError, pyci.fullci_wfn, 10, 2, 3)
    npt.assert_raises(ValueError, pyci.genci_wfn, 10, 2, 1)


@pytest.mark.parametrize("nbasis, nocc", [(16, 8), (64, 1), (64, 4), (65, 1), (65, 4), (129, 3)])
def test_doci_add_all_dets_and_roundtrips(nbasis, nocc):
    wfn = pyci.doci_wfn(nbasis, nocc, nocc)
    wfn.add_all_dets()
    assert len(wfn) == comb(nbasis, nocc)
    dets = wfn.to_det_array()
    assert all(pyci.popcnt(d) == nocc for d in dets[:: max(1, len(dets) // 50)])
    npt.assert_array_equal(pyci.doci_wfn(nbasis, nocc, nocc, dets).to_det_array(), dets)
    occs = wfn.to_occ_array()
    npt.assert_array_equal(pyci.doci_wfn(nbasis, nocc, nocc, occs).to_occ_array(), occs)
    npt.assert_array_equal(wfn.__class__(wfn).to_det_array(), dets)
    with tempfile.TemporaryDirectory() as d:
        f1, f2 = os.path.join(d, "a"), os.path.join(d, "b")
        wfn.to_file(f1)
        pyci.doci_wfn(f1).to_file(f2)
        assert compare(f1, f2, shallow=False)


@pytest.mark.parametrize("nbasis, nocc", [(16, 8), (64, 1), (64, 4), (65, 4), (129, 3)])
def test_doci_add_excited_dets(nbasis, nocc):
    wfn = pyci.doci_wfn(nbasis, nocc, nocc)
    length = 0
    for i in range(nocc + 1):
        length += comb(nocc, i) * comb(nbasis - nocc, i)
        wfn.add_excited_dets(i)
        assert len(wfn) == length
    assert len(wfn) == comb(nbasis, nocc)


@pytest.mark.parametrize("nbasis, nocc_up, nocc_dn", [(8, 3, 3), (64, 1, 1), (64, 2, 1), (65, 2, 1), (129, 2, 1)])
def test_fullci_add_all_dets_and_excited(nbasis, nocc_up, nocc_dn):
    ndet = comb(nbasis, nocc_up) * comb(nbasis, nocc_dn)
    wfn = pyci.fullci_wfn(nbasis, nocc_up, nocc_dn)
    wfn.add_all_dets()
    assert len(wfn) == ndet
    for det in wfn.to_det_array()[:: max(1, ndet // 40)]:
        assert pyci.popcnt(det[0]) == nocc_up and pyci.popcnt(det[1]) == nocc_dn
    occs = wfn.to_occ_array()
    assert occs.shape[2] == nocc_up
    w2 = pyci.fullci_wfn(nbasis, nocc_up, nocc_dn, occs)
    npt.assert_array_equal(w2.to_det_array(), wfn.to_det_array())
    w3 = pyci.fullci_wfn(nbasis, nocc_up, nocc_dn)
    for i in range(nocc_up + nocc_dn + 1):
        w3.add_excited_dets(i)
    assert len(w3) == ndet


def test_index_and_add_det():
    wfn = pyci.fullci_wfn(6, 2, 2)
    wfn.add_all_dets()
    dets = wfn.to_det_array()
    for i in [0, 7, 100, len(wfn) - 1]:
        assert wfn.index_det(dets[i]) == i
        assert wfn.add_det(dets[i]) == -1
    w = pyci.fullci_wfn(6, 2, 2)
    assert w.add_occs(np.array([[0, 1], [2, 3]])) == 0
    assert w.add_occs(np.array([[0, 1], [2, 3]])) == -1
    assert w.index_det(np.array([[0b11], [0b1100]], dtype=np.uint64)) == 0


@pytest.mark.parametrize("case", ["fci_7_3_3_cisd", "doci_12_5_cisd_rect", "genci_12_3_cisd_rect"])
def test_determinant_order_matches_reference(golden, case):
    # The golden determinant lists come from the reference's add_excitations.
    meta = {m["name"]: m for m in golden["csr_cases"]}[case]
    W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn, "genci": pyci.genci_wfn}[meta["wfn"]]
    wfn = W(meta["nbasis"], meta["nocc_up"], meta["nocc_dn"])
    pyci.add_excitations(wfn, *meta["excitations"])
    ref = load_csr_case(case)["dets"]
    npt.assert_array_equal(np.asarray(wfn.to_det_array()).reshape(len(wfn), -1), ref)


@pytest.mark.parametrize("system", ["be_ccpvdz", "h2o_ccpvdz"])
def test_fcidump_roundtrip(system):
    ecore, one, two = load_kat(system)
    h1 = pyci.secondquant_op(ecore, one, two)
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "x.fcidump")
        h1.to_file(f, nelec=4, ms2=0)
        h2 = pyci.secondquant_op(f)
    for a in ["one_mo", "two_mo", "h", "v", "w"]:
        npt.assert_allclose(getattr(h2, a), getattr(h1, a), rtol=0.0, atol=1e-12)
    assert h2.ecore == pytest.approx(h1.ecore, abs=1e-12)
    n = one.shape[0]
    idx = np.arange(n)
    npt.assert_array_equal(h1.v, two[idx[:, None], idx[:, None], idx[None, :], idx[None, :]])


def test_threads():
    pyci.set_num_threads(3)
    assert pyci.get_num_threads() == 3
    pyci.set_num_threads(1)
