r"""Reduced density matrices (compute_rdms) on the GPU against the reference's
own arrays, against the C oracle on wider sets, and the reference's
test_compute_rdms flow (pyci/test/test_routines.py:83-133) through the
drop-in API: traces, and the energy recomputed from the RDMs."""

import os

import numpy as np
import numpy.testing as npt
import pytest

import oracle as O
import pyci_gb300 as pyci
from conftest import load_kat
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

ORC = {"doci": O.DOCI, "fullci": O.FULLCI}
GPU = {"doci": capi.WFN_DOCI, "fullci": capi.WFN_FULLCI}


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def test_rdms_match_reference(ctx, golden):
    # Same terms as the reference, FP64 atomics in place of its serial sums.
    for m in golden["rdm_cases"]:
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rdm_%s.npz" % m["name"]))
        r1, r2 = ctx.compute_rdms(GPU[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets"], z["coeffs"])
        npt.assert_allclose(r1, z["rdm1"], rtol=0, atol=1e-13)
        npt.assert_allclose(r2, z["rdm2"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("kind,n,nu,nd", [("fullci", 10, 4, 3), ("doci", 20, 5, 5), ("fullci", 70, 2, 1),
                                          ("doci", 70, 3, 3)])
def test_rdms_match_oracle_on_subsets(ctx, kind, n, nu, nd):
    # Random subsets (determinants whose excitations leave the set are
    # skipped, as in the reference) and strings wider than one 64-bit word.
    full = O.all_dets(ORC[kind], n, nu, nd)
    rng = np.random.default_rng(n)
    dets = full[np.sort(rng.choice(full.shape[0], size=min(20000, full.shape[0] // 2), replace=False))]
    c = rng.normal(size=dets.shape[0])
    c /= np.linalg.norm(c)
    r1, r2 = ctx.compute_rdms(GPU[kind], n, nu, nd, dets, c)
    o1, o2 = O.compute_rdms(ORC[kind], n, nu, nd, dets, c)
    npt.assert_allclose(r1, o1, rtol=0, atol=1e-12)
    npt.assert_allclose(r2, o2, rtol=0, atol=1e-12)


@pytest.mark.parametrize("kat", [0, 1, 2, 3])
def test_compute_rdms_energies(golden, kat):
    # pyci/test/test_routines.py:83-133 on the known-answer systems: the RDMs'
    # traces and the energy recomputed from them equal the solve's.
    k = golden["kats"][kat]
    ecore, one, two = load_kat(k["system"])
    ham = pyci.secondquant_op(ecore, one, two)
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[k["wfn"]](ham.nbasis, *k["occs"])
    wfn.add_all_dets()
    op = pyci.sparse_op(ham, wfn)
    es, cs = op.solve(n=1, ncv=30, tol=1.0e-6)
    n = ham.nbasis
    if k["wfn"] == "doci":
        d0, d2 = pyci.compute_rdms(wfn, cs[0])
        nocc = k["occs"][0]
        npt.assert_allclose(np.trace(d0), nocc, rtol=0, atol=1.0e-9)
        npt.assert_allclose(np.sum(d2), nocc * (nocc - 1), rtol=0, atol=1.0e-9)
        k0, k2 = pyci.reduce_senzero_integrals(ham.h, ham.v, ham.w, nocc)
        energy = ham.ecore + np.einsum("ij,ij", k0, d0) + np.einsum("ij,ij", k2, d2)
        npt.assert_allclose(energy, es[0], rtol=0.0, atol=1.0e-9)
        rdm1, rdm2 = pyci.spinize_rdms(d0, d2)
    else:
        d1, d2 = pyci.compute_rdms(wfn, cs[0])
        rdm1, rdm2 = pyci.spinize_rdms(d1, d2)
    assert np.all(np.abs(rdm1 - rdm1.T) < 1e-5)
    for i in range(2 * n):
        assert np.all(np.abs(rdm2[i, i, :, :]) < 1e-5)
        assert np.all(np.abs(rdm2[:, :, i, i]) < 1e-5)
    # spin-orbital integrals (alpha block first): 1/2 <pq|rs> G_pqrs
    o2 = np.kron(np.eye(2), one)
    t2 = np.zeros((2 * n,) * 4)
    for s in (0, n):
        for t in (0, n):
            t2[s:s + n, t:t + n, s:s + n, t:t + n] = two
    energy = ecore + np.einsum("ij,ij", o2, rdm1) + 0.5 * np.einsum("ijkl,ijkl", t2, rdm2)
    npt.assert_allclose(energy, es[0], rtol=0.0, atol=1.0e-9)


@pytest.mark.parametrize("n,nocc", [(10, 4), (70, 2), (16, 5)])
def test_genci_rdms_match_oracle(ctx, n, nocc):
    r"""GenCI spin-orbital RDMs (definition-based; the reference's GenCI
    compute_rdms is undefined) and transition RDMs against the oracle's,
    which the CPU tests pin to operator algebra; 70 spin orbitals use two
    words per determinant, (16, 5) a random subset."""
    full = O.all_dets(O.GENCI, n, nocc, 0)
    rng = np.random.default_rng(n + nocc)
    dets = full if full.shape[0] <= 5000 else full[np.sort(rng.choice(full.shape[0], 5000, replace=False))]
    c = rng.normal(size=dets.shape[0])
    c /= np.linalg.norm(c)
    r1, r2 = ctx.compute_rdms(capi.WFN_GENCI, n, nocc, 0, dets, c)
    o1, o2 = O.compute_rdms_genci(n, dets, c)
    npt.assert_allclose(r1, o1, rtol=0, atol=1e-12)
    npt.assert_allclose(r2, o2, rtol=0, atol=1e-12)
    assert np.trace(r1) == pytest.approx(nocc, abs=1e-10)
    sub = np.sort(rng.choice(dets.shape[0], dets.shape[0] // 2, replace=False))
    c2 = rng.normal(size=sub.shape[0])
    t1, t2 = ctx.compute_transition_rdms(capi.WFN_GENCI, n, nocc, 0, dets, c, dets[sub], c2)
    u1, u2 = O.compute_rdms_genci(n, dets, c, dets[sub], c2)
    npt.assert_allclose(t1, u1, rtol=0, atol=1e-12)
    npt.assert_allclose(t2, u2, rtol=0, atol=1e-12)


def test_genci_rdms_drop_in_need_the_exact_flag():
    # Through the drop-in API: genci_exact=True gives the definition-based
    # spin-orbital RDMs, whose energy equals the GenCI eigenvalue; without the
    # flag the call raises (the reference's result is undefined).
    ecore, one, two = synthetic_integrals(3, 5)
    nsp = 3
    n = 2 * nsp
    h = np.kron(np.eye(2), one)
    g = np.zeros((n,) * 4)
    for s in (0, nsp):
        for t in (0, nsp):
            g[s:s + nsp, t:t + nsp, s:s + nsp, t:t + nsp] = two
    ham = pyci.secondquant_op(ecore, h, g)
    wfn = pyci.genci_wfn(n, 3, 0)
    for d in O.all_dets(O.GENCI, n, 3, 0):
        wfn.add_det(d)
    op = pyci.sparse_op(ham, wfn, genci_exact=True)
    es, cs = op.solve(n=1, tol=1e-12)
    with pytest.raises(ValueError):
        pyci.compute_rdms(wfn, cs[0])
    r1, r2 = pyci.compute_rdms(wfn, cs[0], genci_exact=True)
    assert r1.shape == (n, n) and r2.shape == (n, n, n, n)
    energy = ecore + np.einsum("pq,pq", h, r1) + 0.5 * np.einsum("pqrs,pqrs", g, r2)
    npt.assert_allclose(energy, es[0], rtol=0.0, atol=1.0e-9)


def test_transition_rdms_match_reference(ctx, golden):
    for m in golden["trdm_cases"]:
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "trdm_%s.npz" % m["name"]))
        r1, r2 = ctx.compute_transition_rdms(GPU[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets1"],
                                             z["coeffs1"], z["dets2"], z["coeffs2"])
        scale = max(1.0, float(np.abs(z["rdm2"]).max()))
        npt.assert_allclose(r1, z["rdm1"], rtol=0, atol=1e-13 * scale)
        npt.assert_allclose(r2, z["rdm2"], rtol=0, atol=1e-13 * scale)


@pytest.mark.parametrize("kind,n,nu,nd", [("fullci", 9, 3, 3), ("doci", 70, 3, 3)])
def test_transition_rdms_match_oracle(ctx, kind, n, nu, nd):
    full = O.all_dets(ORC[kind], n, nu, nd)
    rng = np.random.default_rng(n + 1)
    d1 = full[np.sort(rng.choice(full.shape[0], size=min(8000, full.shape[0] // 2), replace=False))]
    d2 = full[np.sort(rng.choice(full.shape[0], size=min(8000, full.shape[0] // 2), replace=False))]
    c1, c2 = rng.normal(size=d1.shape[0]), rng.normal(size=d2.shape[0])
    c1 /= np.linalg.norm(c1)
    c2 /= np.linalg.norm(c2)
    r1, r2 = ctx.compute_transition_rdms(GPU[kind], n, nu, nd, d1, c1, d2, c2)
    o1, o2 = O.compute_transition_rdms(ORC[kind], n, nu, nd, d1, c1, d2, c2)
    npt.assert_allclose(r1, o1, rtol=0, atol=1e-12)
    npt.assert_allclose(r2, o2, rtol=0, atol=1e-12)


def test_transition_rdms_drop_in(golden):
    # Between the two lowest states of be/cc-pVDZ FullCI(2,2): the transition
    # 1-RDM traces to <Psi_1|Psi_2> * N = 0; with itself it equals compute_rdms.
    k = next(k for k in golden["kats"] if k["wfn"] == "fullci")
    ham = pyci.secondquant_op(*load_kat(k["system"]))
    wfn = pyci.fullci_wfn(ham.nbasis, *k["occs"])
    wfn.add_all_dets()
    op = pyci.sparse_op(ham, wfn)
    es, cs = op.solve(n=2, tol=1e-10)
    t1, t2 = pyci.compute_transition_rdms(wfn, wfn, cs[0], cs[1])
    assert abs(np.trace(t1[0]) + np.trace(t1[1])) < 1e-8
    s1, s2 = pyci.compute_transition_rdms(wfn, wfn, cs[0], cs[0])
    r1, r2 = pyci.compute_rdms(wfn, cs[0])
    npt.assert_allclose(s1, r1, rtol=0, atol=1e-12)
    npt.assert_allclose(s2, r2, rtol=0, atol=1e-12)
