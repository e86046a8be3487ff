r"""Epstein-Nesbet second-order energy (compute_enpt2) on the GPU: against the
reference's own values, against the C oracle on wider sets, and the
reference's test_enpt2 (pyci/test/test_routines.py:473-491) through the
drop-in API with its published energies."""

import os

import numpy as np
import numpy.testing as npt
import pytest

import oracle as O
import pyci_gb300 as pyci
from conftest import load_kat, unpack_8fold
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


def test_enpt2_matches_reference(ctx, golden):
    for m in golden["enpt2_cases"]:
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "enpt2_%s.npz" % m["name"]))
        one = np.ascontiguousarray(z["one_mo"])
        two = unpack_8fold(one, z["keys"], z["vals"])
        e = ctx.compute_enpt2(GPU[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets"], z["coeffs"], one,
                              two, float(z["energy"]), float(z["ecore"]), m["eps"])
        corr = float(z["result"]) - float(z["energy"])
        assert e == pytest.approx(float(z["result"]), rel=0, abs=1e-12 * max(1.0, abs(corr))), m["name"]


@pytest.mark.parametrize("kind,n,nu,nd,eps", [("fullci", 10, 4, 3, 1e-4), ("doci", 18, 5, 5, 1e-5),
                                              ("fullci", 70, 2, 1, 1e-3), ("doci", 70, 3, 3, 1e-3)])
def test_enpt2_matches_oracle(ctx, kind, n, nu, nd, eps):
    ecore, one, two = synthetic_integrals(n, 80 + n)
    full = O.all_dets(ORC[kind], n, nu, nd)
    rng = np.random.default_rng(n)
    dets = full[np.sort(rng.choice(full.shape[0], size=min(2000, full.shape[0] // 4), replace=False))]
    c = rng.normal(size=dets.shape[0])
    c /= np.linalg.norm(c)
    energy = -5.0 * (nu + nd)  # below every diagonal element: all denominators negative
    e_gpu = ctx.compute_enpt2(GPU[kind], n, nu, nd, dets, c, one, two, energy, ecore, eps)
    e_ref = O.compute_enpt2(ORC[kind], n, nu, nd, dets, c, one, two, energy, ecore, eps)
    assert e_gpu != energy
    assert e_gpu == pytest.approx(e_ref, rel=0, abs=1e-11 * abs(e_ref - energy))


@pytest.mark.parametrize("i", [0, 1, 2, 3])
def test_enpt2_known_answers(golden, i):
    k = golden["enpt2_kats"][i]
    ham = pyci.secondquant_op(*load_kat(k["system"]))
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[k["wfn"]](ham.nbasis, *k["occs"])
    pyci.add_excitations(wfn, *range(0, max(wfn.nocc - 1, 1)))
    op = pyci.sparse_op(ham, wfn)
    es, cs = op.solve()
    e = pyci.compute_enpt2(ham, wfn, cs[0], es[0], 1.0e-4)
    npt.assert_allclose(e, k["enpt2"])


def test_enpt2_edge_cases(ctx):
    ecore, one, two = synthetic_integrals(6, 3)
    full = O.all_dets(O.FULLCI, 6, 2, 2)
    # The full space has no external determinants: the correction is zero.
    assert ctx.compute_enpt2(capi.WFN_FULLCI, 6, 2, 2, full, np.ones(full.shape[0]), one, two, -3.0, 0.0,
                             0.0) == -3.0
    assert ctx.compute_enpt2(capi.WFN_FULLCI, 6, 2, 2, full[:0], np.zeros(0), one, two, -3.0, 0.0, 0.0) == -3.0
    with pytest.raises(capi.GpuError):
        g = O.all_dets(O.GENCI, 6, 3, 0)
        ctx.compute_enpt2(capi.WFN_GENCI, 6, 3, 0, g, np.ones(g.shape[0]), one, two, -3.0, 0.0, 1e-4)
