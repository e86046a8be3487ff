r"""The CPU oracle pinned against the reference: golden CSR arrays built by the
reference's own sparse_op, the reference tests' known-answer energies, and
digests of the reference CSR for the 8- and 24-orbital workloads."""

import numpy as np
import pytest

import oracle as O
from conftest import load_csr_case, load_kat
from pyci_gb300.synth import synthetic_integrals, config_seed

KIND = {"doci": O.DOCI, "fullci": O.FULLCI, "genci": O.GENCI_REF}


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


def test_binomial_and_colex_roundtrip():
    L = O.lib()
    assert L.orc_binomial(12, 5) == 792
    assert L.orc_binomial(32, 8) == 10518300
    for n, k in [(8, 4), (10, 3), (70, 2), (130, 2)]:
        dets = O.all_dets(O.DOCI, n, k, k)
        assert dets.shape[0] == L.orc_binomial(n, k)
        ranks = [L.orc_rank_colex(n, k, O._ptr(np.ascontiguousarray(d))) for d in dets[:: max(1, len(dets) // 97)]]
        assert ranks == list(range(0, len(dets), max(1, len(dets) // 97)))


def test_phase_conventions():
    L = O.lib()
    det = np.array([0b1011011], dtype=np.uint64)  # orbitals 0,1,3,4,6
    # single 1 -> 5: occupied strictly between are 3, 4 -> +1
    assert L.orc_phase_single(O._ptr(det), 1, 5) == 1
    # single 0 -> 2: occupied between: 1 -> -1
    assert L.orc_phase_single(O._ptr(det), 0, 2) == -1
    # double (0,1)->(2,5): perms 1 (0->2 passes 1) + 2 (1->5 passes 3,4) = 3, and
    # i2=1 < a1=2 adds one -> even -> +1
    assert L.orc_phase_double(O._ptr(det), 0, 1, 2, 5) == 1


@pytest.mark.parametrize("case", [c for c in [
    "fci_6_3_2", "fci_7_3_3_cisd", "fci_7_3_2_rect", "fci_5_2_2_sym_nrow", "doci_10_4",
    "doci_12_5_cisd_rect", "doci_9_3_ncol", "genci_10_4", "genci_12_3_cisd_rect"]])
def test_oracle_csr_matches_reference(golden, case):
    meta = {m["name"]: m for m in golden["csr_cases"]}[case]
    ref = load_csr_case(case)
    one, two = ref["one_mo"], ref["two_mo"]
    data, indices, indptr = O.build_csr(KIND[meta["wfn"]], meta["nbasis"], meta["nocc_up"], meta["nocc_dn"],
                                        ref["dets"], one, two, meta["nrow"], meta["ncol"], meta["symmetric"])
    assert np.array_equal(indptr, ref["indptr"])
    assert np.array_equal(indices, ref["indices"])
    if meta["wfn"] == "genci":
        # Rows may hold repeated columns (the reference's GenCI quirk); their
        # order under std::sort is unspecified, so compare per row as multisets.
        for r in range(indptr.shape[0] - 1):
            s, e = indptr[r], indptr[r + 1]
            assert sorted(zip(indices[s:e], data[s:e])) == sorted(zip(ref["indices"][s:e], ref["data"][s:e]))
    else:
        assert np.array_equal(data, ref["data"])  # bit-exact FP64
    nrow, ncol = meta["shape"]
    if meta["symmetric"] and ncol < nrow:
        return  # the reference's self-adjoint product reads x past ncol here (undefined)
    y = O.spmv(data, indices, indptr, ref["x"], symmetric=meta["symmetric"])
    np.testing.assert_allclose(y, ref["y"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind,nb,nu,nd", [(O.FULLCI, 7, 3, 2), (O.DOCI, 10, 4, 4)])
def test_oracle_row_range_build_concatenates_to_the_full_build(kind, nb, nu, nd):
    # The CPU baseline builds a large operator in row slices; the slices must
    # be exactly the rows of the whole build.
    ecore, one, two = synthetic_integrals(nb, 17)
    dets = O.all_dets(kind, nb, nu, nd)
    data, indices, indptr = O.build_csr(kind, nb, nu, nd, dets, one, two)
    n = dets.shape[0]
    cuts = [0, 1, n // 3, n // 3, n - 5, n]
    for r0, r1 in zip(cuts[:-1], cuts[1:]):
        d, i, p = O.build_csr_rows(kind, nb, nu, nd, dets, one, two, r0, r1, nthreads=3)
        assert np.array_equal(p, indptr[r0:r1 + 1] - indptr[r0])
        assert np.array_equal(i, indices[indptr[r0]:indptr[r1]])
        assert np.array_equal(d, data[indptr[r0]:indptr[r1]])


@pytest.mark.parametrize("name", ["fci_8_4_4", "doci_24_6"])
def test_oracle_workload_digest(golden, name):
    from digest import digest
    w = golden["workloads"][name]
    kind = KIND[w["wfn"]]
    ecore, one, two = synthetic_integrals(w["nbasis"], w["seed"])
    dets = O.all_dets(kind, w["nbasis"], *w["occs"])
    data, indices, indptr = O.build_csr(kind, w["nbasis"], w["occs"][0], w["occs"][1], dets, one, two)
    d = digest(data, indices, indptr)
    assert d["nnz"] == w["nnz"]
    assert d["pattern_sum"] == w["pattern_sum"] and d["pattern_xor"] == w["pattern_xor"]
    assert d["value_sum"] == pytest.approx(w["value_sum"], rel=1e-12, abs=1e-9)
    assert d["value_wsum"] == pytest.approx(w["value_wsum"], rel=1e-12, abs=1e-9)


@pytest.mark.parametrize("kat", [0, 1, 2, 3])
def test_oracle_known_answer_energies(golden, kat):
    # pyci/test/test_routines.py:37-54: lowest energy to atol 1e-9.
    k = golden["kats"][kat]
    ecore, one, two = load_kat(k["system"])
    n = one.shape[0]
    kind = KIND[k["wfn"]]
    dets = O.all_dets(kind, n, *k["occs"])
    csr = O.build_csr(kind, n, k["occs"][0], k["occs"][1], dets, one, two)
    e = O.lowest_eigenvalues(*csr, nroot=1)[0] + ecore
    assert abs(e - k["energy"]) < 1e-9


def load_hci_case(name):
    from conftest import unpack_8fold
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "hci_%s.npz" % name))
    one = np.ascontiguousarray(z["one_mo"])
    return {k: z[k] for k in ("dets", "coeffs", "added")}, one, unpack_8fold(one, z["keys"], z["vals"])


def sorted_rows(a):
    return a[np.lexsort(a.T[::-1])] if len(a) else a


def test_add_hci_matches_reference_sets(golden):
    r"""One heat-bath CI step (pyci/src/hci.cpp) on every golden case: the set
    of determinants the oracle adds equals the reference's, and each appears
    once.  The GenCI case replays the reference's virtual-count quirk, which
    adds determinants with one electron too few (reproduced, not fixed)."""
    for m in golden["hci_cases"]:
        z, one, two = load_hci_case(m["name"])
        new = O.add_hci(KIND[m["wfn"]], one.shape[0], m["nocc_up"], m["nocc_dn"], z["dets"], z["coeffs"],
                        one, two, m["eps"])
        assert new.shape[0] == m["nadded"]
        assert np.array_equal(sorted_rows(new), z["added"]), m["name"]
        assert len({tuple(r) for r in new}) == new.shape[0]


def test_add_hci_thresholds():
    # eps = 0 adds exactly the determinants H connects to the start with a
    # nonzero element (|H_ij| > 0); a zero coefficient (eps / |c| = inf) and a
    # huge eps add none.
    ecore, one, two = synthetic_integrals(6, 5)
    dets = O.all_dets(O.FULLCI, 6, 2, 2)
    hf = dets[:1]
    every = O.add_hci(O.FULLCI, 6, 2, 2, hf, np.array([1.0]), one, two, 0.0)
    data, indices, indptr = O.build_csr(O.FULLCI, 6, 2, 2, dets, one, two, symmetric=False)
    cols, vals = indices[indptr[0]:indptr[1]], data[indptr[0]:indptr[1]]
    connected = {tuple(dets[j]) for j, v in zip(cols, vals) if j != 0 and v != 0.0}
    assert {tuple(r) for r in every} == connected
    assert O.add_hci(O.FULLCI, 6, 2, 2, hf, np.array([0.0]), one, two, 1e-9).shape[0] == 0
    assert O.add_hci(O.FULLCI, 6, 2, 2, hf, np.array([1.0]), one, two, 1e9).shape[0] == 0


def load_rdm_case(name):
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rdm_%s.npz" % name))
    return {k: z[k] for k in z.files}


def test_compute_rdms_bit_identical_to_reference(golden):
    r"""The oracle's compute_rdms (pyci/src/rdm.cpp, reference summation order)
    reproduces the reference's arrays exactly; spinize_rdms restated here
    reproduces the reference's utility."""
    from pyci_gb300.utility import spinize_rdms
    for m in golden["rdm_cases"]:
        z = load_rdm_case(m["name"])
        r1, r2 = O.compute_rdms(KIND[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets"], z["coeffs"])
        assert np.array_equal(r1, z["rdm1"]) and np.array_equal(r2, z["rdm2"]), m["name"]
        s1, s2 = spinize_rdms(z["rdm1"], z["rdm2"])
        np.testing.assert_allclose(s1, z["spin1"], rtol=0, atol=1e-15)
        np.testing.assert_allclose(s2, z["spin2"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("kind", ["doci", "fullci"])
def test_rdm_energy_identities(kind):
    r"""<c|H|c> from the RDMs equals the CSR quadratic form: DOCI through the
    reduced seniority-zero integrals (pyci/utility.py:59-91), FullCI through
    the spin-orbital RDMs and integrals."""
    from pyci_gb300.utility import reduce_senzero_integrals, spinize_rdms
    n, nu, nd = (8, 3, 3) if kind == "doci" else (6, 3, 2)
    ecore, one, two = synthetic_integrals(n, 61)
    dets = O.all_dets(KIND[kind], n, nu, nd)
    c = np.random.default_rng(3).normal(size=dets.shape[0])
    c /= np.linalg.norm(c)
    csr = O.build_csr(KIND[kind], n, nu, nd, dets, one, two)
    e_ref = c @ O.spmv(*csr, c)
    r1, r2 = O.compute_rdms(KIND[kind], n, nu, nd, dets, c)
    if kind == "doci":
        assert np.trace(r1) == pytest.approx(nu, abs=1e-12)
        assert np.sum(r2) == pytest.approx(nu * (nu - 1), abs=1e-12)
        h, v, w = O.senzero(one, two)
        k0, k2 = reduce_senzero_integrals(h, v, w, nu)
        e = np.einsum("ij,ij", k0, r1) + np.einsum("ij,ij", k2, r2)
    else:
        s1, s2 = spinize_rdms(r1, r2)
        # spin-orbital integrals (alpha block first), physicist's notation
        o2 = np.kron(np.eye(2), one)
        t2 = np.zeros((2 * n,) * 4)
        for s in (0, n):
            for t in (0, n):
                t2[s:s + n, t:t + n, s:s + n, t:t + n] = two
        # 1/2 <pq|rs> G_pqrs = 1/4 <pq||rs> G_pqrs for the antisymmetric G
        e = np.einsum("ij,ij", o2, s1) + 0.5 * np.einsum("ijkl,ijkl", t2, s2)
        assert np.allclose(s1, s1.T)
    assert e == pytest.approx(e_ref, abs=1e-12)


def test_compute_enpt2_matches_reference(golden):
    from conftest import unpack_8fold
    import os
    for m in golden["enpt2_cases"]:
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "enpt2_%s.npz" % m["name"]))
        one = np.ascontiguousarray(z["one_mo"])
        two = unpack_8fold(one, z["keys"], z["vals"])
        r = O.compute_enpt2(KIND[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets"], z["coeffs"], one, two,
                            float(z["energy"]), float(z["ecore"]), m["eps"])
        # Same terms; the final sum runs in another order than the reference's hash map.
        assert r == pytest.approx(float(z["result"]), rel=0, abs=1e-13 * abs(float(z["result"])))


@pytest.mark.parametrize("i", [0, 1, 2])
def test_compute_enpt2_known_answers(golden, i):
    r"""pyci/test/test_routines.py:473-491 (test_enpt2) with the oracle: CISD-like
    set, FP64 ground state, eps = 1e-4, against the test's published values
    (the 42,504-determinant water case runs on the GPU only)."""
    import pyci_gb300 as pyci
    k = golden["enpt2_kats"][i]
    ecore, one, two = load_kat(k["system"])
    n = one.shape[0]
    wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[k["wfn"]](n, *k["occs"])
    pyci.add_excitations(wfn, *range(0, max(wfn.nocc - 1, 1)))
    dets = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1)
    data, indices, indptr = O.build_csr(KIND[k["wfn"]], n, k["occs"][0], k["occs"][1], dets, one, two)
    H = O.full_matrix(data, indices, indptr).toarray()
    w, v = np.linalg.eigh(H)
    e = O.compute_enpt2(KIND[k["wfn"]], n, k["occs"][0], k["occs"][1], dets, v[:, 0], one, two, w[0] + ecore, ecore,
                        1.0e-4)
    np.testing.assert_allclose(e, k["enpt2"], rtol=1e-7)


def test_transition_rdms_match_reference(golden):
    import os
    for m in golden["trdm_cases"]:
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "trdm_%s.npz" % m["name"]))
        r1, r2 = O.compute_transition_rdms(KIND[m["wfn"]], m["nbasis"], m["nocc_up"], m["nocc_dn"], z["dets1"],
                                           z["coeffs1"], z["dets2"], z["coeffs2"])
        assert np.array_equal(r1, z["rdm1"]) and np.array_equal(r2, z["rdm2"]), m["name"]


@pytest.mark.parametrize("kind", ["doci", "fullci"])
def test_transition_rdms_of_a_state_with_itself(kind):
    # <Psi|...|Psi> through the transition loops (every excitation, no
    # partner terms) sums the same terms as compute_rdms.
    n, nu, nd = (9, 3, 3) if kind == "doci" else (6, 3, 2)
    dets = O.all_dets(KIND[kind], n, nu, nd)
    c = np.random.default_rng(4).normal(size=dets.shape[0])
    t1, t2 = O.compute_transition_rdms(KIND[kind], n, nu, nd, dets, c, dets, c)
    r1, r2 = O.compute_rdms(KIND[kind], n, nu, nd, dets, c)
    np.testing.assert_allclose(t1, r1, rtol=0, atol=1e-12)
    np.testing.assert_allclose(t2, r2, rtol=0, atol=1e-12)
