r"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference source tree:

    make -C oracle ref port            # reference built against the shims + C oracle
    python tests/golden/make_golden.py [--big | --only-big | --only-hci | --only-rdm | --only-enpt2 | --only-trdm]

Outputs (all committed):
  kat_<system>.npz      integrals of the FCIDUMP files the reference's known-answer
                        tests use (pyci/test/data/*.fcidump), unique 8-fold
                        elements only, plus the tests' energies (kat.json)
  csr_<case>.npz        the reference's own CSR (data / indices / indptr) for small
                        synthetic cases, built by pyci.sparse_op of the reference
  hci_<case>.npz        one heat-bath CI step of the reference (pyci.add_hci): input
                        determinants and coefficients, and the set it added
  rdm_<case>.npz        the reference's pyci.compute_rdms (DOCI d0/d2, FullCI
                        rdm1/rdm2) of seeded random coefficient vectors
  trdm_<case>.npz       the reference's pyci.compute_transition_rdms of two sets
  enpt2_<case>.npz      the reference's pyci.compute_enpt2 of a solved ground state
  digests.json          order-independent digests of the reference CSR for the
                        larger synthetic workloads, and reference eigenvalues
The reference is imported from oracle/_ref (the unchanged sources compiled
against project-written Eigen/Spectra/phmap shims).  With --big, the
12-orbital FCI and 32-orbital DOCI workloads are added (minutes, ~40 GB RAM);
their CSR comes from the C oracle, whose output is bit-identical to the
reference's on every smaller case checked here.
"""

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFROOT = os.environ.get("PYCI_REFERENCE", "")
if not os.path.isdir(os.path.join(REFROOT, "pyci", "src")):
    sys.exit("set PYCI_REFERENCE to the reference source tree (the one oracle/_ref was built from)")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from pyci_gb300.synth import synthetic_integrals, config_seed  # noqa: E402

# Known-answer energies of pyci/test/test_routines.py:37-54 (test_solve_sparse)
# and the notebook value (notebooks/pyci_tutorial.ipynb cell 7).
KATS = [
    ("li2_ccpvdz", "doci", (3, 3), -14.878455349),
    ("be_ccpvdz", "doci", (2, 2), -14.600556994),
    ("be_ccpvdz", "fullci", (2, 2), -14.617409507),
    ("h2o_ccpvdz", "doci", (5, 5), -75.634588422),
]

from digest import digest  # noqa: E402


def pack_8fold(two):
    n = two.shape[0]
    g = two.transpose(0, 2, 1, 3)  # chemist's (pq|rs)
    keys, vals = [], []
    for p in range(n):
        for q in range(p + 1):
            pq = p * (p + 1) // 2 + q
            for r in range(n):
                for s in range(r + 1):
                    rs = r * (r + 1) // 2 + s
                    if pq >= rs:
                        v = g[p, q, r, s]
                        if v != 0.0:
                            keys.append((p, q, r, s))
                            vals.append(v)
    return np.array(keys, dtype=np.uint8 if n < 256 else np.uint16), np.array(vals)


def kat_fixtures(pyci):
    meta = []
    for name in sorted({k[0] for k in KATS}):
        ham = pyci.secondquant_op(os.path.join(REFROOT, "pyci", "test", "data", name + ".fcidump"))
        keys, vals = pack_8fold(np.asarray(ham.two_mo))
        np.savez_compressed(os.path.join(HERE, "kat_%s.npz" % name), ecore=np.float64(ham.ecore),
                            one_mo=np.asarray(ham.one_mo), keys=keys, vals=vals)
    for name, kind, occs, energy in KATS:
        meta.append({"system": name, "wfn": kind, "occs": list(occs), "energy": energy})
    return meta


def ref_csr(pyci, kind, n, nu, nd, ecore, one, two, nrow=-1, ncol=-1, symm=True, exc=None):
    ham = pyci.secondquant_op(ecore, one, two)
    W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn, "genci": pyci.genci_wfn}[kind]
    wfn = W(n, nu, nd)
    if exc is None:
        wfn.add_all_dets()
    else:
        pyci.add_excitations(wfn, *exc)
    op = pyci.sparse_op(ham, wfn, nrow, ncol, symm)
    return op, wfn


CSR_CASES = [
    # name, kind, nbasis, nocc_up, nocc_dn, excitations (None = all), nrow, ncol, symmetric, seed
    ("fci_6_3_2", "fullci", 6, 3, 2, None, -1, -1, True, 11),
    ("fci_7_3_3_cisd", "fullci", 7, 3, 3, (0, 1, 2), -1, -1, True, 12),
    ("fci_7_3_2_rect", "fullci", 7, 3, 2, (0, 1, 2), 20, -1, False, 13),
    ("fci_5_2_2_sym_nrow", "fullci", 5, 2, 2, None, 60, -1, True, 14),
    ("doci_10_4", "doci", 10, 4, 4, None, -1, -1, True, 15),
    ("doci_12_5_cisd_rect", "doci", 12, 5, 5, (0, 1, 2), 40, 90, False, 16),
    ("doci_9_3_ncol", "doci", 9, 3, 3, None, -1, 50, True, 17),
    ("genci_10_4", "genci", 10, 4, 0, None, -1, -1, True, 18),
    ("genci_12_3_cisd_rect", "genci", 12, 3, 0, (0, 1, 2), 30, -1, False, 19),
]


def csr_fixtures(pyci):
    meta = []
    for name, kind, n, nu, nd, exc, nrow, ncol, symm, seed in CSR_CASES:
        ecore, one, two = synthetic_integrals(n, seed)
        op, wfn = ref_csr(pyci, kind, n, nu, nd, ecore, one, two, nrow, ncol, symm, exc)
        dets = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1)
        x = np.random.default_rng(seed).normal(size=op.shape[1])
        keys, vals = pack_8fold(two)
        # The integrals travel with the fixture: numpy's einsum may round the
        # last bit differently on another machine, and the CSR values are
        # compared bit for bit.
        np.savez_compressed(os.path.join(HERE, "csr_%s.npz" % name), data=op.data(), indices=op.indices(),
                            indptr=op.indptr(), dets=dets, x=x, y=op(x), ecore=np.float64(ecore),
                            one_mo=one, keys=keys, vals=vals)
        meta.append({"name": name, "wfn": kind, "nbasis": n, "nocc_up": nu, "nocc_dn": nd,
                     "excitations": None if exc is None else list(exc), "nrow": nrow, "ncol": ncol,
                     "symmetric": symm, "seed": seed, "size": int(op.size), "shape": list(op.shape)})
    return meta


HCI_CASES = [
    # name, kind, nbasis, nocc_up, nocc_dn, excitations of the input set, seed, eps
    ("doci_10_4", "doci", 10, 4, 4, (0, 1), 21, 1e-3),
    ("fci_7_3_2", "fullci", 7, 3, 2, (0, 1), 22, 1e-3),
    ("genci_10_4", "genci", 10, 4, 0, (0, 1), 23, 1e-3),
]


def sorted_rows(a):
    r"""Rows of a uint64 array in lexicographic order (an order-free set)."""
    a = np.asarray(a, dtype=np.uint64).reshape(a.shape[0], -1)
    if a.shape[0] == 0:
        return a
    return a[np.lexsort(a.T[::-1])]


def hci_fixtures(pyci):
    r"""One heat-bath CI step of the reference (pyci.add_hci) per case: the
    input determinants and coefficients, and the determinants it added.  The
    reference merges per-thread hash maps, so its order of the added
    determinants is that of its hash map; the fixture keeps them as a sorted
    set.  The last case starts from a solved be/cc-pVDZ FullCI(2,2) Hartree-Fock
    determinant, as the reference's test_run_hci does."""
    meta = []
    cases = [(name, kind, n, nu, nd, exc, seed, eps, None) for name, kind, n, nu, nd, exc, seed, eps in HCI_CASES]
    cases.append(("be_fci_hf", "fullci", None, 2, 2, None, None, 1e-4, "be_ccpvdz"))
    for name, kind, n, nu, nd, exc, seed, eps, system in cases:
        W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn, "genci": pyci.genci_wfn}[kind]
        if system is None:
            ecore, one, two = synthetic_integrals(n, seed)
            ham = pyci.secondquant_op(ecore, one, two)
            wfn = W(n, nu, nd)
            pyci.add_excitations(wfn, *exc)
            coeffs = np.random.default_rng(seed).normal(size=len(wfn))
            coeffs /= np.linalg.norm(coeffs)
        else:
            ham = pyci.secondquant_op(os.path.join(REFROOT, "pyci", "test", "data", system + ".fcidump"))
            ecore, one, two = float(ham.ecore), np.asarray(ham.one_mo), np.asarray(ham.two_mo)
            n = ham.nbasis
            wfn = W(n, nu, nd)
            wfn.add_hartreefock_det()
            op = pyci.sparse_op(ham, wfn)
            es, cs = op.solve(n=1, tol=1.0e-6)
            coeffs = np.asarray(cs[0])
        dets = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1).copy()
        nadded = pyci.add_hci(ham, wfn, coeffs, eps=eps, nthread=1)
        after = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1)
        added = after[dets.shape[0]:]
        keys, vals = pack_8fold(two)
        np.savez_compressed(os.path.join(HERE, "hci_%s.npz" % name), dets=dets, coeffs=coeffs,
                            added=sorted_rows(added), ecore=np.float64(ecore), one_mo=one, keys=keys, vals=vals)
        meta.append({"name": name, "wfn": kind, "nbasis": n, "nocc_up": nu, "nocc_dn": nd, "eps": eps,
                     "seed": seed, "system": system, "ndet": int(dets.shape[0]), "nadded": int(nadded)})
        print("hci", name, dets.shape[0], "->", nadded, flush=True)
    return meta


RDM_CASES = [
    # name, kind, nbasis, nocc_up, nocc_dn, excitations of the set (None = all), seed
    ("doci_10_4", "doci", 10, 4, 4, None, 51),
    ("doci_12_5_cisd", "doci", 12, 5, 5, (0, 1, 2), 52),
    ("fci_6_3_2", "fullci", 6, 3, 2, None, 53),
    ("fci_7_3_3_cisd", "fullci", 7, 3, 3, (0, 1, 2), 54),
]


def rdm_fixtures(pyci):
    r"""The reference's pyci.compute_rdms of seeded random (normalised)
    coefficient vectors on full and CISD determinant sets, and its
    pyci.spinize_rdms of them."""
    meta = []
    for name, kind, n, nu, nd, exc, seed in RDM_CASES:
        W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[kind]
        wfn = W(n, nu, nd)
        if exc is None:
            wfn.add_all_dets()
        else:
            pyci.add_excitations(wfn, *exc)
        coeffs = np.random.default_rng(seed).normal(size=len(wfn))
        coeffs /= np.linalg.norm(coeffs)
        rdm1, rdm2 = pyci.compute_rdms(wfn, coeffs)
        spin1, spin2 = pyci.spinize_rdms(rdm1, rdm2)
        dets = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1)
        np.savez_compressed(os.path.join(HERE, "rdm_%s.npz" % name), dets=dets, coeffs=coeffs,
                            rdm1=np.asarray(rdm1), rdm2=np.asarray(rdm2), spin1=spin1, spin2=spin2)
        meta.append({"name": name, "wfn": kind, "nbasis": n, "nocc_up": nu, "nocc_dn": nd, "seed": seed,
                     "ndet": len(wfn)})
        print("rdm", name, len(wfn), flush=True)
    return meta


TRDM_CASES = [
    # name, kind, nbasis, nocc_up, nocc_dn, excitations of wave function 1 (None = all),
    # of wave function 2, seed
    ("doci_10_4", "doci", 10, 4, 4, (0, 1, 2), None, 61),
    ("fci_6_3_2", "fullci", 6, 3, 2, (0, 1), None, 62),
    ("fci_7_3_3", "fullci", 7, 3, 3, None, (0, 1, 2), 63),
]


def trdm_fixtures(pyci):
    r"""The reference's pyci.compute_transition_rdms between two wave functions
    (different determinant sets) with seeded random coefficient vectors."""
    meta = []
    for name, kind, n, nu, nd, exc1, exc2, seed in TRDM_CASES:
        W = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[kind]
        wfns = []
        for exc in (exc1, exc2):
            w = W(n, nu, nd)
            if exc is None:
                w.add_all_dets()
            else:
                pyci.add_excitations(w, *exc)
            wfns.append(w)
        rng = np.random.default_rng(seed)
        c1 = rng.normal(size=len(wfns[0]))
        c2 = rng.normal(size=len(wfns[1]))
        rdm1, rdm2 = pyci.compute_transition_rdms(wfns[0], wfns[1], c1, c2)
        d1 = np.asarray(wfns[0].to_det_array()).reshape(len(wfns[0]), -1)
        d2 = np.asarray(wfns[1].to_det_array()).reshape(len(wfns[1]), -1)
        np.savez_compressed(os.path.join(HERE, "trdm_%s.npz" % name), dets1=d1, coeffs1=c1, dets2=d2, coeffs2=c2,
                            rdm1=np.asarray(rdm1), rdm2=np.asarray(rdm2))
        meta.append({"name": name, "wfn": kind, "nbasis": n, "nocc_up": nu, "nocc_dn": nd, "seed": seed,
                     "ndet1": len(wfns[0]), "ndet2": len(wfns[1])})
        print("trdm", name, len(wfns[0]), len(wfns[1]), flush=True)
    return meta


ENPT2_CASES = [
    # name, kind, nbasis, nocc_up, nocc_dn, excitations of the set, seed, eps
    ("doci_10_4", "doci", 10, 4, 4, (0, 1), 71, 1e-4),
    ("fci_7_3_2", "fullci", 7, 3, 2, (0, 1), 72, 1e-5),
    ("fci_8_3_3", "fullci", 8, 3, 3, (0, 1, 2), 73, 1e-3),
]
# pyci/test/test_routines.py:473-491 (test_enpt2): system, wave function,
# occupations and the expected ENPT2 energy (the cases whose data files exist).
ENPT2_KATS = [
    ("li2_ccpvdz", "doci", (3, 3), -14.90042952400693),
    ("be_ccpvdz", "doci", (2, 2), -14.61920612157886),
    ("be_ccpvdz", "fullci", (2, 2), -14.61740346031583),
    ("h2o_ccpvdz", "doci", (5, 5), -76.04227376501808),
]


def enpt2_fixtures(pyci):
    r"""The reference's pyci.compute_enpt2 (one thread) on the ground state of
    seeded synthetic Hamiltonians over CISD-like sets, and the known answers of
    its own test_enpt2."""
    meta = []
    for name, kind, n, nu, nd, exc, seed, eps in ENPT2_CASES:
        ecore, one, two = synthetic_integrals(n, seed)
        ham = pyci.secondquant_op(ecore, one, two)
        wfn = {"doci": pyci.doci_wfn, "fullci": pyci.fullci_wfn}[kind](n, nu, nd)
        pyci.add_excitations(wfn, *exc)
        op = pyci.sparse_op(ham, wfn)
        es, cs = op.solve(n=1, tol=1e-12)
        e2 = pyci.compute_enpt2(ham, wfn, cs[0], es[0], eps, nthread=1)
        dets = np.asarray(wfn.to_det_array()).reshape(len(wfn), -1)
        keys, vals = pack_8fold(two)
        np.savez_compressed(os.path.join(HERE, "enpt2_%s.npz" % name), dets=dets, coeffs=np.asarray(cs[0]),
                            energy=np.float64(es[0]), result=np.float64(e2), ecore=np.float64(ecore), one_mo=one,
                            keys=keys, vals=vals)
        meta.append({"name": name, "wfn": kind, "nbasis": n, "nocc_up": nu, "nocc_dn": nd, "seed": seed, "eps": eps,
                     "ndet": len(wfn), "energy": float(es[0]), "enpt2": float(e2)})
        print("enpt2", name, len(wfn), es[0], e2, flush=True)
    kats = [{"system": s, "wfn": w, "occs": list(o), "enpt2": e} for s, w, o, e in ENPT2_KATS]
    return meta, kats


WORKLOADS = [
    # name, kind, nbasis, nocc, config index (seed 1000 + index), roots
    ("fci_8_4_4", "fullci", 8, (4, 4), 1, 4),
    ("doci_24_6", "doci", 24, (6, 6), 2, 1),
]
BIG_WORKLOADS = [
    ("fci_12_5_5", "fullci", 12, (5, 5), 3, 4),
    ("doci_32_8", "doci", 32, (8, 8), 4, 4),
]


def workload_digests(pyci, big):
    out = {}
    for name, kind, n, occs, cfg, nroot in WORKLOADS + (BIG_WORKLOADS if big else []):
        t0 = time.time()
        ecore, one, two = synthetic_integrals(n, config_seed(cfg))
        k = {"doci": O.DOCI, "fullci": O.FULLCI}[kind]
        if (name, kind, n, occs, cfg, nroot) in WORKLOADS:
            op, wfn = ref_csr(pyci, kind, n, occs[0], occs[1], ecore, one, two)
            data, indices, indptr = op.data(), op.indices(), op.indptr()
            source = "reference"
        else:
            dets = O.all_dets(k, n, occs[0], occs[1])
            data, indices, indptr = O.build_csr(k, n, occs[0], occs[1], dets, one, two)
            del dets
            source = "oracle (bit-identical to the reference on every checked case)"
        d = digest(data, indices, indptr)
        evals = O.lowest_eigenvalues(data, indices, indptr, nroot=nroot, tol=1e-12)
        d.update({"wfn": kind, "nbasis": n, "occs": list(occs), "seed": config_seed(cfg),
                  "nrow": int(indptr.shape[0] - 1), "eigenvalues": [float(e) for e in evals],
                  "csr_source": source, "seconds": round(time.time() - t0, 1)})
        out[name] = d
        print(name, d["nnz"], d["eigenvalues"], d["seconds"], "s", flush=True)
        del data, indices, indptr
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true")
    ap.add_argument("--only-big", action="store_true")
    ap.add_argument("--only-hci", action="store_true")
    ap.add_argument("--only-rdm", action="store_true")
    ap.add_argument("--only-enpt2", action="store_true")
    ap.add_argument("--only-trdm", action="store_true")
    args = ap.parse_args()
    import pyci  # the reference, from oracle/_ref
    path = os.path.join(HERE, "digests.json")
    if args.only_hci or args.only_rdm or args.only_enpt2 or args.only_trdm:
        with open(path) as f:
            meta = json.load(f)
        if args.only_trdm:
            meta["trdm_cases"] = trdm_fixtures(pyci)
        if args.only_enpt2:
            meta["enpt2_cases"], meta["enpt2_kats"] = enpt2_fixtures(pyci)
        if args.only_hci:
            meta["hci_cases"] = hci_fixtures(pyci)
        if args.only_rdm:
            meta["rdm_cases"] = rdm_fixtures(pyci)
    elif args.only_big:
        with open(path) as f:
            meta = json.load(f)
        meta["workloads"].update({k: v for k, v in workload_digests(pyci, True).items()
                                  if k in dict((w[0], 1) for w in BIG_WORKLOADS)})
    else:
        enpt2_cases, enpt2_kats = enpt2_fixtures(pyci)
        meta = {"kats": kat_fixtures(pyci), "csr_cases": csr_fixtures(pyci), "hci_cases": hci_fixtures(pyci),
                "rdm_cases": rdm_fixtures(pyci), "trdm_cases": trdm_fixtures(pyci), "enpt2_cases": enpt2_cases,
                "enpt2_kats": enpt2_kats,
                "workloads": workload_digests(pyci, args.big)}
    with open(path, "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
