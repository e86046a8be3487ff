r"""Reduced density matrices from their definition, on the CPU: for small
FullCI and DOCI wave functions the spin-orbital RDMs

    gamma[p, q] = <Psi| a+_p a_q |Psi>,
    Gamma[p, q, r, s] = <Psi| a+_p a+_q a_s a_r |Psi>,

are formed by applying creation and annihilation operators to every
determinant (Jordan-Wigner signs, spin orbitals alpha 0..n-1 then beta
n..2n-1), and compared with the oracle's compute_rdms followed by the
package's spinize_rdms (the reference's pyci.spinize_rdms convention, pinned
by its tests on FullCI(2, 1α1β) and FullCI(3, 2α1β) with coefficients
sqrt(1..N), pyci/test/test_routines.py:494-800).  Transition RDMs are
<Psi_1| ... |Psi_2> with the first wave function as the bra.  This checks the
oracle's restatement and the host-side spinization independently of the
reference's code; the GPU RDMs equal the oracle's (GPU tests)."""

import itertools

import numpy as np
import numpy.testing as npt
import pytest

import oracle as O
import pyci_gb300 as pyci


def spin_orbitals(kind, det, n):
    r"""Occupied spin orbitals of one determinant row of the oracle's array."""
    words = [int(w) for w in det]
    if kind == O.FULLCI:
        nw = len(words) // 2
        alpha = sum(w << (64 * i) for i, w in enumerate(words[:nw]))
        beta = sum(w << (64 * i) for i, w in enumerate(words[nw:]))
    else:  # DOCI: one mask of doubly occupied orbitals
        alpha = beta = sum(w << (64 * i) for i, w in enumerate(words))
    occ = [p for p in range(n) if alpha >> p & 1] + [n + p for p in range(n) if beta >> p & 1]
    return tuple(occ)


def annihilate(state, p):
    r"""a_p |state> for a sorted occupation tuple: (sign, state) or None."""
    if p not in state:
        return None
    k = state.index(p)
    return (-1) ** k, state[:k] + state[k + 1:]


def create(state, p):
    if p in state:
        return None
    k = sum(1 for q in state if q < p)
    return (-1) ** k, state[:k] + (p,) + state[k:]


def apply(ops, state):
    r"""Apply operators right to left: ops = [(op, index), ...] in written order."""
    sign = 1
    for op, p in reversed(ops):
        r = op(state, p)
        if r is None:
            return None
        s, state = r
        sign *= s
    return sign, state


def brute_force_rdms(kind, n, dets, coeffs):
    states = [spin_orbitals(kind, d, n) for d in dets]
    index = {s: i for i, s in enumerate(states)}
    m = 2 * n
    g1 = np.zeros((m, m))
    g2 = np.zeros((m, m, m, m))
    for j, sj in enumerate(states):
        cj = coeffs[j]
        if cj == 0.0:
            continue
        for p, q in itertools.product(range(m), repeat=2):
            r = apply([(create, p), (annihilate, q)], sj)
            if r is not None and r[1] in index:
                g1[p, q] += coeffs[index[r[1]]] * r[0] * cj
        for p, q, r_, s in itertools.product(range(m), repeat=4):
            r = apply([(create, p), (create, q), (annihilate, s), (annihilate, r_)], sj)
            if r is not None and r[1] in index:
                g2[p, q, r_, s] += coeffs[index[r[1]]] * r[0] * cj
    return g1, g2


CASES = [
    # (kind, nbasis, nocc_up, nocc_dn, coefficient pattern)
    (O.FULLCI, 2, 1, 1, "sqrt"),
    (O.FULLCI, 3, 2, 1, "sqrt"),
    (O.FULLCI, 4, 2, 2, "random"),
    (O.FULLCI, 4, 3, 1, "random"),
    (O.DOCI, 4, 2, 2, "random"),
    (O.DOCI, 5, 2, 2, "sqrt"),
]


@pytest.mark.parametrize("kind,n,nu,nd,pattern", CASES)
def test_spinized_rdms_equal_their_definition(kind, n, nu, nd, pattern):
    dets = O.all_dets(kind, n, nu, nd)
    N = dets.shape[0]
    if pattern == "sqrt":
        c = np.sqrt(np.arange(1.0, N + 1.0))
    else:
        c = np.random.default_rng(n * 10 + nu).normal(size=N)
    c /= np.linalg.norm(c)
    d1, d2 = O.compute_rdms(kind, n, nu, nd, dets, c)
    rdm1, rdm2 = pyci.spinize_rdms(d1, d2)
    g1, g2 = brute_force_rdms(kind, n, dets, c)
    npt.assert_allclose(rdm1, g1, rtol=0, atol=1e-13)
    npt.assert_allclose(rdm2, g2, rtol=0, atol=1e-13)
    # Traces: N electrons, N (N - 1) pairs.
    ne = nu + nd
    assert np.trace(rdm1) == pytest.approx(ne, abs=1e-12)
    assert np.einsum("pqpq", rdm2) == pytest.approx(ne * (ne - 1), abs=1e-12)


def brute_force_transition_rdms(kind, n, dets1, c1, dets2, c2):
    r"""<Psi_1| a+_p a_q |Psi_2> and <Psi_1| a+_p a+_q a_s a_r |Psi_2>."""
    bra = {spin_orbitals(kind, d, n): c1[i] for i, d in enumerate(dets1)}
    m = 2 * n
    g1 = np.zeros((m, m))
    g2 = np.zeros((m, m, m, m))
    for j, d in enumerate(dets2):
        sj, cj = spin_orbitals(kind, d, n), c2[j]
        for p, q in itertools.product(range(m), repeat=2):
            r = apply([(create, p), (annihilate, q)], sj)
            if r is not None and r[1] in bra:
                g1[p, q] += bra[r[1]] * r[0] * cj
        for p, q, r_, s in itertools.product(range(m), repeat=4):
            r = apply([(create, p), (create, q), (annihilate, s), (annihilate, r_)], sj)
            if r is not None and r[1] in bra:
                g2[p, q, r_, s] += bra[r[1]] * r[0] * cj
    return g1, g2


@pytest.mark.parametrize("n,nu,nd", [(3, 2, 1), (4, 2, 2)])
def test_spinized_fullci_transition_rdms_equal_their_definition(n, nu, nd):
    dets = O.all_dets(O.FULLCI, n, nu, nd)
    N = dets.shape[0]
    rng = np.random.default_rng(n)
    c1, c2 = rng.normal(size=N), rng.normal(size=N)
    c1 /= np.linalg.norm(c1)
    c2 /= np.linalg.norm(c2)
    # A proper subset on one side: excitations that leave it are dropped.
    keep = np.sort(rng.choice(N, size=N - 2, replace=False))
    d1, d2 = O.compute_transition_rdms(O.FULLCI, n, nu, nd, dets[keep], c1[keep], dets, c2)
    t1, t2 = pyci.spinize_rdms(d1, d2)
    g1, g2 = brute_force_transition_rdms(O.FULLCI, n, dets[keep], c1[keep], dets, c2)
    npt.assert_allclose(t1, g1, rtol=0, atol=1e-13)
    npt.assert_allclose(t2, g2, rtol=0, atol=1e-13)


@pytest.mark.parametrize("n,npair", [(6, 3), (8, 2)])
def test_reduced_senzero_integrals_give_the_doci_energy(n, npair):
    r"""E = ecore + sum(rv * d0) + sum(rw * d2) for a DOCI eigenvector, with
    (rv, rw) from reduce_senzero_integrals(h, v, w, npair) and (d0, d2) from
    the oracle's compute_rdms (pyci/utility.py:59-91; the reference's
    test_compute_rdms energy check).  h, v, w are the seniority-zero integrals
    h_p = <p|h|p>, v_pq = <pp|qq>, w_pq = 2 <pq|pq> - <pq|qp>."""
    from pyci_gb300.synth import synthetic_integrals
    ecore, one, two = synthetic_integrals(n, 60 + n)
    dets = O.all_dets(O.DOCI, n, npair, npair)
    N = dets.shape[0]
    ref = O.build_csr(O.DOCI, n, npair, npair, dets, one, two)
    H = np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)
    w_, v_ = np.linalg.eigh(H)
    c = v_[:, 0]
    d0, d2 = O.compute_rdms(O.DOCI, n, npair, npair, dets, c)
    idx = np.arange(n)
    h = one[idx, idx]
    v = two[idx[:, None], idx[:, None], idx[None, :], idx[None, :]]
    w = 2.0 * two[idx[:, None], idx[None, :], idx[:, None], idx[None, :]] \
        - two[idx[:, None], idx[None, :], idx[None, :], idx[:, None]]
    # The host module's secondquant_op derives the same seniority-zero integrals.
    ham = pyci.secondquant_op(ecore, one, two)
    assert np.array_equal(ham.h, h) and np.array_equal(ham.v, v) and np.array_equal(ham.w, w)
    rv, rw = pyci.reduce_senzero_integrals(ham.h, ham.v, ham.w, npair)
    energy = ecore + np.sum(rv * d0) + np.sum(rw * d2)
    assert energy == pytest.approx(w_[0] + ecore, abs=1e-10)


@pytest.mark.parametrize("n,npair", [(5, 2), (6, 3)])
def test_spinized_doci_transition_rdms_equal_their_definition(n, npair):
    dets = O.all_dets(O.DOCI, n, npair, npair)
    N = dets.shape[0]
    rng = np.random.default_rng(10 * n + npair)
    c1, c2 = rng.normal(size=N), rng.normal(size=N)
    c1 /= np.linalg.norm(c1)
    c2 /= np.linalg.norm(c2)
    keep = np.sort(rng.choice(N, size=N - 3, replace=False))
    d1, d2 = O.compute_transition_rdms(O.DOCI, n, npair, npair, dets[keep], c1[keep], dets, c2)
    t1, t2 = pyci.spinize_rdms(d1, d2)
    g1, g2 = brute_force_transition_rdms(O.DOCI, n, dets[keep], c1[keep], dets, c2)
    npt.assert_allclose(t1, g1, rtol=0, atol=1e-13)
    npt.assert_allclose(t2, g2, rtol=0, atol=1e-13)


def genci_states(dets, n):
    out = []
    for d in dets:
        bits = sum(int(w) << (64 * i) for i, w in enumerate(d))
        out.append(tuple(p for p in range(n) if bits >> p & 1))
    return out


def brute_force_genci(n, dets1, c1, dets2, c2):
    r"""<1| a+_p a_q |2> and <1| a+_p a+_q a_s a_r |2> over n spin orbitals."""
    bra = {s: c1[i] for i, s in enumerate(genci_states(dets1, n))}
    g1 = np.zeros((n, n))
    g2 = np.zeros((n, n, n, n))
    for sj, cj in zip(genci_states(dets2, n), c2):
        for p, q in itertools.product(range(n), repeat=2):
            r = apply([(create, p), (annihilate, q)], sj)
            if r is not None and r[1] in bra:
                g1[p, q] += bra[r[1]] * r[0] * cj
        for p, q, r_, s in itertools.product(range(n), repeat=4):
            r = apply([(create, p), (create, q), (annihilate, s), (annihilate, r_)], sj)
            if r is not None and r[1] in bra:
                g2[p, q, r_, s] += bra[r[1]] * r[0] * cj
    return g1, g2


@pytest.mark.parametrize("n,nocc,pattern", [(4, 2, "sqrt"), (6, 3, "random"), (7, 2, "random"), (6, 4, "subset")])
def test_genci_rdms_equal_their_definition(n, nocc, pattern):
    r"""The oracle's definition-based GenCI RDMs (spin orbitals, GenCI's own
    index space) against operator algebra on every determinant; traces N
    and N (N - 1); a subset wave function drops the excitations that leave it."""
    dets = O.all_dets(O.GENCI, n, nocc, 0)
    N = dets.shape[0]
    rng = np.random.default_rng(7 * n + nocc)
    if pattern == "subset":
        keep = np.sort(rng.choice(N, size=N - 4, replace=False))
        dets = dets[keep]
        N = dets.shape[0]
    c = np.sqrt(np.arange(1.0, N + 1.0)) if pattern == "sqrt" else rng.normal(size=N)
    c /= np.linalg.norm(c)
    r1, r2 = O.compute_rdms_genci(n, dets, c)
    g1, g2 = brute_force_genci(n, dets, c, dets, c)
    npt.assert_allclose(r1, g1, rtol=0, atol=1e-13)
    npt.assert_allclose(r2, g2, rtol=0, atol=1e-13)
    assert np.trace(r1) == pytest.approx(nocc, abs=1e-12)
    assert np.einsum("pqpq", r2) == pytest.approx(nocc * (nocc - 1), abs=1e-12)
    # Transition form: a different ket on a proper subset of the bra's space.
    c2 = rng.normal(size=N)
    sub = np.sort(rng.choice(N, size=N - 2, replace=False))
    t1, t2 = O.compute_rdms_genci(n, dets, c, dets[sub], c2[sub])
    h1, h2 = brute_force_genci(n, dets, c, dets[sub], c2[sub])
    npt.assert_allclose(t1, h1, rtol=0, atol=1e-13)
    npt.assert_allclose(t2, h2, rtol=0, atol=1e-13)


def test_genci_rdms_give_the_genci_energy():
    r"""E = sum h_pq rdm1[p][q] + 1/2 sum <pq|rs> rdm2[p][q][r][s] over spin
    orbitals, for the lowest eigenvector of the exact GenCI Hamiltonian (the
    oracle's GenCI build over the true virtuals) of a spin-orbital space
    built from seeded spatial integrals."""
    from pyci_gb300.synth import synthetic_integrals
    nsp, nocc = 4, 3
    ecore, one, two = synthetic_integrals(nsp, 33)
    n = 2 * nsp
    # Spin-orbital integrals: orbital p < nsp is alpha, p >= nsp beta.
    h = np.zeros((n, n))
    g = np.zeros((n, n, n, n))
    for s1 in (0, 1):
        h[s1 * nsp:(s1 + 1) * nsp, s1 * nsp:(s1 + 1) * nsp] = one
        for s2 in (0, 1):
            g[s1 * nsp:(s1 + 1) * nsp, s2 * nsp:(s2 + 1) * nsp, s1 * nsp:(s1 + 1) * nsp,
              s2 * nsp:(s2 + 1) * nsp] = two
    dets = O.all_dets(O.GENCI, n, nocc, 0)
    N = dets.shape[0]
    ref = O.build_csr(O.GENCI, n, nocc, 0, dets, h, g)
    H = np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)
    w, v = np.linalg.eigh(H)
    r1, r2 = O.compute_rdms_genci(n, dets, v[:, 0])
    energy = np.sum(h * r1) + 0.5 * np.einsum("pqrs,pqrs", g, r2)
    assert energy == pytest.approx(w[0], abs=1e-10)
