r"""The CI Hamiltonian from second quantization, on the CPU: for small FullCI
and DOCI spaces every matrix element <Phi_i| H |Phi_j> of

    H = sum_PQ h_PQ a+_P a_Q + 1/2 sum_PQRS <PQ|RS> a+_P a+_Q a_S a_R

(spin orbitals alpha 0..n-1 then beta n..2n-1; <PQ|RS> = <pq|rs> when P, R
and Q, S have equal spins, physicist's integrals as pyci's two_mo) is formed
by applying the operators to every determinant, and compared with the
oracle's CSR, which is bit-identical to the reference's sparse_op
(pyci/src/sparseop.cpp add_row).  A DOCI space gets the projection of the
same H onto its paired determinants.  This pins the Slater-Condon rules,
phases and orbital orderings independently of the reference's code."""

import itertools

import numpy as np
import pytest

import oracle as O
from pyci_gb300.synth import synthetic_integrals
from test_rdm_bruteforce import annihilate, apply, create, spin_orbitals


def second_quantized_matrix(kind, n, dets, one, two):
    states = [spin_orbitals(kind, d, n) for d in dets]
    index = {s: i for i, s in enumerate(states)}
    m = 2 * n
    spin = [p // n for p in range(m)]
    orb = [p % n for p in range(m)]
    H = np.zeros((len(states), len(states)))
    for j, sj in enumerate(states):
        for P, Q in itertools.product(range(m), repeat=2):
            if spin[P] != spin[Q]:
                continue
            r = apply([(create, P), (annihilate, Q)], sj)
            if r is not None and r[1] in index:
                H[index[r[1]], j] += r[0] * one[orb[P], orb[Q]]
        for P, Q, R, S in itertools.product(range(m), repeat=4):
            if spin[P] != spin[R] or spin[Q] != spin[S]:
                continue
            r = apply([(create, P), (create, Q), (annihilate, S), (annihilate, R)], sj)
            if r is not None and r[1] in index:
                H[index[r[1]], j] += 0.5 * r[0] * two[orb[P], orb[Q], orb[R], orb[S]]
    return H


@pytest.mark.parametrize("kind,n,nu,nd", [(O.FULLCI, 4, 2, 2), (O.FULLCI, 4, 3, 1), (O.FULLCI, 3, 2, 0),
                                          (O.DOCI, 5, 2, 2), (O.DOCI, 4, 1, 1)])
def test_csr_equals_second_quantized_hamiltonian(kind, n, nu, nd):
    ecore, one, two = synthetic_integrals(n, 90 + n)
    dets = O.all_dets(kind, n, nu, nd)
    N = dets.shape[0]
    ref = O.build_csr(kind, n, nu, nd, dets, one, two)
    H = np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)
    H2 = second_quantized_matrix(kind, n, dets, one, two)
    np.testing.assert_allclose(H, H2, rtol=0, atol=1e-12 * np.abs(H2).max())


@pytest.mark.parametrize("n,nocc", [(6, 3), (7, 2)])
def test_genci_csr_equals_spinless_second_quantized_hamiltonian(n, nocc):
    r"""GenCI determinants are sets of nocc occupied spin-orbitals out of n,
    with the integrals given over those spin-orbitals (no spin blocks).  The
    oracle's Slater-Condon form (kind GENCI; the GPU build with
    PYCI_BUILD_GENCI_EXACT) equals the operator-algebra matrix.  The
    reference's own GenCI row loop, reproduced as kind GENCI_REF and by the
    GPU's default GenCI build, differs from it: it walks 2 n - nocc virtual
    entries where n - nocc exist."""
    ecore, one, two = synthetic_integrals(n, 95 + n)
    dets = O.all_dets(O.GENCI, n, nocc, 0)
    N = dets.shape[0]
    states = [tuple(p for p in range(n) if int(d[0]) >> p & 1) for d in dets]
    index = {s: i for i, s in enumerate(states)}
    H2 = np.zeros((N, N))
    for j, sj in enumerate(states):
        for P, Q in itertools.product(range(n), repeat=2):
            r = apply([(create, P), (annihilate, Q)], sj)
            if r is not None and r[1] in index:
                H2[index[r[1]], j] += r[0] * one[P, Q]
        for P, Q, R, S in itertools.product(range(n), repeat=4):
            r = apply([(create, P), (create, Q), (annihilate, S), (annihilate, R)], sj)
            if r is not None and r[1] in index:
                H2[index[r[1]], j] += 0.5 * r[0] * two[P, Q, R, S]
    ref = O.build_csr(O.GENCI, n, nocc, 0, dets, one, two)
    H = np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)
    np.testing.assert_allclose(H, H2, rtol=0, atol=1e-12 * np.abs(H2).max())
