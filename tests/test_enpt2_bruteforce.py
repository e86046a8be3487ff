r"""Epstein-Nesbet second-order energy from its definition, on the CPU: with
the dense Hamiltonian of a whole FullCI or DOCI space (the oracle's CSR),
a selected space P with its ground state c and energy E (ecore included),

    E_PT2 = E + sum over k outside P of (sum_i H_ki c_i)^2 / (E - H_kk - ecore),

against the oracle's compute_enpt2 with eps = 0 (every term kept).  For a
DOCI wave function the reference evaluates the correction in the FullCI
space of the same electrons (pyci/src/enpt2.cpp converts the wave function
first), so k runs over every FullCI determinant outside P, broken pairs
included.  The oracle restates pyci/src/enpt2.cpp and is pinned to the
reference's own values elsewhere; this checks it against the formula
independently."""

import numpy as np
import pytest

import oracle as O
from pyci_gb300.synth import synthetic_integrals


def dense(ref, N):
    return np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)


@pytest.mark.parametrize("kind,n,nu,nd,nsel", [(O.FULLCI, 6, 3, 2, 40), (O.FULLCI, 5, 2, 2, 25),
                                               (O.DOCI, 8, 3, 3, 12)])
def test_enpt2_equals_the_formula(kind, n, nu, nd, nsel):
    ecore, one, two = synthetic_integrals(n, 40 + n)
    dets = O.all_dets(kind, n, nu, nd)
    N = dets.shape[0]
    H = dense(O.build_csr(kind, n, nu, nd, dets, one, two), N)
    # Selected space: the nsel determinants of lowest diagonal energy.
    P = np.sort(np.argsort(np.diag(H), kind="stable")[:nsel])
    w, v = np.linalg.eigh(H[np.ix_(P, P)])
    c = v[:, 0]
    energy = w[0] + ecore
    got = O.compute_enpt2(kind, n, nu, nd, dets[P], c, one, two, energy, ecore, 0.0)
    if kind == O.DOCI:
        # The FullCI image: pair mask -> (alpha, beta) = (mask, mask).
        fdets = O.all_dets(O.FULLCI, n, nu, nd)
        H = dense(O.build_csr(O.FULLCI, n, nu, nd, fdets, one, two), fdets.shape[0])
        row = {(int(a), int(b)): i for i, (a, b) in enumerate(fdets)}
        P = np.array([row[(int(d[0]), int(d[0]))] for d in dets[P]])
        N = fdets.shape[0]
    ext = np.setdiff1d(np.arange(N), P)
    V = H[np.ix_(ext, P)] @ c
    expect = energy + np.sum(V * V / (energy - np.diag(H)[ext] - ecore))
    assert got == pytest.approx(expect, rel=0, abs=1e-11 * max(1.0, abs(expect - energy)))
    assert got < energy  # a ground state: every denominator is negative
