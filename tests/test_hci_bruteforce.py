r"""Heat-bath CI selection from its definition, on the CPU: with the dense
Hamiltonian of a whole FullCI or DOCI space (the oracle's CSR), a selected
space P with coefficients c adds exactly the determinants k outside P with

    max over i in P of |H_ki c_i| > eps

(pyci/src/hci.cpp compares the excitation's matrix element, without its
phase, with eps / |c_i|: the full single-excitation element for FullCI
singles, the antisymmetrised integral for doubles, v_kl for DOCI pair moves).
The oracle's add_hci (which the GPU add_hci matches determinant for
determinant) must return that set, each determinant once."""

import numpy as np
import pytest

import oracle as O
from pyci_gb300.synth import synthetic_integrals


def dense(ref, N):
    return np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)


@pytest.mark.parametrize("kind,n,nu,nd,nsel,eps", [(O.FULLCI, 6, 3, 2, 30, 2e-3), (O.FULLCI, 5, 2, 2, 10, 1e-3),
                                                   (O.DOCI, 9, 3, 3, 15, 1e-3), (O.DOCI, 8, 4, 4, 20, 0.0)])
def test_add_hci_selects_by_the_heat_bath_rule(kind, n, nu, nd, nsel, eps):
    ecore, one, two = synthetic_integrals(n, 70 + n)
    dets = O.all_dets(kind, n, nu, nd)
    N = dets.shape[0]
    H = dense(O.build_csr(kind, n, nu, nd, dets, one, two), N)
    rng = np.random.default_rng(n + nsel)
    P = np.sort(rng.choice(N, size=nsel, replace=False))
    c = rng.normal(size=nsel)
    c /= np.linalg.norm(c)
    W = np.abs(H[:, P] * c[None, :])
    W[P, :] = 0.0  # determinants already in P are never added
    expect = set(np.nonzero(W.max(axis=1) > eps)[0].tolist())
    new = O.add_hci(kind, n, nu, nd, dets[P], c, one, two, eps)
    row = {tuple(int(w) for w in d): i for i, d in enumerate(dets)}
    got = [row[tuple(int(w) for w in d)] for d in new]
    assert len(got) == len(set(got))  # each determinant once
    assert set(got) == expect
    assert 0 < len(expect) < N - nsel or eps == 0.0
