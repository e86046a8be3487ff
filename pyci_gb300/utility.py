r"""Host-side helpers around compute_rdms, restating the reference's numpy
utilities of the same names (pyci/utility.py): the reduced seniority-zero
integrals that pair with DOCI's (d0, d2) matrices, and the conversion of
DOCI matrices or FullCI spin blocks to spin-orbital RDMs."""

import numpy as np

__all__ = ["reduce_senzero_integrals", "spinize_rdms"]


def reduce_senzero_integrals(h, v, w, nocc):
    r"""(rv, rw) such that E = ecore + sum(rv * d0) + sum(rw * d2) for a DOCI
    wave function with `nocc` pairs (pyci/utility.py:59-91): the one-electron
    energies are spread over the pair terms, rv = v + diag(h) f and
    rw = w + (h_p + h_q) f with f = 2 / (2 nocc - 1)."""
    h = np.asarray(h, dtype=np.float64)
    factor = 2.0 / (nocc * 2 - 1)
    rv = np.diag(h) * factor + np.asarray(v, dtype=np.float64)
    rw = (h[:, None] + h[None, :]) * factor + np.asarray(w, dtype=np.float64)
    return rv, rw


def spinize_rdms(d1, d2):
    r"""Spin-orbital (2n x 2n, 2n^4) RDMs from DOCI's (d0, d2) matrices or
    FullCI's spin blocks (pyci/utility.py:94-150); alpha orbitals first.

    DOCI: gamma_pp = d0_pp in both spins; the pair terms d0 (p p -> q q,
    opposite spins) and d2 (p q -> p q, every spin pairing) are placed, then
    the two-particle RDM is antisymmetrised in each index pair.  FullCI: the
    aa / bb / aaaa / bbbb / abab blocks are placed, with baba, abba and baab
    from abab by index exchange."""
    d1 = np.asarray(d1, dtype=np.float64)
    d2 = np.asarray(d2, dtype=np.float64)
    n = d1.shape[1]
    a, b = slice(0, n), slice(n, 2 * n)
    rdm1 = np.zeros((2 * n, 2 * n))
    rdm2 = np.zeros((2 * n,) * 4)
    if d1.ndim == 2:
        idx = np.arange(n)
        rdm1[idx, idx] = np.diagonal(d1)
        rdm1[idx + n, idx + n] = np.diagonal(d1)
        p, q = np.meshgrid(idx, idx, indexing="ij")
        for s, t in ((0, n), (n, 0)):
            rdm2[p + s, p + t, q + s, q + t] += d1  # abab / baba pair transfer
        for s, t in ((0, 0), (n, n), (0, n), (n, 0)):
            rdm2[p + s, q + t, p + s, q + t] += d2  # aaaa, bbbb, abab, baba
        rdm2 = rdm2 - rdm2.transpose(1, 0, 2, 3)
        rdm2 = rdm2 - rdm2.transpose(0, 1, 3, 2)
        rdm2 *= 0.5
    else:
        rdm1[a, a] = d1[0]
        rdm1[b, b] = d1[1]
        rdm2[a, a, a, a] = d2[0]
        rdm2[b, b, b, b] = d2[1]
        rdm2[a, b, a, b] = d2[2]
        rdm2[b, a, b, a] = d2[2].transpose(1, 0, 3, 2)
        rdm2[a, b, b, a] = -d2[2].transpose(0, 1, 3, 2)
        rdm2[b, a, a, b] = -d2[2].transpose(1, 0, 2, 3)
    return rdm1, rdm2
