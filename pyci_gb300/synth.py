r"""Seeded synthetic molecular integrals for benchmarks and tests.

Recipe (all draws from ``numpy.random.default_rng(seed)`` in this order):

1. ``h = diag(linspace(-2, 1, n))``;
2. ``E ~ N(0, 0.05)`` of shape (n, n); ``h += triu(E, 1) + triu(E, 1).T``;
3. for L = 1..2n: ``A ~ N(0, 0.1 / sqrt(L))``, ``B_L = triu(A) + triu(A, 1).T``;
4. chemist's ``g_pqrs = sum_L B_L[p, q] B_L[r, s]`` (positive semidefinite,
   real 8-fold symmetry);
5. ``two_mo = g.transpose(0, 2, 1, 3)`` -- the physicist's ``<pq|rs>`` layout
   that ``secondquant_op(ecore, one_mo, two_mo)`` expects
   (pyci/src/squantop.cpp:163-183); ``one_mo = h``; ``ecore = 0``.

The two-electron tensor is symmetrised explicitly after step 4 so that every
one of its 8 images is bit-identical, as an FCIDUMP file loaded by the
reference would be (pyci/src/squantop.cpp:134-141).
"""

import numpy as np

__all__ = ["synthetic_integrals", "config_seed"]


def config_seed(index):
    r"""Seed for workload ``index`` (1-based) of the standard configuration list."""
    return 1000 + int(index)


def synthetic_integrals(n, seed):
    r"""Return ``(ecore, one_mo, two_mo)`` for ``n`` orbitals.

    ``one_mo`` is float64[n, n]; ``two_mo`` is float64[n, n, n, n] in physicist's
    notation; both C-contiguous.
    """
    rng = np.random.default_rng(seed)
    h = np.diag(np.linspace(-2.0, 1.0, n))
    e = rng.normal(0.0, 0.05, (n, n))
    h = h + np.triu(e, 1) + np.triu(e, 1).T
    bs = np.empty((2 * n, n, n))
    for L in range(1, 2 * n + 1):
        a = rng.normal(0.0, 0.1 / np.sqrt(L), (n, n))
        bs[L - 1] = np.triu(a) + np.triu(a, 1).T
    g = np.einsum("Lpq,Lrs->pqrs", bs, bs, optimize=True)
    # Exact 8-fold symmetry: average the images, then copy one canonical value.
    g = (g + g.transpose(1, 0, 2, 3)) * 0.5
    g = (g + g.transpose(0, 1, 3, 2)) * 0.5
    g = (g + g.transpose(2, 3, 0, 1)) * 0.5
    g = _canonical_8fold(g)
    two_mo = np.ascontiguousarray(g.transpose(0, 2, 1, 3))
    return 0.0, np.ascontiguousarray(h), two_mo


def _canonical_8fold(g):
    r"""Copy, for each 8-fold orbit of (p, q, r, s), one member's value to all members."""
    n = g.shape[0]
    p, q, r, s = np.meshgrid(*(np.arange(n),) * 4, indexing="ij")
    pq = np.maximum(p, q) * (np.maximum(p, q) + 1) // 2 + np.minimum(p, q)
    rs = np.maximum(r, s) * (np.maximum(r, s) + 1) // 2 + np.minimum(r, s)
    # Canonical member: p >= q, r >= s, pq >= rs.
    cp = np.where(pq >= rs, np.maximum(p, q), np.maximum(r, s))
    cq = np.where(pq >= rs, np.minimum(p, q), np.minimum(r, s))
    cr = np.where(pq >= rs, np.maximum(r, s), np.maximum(p, q))
    cs = np.where(pq >= rs, np.minimum(r, s), np.minimum(p, q))
    return np.ascontiguousarray(g[cp, cq, cr, cs])
