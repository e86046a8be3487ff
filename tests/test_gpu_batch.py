r"""The batched multi-problem solver (pyci_gpu_batch_solve): independent
operators of uneven size solved together must give each problem's own lowest
4 eigenvalues, as single solves do."""

import numpy as np
import pytest

import oracle as O
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

PROBLEMS = [  # kind, nbasis, nocc_up, nocc_dn, seed
    (capi.WFN_FULLCI, 4, 2, 2, 41), (capi.WFN_FULLCI, 6, 2, 2, 42), (capi.WFN_FULLCI, 6, 3, 3, 43),
    (capi.WFN_FULLCI, 7, 3, 2, 44), (capi.WFN_DOCI, 10, 4, 4, 45), (capi.WFN_FULLCI, 8, 4, 4, 46),
    (capi.WFN_FULLCI, 8, 2, 2, 47),
]


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def build_all(ctx):
    from math import comb
    ops, ecore, ref = [], [], []
    for kind, n, nu, nd, seed in PROBLEMS:
        e, one, two = synthetic_integrals(n, seed)
        e = 0.25 * seed  # a nonzero core energy per problem
        nd_ = comb(n, nu) * (comb(n, nd) if kind == capi.WFN_FULLCI else 1)
        csr = capi.Csr(ctx, kind, n, nu, nd, None, one, two, flags=capi.BUILD_FULL_COLEX, ndet=nd_)
        ops.append(csr)
        ecore.append(e)
        ref.append(csr.solve(n=4, tol=1e-10, ecore=e)[0])
    return ops, np.array(ecore), np.array(ref)


@pytest.mark.parametrize("mode, atol", [(capi.SOLVE_FP64, 1e-8), (capi.SOLVE_MIXED, 1e-6)])
def test_batch_matches_single_solves(ctx, mode, atol):
    ops, ecore, ref = build_all(ctx)
    evals, stats = capi.batch_solve(ctx, ops, ecore, n=4, tol=1e-9 if mode == capi.SOLVE_FP64 else 1e-6, mode=mode)
    assert evals.shape == (len(ops), 4)
    for p in range(len(ops)):
        assert np.all(np.diff(evals[p]) <= 0)  # decreasing, like the single solve
        np.testing.assert_allclose(evals[p], ref[p], rtol=0, atol=atol)
    assert stats["matvecs"] > 0
    for c in ops:
        c.free()


def test_batch_rejects_bad_input(ctx):
    e, one, two = synthetic_integrals(6, 1)
    dets = O.all_dets(O.FULLCI, 6, 2, 2)
    rect = capi.Csr(ctx, capi.WFN_FULLCI, 6, 2, 2, dets, one, two, nrow=50, symmetric=False)
    with pytest.raises(TypeError):
        capi.batch_solve(ctx, [rect], [0.0])
    rect.free()
