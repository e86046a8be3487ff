r"""The fused Ritz step of the mixed-precision eigensolver (one pass over the
subspace vectors for the Ritz vectors, the residuals and their norms, the
preconditioner and the first Gram product of the block orthonormalisation)
against the separate kernels (PYCI_GPU_RITZ=separate) and the oracle's
eigenvalues: FullCI and DOCI operators, row counts that are and are not
multiples of 4, thick restarts (a small subspace), and 2 to 8 tracked pairs
(subspaces wider than the fused step takes run the separate kernels)."""

import numpy as np
import pytest

import oracle as O
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

# (kind, nbasis, alpha, beta, roots, ncv): 63,504 rows; 10,584 rows with a
# 16-vector subspace (thick restarts); 126 rows (not a multiple of 4); 792 rows
# with 7 roots (8 tracked pairs, a 112-vector subspace); 3,920 rows, 1 root.
CASES = [("fci", 10, 5, 5, 4, -1), ("fci", 9, 4, 3, 4, 16), ("doci", 9, 4, 4, 2, -1),
         ("doci", 12, 5, 5, 7, -1), ("fci", 8, 4, 3, 1, -1)]


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("kind,n,na,nb,nroot,ncv", CASES)
def test_fused_ritz_step(ctx, monkeypatch, kind, n, na, nb, nroot, ncv):
    ecore, one, two = synthetic_integrals(n, 1019)
    wk, ck = (O.FULLCI, capi.WFN_FULLCI) if kind == "fci" else (O.DOCI, capi.WFN_DOCI)
    dets = O.all_dets(wk, n, na, nb)
    ref = O.build_csr(wk, n, na, nb, dets, one, two)
    e_ref = O.lowest_eigenvalues(*ref, nroot=nroot)
    csr = capi.Csr(ctx, ck, n, na, nb, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    runs = {}
    for how in ("fused", "separate"):
        if how == "separate":
            monkeypatch.setenv("PYCI_GPU_RITZ", "separate")
        else:
            monkeypatch.delenv("PYCI_GPU_RITZ", raising=False)
        evals, evecs, st = csr.solve(n=nroot, ncv=ncv, tol=1e-8, mode=capi.SOLVE_MIXED)
        np.testing.assert_allclose(np.sort(evals), e_ref, atol=1e-6)
        # Eigenvectors: unit norm, Rayleigh quotients equal to the eigenvalues.
        for j in range(nroot):
            v = evecs[j]
            assert abs(np.dot(v, v) - 1.0) < 1e-6
            assert abs(np.dot(v, O.spmv(*ref, v)) - evals[j]) < 1e-6
        runs[how] = (np.sort(evals), st)
    (ef, sf), (es, ss) = runs["fused"], runs["separate"]
    np.testing.assert_allclose(ef, es, atol=1e-7)
    # FP32 rounding differs between the two forms; over many thick restarts
    # the iteration counts drift apart by a few (a quarter at most: a gross
    # difference, such as a residual left on a plateau, shows as several
    # times the iterations).
    assert abs(sf["iterations"] - ss["iterations"]) <= max(3, ss["iterations"] // 4), (sf, ss)
    if ncv < 0 and nroot <= 4:
        # One read-back per iteration fewer (the Gram product of the
        # orthonormalisation comes with the residual norms).
        assert sf["host_syncs"] < ss["host_syncs"], (sf, ss)
    csr.free()
