r"""The implicit-column form of full FullCI operators (columns derived from
per-string tables, values streamed in 4-entry packets, x blocks staged in
shared memory) against the oracle's FP64 product: FP32 and double-float
products on the form (FP64 products on the same operators stay on the CSR),
alpha and beta string spaces equal or different, beta counts that need
padding rows, section-B groups that need padding entries, the eigensolver on
the form, and clones."""

import ctypes

import numpy as np
import pytest

import oracle as O
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

# (nbasis, alpha, beta): beta strings 126 (-> 128 rows per alpha string;
# section-B groups of 21 -> 24 entries), 84 (-> 96) with 126 alpha strings
# (separate alpha and beta tables), 56 (-> 64: 8 padding rows), 252 (-> 256).
CASES = [(9, 4, 4), (9, 4, 3), (8, 4, 3), (10, 5, 5)]


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def split_rows(X):
    hi = X.astype(np.float32)
    lo = (X - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([hi, lo], axis=1))


def build(ctx, n, na, nb, seed=1003):
    ecore, one, two = synthetic_integrals(n, seed)
    dets = O.all_dets(O.FULLCI, n, na, nb)
    ref = O.build_csr(O.FULLCI, n, na, nb, dets, one, two)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, n, na, nb, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    return csr, ref, dets, ecore


@pytest.mark.parametrize("n,na,nb", CASES)
def test_fcix_products_against_oracle(ctx, monkeypatch, n, na, nb):
    import torch
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    csr, ref, dets, _ = build(ctx, n, na, nb)
    csr.prepare_mixed()
    assert csr.has_fcix(), "operator did not get the implicit-column form"
    N = dets.shape[0]
    rng = np.random.default_rng(21)
    for k in (1, 2, 3, 4, 5, 8):
        X = rng.normal(size=(N, k)).astype(np.float32).astype(np.float64)
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xf = torch.tensor(X, dtype=torch.float32, device="cuda")
        yf = torch.full((N, k), np.nan, dtype=torch.float32, device="cuda")
        csr.spmm_device(capi.PREC_FP32, k, xf.data_ptr(), yf.data_ptr(), None)
        torch.cuda.synchronize()
        assert csr.product_form(capi.PREC_FP32, k) == capi.FORM_IMPLICIT
        # FP32 values and accumulation: relative error ~ sqrt(row length) * 2^-24
        assert np.abs(yf.cpu().numpy() - Y_ref).max() / np.abs(Y_ref).max() < 1e-5, k
    for k in (1, 2, 4):
        X = rng.normal(size=(N, k))
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xs = torch.tensor(split_rows(X), device="cuda")
        yd = torch.full((N, k), np.nan, dtype=torch.float64, device="cuda")
        csr.spmm_device(capi.PREC_FP64_DF, k, xs.data_ptr(), yd.data_ptr(), None)
        torch.cuda.synchronize()
        assert csr.product_form(capi.PREC_FP64_DF, k) == capi.FORM_IMPLICIT
        # double-float sums: ~2^-44 relative
        np.testing.assert_allclose(yd.cpu().numpy(), Y_ref, rtol=1e-11, atol=1e-11 * np.abs(Y_ref).max())
    # FP64 arithmetic (CSR) and op(x) with host buffers on the same operator
    X = rng.normal(size=(N, 3))
    Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(3)], axis=1)
    xd = torch.tensor(X, dtype=torch.float64, device="cuda")
    yd = torch.full((N, 3), np.nan, dtype=torch.float64, device="cuda")
    csr.spmm_device(capi.PREC_FP64, 3, xd.data_ptr(), yd.data_ptr(), None)
    torch.cuda.synchronize()
    np.testing.assert_allclose(yd.cpu().numpy(), Y_ref, rtol=1e-12, atol=1e-12 * np.abs(Y_ref).max())
    x = rng.normal(size=N)
    np.testing.assert_allclose(csr.matvec(x), O.spmv(*ref, x), rtol=1e-12, atol=1e-12)
    csr.free()


@pytest.mark.parametrize("n,na,nb", [(9, 4, 4), (9, 4, 3)])
def test_fcix_solves_against_dense(ctx, monkeypatch, n, na, nb):
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    csr, ref, dets, ecore = build(ctx, n, na, nb, seed=1009)
    csr.prepare_mixed()
    assert csr.has_fcix()
    e_ref = O.lowest_eigenvalues(*ref, nroot=4)
    for mode, atol in ((capi.SOLVE_FP64, 1e-9), (capi.SOLVE_MIXED, 1e-6)):
        evals, _, _ = csr.solve(n=4, tol=1e-10 if mode == capi.SOLVE_FP64 else 1e-8, mode=mode)
        np.testing.assert_allclose(np.sort(evals), e_ref, atol=atol)
    csr.free()


def test_fcix_clone(ctx, monkeypatch):
    import torch
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    a, ref, dets, _ = build(ctx, 9, 4, 3, seed=1006)
    a.prepare_mixed(drop_fp64=True)
    out = ctypes.c_void_p()
    capi.check(capi.lib().pyci_gpu_csr_clone(a.handle, ctypes.byref(out)))
    b = capi.Csr.__new__(capi.Csr)
    b.handle = out
    N = dets.shape[0]
    X = np.random.default_rng(9).normal(size=(N, 4))
    xf = torch.tensor(X, dtype=torch.float32, device="cuda")
    xs = torch.tensor(split_rows(X), device="cuda")
    res = []
    for op in (a, b):
        yf = torch.empty((N, 4), dtype=torch.float32, device="cuda")
        yd = torch.empty((N, 4), dtype=torch.float64, device="cuda")
        op.spmm_device(capi.PREC_FP32, 4, xf.data_ptr(), yf.data_ptr(), None)
        op.spmm_device(capi.PREC_FP64_DF, 4, xs.data_ptr(), yd.data_ptr(), None)
        torch.cuda.synchronize()
        res.append((yf.cpu().numpy(), yd.cpu().numpy()))
        if op is a:
            a.free()
    assert b.has_fcix()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(4)], axis=1)
    np.testing.assert_allclose(res[1][1], Y_ref, rtol=1e-11, atol=1e-11 * np.abs(Y_ref).max())
    b.free()


def test_deferred_csr_written_on_first_use(ctx, monkeypatch):
    r"""An operator with the implicit-column form is built without its CSR
    entries: shape and size are known, solves run on the form and leave them
    unwritten, and the first export writes them, equal to the oracle's CSR
    and to an eagerly built operator's.  Both operators' implicit-column
    values are the exact split of the CSR values: products with unit vectors
    (one term per row) return the same columns from the form and from the
    CSR, in FP32 and in double-float arithmetic."""
    import torch
    n, na, nb = 9, 4, 3
    csr, ref, dets, ecore = build(ctx, n, na, nb, seed=1011)
    st = csr.storage()
    assert st & capi.STORE_IMPLICIT and st & capi.STORE_DEFERRED and not st & capi.STORE_FP64
    nrow, ncol, size, _ = csr.shape()
    assert (nrow, ncol, size) == (dets.shape[0], dets.shape[0], ref[0].size)
    e_ref = O.lowest_eigenvalues(*ref, nroot=2)
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    for mode, tol, atol in ((capi.SOLVE_MIXED, 1e-8, 1e-6), (capi.SOLVE_FP64, 1e-10, 1e-9)):
        evals, _, _ = csr.solve(n=2, tol=tol, mode=mode)
        np.testing.assert_allclose(np.sort(evals), e_ref, atol=atol)
    assert csr.storage() & capi.STORE_DEFERRED, "a solve on the implicit-column form wrote the CSR"
    data, indices, indptr = csr.export()
    st = csr.storage()
    assert st & capi.STORE_FP64 and not st & capi.STORE_DEFERRED
    assert np.array_equal(data, ref[0]) and np.array_equal(indices, ref[1]) and np.array_equal(indptr, ref[2])
    eager = capi.Csr(ctx, capi.WFN_FULLCI, n, na, nb, dets, *synthetic_integrals(n, 1011)[1:],
                     flags=capi.BUILD_FULL_COLEX | capi.BUILD_EAGER_CSR)
    st = eager.storage()
    assert st & capi.STORE_FP64 and st & capi.STORE_IMPLICIT and not st & capi.STORE_DEFERRED
    d2, i2, p2 = eager.export()
    assert np.array_equal(d2, ref[0]) and np.array_equal(i2, ref[1]) and np.array_equal(p2, ref[2])
    N = dets.shape[0]
    cols = [0, 1, N // 3, N // 2 + 7]
    X = np.zeros((N, 4))
    X[cols, np.arange(4)] = 1.0
    xf = torch.tensor(X, dtype=torch.float32, device="cuda")
    xs = torch.tensor(split_rows(X), device="cuda")
    out = []
    for op, pin in ((csr, "fcix"), (eager, "csr")):
        monkeypatch.setenv("PYCI_GPU_SPMM", pin)
        yf = torch.empty((N, 4), dtype=torch.float32, device="cuda")
        yd = torch.empty((N, 4), dtype=torch.float64, device="cuda")
        op.spmm_device(capi.PREC_FP32, 4, xf.data_ptr(), yf.data_ptr(), None)
        op.spmm_device(capi.PREC_FP64_DF, 4, xs.data_ptr(), yd.data_ptr(), None)
        torch.cuda.synchronize()
        out.append((yf.cpu().numpy(), yd.cpu().numpy()))
    assert csr.product_form(capi.PREC_FP32, 4) == capi.FORM_IMPLICIT
    assert eager.product_form(capi.PREC_FP32, 4) != capi.FORM_IMPLICIT
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    full = O.full_matrix(*ref).toarray()
    np.testing.assert_allclose(out[0][1], full[:, cols], rtol=2e-14, atol=0)
    csr.free()
    eager.free()
