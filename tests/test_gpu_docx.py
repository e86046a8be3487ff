r"""The implicit form of full DOCI operators (columns from each row's
occupation, values from the pair-integral table, nothing stored per entry)
against the oracle's FP64 product: FP32 and double-float products (FP64
arithmetic stays on the CSR), spaces whose row count is not a multiple of
32, one pair and many pairs, the eigensolver on the form, and clones."""

import ctypes

import numpy as np
import pytest

import oracle as O
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

# (nbasis, pairs): 70, 252, 220 and 1820 rows; 7 rows; 1 pair; more than 32
# orbitals (64-bit occupation masks): 7140 and 528 rows.
CASES = [(8, 4), (10, 5), (12, 3), (16, 4), (7, 6), (9, 1), (36, 3), (33, 2)]


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def split_rows(X):
    hi = X.astype(np.float32)
    lo = (X - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([hi, lo], axis=1))


def build(ctx, n, m, seed=1013):
    ecore, one, two = synthetic_integrals(n, seed)
    dets = O.all_dets(O.DOCI, n, m, m)
    ref = O.build_csr(O.DOCI, n, m, m, dets, one, two)
    csr = capi.Csr(ctx, capi.WFN_DOCI, n, m, m, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    return csr, ref, dets, ecore


@pytest.mark.parametrize("n,m", CASES)
def test_docx_products_against_oracle(ctx, monkeypatch, n, m):
    import torch
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    csr, ref, dets, _ = build(ctx, n, m)
    csr.prepare_mixed()
    assert csr.storage() & capi.STORE_IMPLICIT, "operator did not get the implicit DOCI form"
    N = dets.shape[0]
    rng = np.random.default_rng(23)
    scale = float(abs(O.full_matrix(*ref)).sum(axis=1).max())
    for k in (1, 2, 3, 4, 5, 8):
        X = rng.normal(size=(N, k)).astype(np.float32).astype(np.float64)
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xf = torch.tensor(X, dtype=torch.float32, device="cuda")
        yf = torch.full((N, k), np.nan, dtype=torch.float32, device="cuda")
        csr.spmm_device(capi.PREC_FP32, k, xf.data_ptr(), yf.data_ptr(), None)
        torch.cuda.synchronize()
        assert csr.product_form(capi.PREC_FP32, k) == capi.FORM_IMPLICIT
        # FP32 values and accumulation: error ~ row length * 2^-24 of the row's absolute sum
        assert np.abs(yf.cpu().numpy() - Y_ref).max() < 1e-5 * scale * np.abs(X).max(), k
    for k in (1, 2, 4):
        X = rng.normal(size=(N, k))
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xs = torch.tensor(split_rows(X), device="cuda")
        yd = torch.full((N, k), np.nan, dtype=torch.float64, device="cuda")
        csr.spmm_device(capi.PREC_FP64_DF, k, xs.data_ptr(), yd.data_ptr(), None)
        torch.cuda.synchronize()
        assert csr.product_form(capi.PREC_FP64_DF, k) == capi.FORM_IMPLICIT
        np.testing.assert_allclose(yd.cpu().numpy(), Y_ref, rtol=1e-11, atol=1e-11 * scale * np.abs(X).max())
    # FP64 arithmetic (CSR) and op(x) with host buffers on the same operator
    x = rng.normal(size=N)
    np.testing.assert_allclose(csr.matvec(x), O.spmv(*ref, x), rtol=1e-12, atol=1e-12 * scale)
    csr.free()


@pytest.mark.parametrize("n,m", [(10, 5), (12, 3)])
def test_docx_solves_against_dense(ctx, monkeypatch, n, m):
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    csr, ref, dets, ecore = build(ctx, n, m, seed=1017)
    csr.prepare_mixed()
    e_ref = O.lowest_eigenvalues(*ref, nroot=4)
    for mode, atol in ((capi.SOLVE_FP64, 1e-9), (capi.SOLVE_MIXED, 1e-6)):
        evals, _, _ = csr.solve(n=4, tol=1e-10 if mode == capi.SOLVE_FP64 else 1e-8, mode=mode)
        np.testing.assert_allclose(np.sort(evals), e_ref, atol=atol)
    csr.free()


def test_docx_clone(ctx, monkeypatch):
    import torch
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    a, ref, dets, _ = build(ctx, 10, 4, seed=1019)
    out = ctypes.c_void_p()
    capi.check(capi.lib().pyci_gpu_csr_clone(a.handle, ctypes.byref(out)))
    b = capi.Csr.__new__(capi.Csr)
    b.handle = out
    N = dets.shape[0]
    X = np.random.default_rng(9).normal(size=(N, 4))
    xs = torch.tensor(split_rows(X), device="cuda")
    res = []
    for op in (a, b):
        yd = torch.empty((N, 4), dtype=torch.float64, device="cuda")
        op.spmm_device(capi.PREC_FP64_DF, 4, xs.data_ptr(), yd.data_ptr(), None)
        torch.cuda.synchronize()
        res.append(yd.cpu().numpy())
        if op is a:
            a.free()
    assert b.storage() & capi.STORE_IMPLICIT
    assert np.array_equal(res[0], res[1])
    Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(4)], axis=1)
    np.testing.assert_allclose(res[1], Y_ref, rtol=1e-11, atol=1e-11 * np.abs(Y_ref).max())
    b.free()


def test_docx_deferred_csr(ctx, monkeypatch):
    r"""A full DOCI operator is built without its CSR entries and without its
    reference-layout row pointers: size is known from the symmetric pattern,
    solves run on the implicit form, and the first export (or element read)
    writes the entries, equal to the oracle's and to an eager build's."""
    n, m = 12, 4
    csr, ref, dets, ecore = build(ctx, n, m, seed=1021)
    st = csr.storage()
    assert st & capi.STORE_IMPLICIT and st & capi.STORE_DEFERRED and not st & capi.STORE_FP64
    nrow, ncol, size, _ = csr.shape()
    assert (nrow, ncol, size) == (dets.shape[0], dets.shape[0], ref[0].size)
    monkeypatch.setenv("PYCI_GPU_SPMM", "fcix")
    e_ref = O.lowest_eigenvalues(*ref, nroot=2)
    for mode, tol, atol in ((capi.SOLVE_MIXED, 1e-8, 1e-6), (capi.SOLVE_FP64, 1e-10, 1e-9)):
        evals, _, _ = csr.solve(n=2, tol=tol, mode=mode)
        np.testing.assert_allclose(np.sort(evals), e_ref, atol=atol)
    assert csr.storage() & capi.STORE_DEFERRED, "a solve on the implicit DOCI form wrote the CSR"
    data, indices, indptr = csr.export()
    assert not csr.storage() & capi.STORE_DEFERRED
    assert np.array_equal(data, ref[0]) and np.array_equal(indices, ref[1]) and np.array_equal(indptr, ref[2])
    eager = capi.Csr(ctx, capi.WFN_DOCI, n, m, m, dets, *synthetic_integrals(n, 1021)[1:],
                     flags=capi.BUILD_FULL_COLEX | capi.BUILD_EAGER_CSR)
    assert not eager.storage() & capi.STORE_DEFERRED
    d2, i2, p2 = eager.export()
    assert np.array_equal(d2, ref[0]) and np.array_equal(i2, ref[1]) and np.array_equal(p2, ref[2])
    # A fresh deferred operator: an element read writes the entries too.
    third, _, _, _ = build(ctx, n, m, seed=1021)
    full = O.full_matrix(*ref).toarray()
    i, j = nrow - 1, int(ref[1][ref[2][nrow - 1]])
    assert third.get_element(i, j) == full[i, j]
    assert not third.storage() & capi.STORE_DEFERRED
    for c in (csr, eager, third):
        c.free()
