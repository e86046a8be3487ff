r"""GPU parity through the C ABI: CSR pattern bit-exact and FP64 values equal to
the reference's (golden arrays from the reference's own sparse_op, digests of
its full-size CSR), SpMV/SpMM against the oracle, eigenvalues against the
reference tests' known answers and the oracle."""

import numpy as np
import pytest

import oracle as O
from conftest import load_csr_case, load_kat
from pyci_gb300 import capi
from pyci_gb300.synth import synthetic_integrals

pytestmark = pytest.mark.gpu

WFN = {"doci": capi.WFN_DOCI, "fullci": capi.WFN_FULLCI, "genci": capi.WFN_GENCI}
OKIND = {"doci": O.DOCI, "fullci": O.FULLCI}
CASES = ["fci_6_3_2", "fci_7_3_3_cisd", "fci_7_3_2_rect", "fci_5_2_2_sym_nrow", "doci_10_4",
         "doci_12_5_cisd_rect", "doci_9_3_ncol", "genci_10_4", "genci_12_3_cisd_rect"]


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def build_case(ctx, meta, ref, flags=0):
    return capi.Csr(ctx, WFN[meta["wfn"]], meta["nbasis"], meta["nocc_up"], meta["nocc_dn"], ref["dets"],
                    ref["one_mo"], ref["two_mo"], meta["nrow"], meta["ncol"], meta["symmetric"], flags)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", ["colex", "hash"])
def test_csr_matches_reference(ctx, golden, case, mode):
    meta = {m["name"]: m for m in golden["csr_cases"]}[case]
    ref = load_csr_case(case)
    full_space = meta["excitations"] is None
    if mode == "colex" and not full_space:
        pytest.skip("colex ranking applies to full spaces only")
    flags = capi.BUILD_FULL_COLEX if mode == "colex" else capi.BUILD_FORCE_HASH
    csr = build_case(ctx, meta, ref, flags)
    nrow, ncol, size, stored = csr.shape()
    assert (nrow, ncol) == tuple(meta["shape"]) and size == meta["size"]
    data, indices, indptr = csr.export()
    assert np.array_equal(indptr, ref["indptr"])
    assert np.array_equal(indices, ref["indices"])
    if meta["wfn"] == "genci":
        for r in range(nrow):
            s, e = indptr[r], indptr[r + 1]
            assert sorted(zip(indices[s:e], data[s:e])) == sorted(zip(ref["indices"][s:e], ref["data"][s:e]))
    else:
        assert np.array_equal(data, ref["data"])  # bit-exact FP64 matrix elements
    if not (meta["symmetric"] and ncol < nrow):
        y = csr.matvec(ref["x"])
        np.testing.assert_allclose(y, ref["y"], rtol=1e-12, atol=1e-11)
    # get_element returns a stored value of (r, j) (the first of repeated
    # columns, as the reference's lower_bound lookup does) and 0 when absent.
    for r in range(0, nrow, max(1, nrow // 7)):
        s, e = indptr[r], indptr[r + 1]
        for t in range(s, e, max(1, (e - s) // 3)):
            assert csr.get_element(r, int(indices[t])) in set(data[s:e][indices[s:e] == indices[t]])
        absent = int(max(indices[s:e], default=-1)) + 1
        if absent < ncol and absent not in indices[s:e]:
            assert csr.get_element(r, absent) == 0.0
    csr.free()


def test_genci_exact_mode_reproduces_fullci_energy(ctx):
    # Slater-Condon rules over the true virtuals: a spin-orbital GenCI space of
    # 2 alpha + 2 beta electrons in 5 spatial orbitals has the FCI ground state.
    n = 5
    ecore, one, two = synthetic_integrals(n, 3)
    N = 2 * n
    one_g = np.zeros((N, N))
    one_g[:n, :n] = one
    one_g[n:, n:] = one
    two_g = np.zeros((N, N, N, N))
    for s1 in (0, 1):
        for s2 in (0, 1):
            two_g[s1 * n:(s1 + 1) * n, s2 * n:(s2 + 1) * n, s1 * n:(s1 + 1) * n, s2 * n:(s2 + 1) * n] = two
    gdets = O.all_dets(O.GENCI, N, 4, 0)
    g = capi.Csr(ctx, capi.WFN_GENCI, N, 4, 0, gdets, one_g, two_g, flags=capi.BUILD_GENCI_EXACT)
    d, i, p = g.export()
    og = O.build_csr(O.GENCI, N, 4, 0, gdets, one_g, two_g)
    assert np.array_equal(i, og[1]) and np.array_equal(p, og[2]) and np.array_equal(d, og[0])
    fdets = O.all_dets(O.FULLCI, n, 2, 2)
    f = capi.Csr(ctx, capi.WFN_FULLCI, n, 2, 2, fdets, one, two, flags=capi.BUILD_FULL_COLEX)
    eg = g.solve(n=1, tol=1e-10)[0][0]
    ef = f.solve(n=1, tol=1e-10)[0][0]
    assert eg == pytest.approx(ef, abs=1e-9)


@pytest.mark.parametrize("name", ["fci_8_4_4", "doci_24_6", "fci_12_5_5", "doci_32_8"])
def test_workload_digest_and_eigenvalues(ctx, golden, name):
    # The 12-orbital FCI (1.08e9 stored nonzeros) and 32-orbital DOCI (2.03e9)
    # workloads are built at full size: pattern digest exact, value digest to
    # 1e-12 relative, lowest roots within 1 microhartree of the FP64 oracle.
    w = golden["workloads"][name]
    ecore, one, two = synthetic_integrals(w["nbasis"], w["seed"])
    csr = capi.Csr(ctx, WFN[w["wfn"]], w["nbasis"], w["occs"][0], w["occs"][1], None, one, two,
                   flags=capi.BUILD_FULL_COLEX, ndet=w["nrow"])
    nrow, ncol, size, stored = csr.shape()
    assert size == w["nnz"]
    d = csr.digest()
    assert d["pattern_sum"] == w["pattern_sum"] and d["pattern_xor"] == w["pattern_xor"]
    assert d["value_sum"] == pytest.approx(w["value_sum"], rel=1e-12, abs=1e-9)
    assert d["value_abs_sum"] == pytest.approx(w["value_abs_sum"], rel=1e-12)
    assert d["value_wsum"] == pytest.approx(w["value_wsum"], rel=1e-12, abs=1e-9)
    nroot = len(w["eigenvalues"])
    if nrow > 5_000_000:
        csr.prepare_mixed(drop_fp64=True)  # FP32 high/low split only: 12 bytes per entry
    modes = (capi.SOLVE_MIXED,) if nrow > 5_000_000 else (capi.SOLVE_FP64, capi.SOLVE_MIXED)
    for mode in modes:
        evals, evecs, st = csr.solve(n=nroot, tol=1e-8 if mode == capi.SOLVE_FP64 else 1e-6, mode=mode)
        assert np.all(np.diff(evals) <= 0)  # decreasing, the reference's order
        err = np.abs(np.sort(evals) - np.array(w["eigenvalues"]))
        assert err.max() < 1e-6, (mode, err)  # within 1 microhartree
        # eigenvectors: unit norm, H x = e x to the solver's residual
        for k in range(nroot):
            assert np.linalg.norm(evecs[k]) == pytest.approx(1.0, abs=1e-6)
    csr.free()


@pytest.mark.parametrize("nroot", [9, 12])
def test_many_roots_against_dense_eigenvalues(ctx, nroot):
    r"""More wanted roots than one launch's column limit (8): residuals,
    preconditioned corrections and products run in several launches per
    block.  FullCI 7o 3a3b (1,225 determinants) against numpy's dense
    eigenvalues, both precision modes."""
    ecore, one, two = synthetic_integrals(7, 1005)
    dets = O.all_dets(O.FULLCI, 7, 3, 3)
    ref = O.build_csr(O.FULLCI, 7, 3, 3, dets, one, two)
    N = dets.shape[0]
    H = np.stack([O.spmv(*ref, e) for e in np.eye(N)], axis=1)
    exact = np.linalg.eigvalsh(0.5 * (H + H.T))[:nroot]
    csr = capi.Csr(ctx, capi.WFN_FULLCI, 7, 3, 3, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    for mode in (capi.SOLVE_FP64, capi.SOLVE_MIXED):
        evals, evecs, st = csr.solve(n=nroot, tol=1e-8 if mode == capi.SOLVE_FP64 else 1e-6, mode=mode)
        err = np.abs(np.sort(evals) - exact)
        assert err.max() < 1e-6, (mode, err)
        for k in range(nroot):
            assert np.linalg.norm(evecs[k]) == pytest.approx(1.0, abs=1e-6)
    csr.free()


@pytest.mark.parametrize("kat", [0, 1, 2, 3])
def test_known_answer_energies(ctx, golden, kat):
    # pyci/test/test_routines.py:37-54 with the reference's solve(n=1, ncv=30, tol=1e-6).
    k = golden["kats"][kat]
    ecore, one, two = load_kat(k["system"])
    n = one.shape[0]
    dets = O.all_dets(OKIND[k["wfn"]], n, *k["occs"])
    csr = capi.Csr(ctx, WFN[k["wfn"]], n, k["occs"][0], k["occs"][1], dets, one, two, flags=capi.BUILD_FULL_COLEX)
    evals, _, _ = csr.solve(n=1, ncv=30, tol=1e-6, ecore=ecore)
    assert abs(evals[0] - k["energy"]) < 1e-9
    csr.free()


def test_spmm_precisions_against_oracle(ctx):
    import torch
    ecore, one, two = synthetic_integrals(8, 1001)
    dets = O.all_dets(O.FULLCI, 8, 4, 4)
    ref = O.build_csr(O.FULLCI, 8, 4, 4, dets, one, two)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, 8, 4, 4, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    csr.prepare_mixed()
    N = dets.shape[0]
    rng = np.random.default_rng(5)
    for k in (1, 3, 4, 8, 11):
        X = rng.normal(size=(N, k))
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xd = torch.tensor(X, dtype=torch.float64, device="cuda")
        yd = torch.empty((N, k), dtype=torch.float64, device="cuda")
        for prec in (capi.PREC_FP64, capi.PREC_FP64_SPLIT):
            csr.spmm_device(prec, k, xd.data_ptr(), yd.data_ptr(), None)
            torch.cuda.synchronize()
            np.testing.assert_allclose(yd.cpu().numpy(), Y_ref, rtol=1e-12, atol=1e-11)
        xf = xd.float()
        yf = torch.empty((N, k), dtype=torch.float32, device="cuda")
        csr.spmm_device(capi.PREC_FP32, k, xf.data_ptr(), yf.data_ptr(), None)
        torch.cuda.synchronize()
        # FP32 values and accumulation: relative error ~ sqrt(row length) * 2^-24
        err = np.abs(yf.cpu().numpy() - Y_ref).max() / np.abs(Y_ref).max()
        assert err < 1e-5
    csr.free()


@pytest.mark.parametrize("kind,n,nu,nd", [("fullci", 8, 4, 4), ("doci", 16, 6, 6), ("fullci", 9, 4, 2)])
def test_spmm_sell_against_oracle(ctx, monkeypatch, kind, n, nu, nd):
    r"""The FP32 and double-float products on the SELL-32 copy (pinned with
    PYCI_GPU_SPMM=sell or =sell1) and on the CSR kernels (=csr) against the
    oracle's FP64 product; row counts that leave a partial last slice of 32
    rows."""
    import torch
    ecore, one, two = synthetic_integrals(n, 1003)
    dets = O.all_dets(OKIND[kind], n, nu, nd)
    ref = O.build_csr(OKIND[kind], n, nu, nd, dets, one, two)
    N = dets.shape[0]
    rng = np.random.default_rng(8)
    out = {}
    for mode in ("sell", "sell1", "csr"):
        monkeypatch.setenv("PYCI_GPU_SPMM", mode)
        csr = capi.Csr(ctx, WFN[kind], n, nu, nd, dets, one, two, flags=capi.BUILD_FULL_COLEX)
        csr.prepare_mixed(drop_fp64=True)
        for k in (1, 2, 3, 4, 8, 11):
            X = rng.normal(size=(N, k)) if mode == "sell" else out[("x", k)]
            xf = torch.tensor(X, dtype=torch.float32, device="cuda")
            yf = torch.empty((N, k), dtype=torch.float32, device="cuda")
            csr.spmm_device(capi.PREC_FP32, k, xf.data_ptr(), yf.data_ptr(), None)
            torch.cuda.synchronize()
            out[("x", k)] = X
            out[(mode, k)] = yf.cpu().numpy().astype(np.float64)
        for k in (1, 2, 4):
            X = out[("x", k)]
            xs = torch.tensor(split_rows(X), device="cuda")
            yd = torch.empty((N, k), dtype=torch.float64, device="cuda")
            csr.spmm_device(capi.PREC_FP64_DF, k, xs.data_ptr(), yd.data_ptr(), None)
            torch.cuda.synchronize()
            out[(mode, "df", k)] = yd.cpu().numpy()
        csr.free()
    for k in (1, 2, 3, 4, 8, 11):
        X = out[("x", k)].astype(np.float32).astype(np.float64)
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        scale = np.abs(Y_ref).max()
        for mode in ("sell", "sell1", "csr"):
            # FP32 values and accumulation: relative error ~ sqrt(row length) * 2^-24
            assert np.abs(out[(mode, k)] - Y_ref).max() / scale < 1e-5, (mode, k)
    for k in (1, 2, 4):
        X = out[("x", k)]
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        for mode in ("sell", "sell1", "csr"):
            # double-float sums: ~2^-44 relative
            np.testing.assert_allclose(out[(mode, "df", k)], Y_ref, rtol=1e-11, atol=1e-11 * np.abs(Y_ref).max())


def split_rows(X):
    r"""[N][k] FP64 -> [N][2k] FP32: each row's high parts, then its low parts."""
    hi = X.astype(np.float32)
    lo = (X - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([hi, lo], axis=1))


@pytest.mark.parametrize("nb, na", [(8, 4), (10, 4)])  # 10, 4: 26M entries, past the autotuning threshold
def test_spmm_double_float_against_oracle(ctx, nb, na):
    r"""PYCI_PREC_FP64_DF: FP32 arithmetic with double-float sums reproduces the
    FP64 product to ~2^-44 relative."""
    import torch
    ecore, one, two = synthetic_integrals(nb, 1002)
    dets = O.all_dets(O.FULLCI, nb, na, na)
    ref = O.build_csr(O.FULLCI, nb, na, na, dets, one, two)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, nb, na, na, dets, one, two, flags=capi.BUILD_FULL_COLEX)
    csr.prepare_mixed(drop_fp64=True)
    N = dets.shape[0]
    rng = np.random.default_rng(6)
    for k in (1, 2, 4):
        X = rng.normal(size=(N, k))
        Y_ref = np.stack([O.spmv(*ref, X[:, j]) for j in range(k)], axis=1)
        xs = torch.tensor(split_rows(X), device="cuda")
        yd = torch.empty((N, k), dtype=torch.float64, device="cuda")
        for _ in range(2):  # the first call may tune, the second uses the chosen variant
            csr.spmm_device(capi.PREC_FP64_DF, k, xs.data_ptr(), yd.data_ptr(), None)
            torch.cuda.synchronize()
            np.testing.assert_allclose(yd.cpu().numpy(), Y_ref, rtol=1e-11, atol=1e-11 * np.abs(Y_ref).max())
    with pytest.raises(capi.GpuError):
        csr.spmm_device(capi.PREC_FP64_DF, 3, xs.data_ptr(), yd.data_ptr(), None)
    csr.free()


def test_add_all_dets_on_device(ctx):
    for kind, ok, n, nu, nd in [(capi.WFN_FULLCI, O.FULLCI, 8, 3, 2), (capi.WFN_DOCI, O.DOCI, 70, 2, 2),
                                (capi.WFN_GENCI, O.GENCI, 12, 4, 0), (capi.WFN_FULLCI, O.FULLCI, 65, 2, 1)]:
        d = ctx.add_all_dets(kind, n, nu, nd)
        assert np.array_equal(d, O.all_dets(ok, n, nu, nd))


def test_errors_map_to_reference_exceptions(ctx):
    ecore, one, two = synthetic_integrals(6, 9)
    dets = O.all_dets(O.FULLCI, 6, 2, 2)
    sym = capi.Csr(ctx, capi.WFN_FULLCI, 6, 2, 2, dets, one, two)
    with pytest.raises(ValueError):
        sym.solve(n=dets.shape[0])  # n >= nrow
    rect = capi.Csr(ctx, capi.WFN_FULLCI, 6, 2, 2, dets, one, two, nrow=50, symmetric=False)
    with pytest.raises(TypeError):
        rect.solve(n=1)  # nrow != ncol
    with pytest.raises(ValueError):
        capi.Csr(ctx, capi.WFN_DOCI, 6, 3, 2, None, one, two, ndet=10)  # nocc_up != nocc_dn
    with pytest.raises(capi.GpuError):
        sym.solve(n=2, maxiter=1, tol=1e-14)  # did not converge -> RuntimeError
    sym.free()
    rect.free()


def test_update_appends_rows_like_reference(ctx):
    # op.update(ham, wfn) after growing the wave function (pyci/src/sparseop.cpp:175-201):
    # rows built before keep their columns; new rows are appended.
    ecore, one, two = synthetic_integrals(7, 21)
    full = O.all_dets(O.FULLCI, 7, 3, 2)
    small = full[:300]
    csr = capi.Csr(ctx, capi.WFN_FULLCI, 7, 3, 2, small, one, two)
    csr.update(full, one, two)
    d, i, p = csr.export()
    ref = O.build_csr(O.FULLCI, 7, 3, 2, full, one, two)  # symmetric: identical to a fresh build
    assert np.array_equal(p, ref[2]) and np.array_equal(i, ref[1]) and np.array_equal(d, ref[0])
    csr.free()


def test_clone_is_deep(ctx):
    ecore, one, two = synthetic_integrals(6, 4)
    dets = O.all_dets(O.DOCI, 6, 3, 3)
    a = capi.Csr(ctx, capi.WFN_DOCI, 6, 3, 3, dets, one, two)
    h = capi.lib()
    import ctypes
    out = ctypes.c_void_p()
    capi.check(h.pyci_gpu_csr_clone(a.handle, ctypes.byref(out)))
    da = a.export()
    a.free()
    b = capi.Csr.__new__(capi.Csr)
    b.handle = out
    db = b.export()
    for x, y in zip(da, db):
        assert np.array_equal(x, y)
    b.free()


def test_clone_keeps_the_sell_copy(ctx, monkeypatch):
    r"""A clone of a prepared operator carries its SELL-32 copy: the clone's
    FP32 and double-float products (pinned to the SELL kernels) equal the
    original's, after the original is freed."""
    import ctypes

    import torch
    ecore, one, two = synthetic_integrals(8, 1006)
    dets = O.all_dets(O.FULLCI, 8, 4, 3)
    monkeypatch.setenv("PYCI_GPU_SPMM", "sell")
    a = capi.Csr(ctx, capi.WFN_FULLCI, 8, 4, 3, dets, one, two, flags=capi.BUILD_FULL_COLEX)
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
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    b.free()
