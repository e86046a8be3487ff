r"""Python front end of the CPU oracle (test infrastructure only).

Loads ``oracle/build/liboracle.so`` (the C restatement in ``pyci_oracle.c``)
with ctypes and offers numpy-level helpers: determinant enumeration, the
reference-layout CSR build (lower triangle + diagonal when symmetric), SpMV,
and reference eigenvalues.  Only tests, the smoke check and the CPU-baseline
leg of the benchmark use this module; the product never imports it.
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "build", "liboracle.so")

DOCI, FULLCI, GENCI, GENCI_REF = 0, 1, 2, 3
_lib = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


def build():
    r"""Compile the C restatement (make -C oracle port)."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "port"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = ctypes.CDLL(_LIB)
        L.orc_binomial.restype = _i64
        L.orc_binomial.argtypes = [_i64, _i64]
        L.orc_rank_colex.restype = _i64
        L.orc_rank_colex.argtypes = [_i64, _i64, _p]
        L.orc_ndet_all.restype = _i64
        L.orc_ndet_all.argtypes = [ctypes.c_int, _i64, _i64, _i64]
        L.orc_add_all_dets.restype = ctypes.c_int
        L.orc_add_all_dets.argtypes = [ctypes.c_int, _i64, _i64, _i64, _p]
        L.orc_csr_count.restype = ctypes.c_int
        L.orc_csr_count.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _i64, _i64,
                                    ctypes.c_int, ctypes.c_int, _p]
        L.orc_csr_fill.restype = ctypes.c_int
        L.orc_csr_fill.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _i64, _i64,
                                   ctypes.c_int, _p, _p, _p, _p, _p, ctypes.c_int, _p, _p, _p]
        L.orc_csr_count_rows.restype = ctypes.c_int
        L.orc_csr_count_rows.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _i64, _i64, _i64,
                                         ctypes.c_int, ctypes.c_int, _p]
        L.orc_csr_fill_rows.restype = ctypes.c_int
        L.orc_csr_fill_rows.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _i64, _i64, _i64,
                                        ctypes.c_int, _p, _p, _p, _p, _p, ctypes.c_int, _p, _p, _p]
        for f in (L.orc_spmv_general, L.orc_spmv_sym_lower):
            f.restype = None
            f.argtypes = [_i64, _p, _p, _p, _p, _p, ctypes.c_int]
        L.orc_phase_single.restype = ctypes.c_int
        L.orc_phase_single.argtypes = [_p, _i64, _i64]
        L.orc_phase_double.restype = ctypes.c_int
        L.orc_phase_double.argtypes = [_p, _i64, _i64, _i64, _i64]
        L.orc_compute_transition_rdms.restype = ctypes.c_int
        L.orc_compute_transition_rdms.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _p, _i64, _p, _p, _p,
                                                  _p]
        L.orc_compute_rdms.restype = ctypes.c_int
        L.orc_compute_rdms.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _p, _p, _p]
        L.orc_compute_enpt2.restype = ctypes.c_int
        L.orc_compute_enpt2.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _p, _p, _p, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        L.orc_compute_rdms_genci.restype = ctypes.c_int
        L.orc_compute_rdms_genci.argtypes = [_i64, _i64, _p, _p, _i64, _p, _p, _p, _p]
        L.orc_add_hci.restype = ctypes.c_int
        L.orc_add_hci.argtypes = [ctypes.c_int, _i64, _i64, _i64, _i64, _p, _p, _p, _p, ctypes.c_double, _i64, _p,
                                  ctypes.POINTER(_i64)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def nword(nbasis):
    return (nbasis + 63) // 64


def all_dets(kind, nbasis, nocc_up, nocc_dn):
    r"""Every determinant in add_all_dets order: uint64[ndet, nwords]."""
    L = lib()
    nd = L.orc_ndet_all(kind, nbasis, nocc_up, nocc_dn)
    nw = nword(nbasis) * (2 if kind == FULLCI else 1)
    dets = np.zeros((nd, nw), dtype=np.uint64)
    if L.orc_add_all_dets(kind, nbasis, nocc_up, nocc_dn, _ptr(dets)):
        raise RuntimeError("orc_add_all_dets failed")
    return dets


def senzero(one_mo, two_mo):
    r"""h, v, w exactly as pyci/src/squantop.cpp:175-182 derives them."""
    n = one_mo.shape[0]
    h = np.ascontiguousarray(np.diagonal(one_mo).copy())
    idx = np.arange(n)
    v = np.ascontiguousarray(two_mo[idx[:, None], idx[:, None], idx[None, :], idx[None, :]])
    w = np.ascontiguousarray(two_mo[idx[:, None], idx[None, :], idx[:, None], idx[None, :]] * 2
                             - two_mo[idx[:, None], idx[None, :], idx[None, :], idx[:, None]])
    return h, v, w


def build_csr(kind, nbasis, nocc_up, nocc_dn, dets, one_mo, two_mo, nrow=-1, ncol=-1,
              symmetric=True, nthreads=None):
    r"""Reference-layout CSR (data f64, indices i64, indptr i64)."""
    L = lib()
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    ndet = dets.shape[0]
    nrow = ndet if nrow < 0 else nrow
    ncol = ndet if ncol < 0 else ncol
    nthreads = nthreads or os.cpu_count() or 1
    one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
    two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
    h, v, w = senzero(one_mo, two_mo)
    indptr = np.zeros(nrow + 1, dtype=np.int64)
    args = (kind, nbasis, nocc_up, nocc_dn, ndet, _ptr(dets), nrow, ncol, int(bool(symmetric)))
    if L.orc_csr_count(*args, nthreads, _ptr(indptr)):
        raise RuntimeError("orc_csr_count failed")
    nnz = int(indptr[-1])
    indices = np.empty(nnz, dtype=np.int64)
    data = np.empty(nnz, dtype=np.float64)
    if L.orc_csr_fill(*args, _ptr(one_mo), _ptr(two_mo), _ptr(h), _ptr(v), _ptr(w), nthreads,
                      _ptr(indptr), _ptr(indices), _ptr(data)):
        raise RuntimeError("orc_csr_fill failed")
    return data, indices, indptr


def build_csr_rows(kind, nbasis, nocc_up, nocc_dn, dets, one_mo, two_mo, row0, row1, ncol=-1,
                   symmetric=True, nthreads=None, h_v_w=None):
    r"""Rows [row0, row1) of build_csr's CSR (indptr local to the range)."""
    L = lib()
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    ndet = dets.shape[0]
    ncol = ndet if ncol < 0 else ncol
    nthreads = nthreads or os.cpu_count() or 1
    one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
    two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
    h, v, w = h_v_w if h_v_w is not None else senzero(one_mo, two_mo)
    indptr = np.zeros(row1 - row0 + 1, dtype=np.int64)
    args = (kind, nbasis, nocc_up, nocc_dn, ndet, _ptr(dets), row0, row1, ncol, int(bool(symmetric)))
    if L.orc_csr_count_rows(*args, nthreads, _ptr(indptr)):
        raise RuntimeError("orc_csr_count_rows failed")
    nnz = int(indptr[-1])
    indices = np.empty(nnz, dtype=np.int64)
    data = np.empty(nnz, dtype=np.float64)
    if L.orc_csr_fill_rows(*args, _ptr(one_mo), _ptr(two_mo), _ptr(h), _ptr(v), _ptr(w), nthreads,
                           _ptr(indptr), _ptr(indices), _ptr(data)):
        raise RuntimeError("orc_csr_fill_rows failed")
    return data, indices, indptr


def spmv(data, indices, indptr, x, symmetric=True, nthreads=None):
    L = lib()
    nrow = indptr.shape[0] - 1
    x = np.ascontiguousarray(x, dtype=np.float64)
    if symmetric and x.shape[0] < nrow:
        raise ValueError("self-adjoint product needs len(x) >= nrow")
    y = np.zeros(nrow, dtype=np.float64)
    f = L.orc_spmv_sym_lower if symmetric else L.orc_spmv_general
    f(nrow, _ptr(indptr), _ptr(indices), _ptr(data), _ptr(x), _ptr(y), nthreads or os.cpu_count())
    return y


def full_matrix(data, indices, indptr, ncol=None):
    r"""scipy CSR of the full symmetric matrix from its lower triangle."""
    import scipy.sparse as sp
    n = indptr.shape[0] - 1
    low = sp.csr_matrix((data, indices, indptr), shape=(n, ncol or n))
    return (low + low.T - sp.diags(low.diagonal())).tocsr()


def lowest_eigenvalues(data, indices, indptr, nroot=1, tol=1e-12):
    r"""Lowest eigenvalues (ascending) of the symmetric matrix given by its lower CSR.

    Dense eigh for small matrices; ARPACK's implicitly restarted Lanczos
    (scipy.sparse.linalg.eigsh) on the oracle's threaded symmetric SpMV
    otherwise, which never forms the full matrix.  The Lanczos start vector is
    seeded random, as the reference's Spectra solver starts from a random
    vector (SymEigsSolver::init() without coefficients,
    pyci/src/sparseop.cpp:131-132): a structured start such as the all-ones
    vector lies in one spin-flip symmetry sector of a FullCI Hamiltonian with
    nocc_up == nocc_dn, and the other sector's roots then appear only through
    rounding.
    """
    import scipy.sparse.linalg as spl
    n = indptr.shape[0] - 1
    if n <= 3000:
        return np.linalg.eigvalsh(full_matrix(data, indices, indptr).toarray())[:nroot]
    op = spl.LinearOperator((n, n), matvec=lambda x: spmv(data, indices, indptr, np.ravel(x)),
                            dtype=np.float64)
    vals = spl.eigsh(op, k=nroot, which="SA", tol=tol, return_eigenvectors=False,
                     v0=np.random.default_rng(7).standard_normal(n), ncv=max(2 * nroot + 1, 20))
    return np.sort(vals)


def add_hci(kind, nbasis, nocc_up, nocc_dn, dets, coeffs, one_mo, two_mo, eps):
    r"""Determinants heat-bath CI adds to `dets` (uint64[nnew, nwords]), each
    once, in first-occurrence order (pyci/src/hci.cpp:240-262)."""
    L = lib()
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
    two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
    n = _i64(0)
    args = (kind, nbasis, nocc_up, nocc_dn, dets.shape[0], _ptr(dets), _ptr(coeffs), _ptr(one_mo), _ptr(two_mo),
            float(eps))
    if L.orc_add_hci(*args, 0, None, ctypes.byref(n)):
        raise RuntimeError("orc_add_hci failed")
    out = np.zeros((n.value, dets.shape[1]), dtype=np.uint64)
    if n.value and L.orc_add_hci(*args, n.value, _ptr(out), ctypes.byref(n)):
        raise RuntimeError("orc_add_hci failed")
    return out


def compute_rdms(kind, nbasis, nocc_up, nocc_dn, dets, coeffs):
    r"""(rdm1, rdm2) as pyci.compute_rdms returns them (pyci/src/rdm.cpp): DOCI
    (d0, d2) [n, n] each; FullCI rdm1 [2, n, n], rdm2 [3, n, n, n, n]."""
    L = lib()
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    n = nbasis
    if kind == DOCI:
        r1, r2 = np.zeros((n, n)), np.zeros((n, n))
    else:
        r1, r2 = np.zeros((2, n, n)), np.zeros((3, n, n, n, n))
    if L.orc_compute_rdms(kind, n, nocc_up, nocc_dn, dets.shape[0], _ptr(dets), _ptr(coeffs), _ptr(r1), _ptr(r2)):
        raise RuntimeError("orc_compute_rdms failed")
    return r1, r2


def compute_enpt2(kind, nbasis, nocc_up, nocc_dn, dets, coeffs, one_mo, two_mo, energy, ecore, eps):
    r"""Epstein-Nesbet second-order energy of pyci.compute_enpt2 (pyci/src/enpt2.cpp)."""
    L = lib()
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
    two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
    out = ctypes.c_double(0.0)
    if L.orc_compute_enpt2(kind, nbasis, nocc_up, nocc_dn, dets.shape[0], _ptr(dets), _ptr(coeffs), _ptr(one_mo),
                           _ptr(two_mo), float(energy), float(ecore), float(eps), ctypes.byref(out)):
        raise RuntimeError("orc_compute_enpt2 failed")
    return out.value


def compute_rdms_genci(nbasis, dets1, coeffs1, dets2=None, coeffs2=None):
    r"""Spin-orbital (rdm1 [n][n], rdm2 [n][n][n][n]) of a GenCI wave function
    from their definition, <1| a+_p a_q |2> and <1| a+_p a+_q a_s a_r |2>
    (the wave function itself when the second is omitted)."""
    L = lib()
    dets1 = np.ascontiguousarray(dets1, dtype=np.uint64)
    coeffs1 = np.ascontiguousarray(coeffs1, dtype=np.float64)
    dets2 = dets1 if dets2 is None else np.ascontiguousarray(dets2, dtype=np.uint64)
    coeffs2 = coeffs1 if coeffs2 is None else np.ascontiguousarray(coeffs2, dtype=np.float64)
    n = nbasis
    r1, r2 = np.zeros((n, n)), np.zeros((n, n, n, n))
    if L.orc_compute_rdms_genci(n, dets1.shape[0], _ptr(dets1), _ptr(coeffs1), dets2.shape[0], _ptr(dets2),
                                _ptr(coeffs2), _ptr(r1), _ptr(r2)):
        raise RuntimeError("orc_compute_rdms_genci failed")
    return r1, r2


def compute_transition_rdms(kind, nbasis, nocc_up, nocc_dn, dets1, coeffs1, dets2, coeffs2):
    r"""(rdm1, rdm2) as pyci.compute_transition_rdms returns them (pyci/src/rdm.cpp:634-902)."""
    L = lib()
    dets1 = np.ascontiguousarray(dets1, dtype=np.uint64)
    dets2 = np.ascontiguousarray(dets2, dtype=np.uint64)
    coeffs1 = np.ascontiguousarray(coeffs1, dtype=np.float64)
    coeffs2 = np.ascontiguousarray(coeffs2, dtype=np.float64)
    n = nbasis
    if kind == DOCI:
        r1, r2 = np.zeros((n, n)), np.zeros((n, n))
    else:
        r1, r2 = np.zeros((2, n, n)), np.zeros((3, n, n, n, n))
    if L.orc_compute_transition_rdms(kind, n, nocc_up, nocc_dn, dets1.shape[0], _ptr(dets1), _ptr(coeffs1),
                                     dets2.shape[0], _ptr(dets2), _ptr(coeffs2), _ptr(r1), _ptr(r2)):
        raise RuntimeError("orc_compute_transition_rdms failed")
    return r1, r2
