r"""ctypes binding of the C ABI in include/pyci_gb300.h.

The same calls a host written in another language would bind (cgo, JNI,
N-API): plain pointers and sizes, integer status codes, and
``pyci_gpu_last_error`` for the message.  Status codes map to the exceptions
the reference raises (ValueError, TypeError, RuntimeError).
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY = os.path.join(_HERE, "lib", "libpyci_gb300.so")

OK, EINVAL, ETYPE, ENOCONV, ECUDA, ENOMEM, EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6
WFN_DOCI, WFN_FULLCI, WFN_GENCI = 0, 1, 2
BUILD_FULL_COLEX, BUILD_GENCI_EXACT, BUILD_FORCE_HASH, BUILD_EAGER_CSR = 0x1, 0x2, 0x4, 0x8
SOLVE_FP64, SOLVE_MIXED = 0, 1
GRAM_CUDA_CORES, GRAM_TENSOR_CORES = 0, 1
PREC_FP64, PREC_FP32, PREC_FP64_SPLIT, PREC_FP64_DF = 0, 1, 2, 3
STORE_FP64, STORE_SPLIT, STORE_SELL, STORE_IMPLICIT, STORE_DEFERRED = 0x1, 0x2, 0x4, 0x8, 0x10
FORM_UNTUNED, FORM_CSR, FORM_SELL, FORM_IMPLICIT = -1, 0, 1, 2

# Every symbol the header declares.
SYMBOLS = [
    "pyci_gpu_last_error", "pyci_gpu_version", "pyci_gpu_kernel_launches", "pyci_gpu_ctx_create", "pyci_gpu_ctx_destroy",
    "pyci_gpu_ctx_stream", "pyci_gpu_csr_build", "pyci_gpu_csr_update", "pyci_gpu_csr_free",
    "pyci_gpu_csr_clone", "pyci_gpu_csr_shape", "pyci_gpu_csr_export", "pyci_gpu_csr_get_element",
    "pyci_gpu_csr_matvec", "pyci_gpu_csr_matvec_noalloc", "pyci_gpu_csr_spmm_device", "pyci_gpu_csr_prepare_mixed",
    "pyci_gpu_csr_solve", "pyci_gpu_batch_solve", "pyci_gpu_csr_digest", "pyci_gpu_add_all_dets",
    "pyci_gpu_gram_device", "pyci_gpu_add_hci", "pyci_gpu_compute_rdms", "pyci_gpu_compute_enpt2",
    "pyci_gpu_compute_transition_rdms", "pyci_gpu_csr_storage", "pyci_gpu_csr_product_form",
]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("matvecs", ctypes.c_int64),
                ("matvecs_fp64", ctypes.c_int64), ("restarts", ctypes.c_int64),
                ("refinements", ctypes.c_int64), ("seconds", ctypes.c_double),
                ("seconds_spmm", ctypes.c_double), ("max_residual", ctypes.c_double),
                ("host_syncs", ctypes.c_int64), ("seconds_wait", ctypes.c_double)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


_lib = None
_p = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int


def lib():
    r"""Load libpyci_gb300.so (fails loudly if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBRARY):
            raise OSError("libpyci_gb300.so is not built; run `python pyci_gb300/build.py`")
        L = ctypes.CDLL(LIBRARY)
        sig = {
            "pyci_gpu_last_error": (ctypes.c_char_p, []),
            "pyci_gpu_version": (ctypes.c_char_p, []),
            "pyci_gpu_kernel_launches": (_i64, []),
            "pyci_gpu_ctx_create": (_int, [_int, ctypes.POINTER(_p)]),
            "pyci_gpu_ctx_destroy": (_int, [_p]),
            "pyci_gpu_ctx_stream": (_p, [_p]),
            "pyci_gpu_csr_build": (_int, [_p, _int, _i64, _i64, _i64, _i64, _p, _i64, _i64, _int, _p, _p,
                                          _int, ctypes.POINTER(_p)]),
            "pyci_gpu_csr_update": (_int, [_p, _i64, _p, _p, _p, _int]),
            "pyci_gpu_csr_free": (_int, [_p]),
            "pyci_gpu_csr_clone": (_int, [_p, ctypes.POINTER(_p)]),
            "pyci_gpu_csr_shape": (_int, [_p, _p, _p, _p, _p]),
            "pyci_gpu_csr_storage": (_int, [_p, ctypes.POINTER(_int)]),
            "pyci_gpu_csr_product_form": (_int, [_p, _int, _i64, ctypes.POINTER(_int)]),
            "pyci_gpu_csr_export": (_int, [_p, _p, _p, _p]),
            "pyci_gpu_csr_get_element": (_int, [_p, _i64, _i64, _p]),
            "pyci_gpu_csr_matvec": (_int, [_p, _p, _p]),
            "pyci_gpu_csr_matvec_noalloc": (_int, [_p, _p, _p]),
            "pyci_gpu_csr_spmm_device": (_int, [_p, _int, _i64, _p, _p, _p]),
            "pyci_gpu_csr_prepare_mixed": (_int, [_p, _int]),
            "pyci_gpu_csr_solve": (_int, [_p, _i64, _p, _i64, _i64, ctypes.c_double, ctypes.c_double, _int,
                                          _p, _p, ctypes.POINTER(SolveStats)]),
            "pyci_gpu_batch_solve": (_int, [_p, _i64, _p, _i64, _i64, ctypes.c_double, _p, _int, _p, _p, _p,
                                            ctypes.POINTER(SolveStats)]),
            "pyci_gpu_csr_digest": (_int, [_p, _p, _p, _p, _p, _p]),
            "pyci_gpu_add_all_dets": (_int, [_p, _int, _i64, _i64, _i64, _p]),
            "pyci_gpu_gram_device": (_int, [_p, _int, _p, _i64, _p, _i64, _i64, _p]),
            "pyci_gpu_add_hci": (_int, [_p, _int, _i64, _i64, _i64, _i64, _p, _p, _p, _p, ctypes.c_double, _int,
                                        _i64, _p, ctypes.POINTER(_i64)]),
            "pyci_gpu_compute_rdms": (_int, [_p, _int, _i64, _i64, _i64, _i64, _p, _p, _p, _p]),
            "pyci_gpu_compute_transition_rdms": (_int, [_p, _int, _i64, _i64, _i64, _i64, _p, _p, _i64, _p, _p, _p,
                                                        _p]),
            "pyci_gpu_compute_enpt2": (_int, [_p, _int, _i64, _i64, _i64, _i64, _p, _p, _p, _p, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class GpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def check(rc):
    if rc == OK:
        return
    msg = lib().pyci_gpu_last_error().decode()
    if rc == EINVAL:
        raise ValueError(msg)
    if rc == ETYPE:
        raise TypeError(msg)
    raise GpuError(rc, msg)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    r"""A device context (one CUDA device, one stream)."""

    def __init__(self, device=0):
        h = _p()
        check(lib().pyci_gpu_ctx_create(device, ctypes.byref(h)))
        self.handle = h

    @property
    def stream(self):
        return lib().pyci_gpu_ctx_stream(self.handle)

    def close(self):
        if self.handle:
            lib().pyci_gpu_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_all_dets(self, kind, nbasis, nocc_up, nocc_dn):
        from math import comb
        nd = comb(nbasis, nocc_up) * (comb(nbasis, nocc_dn) if kind == WFN_FULLCI else 1)
        nw = ((nbasis + 63) // 64) * (2 if kind == WFN_FULLCI else 1)
        out = np.zeros((nd, nw), dtype=np.uint64)
        check(lib().pyci_gpu_add_all_dets(self.handle, kind, nbasis, nocc_up, nocc_dn, _ptr(out)))
        return out

    def add_hci(self, kind, nbasis, nocc_up, nocc_dn, dets, coeffs, one_mo, two_mo, eps, flags=0):
        r"""New determinants of one heat-bath CI step (uint64[nnew, nwords]), first-occurrence order."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
        two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
        nw = dets.shape[1] if dets.ndim == 2 else ((nbasis + 63) // 64) * (2 if kind == WFN_FULLCI else 1)
        n = _i64(0)
        cap = max(1 << 16, 16 * dets.shape[0])  # a second call (full recount) only past this
        while True:
            out = np.zeros((cap, nw), dtype=np.uint64)
            check(lib().pyci_gpu_add_hci(self.handle, kind, nbasis, nocc_up, nocc_dn, dets.shape[0], _ptr(dets),
                                         _ptr(coeffs), _ptr(one_mo), _ptr(two_mo), float(eps), flags, cap,
                                         _ptr(out), ctypes.byref(n)))
            if n.value <= cap:
                return out[:n.value]
            cap = n.value

    def compute_rdms(self, kind, nbasis, nocc_up, nocc_dn, dets, coeffs):
        r"""(rdm1, rdm2) of a CI vector: DOCI (d0, d2) [n, n]; FullCI [2, n, n], [3, n, n, n, n];
        GenCI (definition-based, spin orbitals) [n, n], [n, n, n, n]."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        r1, r2 = _rdm_arrays(kind, nbasis)
        check(lib().pyci_gpu_compute_rdms(self.handle, kind, nbasis, nocc_up, nocc_dn, dets.shape[0], _ptr(dets),
                                          _ptr(coeffs), _ptr(r1), _ptr(r2)))
        return r1, r2

    def compute_transition_rdms(self, kind, nbasis, nocc_up, nocc_dn, dets1, coeffs1, dets2, coeffs2):
        r"""Transition (rdm1, rdm2) between two wave functions, same layouts as compute_rdms."""
        dets1 = np.ascontiguousarray(dets1, dtype=np.uint64)
        dets2 = np.ascontiguousarray(dets2, dtype=np.uint64)
        coeffs1 = np.ascontiguousarray(coeffs1, dtype=np.float64)
        coeffs2 = np.ascontiguousarray(coeffs2, dtype=np.float64)
        r1, r2 = _rdm_arrays(kind, nbasis)
        check(lib().pyci_gpu_compute_transition_rdms(self.handle, kind, nbasis, nocc_up, nocc_dn, dets1.shape[0],
                                                     _ptr(dets1), _ptr(coeffs1), dets2.shape[0], _ptr(dets2),
                                                     _ptr(coeffs2), _ptr(r1), _ptr(r2)))
        return r1, r2

    def compute_enpt2(self, kind, nbasis, nocc_up, nocc_dn, dets, coeffs, one_mo, two_mo, energy, ecore, eps):
        r"""Epstein-Nesbet second-order energy (energy + correction)."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
        two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
        out = ctypes.c_double(0.0)
        check(lib().pyci_gpu_compute_enpt2(self.handle, kind, nbasis, nocc_up, nocc_dn, dets.shape[0], _ptr(dets),
                                           _ptr(coeffs), _ptr(one_mo), _ptr(two_mo), float(energy), float(ecore),
                                           float(eps), ctypes.byref(out)))
        return out.value

    def gram_device(self, method, a_ptr, p, b_ptr, q, n):
        r"""C = A^T B (f64[p][q], host) for FP32 device vector blocks A [p][n] and B [q][n]."""
        out = np.zeros((p, q), dtype=np.float64)
        check(lib().pyci_gpu_gram_device(self.handle, method, a_ptr, p, b_ptr, q, n, _ptr(out)))
        return out


def _rdm_arrays(kind, n):
    if kind == WFN_FULLCI:
        return np.empty((2, n, n)), np.empty((3, n, n, n, n))
    if kind == WFN_GENCI:
        return np.empty((n, n)), np.empty((n, n, n, n))
    return np.empty((n, n)), np.empty((n, n))


class Csr:
    r"""A device CSR handle (pyci_gpu_csr)."""

    def __init__(self, ctx, kind, nbasis, nocc_up, nocc_dn, dets, one_mo, two_mo, nrow=-1, ncol=-1,
                 symmetric=True, flags=0, ndet=None):
        self.ctx = ctx
        one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
        two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
        if dets is not None:
            dets = np.ascontiguousarray(dets, dtype=np.uint64)
            ndet = dets.shape[0]
        h = _p()
        check(lib().pyci_gpu_csr_build(ctx.handle, kind, nbasis, nocc_up, nocc_dn, ndet, _ptr(dets), nrow,
                                       ncol, int(bool(symmetric)), _ptr(one_mo), _ptr(two_mo), flags,
                                       ctypes.byref(h)))
        self.handle = h

    def free(self):
        if self.handle:
            lib().pyci_gpu_csr_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def shape(self):
        v = [ctypes.c_int64() for _ in range(4)]
        check(lib().pyci_gpu_csr_shape(self.handle, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)  # nrow, ncol, size, nnz_stored

    def storage(self):
        r"""Bit flags STORE_* of the forms the operator holds on the device."""
        f = _int()
        check(lib().pyci_gpu_csr_storage(self.handle, ctypes.byref(f)))
        return f.value

    def product_form(self, precision, k):
        r"""FORM_* kernel form the autotuner chose for products of `precision` at width k."""
        f = _int()
        check(lib().pyci_gpu_csr_product_form(self.handle, precision, k, ctypes.byref(f)))
        return f.value

    def has_fcix(self):
        r"""Whether the operator holds the implicit-column form of a full FullCI space."""
        return bool(self.storage() & STORE_IMPLICIT)

    def export(self):
        nrow, ncol, size, _ = self.shape()
        data = np.empty(size, dtype=np.float64)
        indices = np.empty(size, dtype=np.int64)
        indptr = np.empty(nrow + 1, dtype=np.int64)
        check(lib().pyci_gpu_csr_export(self.handle, _ptr(data), _ptr(indices), _ptr(indptr)))
        return data, indices, indptr

    def get_element(self, i, j):
        out = ctypes.c_double()
        check(lib().pyci_gpu_csr_get_element(self.handle, i, j, ctypes.byref(out)))
        return out.value

    def matvec(self, x):
        nrow, ncol, _, _ = self.shape()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(nrow, dtype=np.float64)
        check(lib().pyci_gpu_csr_matvec(self.handle, _ptr(x), _ptr(y)))
        return y

    def matvec_noalloc(self, x):
        r"""op(x) staged in the library's fixed device arrays (no device allocation)."""
        nrow, ncol, _, _ = self.shape()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(nrow, dtype=np.float64)
        check(lib().pyci_gpu_csr_matvec_noalloc(self.handle, _ptr(x), _ptr(y)))
        return y

    def spmm_device(self, precision, k, x_ptr, y_ptr, stream=None):
        check(lib().pyci_gpu_csr_spmm_device(self.handle, precision, k, x_ptr, y_ptr, stream))

    def prepare_mixed(self, drop_fp64=False):
        check(lib().pyci_gpu_csr_prepare_mixed(self.handle, int(bool(drop_fp64))))

    def solve(self, n=1, c0=None, ncv=-1, maxiter=-1, tol=1e-12, ecore=0.0, mode=SOLVE_FP64, evecs=True):
        r"""(evals, evecs, stats); evecs is None when `evecs` is false (the
        eigenvectors then stay on the device and are not copied out)."""
        nrow = self.shape()[0]
        evals = np.empty(n, dtype=np.float64)
        evecs = np.empty((n, nrow), dtype=np.float64) if evecs else None
        st = SolveStats()
        c0 = None if c0 is None else np.ascontiguousarray(c0, dtype=np.float64)
        check(lib().pyci_gpu_csr_solve(self.handle, n, _ptr(c0), ncv, maxiter, tol, ecore, mode, _ptr(evals),
                                       _ptr(evecs), ctypes.byref(st)))
        return evals, evecs, st.as_dict()

    def digest(self):
        ps, px = ctypes.c_uint64(), ctypes.c_uint64()
        vs, va, vw = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().pyci_gpu_csr_digest(self.handle, ctypes.byref(ps), ctypes.byref(px), ctypes.byref(vs),
                                        ctypes.byref(va), ctypes.byref(vw)))
        return {"pattern_sum": str(ps.value), "pattern_xor": str(px.value), "value_sum": vs.value,
                "value_abs_sum": va.value, "value_wsum": vw.value}

    def update(self, dets, one_mo, two_mo, flags=0):
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        one_mo = np.ascontiguousarray(one_mo, dtype=np.float64)
        two_mo = np.ascontiguousarray(two_mo, dtype=np.float64)
        check(lib().pyci_gpu_csr_update(self.handle, dets.shape[0], _ptr(dets), _ptr(one_mo), _ptr(two_mo),
                                        flags))


def batch_solve(ctx, csrs, ecore, n=4, maxiter=-1, tol=1e-12, mode=SOLVE_FP64, evecs=False):
    r"""Lowest n eigenpairs of every operator in `csrs` (one batched solve).

    Returns (evals [nprob][n], stats) with stats["per_problem_iterations"],
    or (evals, evecs, stats) with evecs a list of [n][nrow_p] arrays when
    `evecs` is true.
    """
    arr = (ctypes.c_void_p * len(csrs))(*[c.handle.value if isinstance(c.handle, ctypes.c_void_p) else c.handle
                                          for c in csrs])
    ec = np.ascontiguousarray(ecore, dtype=np.float64)
    evals = np.empty((len(csrs), n), dtype=np.float64)
    iters = np.zeros(len(csrs), dtype=np.int64)
    vecs, vptr = None, None
    if evecs:
        vecs = [np.empty((n, c.shape()[0]), dtype=np.float64) for c in csrs]
        vptr = (ctypes.c_void_p * len(csrs))(*[v.ctypes.data for v in vecs])
    st = SolveStats()
    check(lib().pyci_gpu_batch_solve(ctx.handle, len(csrs), ctypes.cast(arr, ctypes.c_void_p), n, maxiter, tol,
                                     _ptr(ec), mode, _ptr(evals),
                                     ctypes.cast(vptr, ctypes.c_void_p) if vptr is not None else None,
                                     _ptr(iters), ctypes.byref(st)))
    stats = st.as_dict()
    stats["per_problem_iterations"] = iters.tolist()
    if evecs:
        return evals, vecs, stats
    return evals, stats
