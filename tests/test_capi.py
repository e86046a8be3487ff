r"""The C-ABI library: it loads, and exports every symbol include/pyci_gb300.h
declares (no GPU needed)."""

import ctypes
import os
import re

import pytest

from pyci_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "pyci_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(pyci_gpu_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 18
    assert sorted(capi.SYMBOLS) == names
    lib = capi.lib()
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_error_string():
    lib = capi.lib()
    assert b"sm_103a" in lib.pyci_gpu_version()
    assert isinstance(lib.pyci_gpu_last_error(), bytes)


def test_null_arguments_are_rejected_without_a_gpu():
    lib = capi.lib()
    assert lib.pyci_gpu_ctx_create(0, None) == capi.EINVAL
    assert lib.pyci_gpu_csr_shape(None, None, None, None, None) == capi.EINVAL
    assert lib.pyci_gpu_csr_free(None) == capi.OK
    assert lib.pyci_gpu_ctx_destroy(None) == capi.OK


def test_no_gpu_reports_an_error_instead_of_crashing():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.GpuError):
        capi.Context(0)


def test_argument_errors_of_the_path_neighbours_without_a_gpu():
    # add_hci, compute_rdms, compute_transition_rdms, compute_enpt2 and the
    # Gram product reject bad arguments before any device work.  A zeroed
    # buffer stands in for a context: validation fails before it is used.
    lib = capi.lib()
    fake = ctypes.create_string_buffer(256)
    fake_ctx = ctypes.cast(fake, ctypes.c_void_p)
    n = ctypes.c_int64(0)
    out = ctypes.c_double(0.0)
    buf = ctypes.create_string_buffer(8 * 64)
    p = ctypes.cast(buf, ctypes.c_void_p)
    # NULL context or outputs
    assert lib.pyci_gpu_add_hci(None, capi.WFN_FULLCI, 6, 2, 2, 0, None, None, p, p, 1e-3, 0, 0, None,
                                ctypes.byref(n)) == capi.EINVAL
    assert lib.pyci_gpu_compute_rdms(None, capi.WFN_DOCI, 6, 2, 2, 0, None, None, p, p) == capi.EINVAL
    assert lib.pyci_gpu_compute_transition_rdms(None, capi.WFN_DOCI, 6, 2, 2, 0, None, None, 0, None, None, p,
                                                p) == capi.EINVAL
    assert lib.pyci_gpu_compute_enpt2(None, capi.WFN_DOCI, 6, 2, 2, 0, None, None, p, p, -1.0, 0.0, 1e-4,
                                      ctypes.byref(out)) == capi.EINVAL
    assert lib.pyci_gpu_gram_device(None, 1, p, 1, p, 1, 1, p) == capi.EINVAL
    # determinants without coefficients, negative counts, invalid occupations, unknown method
    assert lib.pyci_gpu_add_hci(fake_ctx, capi.WFN_FULLCI, 6, 2, 2, 3, p, None, p, p, 1e-3, 0, 0, None,
                                ctypes.byref(n)) == capi.EINVAL
    assert lib.pyci_gpu_add_hci(fake_ctx, capi.WFN_FULLCI, 6, 2, 2, -1, p, p, p, p, 1e-3, 0, 0, None,
                                ctypes.byref(n)) == capi.EINVAL
    assert lib.pyci_gpu_add_hci(fake_ctx, capi.WFN_FULLCI, 6, 1, 2, 1, p, p, p, p, 1e-3, 0, 0, None,
                                ctypes.byref(n)) == capi.EINVAL
    assert lib.pyci_gpu_compute_rdms(fake_ctx, capi.WFN_DOCI, 6, 3, 2, 1, p, p, p, p) == capi.EINVAL
    assert lib.pyci_gpu_compute_transition_rdms(fake_ctx, capi.WFN_FULLCI, 6, 2, 2, 1, p, p, -2, p, p, p,
                                                p) == capi.EINVAL
    assert lib.pyci_gpu_compute_enpt2(fake_ctx, capi.WFN_GENCI, 6, 3, 1, 1, p, p, p, p, -1.0, 0.0, 1e-4,
                                      ctypes.byref(out)) == capi.EINVAL
    assert lib.pyci_gpu_gram_device(fake_ctx, 7, p, 1, p, 1, 1, p) == capi.EINVAL
    assert lib.pyci_gpu_gram_device(fake_ctx, 1, p, -1, p, 1, 1, p) == capi.EINVAL
    assert b"invalid" in lib.pyci_gpu_last_error() or len(lib.pyci_gpu_last_error()) > 0


def test_host_module_argument_errors_without_a_gpu():
    import numpy as np
    import pyci_gb300 as pyci
    from pyci_gb300.synth import synthetic_integrals
    ecore, one, two = synthetic_integrals(6, 3)
    ham = pyci.secondquant_op(ecore, one, two)
    wfn = pyci.fullci_wfn(6, 2, 2)
    wfn.add_all_dets()
    with pytest.raises(ValueError):
        pyci.add_hci(ham, wfn, np.ones(3), eps=1e-3)  # fewer coefficients than determinants
    with pytest.raises(ValueError):
        pyci.compute_rdms(wfn, np.ones(3))
    with pytest.raises(ValueError):
        pyci.compute_enpt2(ham, wfn, np.ones(3), -1.0)
    other = pyci.fullci_wfn(6, 3, 2)
    other.add_hartreefock_det()
    with pytest.raises(ValueError):
        pyci.compute_transition_rdms(wfn, other, np.ones(len(wfn)), np.ones(len(other)))
    ham7 = pyci.secondquant_op(*synthetic_integrals(7, 3))
    with pytest.raises(ValueError):
        pyci.add_hci(ham7, wfn, np.ones(len(wfn)))  # Hamiltonian of another basis


def test_solve_stats_layout_matches_the_header(tmp_path):
    r"""The ctypes mirror of pyci_gpu_solve_stats has the C struct's field
    offsets and size (compiled against include/pyci_gb300.h with the host C
    compiler)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in capi.SolveStats._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"pyci_gb300.h\"\nint main(void) {\n"
                   + "".join('    printf("%%s %%zu\\n", "%s", offsetof(pyci_gpu_solve_stats, %s));\n' % (f, f)
                             for f in fields)
                   + '    printf("sizeof %zu\\n", sizeof(pyci_gpu_solve_stats));\n    return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                        text=True).stdout.splitlines())
    for f in fields:
        assert int(out[f]) == getattr(capi.SolveStats, f).offset, f
    assert int(out["sizeof"]) == ctypes.sizeof(capi.SolveStats)
