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
