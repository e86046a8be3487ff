r"""op(x) through pyci_gpu_csr_matvec_noalloc, the entry point that stages x and
y in the library's fixed device arrays instead of allocating device memory.
It serves callers that cannot let a library allocate device memory while
they run (a host whose own allocator has reserved the GPU's memory, or one
that must know the library's device footprint in advance).  Its output must
match the allocating pyci_gpu_csr_matvec on consecutive calls, a warm call
must leave the device's free memory unchanged, and sizes past the arrays'
limit must be rejected.  Collected last on purpose: if it fails, a run that
stops at the first failure has already run every other test."""

import numpy as np
import pytest

import oracle as O
from conftest import load_csr_case
from pyci_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("case", ["fci_6_3_2", "fci_7_3_2_rect", "genci_10_4"])
def test_noalloc_matches_allocating_matvec(ctx, golden, case):
    meta = {m["name"]: m for m in golden["csr_cases"]}[case]
    ref = load_csr_case(case)
    kind = {"doci": capi.WFN_DOCI, "fullci": capi.WFN_FULLCI, "genci": capi.WFN_GENCI}[meta["wfn"]]
    csr = capi.Csr(ctx, kind, meta["nbasis"], meta["nocc_up"], meta["nocc_dn"], ref["dets"], ref["one_mo"],
                   ref["two_mo"], meta["nrow"], meta["ncol"], meta["symmetric"])
    rng = np.random.default_rng(7)
    ncol = csr.shape()[1]
    for _ in range(2):  # two calls in a row: the shared arrays keep the previous call's contents
        x = rng.normal(size=ncol)
        y_alloc = csr.matvec(x)
        y_noalloc = csr.matvec_noalloc(x)
        np.testing.assert_allclose(y_noalloc, y_alloc, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(csr.matvec_noalloc(ref["x"]), ref["y"], rtol=1e-12, atol=1e-11)
    csr.free()


def _free_device_memory():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_allocates_no_device_memory(ctx):
    # After a warm call (kernels loaded, product variant chosen), further calls
    # must not change the device's free memory; the allocating matvec, by
    # contrast, takes its x and y buffers from the device's memory pool.
    from math import comb
    from pyci_gb300.synth import synthetic_integrals
    ecore, one, two = synthetic_integrals(10, 1010)
    n = comb(10, 5) ** 2
    csr = capi.Csr(ctx, capi.WFN_FULLCI, 10, 5, 5, None, one, two, flags=capi.BUILD_FULL_COLEX, ndet=n)
    x = np.random.default_rng(5).normal(size=n)
    y_ref = csr.matvec(x)
    csr.matvec_noalloc(x)  # warm call
    before = _free_device_memory()
    for _ in range(3):
        y = csr.matvec_noalloc(x)
    after = _free_device_memory()
    assert after == before, "free device memory changed by %d bytes" % (before - after)
    np.testing.assert_allclose(y, y_ref, rtol=1e-12, atol=1e-12)
    csr.free()


def test_noalloc_full_size_fci(ctx):
    # 12 orbitals, 5 alpha + 5 beta: 627,264 rows, inside the 2^20 limit.
    from math import comb
    from pyci_gb300.synth import synthetic_integrals
    ecore, one, two = synthetic_integrals(12, 1003)
    n = comb(12, 5) ** 2
    csr = capi.Csr(ctx, capi.WFN_FULLCI, 12, 5, 5, None, one, two, flags=capi.BUILD_FULL_COLEX, ndet=n)
    rng = np.random.default_rng(3)
    for _ in range(2):
        x = rng.normal(size=n)
        np.testing.assert_allclose(csr.matvec_noalloc(x), csr.matvec(x), rtol=1e-12, atol=1e-12)
    csr.free()


def test_noalloc_rejects_sizes_past_the_limit(ctx):
    # A 10-row slice of the 28-orbital, 7-pair DOCI space has 1,184,040 columns.
    from pyci_gb300.synth import synthetic_integrals
    ecore, one, two = synthetic_integrals(28, 5)
    n = O.lib().orc_binomial(28, 7)
    assert n > 1 << 20
    csr = capi.Csr(ctx, capi.WFN_DOCI, 28, 7, 7, None, one, two, nrow=10, symmetric=False,
                   flags=capi.BUILD_FULL_COLEX, ndet=n)
    x = np.ones(n)
    with pytest.raises(ValueError, match="at most"):
        csr.matvec_noalloc(x)
    assert np.isfinite(csr.matvec(x)).all()  # the allocating path still works
    csr.free()
