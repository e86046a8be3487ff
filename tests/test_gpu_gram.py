r"""Tall-skinny Gram products V^T W of the mixed-precision eigensolver: the
tensor-core (tcgen05, TF32 high/low split) and CUDA-core kernels against an
FP64 product of the same FP32 vectors, through the C ABI."""

import numpy as np
import pytest

from pyci_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = capi.Context(0)
    yield c
    c.close()


def gram_case(ctx, p, q, n, seed, same=False):
    import torch
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((p, n)).astype(np.float32)
    b = a[:q].copy() if same else rng.standard_normal((q, n)).astype(np.float32)
    ad = torch.tensor(a, device="cuda")
    bd = torch.tensor(b, device="cuda")
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    scale = np.outer(np.linalg.norm(a.astype(np.float64), axis=1), np.linalg.norm(b.astype(np.float64), axis=1))
    out = {}
    for method in (capi.GRAM_CUDA_CORES, capi.GRAM_TENSOR_CORES):
        out[method] = ctx.gram_device(method, ad.data_ptr(), p, bd.data_ptr(), q, n)
    return ref, scale, out


# Shapes: the eigensolver's (subspace m up to 64 against a block of <= 8), the
# largest tile (128 x 8) and a wide block with a partial last tile (both
# TMA-fed), more than one tile of A (p > 128) and of B (q > 8), N not a
# multiple of 4 (scalar loads) and N smaller than one 32-row tile.
@pytest.mark.parametrize("p,q,n", [(64, 4, 1 << 20), (128, 8, 627264), (100, 4, 1000004), (5, 3, 4900),
                                   (1, 1, 37), (7, 2, 5), (130, 9, 100003), (33, 8, 134596)])
def test_gram_tensor_cores_match_fp64(ctx, p, q, n):
    ref, scale, out = gram_case(ctx, p, q, n, seed=p * 1000 + q)
    for method, c in out.items():
        # FP32 (or split-TF32) products, FP32 sums within each CTA's rows,
        # FP64 across CTAs: relative to |a_i| |b_j| well below 1e-6.
        err = np.abs(c - ref) / scale
        assert err.max() < 2e-6, (method, err.max())
    # Both paths compute the same sums to the same accuracy.
    assert np.abs(out[capi.GRAM_TENSOR_CORES] - out[capi.GRAM_CUDA_CORES]).max() / scale.max() < 2e-6


@pytest.mark.parametrize("p", [8, 128])
def test_gram_of_orthonormal_block_is_identity(ctx, p):
    import torch
    n, k = 100000, 8
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.standard_normal((n, p)))
    v = np.ascontiguousarray(q.T).astype(np.float32)
    vd = torch.tensor(v, device="cuda")
    g = ctx.gram_device(capi.GRAM_TENSOR_CORES, vd.data_ptr(), p, vd.data_ptr(), k, n)
    # FP32 rounding of the vectors alone moves the Gram by ~1e-7; the tensor
    # core's own accumulation must add no bias on top (it did, -3e-6, with
    # one accumulator per CTA).
    assert np.abs(g - np.eye(p, k)).max() < 1e-6
    np.testing.assert_allclose(g[:k], g[:k].T, atol=1e-7)


def test_gram_repeats_bit_identically(ctx):
    import torch
    rng = np.random.default_rng(3)
    a = torch.tensor(rng.standard_normal((48, 300001)).astype(np.float32), device="cuda")
    b = torch.tensor(rng.standard_normal((4, 300001)).astype(np.float32), device="cuda")
    c1 = ctx.gram_device(capi.GRAM_TENSOR_CORES, a.data_ptr(), 48, b.data_ptr(), 4, 300001)
    c2 = ctx.gram_device(capi.GRAM_TENSOR_CORES, a.data_ptr(), 48, b.data_ptr(), 4, 300001)
    assert np.array_equal(c1, c2)
