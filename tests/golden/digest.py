r"""Order-independent digest of a CSR matrix (the definition that
pyci_gpu_csr_digest computes on the device), in numpy."""

import numpy as np

__all__ = ["digest", "mix64"]

MASK = (1 << 64) - 1


def mix64(x):
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x ^ (x >> np.uint64(30))
        x = x * np.uint64(0xBF58476D1CE4E5B9)
        x = x ^ (x >> np.uint64(27))
        x = x * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return x


def digest(data, indices, indptr):
    r"""The order-independent CSR digest of pyci_gpu_csr_digest."""
    n = indptr.shape[0] - 1
    psum = 0
    pxor = 0
    vsum = vabs = vw = 0.0
    r0 = 0
    while r0 < n:
        # Rows [r0, r1) holding at most ~16M entries.
        r1 = int(np.searchsorted(indptr, indptr[r0] + (1 << 24), side="right")) - 1
        r1 = min(max(r1, r0 + 1), n)
        s, e = int(indptr[r0]), int(indptr[r1])
        rows = np.repeat(np.arange(r0, r1, dtype=np.int64), np.diff(indptr[r0:r1 + 1]))
        i = rows.astype(np.uint64)
        j = indices[s:e].astype(np.uint64)
        h = mix64((i << np.uint64(32)) + j)
        psum = (psum + int(h.sum(dtype=np.uint64))) & MASK
        pxor ^= int(np.bitwise_xor.reduce(h)) if h.size else 0
        d = data[s:e]
        vsum += float(d.sum())
        vabs += float(np.abs(d).sum())
        w = 1.0 + ((rows * 31 + indices[s:e] * 17) % 1024) / 1024.0
        vw += float((d * w).sum())
        r0 = r1
    return {"pattern_sum": str(psum), "pattern_xor": str(pxor), "value_sum": vsum,
            "value_abs_sum": vabs, "value_wsum": vw, "nnz": int(indices.shape[0])}
