// Auxiliary device operations on the CSR handle: export to the reference's
// layout, order-independent digests, the FP32 high/low value split, and
// add_all_dets' determinant generation.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "detops.cuh"
#include "internal.h"
#include "split_bits.h"

namespace pyci_gpu {

// Copy row r's first len(r) entries (the reference layout's row) to the
// output arrays; cols widened to int64, values from f64 or from hi + lo.
__global__ void export_rows_kernel(int64_t r0, int64_t r1, const int64_t *rowptr,
                                   const int32_t *cols, const double *vals, const float *hi,
                                   const float *lo, const int32_t *lower_len,
                                   const int64_t *ref_rowptr, int64_t out_base,
                                   int64_t *out_idx, double *out_val) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = r0 + warp; r < r1; r += nwarps) {
        const int64_t src = rowptr[r];
        const int64_t len = lower_len ? lower_len[r] : rowptr[r + 1] - src;
        const int64_t dst = (ref_rowptr ? ref_rowptr[r] : src) - out_base;
        for (int64_t t = lane; t < len; t += 32) {
            if (out_idx)
                out_idx[dst + t] = cols[src + t];
            if (out_val)
                out_val[dst + t] = vals ? vals[src + t]
                                        : static_cast<double>(hi[src + t]) + static_cast<double>(lo[src + t]);
        }
    }
}

__global__ void digest_kernel(int64_t nrow, const int64_t *rowptr, const int32_t *cols,
                              const double *vals, const float *hi, const float *lo,
                              const int32_t *lower_len, unsigned long long *psum,
                              unsigned long long *pxor, double *vsum, double *vabs, double *vwsum) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    unsigned long long s = 0, x = 0;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int64_t r = warp; r < nrow; r += nwarps) {
        const int64_t src = rowptr[r];
        const int64_t len = lower_len ? lower_len[r] : rowptr[r + 1] - src;
        for (int64_t t = lane; t < len; t += 32) {
            const int64_t j = cols[src + t];
            const uint64_t h = mix64((static_cast<uint64_t>(r) << 32) + static_cast<uint64_t>(j));
            s += h;
            x ^= h;
            const double v = vals ? vals[src + t]
                                  : static_cast<double>(hi[src + t]) + static_cast<double>(lo[src + t]);
            a += v;
            b += fabs(v);
            c += v * (1.0 + static_cast<double>((r * 31 + j * 17) % 1024) / 1024.0);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        x ^= __shfl_xor_sync(0xffffffffu, x, o);
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
        atomicAdd(psum, s);
        atomicXor(pxor, x);
        atomicAdd(vsum, a);
        atomicAdd(vabs, b);
        atomicAdd(vwsum, c);
    }
}

// hi[i] = fl32(v[i]), lo[i] = fl32(v[i] - hi[i]) by integer arithmetic
// (split_bits.h).  Each thread handles 4 x 2 values per step: four
// independent 16-byte loads in flight before any arithmetic, 8-byte stores.
__global__ void split_kernel(int64_t n, const double *__restrict__ v, float *__restrict__ hi, float *__restrict__ lo) {
    constexpr int U = 4;
    const int64_t n2 = n / 2;                 // double2 elements
    const int64_t nb = n2 / U;                // full groups of U
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const double2 *v2 = reinterpret_cast<const double2 *>(v);
    float2 *h2 = reinterpret_cast<float2 *>(hi), *l2 = reinterpret_cast<float2 *>(lo);
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < nb; g += stride) {
        double2 d[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            d[u] = __ldcs(v2 + g + u * nb);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            float2 h, l;
            split_hi_lo(d[u].x, h.x, l.x);
            split_hi_lo(d[u].y, h.y, l.y);
            h2[g + u * nb] = h;
            l2[g + u * nb] = l;
        }
    }
    // Leftover double2 elements and a final odd value.
    for (int64_t i = U * nb + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n2; i += stride) {
        const double2 d = v2[i];
        float2 h, l;
        split_hi_lo(d.x, h.x, l.x);
        split_hi_lo(d.y, h.y, l.y);
        h2[i] = h;
        l2[i] = l;
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        split_hi_lo(v[n - 1], hi[n - 1], lo[n - 1]);
}

// Colex unranking into an arbitrary number of words (pyci/src/common.cpp:139-153).
__device__ void unrank_words(int64_t rank, int nbasis, int nocc, const int64_t *binom, int ldk,
                             uint64_t *out, int nword) {
    for (int w = 0; w < nword; ++w)
        out[w] = 0;
    int p = nbasis - 1;
    for (int j = nocc; j >= 1; --j) {
        while (p >= 0 && binom[p * ldk + j] > rank)
            --p;
        if (p < 0)
            return;
        out[p >> 6] |= 1ULL << (p & 63);
        rank -= binom[p * ldk + j];
        --p;
    }
}

// SELL-32 slice sizes: len[s] = 32 x (longest row of rows 32 s .. 32 s + 31).
__global__ void sell_sizes_kernel(int64_t nrow, const int64_t *__restrict__ rowptr, int64_t nslice,
                                  int64_t *__restrict__ len) {
    for (int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; s < nslice;
         s += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t longest = 0;
        const int64_t r1 = min(nrow, 32 * s + 32);
        for (int64_t r = 32 * s; r < r1; ++r)
            longest = max(longest, rowptr[r + 1] - rowptr[r]);
        len[s] = 32 * longest;
    }
}

// One warp per slice, in chunks of 32 entries: the warp loads entries
// j .. j + 31 of each of the slice's 32 rows (one coalesced 128-byte load per
// row and array) into a shared-memory tile, then writes position j' of all 32
// rows as one coalesced 128-byte store (off[s] + 32 j' + l for row 32 s + l),
// for the columns and both FP32 value halves.  Past a row's end the row's
// last column is repeated with zero values (a valid column near the lane's
// others); rows past nrow use column 0.
__global__ void __launch_bounds__(256) sell_fill_kernel(int64_t nrow, const int64_t *__restrict__ rowptr,
                                                        const int32_t *__restrict__ cols,
                                                        const float *__restrict__ hi, const float *__restrict__ lo,
                                                        int64_t nslice, const int64_t *__restrict__ off,
                                                        int32_t *__restrict__ scols, float *__restrict__ svals,
                                                        float *__restrict__ slo) {
    __shared__ uint32_t tile[8][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t s = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; s < nslice; s += nwarps) {
        const int64_t r = 32 * s + lane;
        const int64_t start = r < nrow ? rowptr[r] : 0;
        const int64_t len = r < nrow ? rowptr[r + 1] - start : 0;
        const int32_t last = len > 0 ? cols[start + len - 1] : 0;
        const int64_t o = off[s], L = (off[s + 1] - o) >> 5;
        for (int64_t j = 0; j < L; j += 32) {
            for (int a = 0; a < 3; ++a) {
                // 8 rows' loads in flight before their shared-memory stores.
                for (int r8 = 0; r8 < 32; r8 += 8) {
                    uint32_t v[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int rr = r8 + u;
                        const int64_t st = __shfl_sync(0xffffffffu, start, rr);
                        const int64_t ln = __shfl_sync(0xffffffffu, len, rr);
                        const int32_t lc = __shfl_sync(0xffffffffu, last, rr);
                        const int64_t e = j + lane;
                        if (a == 0)
                            v[u] = static_cast<uint32_t>(e < ln ? __ldcs(cols + st + e) : lc);
                        else if (a == 1)
                            v[u] = e < ln ? __float_as_uint(__ldcs(hi + st + e)) : 0u;
                        else
                            v[u] = e < ln ? __float_as_uint(__ldcs(lo + st + e)) : 0u;
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        tile[warp][r8 + u][lane] = v[u];
                }
                __syncwarp();
                const int64_t n = (L - j < 32) ? (L - j) : 32;
                for (int jj = 0; jj < n; ++jj) {
                    const uint32_t v = tile[warp][lane][jj];
                    const int64_t at = o + 32 * (j + jj) + lane;
                    if (a == 0)
                        scols[at] = static_cast<int32_t>(v);
                    else if (a == 1)
                        svals[at] = __uint_as_float(v);
                    else
                        slo[at] = __uint_as_float(v);
                }
                __syncwarp();
            }
        }
    }
}

__global__ void all_dets_kernel(int64_t ndet, int two_spin, int64_t nbeta, int nbasis, int nocc_up,
                                int nocc_dn, const int64_t *binom, int ldk, int nword,
                                uint64_t *dets) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < ndet;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (two_spin) {
            unrank_words(i / nbeta, nbasis, nocc_up, binom, ldk, dets + i * 2 * nword, nword);
            unrank_words(i % nbeta, nbasis, nocc_dn, binom, ldk, dets + i * 2 * nword + nword, nword);
        } else {
            unrank_words(i, nbasis, nocc_up, binom, ldk, dets + i * nword, nword);
        }
    }
}

} // namespace pyci_gpu

using namespace pyci_gpu;

static unsigned grid_for(const pyci_gpu_ctx *ctx, int64_t n, int threads) {
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = static_cast<int64_t>(ctx->num_sms) * 16;
    return static_cast<unsigned>(std::max<int64_t>(1, std::min(want, cap)));
}

int csr_export_device(const pyci_gpu_csr *csr, double *data, int64_t *indices, int64_t *indptr) {
    cudaStream_t st = csr->ctx->stream;
    if (data || indices || !(csr->symmetric ? csr->ref_rowptr : csr->rowptr)) {
        int rc = csr_materialize(csr);
        if (rc)
            return rc;
    }
    const int64_t nrow = csr->nrow;
    const int64_t *d_refptr = csr->symmetric ? csr->ref_rowptr : csr->rowptr;
    std::vector<int64_t> ptr(nrow + 1);
    PYCI_CUDA_TRY(cudaMemcpyAsync(ptr.data(), d_refptr, sizeof(int64_t) * (nrow + 1),
                                  cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    if (indptr)
        std::copy(ptr.begin(), ptr.end(), indptr);
    if (!data && !indices)
        return PYCI_GPU_OK;
    const int64_t budget = int64_t(1) << 27; // entries per staging chunk
    int64_t *d_idx = nullptr;
    double *d_val = nullptr;
    const int64_t stage = std::min<int64_t>(budget, std::max<int64_t>(ptr[nrow], 1));
    if (indices)
        PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_idx), sizeof(int64_t) * stage, st));
    if (data)
        PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_val), sizeof(double) * stage, st));
    int64_t r0 = 0;
    int rc = PYCI_GPU_OK;
    while (r0 < nrow) {
        // Largest r1 with ptr[r1] - ptr[r0] <= stage (at least one row).
        int64_t r1 = std::upper_bound(ptr.begin() + r0 + 1, ptr.end(), ptr[r0] + stage) - ptr.begin() - 1;
        if (r1 <= r0)
            r1 = r0 + 1;
        if (ptr[r1] - ptr[r0] > stage) {
            set_error("a single row exceeds the export staging buffer");
            rc = PYCI_GPU_ENOMEM;
            break;
        }
        export_rows_kernel<<<grid_for(csr->ctx, (r1 - r0) * 32, 256), 256, 0, st>>>(
            r0, r1, csr->rowptr, csr->cols, csr->vals, csr->hi, csr->lo,
            csr->symmetric ? csr->lower_len : nullptr, csr->symmetric ? csr->ref_rowptr : nullptr,
            ptr[r0], d_idx, d_val), ::pyci_gpu::note_launch();
        const int64_t cnt = ptr[r1] - ptr[r0];
        if (indices)
            PYCI_CUDA_TRY(cudaMemcpyAsync(indices + ptr[r0], d_idx, sizeof(int64_t) * cnt,
                                          cudaMemcpyDeviceToHost, st));
        if (data)
            PYCI_CUDA_TRY(cudaMemcpyAsync(data + ptr[r0], d_val, sizeof(double) * cnt,
                                          cudaMemcpyDeviceToHost, st));
        PYCI_CUDA_TRY(cudaStreamSynchronize(st));
        r0 = r1;
    }
    if (d_idx)
        cudaFreeAsync(d_idx, st);
    if (d_val)
        cudaFreeAsync(d_val, st);
    PYCI_CUDA_TRY(cudaGetLastError());
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    return rc;
}

int csr_digest_device(const pyci_gpu_csr *csr, uint64_t *psum, uint64_t *pxor, double *vsum,
                      double *vabs, double *vwsum) {
    cudaStream_t st = csr->ctx->stream;
    int rc0 = csr_materialize(csr);
    if (rc0)
        return rc0;
    struct Acc {
        unsigned long long s, x;
        double a, b, c;
    };
    Acc *d = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d), sizeof(Acc), st));
    PYCI_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(Acc), st));
    if (csr->nrow > 0)
        digest_kernel<<<grid_for(csr->ctx, csr->nrow * 32, 256), 256, 0, st>>>(
            csr->nrow, csr->rowptr, csr->cols, csr->vals, csr->hi, csr->lo,
            csr->symmetric ? csr->lower_len : nullptr, &d->s, &d->x, &d->a, &d->b, &d->c), ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    Acc h{};
    PYCI_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(Acc), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFreeAsync(d, st);
    if (psum)
        *psum = h.s;
    if (pxor)
        *pxor = h.x;
    if (vsum)
        *vsum = h.a;
    if (vabs)
        *vabs = h.b;
    if (vwsum)
        *vwsum = h.c;
    return PYCI_GPU_OK;
}

// SELL-32 copy of the split operator (see pyci_gpu_csr::sell_*), built when
// the slices' padding adds at most 1/16 to the stored entries (full FullCI
// and DOCI spaces have equal rows: no padding).  Skipped silently otherwise;
// the SpMM autotuner then never sees the variant.
static int sell_build(pyci_gpu_csr *csr) {
    cudaStream_t st = csr->ctx->stream;
    if (csr->lower_only || csr->nnz == 0 || csr->ncol == 0 || csr->nrow == 0 || csr->sell_cols)
        return PYCI_GPU_OK;
    const int64_t nslice = (csr->nrow + 31) / 32;
    int64_t *len = nullptr, *off = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&len), sizeof(int64_t) * nslice, st));
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&off), sizeof(int64_t) * (nslice + 1), st));
    sell_sizes_kernel<<<grid_for(csr->ctx, nslice, 256), 256, 0, st>>>(csr->nrow, csr->rowptr, nslice, len),
        ::pyci_gpu::note_launch();
    int rc = device_exclusive_scan(len, nslice, off, st);
    int64_t total = 0;
    if (rc == PYCI_GPU_OK) {
        cudaError_t e = cudaMemcpyAsync(&total, off + nslice, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            rc = cuda_status(e, "SELL sizes");
    }
    cudaFreeAsync(len, st);
    if (rc != PYCI_GPU_OK || total > csr->nnz + csr->nnz / 16) {
        cudaFreeAsync(off, st);
        return rc;
    }
    int32_t *scols = nullptr;
    float *svals = nullptr, *slo = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void **>(&scols), sizeof(int32_t) * total, st) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void **>(&svals), sizeof(float) * total, st) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void **>(&slo), sizeof(float) * total, st) != cudaSuccess) {
        // Out of device memory: the CSR kernels serve the split products.
        cudaGetLastError();
        if (scols)
            cudaFreeAsync(scols, st);
        if (svals)
            cudaFreeAsync(svals, st);
        cudaFreeAsync(off, st);
        return PYCI_GPU_OK;
    }
    sell_fill_kernel<<<grid_for(csr->ctx, nslice * 32, 256), 256, 0, st>>>(csr->nrow, csr->rowptr, csr->cols, csr->hi,
                                                                           csr->lo, nslice, off, scols, svals, slo),
        ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    csr->nslice = nslice;
    csr->sell_nnz = total;
    csr->sell_off = off;
    csr->sell_cols = scols;
    csr->sell_vals = svals;
    csr->sell_lo = slo;
    return PYCI_GPU_OK;
}

// The exact FP32 high/low split in CSR order (for the CSR and SELL-32
// kernels and the batched solver); a no-op once it exists.
int csr_ensure_split(pyci_gpu_csr *csr) {
    if (csr->hi && csr->lo)
        return PYCI_GPU_OK;
    cudaStream_t st = csr->ctx->stream;
    int rc = csr_materialize(csr);
    if (rc)
        return rc;
    if (!csr->vals) {
        set_error("operator has no FP64 values to split");
        return PYCI_GPU_EINVAL;
    }
    const int64_t n = csr->nnz ? csr->nnz : 1;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->hi), sizeof(float) * n, st));
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->lo), sizeof(float) * n, st));
    if (csr->nnz > 0)
        split_kernel<<<grid_for(csr->ctx, csr->nnz, 256), 256, 0, st>>>(csr->nnz, csr->vals, csr->hi, csr->lo),
            ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    if (csr->drop_fp64) {
        PYCI_CUDA_TRY(cudaFreeAsync(csr->vals, st));
        csr->vals = nullptr;
    }
    return PYCI_GPU_OK;
}

int csr_prepare_mixed_device(pyci_gpu_csr *csr, int drop_fp64) {
    cudaStream_t st = csr->ctx->stream;
    if (drop_fp64)
        csr->drop_fp64 = true;
    if (has_implicit(csr)) {
        // A full FullCI or DOCI space: the implicit form, which
        // serves the FP32 and double-float products; the CSR-order split is
        // made on demand (csr_ensure_split), or here when the FP64 values go.
        if (drop_fp64 && csr->vals) {
            int rc = csr_ensure_split(csr);
            if (rc)
                return rc;
        }
    } else if (!csr->hi) {
        if (!csr->vals) {
            set_error("operator has no FP64 values to split");
            return PYCI_GPU_EINVAL;
        }
        const int64_t n = csr->nnz ? csr->nnz : 1;
        PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->hi), sizeof(float) * n, st));
        PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->lo), sizeof(float) * n, st));
        if (csr->nnz > 0)
            split_kernel<<<grid_for(csr->ctx, csr->nnz, 256), 256, 0, st>>>(csr->nnz, csr->vals,
                                                                           csr->hi, csr->lo), ::pyci_gpu::note_launch();
        PYCI_CUDA_TRY(cudaGetLastError());
        int rc = sell_build(csr);
        if (rc)
            return rc;
    }
    if (drop_fp64 && csr->vals) {
        PYCI_CUDA_TRY(cudaFreeAsync(csr->vals, st));
        csr->vals = nullptr;
    }
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    return PYCI_GPU_OK;
}

int add_all_dets_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                        int64_t nocc_dn, uint64_t *dets_host) {
    cudaStream_t st = ctx->stream;
    const int two = (kind == PYCI_WFN_FULLCI);
    const int64_t na = host_binomial(nbasis, nocc_up);
    const int64_t nb = two ? host_binomial(nbasis, nocc_dn) : 1;
    if (na == INT64_MAX || nb == INT64_MAX || (nb && na > INT64_MAX / nb)) {
        set_error("cannot generate > 2 ** 63 determinants");
        return PYCI_GPU_EINVAL;
    }
    const int64_t ndet = na * nb;
    const int nword = static_cast<int>((nbasis + 63) / 64);
    const int ldk = static_cast<int>(std::max(nocc_up, nocc_dn) + 2);
    std::vector<int64_t> binom((nbasis + 1) * ldk);
    for (int64_t m = 0; m <= nbasis; ++m)
        for (int k = 0; k < ldk; ++k)
            binom[m * ldk + k] = host_binomial(m, k);
    int64_t *d_binom = nullptr;
    uint64_t *d_dets = nullptr;
    const int64_t words = ndet * nword * (two ? 2 : 1);
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_binom), sizeof(int64_t) * binom.size(), st));
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_dets), sizeof(uint64_t) * (words ? words : 1), st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_binom, binom.data(), sizeof(int64_t) * binom.size(),
                                  cudaMemcpyHostToDevice, st));
    if (ndet > 0)
        all_dets_kernel<<<grid_for(ctx, ndet, 256), 256, 0, st>>>(
            ndet, two, nb, static_cast<int>(nbasis), static_cast<int>(nocc_up),
            static_cast<int>(nocc_dn), d_binom, ldk, nword, d_dets), ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    PYCI_CUDA_TRY(cudaMemcpyAsync(dets_host, d_dets, sizeof(uint64_t) * words, cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFreeAsync(d_binom, st);
    cudaFreeAsync(d_dets, st);
    return PYCI_GPU_OK;
}
