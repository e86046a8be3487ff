// Implicit products for full DOCI spaces ("DOCX"), part of
// SparseOp::perform_op (pyci/src/sparseop.cpp:96-112).
//
// In a full DOCI space every determinant is a set S of m doubly occupied
// orbitals out of n, ranked in colex order, rank(S) = sum over the sorted
// members o_0 < ... < o_{m-1} of C(o_i, i + 1).  Row S holds its diagonal and
// one entry per pair move p -> q (p in S, q not in S), with value v[p][q]
// (the pair-excitation integral, the same for every row:
// pyci/src/sparseop.cpp:220-258) and column rank(S - p + q).  So a product
// needs no stored entries at all: each lane owns one row, derives the
// columns from its occupation and reads v from shared memory; only x, y and
// the diagonal move through HBM.
//
// Column of p -> q.  With S_p = S - {p} (members sp_0 < ... < sp_{m-2}) and
// k = the number of members of S_p below q, the members below q keep their
// index, q takes index k and the members above move up by one, so
//   rank(S_p + q) = H_p[k] + C(q, k + 1),
//   H_p[k] = sum_{i < k} C(sp_i, i + 1) + sum_{i >= k} C(sp_i, i + 2).
// Each lane builds H_p (m values) once per occupied p in shared memory; per
// move the column is a population count, two shared-memory reads and an
// add.  Ranks are below 2^31; the sums run in 32-bit unsigned arithmetic
// (binomials reduced mod 2^32), exact because the result is.
//
// Tables: binomials C(o, k) for o <= n, k <= m + 1 (int64), and v split into
// FP32 high and low parts.  The diagonal is the operator's (FP64, split per
// row for the double-float product).

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>

#include "dfarith.cuh"
#include "internal.h"
#include "split_bits.h"

namespace pyci_gpu {

struct DxArgs {
    int64_t nrow;
    int n, m, ldk;
    const int64_t *binom; // [(n + 1) * ldk]
    const float *v;       // [2][n][n]: high parts, then low parts
    const double *diag;   // [nrow]
    int64_t ycol;         // FP32 output: 0 = rows of K values, else column k at y + k * ycol
};

__host__ __device__ inline size_t dx_align16(size_t b) { return (b + 15) / 16 * 16; }

// Shared memory: binomials (int64 for the unranking, uint32 mod 2^32 for the
// columns), v (high, low), then per warp the lanes' occupied orbitals and
// H_p, [m][32] each.
__host__ __device__ inline size_t dx_fixed_bytes(int n, int ldk) {
    return dx_align16(sizeof(int64_t) * (n + 1) * ldk) + dx_align16(sizeof(uint32_t) * (n + 1) * ldk) +
           dx_align16(sizeof(float) * 2 * n * n);
}
__host__ __device__ inline size_t dx_warp_bytes(int m) { return 2 * dx_align16(sizeof(int) * m * 32); }

// MODE 0: FP32 (x, y float [N][K]); MODE 2: double-float (xs float [N][2K],
// y double [N][K]).  One warp per 32 consecutive rows; M: the occupation
// mask type (32 bits when n <= 32).
template<int MODE, int K, typename M>
__global__ void __launch_bounds__(256) docx_spmm_kernel(DxArgs A, const float *__restrict__ x, void *__restrict__ yv) {
    constexpr int XW = MODE == 2 ? 2 * K : K; // floats per x row
    constexpr int MB = 8 * sizeof(M);
    extern __shared__ __align__(16) unsigned char dx_smem[];
    const int n = A.n, m = A.m, ldk = A.ldk, nb = (n + 1) * ldk;
    int64_t *bn = reinterpret_cast<int64_t *>(dx_smem);
    uint32_t *bu = reinterpret_cast<uint32_t *>(dx_smem + dx_align16(sizeof(int64_t) * nb));
    float *vh = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(bu) + dx_align16(sizeof(uint32_t) * nb));
    float *vl = vh + n * n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *mine = dx_smem + dx_fixed_bytes(n, ldk) + dx_warp_bytes(m) * warp;
    int *occ = reinterpret_cast<int *>(mine);
    uint32_t *H = reinterpret_cast<uint32_t *>(mine + dx_align16(sizeof(int) * m * 32));
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        const int64_t c = __ldg(A.binom + i);
        bn[i] = c;
        bu[i] = static_cast<uint32_t>(c);
    }
    for (int i = threadIdx.x; i < 2 * n * n; i += blockDim.x)
        vh[i] = __ldg(A.v + i);
    __syncthreads();
    const int64_t row = (static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp) * 32 + lane;
    if (row - lane >= A.nrow)
        return;
    const bool valid = row < A.nrow;
    const int s = static_cast<int>(valid ? row : A.nrow - 1);
    // Occupation of row s (colex unranking).
    M S = 0;
    {
        int64_t r = s;
        int o = n - 1;
        for (int j = m; j >= 1; --j) {
            while (bn[o * ldk + j] > r)
                --o;
            S |= M(1) << o;
            occ[(j - 1) * 32 + lane] = o;
            r -= bn[o * ldk + j];
            --o;
        }
    }
    float acc[K], cc[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
        acc[k] = cc[k] = 0.0f;
    {
        float dh, dl;
        split_hi_lo(__ldg(A.diag + s), dh, dl);
        df_acc<MODE, K>(x + static_cast<int64_t>(s) * XW, dh, dl, acc, cc);
    }
    const M full = n >= MB ? ~M(0) : ((M(1) << n) - 1);
    const int nv = n - m;
    const int last = static_cast<int>(A.nrow - 1);
    for (int a = 0; a < m; ++a) {
        const int p = occ[a * 32 + lane];
        const M Sp = S & ~(M(1) << p);
        // H_p[k], k = 0 .. m - 1: suffix sums of C(sp_i, i + 2), then the
        // prefix sums of C(sp_i, i + 1) added (sp_i = occ[i] below a, occ[i + 1] from a on).
        {
            uint32_t hs = 0;
            H[(m - 1) * 32 + lane] = 0;
            for (int k = m - 2; k >= 0; --k) {
                const int sp = occ[(k < a ? k : k + 1) * 32 + lane];
                hs += bu[sp * ldk + k + 2];
                H[k * 32 + lane] = hs;
            }
            uint32_t ls = 0;
            for (int k = 0; k < m; ++k) {
                H[k * 32 + lane] += ls;
                if (k < m - 1)
                    ls += bu[occ[(k < a ? k : k + 1) * 32 + lane] * ldk + k + 1];
            }
        }
        const float *ph = vh + p * n, *pl = vl + p * n;
        M vir = ~S & full;
        // Four moves at a time: their x rows are loaded before any is used.
        for (int j0 = 0; j0 < nv; j0 += 4) {
            int rr[4];
            float wh[4], wl[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                rr[u] = s;
                wh[u] = wl[u] = 0.0f;
                if (j0 + u < nv) {
                    int q;
                    if constexpr (MB == 32)
                        q = __ffs(static_cast<int>(vir)) - 1;
                    else
                        q = __ffsll(static_cast<long long>(vir)) - 1;
                    vir &= vir - 1;
                    const M below = Sp & ((M(1) << q) - 1);
                    const int kq = MB == 32 ? __popc(static_cast<unsigned>(below)) : __popcll(below);
                    const int r = static_cast<int>(H[kq * 32 + lane] + bu[q * ldk + kq + 1]);
                    rr[u] = min(max(r, 0), last); // in range by construction
                    wh[u] = ph[q];
                    if (MODE == 2)
                        wl[u] = pl[q];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                df_acc<MODE, K>(x + static_cast<int64_t>(rr[u]) * XW, wh[u], wl[u], acc, cc);
        }
    }
    if (valid) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if constexpr (MODE == 0)
                static_cast<float *>(yv)[A.ycol ? k * A.ycol + row : row * K + k] = acc[k];
            else
                static_cast<double *>(yv)[row * K + k] = static_cast<double>(acc[k]) + static_cast<double>(cc[k]);
        }
    }
}

template<int MODE, int K, typename M>
bool dx_launch_m(const pyci_gpu_csr *csr, const void *x, void *y, cudaStream_t st, int64_t ycol) {
    DxArgs A;
    A.ycol = ycol;
    A.nrow = csr->nrow;
    A.n = csr->dx_n;
    A.m = csr->dx_m;
    A.ldk = csr->dx_ldk;
    A.binom = csr->dx_binom;
    A.v = csr->dx_v;
    A.diag = csr->diag;
    static const size_t limit = [&] {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, docx_spmm_kernel<MODE, K, M>);
        const size_t lim = csr->ctx->smem_optin > fa.sharedSizeBytes ? csr->ctx->smem_optin - fa.sharedSizeBytes : 0;
        cudaFuncSetAttribute(docx_spmm_kernel<MODE, K, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(lim));
        return lim;
    }();
    // Up to 8 warps per block while shared memory stays <= 64 KB.
    const size_t fixed = dx_fixed_bytes(A.n, A.ldk), per = dx_warp_bytes(A.m);
    int warps = 8;
    while (warps > 1 && fixed + per * warps > 64 * 1024)
        --warps;
    const size_t smem = fixed + per * warps;
    if (smem > limit)
        return false;
    const int64_t rows_per_block = 32 * warps;
    const int64_t blocks = (A.nrow + rows_per_block - 1) / rows_per_block;
    if (blocks <= 0)
        return true;
    docx_spmm_kernel<MODE, K, M><<<static_cast<unsigned>(blocks), 32 * warps, smem, st>>>(
        A, static_cast<const float *>(x), y);
    note_launch();
    return true;
}

template<int MODE, int K>
bool dx_launch_k(const pyci_gpu_csr *csr, const void *x, void *y, cudaStream_t st, int64_t ycol = 0) {
    return csr->dx_n <= 32 ? dx_launch_m<MODE, K, uint32_t>(csr, x, y, st, ycol)
                           : dx_launch_m<MODE, K, uint64_t>(csr, x, y, st, ycol);
}

} // namespace pyci_gpu

using namespace pyci_gpu;

bool docx_launch(const pyci_gpu_csr *csr, int mode, int K, const void *x, int64_t ldx, void *y, int64_t ldy,
                 cudaStream_t st) {
    if (!csr->dx_v || !csr->dx_binom || !csr->diag || csr->nrow >= INT32_MAX)
        return false;
    if (mode == 0) {
        const size_t align = (K % 4 == 0) ? 16 : (K == 2 ? 8 : 4);
        if (ldx != K || ldy != K || reinterpret_cast<uintptr_t>(x) % align)
            return false;
        switch (K) {
        case 1: return dx_launch_k<0, 1>(csr, x, y, st);
        case 2: return dx_launch_k<0, 2>(csr, x, y, st);
        case 3: return dx_launch_k<0, 3>(csr, x, y, st);
        case 4: return dx_launch_k<0, 4>(csr, x, y, st);
        case 5: return dx_launch_k<0, 5>(csr, x, y, st);
        case 6: return dx_launch_k<0, 6>(csr, x, y, st);
        case 7: return dx_launch_k<0, 7>(csr, x, y, st);
        case 8: return dx_launch_k<0, 8>(csr, x, y, st);
        default: return false;
        }
    }
    if (mode != 2 || ldx != 2 * K || ldy != K || reinterpret_cast<uintptr_t>(x) % 16)
        return false;
    switch (K) {
    case 1: return dx_launch_k<2, 1>(csr, x, y, st);
    case 2: return dx_launch_k<2, 2>(csr, x, y, st);
    case 4: return dx_launch_k<2, 4>(csr, x, y, st);
    default: return false;
    }
}

bool docx_launch_columns(const pyci_gpu_csr *csr, int K, const float *x, float *y, cudaStream_t st) {
    if (!csr->dx_v || !csr->dx_binom || !csr->diag || csr->nrow >= INT32_MAX)
        return false;
    const size_t align = (K % 4 == 0) ? 16 : (K == 2 ? 8 : 4);
    if (reinterpret_cast<uintptr_t>(x) % align)
        return false;
    const int64_t n = csr->nrow;
    switch (K) {
    case 1: return dx_launch_k<0, 1>(csr, x, y, st, n);
    case 2: return dx_launch_k<0, 2>(csr, x, y, st, n);
    case 3: return dx_launch_k<0, 3>(csr, x, y, st, n);
    case 4: return dx_launch_k<0, 4>(csr, x, y, st, n);
    case 5: return dx_launch_k<0, 5>(csr, x, y, st, n);
    case 6: return dx_launch_k<0, 6>(csr, x, y, st, n);
    case 7: return dx_launch_k<0, 7>(csr, x, y, st, n);
    case 8: return dx_launch_k<0, 8>(csr, x, y, st, n);
    default: return false;
    }
}
