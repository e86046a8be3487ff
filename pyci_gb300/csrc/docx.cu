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
// Column of p -> q.  With a = index of p in S and b = number of members
// below q (p included when p < q): moving p to q shifts the index of every
// member between them by one, so
//   q > p:  rank' = rank - C(p, a + 1) + C(q, b) + sum_{a < i < b} (C(o_i, i) - C(o_i, i + 1))
//   q < p:  rank' = rank - C(p, a + 1) + C(q, b + 1) + sum_{b <= i < a} (C(o_i, i + 2) - C(o_i, i + 1))
// and the sums are differences of per-row prefix sums Dd, Du that each lane
// keeps in shared memory; b is a population count.
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
};

__host__ __device__ inline size_t dx_align16(size_t b) { return (b + 15) / 16 * 16; }

// Shared memory: binomials, v (high, low), then per warp the lanes'
// occupied orbitals [m][32] (int) and prefix sums Dd, Du [m + 1][32] (int64).
__host__ __device__ inline size_t dx_fixed_bytes(int n, int ldk) {
    return dx_align16(sizeof(int64_t) * (n + 1) * ldk) + dx_align16(sizeof(float) * 2 * n * n);
}
__host__ __device__ inline size_t dx_warp_bytes(int m) {
    return dx_align16(sizeof(int) * m * 32) + 2 * dx_align16(sizeof(int64_t) * (m + 1) * 32);
}

// MODE 0: FP32 (x, y float [N][K]); MODE 2: double-float (xs float [N][2K],
// y double [N][K]).  One warp per 32 consecutive rows.
template<int MODE, int K>
__global__ void __launch_bounds__(256) docx_spmm_kernel(DxArgs A, const float *__restrict__ x, void *__restrict__ yv) {
    constexpr int XW = MODE == 2 ? 2 * K : K; // floats per x row
    extern __shared__ __align__(16) unsigned char dx_smem[];
    const int n = A.n, m = A.m, ldk = A.ldk;
    int64_t *bn = reinterpret_cast<int64_t *>(dx_smem);
    float *vh = reinterpret_cast<float *>(dx_smem + dx_align16(sizeof(int64_t) * (n + 1) * ldk));
    float *vl = vh + n * n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *mine = dx_smem + dx_fixed_bytes(n, ldk) + dx_warp_bytes(m) * warp;
    int *occ = reinterpret_cast<int *>(mine);
    int64_t *Dd = reinterpret_cast<int64_t *>(mine + dx_align16(sizeof(int) * m * 32));
    int64_t *Du = Dd + dx_align16(sizeof(int64_t) * (m + 1) * 32) / sizeof(int64_t);
    for (int i = threadIdx.x; i < (n + 1) * ldk; i += blockDim.x)
        bn[i] = __ldg(A.binom + i);
    for (int i = threadIdx.x; i < 2 * n * n; i += blockDim.x)
        vh[i] = __ldg(A.v + i);
    __syncthreads();
    const int64_t row = (static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp) * 32 + lane;
    if (row - lane >= A.nrow)
        return;
    const bool valid = row < A.nrow;
    const int64_t s = valid ? row : A.nrow - 1;
    // Occupation of row s (colex unranking), then the prefix sums.
    uint64_t S = 0;
    {
        int64_t r = s;
        int o = n - 1;
        for (int j = m; j >= 1; --j) {
            while (bn[o * ldk + j] > r)
                --o;
            S |= 1ULL << o;
            r -= bn[o * ldk + j];
            --o;
        }
        uint64_t w = S;
        int64_t dd = 0, du = 0;
        Dd[lane] = 0;
        Du[lane] = 0;
        for (int i = 0; i < m; ++i) {
            const int oi = __ffsll(static_cast<long long>(w)) - 1;
            w &= w - 1;
            occ[i * 32 + lane] = oi;
            const int64_t c1 = bn[oi * ldk + i + 1];
            dd += bn[oi * ldk + i] - c1;
            du += bn[oi * ldk + i + 2] - c1;
            Dd[(i + 1) * 32 + lane] = dd;
            Du[(i + 1) * 32 + lane] = du;
        }
    }
    __syncwarp();
    float acc[K], cc[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
        acc[k] = cc[k] = 0.0f;
    {
        float dh, dl;
        split_hi_lo(__ldg(A.diag + s), dh, dl);
        df_acc<MODE, K>(x + s * XW, dh, dl, acc, cc);
    }
    const uint64_t full = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    const int nv = n - m;
    for (int a = 0; a < m; ++a) {
        const int p = occ[a * 32 + lane];
        const int64_t base = s - bn[p * ldk + a + 1];
        const int64_t dda = Dd[(a + 1) * 32 + lane], dua = Du[a * 32 + lane];
        const float *ph = vh + p * n, *pl = vl + p * n;
        uint64_t vir = ~S & full;
        // Four moves at a time: their x rows are loaded before any is used.
        for (int j0 = 0; j0 < nv; j0 += 4) {
            int64_t rr[4];
            float wh[4], wl[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                rr[u] = s;
                wh[u] = wl[u] = 0.0f;
                if (j0 + u < nv) {
                    const int q = __ffsll(static_cast<long long>(vir)) - 1;
                    vir &= vir - 1;
                    const int b = __popcll(S & ((1ULL << q) - 1));
                    const int64_t r = q > p ? base + bn[q * ldk + b] + Dd[b * 32 + lane] - dda
                                            : base + bn[q * ldk + b + 1] + dua - Du[b * 32 + lane];
                    rr[u] = min(max(r, static_cast<int64_t>(0)), A.nrow - 1); // in range by construction
                    wh[u] = ph[q];
                    wl[u] = pl[q];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                df_acc<MODE, K>(x + rr[u] * XW, wh[u], wl[u], acc, cc);
        }
    }
    if (valid) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if constexpr (MODE == 0)
                static_cast<float *>(yv)[row * K + k] = acc[k];
            else
                static_cast<double *>(yv)[row * K + k] = static_cast<double>(acc[k]) + static_cast<double>(cc[k]);
        }
    }
}

template<int MODE, int K>
bool dx_launch_k(const pyci_gpu_csr *csr, const void *x, void *y, cudaStream_t st) {
    DxArgs A;
    A.nrow = csr->nrow;
    A.n = csr->dx_n;
    A.m = csr->dx_m;
    A.ldk = csr->dx_ldk;
    A.binom = csr->dx_binom;
    A.v = csr->dx_v;
    A.diag = csr->diag;
    static const size_t limit = [&] {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, docx_spmm_kernel<MODE, K>);
        const size_t lim = csr->ctx->smem_optin > fa.sharedSizeBytes ? csr->ctx->smem_optin - fa.sharedSizeBytes : 0;
        cudaFuncSetAttribute(docx_spmm_kernel<MODE, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
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
    docx_spmm_kernel<MODE, K><<<static_cast<unsigned>(blocks), 32 * warps, smem, st>>>(
        A, static_cast<const float *>(x), y);
    note_launch();
    return true;
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
