// Batched eigensolve of many independent CI operators of uneven size.
//
// No counterpart in the reference, which solves one operator at a time
// (SparseOp::solve_ci, pyci/src/sparseop.cpp:114-146).  All problems advance
// together through the block-Davidson iteration of davidson.cu, on vectors
// concatenated over problems (problem p owns rows [row0_p, row0_p + N_p) of
// every basis vector):
//   * one SpMM launch per iteration multiplies every active problem's new
//     block (a block-diagonal product; each row group looks its problem up in
//     a row-offset table), replayed from a CUDA graph with fixed buffers;
//   * Gram products and linear combinations are segmented by problem and
//     visit only the rows of the problems they concern;
//   * each problem has its own subspace size: its new block holds only the
//     corrections of its unconverged roots that survive orthogonalisation,
//     written at its own next slots, and it restarts on its own when its
//     next block would not fit;
//   * each problem's Rayleigh-Ritz, convergence test and restart are its own;
//     converged problems leave the active set.
// Mixed mode: FP32 values/vectors; at the end every problem's Ritz block is
// rebuilt in FP64 and Rayleigh-Ritz'd against the FP64 (high + low) operator.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <thread>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include <type_traits>

#include "dense.h"
#include "internal.h"

namespace pyci_gpu {

struct BatchOp {
    const int64_t *rowptr;
    const int32_t *cols;
    const double *vals;
    const float *hi, *lo;
    int64_t row0, nrow;
};

// Rows of a subset of the problems, numbered densely: subset member k is
// problem aprob[k] and owns dense rows [arow0[k], arow0[k + 1]); *count
// members.  Every pointer is device memory, so a captured graph sees updates.
struct RowSet {
    const int64_t *arow0;
    const int *aprob;
    const int *count;
};

// Last k in [0, n) with start[k] <= r.
__device__ __forceinline__ int find_segment(const int64_t *start, int n, int64_t r) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= r)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Dense row c of the subset -> problem and global row.
__device__ __forceinline__ void rowset_row(const RowSet &rs, int nseg, const int64_t *row0, int64_t c, int &prob,
                                           int64_t &r) {
    const int k = find_segment(rs.arow0, nseg, c);
    prob = rs.aprob[k];
    r = row0[prob] + (c - rs.arow0[k]);
}

// Calls f(prob, r) for every row r of the subset's problems (grid-stride).
template<typename F>
__device__ __forceinline__ void for_rows(const RowSet &rs, const int64_t *row0, F &&f) {
    const int nseg = *rs.count;
    const int64_t total = rs.arow0[nseg];
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int prob;
        int64_t r;
        rowset_row(rs, nseg, row0, c, prob, r);
        f(prob, r);
    }
}

// Y[r][0..K) = sum_e A_p[r][e] X[row0_p + col_e][0..K) for every row r of the
// subset's problems; other rows are left untouched.
// VK: 0 = FP64 values, 1 = FP32 high part, 2 = FP64 from high + low.
template<int VK, int K, int LANES, typename XT>
__global__ void __launch_bounds__(256) batch_spmm_kernel(const BatchOp *__restrict__ ops, RowSet rs,
                                                         const XT *__restrict__ x, XT *__restrict__ y) {
    typedef typename std::conditional<VK == 1, float, double>::type acc_t;
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    const int nseg = *rs.count;
    const int64_t total = rs.arow0[nseg];
    for (int64_t c = group; c < total; c += ngroups) {
        const int k = find_segment(rs.arow0, nseg, c);
        const BatchOp op = ops[rs.aprob[k]];
        const int64_t lr = c - rs.arow0[k];
        const int64_t r = op.row0 + lr;
        const int64_t start = op.rowptr[lr], end = op.rowptr[lr + 1];
        const XT *xb = x + op.row0 * K;
        acc_t acc[K];
#pragma unroll
        for (int j = 0; j < K; ++j)
            acc[j] = 0;
        for (int64_t e = start + lane; e < end; e += LANES) {
            const int64_t col = __ldcs(op.cols + e);
            acc_t v;
            if (VK == 0)
                v = static_cast<acc_t>(__ldcs(op.vals + e));
            else if (VK == 1)
                v = static_cast<acc_t>(__ldcs(op.hi + e));
            else
                v = static_cast<acc_t>(static_cast<double>(__ldcs(op.hi + e)) + static_cast<double>(__ldcs(op.lo + e)));
            const XT *xr = xb + col * K;
            if constexpr (K == 4 && sizeof(XT) == 4) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(xr));
                acc[0] += v * q.x;
                acc[1] += v * q.y;
                acc[2] += v * q.z;
                acc[3] += v * q.w;
            } else {
#pragma unroll
                for (int j = 0; j < K; ++j)
                    acc[j] += v * static_cast<acc_t>(__ldg(xr + j));
            }
        }
#pragma unroll
        for (int j = 0; j < K; ++j) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1)
                acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o, LANES);
        }
        if (lane < K) {
            acc_t out = acc[0];
#pragma unroll
            for (int j = 1; j < K; ++j)
                if (lane == j)
                    out = acc[j];
            y[r * K + lane] = static_cast<XT>(out);
        }
    }
}

// One SpMM tile: rows [lr0, lr1) of problem prob, `lanes` lanes per row.
struct BatchTile {
    int64_t lr0, lr1;
    int prob, lanes;
};

// Rows [lr0, lr1) of one problem at LANES lanes per row, by one block.
template<int VK, int K, int LANES, typename XT>
__device__ __forceinline__ void tile_rows(const BatchOp &op, int64_t lr0, int64_t lr1, const XT *__restrict__ x,
                                          XT *__restrict__ y) {
    typedef typename std::conditional<VK == 1, float, double>::type acc_t;
    const int lane = threadIdx.x % LANES;
    const int group = threadIdx.x / LANES, ngroups = blockDim.x / LANES;
    const XT *xb = x + op.row0 * K;
    for (int64_t lr = lr0 + group; lr < lr1; lr += ngroups) {
        const int64_t start = op.rowptr[lr], end = op.rowptr[lr + 1];
        acc_t acc[K];
#pragma unroll
        for (int j = 0; j < K; ++j)
            acc[j] = 0;
        for (int64_t e = start + lane; e < end; e += LANES) {
            const int64_t col = __ldcs(op.cols + e);
            acc_t v;
            if (VK == 0)
                v = static_cast<acc_t>(__ldcs(op.vals + e));
            else if (VK == 1)
                v = static_cast<acc_t>(__ldcs(op.hi + e));
            else
                v = static_cast<acc_t>(static_cast<double>(__ldcs(op.hi + e)) + static_cast<double>(__ldcs(op.lo + e)));
            const XT *xr = xb + col * K;
            if constexpr (K == 4 && sizeof(XT) == 4) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(xr));
                acc[0] += v * q.x;
                acc[1] += v * q.y;
                acc[2] += v * q.z;
                acc[3] += v * q.w;
            } else {
#pragma unroll
                for (int j = 0; j < K; ++j)
                    acc[j] += v * static_cast<acc_t>(__ldg(xr + j));
            }
        }
#pragma unroll
        for (int j = 0; j < K; ++j) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1)
                acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o, LANES);
        }
        if (lane < K) {
            acc_t out = acc[0];
#pragma unroll
            for (int j = 1; j < K; ++j)
                if (lane == j)
                    out = acc[j];
            y[(op.row0 + lr) * K + lane] = static_cast<XT>(out);
        }
    }
}

// The block-diagonal product of every active problem in one persistent
// launch: a grid of (SMs x resident blocks) walks the tile list (tile t by
// block t mod grid), each tile at its problem's tuned lanes per row.  Tiles
// and their count live in device memory, so a captured graph replays the
// launch with the current active set.
template<int VK, int K, typename XT>
__global__ void __launch_bounds__(256) batch_tile_spmm_kernel(const BatchOp *__restrict__ ops,
                                                              const BatchTile *__restrict__ tiles,
                                                              const int *__restrict__ ntiles,
                                                              const XT *__restrict__ x, XT *__restrict__ y) {
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const BatchTile T = tiles[t];
        const BatchOp op = ops[T.prob];
        if (T.lanes == 8)
            tile_rows<VK, K, 8>(op, T.lr0, T.lr1, x, y);
        else if (T.lanes == 16)
            tile_rows<VK, K, 16>(op, T.lr0, T.lr1, x, y);
        else
            tile_rows<VK, K, 32>(op, T.lr0, T.lr1, x, y);
    }
}

// Block-diagonal FP64-accurate product in FP32 arithmetic for the final
// Rayleigh-Ritz step: y[r][0..4) = (hi + lo) x over problem rows, x split as
// xs[r] = (4 high parts, 4 low parts); exact products via FMA and
// double-float (TwoSum) sums, as the single-operator double-float SpMM.
__device__ __forceinline__ void df_acc(float &s, float &c, float p) {
    const float u = __fadd_rn(s, p);
    const float z = __fadd_rn(u, -s);
    const float d = __fadd_rn(__fadd_rn(s, -__fadd_rn(u, -z)), __fadd_rn(p, -z));
    s = u;
    c = __fadd_rn(c, d);
}

template<int LANES>
__global__ void __launch_bounds__(256) batch_spmm_df_kernel(const BatchOp *__restrict__ ops, RowSet rs,
                                                            const float *__restrict__ xs, double *__restrict__ y) {
    constexpr int K = 4;
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    const int nseg = *rs.count;
    const int64_t total = rs.arow0[nseg];
    for (int64_t c0 = group; c0 < total; c0 += ngroups) {
        const int kk = find_segment(rs.arow0, nseg, c0);
        const BatchOp op = ops[rs.aprob[kk]];
        const int64_t lr = c0 - rs.arow0[kk];
        const int64_t r = op.row0 + lr;
        const int64_t start = op.rowptr[lr], end = op.rowptr[lr + 1];
        const float *xb = xs + op.row0 * (2 * K);
        float s[K], c[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            s[k] = c[k] = 0.0f;
        // One term: (vh + vl) (xh + xl) of column col into the double-float sums.
        auto term = [&](int64_t col, float vh, float vl) {
            const float4 a = __ldg(reinterpret_cast<const float4 *>(xb + col * (2 * K)));
            const float4 b = __ldg(reinterpret_cast<const float4 *>(xb + col * (2 * K)) + 1);
            const float xh[K] = {a.x, a.y, a.z, a.w}, xl[K] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float p = __fmul_rn(vh, xh[k]);
                const float err = fmaf(vh, xh[k], -p);
                const float t = fmaf(vh, xl[k], fmaf(vl, xh[k], err));
                df_acc(s[k], c[k], p);
                c[k] = __fadd_rn(c[k], t);
            }
        };
        // Head up to a 4-aligned index, body of 4 entries per lane per step
        // (16-byte loads of columns and both value halves), tail.
        const int64_t a0 = min(end, (start + 3) & ~static_cast<int64_t>(3));
        const int64_t a1 = max(a0, end & ~static_cast<int64_t>(3));
        if (start + lane < a0)
            term(__ldcs(op.cols + start + lane), __ldcs(op.hi + start + lane), __ldcs(op.lo + start + lane));
        for (int64_t e = a0 + 4 * lane; e < a1; e += 4 * LANES) {
            const int4 c4 = __ldcs(reinterpret_cast<const int4 *>(op.cols + e));
            const float4 h4 = __ldcs(reinterpret_cast<const float4 *>(op.hi + e));
            const float4 l4 = __ldcs(reinterpret_cast<const float4 *>(op.lo + e));
            term(c4.x, h4.x, l4.x);
            term(c4.y, h4.y, l4.y);
            term(c4.z, h4.z, l4.z);
            term(c4.w, h4.w, l4.w);
        }
        if (a1 + lane < end)
            term(__ldcs(op.cols + a1 + lane), __ldcs(op.hi + a1 + lane), __ldcs(op.lo + a1 + lane));
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1) {
                const float s2 = __shfl_xor_sync(0xffffffffu, s[k], o, LANES);
                const float c2 = __shfl_xor_sync(0xffffffffu, c[k], o, LANES);
                df_acc(s[k], c[k], s2);
                c[k] = __fadd_rn(c[k], c2);
            }
        }
        if (lane < K) {
            double out = static_cast<double>(s[0]) + static_cast<double>(c[0]);
#pragma unroll
            for (int k = 1; k < K; ++k)
                if (lane == k)
                    out = static_cast<double>(s[k]) + static_cast<double>(c[k]);
            y[r * K + lane] = out;
        }
    }
}

// xs[r] = (fl32(X[j][r]), j < 4; fl32(X[j][r] - fl32(X[j][r])), j < 4) for the subset's rows.
__global__ void batch_pack_split_kernel(const double *__restrict__ X, int64_t N, RowSet rs,
                                        const int64_t *__restrict__ row0, float *__restrict__ xs) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        (void)prob;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double v = X[j * N + r];
            const float h = static_cast<float>(v);
            xs[r * 8 + j] = h;
            xs[r * 8 + 4 + j] = static_cast<float>(v - static_cast<double>(h));
        }
    });
}

// Xi[r][j] = V[base[prob] + j][r], j < K, for the subset's rows.
template<typename T, int K>
__global__ void batch_pack_kernel(const T *__restrict__ V, int64_t N, const int *__restrict__ base, RowSet rs,
                                  const int64_t *__restrict__ row0, T *__restrict__ Xi) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        const int64_t b0 = base[prob];
#pragma unroll
        for (int j = 0; j < K; ++j)
            Xi[r * K + j] = V[(b0 + j) * N + r];
    });
}

// W[base[prob] + j][r] = Yi[r][j] and, when Wnew is given, Wnew[j][r] too.
template<typename T, int K>
__global__ void batch_unpack_kernel(const T *__restrict__ Yi, int64_t N, const int *__restrict__ base, RowSet rs,
                                    const int64_t *__restrict__ row0, T *__restrict__ W, T *__restrict__ Wnew) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        const int64_t b0 = base[prob];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const T v = Yi[r * K + j];
            W[(b0 + j) * N + r] = v;
            if (Wnew)
                Wnew[j * N + r] = v;
        }
    });
}

// Segmented Gram product.  Tile t covers rows [tile_lo[t], tile_hi[t]) of
// problem tile_prob[t]; partial[t][i * q + j] = sum over those rows of
// A[i][r] * B[j][r] for i < alen[prob] (zero beyond, and A is not read there).
constexpr int kSegMaxP = 64;
constexpr int kSegMaxQ = 8;

template<typename T, int PI, int QC>
__global__ void __launch_bounds__(256) seg_gram_kernel(const T *__restrict__ A, int p, const T *__restrict__ B, int q,
                                                       int64_t N, const int64_t *__restrict__ tile_lo,
                                                       const int64_t *__restrict__ tile_hi,
                                                       const int *__restrict__ tile_prob, const int *__restrict__ alen,
                                                       int ntiles, double *__restrict__ partial) {
    // Block (x, y): tiles x, x + gridDim.x, ...; A rows i in [y * PI, y * PI + PI).
    const int i0 = blockIdx.y * PI;
    const int pq = p * q;
    __shared__ double red[8][PI * QC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int plim = alen ? min(p, alen[tile_prob[t]]) : p;
        const int ni = max(0, min(PI, plim - i0));
        T acc[PI][QC];
#pragma unroll
        for (int ii = 0; ii < PI; ++ii)
#pragma unroll
            for (int j = 0; j < QC; ++j)
                acc[ii][j] = T(0);
        if (ni > 0) {
            for (int64_t r = tile_lo[t] + threadIdx.x; r < tile_hi[t]; r += blockDim.x) {
                T bv[QC];
#pragma unroll
                for (int j = 0; j < QC; ++j)
                    bv[j] = (j < q) ? B[j * N + r] : T(0);
#pragma unroll
                for (int ii = 0; ii < PI; ++ii)
                    if (ii < ni) {
                        const T a = A[(i0 + ii) * N + r];
#pragma unroll
                        for (int j = 0; j < QC; ++j)
                            acc[ii][j] += a * bv[j];
                    }
            }
        }
#pragma unroll
        for (int ii = 0; ii < PI; ++ii)
#pragma unroll
            for (int j = 0; j < QC; ++j) {
                double v = static_cast<double>(acc[ii][j]);
                for (int o = 16; o > 0; o >>= 1)
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0)
                    red[warp][ii * QC + j] = v;
            }
        __syncthreads();
        const int nrow_out = min(PI, p - i0);
        for (int idx = threadIdx.x; idx < nrow_out * q; idx += blockDim.x) {
            const int ii = idx / q, j = idx % q;
            double v = 0.0;
            for (int w = 0; w < nwarps; ++w)
                v += red[w][ii * QC + j];
            partial[static_cast<int64_t>(t) * pq + (i0 + ii) * q + j] = v;
        }
        __syncthreads();
    }
}

// out[prob][idx] = sum over the problem's tiles of partial[t][idx].
__global__ void seg_reduce_kernel(const double *__restrict__ partial, int pq, const int *__restrict__ tile_begin,
                                  double *__restrict__ out) {
    const int prob = blockIdx.x / pq, idx = blockIdx.x % pq;
    double s = 0.0;
    for (int t = tile_begin[prob] + threadIdx.x; t < tile_begin[prob + 1]; t += blockDim.x)
        s += partial[static_cast<int64_t>(t) * pq + idx];
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (blockDim.x >> 5); ++w)
            t += red[w];
        out[blockIdx.x] = t;
    }
}

// out[obase[prob] + j][r] = beta * (same) + sum_{i < vlen[prob]} Y[prob][i * q + j] * V[i][r]
// over the rows of the active tiles whose problem has mask[prob] != 0 (mask,
// obase, vlen optional: all, 0 and p).  A block takes whole tiles, each
// inside one problem, and stages that problem's coefficients in shared
// memory once per tile.
template<typename TV, typename TO, typename ACC>
__global__ void __launch_bounds__(256) seg_combine_kernel(const TV *__restrict__ V, int p, int64_t N,
                                                          const double *__restrict__ Y, int q, double beta,
                                                          const int64_t *__restrict__ tile_lo,
                                                          const int64_t *__restrict__ tile_hi,
                                                          const int *__restrict__ tile_prob, int ntiles,
                                                          const int *__restrict__ mask, const int *__restrict__ vlen,
                                                          const int *__restrict__ obase, TO *__restrict__ out) {
    __shared__ ACC sy[kSegMaxP * kSegMaxQ];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int prob = tile_prob[t];
        if (mask && !mask[prob])
            continue;
        const int plim = vlen ? min(p, vlen[prob]) : p;
        const double *Yp = Y + static_cast<int64_t>(prob) * p * q;
        __syncthreads(); // the previous tile's coefficients are no longer read
        for (int e = threadIdx.x; e < plim * q; e += blockDim.x)
            sy[e] = static_cast<ACC>(Yp[e]);
        __syncthreads();
        const int64_t b0 = obase ? obase[prob] : 0;
        for (int64_t r = tile_lo[t] + threadIdx.x; r < tile_hi[t]; r += blockDim.x) {
            ACC acc[kSegMaxQ];
#pragma unroll
            for (int j = 0; j < kSegMaxQ; ++j)
                acc[j] = 0;
            for (int i = 0; i < plim; ++i) {
                const ACC v = static_cast<ACC>(V[i * N + r]);
#pragma unroll
                for (int j = 0; j < kSegMaxQ; ++j)
                    if (j < q)
                        acc[j] += sy[i * q + j] * v;
            }
#pragma unroll
            for (int j = 0; j < kSegMaxQ; ++j)
                if (j < q) {
                    TO *o = out + (b0 + j) * N + r;
                    *o = (beta == 0.0) ? static_cast<TO>(acc[j]) : static_cast<TO>(static_cast<ACC>(*o) + acc[j]);
                }
        }
    }
}

// dst[j][r] = src[j][r], j < ncols, for the subset's rows.
template<typename T>
__global__ void seg_copy_kernel(const T *__restrict__ src, int ncols, int64_t N, RowSet rs,
                                const int64_t *__restrict__ row0, T *__restrict__ dst) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        (void)prob;
        for (int j = 0; j < ncols; ++j)
            dst[j * N + r] = src[j * N + r];
    });
}

// R[j][r] = AX[j][r] - theta[prob(r)][j] X[j][r].  FP32 vectors: theta
// split into FP32 high + low parts applied with two FMAs (no FP64
// arithmetic, which is scarce on this GPU).
template<typename T>
__global__ void seg_residual_kernel(const T *__restrict__ AX, const T *__restrict__ X, const double *__restrict__ theta,
                                    int q, int64_t N, RowSet rs, const int64_t *__restrict__ row0, T *__restrict__ R) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        for (int j = 0; j < q; ++j) {
            const double t = theta[prob * q + j];
            if constexpr (sizeof(T) == 4) {
                const float th = static_cast<float>(t), tl = static_cast<float>(t - static_cast<double>(th));
                const float x = X[j * N + r];
                R[j * N + r] = fmaf(-tl, x, fmaf(-th, x, AX[j * N + r]));
            } else {
                R[j * N + r] = AX[j * N + r] - t * X[j * N + r];
            }
        }
    });
}

// out[c][r] = R[j][r] / (theta[prob][j] - D[r]) for the root j = sel[prob][c]
// (c < b), 0 where sel is -1; theta has nt entries per problem.
template<typename T>
__global__ void seg_precondition_kernel(const T *__restrict__ R, const double *__restrict__ theta, int nt,
                                        const int *__restrict__ sel, const double *__restrict__ diag, int b,
                                        int64_t N, RowSet rs, const int64_t *__restrict__ row0, T *__restrict__ out) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        const double d = diag[r];
        for (int c = 0; c < b; ++c) {
            const int j = sel[prob * b + c];
            T v = T(0);
            if (j >= 0) {
                double den = theta[prob * nt + j] - d;
                if (fabs(den) < 1e-8)
                    den = (den < 0.0) ? -1e-8 : 1e-8;
                if constexpr (sizeof(T) == 4)
                    v = R[j * N + r] / static_cast<float>(den); // FP32 quotient
                else
                    v = R[j * N + r] / den;
            }
            out[c * N + r] = v;
        }
    });
}

template<typename TI, typename TO>
__global__ void batch_convert_kernel(const TI *__restrict__ in, TO *__restrict__ out, int64_t n) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[r] = static_cast<TO>(in[r]);
}

// Start block: T[j][r] = [local row == pick[prob][j]] + amp_prob * noise(local row, j)
// for j < b (pick -1: no unit part); amp_prob = kGuessNoise / sqrt(N_prob).
template<typename T>
__global__ void seg_guess_kernel(T *__restrict__ Tb, int b, int64_t N, RowSet rs, const int64_t *__restrict__ row0,
                                 const int64_t *__restrict__ pick) {
    for_rows(rs, row0, [&](int prob, int64_t r) {
        const int64_t lr = r - row0[prob];
        const double amp = kGuessNoise / sqrt(static_cast<double>(row0[prob + 1] - row0[prob]));
        for (int j = 0; j < b; ++j)
            Tb[j * N + r] = static_cast<T>((pick[prob * b + j] == lr ? 1.0 : 0.0) +
                                           amp * guess_noise(static_cast<uint64_t>(lr), static_cast<uint64_t>(j)));
    });
}

} // namespace pyci_gpu

using namespace pyci_gpu;

namespace {

// Tile-class tuning results shared by batches of the same shape in this
// process: key = (value kind, class rows, class stored entries) -> lanes.
std::mutex g_class_tune_mutex;
std::map<std::tuple<int, int64_t, int64_t>, int> g_class_tune;

// f(i) for i in [0, n) on up to 16 host threads (dynamic scheduling): the
// per-problem Rayleigh-Ritz eigenproblems of one iteration are independent.
template<typename F>
void host_parallel_for(int n, F f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = std::min(n, static_cast<int>(std::min(16u, hw)));
    if (nt <= 1 || n < 4) {
        for (int i = 0; i < n; ++i)
            f(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1))
                f(i);
        });
    for (auto &th : pool)
        th.join();
}

// A RowSet in device memory plus its host mirror.
struct DevRowSet {
    int64_t *arow0 = nullptr;
    int *aprob = nullptr;
    int *count = nullptr;
    int64_t total = 0;
    std::vector<int> members;
    RowSet view() const { return RowSet{arow0, aprob, count}; }
};

// Host-side state of the batched solver.
template<typename T>
class Batch {
public:
    // nroot roots wanted per problem; nroot + 1 Ritz pairs are tracked (one
    // guard pair, as in the single-operator solver), corrections for at most
    // nroot of them per iteration.
    Batch(pyci_gpu_ctx *ctx, std::vector<pyci_gpu_csr *> ops, int nroot, int mmax, bool mixed)
        : ctx_(ctx), st_(ctx->stream), ops_(std::move(ops)), P_(static_cast<int>(ops_.size())), b_(nroot),
          nt_(nroot + 1), mmax_(mmax), mixed_(mixed) {}

    ~Batch() {
        if (graph_exec_)
            cudaGraphExecDestroy(graph_exec_);
        for (void *p : allocs_)
            cudaFreeAsync(p, st_);
        cudaStreamSynchronize(st_);
    }

    int run(int64_t maxiter, double tol, const double *ecore, double *evals, double *const *evecs,
            int64_t *iterations, pyci_gpu_solve_stats *stats);

private:
    template<typename U>
    int alloc(U **p, int64_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, sizeof(U) * std::max<int64_t>(n, 1), st_);
        if (e != cudaSuccess)
            return cuda_status(e, "cudaMallocAsync (batched solver)");
        allocs_.push_back(q);
        *p = static_cast<U *>(q);
        return PYCI_GPU_OK;
    }
    unsigned grid(int64_t n) const {
        return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx_->num_sms * 8)));
    }

    int alloc_rowset(DevRowSet &rs) {
        int rc;
        if ((rc = alloc(&rs.arow0, P_ + 1)) || (rc = alloc(&rs.aprob, P_)) || (rc = alloc(&rs.count, 1)))
            return rc;
        return PYCI_GPU_OK;
    }

    // rs = the problems with mask[p] != 0.
    int set_rowset(DevRowSet &rs, const std::vector<int> &mask) {
        std::vector<int64_t> a(1, 0);
        rs.members.clear();
        for (int p = 0; p < P_; ++p)
            if (mask[p]) {
                rs.members.push_back(p);
                a.push_back(a.back() + ops_[p]->nrow);
            }
        const int n = static_cast<int>(rs.members.size());
        rs.total = a.back();
        PYCI_CUDA_TRY(cudaMemcpyAsync(rs.arow0, a.data(), sizeof(int64_t) * a.size(), cudaMemcpyHostToDevice, st_));
        if (n)
            PYCI_CUDA_TRY(cudaMemcpyAsync(rs.aprob, rs.members.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st_));
        PYCI_CUDA_TRY(cudaMemcpyAsync(rs.count, &n, sizeof(int), cudaMemcpyHostToDevice, st_));
        PYCI_CUDA_TRY(cudaStreamSynchronize(st_)); // host sources are stack/heap temporaries
        return PYCI_GPU_OK;
    }

    // Active set (rows and Gram tiles) = the problems with mask[p] != 0.
    int set_active(const std::vector<int> &mask) {
        int rc;
        tiles_dirty_ = true;
        if ((rc = set_rowset(act_, mask)))
            return rc;
        for (int c = 0; c < kClasses; ++c) {
            std::vector<int> mc(P_, 0), m32(P_, 0);
            for (int p = 0; p < P_; ++p) {
                mc[p] = mask[p] && cls_of_[p] == c;
                m32[p] = mc[p] && !imp_[p];
            }
            if ((rc = set_rowset(cls_[c], mc)) || (rc = set_rowset(cls32_[c], m32)))
                return rc;
        }
        std::vector<int64_t> tlo, thi;
        std::vector<int> tprob, tbeg(P_ + 1, 0);
        const int64_t tile = 8192;
        for (int p = 0; p < P_; ++p) {
            tbeg[p] = static_cast<int>(tlo.size());
            if (!mask[p])
                continue;
            for (int64_t r = row0_[p]; r < row0_[p + 1]; r += tile) {
                tlo.push_back(r);
                thi.push_back(std::min(r + tile, row0_[p + 1]));
                tprob.push_back(p);
            }
        }
        tbeg[P_] = static_cast<int>(tlo.size());
        ntiles_ = static_cast<int>(tlo.size());
        if (ntiles_) {
            PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_lo_, tlo.data(), sizeof(int64_t) * ntiles_, cudaMemcpyHostToDevice, st_));
            PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_hi_, thi.data(), sizeof(int64_t) * ntiles_, cudaMemcpyHostToDevice, st_));
            PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_prob_, tprob.data(), sizeof(int) * ntiles_, cudaMemcpyHostToDevice, st_));
        }
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_begin_, tbeg.data(), sizeof(int) * (P_ + 1), cudaMemcpyHostToDevice, st_));
        PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
        return PYCI_GPU_OK;
    }

    // Per-problem small integer table (e.g. subspace sizes) to the device,
    // asynchronously (pinned staging).
    int upload_ints(int *dst, const std::vector<int> &v) { return ctx_->ring->upload(dst, v.data(), sizeof(int) * v.size(), st_); }

    // G[prob] (p x q, row-major) = A^T B over the active problems' rows; A
    // has p vectors (only the first alen[prob] are read when alen is given),
    // B has q.  Inactive problems get zeros.
    template<typename U>
    int gram(const U *A, int p, const U *B, int q, std::vector<double> &G, const int *alen = nullptr) {
        G.assign(static_cast<size_t>(P_) * p * q, 0.0);
        if (ntiles_ == 0)
            return PYCI_GPU_OK;
        for (int i0 = 0; i0 < p; i0 += kSegMaxP) {
            const int pp = std::min(kSegMaxP, p - i0);
            for (int j0 = 0; j0 < q; j0 += kSegMaxQ) {
                const int qq = std::min(kSegMaxQ, q - j0);
                const int pi = (qq <= 4) ? 8 : 4;
                const unsigned gy = static_cast<unsigned>((pp + pi - 1) / pi);
                const unsigned nb = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(ntiles_, ctx_->num_sms * 8 / gy)));
                const U *Ai = A + static_cast<int64_t>(i0) * N_;
                const U *Bj = B + static_cast<int64_t>(j0) * N_;
                const int *al = (i0 == 0) ? alen : nullptr;
                const dim3 g(nb, gy);
                if (qq <= 1)
                    seg_gram_kernel<U, 8, 1><<<g, 256, 0, st_>>>(Ai, pp, Bj, qq, N_, d_tile_lo_, d_tile_hi_,
                                                                 d_tile_prob_, al, ntiles_, d_partial_);
                else if (qq <= 2)
                    seg_gram_kernel<U, 8, 2><<<g, 256, 0, st_>>>(Ai, pp, Bj, qq, N_, d_tile_lo_, d_tile_hi_,
                                                                 d_tile_prob_, al, ntiles_, d_partial_);
                else if (qq <= 4)
                    seg_gram_kernel<U, 8, 4><<<g, 256, 0, st_>>>(Ai, pp, Bj, qq, N_, d_tile_lo_, d_tile_hi_,
                                                                 d_tile_prob_, al, ntiles_, d_partial_);
                else
                    seg_gram_kernel<U, 4, 8><<<g, 256, 0, st_>>>(Ai, pp, Bj, qq, N_, d_tile_lo_, d_tile_hi_,
                                                                 d_tile_prob_, al, ntiles_, d_partial_);
                ::pyci_gpu::note_launch();
                seg_reduce_kernel<<<P_ * pp * qq, 128, 0, st_>>>(d_partial_, pp * qq, d_tile_begin_, d_small_),
                    ::pyci_gpu::note_launch();
                std::vector<double> tmp(static_cast<size_t>(P_) * pp * qq);
                PYCI_CUDA_TRY(cudaMemcpyAsync(tmp.data(), d_small_, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, st_));
                PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
                for (int pr = 0; pr < P_; ++pr)
                    for (int i = 0; i < pp; ++i)
                        for (int j = 0; j < qq; ++j)
                            G[(static_cast<size_t>(pr) * p + i0 + i) * q + j0 + j] =
                                tmp[(static_cast<size_t>(pr) * pp + i) * qq + j];
            }
        }
        return PYCI_GPU_OK;
    }

    // out[obase + j] = beta out[obase + j] + sum_{i < vlen} Y[prob][i][j] V[i]
    // (Y host: [P][p][q]) over the rows of the active problems, or of those
    // with mask[prob] != 0 (a device array) when mask is given.
    template<typename TV, typename TO, typename ACC>
    int combine(const TV *V, int p, const std::vector<double> &Y, int q, double beta, TO *out,
                const int *vlen = nullptr, const int *obase = nullptr, const int *mask = nullptr) {
        if (p > kSegMaxP) {
            set_error("batched combine: p = %d beyond limits", p);
            return PYCI_GPU_EUNSUPPORTED;
        }
        if (ntiles_ == 0)
            return PYCI_GPU_OK;
        // Output columns in chunks of kSegMaxQ.
        for (int j0 = 0; j0 < q; j0 += kSegMaxQ) {
            const int qq = std::min(kSegMaxQ, q - j0);
            const double *coef = Y.data();
            std::vector<double> sub;
            if (qq != q) {
                sub.resize(static_cast<size_t>(P_) * p * qq);
                for (int pr = 0; pr < P_; ++pr)
                    for (int i = 0; i < p; ++i)
                        for (int j = 0; j < qq; ++j)
                            sub[(static_cast<size_t>(pr) * p + i) * qq + j] = Y[(static_cast<size_t>(pr) * p + i) * q + j0 + j];
                coef = sub.data();
            }
            int rc = ctx_->ring->upload(d_coef_, coef, sizeof(double) * P_ * p * qq, st_);
            if (rc)
                return rc;
            const unsigned nb = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(ntiles_, ctx_->num_sms * 8)));
            seg_combine_kernel<TV, TO, ACC><<<nb, 256, 0, st_>>>(V, p, N_, d_coef_, qq, beta, d_tile_lo_, d_tile_hi_,
                                                                 d_tile_prob_, ntiles_, mask, vlen, obase,
                                                                 out + static_cast<int64_t>(j0) * N_),
                ::pyci_gpu::note_launch();
        }
        return PYCI_GPU_OK;
    }

    // W[m_p + j] = H V[m_p + j] (j < b) for every active problem, and the
    // same products into Wnew_[j]; one graph replay (pack, one SpMM per tile
    // class, unpack).
    int apply_block(int prec, T *V, T *W);

    // Block-diagonal product Xi_ -> Yi_ over the rows of rs at `lanes` lanes
    // per row.
    void spmm_class(int prec, int lanes, const DevRowSet &rs) {
        const int64_t rows = std::max<int64_t>(rs.total, 1);
        const unsigned blocks = static_cast<unsigned>(
            std::max<int64_t>(1, std::min<int64_t>(ctx_->num_sms * 32, (rows * lanes + 255) / 256)));
        const RowSet v = rs.view();
        if (prec == PYCI_PREC_FP32) {
            if (lanes == 8)
                batch_spmm_kernel<1, 4, 8, T><<<blocks, 256, 0, st_>>>(d_ops_, v, Xi_, Yi_);
            else if (lanes == 16)
                batch_spmm_kernel<1, 4, 16, T><<<blocks, 256, 0, st_>>>(d_ops_, v, Xi_, Yi_);
            else
                batch_spmm_kernel<1, 4, 32, T><<<blocks, 256, 0, st_>>>(d_ops_, v, Xi_, Yi_);
        } else if (prec == PYCI_PREC_FP64_SPLIT) {
            batch_spmm_kernel<2, 4, 32, T><<<blocks, 256, 0, st_>>>(d_ops_, v, Xi_, Yi_);
        } else {
            batch_spmm_kernel<0, 4, 32, T><<<blocks, 256, 0, st_>>>(d_ops_, v, Xi_, Yi_);
        }
    }

    // The CSR launches' row set of class c at precision prec.
    const DevRowSet &cls_for(int prec, int c) const { return prec == PYCI_PREC_FP32 ? cls32_[c] : cls_[c]; }

    // FP32 products of the active problems with an implicit form, one launch
    // each on their rows of Xi_ / Yi_ (K = 4, row stride 4); returns the
    // number of launches.
    int spmm_implicit(int prec) {
        int n = 0;
        if constexpr (std::is_same<T, float>::value) {
            if (prec != PYCI_PREC_FP32)
                return 0;
            for (int p : act_.members)
                if (imp_[p] && implicit_launch(ops_[p], 0, 4, Xi_ + row0_[p] * 4, 4, Yi_ + row0_[p] * 4, 4, st_))
                    ++n;
        }
        return n;
    }

    // Tile list of the active problems (at FP32 without those with an
    // implicit form): row blocks of about target stored entries (a multiple
    // of the rows one block covers at once), at each problem's class lanes
    // per row; uploaded with its count.
    int build_tiles(int64_t target, int prec) {
        std::vector<BatchTile> t;
        tiles_prec_ = prec;
        for (int p : act_.members) {
            if (prec == PYCI_PREC_FP32 && imp_[p])
                continue;
            const pyci_gpu_csr *c = ops_[p];
            const int lanes = cls_lanes_[cls_of_[p]];
            const int64_t per = 256 / lanes;
            const double avg = c->nrow ? static_cast<double>(c->nnz) / c->nrow : 1.0;
            int64_t rows = std::max<int64_t>(per, static_cast<int64_t>(target / std::max(avg, 1.0)));
            rows = (rows + per - 1) / per * per;
            for (int64_t r = 0; r < c->nrow; r += rows)
                t.push_back(BatchTile{r, std::min(r + rows, c->nrow), p, lanes});
        }
        if (static_cast<int64_t>(t.size()) > tile_cap_) {
            set_error("batched SpMM: %zu tiles exceed the %lld allocated", t.size(), static_cast<long long>(tile_cap_));
            return PYCI_GPU_EUNSUPPORTED;
        }
        const int n = static_cast<int>(t.size());
        if (n)
            PYCI_CUDA_TRY(cudaMemcpyAsync(d_tiles_, t.data(), sizeof(BatchTile) * n, cudaMemcpyHostToDevice, st_));
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_ntiles_, &n, sizeof(int), cudaMemcpyHostToDevice, st_));
        PYCI_CUDA_TRY(cudaStreamSynchronize(st_)); // host sources are temporaries
        tiles_dirty_ = false;
        return PYCI_GPU_OK;
    }

    // The block-diagonal product Xi_ -> Yi_ of every active problem in one
    // persistent launch over the tile list.
    void spmm_tiles(int prec) {
        if (prec == PYCI_PREC_FP32)
            batch_tile_spmm_kernel<1, 4, T><<<tile_grid_, 256, 0, st_>>>(d_ops_, d_tiles_, d_ntiles_, Xi_, Yi_);
        else if (prec == PYCI_PREC_FP64_SPLIT)
            batch_tile_spmm_kernel<2, 4, T><<<tile_grid_, 256, 0, st_>>>(d_ops_, d_tiles_, d_ntiles_, Xi_, Yi_);
        else
            batch_tile_spmm_kernel<0, 4, T><<<tile_grid_, 256, 0, st_>>>(d_ops_, d_tiles_, d_ntiles_, Xi_, Yi_);
    }

    // Two Cholesky-QR passes of the b vectors in Tnew_ inside each active
    // problem's block: columns with use == 0 are left out, dependent ones are
    // dropped (use set to 0).  The kept orthonormal vectors of problem p are
    // written, compacted, to V[base_p], V[base_p + 1], ... (base = d_base_,
    // zero vectors after them up to b); knew[p] = how many.  tmp: b vectors.
    int cholqr_block(std::vector<int> &use, T *tmp, T *V, std::vector<int> &knew);

    pyci_gpu_ctx *ctx_;
    cudaStream_t st_;
    std::vector<pyci_gpu_csr *> ops_;
    int P_, b_, nt_, mmax_;
    bool mixed_;
    int64_t N_ = 0;
    int ntiles_ = 0;
    std::vector<void *> allocs_;
    std::vector<int64_t> row0_;
    DevRowSet act_, sel_;
    // SpMM tile classes: problems grouped by mean row length (nominal 8, 16,
    // 32 lanes per row); cls_[c] holds the active members of class c and
    // cls_lanes_[c] the lanes per row the autotuner chose for it.
    static constexpr int kClasses = 3;
    DevRowSet cls_[kClasses];
    // The FP32 products of problems with an implicit form (full FullCI or
    // DOCI spaces) run on that form, one launch per such active problem on
    // its rows of Xi_ / Yi_; cls32_[c] holds the active members of class c
    // without them, for the FP32 CSR launches.
    std::vector<char> imp_;
    DevRowSet cls32_[kClasses];
    std::vector<int> graph_members_;
    int graph_imp_launches_ = 0;
    bool imp_warm_ = false;
    int tiles_prec_ = -1;
    std::vector<int> cls_of_;
    int cls_lanes_[kClasses] = {8, 16, 32};
    bool cls_tuned_ = false;
    int64_t *d_row0_ = nullptr, *d_tile_lo_ = nullptr, *d_tile_hi_ = nullptr;
    int *d_tile_begin_ = nullptr, *d_tile_prob_ = nullptr, *d_sel_ = nullptr, *d_base_ = nullptr, *d_len_ = nullptr;
    int *d_zero_ = nullptr, *d_mask_ = nullptr;
    double *d_partial_ = nullptr, *d_small_ = nullptr, *d_coef_ = nullptr, *d_theta_ = nullptr, *d_diag_ = nullptr;
    BatchOp *d_ops_ = nullptr;
    T *Tnew_ = nullptr, *Wnew_ = nullptr, *Xi_ = nullptr, *Yi_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_prec_ = -1;
    const void *graph_v_ = nullptr;
    // Persistent SpMM tiles (batch_tile_spmm_kernel): the active problems'
    // row blocks of about tile_nnz_ stored entries each, at their class's
    // lanes per row; rebuilt when the active set changes.  tile_nnz_ = 0:
    // the tuner chose the per-class launches instead.
    BatchTile *d_tiles_ = nullptr;
    int *d_ntiles_ = nullptr;
    int64_t tile_cap_ = 0, tile_nnz_ = 1 << 18;
    bool tiles_dirty_ = true, tiles_tuned_ = false;
    unsigned tile_grid_ = 1;
    bool all_vals_ = true;
    int64_t matvecs_ = 0;
    double spmm_ms_ = 0.0;
};

template<typename T>
int Batch<T>::apply_block(int prec, T *V, T *W) {
    // Buffers and the row set live at fixed device addresses, so the graph
    // is captured once per precision and replayed every iteration.
    if (prec == PYCI_PREC_FP64 && !all_vals_)
        prec = PYCI_PREC_FP64_SPLIT;
    // Graphs that launch implicit-form products bake in the active set.
    bool any_imp = false;
    for (int p : act_.members)
        any_imp = any_imp || (prec == PYCI_PREC_FP32 && imp_[p]);
    if (!graph_exec_ || graph_prec_ != prec || graph_v_ != V || (any_imp && graph_members_ != act_.members)) {
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        const RowSet rs = act_.view();
        const unsigned gr = grid(N_);
        if (!cls_tuned_) {
            // Autotuner: time each class's product at 8, 16 and 32 lanes per
            // row (one warm-up + one timed launch each) and keep the fastest.
            batch_pack_kernel<T, 4><<<gr, 256, 0, st_>>>(V, N_, d_base_, rs, d_row0_, Xi_);
            cudaEvent_t ea, eb;
            cudaEventCreate(&ea);
            cudaEventCreate(&eb);
            for (int c = 0; c < kClasses; ++c) {
                const DevRowSet &rc_ = cls_for(prec, c);
                if (rc_.total == 0)
                    continue;
                int64_t cls_nnz = 0;
                for (int p : rc_.members)
                    cls_nnz += ops_[p]->nnz;
                const auto key = std::make_tuple(prec, rc_.total, cls_nnz);
                {
                    std::lock_guard<std::mutex> lock(g_class_tune_mutex);
                    auto it = g_class_tune.find(key);
                    if (it != g_class_tune.end()) {
                        cls_lanes_[c] = it->second;
                        continue;
                    }
                }
                float best = 1e30f;
                for (int lanes : {8, 16, 32}) {
                    for (int rep = 0; rep < 2; ++rep) {
                        if (rep == 1)
                            cudaEventRecord(ea, st_);
                        spmm_class(prec, lanes, rc_);
                        if (rep == 1)
                            cudaEventRecord(eb, st_);
                    }
                    PYCI_CUDA_TRY(cudaEventSynchronize(eb));
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ea, eb);
                    if (ms < best) {
                        best = ms;
                        cls_lanes_[c] = lanes;
                    }
                }
                std::lock_guard<std::mutex> lock(g_class_tune_mutex);
                g_class_tune[key] = cls_lanes_[c];
            }
            cudaEventDestroy(ea);
            cudaEventDestroy(eb);
            cls_tuned_ = true;
        }
        if (!tiles_tuned_) {
            // Form of the product: one grid-stride launch per tile class, or
            // the persistent launch over tile lists of ~64K, ~256K or ~1M
            // stored entries per tile (lanes per row as tuned above); the
            // fastest is kept (tile_nnz_ = 0: per-class launches).
            int64_t nnz_act = 0;
            for (int p : act_.members)
                if (!(prec == PYCI_PREC_FP32 && imp_[p]))
                    nnz_act += ops_[p]->nnz;
            const auto key = std::make_tuple(prec + 16, act_.total, nnz_act);
            bool cached = false;
            {
                std::lock_guard<std::mutex> lock(g_class_tune_mutex);
                auto it = g_class_tune.find(key);
                if (it != g_class_tune.end()) {
                    tile_nnz_ = it->second ? int64_t(1) << it->second : 0;
                    cached = true;
                }
            }
            if (!cached) {
                batch_pack_kernel<T, 4><<<gr, 256, 0, st_>>>(V, N_, d_base_, rs, d_row0_, Xi_);
                cudaEvent_t ea, eb;
                cudaEventCreate(&ea);
                cudaEventCreate(&eb);
                // Candidate 0: one grid-stride launch per tile class.
                for (int c = 0; c < kClasses; ++c)
                    spmm_class(prec, cls_lanes_[c], cls_for(prec, c));
                cudaEventRecord(ea, st_);
                for (int c = 0; c < kClasses; ++c)
                    spmm_class(prec, cls_lanes_[c], cls_for(prec, c));
                cudaEventRecord(eb, st_);
                PYCI_CUDA_TRY(cudaEventSynchronize(eb));
                float best = 1e30f;
                cudaEventElapsedTime(&best, ea, eb);
                int best_sh = 0;
                for (int sh : {16, 18, 20}) {
                    int rc = build_tiles(int64_t(1) << sh, prec);
                    if (rc)
                        return rc;
                    spmm_tiles(prec);
                    cudaEventRecord(ea, st_);
                    spmm_tiles(prec);
                    cudaEventRecord(eb, st_);
                    PYCI_CUDA_TRY(cudaEventSynchronize(eb));
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ea, eb);
                    if (ms < best) {
                        best = ms;
                        best_sh = sh;
                    }
                }
                cudaEventDestroy(ea);
                cudaEventDestroy(eb);
                tile_nnz_ = best_sh ? int64_t(1) << best_sh : 0;
                tiles_dirty_ = true;
                std::lock_guard<std::mutex> lock(g_class_tune_mutex);
                g_class_tune[key] = best_sh;
            }
            tiles_tuned_ = true;
        }
        if ((tiles_dirty_ || tiles_prec_ != prec) && tile_nnz_) {
            int rc = build_tiles(tile_nnz_, prec);
            if (rc)
                return rc;
        }
        // One run outside any capture: the implicit-form launchers set their
        // kernels' shared-memory limits on first use.
        if (any_imp && !imp_warm_) {
            batch_pack_kernel<T, 4><<<gr, 256, 0, st_>>>(V, N_, d_base_, rs, d_row0_, Xi_);
            spmm_implicit(prec);
            imp_warm_ = true;
        }
        cudaGraph_t g;
        PYCI_CUDA_TRY(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        batch_pack_kernel<T, 4><<<gr, 256, 0, st_>>>(V, N_, d_base_, rs, d_row0_, Xi_);
        if (tile_nnz_) {
            spmm_tiles(prec);
        } else {
            for (int c = 0; c < kClasses; ++c)
                spmm_class(prec, cls_lanes_[c], cls_for(prec, c));
        }
        graph_imp_launches_ = spmm_implicit(prec);
        batch_unpack_kernel<T, 4><<<gr, 256, 0, st_>>>(Yi_, N_, d_base_, rs, d_row0_, W, Wnew_);
        cudaError_t e = cudaStreamEndCapture(st_, &g);
        if (e != cudaSuccess)
            return cuda_status(e, "graph capture");
        e = cudaGraphInstantiate(&graph_exec_, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess)
            return cuda_status(e, "graph instantiate");
        graph_prec_ = prec;
        graph_v_ = V;
        graph_members_ = act_.members;
    }
    if ((tiles_dirty_ || tiles_prec_ != prec) && tile_nnz_) {
        int rc = build_tiles(tile_nnz_, prec); // active set changed: the graph reads the new list
        if (rc)
            return rc;
    }
    cudaEvent_t a, c;
    cudaEventCreate(&a);
    cudaEventCreate(&c);
    cudaEventRecord(a, st_);
    PYCI_CUDA_TRY(cudaGraphLaunch(graph_exec_, st_));
    for (int i = 0; i < (tile_nnz_ ? 3 : 2 + kClasses) + graph_imp_launches_; ++i) // pack, the products, unpack
        ::pyci_gpu::note_launch();
    cudaEventRecord(c, st_);
    PYCI_CUDA_TRY(cudaEventSynchronize(c));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, c);
    spmm_ms_ += ms;
    cudaEventDestroy(a);
    cudaEventDestroy(c);
    return PYCI_GPU_OK;
}

template<typename T>
int Batch<T>::cholqr_block(std::vector<int> &use, T *tmp, T *V, std::vector<int> &knew) {
    const int b = b_, P = P_;
    std::vector<double> Gc;
    int rc;
    knew.assign(P, 0);
    const T *src = Tnew_;
    for (int pass = 0; pass < 2; ++pass) {
        if ((rc = gram<T>(src, b, src, b, Gc)))
            return rc;
        std::vector<double> Y(static_cast<size_t>(P) * b * b, 0.0);
        for (int p = 0; p < P; ++p) {
            const double *S = &Gc[static_cast<size_t>(p) * b * b];
            std::vector<double> L(static_cast<size_t>(b) * b, 0.0);
            std::vector<char> keep(b, 0);
            for (int j = 0; j < b; ++j) {
                if (!use[p * b + j])
                    continue;
                double d = S[j * b + j];
                for (int t = 0; t < j; ++t)
                    if (keep[t])
                        d -= L[j * b + t] * L[j * b + t];
                if (!(d > (mixed_ ? 1e-6 : 1e-14) * S[j * b + j]) || !(d > 0.0)) {
                    use[p * b + j] = 0; // dependent: drop
                    continue;
                }
                keep[j] = 1;
                L[j * b + j] = std::sqrt(d);
                for (int i = j + 1; i < b; ++i) {
                    double x = S[i * b + j];
                    for (int t = 0; t < j; ++t)
                        if (keep[t])
                            x -= L[i * b + t] * L[j * b + t];
                    L[i * b + j] = x / L[j * b + j];
                }
            }
            // Inverse of the kept lower-triangular factor.
            std::vector<double> Li(static_cast<size_t>(b) * b, 0.0);
            for (int j = 0; j < b; ++j) {
                if (!keep[j])
                    continue;
                Li[j * b + j] = 1.0 / L[j * b + j];
                for (int i = j + 1; i < b; ++i) {
                    if (!keep[i])
                        continue;
                    double x = 0.0;
                    for (int t = j; t < i; ++t)
                        if (keep[t])
                            x -= L[i * b + t] * Li[t * b + j];
                    Li[i * b + j] = x / L[i * b + i];
                }
            }
            // Output column c = c-th kept vector on the last pass (compacted),
            // column j = vector j on the first.
            int c = 0;
            for (int j = 0; j < b; ++j) {
                if (!keep[j])
                    continue;
                const int col = (pass == 1) ? c : j;
                for (int i = 0; i < b; ++i)
                    Y[(static_cast<size_t>(p) * b + i) * b + col] = Li[j * b + i];
                ++c;
            }
            if (pass == 1)
                knew[p] = c;
        }
        if (pass == 0) {
            if ((rc = combine<T, T, T>(src, b, Y, b, 0.0, tmp)))
                return rc;
            src = tmp;
        } else {
            if ((rc = combine<T, T, T>(src, b, Y, b, 0.0, V, nullptr, d_base_)))
                return rc;
        }
    }
    // After the second pass, kept vectors sit in the first knew slots: the
    // use flags are re-derived from that order by the caller when needed.
    return PYCI_GPU_OK;
}

template<typename T>
int Batch<T>::run(int64_t maxiter, double tol, const double *ecore, double *evals, double *const *evecs,
                  int64_t *iterations, pyci_gpu_solve_stats *stats) {
    const auto t_start = std::chrono::steady_clock::now();
    const int b = b_, nt = nt_, P = P_, mmax = mmax_;
    int rc;
    row0_.assign(P + 1, 0);
    for (int p = 0; p < P; ++p)
        row0_[p + 1] = row0_[p] + ops_[p]->nrow;
    N_ = row0_[P];
    const int64_t N = N_;
    int64_t ntiles_all = 0;
    for (int p = 0; p < P; ++p)
        ntiles_all += (ops_[p]->nrow + 8191) / 8192;
    for (int p = 0; p < P; ++p)
        all_vals_ = all_vals_ && ops_[p]->vals;
    std::vector<BatchOp> hops(P);
    for (int p = 0; p < P; ++p)
        hops[p] = BatchOp{ops_[p]->rowptr, ops_[p]->cols, ops_[p]->vals, ops_[p]->hi, ops_[p]->lo, row0_[p], ops_[p]->nrow};

    T *V, *W, *X, *AX, *R, *Xk, *Wk, *Xfinal;
    // Kept at a thick restart: the lowest 4 b Ritz vectors (16 for 4 roots),
    // leaving room for a full block.
    const int nkeep = std::max(nt, std::min(mmax - b, 4 * b));
    if ((rc = alloc(&V, static_cast<int64_t>(mmax) * N)) || (rc = alloc(&W, static_cast<int64_t>(mmax) * N)) ||
        (rc = alloc(&X, static_cast<int64_t>(nt) * N)) || (rc = alloc(&AX, static_cast<int64_t>(nt) * N)) ||
        (rc = alloc(&R, static_cast<int64_t>(nt) * N)) || (rc = alloc(&Xk, static_cast<int64_t>(nkeep) * N)) ||
        (rc = alloc(&Wk, static_cast<int64_t>(nkeep) * N)) || (rc = alloc(&Xfinal, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&Tnew_, static_cast<int64_t>(b) * N)) || (rc = alloc(&Wnew_, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&Xi_, N * 4)) || (rc = alloc(&Yi_, N * 4)) || (rc = alloc(&d_row0_, P + 1)) ||
        (rc = alloc(&d_tile_lo_, ntiles_all)) || (rc = alloc(&d_tile_hi_, ntiles_all)) ||
        (rc = alloc(&d_tile_prob_, ntiles_all)) || (rc = alloc(&d_tile_begin_, P + 1)) ||
        (rc = alloc(&d_sel_, P * b)) || (rc = alloc(&d_base_, P)) || (rc = alloc(&d_len_, P)) ||
        (rc = alloc(&d_zero_, P)) || (rc = alloc(&d_mask_, P)) || (rc = alloc(&d_partial_, ntiles_all * kSegMaxP * kSegMaxQ)) ||
        (rc = alloc(&d_small_, static_cast<int64_t>(P) * kSegMaxP * kSegMaxQ)) ||
        (rc = alloc(&d_coef_, static_cast<int64_t>(P) * mmax * std::max(mmax, kSegMaxQ))) ||
        (rc = alloc(&d_theta_, static_cast<int64_t>(P) * nt)) || (rc = alloc(&d_diag_, N)) || (rc = alloc(&d_ops_, P)) ||
        (rc = alloc_rowset(act_)) || (rc = alloc_rowset(sel_)) || (rc = alloc_rowset(cls_[0])) ||
        (rc = alloc_rowset(cls_[1])) || (rc = alloc_rowset(cls_[2])) || (rc = alloc_rowset(cls32_[0])) ||
        (rc = alloc_rowset(cls32_[1])) || (rc = alloc_rowset(cls32_[2])))
        return rc;
    // Tile capacity: every problem cut at the smallest tile size the tuner
    // tries (2^16 entries) or 8 rows, whichever gives more tiles.
    for (int p = 0; p < P; ++p) {
        const double avg = ops_[p]->nrow ? static_cast<double>(ops_[p]->nnz) / ops_[p]->nrow : 1.0;
        const int64_t rows = std::max<int64_t>(8, static_cast<int64_t>((int64_t(1) << 16) / std::max(avg, 1.0)) / 8 * 8);
        tile_cap_ += (ops_[p]->nrow + rows - 1) / rows + 1;
    }
    if ((rc = alloc(&d_tiles_, tile_cap_)) || (rc = alloc(&d_ntiles_, 1)))
        return rc;
    {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_tile_spmm_kernel<1, 4, T>, 256, 0) !=
                cudaSuccess || per_sm < 1)
            per_sm = 1;
        tile_grid_ = static_cast<unsigned>(ctx_->num_sms * per_sm);
    }
    // Every vector buffer starts at zero, so slots a problem has not written
    // yet hold finite values wherever a kernel reads them.
    for (auto pr : {std::make_pair(V, mmax), std::make_pair(W, mmax), std::make_pair(X, nt), std::make_pair(AX, nt),
                    std::make_pair(R, nt), std::make_pair(Xk, nkeep), std::make_pair(Wk, nkeep),
                    std::make_pair(Xfinal, b), std::make_pair(Tnew_, b), std::make_pair(Wnew_, b)})
        PYCI_CUDA_TRY(cudaMemsetAsync(pr.first, 0, sizeof(T) * pr.second * N, st_));
    PYCI_CUDA_TRY(cudaMemsetAsync(Xi_, 0, sizeof(T) * 4 * N, st_));
    PYCI_CUDA_TRY(cudaMemsetAsync(Yi_, 0, sizeof(T) * 4 * N, st_));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_zero_, 0, sizeof(int) * P, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_row0_, row0_.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_ops_, hops.data(), sizeof(BatchOp) * P, cudaMemcpyHostToDevice, st_));
    for (int p = 0; p < P; ++p)
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_diag_ + row0_[p], ops_[p]->diag, sizeof(double) * ops_[p]->nrow,
                                      cudaMemcpyDeviceToDevice, st_));
    cls_of_.assign(P, 0);
    imp_.assign(P, 0);
    for (int p = 0; p < P; ++p) {
        const double avg = ops_[p]->nrow ? static_cast<double>(ops_[p]->nnz) / ops_[p]->nrow : 0.0;
        cls_of_[p] = avg >= 96 ? 2 : (avg >= 24 ? 1 : 0);
        imp_[p] = mixed_ && has_implicit(ops_[p]) && !pinned_to_csr();
    }
    std::vector<int> active(P, 1);
    if ((rc = set_active(active)))
        return rc;

    // Initial block: unit vectors on each problem's b lowest diagonal
    // elements plus a small seeded component in every row, orthonormalised
    // inside each problem's block into slots 0..b-1.
    std::vector<double> diag(N);
    PYCI_CUDA_TRY(cudaMemcpyAsync(diag.data(), d_diag_, sizeof(double) * N, cudaMemcpyDeviceToHost, st_));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
    std::vector<int64_t> pick(static_cast<size_t>(P) * b, -1);
    for (int p = 0; p < P; ++p) {
        const int64_t n = ops_[p]->nrow;
        std::vector<int64_t> order(n);
        std::iota(order.begin(), order.end(), 0);
        const int64_t take = std::min<int64_t>(n, b);
        std::partial_sort(order.begin(), order.begin() + take, order.end(), [&](int64_t x, int64_t y) {
            const double dx = diag[row0_[p] + x], dy = diag[row0_[p] + y];
            return dx < dy || (dx == dy && x < y);
        });
        for (int j = 0; j < take; ++j)
            pick[static_cast<size_t>(p) * b + j] = order[j];
    }
    int64_t *d_pick;
    if ((rc = alloc(&d_pick, static_cast<int64_t>(pick.size()))))
        return rc;
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_pick, pick.data(), sizeof(int64_t) * pick.size(), cudaMemcpyHostToDevice, st_));
    seg_guess_kernel<T><<<grid(N), 256, 0, st_>>>(Tnew_, b, N, act_.view(), d_row0_, d_pick), ::pyci_gpu::note_launch();

    // Per-problem Davidson state: subspace size m[p], projected matrix G[p].
    std::vector<int> m(P, 0), knew(P, 0);
    std::vector<std::vector<double>> G(P, std::vector<double>(static_cast<size_t>(mmax) * mmax, 0.0));
    std::vector<double> theta_all(static_cast<size_t>(P) * nt, 0.0);
    // use[p][c]: column c of the new block is live; conv[p][j]: tracked root j converged.
    std::vector<int> use(static_cast<size_t>(P) * b, 1), conv(static_cast<size_t>(P) * nt, 0);
    for (int p = 0; p < P; ++p)
        for (int j = 0; j < b; ++j)
            use[p * b + j] = (j < ops_[p]->nrow) ? 1 : 0;
    std::vector<int64_t> conv_iter(P, 0);
    if ((rc = upload_ints(d_base_, m)) || (rc = cholqr_block(use, Xk, V, knew)))
        return rc;
    const double eps23 = std::pow(std::numeric_limits<double>::epsilon(), 2.0 / 3.0);
    const double floor_ = mixed_ ? 1e-5 : 0.0;
    const int prec = mixed_ ? PYCI_PREC_FP32 : PYCI_PREC_FP64;
    int64_t iter = 0, restarts = 0;
    int nactive = P;
    std::vector<double> Gc;
    for (iter = 0; iter < maxiter && nactive > 0; ++iter) {
        // W = H V on each problem's new slots [m_p, m_p + b) (d_base_ = m).
        if ((rc = apply_block(prec, V, W)))
            return rc;
        int mcap = 0;
        for (int p = 0; p < P; ++p)
            if (active[p]) {
                matvecs_ += knew[p];
                mcap = std::max(mcap, m[p] + knew[p]);
            }
        // New columns of the projected matrices.
        std::vector<int> len(P, 0);
        for (int p = 0; p < P; ++p)
            len[p] = m[p] + knew[p];
        if ((rc = upload_ints(d_len_, len)) || (rc = gram<T>(V, mcap, Wnew_, b, Gc, d_len_)))
            return rc;
        for (int p = 0; p < P; ++p) {
            if (!active[p])
                continue;
            for (int i = 0; i < m[p] + knew[p]; ++i)
                for (int j = 0; j < knew[p]; ++j) {
                    const double g = Gc[(static_cast<size_t>(p) * mcap + i) * b + j];
                    G[p][static_cast<size_t>(i) * mmax + m[p] + j] = g;
                    G[p][static_cast<size_t>(m[p] + j) * mmax + i] = g;
                }
            m[p] += knew[p];
        }
        // Rayleigh-Ritz per active problem.
        int mrr = 0;
        for (int p = 0; p < P; ++p)
            if (active[p])
                mrr = std::max(mrr, m[p]);
        std::vector<double> Yb(static_cast<size_t>(P) * mrr * nt, 0.0), Yk(static_cast<size_t>(P) * mrr * nkeep, 0.0);
        std::vector<char> rr_failed(P, 0);
        host_parallel_for(P, [&](int p) {
            if (!active[p])
                return;
            const int mv = m[p];
            std::vector<double> Gm(static_cast<size_t>(mv) * mv), th, Y;
            for (int i = 0; i < mv; ++i)
                for (int j = 0; j < mv; ++j)
                    Gm[static_cast<size_t>(i) * mv + j] = G[p][static_cast<size_t>(i) * mmax + j];
            if (!symmetric_eigen(mv, Gm, th, Y)) {
                rr_failed[p] = 1;
                return;
            }
            for (int j = 0; j < nt; ++j) {
                theta_all[p * nt + j] = (j < mv) ? th[j] : 0.0;
                if (j < mv)
                    for (int i = 0; i < mv; ++i)
                        Yb[(static_cast<size_t>(p) * mrr + i) * nt + j] = Y[static_cast<size_t>(i) * mv + j];
            }
            for (int j = 0; j < std::min(nkeep, mv); ++j)
                for (int i = 0; i < mv; ++i)
                    Yk[(static_cast<size_t>(p) * mrr + i) * nkeep + j] = Y[static_cast<size_t>(i) * mv + j];
        });
        for (int p = 0; p < P; ++p)
            if (rr_failed[p]) {
                set_error("Rayleigh-Ritz eigensolver failed (problem %d)", p);
                return PYCI_GPU_ENOCONV;
            }
        if ((rc = upload_ints(d_len_, m)) || (rc = combine<T, T, T>(V, mrr, Yb, nt, 0.0, X, d_len_)) ||
            (rc = combine<T, T, T>(W, mrr, Yb, nt, 0.0, AX, d_len_)))
            return rc;
        if ((rc = ctx_->ring->upload(d_theta_, theta_all.data(), sizeof(double) * P * nt, st_)))
            return rc;
        seg_residual_kernel<T><<<grid(act_.total), 256, 0, st_>>>(AX, X, d_theta_, nt, N, act_.view(), d_row0_, R),
            ::pyci_gpu::note_launch();
        if ((rc = gram<T>(R, nt, R, nt, Gc)))
            return rc;
        std::vector<int> finished;
        for (int p = 0; p < P; ++p) {
            if (!active[p])
                continue;
            bool done = true;
            for (int j = 0; j < nt; ++j) {
                const double rn = std::sqrt(std::max(Gc[(static_cast<size_t>(p) * nt + j) * nt + j], 0.0));
                const double thr = std::max(tol * std::max(eps23, std::fabs(theta_all[p * nt + j])), floor_);
                const bool cj = !(j < ops_[p]->nrow) || rn <= thr || m[p] >= ops_[p]->nrow;
                conv[p * nt + j] = cj ? 1 : 0;
                if (j < b)
                    done = done && cj; // the guard pair (j = b) need not converge
            }
            if (done)
                finished.push_back(p);
        }
        // Problems whose corrections were all dependent last time cannot grow
        // their subspace: they finish with their current Ritz vectors.
        for (int p = 0; p < P; ++p)
            if (active[p] && iter > 0 && knew[p] == 0 &&
                std::find(finished.begin(), finished.end(), p) == finished.end())
                finished.push_back(p);
        if (!finished.empty()) {
            std::vector<int> mask(P, 0);
            for (int p : finished) {
                mask[p] = 1;
                active[p] = 0;
                conv_iter[p] = iter + 1;
                --nactive;
            }
            // Keep the finished problems' Ritz vectors for the final FP64 step.
            if ((rc = set_rowset(sel_, mask)))
                return rc;
            seg_copy_kernel<T><<<grid(sel_.total), 256, 0, st_>>>(X, b, N, sel_.view(), d_row0_, Xfinal),
                ::pyci_gpu::note_launch();
            if ((rc = set_active(active)))
                return rc;
        }
        if (nactive == 0)
            break;
        // Thick restart of the problems whose next block would not fit.
        std::vector<int> rmask(P, 0);
        bool any_restart = false;
        for (int p = 0; p < P; ++p)
            if (active[p] && m[p] + b > mmax) {
                rmask[p] = 1;
                any_restart = true;
            }
        if (any_restart) {
            if ((rc = set_rowset(sel_, rmask)) || (rc = upload_ints(d_mask_, rmask)) ||
                (rc = combine<T, T, T>(V, mrr, Yk, nkeep, 0.0, Xk, d_len_, nullptr, d_mask_)) ||
                (rc = combine<T, T, T>(W, mrr, Yk, nkeep, 0.0, Wk, d_len_, nullptr, d_mask_)))
                return rc;
            seg_copy_kernel<T><<<grid(sel_.total), 256, 0, st_>>>(Xk, nkeep, N, sel_.view(), d_row0_, V),
                ::pyci_gpu::note_launch();
            seg_copy_kernel<T><<<grid(sel_.total), 256, 0, st_>>>(Wk, nkeep, N, sel_.view(), d_row0_, W),
                ::pyci_gpu::note_launch();
            // Projected matrix of the kept Ritz vectors, recomputed.
            if ((rc = gram<T>(V, nkeep, W, nkeep, Gc)))
                return rc;
            for (int p = 0; p < P; ++p) {
                if (!rmask[p])
                    continue;
                ++restarts;
                const int kept = std::min(nkeep, m[p]);
                std::fill(G[p].begin(), G[p].end(), 0.0);
                for (int i = 0; i < kept; ++i)
                    for (int j = 0; j < kept; ++j)
                        G[p][static_cast<size_t>(i) * mmax + j] = Gc[(static_cast<size_t>(p) * nkeep + i) * nkeep + j];
                m[p] = kept;
            }
        }
        // Corrections of the lowest unconverged roots (at most b per active
        // problem) into Tnew_.
        // The block-diagonal product is always b wide, so a problem with fewer
        // unconverged roots fills its block with the lowest converged ones.
        std::vector<int> sel(static_cast<size_t>(P) * b, -1);
        for (int p = 0; p < P; ++p) {
            int c = 0;
            if (active[p]) {
                for (int j = 0; j < nt && c < b; ++j)
                    if (!conv[p * nt + j])
                        sel[p * b + c++] = j;
                for (int j = 0; j < nt && c < b && j < m[p]; ++j)
                    if (conv[p * nt + j] && m[p] < ops_[p]->nrow)
                        sel[p * b + c++] = j;
            }
            for (int cc = 0; cc < b; ++cc)
                use[p * b + cc] = (sel[p * b + cc] >= 0) ? 1 : 0;
        }
        if ((rc = ctx_->ring->upload(d_sel_, sel.data(), sizeof(int) * P * b, st_)))
            return rc;
        seg_precondition_kernel<T><<<grid(act_.total), 256, 0, st_>>>(R, d_theta_, nt, d_sel_, d_diag_, b, N,
                                                                       act_.view(), d_row0_, Tnew_),
            ::pyci_gpu::note_launch();
        // Two passes of segmented block Gram-Schmidt against each basis.
        int mgs = 0;
        for (int p = 0; p < P; ++p)
            if (active[p])
                mgs = std::max(mgs, m[p]);
        if ((rc = upload_ints(d_len_, m)))
            return rc;
        for (int pass = 0; pass < 2; ++pass) {
            if ((rc = gram<T>(V, mgs, Tnew_, b, Gc, d_len_)))
                return rc;
            std::vector<double> C(static_cast<size_t>(P) * mgs * b, 0.0);
            for (int p = 0; p < P; ++p)
                if (active[p])
                    for (int i = 0; i < m[p]; ++i)
                        for (int j = 0; j < b; ++j)
                            C[(static_cast<size_t>(p) * mgs + i) * b + j] = -Gc[(static_cast<size_t>(p) * mgs + i) * b + j];
            if ((rc = combine<T, T, T>(V, mgs, C, b, 1.0, Tnew_, d_len_)))
                return rc;
        }
        // Orthonormalise inside each block into the next slots.
        if ((rc = upload_ints(d_base_, m)) || (rc = cholqr_block(use, Xk, V, knew)))
            return rc;
    }
    if (nactive > 0) {
        set_error("did not converge (%d of %d problems)", nactive, P);
        return PYCI_GPU_ENOCONV;
    }
    // Final Rayleigh-Ritz of every problem's Ritz block against the FP64
    // operator (high + low in mixed mode), with FP64 residual norms.
    std::fill(active.begin(), active.end(), 1);
    if ((rc = set_active(active)))
        return rc;
    double *X64, *AX64, *E64, *AE64, *R64, *Xi64, *Yi64;
    if ((rc = alloc(&X64, static_cast<int64_t>(b) * N)) || (rc = alloc(&AX64, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&E64, static_cast<int64_t>(b) * N)) || (rc = alloc(&AE64, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&R64, static_cast<int64_t>(b) * N)) || (rc = alloc(&Xi64, N * 4)) || (rc = alloc(&Yi64, N * 4)))
        return rc;
    batch_convert_kernel<T, double><<<grid(static_cast<int64_t>(b) * N), 256, 0, st_>>>(Xfinal, X64, static_cast<int64_t>(b) * N),
        ::pyci_gpu::note_launch();
    {
        const RowSet rs = act_.view();
        const unsigned gr = grid(N);
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ctx_->num_sms * 32, (N * 32 + 255) / 256));
        if (mixed_ || !all_vals_) {
            // FP64-accurate products in FP32 arithmetic from high + low values.
            float *xs = reinterpret_cast<float *>(Xi64); // [N][8] floats fit in [N][4] doubles
            batch_pack_split_kernel<<<gr, 256, 0, st_>>>(X64, N, rs, d_row0_, xs), ::pyci_gpu::note_launch();
            batch_spmm_df_kernel<16><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, rs, xs, Yi64),
                ::pyci_gpu::note_launch();
        } else {
            batch_pack_kernel<double, 4><<<gr, 256, 0, st_>>>(X64, N, d_zero_, rs, d_row0_, Xi64), ::pyci_gpu::note_launch();
            batch_spmm_kernel<0, 4, 32, double><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, rs, Xi64, Yi64),
                ::pyci_gpu::note_launch();
        }
        batch_unpack_kernel<double, 4><<<gr, 256, 0, st_>>>(Yi64, N, d_zero_, rs, d_row0_, AX64, nullptr),
            ::pyci_gpu::note_launch();
        matvecs_ += static_cast<int64_t>(P) * b;
    }
    std::vector<double> S64, H64;
    if ((rc = gram<double>(X64, b, X64, b, S64)) || (rc = gram<double>(X64, b, AX64, b, H64)))
        return rc;
    // Coefficients of the FP64 eigenvectors in the Ritz block, per problem,
    // in decreasing order of eigenvalue (the reference's result order).
    std::vector<double> C(static_cast<size_t>(P) * b * b, 0.0), eord(static_cast<size_t>(P) * b, 0.0);
    for (int p = 0; p < P; ++p) {
        // Generalised b x b problem H y = e S y via S^{-1/2}.
        const int n = static_cast<int>(std::min<int64_t>(b, ops_[p]->nrow));
        std::vector<double> S(static_cast<size_t>(n) * n), H(static_cast<size_t>(n) * n), se, sv;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                S[i * n + j] = S64[(static_cast<size_t>(p) * b + i) * b + j];
                H[i * n + j] = 0.5 * (H64[(static_cast<size_t>(p) * b + i) * b + j] + H64[(static_cast<size_t>(p) * b + j) * b + i]);
            }
        symmetric_eigen(n, S, se, sv);
        std::vector<double> Sm(static_cast<size_t>(n) * n, 0.0); // S^{-1/2}
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int t = 0; t < n; ++t)
                    Sm[i * n + j] += sv[i * n + t] * sv[j * n + t] / std::sqrt(std::max(se[t], 1e-300));
        std::vector<double> A(static_cast<size_t>(n) * n, 0.0), tmp(static_cast<size_t>(n) * n, 0.0), e, v;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int t = 0; t < n; ++t)
                    tmp[i * n + j] += Sm[i * n + t] * H[t * n + j];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int t = 0; t < n; ++t)
                    A[i * n + j] += tmp[i * n + t] * Sm[t * n + j];
        symmetric_eigen(n, A, e, v);
        for (int c = 0; c < n; ++c) {
            const int src = n - 1 - c;
            eord[static_cast<size_t>(p) * b + c] = e[src];
            // y = S^{-1/2} v[:, src]
            for (int i = 0; i < n; ++i) {
                double y = 0.0;
                for (int t = 0; t < n; ++t)
                    y += Sm[i * n + t] * v[t * n + src];
                C[(static_cast<size_t>(p) * b + i) * b + c] = y;
            }
        }
        for (int c = 0; c < b; ++c)
            evals[static_cast<size_t>(p) * b + c] = (c < n) ? eord[static_cast<size_t>(p) * b + c] + ecore[p] : 0.0;
    }
    // Eigenvectors E = X C and residuals H E - e E in FP64.
    if ((rc = combine<double, double, double>(X64, b, C, b, 0.0, E64)) ||
        (rc = combine<double, double, double>(AX64, b, C, b, 0.0, AE64)))
        return rc;
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_theta_, eord.data(), sizeof(double) * P * b, cudaMemcpyHostToDevice, st_));
    seg_residual_kernel<double><<<grid(N), 256, 0, st_>>>(AE64, E64, d_theta_, b, N, act_.view(), d_row0_, R64),
        ::pyci_gpu::note_launch();
    std::vector<double> RR;
    if ((rc = gram<double>(R64, b, R64, b, RR)))
        return rc;
    double max_res = 0.0;
    for (int p = 0; p < P; ++p)
        for (int j = 0; j < std::min<int64_t>(b, ops_[p]->nrow); ++j)
            max_res = std::max(max_res, std::sqrt(std::max(RR[(static_cast<size_t>(p) * b + j) * b + j], 0.0)));
    if (evecs) {
        for (int p = 0; p < P; ++p) {
            if (!evecs[p])
                continue;
            for (int c = 0; c < b; ++c)
                PYCI_CUDA_TRY(cudaMemcpyAsync(evecs[p] + static_cast<int64_t>(c) * ops_[p]->nrow,
                                              E64 + static_cast<int64_t>(c) * N + row0_[p],
                                              sizeof(double) * ops_[p]->nrow, cudaMemcpyDeviceToHost, st_));
        }
    }
    PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
    if (iterations)
        for (int p = 0; p < P; ++p)
            iterations[p] = conv_iter[p];
    if (stats) {
        stats->iterations = iter + 1;
        stats->matvecs = matvecs_;
        stats->matvecs_fp64 = mixed_ ? static_cast<int64_t>(P) * b : matvecs_;
        stats->restarts = restarts;
        stats->refinements = 1;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->seconds_spmm = spmm_ms_ * 1e-3;
        stats->max_residual = max_res;
        stats->host_syncs = 0; // not counted by the batched solver
        stats->seconds_wait = 0.0;
    }
    return PYCI_GPU_OK;
}

} // namespace

extern "C" int pyci_gpu_batch_solve(pyci_gpu_ctx *ctx, int64_t nprob, pyci_gpu_csr *const *ops, int64_t n,
                                    int64_t maxiter, double tol, const double *ecore, int mode, double *evals,
                                    double *const *evecs, int64_t *iterations, pyci_gpu_solve_stats *stats) {
    if (!ctx || !ops || !ecore || !evals || nprob <= 0) {
        set_error("NULL argument or empty batch");
        return PYCI_GPU_EINVAL;
    }
    if (n != 4) {
        set_error("the batched solver computes 4 roots per problem (n = %lld)", (long long)n);
        return PYCI_GPU_EUNSUPPORTED;
    }
    std::vector<pyci_gpu_csr *> v(ops, ops + nprob);
    for (auto *c : v) {
        if (!c || c->ctx != ctx) {
            set_error("every operator must belong to the given context");
            return PYCI_GPU_EINVAL;
        }
        if (!c->symmetric || c->nrow != c->ncol || c->lower_only) {
            set_error("batched solve needs square symmetric operators with both triangles stored");
            return PYCI_GPU_ETYPE;
        }
        if (c->nrow <= n) {
            set_error("every problem needs more than n rows");
            return PYCI_GPU_EINVAL;
        }
    }
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t iters = (maxiter > 0) ? maxiter : 1000;
    const int mmax = 64; // per-problem subspace (restarts keep 16)
    if (mode == PYCI_SOLVE_MIXED) {
        for (auto *c : v) {
            // The batched kernels read the CSR-order split.  One operator at
            // a time: a deferred CSR is written, split, and its FP64 values
            // freed again when prepare_mixed(drop_fp64) asked for that, so
            // the FP64 values of all operators never coexist.
            int rc = csr_materialize(c);
            if (!rc)
                rc = csr_prepare_mixed_device(c, 0);
            if (!rc)
                rc = csr_ensure_split(c);
            if (rc)
                return rc;
        }
        Batch<float> bsolve(ctx, v, static_cast<int>(n), mmax, true);
        return bsolve.run(iters, tol, ecore, evals, evecs, iterations, stats);
    }
    for (auto *c : v) {
        // The batched kernels read the CSR: write deferred entries first.
        int rc = csr_materialize(c);
        if (rc)
            return rc;
        if (!c->vals && !(c->hi && c->lo)) {
            set_error("FP64 batched solve needs FP64 values");
            return PYCI_GPU_EINVAL;
        }
    }
    Batch<double> bsolve(ctx, v, static_cast<int>(n), mmax, false);
    return bsolve.run(iters, tol, ecore, evals, evecs, iterations, stats);
}
