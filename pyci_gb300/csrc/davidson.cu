// Block Davidson eigensolver on the device CSR, replacing SparseOp::solve_ci
// (pyci/src/sparseop.cpp:114-146), which runs Spectra's implicitly restarted
// Lanczos on the host.  Same contract: the n algebraically smallest
// eigenpairs, ecore added, returned in decreasing order (Spectra's result
// order), ValueError / TypeError / RuntimeError conditions preserved.
//
// Layout: basis V and W = H V as [m][N] (one vector per row, contiguous, for
// coalesced tall-skinny products); the SpMM reads an interleaved [N][k]
// copy.  Per iteration: W_new = H V_new (one SpMM for the whole block),
// Gram column V^T W_new, Rayleigh-Ritz on the host (m <= ~64), Ritz vectors
// and residuals, diagonal (Davidson) preconditioning, two-pass block
// Gram-Schmidt, thick restart to the lowest Ritz vectors.
//
// Two precisions:
//   FP64  -- values, vectors and products in FP64.
//   MIXED -- FP32 values (high part of an exact FP32 high/low split), FP32
//            vectors and SpMM; Gram sums finish in FP64; Rayleigh-Ritz in
//            FP64.  When the FP32 residuals meet the tolerance, the Ritz
//            vectors are rebuilt in FP64, multiplied by the FP64 operator
//            (high + low values), re-orthonormalised and Rayleigh-Ritz'd in
//            FP64; FP64 residuals decide convergence and, if still too large,
//            seed further FP32 iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

#include "dense.h"
#include "dfarith.cuh"
#include "internal.h"
#include "split_bits.h"

namespace pyci_gpu {

constexpr int kMaxGramP = 128;
constexpr int kMaxQ = 8;
// FP32 Gram products with at least this many A vectors run on the tensor
// cores (gram_tc.cu); narrower ones on the CUDA cores, where the tensor-core
// version is bound by its per-tile MMA latency.  With the CUDA-core kernel's
// vector blocks of one row range running together (B re-read from L2), the
// tensor cores win only for the widest blocks (10.5M-row vectors, wall time
// per call: p = 128, q = 8: 2.06 vs 2.42 ms; p = 64, q = 4: 1.07 vs 1.20 ms
// with ~0.5 ms of call overhead in both; in the 32-orbital DOCI solve the
// p >= 48 tensor-core Grams took 0.92 ms of device time each).
constexpr int kGramTcMinP = 96;

// Xi[r * kp + j] = V[j * N + r] for j < k, 0 for k <= j < kp (padding to a
// width the SpMM gathers with vector loads).
template<typename T>
__global__ void pack_kernel(const T *__restrict__ V, int64_t N, int k, int kp, T *__restrict__ Xi) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        for (int j = 0; j < kp; ++j)
            Xi[r * kp + j] = (j < k) ? V[j * N + r] : T(0);
}

// xs[r][j] = fl32(V[j][r]), xs[r][K + j] = fl32(V[j][r] - xs[r][j]) for j < k,
// zero for k <= j < K: the split operand of the double-float SpMM.
__global__ void pack_split_kernel(const double *__restrict__ V, int64_t N, int k, int K, float *__restrict__ xs) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        for (int j = 0; j < K; ++j) {
            const double v = (j < k) ? V[j * N + r] : 0.0;
            const float h = static_cast<float>(v);
            xs[r * 2 * K + j] = h;
            xs[r * 2 * K + K + j] = static_cast<float>(v - static_cast<double>(h));
        }
}

// W[j * N + r] = Yi[r * kp + j] for j < k; FP32 rows of a multiple of 4
// entries are read with 16-byte loads (one per 4 entries instead of 4).
template<typename T>
__global__ void unpack_kernel(const T *__restrict__ Yi, int64_t N, int k, int kp, T *__restrict__ W) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if constexpr (sizeof(T) == 4) {
            if (kp % 4 == 0) {
                for (int j4 = 0; j4 < k; j4 += 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(Yi + r * kp + j4);
                    W[j4 * N + r] = v.x;
                    if (j4 + 1 < k)
                        W[(j4 + 1) * N + r] = v.y;
                    if (j4 + 2 < k)
                        W[(j4 + 2) * N + r] = v.z;
                    if (j4 + 3 < k)
                        W[(j4 + 3) * N + r] = v.w;
                }
                continue;
            }
        }
        for (int j = 0; j < k; ++j)
            W[j * N + r] = Yi[r * kp + j];
    }
}

// Width the SpMM reads with 8/16-byte vector gathers: 3 -> 4, 5..7 -> 8.
inline int padded_width(int k) { return k == 3 ? 4 : (k > 4 && k < 8 ? 8 : k); }

// Vectors per SpMM launch in the eigensolver: blocks wider than 4 run as
// several products of at most 4 (a 5-vector block as 4 + 1 instead of one
// product padded to 8), since the gather-bound product costs about as much
// per gathered byte at any width.
constexpr int kSpmmChunk = 4;

// R consecutive entries of a vector from one 16-byte load (R = 16 /
// sizeof(T)), or one entry (R = 1).
template<typename T, int R>
__device__ __forceinline__ void load_rows(const T *__restrict__ p, T (&v)[R]) {
    if constexpr (R == 1) {
        v[0] = p[0];
    } else if constexpr (sizeof(T) == 4) {
        static_assert(R == 4, "four floats per 16-byte load");
        const float4 w = *reinterpret_cast<const float4 *>(p);
        v[0] = w.x, v[1] = w.y, v[2] = w.z, v[3] = w.w;
    } else {
        static_assert(R == 2, "two doubles per 16-byte load");
        const double2 w = *reinterpret_cast<const double2 *>(p);
        v[0] = w.x, v[1] = w.y;
    }
}

// Stores R consecutive entries (R = 1, or 16 / sizeof(TV) of the input
// vectors: one 16-byte store per 4 floats or per 2 doubles).
template<typename T, int R>
__device__ __forceinline__ void store_rows(T *__restrict__ p, const T (&v)[R]) {
    if constexpr (R == 1) {
        p[0] = v[0];
    } else if constexpr (sizeof(T) == 4) {
        static_assert(R == 4, "four floats per 16-byte store");
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int t = 0; t < R; t += 2)
            *reinterpret_cast<double2 *>(p + t) = make_double2(v[t], v[t + 1]);
    }
}

// Row-streaming Gram product: block (x, y) sums A[i][r] * B[j][r] over a
// grid-stride set of rows (row blocks along y) for i in [x * PI, x * PI + PI),
// j < q <= QC, with a per-thread PI x QC register tile (one coalesced pass
// over the rows), then reduces across the block; partial[y][i * q + j].  The
// vector blocks of one row range are neighbouring block indices (x fastest),
// so they run together and B's rows, read by each of them, come from L2.  QC is the smallest of
// 1, 2, 4, 8 that holds q, so the tile (and the register count) follows q.
// R > 1: each thread step takes R consecutive rows with 16-byte loads (N a
// multiple of R, vectors 16-byte aligned), R times the bytes in flight per
// load instruction of the one-row form.
template<typename T, int PI, int QC, int R>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) gram_rows_kernel(const T *__restrict__ A, int p,
                                                                            const T *__restrict__ B,
                                                        int q, int64_t N, double *__restrict__ partial) {
    const int i0 = blockIdx.x * PI;
    const int ni = min(PI, p - i0);
    T acc[PI][QC];
#pragma unroll
    for (int ii = 0; ii < PI; ++ii)
#pragma unroll
        for (int j = 0; j < QC; ++j)
            acc[ii][j] = T(0);
    const int64_t nu = N / R;
    for (int64_t u = blockIdx.y * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < nu;
         u += static_cast<int64_t>(gridDim.y) * blockDim.x) {
        const int64_t r = u * R;
        T bv[QC][R];
#pragma unroll
        for (int j = 0; j < QC; ++j) {
            if (j < q) {
                load_rows<T, R>(B + j * N + r, bv[j]);
            } else {
#pragma unroll
                for (int t = 0; t < R; ++t)
                    bv[j][t] = T(0);
            }
        }
#pragma unroll
        for (int ii = 0; ii < PI; ++ii) {
            if (ii < ni) {
                T a[R];
                load_rows<T, R>(A + (i0 + ii) * N + r, a);
#pragma unroll
                for (int j = 0; j < QC; ++j)
#pragma unroll
                    for (int t = 0; t < R; ++t)
                        acc[ii][j] += a[t] * bv[j][t];
            }
        }
    }
    __shared__ double red[8][PI * QC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Warp sums in T (FP32 for FP32 vectors: this GPU's FP64 add rate is a
    // small fraction of its FP32 rate, and 5 levels of FP64 adds on every
    // accumulator cost as much as the row pass of a short product); FP64
    // from the cross-warp sum on.
#pragma unroll
    for (int ii = 0; ii < PI; ++ii)
#pragma unroll
        for (int j = 0; j < QC; ++j) {
            T v = acc[ii][j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0)
                red[warp][ii * QC + j] = static_cast<double>(v);
        }
    __syncthreads();
    const int nwarps = blockDim.x >> 5;
    for (int idx = threadIdx.x; idx < ni * q; idx += blockDim.x) {
        const int ii = idx / q, j = idx % q;
        double v = 0.0;
        for (int w = 0; w < nwarps; ++w)
            v += red[w][ii * QC + j];
        partial[static_cast<int64_t>(blockIdx.y) * p * q + (i0 + ii) * q + j] = v;
    }
}

// The FP64 solve's Gram products in double-float arithmetic: each FP64
// element is split into FP32 high and low parts (integer arithmetic, exact),
// each product (ah + al)(bh + bl) formed with an FMA for the error of ah bh
// and FP32 cross terms, summed with TwoSum per thread, and the thread sums
// added in FP64 from the warp reduction on.  About 2^-47 relative per
// product against 2^-53 in FP64, at FP32 issue rates: this GPU's FP64 pipe
// runs a small fraction of them, and bounds the FP64 form of this product
// (2 p q FMAs per row against 8 (p + q) bytes read).
template<int PI, int QC>
__global__ void __launch_bounds__(256) gram_rows_df_kernel(const double *__restrict__ A, int p,
                                                           const double *__restrict__ B, int q, int64_t N,
                                                           double *__restrict__ partial) {
    const int i0 = blockIdx.x * PI;
    const int ni = min(PI, p - i0);
    float s[PI][QC], c[PI][QC];
#pragma unroll
    for (int ii = 0; ii < PI; ++ii)
#pragma unroll
        for (int j = 0; j < QC; ++j)
            s[ii][j] = c[ii][j] = 0.0f;
    for (int64_t r = blockIdx.y * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.y) * blockDim.x) {
        float bh[QC], bl[QC];
#pragma unroll
        for (int j = 0; j < QC; ++j) {
            bh[j] = bl[j] = 0.0f;
            if (j < q)
                split_hi_lo(B[j * N + r], bh[j], bl[j]);
        }
#pragma unroll
        for (int ii = 0; ii < PI; ++ii) {
            if (ii < ni) {
                float ah, al;
                split_hi_lo(A[(i0 + ii) * N + r], ah, al);
                df_term<QC>(ah, al, bh, bl, s[ii], c[ii]);
            }
        }
    }
    __shared__ double red[8][PI * QC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int ii = 0; ii < PI; ++ii)
#pragma unroll
        for (int j = 0; j < QC; ++j) {
            double v = static_cast<double>(s[ii][j]) + static_cast<double>(c[ii][j]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0)
                red[warp][ii * QC + j] = v;
        }
    __syncthreads();
    const int nwarps = blockDim.x >> 5;
    for (int idx = threadIdx.x; idx < ni * q; idx += blockDim.x) {
        const int ii = idx / q, j = idx % q;
        double v = 0.0;
        for (int w = 0; w < nwarps; ++w)
            v += red[w][ii * QC + j];
        partial[static_cast<int64_t>(blockIdx.y) * p * q + (i0 + ii) * q + j] = v;
    }
}

// Launch gram_rows_kernel with the register tile that fits q (<= 8): rows
// of A per block PI = 8 (4 when q > 4).  budget: blocks to aim for.  Returns
// the number of partial sums per entry (blocks along x).
// One wave of blocks: the grid holds at most as many blocks as are resident
// at once (occupancy of the instantiation, at most 4 per SM), so no block
// runs in a second, partly idle wave.  budget = 4 blocks per SM; partial
// holds budget blocks' sums.
template<typename T, int PI, int QC, int R>
unsigned launch_gram_tile(unsigned budget, cudaStream_t st, const T *A, int p, const T *B, int q, int64_t N,
                          double *partial) {
    static const int per_sm = [] {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gram_rows_kernel<T, PI, QC, R>, 256, 0) != cudaSuccess)
            n = 1;
        return std::max(1, std::min(4, n));
    }();
    const int64_t wave = static_cast<int64_t>(budget / 4) * per_sm;
    const unsigned gy = static_cast<unsigned>((p + PI - 1) / PI);
    const unsigned nb = static_cast<unsigned>(
        std::max<int64_t>(1, std::min<int64_t>(std::max<int64_t>(1, wave / gy), (N / R + 255) / 256)));
    gram_rows_kernel<T, PI, QC, R><<<dim3(gy, nb), 256, 0, st>>>(A, p, B, q, N, partial);
    return nb;
}

template<typename T, int R>
unsigned launch_gram_rows_r(unsigned budget, cudaStream_t st, const T *A, int p, const T *B, int q, int64_t N,
                            double *partial) {
    if (q <= 1)
        return launch_gram_tile<T, 8, 1, R>(budget, st, A, p, B, q, N, partial);
    if (q <= 2)
        return launch_gram_tile<T, 8, 2, R>(budget, st, A, p, B, q, N, partial);
    if (q <= 4)
        return launch_gram_tile<T, 8, 4, R>(budget, st, A, p, B, q, N, partial);
    return launch_gram_tile<T, 4, 8, R>(budget, st, A, p, B, q, N, partial);
}

// 16-byte row loads when N is a multiple of 16 / sizeof(T) and both vector
// sets start on 16-byte boundaries (every vector then does).
// launch_gram_tile's grid for gram_rows_df_kernel (one row per thread step).
template<int PI, int QC>
unsigned launch_gram_df_tile(unsigned budget, cudaStream_t st, const double *A, int p, const double *B, int q,
                             int64_t N, double *partial) {
    static const int per_sm = [] {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gram_rows_df_kernel<PI, QC>, 256, 0) != cudaSuccess)
            n = 1;
        return std::max(1, std::min(4, n));
    }();
    const int64_t wave = static_cast<int64_t>(budget / 4) * per_sm;
    const unsigned gy = static_cast<unsigned>((p + PI - 1) / PI);
    const unsigned nb = static_cast<unsigned>(
        std::max<int64_t>(1, std::min<int64_t>(std::max<int64_t>(1, wave / gy), (N + 255) / 256)));
    gram_rows_df_kernel<PI, QC><<<dim3(gy, nb), 256, 0, st>>>(A, p, B, q, N, partial);
    return nb;
}

unsigned launch_gram_df(unsigned budget, cudaStream_t st, const double *A, int p, const double *B, int q, int64_t N,
                        double *partial) {
    // Register tiles of at most 16 (sum, error) pairs per thread.
    if (q <= 1)
        return launch_gram_df_tile<8, 1>(budget, st, A, p, B, q, N, partial);
    if (q <= 2)
        return launch_gram_df_tile<8, 2>(budget, st, A, p, B, q, N, partial);
    if (q <= 4)
        return launch_gram_df_tile<4, 4>(budget, st, A, p, B, q, N, partial);
    return launch_gram_df_tile<2, 8>(budget, st, A, p, B, q, N, partial);
}

template<typename T>
unsigned launch_gram_rows(unsigned budget, cudaStream_t st, const T *A, int p, const T *B, int q, int64_t N,
                          double *partial) {
    constexpr int R = 16 / sizeof(T);
    if (N % R == 0 && reinterpret_cast<uintptr_t>(A) % 16 == 0 && reinterpret_cast<uintptr_t>(B) % 16 == 0)
        return launch_gram_rows_r<T, R>(budget, st, A, p, B, q, N, partial);
    return launch_gram_rows_r<T, 1>(budget, st, A, p, B, q, N, partial);
}

__global__ void reduce_partials_kernel(const double *__restrict__ partial, int nblocks, int pq,
                                       double *__restrict__ out) {
    const int idx = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        s += partial[static_cast<int64_t>(b) * pq + idx];
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0)
            out[idx] = s;
    }
}

// Coefficients of one double-float combination launch: FP32 high and low
// parts of each FP64 coefficient.
struct CoefBlockDF {
    float h[kMaxGramP * kMaxQ], l[kMaxGramP * kMaxQ];
};

// The FP64 solve's combinations in double-float arithmetic (see
// gram_rows_df_kernel): out[j][r] = beta out[j][r] + sum_i Y[i][j] V[i][r]
// with V's elements split exactly into FP32 high and low parts, products and
// sums in FP32 with TwoSum, and FP64 only for the final beta step.  Two rows
// per thread step (16-byte loads) when N is even and the vectors 16-byte
// aligned (R = 2), else one.
template<int R>
__global__ void __launch_bounds__(256) combine_df_kernel(const double *__restrict__ V, int p, int64_t N,
                                                         const __grid_constant__ CoefBlockDF Y, int q, double beta,
                                                         double *__restrict__ out) {
    const int64_t nu = N / R;
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < nu;
         u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = u * R;
        float s[kMaxQ][R], c[kMaxQ][R];
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
#pragma unroll
            for (int t = 0; t < R; ++t)
                s[j][t] = c[j][t] = 0.0f;
#pragma unroll 4
        for (int i = 0; i < p; ++i) {
            double v[R];
            if constexpr (R == 2) {
                const double2 w = *reinterpret_cast<const double2 *>(V + i * N + r);
                v[0] = w.x;
                v[1] = w.y;
            } else {
                v[0] = V[i * N + r];
            }
            float vh[R], vl[R];
#pragma unroll
            for (int t = 0; t < R; ++t)
                split_hi_lo(v[t], vh[t], vl[t]);
#pragma unroll
            for (int j = 0; j < kMaxQ; ++j)
                if (j < q) {
                    const float yh = Y.h[i * q + j], yl = Y.l[i * q + j];
#pragma unroll
                    for (int t = 0; t < R; ++t) {
                        const float pr = __fmul_rn(yh, vh[t]);
                        const float err = fmaf(yh, vh[t], -pr);
                        const float tt = fmaf(yh, vl[t], fmaf(yl, vh[t], err));
                        df_two_sum(s[j][t], c[j][t], pr);
                        c[j][t] = __fadd_rn(c[j][t], tt);
                    }
                }
        }
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
            if (j < q) {
                double *o = out + j * N + r;
#pragma unroll
                for (int t = 0; t < R; ++t) {
                    const double sum = static_cast<double>(s[j][t]) + static_cast<double>(c[j][t]);
                    o[t] = beta == 0.0 ? sum : fma(beta, o[t], sum);
                }
            }
    }
}

// Coefficients of one combination launch (p x q <= kMaxGramP x kMaxQ,
// row-major), passed as a kernel parameter: no host -> device copy in the
// stream between the kernels (4 KB for FP32, 8 KB for FP64 accumulation).
template<typename ACC>
struct CoefBlock {
    ACC y[kMaxGramP * kMaxQ];
};

// out[j][r] = beta * out[j][r] + sum_{i < p} Y[i * q + j] * V[i][r]
// (accumulated in ACC; q <= kMaxQ).  R > 1: R consecutive rows per thread
// step with 16-byte loads and stores (N a multiple of R, 16-byte aligned
// vectors); R = 1 otherwise.  Y is read from the parameter bank with
// warp-uniform indices (broadcast).
template<typename TV, typename TO, typename ACC, int R>
__global__ void __launch_bounds__(256, sizeof(TV) == 4 ? 4 : 2) combine_kernel(const TV *__restrict__ V, int p,
                                                                              int64_t N,
                                                      const __grid_constant__ CoefBlock<ACC> Y, int q,
                                                      double beta, TO *__restrict__ out) {
    const ACC *sy = Y.y;
    const int64_t nu = N / R;
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < nu;
         u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = u * R;
        ACC acc[kMaxQ][R];
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
#pragma unroll
            for (int t = 0; t < R; ++t)
                acc[j][t] = 0;
        // Unrolled so several vectors' loads are in flight per thread (a
        // thread often handles a single row step).
#pragma unroll 8
        for (int i = 0; i < p; ++i) {
            TV v[R];
            load_rows<TV, R>(V + i * N + r, v);
#pragma unroll
            for (int j = 0; j < kMaxQ; ++j)
                if (j < q) {
                    const ACC y = sy[i * q + j];
#pragma unroll
                    for (int t = 0; t < R; ++t)
                        acc[j][t] += y * static_cast<ACC>(v[t]);
                }
        }
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
            if (j < q) {
                TO *o = out + j * N + r;
                TO w[R];
                if (beta == 0.0) {
#pragma unroll
                    for (int t = 0; t < R; ++t)
                        w[t] = static_cast<TO>(acc[j][t]);
                } else {
#pragma unroll
                    for (int t = 0; t < R; ++t)
                        w[t] = static_cast<TO>(static_cast<ACC>(beta) * static_cast<ACC>(o[t]) + acc[j][t]);
                }
                store_rows<TO, R>(o, w);
            }
    }
}

// R[j] = AX[j] - theta[j] X[j]; then, if precondition, R[j] /= (theta[j] - D)
// with |theta - D| floored at 1e-8 (Davidson's diagonal preconditioner).
// R[j] = AX[j] - theta[j] X[j].  FP32 vectors: theta is split into
// theta_hi + theta_lo (both FP32) and applied with two FMAs, so the result
// carries the FP32 rounding of AX and X only, with no FP64 arithmetic (which
// is scarce on this GPU).
// Ritz values of one launch (at most kMaxQ), passed as a kernel parameter.
struct Theta {
    double t[kMaxQ];
};

template<typename T>
__global__ void residual_kernel(const T *__restrict__ AX, const T *__restrict__ X, const __grid_constant__ Theta th,
                                int q, int64_t N, T *__restrict__ R) {
    const double *theta = th.t;
    if constexpr (sizeof(T) == 4) {
        float th_hi[kMaxQ], th_lo[kMaxQ];
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j) {
            const double t = (j < q) ? theta[j] : 0.0;
            th_hi[j] = static_cast<float>(t);
            th_lo[j] = static_cast<float>(t - static_cast<double>(th_hi[j]));
        }
        for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
             r += static_cast<int64_t>(gridDim.x) * blockDim.x)
#pragma unroll
            for (int j = 0; j < kMaxQ; ++j)
                if (j < q) {
                    const float x = X[j * N + r];
                    R[j * N + r] = fmaf(-th_lo[j], x, fmaf(-th_hi[j], x, AX[j * N + r]));
                }
    } else {
        for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
             r += static_cast<int64_t>(gridDim.x) * blockDim.x)
            for (int j = 0; j < q; ++j)
                R[j * N + r] = AX[j * N + r] - theta[j] * X[j * N + r];
    }
}

// Residual columns to precondition (at most kMaxQ) with their Ritz values,
// passed by value.
struct Cols {
    int n;
    int src[kMaxQ];
    double theta[kMaxQ];
};

// out[c] = R[j] / (theta[j] - D) for j = cols.src[c], with |theta - D|
// floored at 1e-8 (Davidson's diagonal preconditioner); one launch for the
// whole block of corrections.  FP32 output: the quotient is taken in FP32.
template<typename TI, typename TO>
__global__ void precondition_kernel(const TI *__restrict__ R, const double *__restrict__ diag,
                                    const __grid_constant__ Cols cols, int64_t N, TO *__restrict__ out) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double d = diag[r];
        if constexpr (sizeof(TO) == 4) {
            // FP32 corrections: the quotient in FP32 arithmetic (one FP64
            // conversion per row; this GPU's FP64 rate is a small fraction of
            // its FP32 rate, and a preconditioner needs no FP64 accuracy).
            const float df = static_cast<float>(d);
            for (int c = 0; c < cols.n; ++c) {
                const int j = cols.src[c];
                float den = static_cast<float>(cols.theta[c]) - df;
                if (fabsf(den) < 1e-8f)
                    den = (den < 0.0f) ? -1e-8f : 1e-8f;
                out[c * N + r] = static_cast<float>(R[j * N + r]) * __frcp_rn(den);
            }
        } else {
            for (int c = 0; c < cols.n; ++c) {
                const int j = cols.src[c];
                double den = cols.theta[c] - d;
                if (fabs(den) < 1e-8)
                    den = (den < 0.0) ? -1e-8 : 1e-8;
                out[c * N + r] = static_cast<TO>(static_cast<double>(R[j * N + r]) / den);
            }
        }
    }
}

// Fused Ritz step of the FP32 solve: one pass over the rows of V and W (m
// vectors each) for the Q Ritz pairs with coefficients Y (m x Q, row-major)
// and values theta:
//   X_j = sum_i Y[i][j] V_i, AX_j = sum_i Y[i][j] W_i   (combine_kernel's sums)
//   R_j = AX_j - theta_j X_j                            (residual_kernel's FMAs)
//   T_j = R_j / (theta_j - D), |.| floored at 1e-8      (precondition_kernel's quotient)
// T_j goes to T + j N.  Per block it writes the partial sums
//   partial[b][i Q + j]    = sum_r A_i[r] T_j[r],  A = [V_0 .. V_{m-1}, T_0 .. T_{Q-1}]
//   partial[b][MA Q + j]   = sum_r R_j[r]^2        (MA = m + Q <= kRitzMaxA)
// i.e. the residual norms and the first Gram product [V T]^T T of the block
// orthonormalisation, without a second read of V from memory: each 256-row
// tile's V and T rows are staged in shared memory (MA x 1 KB) and the Gram
// sums taken there, warp w owning the A rows w, w + 8, ..., lane l the tile
// rows l, l + 32, ...  Sums as in gram_rows_kernel: FP32 per thread and warp,
// FP64 across warps and blocks.
constexpr int kRitzTile = 256;
constexpr int kRitzRowsPerWarp = 9;
constexpr int kRitzMaxA = (kRitzTile / 32) * kRitzRowsPerWarp;
// Shared memory of a staged-tile kernel at most (the tiles' rows, 1 KB
// each; two buffers of them where they fit).
constexpr int kStagedMaxBytes = 220 * 1024;

// Bulk-copy staging of the tiles (BULK kernels, N a multiple of 4 so that
// every row range of every vector starts on 16 bytes): one mbarrier per
// block, armed with the tile's byte count by one lane; the lanes of warp 0
// issue one cp.async.bulk per vector (up to 1 KB each), so a whole tile is
// in flight at once.  Waits are bounded: a block that gives up writes NaN
// partial sums, which the host reports.
constexpr uint32_t kStageWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t stage_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void stage_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arms the barrier for `bytes` (after the generic-proxy accesses of the
// previous tile, which the block barrier before this call has ordered).
__device__ __forceinline__ void stage_arm(uint32_t bar, uint32_t bytes) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Rows [base, base + bytes / 4) of vectors src_0 .. src_{n-1} (stride N)
// into dst[i][0 ..), one bulk copy per vector, issued by the 32 lanes.
__device__ __forceinline__ void stage_rows(float *dst, const float *src, int n, int64_t N, int64_t base,
                                           uint32_t bytes, uint32_t bar, int lane) {
    for (int i = lane; i < n; i += 32)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         stage_addr(dst + i * kRitzTile)),
                     "l"(src + i * N + base), "r"(bytes), "r"(bar)
                     : "memory");
}

__device__ __forceinline__ bool stage_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kStageWaitLimit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok)
            return true;
    }
    return false;
}

// Gram sums of one staged tile: acc[ii][j] += sum over the lane's tile rows
// of A_i T_j, A = [Av_0 .. Av_{m-1}, At_0 .. At_{Q-1}] (i = warp + 8 ii < MA),
// T_j = At_j (rows of kRitzTile floats).  Lane l takes the rows
// 4 l .. 4 l + 3 and 128 + 4 l .. 128 + 4 l + 3 with 16-byte shared loads.
template<int Q, int RPW>
__device__ __forceinline__ void tile_gram(const float *Av, const float *At, int m, int MA, int warp, int lane,
                                          float (&acc)[RPW][Q]) {
#pragma unroll
    for (int h = 0; h < kRitzTile / 128; ++h) {
        const int c = 4 * lane + 128 * h;
        float4 tq[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j)
            tq[j] = *reinterpret_cast<const float4 *>(At + j * kRitzTile + c);
#pragma unroll
        for (int ii = 0; ii < RPW; ++ii) {
            const int i = warp + 8 * ii;
            if (i < MA) {
                const float4 a = *reinterpret_cast<const float4 *>(i < m ? Av + i * kRitzTile + c
                                                                         : At + (i - m) * kRitzTile + c);
#pragma unroll
                for (int j = 0; j < Q; ++j)
                    acc[ii][j] += a.x * tq[j].x + a.y * tq[j].y + a.z * tq[j].z + a.w * tq[j].w;
            }
        }
    }
}

// Warp sums of the Gram entries (each (i, j) belongs to one warp) to
// out[i Q + j].
template<int Q, int RPW>
__device__ __forceinline__ void write_gram(const float (&acc)[RPW][Q], int MA, int warp, int lane, double *out) {
#pragma unroll
    for (int ii = 0; ii < RPW; ++ii) {
        const int i = warp + 8 * ii;
        if (i < MA) {
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                float v = acc[ii][j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0)
                    out[i * Q + j] = static_cast<double>(v);
            }
        }
    }
}

// Tile t of a block (grid stride over 256-row tiles) and its row count.
__device__ __forceinline__ int64_t tile_base(int64_t t) {
    return (static_cast<int64_t>(blockIdx.x) + t * gridDim.x) * kRitzTile;
}

__device__ __forceinline__ int64_t block_tiles(int64_t N) {
    const int64_t all = (N + kRitzTile - 1) / kRitzTile;
    return all > blockIdx.x ? (all - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
}

// Bulk-copy staging with `stages` (1 or 2) buffers per block: tile t goes
// to buffer t % stages and is waited for with parity (t / stages) & 1; the
// copies of tile t + stages are issued once tile t's buffer is free, so with
// two buffers the next tile lands while this one is computed.  Each
// buffer holds the rows of two vector sets (n1 and n2 vectors).
struct StagedTiles {
    float *buf;          // buffer s at buf + s * (n1 + n2) * kRitzTile
    uint64_t *bars;      // one mbarrier per buffer
    int stages, n1, n2;
    const float *src1, *src2;
    int64_t N;
    __device__ float *set1(int s) const { return buf + static_cast<size_t>(s) * (n1 + n2) * kRitzTile; }
    __device__ float *set2(int s) const { return set1(s) + static_cast<size_t>(n1) * kRitzTile; }
    // Warp 0 only.
    __device__ void issue(int64_t t, int lane) const {
        const int s = static_cast<int>(t % stages);
        const int64_t base = tile_base(t);
        const int rows = static_cast<int>(N - base < kRitzTile ? N - base : kRitzTile);
        const uint32_t bytes = static_cast<uint32_t>(rows) * 4u, bar = stage_addr(&bars[s]);
        if (lane == 0)
            stage_arm(bar, static_cast<uint32_t>(n1 + n2) * bytes);
        __syncwarp();
        stage_rows(set1(s), src1, n1, N, base, bytes, bar, lane);
        stage_rows(set2(s), src2, n2, N, base, bytes, bar, lane);
    }
    __device__ bool wait(int64_t t) const {
        return stage_wait(stage_addr(&bars[t % stages]), static_cast<uint32_t>((t / stages) & 1));
    }
};

template<int Q, bool BULK, int RPW>
__global__ void __launch_bounds__(kRitzTile, RPW <= 5 ? 3 : 2) ritz_fused_kernel(const float *__restrict__ V,
                                                                  const float *__restrict__ W, int m, int64_t N,
                                                                  const __grid_constant__ CoefBlock<float> Y,
                                                                  const __grid_constant__ Theta th,
                                                                  const double *__restrict__ diag,
                                                                  float *__restrict__ T, double *__restrict__ partial,
                                                                  int stages) {
    // T rows [Q][kRitzTile], then V rows [m][kRitzTile] (register loads), or
    // `stages` buffers of V and W rows (bulk copies).
    extern __shared__ __align__(16) float sm[];
    __shared__ __align__(8) uint64_t bars[2];
    const int MA = m + Q;
    float *Tt = sm;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t pq = static_cast<int64_t>(MA) * Q + Q;
    double *out = partial + static_cast<int64_t>(blockIdx.x) * pq;
    float th_hi[Q], th_lo[Q], nrm[Q], acc[RPW][Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        th_hi[j] = static_cast<float>(th.t[j]);
        th_lo[j] = static_cast<float>(th.t[j] - static_cast<double>(th_hi[j]));
        nrm[j] = 0.0f;
#pragma unroll
        for (int ii = 0; ii < RPW; ++ii)
            acc[ii][j] = 0.0f;
    }
    const StagedTiles st{sm + Q * kRitzTile, bars, stages, m, m, V, W, N};
    const int64_t ntile = block_tiles(N);
    if constexpr (BULK) {
        if (tid < stages)
            stage_init(stage_addr(&bars[tid]));
        __syncthreads();
        if (warp == 0)
            for (int64_t t = 0; t < stages && t < ntile; ++t)
                st.issue(t, lane);
    }
    bool failed = false;
    int64_t t = 0;
    for (; t < ntile; ++t) {
        const int64_t base = tile_base(t);
        const int rows = static_cast<int>(N - base < kRitzTile ? N - base : kRitzTile);
        const int64_t r = base + tid;
        const bool ok = tid < rows;
        const int s = BULK ? static_cast<int>(t % stages) : 0;
        float *Vs = BULK ? st.set1(s) : sm + Q * kRitzTile;
        float *Ws = st.set2(s);
        // The diagonal before the tile's wait: its memory latency overlaps
        // the copies instead of following them.
        const float df = ok ? static_cast<float>(diag[r]) : 0.0f;
        if constexpr (BULK) {
            if (__syncthreads_or(!st.wait(t))) {
                failed = true;
                break;
            }
            // Rows past N (last tile): zeros in this thread's own staged
            // column (the copy left it), so the loop reads without a test
            // and the Gram sums see zeros.
            if (!ok)
                for (int i = 0; i < m; ++i)
                    Vs[i * kRitzTile + tid] = Ws[i * kRitzTile + tid] = 0.0f;
        }
        float x[Q], ax[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j)
            x[j] = ax[j] = 0.0f;
#pragma unroll 8
        for (int i = 0; i < m; ++i) {
            float v, w;
            if constexpr (BULK) {
                v = Vs[i * kRitzTile + tid];
                w = Ws[i * kRitzTile + tid];
            } else {
                v = ok ? V[i * N + r] : 0.0f;
                w = ok ? W[i * N + r] : 0.0f;
                Vs[i * kRitzTile + tid] = v;
            }
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const float y = Y.y[i * Q + j];
                x[j] += y * v;
                ax[j] += y * w;
            }
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float res = fmaf(-th_lo[j], x[j], fmaf(-th_hi[j], x[j], ax[j]));
            nrm[j] += res * res;
            float den = th_hi[j] - df;
            if (fabsf(den) < 1e-8f)
                den = (den < 0.0f) ? -1e-8f : 1e-8f;
            const float tv = res * __frcp_rn(den);
            Tt[j * kRitzTile + tid] = ok ? tv : 0.0f;
            if (ok)
                T[j * N + r] = tv;
        }
        __syncthreads();
        tile_gram<Q, RPW>(Vs, Tt, m, MA, warp, lane, acc);
        __syncthreads();
        if constexpr (BULK) {
            if (warp == 0 && t + stages < ntile)
                st.issue(t + stages, lane);
        }
    }
    if constexpr (BULK) {
        if (failed) {
            // Let the copies in flight land (bounded), then report through
            // NaN sums.
            for (int64_t u = t; u < t + stages && u < ntile; ++u)
                st.wait(u);
            for (int64_t e = tid; e < pq; e += kRitzTile)
                out[e] = __longlong_as_double(0x7ff8000000000000LL);
            return;
        }
    }
    write_gram<Q, RPW>(acc, MA, warp, lane, out);
    // Residual norms: warp sums in FP32, then the 8 warps in FP64 (the T
    // rows are free after the last tile's barrier).
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        float v = nrm[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0)
            Tt[warp * Q + j] = v;
    }
    __syncthreads();
    if (tid < Q) {
        double sum = 0.0;
        for (int w = 0; w < kRitzTile / 32; ++w)
            sum += static_cast<double>(Tt[w * Q + tid]);
        out[static_cast<int64_t>(MA) * Q + tid] = sum;
    }
}

// First Gram-Schmidt pass of a block orthonormalisation fused with the
// Gram product of the second: for c < Q
//   T1_c = sum_{i < m} Y[i][c] V_i + sum_{a < b} Y[m + a][c] Tsrc_a
// (combine2_kernel's sums) to out + c N, and per block
//   partial[b][i Q + c] = sum_r A_i[r] T1_c[r],  A = [V_0 .. V_{m-1}, T1_0 .. T1_{Q-1}]
// with the tile staging of ritz_fused_kernel (V read once).
template<int Q, bool BULK, int RPW>
__global__ void __launch_bounds__(kRitzTile, RPW <= 5 ? 3 : 2) project_gram_kernel(const float *__restrict__ V, int m,
                                                                    const float *__restrict__ Tsrc, int b, int64_t N,
                                                                    const __grid_constant__ CoefBlock<float> Y,
                                                                    float *__restrict__ out,
                                                                    double *__restrict__ partial, int stages) {
    // T1 rows [Q][kRitzTile], then V rows [m][kRitzTile] (register loads),
    // or `stages` buffers of V and Tsrc rows (bulk copies).
    extern __shared__ __align__(16) float sm[];
    __shared__ __align__(8) uint64_t bars[2];
    const int MA = m + Q;
    float *Tt = sm;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double *pout = partial + static_cast<int64_t>(blockIdx.x) * MA * Q;
    float acc[RPW][Q];
#pragma unroll
    for (int ii = 0; ii < RPW; ++ii)
#pragma unroll
        for (int j = 0; j < Q; ++j)
            acc[ii][j] = 0.0f;
    const StagedTiles st{sm + Q * kRitzTile, bars, stages, m, b, V, Tsrc, N};
    const int64_t ntile = block_tiles(N);
    if constexpr (BULK) {
        if (tid < stages)
            stage_init(stage_addr(&bars[tid]));
        __syncthreads();
        if (warp == 0)
            for (int64_t t = 0; t < stages && t < ntile; ++t)
                st.issue(t, lane);
    }
    bool failed = false;
    int64_t t = 0;
    for (; t < ntile; ++t) {
        const int64_t base = tile_base(t);
        const int rows = static_cast<int>(N - base < kRitzTile ? N - base : kRitzTile);
        const int64_t r = base + tid;
        const bool ok = tid < rows;
        const int s = BULK ? static_cast<int>(t % stages) : 0;
        float *Vs = BULK ? st.set1(s) : sm + Q * kRitzTile;
        float *Ts = st.set2(s);
        if constexpr (BULK) {
            if (__syncthreads_or(!st.wait(t))) {
                failed = true;
                break;
            }
            if (!ok) {
                for (int i = 0; i < m; ++i)
                    Vs[i * kRitzTile + tid] = 0.0f;
                for (int a = 0; a < b; ++a)
                    Ts[a * kRitzTile + tid] = 0.0f;
            }
        }
        float t1[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j)
            t1[j] = 0.0f;
#pragma unroll 8
        for (int i = 0; i < m; ++i) {
            float v;
            if constexpr (BULK) {
                v = Vs[i * kRitzTile + tid];
            } else {
                v = ok ? V[i * N + r] : 0.0f;
                Vs[i * kRitzTile + tid] = v;
            }
#pragma unroll
            for (int j = 0; j < Q; ++j)
                t1[j] += Y.y[i * Q + j] * v;
        }
        for (int a = 0; a < b; ++a) {
            float v;
            if constexpr (BULK)
                v = Ts[a * kRitzTile + tid];
            else
                v = ok ? Tsrc[a * N + r] : 0.0f;
#pragma unroll
            for (int j = 0; j < Q; ++j)
                t1[j] += Y.y[(m + a) * Q + j] * v;
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            Tt[j * kRitzTile + tid] = t1[j];
            if (ok)
                out[j * N + r] = t1[j];
        }
        __syncthreads();
        tile_gram<Q, RPW>(Vs, Tt, m, MA, warp, lane, acc);
        __syncthreads();
        if constexpr (BULK) {
            if (warp == 0 && t + stages < ntile)
                st.issue(t + stages, lane);
        }
    }
    if constexpr (BULK) {
        if (failed) {
            for (int64_t u = t; u < t + stages && u < ntile; ++u)
                st.wait(u);
            for (int64_t e = tid; e < static_cast<int64_t>(MA) * Q; e += kRitzTile)
                pout[e] = __longlong_as_double(0x7ff8000000000000LL);
            return;
        }
    }
    write_gram<Q, RPW>(acc, MA, warp, lane, pout);
}

// out[j][r] = sum_{i < p1} Y[i][j] V1[i][r] + sum_{i < p2} Y[p1 + i][j] V2[i][r]
// for j < q (FP32, i ascending: combine_kernel's sums over the two vector
// sets as one); when xi is given, the same values also go to xi[r kp + j]
// (zero for q <= j < kp), the packed operand of the next product
// (pack_kernel's layout).  out must not overlap V1 or V2.  R = 4: four
// consecutive rows per thread step with 16-byte loads and stores (N a
// multiple of 4, 16-byte aligned vectors); R = 1 otherwise.
template<int R>
__global__ void __launch_bounds__(256, 2) combine2_kernel(const float *__restrict__ V1, int p1,
                                                          const float *__restrict__ V2, int p2, int64_t N,
                                                          const __grid_constant__ CoefBlock<float> Y, int q,
                                                          float *__restrict__ out, float *__restrict__ xi, int kp) {
    const int p = p1 + p2;
    const int64_t nu = N / R;
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < nu;
         u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = u * R;
        float acc[kMaxQ][R];
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
#pragma unroll
            for (int t = 0; t < R; ++t)
                acc[j][t] = 0.0f;
#pragma unroll 8
        for (int i = 0; i < p; ++i) {
            const float *src = (i < p1) ? V1 + i * N : V2 + (i - p1) * N;
            float v[R];
            load_rows<float, R>(src + r, v);
#pragma unroll
            for (int j = 0; j < kMaxQ; ++j)
                if (j < q) {
                    const float y = Y.y[i * q + j];
#pragma unroll
                    for (int t = 0; t < R; ++t)
                        acc[j][t] += y * v[t];
                }
        }
#pragma unroll
        for (int j = 0; j < kMaxQ; ++j)
            if (j < q) {
                float w[R];
#pragma unroll
                for (int t = 0; t < R; ++t)
                    w[t] = acc[j][t];
                store_rows<float, R>(out + j * N + r, w);
            }
        if (xi) {
#pragma unroll
            for (int t = 0; t < R; ++t) {
                float *row = xi + (r + t) * kp;
                if (kp % 4 == 0) {
#pragma unroll
                    for (int j4 = 0; j4 < kMaxQ; j4 += 4)
                        if (j4 < kp)
                            *reinterpret_cast<float4 *>(row + j4) =
                                make_float4(j4 < q ? acc[j4][t] : 0.0f, j4 + 1 < q ? acc[j4 + 1][t] : 0.0f,
                                            j4 + 2 < q ? acc[j4 + 2][t] : 0.0f, j4 + 3 < q ? acc[j4 + 3][t] : 0.0f);
                } else {
#pragma unroll
                    for (int j = 0; j < kMaxQ; ++j)
                        if (j < kp)
                            row[j] = j < q ? acc[j][t] : 0.0f;
                }
            }
        }
    }
}

// L^{-1} (row-major, lower) for the Cholesky factor S = L L^T of a k x k
// symmetric matrix (row-major); false when a pivot is not above tol times its
// diagonal entry (S not safely positive definite).
inline bool cholesky_inverse(const std::vector<double> &S, int k, double tol, std::vector<double> &Linv) {
    std::vector<double> L(static_cast<size_t>(k) * k, 0.0);
    for (int j = 0; j < k; ++j) {
        double d = S[static_cast<size_t>(j) * k + j];
        for (int t = 0; t < j; ++t)
            d -= L[static_cast<size_t>(j) * k + t] * L[static_cast<size_t>(j) * k + t];
        if (!(d > tol * S[static_cast<size_t>(j) * k + j]) || !(d > 0.0))
            return false;
        L[static_cast<size_t>(j) * k + j] = std::sqrt(d);
        for (int i = j + 1; i < k; ++i) {
            double x = S[static_cast<size_t>(i) * k + j];
            for (int t = 0; t < j; ++t)
                x -= L[static_cast<size_t>(i) * k + t] * L[static_cast<size_t>(j) * k + t];
            L[static_cast<size_t>(i) * k + j] = x / L[static_cast<size_t>(j) * k + j];
        }
    }
    Linv.assign(static_cast<size_t>(k) * k, 0.0);
    for (int j = 0; j < k; ++j) {
        Linv[static_cast<size_t>(j) * k + j] = 1.0 / L[static_cast<size_t>(j) * k + j];
        for (int i = j + 1; i < k; ++i) {
            double x = 0.0;
            for (int t = j; t < i; ++t)
                x -= L[static_cast<size_t>(i) * k + t] * Linv[static_cast<size_t>(t) * k + j];
            Linv[static_cast<size_t>(i) * k + j] = x / L[static_cast<size_t>(i) * k + i];
        }
    }
    return true;
}

// Columns todo[c0 .. c0 + kMaxQ) of a correction list, with their Ritz values.
inline Cols make_cols(const std::vector<int> &todo, size_t c0, const std::vector<double> &theta) {
    Cols c{};
    c.n = static_cast<int>(std::min<size_t>(kMaxQ, todo.size() - c0));
    for (int i = 0; i < c.n; ++i) {
        c.src[i] = todo[c0 + i];
        c.theta[i] = theta[todo[c0 + i]];
    }
    return c;
}

template<typename T>
__global__ void scale_kernel(T *v, int64_t N, double s) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        v[r] = static_cast<T>(static_cast<double>(v[r]) * s);
}

template<typename TI, typename TO>
__global__ void convert_kernel(const TI *__restrict__ in, TO *__restrict__ out, int64_t n) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[r] = static_cast<TO>(in[r]);
}

// V[j] = unit vector e_{idx[j]}.
template<typename T>
__global__ void unit_kernel(T *V, int64_t N, const int64_t *idx, int k) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        for (int j = 0; j < k; ++j)
            V[j * N + r] = (r == idx[j]) ? T(1) : T(0);
}

// Arg-min of (d[r], r) over the rows whose pair is above *prev (pairs
// ordered by value, then row; all rows when prev is null), as (key, row) in
// a longlong2 per block ((LLONG_MAX, -1) when a block has no candidate);
// argmin_final_kernel reduces the blocks.  The comparisons run on an
// order-preserving integer key of the value (sign-magnitude bits mapped to
// two's complement, -0 as +0): no FP64 instruction, whose rate on this GPU
// would bound the pass rather than its bytes.
__device__ __forceinline__ long long order_key(double v) {
    long long b = __double_as_longlong(v);
    if (b == static_cast<long long>(0x8000000000000000ULL))
        b = 0;
    return b >= 0 ? b : b ^ 0x7FFFFFFFFFFFFFFFLL;
}

__device__ __forceinline__ bool pair_less(long long ka, long long ia, long long kb, long long ib) {
    return ka < kb || (ka == kb && ia < ib);
}

__device__ __forceinline__ void pair_min_block(long long &v, long long &i) {
    __shared__ long long sv[32], si[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long ov = __shfl_xor_sync(0xffffffffu, v, o), oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (pair_less(ov, oi, v, i))
            v = ov, i = oi;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
        sv[w] = v, si[w] = i;
    __syncthreads();
    if (w == 0) {
        v = lane < static_cast<int>(blockDim.x >> 5) ? sv[lane] : LLONG_MAX;
        i = lane < static_cast<int>(blockDim.x >> 5) ? si[lane] : -1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long ov = __shfl_xor_sync(0xffffffffu, v, o), oi = __shfl_xor_sync(0xffffffffu, i, o);
            if (pair_less(ov, oi, v, i))
                v = ov, i = oi;
        }
    }
}

__global__ void argmin_above_kernel(const double *__restrict__ d, int64_t N, const longlong2 *prev,
                                    longlong2 *__restrict__ partial) {
    const long long lv = prev ? prev->x : LLONG_MIN, li = prev ? prev->y : -1;
    long long bv = LLONG_MAX, bi = -1;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    for (; r + 3 * stride < N; r += 4 * stride) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            v[u] = __ldg(d + r + u * stride);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long kv = order_key(v[u]), ri = r + u * stride;
            if (pair_less(lv, li, kv, ri) && pair_less(kv, ri, bv, bi))
                bv = kv, bi = ri;
        }
    }
    for (; r < N; r += stride) {
        const long long kv = order_key(d[r]), ri = r;
        if (pair_less(lv, li, kv, ri) && pair_less(kv, ri, bv, bi))
            bv = kv, bi = ri;
    }
    pair_min_block(bv, bi);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = make_longlong2(bv, bi);
}

__global__ void argmin_final_kernel(const longlong2 *__restrict__ partial, int nb, longlong2 *out) {
    long long bv = LLONG_MAX, bi = -1;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const longlong2 p = partial[b];
        if (p.y >= 0 && pair_less(p.x, p.y, bv, bi))
            bv = p.x, bi = p.y;
    }
    pair_min_block(bv, bi);
    if (threadIdx.x == 0)
        *out = make_longlong2(bv, bi);
}

// v = e_idx + amp * noise(., col): one perturbed start vector.
template<typename T>
__global__ void guess_kernel(T *v, int64_t N, int64_t idx, double amp, int col) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        v[r] = static_cast<T>((r == idx ? 1.0 : 0.0) + amp * guess_noise(static_cast<uint64_t>(r), static_cast<uint64_t>(col)));
}

// ------------------------------------------------------------------------

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    double total_ms = 0.0;
};

template<typename T>
class Davidson {
public:
    // nroot: block size (Ritz pairs tracked); nwant <= nroot: roots that must
    // converge and are returned (the rest are buffer vectors).
    Davidson(pyci_gpu_csr *csr, int64_t nroot, int64_t nwant, int64_t mmax, bool mixed)
        : csr_(csr), st_(csr->ctx->stream), N_(csr->nrow), nroot_(nroot), nwant_(nwant), mmax_(mmax),
          mixed_(mixed) {
        // PYCI_GPU_FP64_PRODUCT=native keeps FP64 arithmetic in the FP64
        // solve's products even when the split is there.
        const char *e = std::getenv("PYCI_GPU_FP64_PRODUCT");
        fp64_df_ = !mixed && ((csr->hi && csr->lo) || has_implicit(csr)) && !csr->lower_only &&
                   !(e && !std::strcmp(e, "native"));
        // PYCI_GPU_FP64_LINALG=native keeps FP64 arithmetic in the FP64
        // Gram products and combinations (double-float by default).
        const char *l = std::getenv("PYCI_GPU_FP64_LINALG");
        df_linalg_ = !(l && !std::strcmp(l, "native"));
        const char *f = std::getenv("PYCI_GPU_RITZ");
        ritz_fused_ = !(f && !std::strcmp(f, "separate"));
    }

    ~Davidson() {
        for (void *p : allocs_)
            cudaFreeAsync(p, st_);
        for (auto &pr : timers_) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
        cudaStreamSynchronize(st_);
        if (holds_ctx_buffer_)
            csr_->ctx->mapped_busy = false;
        else if (h_small_)
            cudaFreeHost(h_small_);
    }

    int run(const double *c0, int64_t maxiter, double tol, double ecore, double *evals, double *evecs,
            pyci_gpu_solve_stats *stats);

private:
    template<typename U>
    int alloc(U **p, int64_t n) {
        void *q = nullptr;
        const auto t0 = std::chrono::steady_clock::now();
        cudaError_t e = cudaMallocAsync(&q, sizeof(U) * std::max<int64_t>(n, 1), st_);
        alloc_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (e != cudaSuccess)
            return cuda_status(e, "cudaMallocAsync (eigensolver workspace)");
        allocs_.push_back(q);
        *p = static_cast<U *>(q);
        return PYCI_GPU_OK;
    }

    unsigned grid(int64_t n) const {
        const int64_t want = (n + 255) / 256;
        return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(want, csr_->ctx->num_sms * 8)));
    }

    // C (p x q, row-major, host) = A^T B for vector sets A (p) and B (q).
    template<typename U>
    int gram(const U *A, int p, const U *B, int q, std::vector<double> &C) {
        C.assign(static_cast<size_t>(p) * q, 0.0);
        for (int i0 = 0; i0 < p; i0 += kMaxGramP) {
            const int pp = std::min(kMaxGramP, p - i0);
            for (int j0 = 0; j0 < q; j0 += kMaxQ) {
                const int qq = std::min(kMaxQ, q - j0);
                const U *Ai = A + static_cast<int64_t>(i0) * N_;
                const U *Bj = B + static_cast<int64_t>(j0) * N_;
                unsigned nb;
                bool on_tc = false;
                if constexpr (std::is_same<U, float>::value) {
                    on_tc = gram_tc_enabled() && pp >= kGramTcMinP;
                }
                const int trg = tr_open(kTrGram);
                if (on_tc) {
                    nb = launch_gram_tc(gram_blocks_, st_, reinterpret_cast<const float *>(Ai), pp,
                                        reinterpret_cast<const float *>(Bj), qq, N_, d_partial_);
                } else if (std::is_same<U, double>::value && df_linalg_) {
                    nb = launch_gram_df(gram_blocks_, st_, reinterpret_cast<const double *>(Ai), pp,
                                        reinterpret_cast<const double *>(Bj), qq, N_, d_partial_);
                    ::pyci_gpu::note_launch();
                } else {
                    nb = launch_gram_rows<U>(gram_blocks_, st_, Ai, pp, Bj, qq, N_, d_partial_);
                    ::pyci_gpu::note_launch();
                }
                // Sums straight into the mapped pinned buffer when the
                // device can write host memory (no copy in the stream).
                reduce_partials_kernel<<<pp * qq, 256, 0, st_>>>(d_partial_, nb, pp * qq,
                                                                 d_mapped_ ? d_mapped_ : d_small_),
                    ::pyci_gpu::note_launch();
                tr_close(trg);
                // Otherwise read back through the pinned buffer: one DMA,
                // then one synchronisation (a pageable copy would block
                // inside the copy call instead).
                const auto t0 = std::chrono::steady_clock::now();
                cudaError_t e = cudaSuccess;
                if (!d_mapped_)
                    e = cudaMemcpyAsync(h_small_, d_small_, sizeof(double) * pp * qq, cudaMemcpyDeviceToHost, st_);
                if (e != cudaSuccess)
                    return cuda_status(e, "gram copy");
                const int trs = tr_open(kTrSync);
                e = cudaStreamSynchronize(st_);
                tr_close(trs);
                wait_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                ++syncs_;
                if (e != cudaSuccess)
                    return cuda_status(e, "gram");
                const double *tmp = h_small_;
                if (on_tc) {
                    for (int e2 = 0; e2 < pp * qq; ++e2)
                        if (!std::isfinite(tmp[e2]) && gram_tc_error(true)) {
                            set_error("tensor-core Gram product: MMA completion wait timed out");
                            return PYCI_GPU_ECUDA;
                        }
                }
                for (int i = 0; i < pp; ++i)
                    for (int j = 0; j < qq; ++j)
                        C[static_cast<size_t>(i0 + i) * q + j0 + j] = tmp[static_cast<size_t>(i) * qq + j];
            }
        }
        return PYCI_GPU_OK;
    }

    // out[j] = beta out[j] + sum_i Y[i][j] V[i]  (Y host, p x q row-major).
    template<typename TV, typename TO, typename ACC>
    int combine(const TV *V, int p, const std::vector<double> &Y, int q, double beta, TO *out) {
        if constexpr (std::is_same<TV, double>::value && std::is_same<TO, double>::value &&
                      std::is_same<ACC, double>::value) {
            if (df_linalg_)
                return combine_df(V, p, Y, q, beta, out);
        }
        const int trk = tr_open(kTrCombine);
        struct Close {
            Davidson *d;
            int h;
            ~Close() { d->tr_close(h); }
        } close{this, trk};
        for (int j0 = 0; j0 < q; j0 += kMaxQ) {
            const int qq = std::min(kMaxQ, q - j0);
            for (int i0 = 0; i0 < p; i0 += kMaxGramP) {
                const int pp = std::min(kMaxGramP, p - i0);
                CoefBlock<ACC> sub;
                for (int i = 0; i < pp; ++i)
                    for (int j = 0; j < qq; ++j)
                        sub.y[i * qq + j] = static_cast<ACC>(Y[static_cast<size_t>(i0 + i) * q + j0 + j]);
                const TV *Vi = V + static_cast<int64_t>(i0) * N_;
                TO *Oj = out + static_cast<int64_t>(j0) * N_;
                const double bt = (i0 == 0) ? beta : 1.0;
                constexpr int R = 16 / sizeof(TV);
                if (N_ % R == 0 && reinterpret_cast<uintptr_t>(Vi) % 16 == 0 &&
                    reinterpret_cast<uintptr_t>(Oj) % 16 == 0)
                    combine_kernel<TV, TO, ACC, R><<<grid(N_ / R), 256, 0, st_>>>(Vi, pp, N_, sub, qq, bt, Oj);
                else
                    combine_kernel<TV, TO, ACC, 1><<<grid(N_), 256, 0, st_>>>(Vi, pp, N_, sub, qq, bt, Oj);
                ::pyci_gpu::note_launch();
            }
        }
        return PYCI_GPU_OK;
    }

    // combine<double, double, double> in double-float arithmetic
    // (combine_df_kernel).
    int combine_df(const double *V, int p, const std::vector<double> &Y, int q, double beta, double *out) {
        const int trk = tr_open(kTrCombine);
        struct Close {
            Davidson *d;
            int h;
            ~Close() { d->tr_close(h); }
        } close{this, trk};
        for (int j0 = 0; j0 < q; j0 += kMaxQ) {
            const int qq = std::min(kMaxQ, q - j0);
            for (int i0 = 0; i0 < p; i0 += kMaxGramP) {
                const int pp = std::min(kMaxGramP, p - i0);
                CoefBlockDF sub;
                for (int i = 0; i < pp; ++i)
                    for (int j = 0; j < qq; ++j)
                        split_hi_lo(Y[static_cast<size_t>(i0 + i) * q + j0 + j], sub.h[i * qq + j], sub.l[i * qq + j]);
                const double *Vi = V + static_cast<int64_t>(i0) * N_;
                double *Oj = out + static_cast<int64_t>(j0) * N_;
                const double bt = (i0 == 0) ? beta : 1.0;
                if (N_ % 2 == 0 && reinterpret_cast<uintptr_t>(Vi) % 16 == 0 && reinterpret_cast<uintptr_t>(Oj) % 16 == 0)
                    combine_df_kernel<2><<<grid(N_ / 2), 256, 0, st_>>>(Vi, pp, N_, sub, qq, bt, Oj);
                else
                    combine_df_kernel<1><<<grid(N_), 256, 0, st_>>>(Vi, pp, N_, sub, qq, bt, Oj);
                ::pyci_gpu::note_launch();
            }
        }
        return PYCI_GPU_OK;
    }

    // Staged-tile kernels (ritz_fused_kernel, project_gram_kernel), by
    // Q - 1 and by BULK (bulk-copy staging when N is a multiple of 4).
    using RitzFn = void (*)(const float *, const float *, int, int64_t, CoefBlock<float>, Theta, const double *,
                            float *, double *, int);
    using ProjectFn = void (*)(const float *, int, const float *, int, int64_t, CoefBlock<float>, float *, double *,
                               int);
    // Rows of [V T] per warp in the Gram sums: 5 (MA <= 40 and at most 5
    // pairs: three blocks per SM in 80 registers) or 9.
    static int staged_rpw(int MA, int q) { return (MA <= 40 && q <= 5) ? 5 : kRitzRowsPerWarp; }
#define PYCI_STAGED_TABLE(K, B, R)                                                                                  \
    { K<1, B, R>, K<2, B, R>, K<3, B, R>, K<4, B, R>, K<5, B, R>, K<6, B, R>, K<7, B, R>, K<8, B, R> }
    static RitzFn ritz_fn(int q, bool bulk, int rpw) {
        static const RitzFn f[2][2][kMaxQ] = {
            {PYCI_STAGED_TABLE(ritz_fused_kernel, false, 5), PYCI_STAGED_TABLE(ritz_fused_kernel, false, 9)},
            {PYCI_STAGED_TABLE(ritz_fused_kernel, true, 5), PYCI_STAGED_TABLE(ritz_fused_kernel, true, 9)}};
        return f[bulk ? 1 : 0][rpw <= 5 ? 0 : 1][q - 1];
    }
    static ProjectFn project_fn(int q, bool bulk, int rpw) {
        static const ProjectFn f[2][2][kMaxQ] = {
            {PYCI_STAGED_TABLE(project_gram_kernel, false, 5), PYCI_STAGED_TABLE(project_gram_kernel, false, 9)},
            {PYCI_STAGED_TABLE(project_gram_kernel, true, 5), PYCI_STAGED_TABLE(project_gram_kernel, true, 9)}};
        return f[bulk ? 1 : 0][rpw <= 5 ? 0 : 1][q - 1];
    }
#undef PYCI_STAGED_TABLE
    // The shared-memory limit of every staged-tile kernel, set once.
    static void staged_attributes() {
        static const bool done = [] {
            for (int bulk = 0; bulk < 2; ++bulk)
                for (int rpw : {5, kRitzRowsPerWarp})
                    for (int q = 1; q <= kMaxQ; ++q) {
                        cudaFuncSetAttribute(ritz_fn(q, bulk, rpw), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kStagedMaxBytes);
                        cudaFuncSetAttribute(project_fn(q, bulk, rpw), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kStagedMaxBytes);
                    }
            return true;
        }();
        (void)done;
    }

    // Blocks for a staged-tile kernel with `smem` bytes of tiles: the
    // resident blocks of one wave, at most gram_blocks_ (the partial sums'
    // rows).
    unsigned staged_grid(const void *fn, size_t smem) const {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kRitzTile, smem) != cudaSuccess)
            per_sm = 1;
        per_sm = std::max(1, per_sm);
        return static_cast<unsigned>(std::max<int64_t>(
            1, std::min<int64_t>({static_cast<int64_t>(gram_blocks_), static_cast<int64_t>(per_sm) * csr_->ctx->num_sms,
                                  (N_ + kRitzTile - 1) / kRitzTile})));
    }

    // Sums the nb blocks' pq partial sums and reads them back (one host
    // synchronisation).
    int read_partials(unsigned nb, int pq, std::vector<double> &h, const char *what) {
        reduce_partials_kernel<<<pq, 256, 0, st_>>>(d_partial_, nb, pq, d_mapped_ ? d_mapped_ : d_small_),
            ::pyci_gpu::note_launch();
        const auto t0 = std::chrono::steady_clock::now();
        cudaError_t e = cudaSuccess;
        if (!d_mapped_)
            e = cudaMemcpyAsync(h_small_, d_small_, sizeof(double) * pq, cudaMemcpyDeviceToHost, st_);
        const int trs = tr_open(kTrSync);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st_);
        tr_close(trs);
        wait_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        ++syncs_;
        if (e != cudaSuccess)
            return cuda_status(e, what);
        h.assign(h_small_, h_small_ + pq);
        return PYCI_GPU_OK;
    }

    // Fused Ritz step (ritz_fused_kernel, FP32 vectors): Tb[0..q) = the
    // preconditioned residuals of the q Ritz pairs with coefficients Yb
    // (m x q) and values theta; P = [V Tb]^T Tb ((m + q) x q, row-major);
    // rn2 = squared residual norms.  One host synchronisation.
    int ritz_fused(const float *V, const float *W, int m, const std::vector<double> &Yb, int q,
                   const std::vector<double> &theta, const double *diag, float *Tb, std::vector<double> &P,
                   std::vector<double> &rn2) {
        staged_attributes();
        CoefBlock<float> y;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < q; ++j)
                y.y[i * q + j] = static_cast<float>(Yb[static_cast<size_t>(i) * q + j]);
        Theta th{};
        for (int j = 0; j < q; ++j)
            th.t[j] = theta[j];
        const int MA = m + q;
        // Bulk copies when every row range starts on 16 bytes; one buffer
        // (two buffers, one block per SM, took 1.6x as long on a 10.5M-row
        // subspace: the tile arithmetic, not the copies, bounds this kernel,
        // and it needs the blocks).
        const bool bulk = N_ % 4 == 0;
        const size_t row = sizeof(float) * kRitzTile;
        const int stages = 1;
        const size_t smem = row * (bulk ? q + stages * 2 * m : q + m);
        const RitzFn fn = ritz_fn(q, bulk, staged_rpw(MA, q));
        const unsigned nb = staged_grid(reinterpret_cast<const void *>(fn), smem);
        const int trk = tr_open(kTrRitz);
        fn<<<nb, kRitzTile, smem, st_>>>(V, W, m, N_, y, th, diag, Tb, d_partial_, stages);
        ::pyci_gpu::note_launch();
        tr_close(trk);
        std::vector<double> h;
        const int pq = MA * q + q;
        int rc = read_partials(nb, pq, h, "fused Ritz step");
        if (rc)
            return rc;
        for (double v : h)
            if (!std::isfinite(v)) {
                set_error("fused Ritz step: non-finite sums (a staged-tile wait timed out, or non-finite vectors)");
                return PYCI_GPU_ECUDA;
            }
        P.assign(h.begin(), h.begin() + static_cast<size_t>(MA) * q);
        rn2.assign(h.begin() + static_cast<size_t>(MA) * q, h.end());
        return PYCI_GPU_OK;
    }

    // T1 = [V Tsrc] Y (project_gram_kernel; V: m vectors, Tsrc: b, Y
    // (m + b) x k row-major, k <= kMaxQ) into out; P = [V T1]^T T1
    // ((m + k) x k).  One host synchronisation.
    int project_gram(const float *V, int m, const float *Tsrc, int b, const CoefBlock<float> &y, int k, float *out,
                     std::vector<double> &P) {
        staged_attributes();
        const int MA = m + k;
        const bool bulk = N_ % 4 == 0;
        const size_t row = sizeof(float) * kRitzTile;
        const int stages = 1;
        const size_t smem = row * (bulk ? k + stages * (m + b) : k + m);
        const ProjectFn fn = project_fn(k, bulk, staged_rpw(MA, k));
        const unsigned nb = staged_grid(reinterpret_cast<const void *>(fn), smem);
        const int trk = tr_open(kTrProject);
        fn<<<nb, kRitzTile, smem, st_>>>(V, m, Tsrc, b, N_, y, out, d_partial_, stages);
        ::pyci_gpu::note_launch();
        tr_close(trk);
        int rc = read_partials(nb, MA * k, P, "orthonormalisation pass");
        if (rc)
            return rc;
        for (double v : P)
            if (!std::isfinite(v)) {
                set_error("orthonormalisation pass: non-finite sums (a staged-tile wait timed out, or non-finite vectors)");
                return PYCI_GPU_ECUDA;
            }
        return PYCI_GPU_OK;
    }

    // The fused Ritz step applies (FP32 solve, no full-space Rayleigh-Ritz,
    // at most kMaxQ pairs and kRitzMaxA rows of [V T]); PYCI_GPU_RITZ=separate
    // keeps the separate combinations, residual, norms, preconditioner and
    // Gram product.
    bool ritz_fused_on(int m, int q) const {
        return std::is_same<T, float>::value && mixed_ && ritz_fused_ && q >= 1 && q <= kMaxQ && m + q <= kRitzMaxA;
    }

    // Row width of the packed FP32 operand of a k-vector product: the
    // implicit DOCI form takes 5 vectors as they are (4.0 ms on the 32o DOCI
    // against 5.5 ms padded to 8, which its 6- and 7-wide forms match);
    // otherwise padded_width.
    int xwidth(int k) const { return (csr_->dx_v && k == 5) ? 5 : padded_width(k); }

    // Vectors per product launch: on the SELL-32 copy or the implicit-column
    // form the FP32 product streams the matrix once per launch and is bound by
    // that stream, so up to 8 vectors share one launch.
    int spmm_chunk(int prec) const {
        return (prec == PYCI_PREC_FP32 && (csr_->sell_cols || has_implicit(csr_))) ? kMaxQ : kSpmmChunk;
    }

    // W[0..k) = H V[0..k) (storage precision of T; FP64 uses f64 values).
    int apply(const T *V, int k, T *W, int prec) {
        // On the SELL-32 copy or the implicit-column form the FP32 product
        // streams the matrix once per launch and is bound by that stream, so
        // up to 8 vectors share one launch (a 5-vector block as one product
        // padded to 8, not 4 + 1).  FP64 solves on an operator that holds the
        // exact high/low split multiply in double-float arithmetic.
        const int chunk = spmm_chunk(prec);
        // The block orthonormalisation may have written the packed operand
        // already (combine2_kernel).
        const bool packed = (xi_src_ == V && xi_k_ == k && k <= chunk);
        xi_src_ = nullptr;
        for (int j0 = 0; j0 < k; j0 += chunk) {
            const int kk = std::min(chunk, k - j0);
            const bool df = std::is_same<T, double>::value && fp64_df_;
            const int kp = df ? padded_width(kk) : xwidth(kk);
            const int trp = tr_open(kTrPack);
            if (packed)
                ;
            else if (df)
                pack_split_kernel<<<grid(N_), 256, 0, st_>>>(reinterpret_cast<const double *>(V) + static_cast<int64_t>(j0) * N_,
                                                             N_, kk, kp, reinterpret_cast<float *>(Xi_)),
                    ::pyci_gpu::note_launch();
            else
                pack_kernel<T><<<grid(N_), 256, 0, st_>>>(V + static_cast<int64_t>(j0) * N_, N_, kk, kp, Xi_),
                    ::pyci_gpu::note_launch();
            tr_close(trp);
            const size_t tk = timer_begin();
            // The implicit DOCI form writes the FP32 block straight into W's
            // columns (no unpack) when it needs no padding.
            if constexpr (std::is_same<T, float>::value) {
                if (prec == PYCI_PREC_FP32 && kp == kk && csr_->dx_v &&
                    docx_launch_columns(csr_, kk, Xi_, W + static_cast<int64_t>(j0) * N_, st_)) {
                    timer_end(tk);
                    matvecs_ += kk;
                    continue;
                }
            }
            int rc = df ? csr_spmm_df(csr_, kp, reinterpret_cast<const float *>(Xi_), reinterpret_cast<double *>(Yi_), st_)
                        : csr_spmm(csr_, prec, kp, Xi_, Yi_, st_);
            if (rc)
                return rc;
            timer_end(tk);
            const int tru = tr_open(kTrPack);
            unpack_kernel<T><<<grid(N_), 256, 0, st_>>>(Yi_, N_, kk, kp, W + static_cast<int64_t>(j0) * N_), ::pyci_gpu::note_launch();
            tr_close(tru);
            matvecs_ += kk;
        }
        return PYCI_GPU_OK;
    }

    // R[j] = AX[j] - theta[j] X[j] for j < q, in launches of at most kMaxQ
    // columns.
    template<typename U>
    void residuals(const U *AX, const U *X, int q, const std::vector<double> &theta, U *R) {
        for (int j0 = 0; j0 < q; j0 += kMaxQ) {
            const int64_t o = static_cast<int64_t>(j0) * N_;
            const int qq = std::min(kMaxQ, q - j0);
            Theta th{};
            for (int j = 0; j < qq; ++j)
                th.t[j] = theta[j0 + j];
            const int trk = tr_open(kTrRows);
            residual_kernel<U><<<grid(N_), 256, 0, st_>>>(AX + o, X + o, th, qq, N_, R + o), ::pyci_gpu::note_launch();
            tr_close(trk);
        }
    }

    // out[c] = preconditioned R[todo[c]] (Ritz value theta[todo[c]]), in
    // launches of at most kMaxQ columns.
    template<typename U>
    void precondition(const U *R, const double *diag, const std::vector<int> &todo, const std::vector<double> &theta,
                      T *out) {
        const int trk = tr_open(kTrRows);
        for (size_t c0 = 0; c0 < todo.size(); c0 += kMaxQ)
            precondition_kernel<U, T><<<grid(N_), 256, 0, st_>>>(R, diag, make_cols(todo, c0, theta), N_,
                                                                  out + static_cast<int64_t>(c0) * N_),
                ::pyci_gpu::note_launch();
        tr_close(trk);
    }

    // Rows of the k lowest diagonal elements, ascending (ties by row), found
    // on the device: k passes of a grid-wide arg-min over the (value, row)
    // pairs above the previous pick, one read of the diagonal each.
    int lowest_diagonal(const double *d_diag, int64_t N, int k, std::vector<int64_t> &order) {
        longlong2 *picks = nullptr, *partial = nullptr;
        const unsigned nb = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((N + 255) / 256, 8 * csr_->ctx->num_sms)));
        int rc;
        if ((rc = alloc(&picks, k)) || (rc = alloc(&partial, nb)))
            return rc;
        for (int j = 0; j < k; ++j) {
            argmin_above_kernel<<<nb, 256, 0, st_>>>(d_diag, N, j > 0 ? picks + j - 1 : nullptr, partial);
            argmin_final_kernel<<<1, 256, 0, st_>>>(partial, nb, picks + j);
            ::pyci_gpu::note_launch();
            ::pyci_gpu::note_launch();
        }
        std::vector<longlong2> h(k);
        PYCI_CUDA_TRY(cudaMemcpyAsync(h.data(), picks, sizeof(longlong2) * k, cudaMemcpyDeviceToHost, st_));
        PYCI_CUDA_TRY(wait());
        order.resize(k);
        for (int j = 0; j < k; ++j)
            order[j] = static_cast<int64_t>(h[j].y);
        return PYCI_GPU_OK;
    }

    // Orthonormalise vectors V[m..m+k) against V[0..m) and each other;
    // returns the number kept (compacted to V[m..)).
    int orthonormalize(T *V, int m, int k, int &kept);
    // Vector-by-vector classical Gram-Schmidt (two passes); drops
    // near-dependent vectors.
    int orthonormalize_mgs(T *V, int m, int k, int &kept);
    // orthonormalize for the columns todo of Tb (b vectors apart from V)
    // into V[m..), given C1 = V[0..m)^T Tb (m x b) and TT = Tb^T Tb (b x b)
    // from the fused Ritz step: one combination when one Gram-Schmidt pass is
    // enough (orthonormalize's criterion), else the columns are copied to
    // V[m..) and orthonormalised there.
    int orthonormalize_pre(T *V, int m, const T *Tb, int b, const std::vector<int> &todo,
                           const std::vector<double> &C1, const std::vector<double> &TT, int prec, int &kept);
    // Set when the last block orthonormalisation also wrote the packed
    // product operand of xi_src_[0..xi_k_) into Xi_.
    const T *xi_src_ = nullptr;
    int xi_k_ = 0;

    pyci_gpu_csr *csr_;
    cudaStream_t st_;
    int64_t N_, nroot_, nwant_, mmax_;
    bool mixed_;
    std::vector<void *> allocs_;
    // SpMM timing: an event pair per product, read once at the end of the
    // solve (no synchronisation per product).
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timers_;
    size_t timer_begin() {
        std::pair<cudaEvent_t, cudaEvent_t> pr{nullptr, nullptr};
        cudaEventCreate(&pr.first);
        cudaEventCreate(&pr.second);
        cudaEventRecord(pr.first, st_);
        timers_.push_back(pr);
        return timers_.size() - 1;
    }
    void timer_end(size_t k) { cudaEventRecord(timers_[k].second, st_); }
    // PYCI_GPU_SOLVE_TRACE: device time by kind of step, from event pairs
    // around its launches, and the gaps at the host synchronisations (from
    // the end of the queued work to the host's next enqueue).
    enum { kTrGram, kTrRitz, kTrProject, kTrCombine, kTrPack, kTrRows, kTrSync, kTrKinds };
    std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>> tr_;
    int tr_open(int kind) {
        if (!trace_)
            return -1;
        cudaEvent_t a = nullptr, b = nullptr;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st_);
        tr_.emplace_back(kind, a, b);
        return static_cast<int>(tr_.size()) - 1;
    }
    void tr_close(int h) {
        if (h >= 0)
            cudaEventRecord(std::get<2>(tr_[static_cast<size_t>(h)]), st_);
    }
    std::string tr_summary() {
        static const char *names[kTrKinds] = {"gram", "ritz", "project", "combine", "pack", "rows", "sync gaps"};
        double t[kTrKinds] = {};
        int n[kTrKinds] = {};
        for (auto &e : tr_) {
            float ms = 0.0f;
            if (cudaEventSynchronize(std::get<2>(e)) == cudaSuccess &&
                cudaEventElapsedTime(&ms, std::get<1>(e), std::get<2>(e)) == cudaSuccess)
                t[std::get<0>(e)] += ms;
            ++n[std::get<0>(e)];
            cudaEventDestroy(std::get<1>(e));
            cudaEventDestroy(std::get<2>(e));
        }
        tr_.clear();
        std::string out;
        char buf[96];
        for (int k = 0; k < kTrKinds; ++k) {
            std::snprintf(buf, sizeof(buf), "%s%s %.3f ms (%d)", k ? ", " : "", names[k], t[k], n[k]);
            out += buf;
        }
        return out;
    }
    double timed_total_ms() {
        double total = 0.0;
        for (auto &pr : timers_) {
            float ms = 0.0f;
            if (cudaEventSynchronize(pr.second) == cudaSuccess && cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
                total += ms;
        }
        return total;
    }
    // Host-side synchronisation with the stream, counted and timed.
    cudaError_t wait() {
        const auto t0 = std::chrono::steady_clock::now();
        const int trs = tr_open(kTrSync);
        const cudaError_t e = cudaStreamSynchronize(st_);
        tr_close(trs);
        wait_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        ++syncs_;
        return e;
    }
    int64_t syncs_ = 0;
    double wait_s_ = 0.0, eig_s_ = 0.0;
    const bool trace_ = std::getenv("PYCI_GPU_SOLVE_TRACE") != nullptr;
    double *h_small_ = nullptr;  // pinned [kMaxGramP * kMaxQ]
    double *d_mapped_ = nullptr; // device alias of h_small_ (mapped), or null
    bool holds_ctx_buffer_ = false; // h_small_ is the context's buffer
    double alloc_s_ = 0.0, evec_s_ = 0.0; // host time in workspace allocations / the eigenvector copies (trace)
    bool eig(int m, const std::vector<double> &a, std::vector<double> &w, std::vector<double> &z) {
        const auto t0 = std::chrono::steady_clock::now();
        const bool ok = symmetric_eigen(m, a, w, z);
        eig_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return ok;
    }
    int64_t matvecs_ = 0, matvecs64_ = 0;
    unsigned gram_blocks_ = 1;
    T *Xi_ = nullptr, *Yi_ = nullptr, *Sb_ = nullptr;
    // FP64 solves: products in double-float arithmetic on the exact
    // high/low split (FP32 instructions, ~2^-44 relative) when the operator
    // holds the split.  GB300's FP64 rate bounds a 4-vector product with
    // FP64 arithmetic at 4 FMAs per stored entry / (FP64 FMA rate), several
    // times the time the same product takes to stream its bytes.
    bool fp64_df_ = false;
    // FP64 Gram products and combinations in double-float arithmetic
    // (gram_rows_df_kernel, combine_df_kernel): the FP64 forms are bound by
    // the FP64 pipe, not by the vectors' bytes.
    bool df_linalg_ = true;
    // Fused Ritz step of the FP32 solve (ritz_fused_kernel).
    bool ritz_fused_ = true;
    double *d_partial_ = nullptr, *d_small_ = nullptr;
};

template<typename T>
int Davidson<T>::orthonormalize(T *V, int m, int k, int &kept) {
    // Block classical Gram-Schmidt against V[0..m) (two passes), then two
    // Cholesky-QR passes inside the block.  The block T sits right after
    // V[0..m), so the second Gram-Schmidt pass's product [V T]^T T also gives
    // T^T T; after that pass T'^T T' = T^T T - C2^T C2 (C2 = V^T T, small), so
    // the first Cholesky-QR needs no product of its own and one combination
    // applies both: 3 Gram products (host synchronisations) per call.  A
    // near-singular block falls back to the vector-by-vector path, which drops
    // dependent directions.
    T *Tb = V + static_cast<int64_t>(m) * N_;
    std::vector<double> C, S;
    int rc;
    const double piv_tol = mixed_ ? 1e-6 : 1e-14;
    // Cholesky S = L L^T and Linv = L^{-1}; false when S is not safely positive
    // definite.  kappa: (max r_j / min r_j)^2 with r_j = L_jj / sqrt(S_jj), a
    // cheap estimate of the condition of S with its columns scaled to unit
    // norm.  The FP32 combination T L^{-T} rounds each term relative to
    // |t_a| |(L^{-T})_ac|, which does not change under column scaling, so
    // corrections of very different norms (converged roots topping up a
    // block) need no extra pass on that account.
    double kappa = 0.0;
    auto cholesky_inv = [&](const std::vector<double> &Sm, std::vector<double> &Linv) -> bool {
        std::vector<double> L(static_cast<size_t>(k) * k, 0.0);
        for (int j = 0; j < k; ++j) {
            double d = Sm[static_cast<size_t>(j) * k + j];
            for (int t = 0; t < j; ++t)
                d -= L[static_cast<size_t>(j) * k + t] * L[static_cast<size_t>(j) * k + t];
            if (!(d > piv_tol * Sm[static_cast<size_t>(j) * k + j]) || !(d > 0.0))
                return false;
            L[static_cast<size_t>(j) * k + j] = std::sqrt(d);
            for (int i = j + 1; i < k; ++i) {
                double x = Sm[static_cast<size_t>(i) * k + j];
                for (int t = 0; t < j; ++t)
                    x -= L[static_cast<size_t>(i) * k + t] * L[static_cast<size_t>(j) * k + t];
                L[static_cast<size_t>(i) * k + j] = x / L[static_cast<size_t>(j) * k + j];
            }
        }
        double lmax = 0.0, lmin = std::numeric_limits<double>::infinity();
        for (int j = 0; j < k; ++j) {
            const double r = L[static_cast<size_t>(j) * k + j] / std::sqrt(Sm[static_cast<size_t>(j) * k + j]);
            lmax = std::max(lmax, r);
            lmin = std::min(lmin, r);
        }
        kappa = (lmax / lmin) * (lmax / lmin);
        Linv.assign(static_cast<size_t>(k) * k, 0.0);
        for (int j = 0; j < k; ++j) {
            Linv[static_cast<size_t>(j) * k + j] = 1.0 / L[static_cast<size_t>(j) * k + j];
            for (int i = j + 1; i < k; ++i) {
                double x = 0.0;
                for (int t = j; t < i; ++t)
                    x -= L[static_cast<size_t>(i) * k + t] * Linv[static_cast<size_t>(t) * k + j];
                Linv[static_cast<size_t>(i) * k + j] = x / L[static_cast<size_t>(i) * k + i];
            }
        }
        return true;
    };
    // T' = (T - V C1) L^{-T} from C1 = V^T T and L L^T = S (the Gram of
    // T - V C1) as one combination of [V T] into Sb_, then copied to T.
    auto apply_fused = [&](const std::vector<double> &C1, const std::vector<double> &Linv) -> int {
        std::vector<double> Y(static_cast<size_t>(m + k) * k, 0.0);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < k; ++j) {
                double x = 0.0;
                for (int t = 0; t < k; ++t)
                    x -= C1[static_cast<size_t>(i) * k + t] * Linv[static_cast<size_t>(j) * k + t];
                Y[static_cast<size_t>(i) * k + j] = x;
            }
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
                Y[static_cast<size_t>(m + i) * k + j] = Linv[static_cast<size_t>(j) * k + i];
        int r2 = combine<T, T, T>(V, m + k, Y, k, 0.0, Sb_);
        if (r2)
            return r2;
        PYCI_CUDA_TRY(cudaMemcpyAsync(Tb, Sb_, sizeof(T) * k * N_, cudaMemcpyDeviceToDevice, st_));
        return PYCI_GPU_OK;
    };
    if (k > 1 && k <= kMaxQ) {
        bool ok = true;
        int passes_left = 2; // Cholesky-QR passes still to do
        bool single = false;
        if (m > 0) {
            // One Gram product [V T]^T T gives C1 = V^T T and T^T T, so
            // T - V C1 has the Gram S = T^T T - C1^T C1.  When every column
            // keeps at least half its squared norm (||t'|| >= ||t|| / sqrt 2:
            // one classical Gram-Schmidt pass is then enough, the criterion
            // of Daniel, Gragg, Kaufman and Stewart) and S is well
            // conditioned, one combination finishes the block: 1 Gram product
            // and 1 combination instead of 2 and 2.
            if ((rc = gram<T>(V, m + k, Tb, k, C)))
                return rc;
            std::vector<double> S1(static_cast<size_t>(k) * k);
            bool keeps = true;
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    double x = C[static_cast<size_t>(m + i) * k + j];
                    for (int t = 0; t < m; ++t)
                        x -= C[static_cast<size_t>(t) * k + i] * C[static_cast<size_t>(t) * k + j];
                    S1[static_cast<size_t>(i) * k + j] = x;
                    if (i == j && !(x >= 0.5 * C[static_cast<size_t>(m + i) * k + i]))
                        keeps = false;
                }
            std::vector<double> Linv;
            if (keeps && cholesky_inv(S1, Linv) && kappa < 10.0) {
                if ((rc = apply_fused(C, Linv)))
                    return rc;
                single = true;
                passes_left = 0;
            }
        }
        if (m > 0 && !single) {
            // Pass 1 (C holds [V T]^T T: its first m rows are V^T T).
            C.resize(static_cast<size_t>(m) * k);
            for (double &c : C)
                c = -c;
            if ((rc = combine<T, T, T>(V, m, C, k, 1.0, Tb)))
                return rc;
            // Pass 2 fused with the first Cholesky-QR.
            if ((rc = gram<T>(V, m + k, Tb, k, C)))
                return rc;
            std::vector<double> Sm(static_cast<size_t>(k) * k);
            double cmax = 0.0, smin = std::numeric_limits<double>::infinity();
            for (int i = 0; i < k; ++i)
                smin = std::min(smin, C[static_cast<size_t>(m + i) * k + i]);
            for (size_t e = 0; e < static_cast<size_t>(m) * k; ++e)
                cmax = std::max(cmax, std::fabs(C[e]));
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    double x = C[static_cast<size_t>(m + i) * k + j];
                    for (int t = 0; t < m; ++t)
                        x -= C[static_cast<size_t>(t) * k + i] * C[static_cast<size_t>(t) * k + j];
                    Sm[static_cast<size_t>(i) * k + j] = x;
                }
            std::vector<double> Linv;
            if (smin > 0.0 && cmax * cmax <= 1e-4 * smin && cholesky_inv(Sm, Linv)) {
                // new = (T - V C2) L^{-T}.
                if ((rc = apply_fused(C, Linv)))
                    return rc;
                // A well-conditioned block is orthonormal to ~kappa * eps
                // after one pass: skip the second (one product and one
                // synchronisation fewer per iteration).
                passes_left = (kappa < 10.0) ? 0 : 1;
            } else {
                // Plain second pass (the block was far from orthogonal to V).
                for (size_t e = 0; e < static_cast<size_t>(m) * k; ++e)
                    C[e] = -C[e];
                C.resize(static_cast<size_t>(m) * k);
                if ((rc = combine<T, T, T>(V, m, C, k, 1.0, Tb)))
                    return rc;
            }
        }
        for (int pass = 0; pass < passes_left && ok; ++pass) {
            if ((rc = gram<T>(Tb, k, Tb, k, S)))
                return rc;
            std::vector<double> Linv;
            if (!cholesky_inv(S, Linv)) {
                ok = false;
                break;
            }
            // new_j = sum_i Linv[j][i] T_i  ->  coefficient matrix Y[i][j] = Linv[j][i]
            std::vector<double> Y(static_cast<size_t>(k) * k);
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j)
                    Y[static_cast<size_t>(i) * k + j] = Linv[static_cast<size_t>(j) * k + i];
            if ((rc = combine<T, T, T>(Tb, k, Y, k, 0.0, Sb_)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(Tb, Sb_, sizeof(T) * k * N_, cudaMemcpyDeviceToDevice, st_));
        }
        if (ok) {
            kept = k;
            return PYCI_GPU_OK;
        }
    }
    return orthonormalize_mgs(V, m, k, kept);
}

template<typename T>
int Davidson<T>::orthonormalize_mgs(T *V, int m, int k, int &kept) {
    const double drop = mixed_ ? 1e-3 : 1e-8;
    kept = 0;
    std::vector<double> C;
    for (int j = 0; j < k; ++j) {
        T *t = V + static_cast<int64_t>(m + j) * N_;
        int rc = gram<T>(t, 1, t, 1, C);
        if (rc)
            return rc;
        const double n0 = std::sqrt(std::max(C[0], 0.0));
        if (!(n0 > 0.0) || !std::isfinite(n0))
            continue;
        const int have = m + kept;
        for (int pass = 0; pass < 2 && have > 0; ++pass) {
            rc = gram<T>(V, have, t, 1, C);
            if (rc)
                return rc;
            for (double &c : C)
                c = -c;
            rc = combine<T, T, T>(V, have, C, 1, 1.0, t);
            if (rc)
                return rc;
        }
        rc = gram<T>(t, 1, t, 1, C);
        if (rc)
            return rc;
        const double n1 = std::sqrt(std::max(C[0], 0.0));
        if (!(n1 > drop * n0))
            continue;
        T *dst = V + static_cast<int64_t>(m + kept) * N_;
        scale_kernel<T><<<grid(N_), 256, 0, st_>>>(t, N_, 1.0 / n1), ::pyci_gpu::note_launch();
        if (dst != t)
            cudaMemcpyAsync(dst, t, sizeof(T) * N_, cudaMemcpyDeviceToDevice, st_);
        ++kept;
    }
    return PYCI_GPU_OK;
}

template<typename T>
int Davidson<T>::orthonormalize_pre(T *V, int m, const T *Tb, int b, const std::vector<int> &todo,
                                    const std::vector<double> &C1, const std::vector<double> &TT, int prec,
                                    int &kept) {
    const int k = static_cast<int>(todo.size());
    kept = 0;
    if (k == 0)
        return PYCI_GPU_OK;
    T *out = V + static_cast<int64_t>(m) * N_;
    if constexpr (std::is_same<T, float>::value) {
        const bool pack = k <= spmm_chunk(prec);
        const int kp = xwidth(k);
        // (Q - V C) L^{-T} for the block Q (b vectors, columns cols of it
        // chosen, k of them) into out (also packed into Xi_ when xi): rows of
        // V, then the rows of Q.
        auto finish = [&](const float *Q, int nq, const std::vector<int> &cols, const std::vector<double> &C, int ldc,
                          const std::vector<double> &Linv, bool xi) {
            CoefBlock<float> y{};
            for (int i = 0; i < m; ++i)
                for (int c = 0; c < k; ++c) {
                    double x = 0.0;
                    for (int a = 0; a < k; ++a)
                        x -= C[static_cast<size_t>(i) * ldc + cols[a]] * Linv[static_cast<size_t>(c) * k + a];
                    y.y[i * k + c] = static_cast<float>(x);
                }
            for (int a = 0; a < k; ++a)
                for (int c = 0; c < k; ++c)
                    y.y[(m + cols[a]) * k + c] = static_cast<float>(Linv[static_cast<size_t>(c) * k + a]);
            float *xp = xi ? reinterpret_cast<float *>(Xi_) : nullptr;
            const int trk = tr_open(kTrCombine);
            if (N_ % 4 == 0)
                combine2_kernel<4><<<grid(N_ / 4), 256, 0, st_>>>(V, m, Q, nq, N_, y, k, out, xp, kp);
            else
                combine2_kernel<1><<<grid(N_), 256, 0, st_>>>(V, m, Q, nq, N_, y, k, out, xp, kp);
            ::pyci_gpu::note_launch();
            tr_close(trk);
            if (xi) {
                xi_src_ = out;
                xi_k_ = k;
            }
        };
        // Cholesky of S with orthonormalize's column-scaled conditioning
        // estimate.
        auto chol = [&](const std::vector<double> &S, std::vector<double> &Linv, double &kappa) -> bool {
            if (!cholesky_inverse(S, k, 1e-6, Linv))
                return false;
            double lmax = 0.0, lmin = std::numeric_limits<double>::infinity();
            for (int j = 0; j < k; ++j) {
                const double l = 1.0 / Linv[static_cast<size_t>(j) * k + j] / std::sqrt(S[static_cast<size_t>(j) * k + j]);
                lmax = std::max(lmax, l);
                lmin = std::min(lmin, l);
            }
            kappa = (lmax / lmin) * (lmax / lmin);
            return true;
        };
        // S = Tc^T Tc - C^T C for the chosen columns Tc (C = V^T Tc): the Gram
        // of Tc - V C.  One pass is enough when every column keeps at least
        // half its squared norm and S is well conditioned (orthonormalize's
        // criterion).
        std::vector<double> S(static_cast<size_t>(k) * k);
        bool keeps = true;
        for (int a = 0; a < k; ++a)
            for (int c = 0; c < k; ++c) {
                const int ta = todo[a], tc = todo[c];
                double x = TT[static_cast<size_t>(ta) * b + tc];
                for (int i = 0; i < m; ++i)
                    x -= C1[static_cast<size_t>(i) * b + ta] * C1[static_cast<size_t>(i) * b + tc];
                S[static_cast<size_t>(a) * k + c] = x;
                if (a == c && !(x >= 0.5 * TT[static_cast<size_t>(ta) * b + ta]))
                    keeps = false;
            }
        std::vector<double> Linv;
        double kappa = 0.0;
        if (keeps && chol(S, Linv, kappa) && kappa < 10.0) {
            finish(Tb, b, todo, C1, b, Linv, pack);
            kept = k;
            return PYCI_GPU_OK;
        }
        // Two passes: T1 = Tc - V C (into Sb_) with the Gram product
        // [V T1]^T T1 in the same read of V, then (T1 - V C2) L^{-T} from the
        // Cholesky factor of T1^T T1 - C2^T C2 when T1 is nearly orthogonal
        // to V (orthonormalize's second pass).
        {
            CoefBlock<float> y{};
            for (int i = 0; i < m; ++i)
                for (int c = 0; c < k; ++c)
                    y.y[i * k + c] = static_cast<float>(-C1[static_cast<size_t>(i) * b + todo[c]]);
            for (int c = 0; c < k; ++c)
                y.y[(m + todo[c]) * k + c] = 1.0f;
            std::vector<double> P2;
            int rc = project_gram(V, m, Tb, b, y, k, Sb_, P2);
            if (rc)
                return rc;
            std::vector<double> Sm(static_cast<size_t>(k) * k);
            double cmax = 0.0, smin = std::numeric_limits<double>::infinity();
            for (int i = 0; i < k; ++i)
                smin = std::min(smin, P2[static_cast<size_t>(m + i) * k + i]);
            for (size_t e = 0; e < static_cast<size_t>(m) * k; ++e)
                cmax = std::max(cmax, std::fabs(P2[e]));
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    double x = P2[static_cast<size_t>(m + i) * k + j];
                    for (int t = 0; t < m; ++t)
                        x -= P2[static_cast<size_t>(t) * k + i] * P2[static_cast<size_t>(t) * k + j];
                    Sm[static_cast<size_t>(i) * k + j] = x;
                }
            std::vector<int> ident(k);
            std::iota(ident.begin(), ident.end(), 0);
            if (smin > 0.0 && cmax * cmax <= 1e-4 * smin && chol(Sm, Linv, kappa)) {
                const bool again = !(kappa < 10.0);
                finish(Sb_, k, ident, P2, k, Linv, pack && !again);
                kept = k;
                if (!again)
                    return PYCI_GPU_OK;
                // One Cholesky-QR pass more (orthonormalize's criterion).
                std::vector<double> G2;
                if ((rc = gram<T>(out, k, out, k, G2)))
                    return rc;
                if (!cholesky_inverse(G2, k, 1e-6, Linv))
                    return orthonormalize(V, m, k, kept);
                std::vector<double> Y(static_cast<size_t>(k) * k);
                for (int i = 0; i < k; ++i)
                    for (int j = 0; j < k; ++j)
                        Y[static_cast<size_t>(i) * k + j] = Linv[static_cast<size_t>(j) * k + i];
                if ((rc = combine<T, T, T>(out, k, Y, k, 0.0, Sb_)))
                    return rc;
                PYCI_CUDA_TRY(cudaMemcpyAsync(out, Sb_, sizeof(T) * k * N_, cudaMemcpyDeviceToDevice, st_));
                return PYCI_GPU_OK;
            }
            // Far from orthogonal after one pass: the general path on T1.
            PYCI_CUDA_TRY(cudaMemcpyAsync(out, Sb_, sizeof(T) * k * N_, cudaMemcpyDeviceToDevice, st_));
            return orthonormalize(V, m, k, kept);
        }
    } else {
        for (int c = 0; c < k; ++c)
            PYCI_CUDA_TRY(cudaMemcpyAsync(out + static_cast<int64_t>(c) * N_, Tb + static_cast<int64_t>(todo[c]) * N_,
                                          sizeof(T) * N_, cudaMemcpyDeviceToDevice, st_));
        return orthonormalize(V, m, k, kept);
    }
}

template<typename T>
int Davidson<T>::run(const double *c0, int64_t maxiter, double tol, double ecore, double *evals,
                     double *evecs, pyci_gpu_solve_stats *stats) {
    const auto t_start = std::chrono::steady_clock::now();
    const int64_t N = N_;
    const int b = static_cast<int>(nroot_);
    const int nw = static_cast<int>(nwant_);
    const int mmax = static_cast<int>(mmax_);
    const bool full_space = (N <= mmax);
    const int prec = mixed_ ? PYCI_PREC_FP32 : PYCI_PREC_FP64;
    int rc;
    gram_blocks_ = static_cast<unsigned>(csr_->ctx->num_sms * 4);
    // The eigenvector buffer is written once, at the end; the first touch of
    // fresh host memory (page faults, up to ~9 ms for the 20 MB of four
    // 627,264-row vectors) runs on another host thread while the GPU
    // iterates.  Joined before the copies, and on every return.
    std::thread prefault;
    if (evecs)
        prefault = std::thread([evecs, bytes = sizeof(double) * static_cast<size_t>(nw) * static_cast<size_t>(N)] {
            std::memset(evecs, 0, bytes);
        });
    struct Join {
        std::thread &t;
        ~Join() {
            if (t.joinable())
                t.join();
        }
    } join_prefault{prefault};


    T *V, *W, *Xr, *AXr, *R;
    // Vectors kept at a thick restart; leaves room for a full new block.
    // Kept at a thick restart: the lowest max(4 nw, 2 b) Ritz vectors, leaving
    // room for a full block of nw corrections.
    const int nkeep_max = std::max(b, std::min(mmax - nw, std::max(4 * nw, 2 * b)));
    if ((rc = alloc(&V, static_cast<int64_t>(mmax) * N)) || (rc = alloc(&W, static_cast<int64_t>(mmax) * N)) ||
        (rc = alloc(&Xr, static_cast<int64_t>(std::max(nkeep_max, b)) * N)) ||
        (rc = alloc(&AXr, static_cast<int64_t>(std::max(nkeep_max, b)) * N)) ||
        (rc = alloc(&R, static_cast<int64_t>(b) * N)) || (rc = alloc(&Xi_, N * kMaxQ)) ||
        (rc = alloc(&Yi_, N * kMaxQ)) || (rc = alloc(&Sb_, N * kMaxQ)) || (rc = alloc(&d_partial_, static_cast<int64_t>(gram_blocks_) * kMaxGramP * kMaxQ)) ||
        (rc = alloc(&d_small_, kMaxGramP * kMaxQ)))
        return rc;
    {
        // The context's mapped buffer when no other solve holds it, else one
        // of this solve's own.
        pyci_gpu_ctx *ctx = csr_->ctx;
        bool expected = false;
        const bool shared = ctx->mapped_busy.compare_exchange_strong(expected, true);
        double **host = shared ? &ctx->mapped_host : &h_small_;
        if (!*host) {
            const cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(host), sizeof(double) * kMaxGramP * kMaxQ,
                                                cudaHostAllocMapped);
            if (e != cudaSuccess) {
                if (shared)
                    ctx->mapped_busy = false;
                return cuda_status(e, "cudaHostAlloc (eigensolver read-back)");
            }
            int can_map = 0;
            cudaDeviceGetAttribute(&can_map, cudaDevAttrCanMapHostMemory, ctx->device);
            void *dp = nullptr;
            if (shared)
                ctx->mapped_dev = (can_map && cudaHostGetDevicePointer(&dp, *host, 0) == cudaSuccess)
                                      ? static_cast<double *>(dp) : nullptr;
            else if (can_map && cudaHostGetDevicePointer(&dp, *host, 0) == cudaSuccess)
                d_mapped_ = static_cast<double *>(dp);
            cudaGetLastError();
        }
        if (shared) {
            h_small_ = ctx->mapped_host;
            d_mapped_ = ctx->mapped_dev;
            holds_ctx_buffer_ = true;
        }
    }
    double *d_diag = csr_->diag;


    // Initial block.
    int m = 0, knew = 0;
    if (full_space) {
        std::vector<int64_t> idx(N);
        std::iota(idx.begin(), idx.end(), 0);
        int64_t *d_idx;
        if ((rc = alloc(&d_idx, N)))
            return rc;
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_idx, idx.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice, st_));
        for (int64_t j0 = 0; j0 < N; j0 += 64)
            unit_kernel<T><<<grid(N), 256, 0, st_>>>(V + j0 * N, N, d_idx + j0, static_cast<int>(std::min<int64_t>(64, N - j0))), ::pyci_gpu::note_launch();
        PYCI_CUDA_TRY(wait());
        knew = static_cast<int>(N);
    } else {
        // Unit vectors on the lowest diagonal elements (after c0, if given),
        // each with a small seeded component in every row, topped up until
        // the block holds b independent vectors.
        const int64_t nsort = std::min<int64_t>(N, 2 * b + 8);
        std::vector<int64_t> order;
        if ((rc = lowest_diagonal(d_diag, N, static_cast<int>(nsort), order)))
            return rc;
        const double amp = kGuessNoise / std::sqrt(static_cast<double>(N));
        int64_t next = 0;
        if (c0) {
            std::vector<T> hc(N);
            for (int64_t r = 0; r < N; ++r)
                hc[r] = static_cast<T>(c0[r]);
            PYCI_CUDA_TRY(cudaMemcpyAsync(V, hc.data(), sizeof(T) * N, cudaMemcpyHostToDevice, st_));
            PYCI_CUDA_TRY(wait());
            if ((rc = orthonormalize(V, 0, 1, knew)))
                return rc;
        }
        // All missing start vectors at once, then one block
        // orthonormalisation (a few host round trips instead of several per
        // vector); dependent ones are dropped and replaced.
        while (knew < b && next < N) {
            const int need = static_cast<int>(std::min<int64_t>(b - knew, N - next));
            for (int j = 0; j < need; ++j, ++next) {
                const int64_t pick = (next < nsort) ? order[next] : next;
                guess_kernel<T><<<grid(N), 256, 0, st_>>>(V + static_cast<int64_t>(knew + j) * N, N, pick, amp,
                                                            static_cast<int>(next)),
                    ::pyci_gpu::note_launch();
            }
            int got = 0;
            if ((rc = orthonormalize(V, knew, need, got)))
                return rc;
            knew += got;
        }
        if (knew < b) {
            set_error("could not build an initial block");
            return PYCI_GPU_ENOCONV;
        }
    }

    std::vector<double> G(static_cast<size_t>(mmax) * mmax, 0.0), theta, Y, Gc;
    std::vector<double> rnorm(b, 0.0);
    // Previous iteration's FP32 residual norms and the last kPlateau of them
    // per root (mixed mode's stall tests).
    std::vector<double> rprev(b, std::numeric_limits<double>::infinity());
    constexpr int kPlateau = 5;
    std::vector<std::vector<double>> rhist(b);
    const double eps23 = std::pow(std::numeric_limits<double>::epsilon(), 2.0 / 3.0);
    const double mixed_floor = 1e-5;
    int64_t iter = 0, restarts = 0, refinements = 0;
    bool converged = false;
    std::vector<double> final_theta(b);
    double max_res = 0.0;
    double *X64 = nullptr, *AX64 = nullptr, *R64 = nullptr, *Xi64 = nullptr, *Yi64 = nullptr;

    for (iter = 0; iter < maxiter; ++iter) {
        // W for the new block.
        if (knew > 0) {
            if ((rc = apply(V + static_cast<int64_t>(m) * N, knew, W + static_cast<int64_t>(m) * N, prec)))
                return rc;
            // Projected matrix: new columns.
            if ((rc = gram<T>(V, m + knew, W + static_cast<int64_t>(m) * N, knew, Gc)))
                return rc;
            for (int i = 0; i < m + knew; ++i)
                for (int j = 0; j < knew; ++j) {
                    G[static_cast<size_t>(i) * mmax + m + j] = Gc[static_cast<size_t>(i) * knew + j];
                    G[static_cast<size_t>(m + j) * mmax + i] = Gc[static_cast<size_t>(i) * knew + j];
                }
            m += knew;
        }
        std::vector<double> Gm(static_cast<size_t>(m) * m);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j)
                Gm[static_cast<size_t>(i) * m + j] = G[static_cast<size_t>(i) * mmax + j];
        if (!eig(m, Gm, theta, Y)) {
            set_error("Rayleigh-Ritz eigensolver failed");
            return PYCI_GPU_ENOCONV;
        }
        // Ritz vectors and residuals of the b lowest.
        std::vector<double> Yb(static_cast<size_t>(m) * b);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < b; ++j)
                Yb[static_cast<size_t>(i) * b + j] = Y[static_cast<size_t>(i) * m + j];
        // Fused (FP32): R holds the preconditioned residuals of all b pairs,
        // Pf = [V R]^T R; Xr and AXr are formed only where needed.
        const bool fused = ritz_fused_on(m, b);
        std::vector<double> Pf, rn2(b);
        if (fused) {
            if constexpr (std::is_same<T, float>::value) {
                if ((rc = ritz_fused(V, W, m, Yb, b, theta, d_diag, R, Pf, rn2)))
                    return rc;
            }
        } else {
            if ((rc = combine<T, T, T>(V, m, Yb, b, 0.0, Xr)) || (rc = combine<T, T, T>(W, m, Yb, b, 0.0, AXr)))
                return rc;
            residuals<T>(AXr, Xr, b, theta, R);
            if ((rc = gram<T>(R, b, R, b, Gc)))
                return rc;
            for (int j = 0; j < b; ++j)
                rn2[j] = Gc[static_cast<size_t>(j) * b + j];
        }
        bool all = true;
        std::vector<int> todo;
        for (int j = 0; j < b; ++j) {
            rnorm[j] = std::sqrt(std::max(rn2[j], 0.0));
            double thr = tol * std::max(eps23, std::fabs(theta[j]));
            if (mixed_)
                thr = std::max(thr, mixed_floor);
            if (full_space)
                thr = std::numeric_limits<double>::infinity();
            // Mixed mode: a residual within 2x of the threshold that fell by
            // less than 30 % since the last iteration sits on the FP32
            // rounding floor of H x (~1e-6 |theta|); more FP32 iterations
            // cannot lower it, so the root goes to the FP64 refinement, whose
            // own test decides.  So does one within 4x of the threshold that
            // has not improved by 10 % on the best of its last 5 values (a
            // floor slightly above 2x: seen at 2.0-2.4e-5 against 1e-5 over
            // 270 restarts of a 16-vector subspace).
            double best = std::numeric_limits<double>::infinity();
            if (static_cast<int>(rhist[j].size()) == kPlateau)
                best = *std::min_element(rhist[j].begin(), rhist[j].end());
            const bool stalled = mixed_ && ((rnorm[j] <= 2.0 * thr && rnorm[j] > 0.7 * rprev[j]) ||
                                            (rnorm[j] <= 4.0 * thr && rnorm[j] > 0.9 * best));
            rprev[j] = rnorm[j];
            if (static_cast<int>(rhist[j].size()) == kPlateau)
                rhist[j].erase(rhist[j].begin());
            rhist[j].push_back(rnorm[j]);
            if (!(rnorm[j] <= thr) && !stalled) {
                if (j < nw)
                    all = false;
                todo.push_back(j);
            }
        }
        // Corrections for at most nw roots per iteration, lowest first: the
        // guard Ritz pairs beyond nw steer the subspace without widening the
        // SpMM.  In mixed precision a block with fewer unconverged roots is
        // topped up with the lowest converged ones: the FP32 product is bound
        // by streaming the matrix, so a narrower block saves little (2
        // vectors cost ~3/4 of 4) and the extra directions keep improving the
        // converged roots.  (The FP64 product's cost grows with the width.)
        if (trace_) {
            double rmax = 0.0;
            for (int j = 0; j < nw; ++j)
                rmax = std::max(rmax, rnorm[j]);
            std::fprintf(stderr, "  iter %lld m %d max_res(wanted) %.3e unconverged %d\n", static_cast<long long>(iter), m,
                         rmax, static_cast<int>(todo.size()));
        }
        if (static_cast<int>(todo.size()) > nw)
            todo.resize(nw);
        if (mixed_ && !all && !full_space && static_cast<int>(todo.size()) < nw) {
            for (int j = 0; j < b && static_cast<int>(todo.size()) < nw; ++j)
                if (std::find(todo.begin(), todo.end(), j) == todo.end())
                    todo.push_back(j);
            std::sort(todo.begin(), todo.end());
        }
        if (all) {
            if (!mixed_) {
                converged = true;
                final_theta.assign(theta.begin(), theta.begin() + b);
                max_res = *std::max_element(rnorm.begin(), rnorm.begin() + nw);
                break;
            }
            // FP64 refinement of the nw wanted Ritz vectors (the guard pairs
            // only steer the FP32 subspace).
            ++refinements;
            const int br = nw;
            if (!X64) {
                if ((rc = alloc(&X64, static_cast<int64_t>(br) * N)) || (rc = alloc(&AX64, static_cast<int64_t>(br) * N)) ||
                    (rc = alloc(&R64, static_cast<int64_t>(br) * N)) || (rc = alloc(&Xi64, N * kMaxQ)) ||
                    (rc = alloc(&Yi64, N * kMaxQ)))
                    return rc;
            }
            std::vector<double> Ybr(static_cast<size_t>(m) * br);
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < br; ++j)
                    Ybr[static_cast<size_t>(i) * br + j] = Yb[static_cast<size_t>(i) * b + j];
            // Accumulated in the storage precision: errors in the Ritz
            // vectors enter the refined Rayleigh quotients only to second order.
            if ((rc = combine<T, double, T>(V, m, Ybr, br, 0.0, X64)))
                return rc;
            // Orthonormalise X64 in FP64: Cholesky QR twice (the Ritz vectors
            // of the FP32 subspace are orthonormal to ~1e-7, so X^T X is
            // close to I; 2 host round trips); vector-by-vector Gram-Schmidt
            // if X^T X is not safely positive definite.
            bool cholqr_ok = br > 1;
            for (int pass = 0; pass < 2 && cholqr_ok; ++pass) {
                if ((rc = gram<double>(X64, br, X64, br, Gc)))
                    return rc;
                std::vector<double> Linv;
                if (!cholesky_inverse(Gc, br, 1e-8, Linv)) {
                    cholqr_ok = false;
                    break;
                }
                std::vector<double> Yc(static_cast<size_t>(br) * br);
                for (int i = 0; i < br; ++i)
                    for (int j = 0; j < br; ++j)
                        Yc[static_cast<size_t>(i) * br + j] = Linv[static_cast<size_t>(j) * br + i];
                if ((rc = combine<double, double, double>(X64, br, Yc, br, 0.0, R64)))
                    return rc;
                PYCI_CUDA_TRY(cudaMemcpyAsync(X64, R64, sizeof(double) * br * N, cudaMemcpyDeviceToDevice, st_));
            }
            for (int j = 0; j < br && !cholqr_ok; ++j) {
                double *xj = X64 + static_cast<int64_t>(j) * N;
                for (int pass = 0; pass < 2 && j > 0; ++pass) {
                    if ((rc = gram<double>(X64, j, xj, 1, Gc)))
                        return rc;
                    for (double &c : Gc)
                        c = -c;
                    if ((rc = combine<double, double, double>(X64, j, Gc, 1, 1.0, xj)))
                        return rc;
                }
                if ((rc = gram<double>(xj, 1, xj, 1, Gc)))
                    return rc;
                scale_kernel<double><<<grid(N), 256, 0, st_>>>(xj, N, 1.0 / std::sqrt(Gc[0])), ::pyci_gpu::note_launch();
            }
            for (int j0 = 0; j0 < br; j0 += kSpmmChunk) {
                // FP64-accurate product in FP32 arithmetic (double-float).
                const int kk = std::min(kSpmmChunk, br - j0);
                const int kp = padded_width(kk);
                float *xs = reinterpret_cast<float *>(Xi64); // [N][2 kp] floats fit in [N][kMaxQ] doubles
                pack_split_kernel<<<grid(N), 256, 0, st_>>>(X64 + static_cast<int64_t>(j0) * N, N, kk, kp, xs),
                    ::pyci_gpu::note_launch();
                const size_t tk = timer_begin();
                if ((rc = csr_spmm_df(csr_, kp, xs, Yi64, st_)))
                    return rc;
                timer_end(tk);
                unpack_kernel<double><<<grid(N), 256, 0, st_>>>(Yi64, N, kk, kp, AX64 + static_cast<int64_t>(j0) * N), ::pyci_gpu::note_launch();
                matvecs_ += kk;
                matvecs64_ += kk;
            }
            std::vector<double> G64, th64, Z;
            if ((rc = gram<double>(X64, br, AX64, br, G64)))
                return rc;
            if (!eig(br, G64, th64, Z)) {
                set_error("Rayleigh-Ritz eigensolver failed");
                return PYCI_GPU_ENOCONV;
            }
            // Rotate X64 and AX64 into the FP64 Ritz basis (R64 as scratch).
            if ((rc = combine<double, double, double>(X64, br, Z, br, 0.0, R64)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(X64, R64, sizeof(double) * br * N, cudaMemcpyDeviceToDevice, st_));
            if ((rc = combine<double, double, double>(AX64, br, Z, br, 0.0, R64)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(AX64, R64, sizeof(double) * br * N, cudaMemcpyDeviceToDevice, st_));
            residuals<double>(AX64, X64, br, th64, R64);
            bool ok64 = true;
            todo.clear();
            max_res = 0.0;
            if ((rc = gram<double>(R64, br, R64, br, Gc)))
                return rc;
            for (int j = 0; j < br; ++j) {
                const double r64 = std::sqrt(std::max(Gc[static_cast<size_t>(j) * br + j], 0.0));
                const double thr = std::max(tol * std::max(eps23, std::fabs(th64[j])), 2.0 * mixed_floor);
                max_res = std::max(max_res, r64);
                if (!(r64 <= thr)) {
                    ok64 = false;
                    todo.push_back(j);
                }
            }
            if (trace_)
                std::fprintf(stderr, "  refinement %lld max_res64 %.3e %s\n", static_cast<long long>(refinements), max_res,
                             ok64 ? "converged" : "continue");
            if (ok64 || refinements >= 8) {
                converged = ok64;
                final_theta = th64;
                break;
            }
            // Seed the FP32 subspace with the FP64-preconditioned residuals.
            if (m + static_cast<int>(todo.size()) > mmax) {
                // Collapse onto the b FP32 Ritz vectors of this iteration
                // (projected matrix diag(theta)).
                if (fused && ((rc = combine<T, T, T>(V, m, Yb, b, 0.0, Xr)) ||
                              (rc = combine<T, T, T>(W, m, Yb, b, 0.0, AXr))))
                    return rc;
                PYCI_CUDA_TRY(cudaMemcpyAsync(V, Xr, sizeof(T) * b * N, cudaMemcpyDeviceToDevice, st_));
                PYCI_CUDA_TRY(cudaMemcpyAsync(W, AXr, sizeof(T) * b * N, cudaMemcpyDeviceToDevice, st_));
                std::fill(G.begin(), G.end(), 0.0);
                for (int i = 0; i < b; ++i)
                    G[static_cast<size_t>(i) * mmax + i] = theta[i];
                m = b;
                ++restarts;
            }
            const int q = static_cast<int>(todo.size());
            precondition<double>(R64, d_diag, todo, th64, V + static_cast<int64_t>(m) * N);
            if ((rc = orthonormalize(V, m, q, knew)))
                return rc;
            continue;
        }
        if (full_space) {
            set_error("Rayleigh-Ritz on the full space left residuals above the tolerance");
            return PYCI_GPU_ENOCONV;
        }
        // Thick restart when the block does not fit.
        const int nt = static_cast<int>(todo.size());
        if (m + nt > mmax) {
            const int nkeep = std::min(m, nkeep_max);
            std::vector<double> Yk(static_cast<size_t>(m) * nkeep);
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < nkeep; ++j)
                    Yk[static_cast<size_t>(i) * nkeep + j] = Y[static_cast<size_t>(i) * m + j];
            T *tmpX = Xr, *tmpW = AXr; // both hold nkeep_max vectors
            if ((rc = combine<T, T, T>(V, m, Yk, nkeep, 0.0, tmpX)) || (rc = combine<T, T, T>(W, m, Yk, nkeep, 0.0, tmpW)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(V, tmpX, sizeof(T) * nkeep * N, cudaMemcpyDeviceToDevice, st_));
            PYCI_CUDA_TRY(cudaMemcpyAsync(W, tmpW, sizeof(T) * nkeep * N, cudaMemcpyDeviceToDevice, st_));
            std::fill(G.begin(), G.end(), 0.0);
            for (int i = 0; i < nkeep; ++i)
                G[static_cast<size_t>(i) * mmax + i] = theta[i];
            if (fused) {
                // The kept basis is V Yk: its products with R are Yk^T (V^T R).
                std::vector<double> Pk(static_cast<size_t>(nkeep + b) * b, 0.0);
                for (int a = 0; a < nkeep; ++a)
                    for (int j = 0; j < b; ++j) {
                        double x = 0.0;
                        for (int i = 0; i < m; ++i)
                            x += Yk[static_cast<size_t>(i) * nkeep + a] * Pf[static_cast<size_t>(i) * b + j];
                        Pk[static_cast<size_t>(a) * b + j] = x;
                    }
                std::copy(Pf.begin() + static_cast<size_t>(m) * b, Pf.begin() + static_cast<size_t>(m + b) * b,
                          Pk.begin() + static_cast<size_t>(nkeep) * b);
                Pf.swap(Pk);
            }
            m = nkeep;
            ++restarts;
        }
        // Preconditioned residuals of the unconverged roots.
        const int q = static_cast<int>(todo.size());
        if (fused) {
            const std::vector<double> C1(Pf.begin(), Pf.begin() + static_cast<size_t>(m) * b),
                TT(Pf.begin() + static_cast<size_t>(m) * b, Pf.begin() + static_cast<size_t>(m + b) * b);
            if ((rc = orthonormalize_pre(V, m, R, b, todo, C1, TT, prec, knew)))
                return rc;
        } else {
            precondition<T>(R, d_diag, todo, theta, V + static_cast<int64_t>(m) * N);
            if ((rc = orthonormalize(V, m, q, knew)))
                return rc;
        }
        if (knew == 0) {
            set_error("did not converge");
            return PYCI_GPU_ENOCONV;
        }
    }
    if (!converged) {
        set_error("did not converge");
        return PYCI_GPU_ENOCONV;
    }
    // Results: decreasing order (Spectra's result order).
    const auto t_evec = std::chrono::steady_clock::now();
    if (prefault.joinable())
        prefault.join();
    for (int c = 0; c < nw; ++c) {
        const int src = nw - 1 - c;
        evals[c] = final_theta[src] + ecore;
        if (evecs) {
            if (mixed_) {
                PYCI_CUDA_TRY(cudaMemcpyAsync(evecs + static_cast<int64_t>(c) * N, X64 + static_cast<int64_t>(src) * N,
                                              sizeof(double) * N, cudaMemcpyDeviceToHost, st_));
            } else {
                PYCI_CUDA_TRY(cudaMemcpyAsync(evecs + static_cast<int64_t>(c) * N, Xr + static_cast<int64_t>(src) * N,
                                              sizeof(double) * N, cudaMemcpyDeviceToHost, st_));
            }
        }
    }
    PYCI_CUDA_TRY(wait());
    evec_s_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_evec).count();
    if (stats) {
        stats->iterations = iter + 1;
        stats->matvecs = matvecs_;
        stats->matvecs_fp64 = mixed_ ? matvecs64_ : matvecs_;
        stats->restarts = restarts;
        stats->refinements = refinements;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->seconds_spmm = timed_total_ms() * 1e-3;
        stats->max_residual = max_res;
        stats->host_syncs = syncs_;
        stats->seconds_wait = wait_s_;
    }
    // PYCI_GPU_SOLVE_TRACE: one line per solve on stderr with the host-side
    // breakdown (blocked in read-backs, Rayleigh-Ritz).
    if (trace_)
        std::fprintf(stderr, "solve trace: total %.3f ms, spmm %.3f ms, wait %.3f ms (%lld syncs), eig %.3f ms, "
                             "allocations %.3f ms, eigenvectors out %.3f ms, iters %lld; device: %s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() * 1e3,
                     timed_total_ms(), wait_s_ * 1e3, static_cast<long long>(syncs_), eig_s_ * 1e3, alloc_s_ * 1e3,
                     evec_s_ * 1e3, static_cast<long long>(iter + 1), tr_summary().c_str());
    return PYCI_GPU_OK;
}

bool gram_tc_enabled() {
    static const bool on = [] {
        const char *e = std::getenv("PYCI_GPU_GRAM");
        return !(e && std::strcmp(e, "cuda") == 0);
    }();
    return on;
}

int gram_device(pyci_gpu_ctx *ctx, int method, const float *A, int64_t p, const float *B, int64_t q, int64_t N,
                double *C) {
    cudaStream_t st = ctx->stream;
    const unsigned budget = static_cast<unsigned>(ctx->num_sms * 4);
    double *partial = nullptr, *small = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(&partial, sizeof(double) * budget * kMaxGramP * kMaxQ, st));
    PYCI_CUDA_TRY(cudaMallocAsync(&small, sizeof(double) * kMaxGramP * kMaxQ, st));
    int rc = PYCI_GPU_OK;
    std::vector<double> tmp(static_cast<size_t>(kMaxGramP) * kMaxQ);
    for (int64_t i0 = 0; i0 < p && rc == PYCI_GPU_OK; i0 += kMaxGramP) {
        const int pp = static_cast<int>(std::min<int64_t>(kMaxGramP, p - i0));
        for (int64_t j0 = 0; j0 < q && rc == PYCI_GPU_OK; j0 += kMaxQ) {
            const int qq = static_cast<int>(std::min<int64_t>(kMaxQ, q - j0));
            const float *Ai = A + i0 * N, *Bj = B + j0 * N;
            unsigned nb;
            if (method == 1) {
                nb = launch_gram_tc(budget, st, Ai, pp, Bj, qq, N, partial);
            } else {
                nb = launch_gram_rows<float>(budget, st, Ai, pp, Bj, qq, N, partial);
                note_launch();
            }
            reduce_partials_kernel<<<pp * qq, 256, 0, st>>>(partial, nb, pp * qq, small), note_launch();
            cudaError_t e = cudaMemcpyAsync(tmp.data(), small, sizeof(double) * pp * qq, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = cuda_status(e, "Gram product");
                break;
            }
            if (method == 1 && gram_tc_error(true)) {
                set_error("tensor-core Gram product: MMA completion wait timed out");
                rc = PYCI_GPU_ECUDA;
                break;
            }
            for (int i = 0; i < pp; ++i)
                for (int j = 0; j < qq; ++j)
                    C[(i0 + i) * q + j0 + j] = tmp[static_cast<size_t>(i) * qq + j];
        }
    }
    cudaFreeAsync(partial, st);
    cudaFreeAsync(small, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == PYCI_GPU_OK && e != cudaSuccess)
        rc = cuda_status(e, "Gram product");
    return rc;
}

} // namespace pyci_gpu

using namespace pyci_gpu;

int davidson_solve(pyci_gpu_csr *csr, int64_t n, const double *c0, int64_t ncv, int64_t maxiter,
                   double tol, double ecore, int mode, double *evals, double *evecs,
                   pyci_gpu_solve_stats *stats) {
    const int64_t N = csr->nrow;
    // Ritz pairs tracked: the n wanted roots plus PYCI_GPU_DAVIDSON_EXTRA
    // guard pairs (default 1), never more than N - 1.  Convergence is tested
    // on the n wanted roots only, and each iteration adds corrections for at
    // most n roots.  Without a guard pair, a root whose start-vector overlap
    // is small can be passed over: the n tracked pairs converge to the roots
    // above it (seen on random FullCI Hamiltonians with nearly degenerate
    // 4th and 5th roots).
    int64_t extra = 1;
    if (const char *env = std::getenv("PYCI_GPU_DAVIDSON_EXTRA"))
        extra = std::max<int64_t>(0, std::atol(env));
    const int64_t b = std::max<int64_t>(n, std::min<int64_t>(n + extra, N - 1));
    // Subspace: 16 n vectors by default (64 for 4 roots).  A larger subspace
    // restarts less often; on random FullCI Hamiltonians 64 vectors keeping
    // 16 at each restart took ~30 % fewer iterations than 32 keeping 10.
    int64_t mmax = (ncv > 0) ? ncv : std::max<int64_t>(16 * n, 24);
    mmax = std::max<int64_t>(mmax, 2 * b + 2);
    if (N <= std::max<int64_t>(64, 3 * n) || N <= mmax)
        mmax = std::max<int64_t>(mmax, N); // full space: exact Rayleigh-Ritz
    mmax = std::min<int64_t>(mmax, std::max<int64_t>(N, 1));
    const int64_t blk = (mmax >= N) ? n : b;
    const int64_t iters = (maxiter > 0) ? maxiter : std::max<int64_t>(1000, 10 * n);
    if (mode == PYCI_SOLVE_MIXED) {
        int rc = csr_prepare_mixed_device(csr, 0);
        if (rc)
            return rc;
        Davidson<float> d(csr, blk, n, mmax, true);
        return d.run(c0, iters, tol, ecore, evals, evecs, stats);
    }
    if (!csr->vals && !(csr->hi && csr->lo) && !has_implicit(csr) && !csr->deferred) {
        set_error("operator has no values");
        return PYCI_GPU_EINVAL;
    }
    // Without FP64 values (dropped after the split, or a deferred CSR), the
    // FP64 products use high + low, equal to the FP64 values within 2^-48
    // relative (in double-float arithmetic on the implicit-column form).
    Davidson<double> d(csr, blk, n, mmax, false);
    return d.run(c0, iters, tol, ecore, evals, evecs, stats);
}
