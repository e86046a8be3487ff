// Batched eigensolve of many independent CI operators of uneven size.
//
// No counterpart in the reference, which solves one operator at a time
// (SparseOp::solve_ci, pyci/src/sparseop.cpp:114-146).  All problems advance
// in lockstep through the same block-Davidson iteration as davidson.cu, on
// vectors concatenated over problems (problem p owns rows [row0_p, row0_p +
// N_p) of every basis vector):
//   * one SpMM launch per iteration multiplies every active problem's block
//     (a block-diagonal product; each row group looks its problem up in the
//     row-offset table), replayed from a CUDA graph with fixed buffers;
//   * Gram products and linear combinations are segmented by problem;
//   * each problem's Rayleigh-Ritz, convergence test, thick restart and
//     dropping of dependent directions are its own; converged problems leave
//     the active set (their rows are skipped by the product).
// Mixed mode: FP32 values/vectors; at the end every problem's Ritz block is
// rebuilt in FP64 and Rayleigh-Ritz'd against the FP64 (high + low) operator.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

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

__device__ __forceinline__ int find_problem(const int64_t *row0, int nprob, int64_t r) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (row0[mid] <= r)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Y[r][0..K) = sum_e A_p[r][e] X[row0_p + col_e][0..K) for every row r of an
// active problem; rows of inactive problems are left untouched.
// VK: 0 = FP64 values, 1 = FP32 high part, 2 = FP64 from high + low.
template<int VK, int K, int LANES, typename XT>
__global__ void __launch_bounds__(256) batch_spmm_kernel(const BatchOp *__restrict__ ops, const int64_t *__restrict__ row0,
                                                         int nprob, int64_t ntotal, const int *__restrict__ active,
                                                         const XT *__restrict__ x, XT *__restrict__ y) {
    typedef typename std::conditional<VK == 1, float, double>::type acc_t;
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    for (int64_t r = group; r < ntotal; r += ngroups) {
        const int p = find_problem(row0, nprob, r);
        if (!active[p])
            continue;
        const BatchOp op = ops[p];
        const int64_t lr = r - op.row0;
        const int64_t start = op.rowptr[lr], end = op.rowptr[lr + 1];
        const XT *xb = x + op.row0 * K;
        acc_t acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            acc[k] = 0;
        for (int64_t e = start + lane; e < end; e += LANES) {
            const int64_t c = __ldcs(op.cols + e);
            acc_t v;
            if (VK == 0)
                v = static_cast<acc_t>(__ldcs(op.vals + e));
            else if (VK == 1)
                v = static_cast<acc_t>(__ldcs(op.hi + e));
            else
                v = static_cast<acc_t>(static_cast<double>(__ldcs(op.hi + e)) + static_cast<double>(__ldcs(op.lo + e)));
            const XT *xr = xb + c * K;
            if constexpr (K == 4 && sizeof(XT) == 4) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(xr));
                acc[0] += v * q.x;
                acc[1] += v * q.y;
                acc[2] += v * q.z;
                acc[3] += v * q.w;
            } else {
#pragma unroll
                for (int k = 0; k < K; ++k)
                    acc[k] += v * static_cast<acc_t>(__ldg(xr + k));
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1)
                acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o, LANES);
        }
        if (lane < K) {
            acc_t out = acc[0];
#pragma unroll
            for (int k = 1; k < K; ++k)
                if (lane == k)
                    out = acc[k];
            y[r * K + lane] = static_cast<XT>(out);
        }
    }
}

// Xi[r][0..K) from the K vectors V[j][r] (zero past k).
template<typename T, int K>
__global__ void batch_pack_kernel(const T *__restrict__ V, int64_t N, int k, T *__restrict__ Xi) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
#pragma unroll
        for (int j = 0; j < K; ++j)
            Xi[r * K + j] = (j < k) ? V[j * N + r] : T(0);
}

template<typename T, int K>
__global__ void batch_unpack_kernel(const T *__restrict__ Yi, int64_t N, int k, T *__restrict__ W) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        for (int j = 0; j < k; ++j)
            W[j * N + r] = Yi[r * K + j];
}

// Segmented Gram product.  Tile t covers rows [tile_lo[t], tile_hi[t]) of one
// problem; partial[t][i * q + j] = sum over those rows of A[i][r] * B[j][r].
constexpr int kSegTile = 32;
constexpr int kSegMaxP = 64;
constexpr int kSegMaxQ = 8;

template<typename T>
__global__ void __launch_bounds__(256) seg_gram_kernel(const T *__restrict__ A, int p, const T *__restrict__ B, int q,
                                                       int64_t N, const int64_t *__restrict__ tile_lo,
                                                       const int64_t *__restrict__ tile_hi, int ntiles,
                                                       double *__restrict__ partial) {
    __shared__ T sa[kSegMaxP][kSegTile + 1];
    __shared__ T sb[kSegMaxQ][kSegTile + 1];
    const int pq = p * q;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int64_t r0 = tile_lo[t]; r0 < tile_hi[t]; r0 += kSegTile) {
            const int64_t rend = tile_hi[t];
            for (int e = threadIdx.x; e < p * kSegTile; e += blockDim.x) {
                const int i = e / kSegTile, c = e % kSegTile;
                sa[i][c] = (r0 + c < rend) ? A[i * N + r0 + c] : T(0);
            }
            for (int e = threadIdx.x; e < q * kSegTile; e += blockDim.x) {
                const int j = e / kSegTile, c = e % kSegTile;
                sb[j][c] = (r0 + c < rend) ? B[j * N + r0 + c] : T(0);
            }
            __syncthreads();
            int slot = 0;
            for (int idx = threadIdx.x; idx < pq; idx += blockDim.x, ++slot) {
                const int i = idx / q, j = idx % q;
                T s = 0;
#pragma unroll 8
                for (int c = 0; c < kSegTile; ++c)
                    s += sa[i][c] * sb[j][c];
                acc[slot] += static_cast<double>(s);
            }
            __syncthreads();
        }
        int slot = 0;
        for (int idx = threadIdx.x; idx < pq; idx += blockDim.x, ++slot)
            partial[static_cast<int64_t>(t) * pq + idx] = acc[slot];
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

// out[j][r] = beta * out[j][r] + sum_i Y[prob(r)][i * q + j] * V[i][r].
template<typename TV, typename TO, typename ACC>
__global__ void __launch_bounds__(256) seg_combine_kernel(const TV *__restrict__ V, int p, int64_t N,
                                                          const double *__restrict__ Y, int q, double beta,
                                                          const int64_t *__restrict__ row0, int nprob,
                                                          TO *__restrict__ out) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int prob = find_problem(row0, nprob, r);
        const double *Yp = Y + static_cast<int64_t>(prob) * p * q;
        ACC acc[kSegMaxQ];
#pragma unroll
        for (int j = 0; j < kSegMaxQ; ++j)
            acc[j] = 0;
        for (int i = 0; i < p; ++i) {
            const ACC v = static_cast<ACC>(V[i * N + r]);
#pragma unroll
            for (int j = 0; j < kSegMaxQ; ++j)
                if (j < q)
                    acc[j] += static_cast<ACC>(__ldg(&Yp[i * q + j])) * v;
        }
#pragma unroll
        for (int j = 0; j < kSegMaxQ; ++j)
            if (j < q) {
                TO *o = out + j * N + r;
                *o = (beta == 0.0) ? static_cast<TO>(acc[j]) : static_cast<TO>(static_cast<ACC>(*o) + acc[j]);
            }
    }
}

// R[j][r] = AX[j][r] - theta[prob(r)][j] X[j][r]
template<typename T>
__global__ void seg_residual_kernel(const T *__restrict__ AX, const T *__restrict__ X, const double *__restrict__ theta,
                                    int q, int64_t N, const int64_t *__restrict__ row0, int nprob, T *__restrict__ R) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int prob = find_problem(row0, nprob, r);
        for (int j = 0; j < q; ++j)
            R[j * N + r] = static_cast<T>(static_cast<double>(AX[j * N + r]) -
                                          theta[prob * q + j] * static_cast<double>(X[j * N + r]));
    }
}

// out[j][r] = use[prob][j] ? R[j][r] / (theta[prob][j] - D[r]) : 0
template<typename T>
__global__ void seg_precondition_kernel(const T *__restrict__ R, const double *__restrict__ theta,
                                        const int *__restrict__ use, const double *__restrict__ diag, int q,
                                        int64_t N, const int64_t *__restrict__ row0, int nprob, T *__restrict__ out) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < N;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int prob = find_problem(row0, nprob, r);
        const double d = diag[r];
        for (int j = 0; j < q; ++j) {
            double den = theta[prob * q + j] - d;
            if (fabs(den) < 1e-8)
                den = (den < 0.0) ? -1e-8 : 1e-8;
            out[j * N + r] = use[prob * q + j] ? static_cast<T>(static_cast<double>(R[j * N + r]) / den) : T(0);
        }
    }
}

template<typename TI, typename TO>
__global__ void batch_convert_kernel(const TI *__restrict__ in, TO *__restrict__ out, int64_t n) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[r] = static_cast<TO>(in[r]);
}

__global__ void set_units_kernel(float *Vf, double *Vd, int64_t N, const int64_t *pos, int count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) {
        // pos[t] = slot * N + row
        if (Vf)
            Vf[pos[t]] = 1.0f;
        if (Vd)
            Vd[pos[t]] = 1.0;
    }
}

} // namespace pyci_gpu

using namespace pyci_gpu;

namespace {

// Host-side state of the batched solver.
template<typename T>
class Batch {
public:
    Batch(pyci_gpu_ctx *ctx, std::vector<pyci_gpu_csr *> ops, int nroot, int mmax, bool mixed)
        : ctx_(ctx), st_(ctx->stream), ops_(std::move(ops)), P_(static_cast<int>(ops_.size())), b_(nroot),
          mmax_(mmax), mixed_(mixed) {}

    ~Batch() {
        if (graph_exec_)
            cudaGraphExecDestroy(graph_exec_);
        for (void *p : allocs_)
            cudaFreeAsync(p, st_);
        cudaStreamSynchronize(st_);
    }

    int run(int64_t maxiter, double tol, const double *ecore, double *evals, pyci_gpu_solve_stats *stats);

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

    // G[prob] (p x q, row-major) = A^T B segment by segment; A has p vectors, B q.
    template<typename U>
    int gram(const U *A, int p, const U *B, int q, std::vector<double> &G) {
        G.assign(static_cast<size_t>(P_) * p * q, 0.0);
        for (int i0 = 0; i0 < p; i0 += kSegMaxP) {
            const int pp = std::min(kSegMaxP, p - i0);
            for (int j0 = 0; j0 < q; j0 += kSegMaxQ) {
                const int qq = std::min(kSegMaxQ, q - j0);
                const unsigned nb = static_cast<unsigned>(std::min<int64_t>(ntiles_, ctx_->num_sms * 8));
                seg_gram_kernel<U><<<nb, 256, 0, st_>>>(A + static_cast<int64_t>(i0) * N_, pp, B + static_cast<int64_t>(j0) * N_,
                                                        qq, N_, d_tile_lo_, d_tile_hi_, ntiles_, d_partial_),
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

    // out[j] = beta out[j] + sum_i Y[prob][i][j] V[i] (Y host: [P][p][q]).
    template<typename TV, typename TO, typename ACC>
    int combine(const TV *V, int p, const std::vector<double> &Y, int q, double beta, TO *out) {
        if (p > kSegMaxP * 4 || q > kSegMaxQ) {
            set_error("batched combine: p = %d, q = %d beyond limits", p, q);
            return PYCI_GPU_EUNSUPPORTED;
        }
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_coef_, Y.data(), sizeof(double) * Y.size(), cudaMemcpyHostToDevice, st_));
        seg_combine_kernel<TV, TO, ACC><<<grid(N_), 256, 0, st_>>>(V, p, N_, d_coef_, q, beta, d_row0_, P_, out),
            ::pyci_gpu::note_launch();
        return PYCI_GPU_OK;
    }

    // W_new = H V_new for the b-vector block in Tnew_ -> Wnew_ (graph replay).
    int apply_block(int prec);

    pyci_gpu_ctx *ctx_;
    cudaStream_t st_;
    std::vector<pyci_gpu_csr *> ops_;
    int P_, b_, mmax_;
    bool mixed_;
    int64_t N_ = 0;
    int ntiles_ = 0;
    std::vector<void *> allocs_;
    std::vector<int64_t> row0_;
    int64_t *d_row0_ = nullptr, *d_tile_lo_ = nullptr, *d_tile_hi_ = nullptr;
    int *d_tile_begin_ = nullptr, *d_active_ = nullptr, *d_use_ = nullptr;
    double *d_partial_ = nullptr, *d_small_ = nullptr, *d_coef_ = nullptr, *d_theta_ = nullptr, *d_diag_ = nullptr;
    BatchOp *d_ops_ = nullptr;
    T *Tnew_ = nullptr, *Wnew_ = nullptr, *Xi_ = nullptr, *Yi_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_prec_ = -1;
    bool all_vals_ = true;
    int64_t matvecs_ = 0, launches_graph_ = 0;
    double spmm_ms_ = 0.0;
};

template<typename T>
int Batch<T>::apply_block(int prec) {
    // One graph: pack the block, one batched SpMM over every active problem,
    // unpack.  Buffers are fixed, so the graph is captured once per precision.
    if (prec == PYCI_PREC_FP64 && !all_vals_)
        prec = PYCI_PREC_FP64_SPLIT;
    if (!graph_exec_ || graph_prec_ != prec) {
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        cudaGraph_t g;
        PYCI_CUDA_TRY(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        const unsigned gr = grid(N_);
        batch_pack_kernel<T, 4><<<gr, 256, 0, st_>>>(Tnew_, N_, b_, Xi_);
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ctx_->num_sms * 32, (N_ * 32 + 255) / 256));
        if (prec == PYCI_PREC_FP32)
            batch_spmm_kernel<1, 4, 32, T><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, d_row0_, P_, N_, d_active_, Xi_, Yi_);
        else if (prec == PYCI_PREC_FP64_SPLIT)
            batch_spmm_kernel<2, 4, 32, T><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, d_row0_, P_, N_, d_active_, Xi_, Yi_);
        else
            batch_spmm_kernel<0, 4, 32, T><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, d_row0_, P_, N_, d_active_, Xi_, Yi_);
        batch_unpack_kernel<T, 4><<<gr, 256, 0, st_>>>(Yi_, N_, b_, Wnew_);
        cudaError_t e = cudaStreamEndCapture(st_, &g);
        if (e != cudaSuccess)
            return cuda_status(e, "graph capture");
        e = cudaGraphInstantiate(&graph_exec_, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess)
            return cuda_status(e, "graph instantiate");
        graph_prec_ = prec;
    }
    cudaEvent_t a, c;
    cudaEventCreate(&a);
    cudaEventCreate(&c);
    cudaEventRecord(a, st_);
    PYCI_CUDA_TRY(cudaGraphLaunch(graph_exec_, st_));
    ::pyci_gpu::note_launch();
    ::pyci_gpu::note_launch();
    ::pyci_gpu::note_launch();
    cudaEventRecord(c, st_);
    PYCI_CUDA_TRY(cudaEventSynchronize(c));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, c);
    spmm_ms_ += ms;
    cudaEventDestroy(a);
    cudaEventDestroy(c);
    ++launches_graph_;
    return PYCI_GPU_OK;
}

template<typename T>
int Batch<T>::run(int64_t maxiter, double tol, const double *ecore, double *evals, pyci_gpu_solve_stats *stats) {
    const auto t_start = std::chrono::steady_clock::now();
    const int b = b_, P = P_, mmax = mmax_;
    int rc;
    // Problem layout and tiles.
    row0_.assign(P + 1, 0);
    for (int p = 0; p < P; ++p)
        row0_[p + 1] = row0_[p] + ops_[p]->nrow;
    N_ = row0_[P];
    const int64_t N = N_;
    std::vector<int64_t> tlo, thi;
    std::vector<int> tbeg(P + 1, 0);
    const int64_t tile = 8192;
    for (int p = 0; p < P; ++p) {
        tbeg[p] = static_cast<int>(tlo.size());
        for (int64_t r = row0_[p]; r < row0_[p + 1]; r += tile) {
            tlo.push_back(r);
            thi.push_back(std::min(r + tile, row0_[p + 1]));
        }
    }
    tbeg[P] = static_cast<int>(tlo.size());
    ntiles_ = static_cast<int>(tlo.size());
    for (int p = 0; p < P; ++p)
        all_vals_ = all_vals_ && ops_[p]->vals;
    std::vector<BatchOp> hops(P);
    for (int p = 0; p < P; ++p)
        hops[p] = BatchOp{ops_[p]->rowptr, ops_[p]->cols, ops_[p]->vals, ops_[p]->hi, ops_[p]->lo, row0_[p], ops_[p]->nrow};

    T *V, *W, *X, *AX, *R, *Xk, *Wk, *Xfinal;
    const int nkeep = std::max(b, std::min(mmax - b, 2 * b));
    if ((rc = alloc(&V, static_cast<int64_t>(mmax) * N)) || (rc = alloc(&W, static_cast<int64_t>(mmax) * N)) ||
        (rc = alloc(&X, static_cast<int64_t>(b) * N)) || (rc = alloc(&AX, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&R, static_cast<int64_t>(b) * N)) || (rc = alloc(&Xk, static_cast<int64_t>(nkeep) * N)) ||
        (rc = alloc(&Wk, static_cast<int64_t>(nkeep) * N)) || (rc = alloc(&Xfinal, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&Tnew_, static_cast<int64_t>(b) * N)) || (rc = alloc(&Wnew_, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&Xi_, N * 4)) || (rc = alloc(&Yi_, N * 4)) ||
        (rc = alloc(&d_row0_, P + 1)) || (rc = alloc(&d_tile_lo_, ntiles_)) || (rc = alloc(&d_tile_hi_, ntiles_)) ||
        (rc = alloc(&d_tile_begin_, P + 1)) || (rc = alloc(&d_active_, P)) || (rc = alloc(&d_use_, P * b)) ||
        (rc = alloc(&d_partial_, static_cast<int64_t>(ntiles_) * kSegMaxP * kSegMaxQ)) ||
        (rc = alloc(&d_small_, static_cast<int64_t>(P) * kSegMaxP * kSegMaxQ)) ||
        (rc = alloc(&d_coef_, static_cast<int64_t>(P) * mmax * std::max(mmax, kSegMaxQ))) ||
        (rc = alloc(&d_theta_, static_cast<int64_t>(P) * b)) || (rc = alloc(&d_diag_, N)) || (rc = alloc(&d_ops_, P)))
        return rc;
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_row0_, row0_.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_lo_, tlo.data(), sizeof(int64_t) * ntiles_, cudaMemcpyHostToDevice, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_hi_, thi.data(), sizeof(int64_t) * ntiles_, cudaMemcpyHostToDevice, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_tile_begin_, tbeg.data(), sizeof(int) * (P + 1), cudaMemcpyHostToDevice, st_));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_ops_, hops.data(), sizeof(BatchOp) * P, cudaMemcpyHostToDevice, st_));
    for (int p = 0; p < P; ++p)
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_diag_ + row0_[p], ops_[p]->diag, sizeof(double) * ops_[p]->nrow,
                                      cudaMemcpyDeviceToDevice, st_));
    std::vector<int> active(P, 1);
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_active_, active.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st_));

    // Initial block: unit vectors on each problem's b lowest diagonal elements.
    std::vector<double> diag(N);
    PYCI_CUDA_TRY(cudaMemcpyAsync(diag.data(), d_diag_, sizeof(double) * N, cudaMemcpyDeviceToHost, st_));
    PYCI_CUDA_TRY(cudaMemsetAsync(Tnew_, 0, sizeof(T) * b * N, st_));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
    std::vector<int64_t> pos;
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
            pos.push_back(static_cast<int64_t>(j) * N + row0_[p] + order[j]);
    }
    int64_t *d_pos;
    if ((rc = alloc(&d_pos, static_cast<int64_t>(pos.size()))))
        return rc;
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_pos, pos.data(), sizeof(int64_t) * pos.size(), cudaMemcpyHostToDevice, st_));
    set_units_kernel<<<static_cast<unsigned>((pos.size() + 255) / 256), 256, 0, st_>>>(
        sizeof(T) == 4 ? reinterpret_cast<float *>(Tnew_) : nullptr,
        sizeof(T) == 8 ? reinterpret_cast<double *>(Tnew_) : nullptr, N, d_pos, static_cast<int>(pos.size())),
        ::pyci_gpu::note_launch();

    // Per-problem Davidson state.
    std::vector<std::vector<double>> G(P, std::vector<double>(static_cast<size_t>(mmax) * mmax, 0.0));
    std::vector<std::vector<char>> valid(P, std::vector<char>(mmax, 0));
    std::vector<std::vector<double>> theta_final(P);
    std::vector<double> theta_all(static_cast<size_t>(P) * b, 0.0);
    std::vector<int> use(static_cast<size_t>(P) * b, 1);
    for (int p = 0; p < P; ++p)
        for (int j = 0; j < b; ++j)
            use[p * b + j] = (j < ops_[p]->nrow) ? 1 : 0;
    const double eps23 = std::pow(std::numeric_limits<double>::epsilon(), 2.0 / 3.0);
    const double floor_ = mixed_ ? 1e-5 : 0.0;
    const int prec = mixed_ ? PYCI_PREC_FP32 : PYCI_PREC_FP64;
    int m = 0;
    int64_t iter = 0;
    int nactive = P;
    std::vector<double> Gc;
    for (iter = 0; iter < maxiter && nactive > 0; ++iter) {
        // New block (in Tnew_, already orthonormal): W_new = H T_new, then append.
        if ((rc = apply_block(prec)))
            return rc;
        matvecs_ += static_cast<int64_t>(nactive) * b;
        PYCI_CUDA_TRY(cudaMemcpyAsync(V + static_cast<int64_t>(m) * N, Tnew_, sizeof(T) * b * N, cudaMemcpyDeviceToDevice, st_));
        PYCI_CUDA_TRY(cudaMemcpyAsync(W + static_cast<int64_t>(m) * N, Wnew_, sizeof(T) * b * N, cudaMemcpyDeviceToDevice, st_));
        for (int p = 0; p < P; ++p)
            for (int j = 0; j < b; ++j)
                valid[p][m + j] = active[p] ? static_cast<char>(use[p * b + j]) : 0;
        if ((rc = gram<T>(V, m + b, W + static_cast<int64_t>(m) * N, b, Gc)))
            return rc;
        for (int p = 0; p < P; ++p)
            for (int i = 0; i < m + b; ++i)
                for (int j = 0; j < b; ++j) {
                    const double g = Gc[(static_cast<size_t>(p) * (m + b) + i) * b + j];
                    G[p][static_cast<size_t>(i) * mmax + m + j] = g;
                    G[p][static_cast<size_t>(m + j) * mmax + i] = g;
                }
        m += b;
        // Rayleigh-Ritz per active problem over its valid slots.
        std::vector<double> Yb(static_cast<size_t>(P) * m * b, 0.0), Yk(static_cast<size_t>(P) * m * nkeep, 0.0);
        std::vector<int> nvalid(P, 0);
        for (int p = 0; p < P; ++p) {
            if (!active[p])
                continue;
            std::vector<int> idx;
            for (int i = 0; i < m; ++i)
                if (valid[p][i])
                    idx.push_back(i);
            const int mv = static_cast<int>(idx.size());
            nvalid[p] = mv;
            std::vector<double> Gm(static_cast<size_t>(mv) * mv), th, Y;
            for (int i = 0; i < mv; ++i)
                for (int j = 0; j < mv; ++j)
                    Gm[static_cast<size_t>(i) * mv + j] = G[p][static_cast<size_t>(idx[i]) * mmax + idx[j]];
            if (!symmetric_eigen(mv, Gm, th, Y)) {
                set_error("Rayleigh-Ritz eigensolver failed (problem %d)", p);
                return PYCI_GPU_ENOCONV;
            }
            for (int j = 0; j < b; ++j) {
                theta_all[p * b + j] = (j < mv) ? th[j] : 0.0;
                if (j < mv)
                    for (int i = 0; i < mv; ++i)
                        Yb[(static_cast<size_t>(p) * m + idx[i]) * b + j] = Y[static_cast<size_t>(i) * mv + j];
            }
            for (int j = 0; j < std::min(nkeep, mv); ++j)
                for (int i = 0; i < mv; ++i)
                    Yk[(static_cast<size_t>(p) * m + idx[i]) * nkeep + j] = Y[static_cast<size_t>(i) * mv + j];
            theta_final[p].assign(th.begin(), th.begin() + std::min(mv, b));
        }
        if ((rc = combine<T, T, T>(V, m, Yb, b, 0.0, X)) || (rc = combine<T, T, T>(W, m, Yb, b, 0.0, AX)))
            return rc;
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_theta_, theta_all.data(), sizeof(double) * P * b, cudaMemcpyHostToDevice, st_));
        seg_residual_kernel<T><<<grid(N), 256, 0, st_>>>(AX, X, d_theta_, b, N, d_row0_, P, R), ::pyci_gpu::note_launch();
        if ((rc = gram<T>(R, b, R, b, Gc)))
            return rc;
        for (int p = 0; p < P; ++p) {
            if (!active[p])
                continue;
            bool done = true;
            for (int j = 0; j < b; ++j) {
                const double rn = std::sqrt(std::max(Gc[(static_cast<size_t>(p) * b + j) * b + j], 0.0));
                double thr = std::max(tol * std::max(eps23, std::fabs(theta_all[p * b + j])), floor_);
                const bool conv = !(j < ops_[p]->nrow) || rn <= thr || nvalid[p] >= ops_[p]->nrow;
                use[p * b + j] = conv ? 0 : 1;
                done = done && conv;
            }
            if (done) {
                // Keep this problem's Ritz vectors for the final FP64 step.
                active[p] = 0;
                --nactive;
                for (int j = 0; j < b; ++j)
                    PYCI_CUDA_TRY(cudaMemcpyAsync(Xfinal + static_cast<int64_t>(j) * N + row0_[p],
                                                  X + static_cast<int64_t>(j) * N + row0_[p],
                                                  sizeof(T) * ops_[p]->nrow, cudaMemcpyDeviceToDevice, st_));
                for (int j = 0; j < b; ++j)
                    use[p * b + j] = 0;
            }
        }
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_active_, active.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st_));
        if (nactive == 0)
            break;
        // Thick restart (all problems together) when the next block does not fit.
        if (m + b > mmax) {
            if ((rc = combine<T, T, T>(V, m, Yk, nkeep, 0.0, Xk)) || (rc = combine<T, T, T>(W, m, Yk, nkeep, 0.0, Wk)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(V, Xk, sizeof(T) * nkeep * N, cudaMemcpyDeviceToDevice, st_));
            PYCI_CUDA_TRY(cudaMemcpyAsync(W, Wk, sizeof(T) * nkeep * N, cudaMemcpyDeviceToDevice, st_));
            for (int p = 0; p < P; ++p) {
                std::fill(G[p].begin(), G[p].end(), 0.0);
                std::fill(valid[p].begin(), valid[p].end(), 0);
                if (!active[p])
                    continue;
                // Ritz values of the kept vectors (recomputed from the last RR).
                const int kept = std::min(nkeep, nvalid[p]);
                std::vector<int> idx;
                for (int i = 0; i < m; ++i)
                    idx.push_back(i);
                for (int j = 0; j < kept; ++j) {
                    valid[p][j] = 1;
                }
            }
            // Projected matrix of the kept Ritz vectors: diagonal of their Ritz values.
            if ((rc = gram<T>(V, nkeep, W, nkeep, Gc)))
                return rc;
            for (int p = 0; p < P; ++p)
                for (int i = 0; i < nkeep; ++i)
                    for (int j = 0; j < nkeep; ++j)
                        G[p][static_cast<size_t>(i) * mmax + j] = valid[p][i] && valid[p][j]
                                                                      ? Gc[(static_cast<size_t>(p) * nkeep + i) * nkeep + j]
                                                                      : 0.0;
            m = nkeep;
        }
        // Corrections of unconverged roots of active problems into Tnew_.
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_use_, use.data(), sizeof(int) * P * b, cudaMemcpyHostToDevice, st_));
        seg_precondition_kernel<T><<<grid(N), 256, 0, st_>>>(R, d_theta_, d_use_, d_diag_, b, N, d_row0_, P, Tnew_),
            ::pyci_gpu::note_launch();
        // Two passes of segmented block Gram-Schmidt against the basis.
        for (int pass = 0; pass < 2; ++pass) {
            if ((rc = gram<T>(V, m, Tnew_, b, Gc)))
                return rc;
            std::vector<double> C(static_cast<size_t>(P) * m * b, 0.0);
            for (int p = 0; p < P; ++p)
                for (int i = 0; i < m; ++i)
                    if (valid[p][i])
                        for (int j = 0; j < b; ++j)
                            C[(static_cast<size_t>(p) * m + i) * b + j] = -Gc[(static_cast<size_t>(p) * m + i) * b + j];
            if ((rc = combine<T, T, T>(V, m, C, b, 1.0, Tnew_)))
                return rc;
        }
        // Cholesky QR (twice) inside each problem's block, dropping dependent vectors.
        for (int pass = 0; pass < 2; ++pass) {
            if ((rc = gram<T>(Tnew_, b, Tnew_, b, Gc)))
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
                for (int i = 0; i < b; ++i)
                    for (int j = 0; j < b; ++j)
                        Y[(static_cast<size_t>(p) * b + i) * b + j] = Li[j * b + i];
            }
            if ((rc = combine<T, T, T>(Tnew_, b, Y, b, 0.0, Xk)))
                return rc;
            PYCI_CUDA_TRY(cudaMemcpyAsync(Tnew_, Xk, sizeof(T) * b * N, cudaMemcpyDeviceToDevice, st_));
        }
    }
    if (nactive > 0) {
        set_error("did not converge (%d of %d problems)", nactive, P);
        return PYCI_GPU_ENOCONV;
    }
    // Final Rayleigh-Ritz of every problem's Ritz block against the FP64
    // operator (high + low in mixed mode).
    double *X64, *AX64, *Xi64, *Yi64;
    if ((rc = alloc(&X64, static_cast<int64_t>(b) * N)) || (rc = alloc(&AX64, static_cast<int64_t>(b) * N)) ||
        (rc = alloc(&Xi64, N * 4)) || (rc = alloc(&Yi64, N * 4)))
        return rc;
    batch_convert_kernel<T, double><<<grid(static_cast<int64_t>(b) * N), 256, 0, st_>>>(Xfinal, X64, static_cast<int64_t>(b) * N),
        ::pyci_gpu::note_launch();
    std::fill(active.begin(), active.end(), 1);
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_active_, active.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st_));
    {
        const unsigned gr = grid(N);
        batch_pack_kernel<double, 4><<<gr, 256, 0, st_>>>(X64, N, b, Xi64), ::pyci_gpu::note_launch();
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ctx_->num_sms * 32, (N * 32 + 255) / 256));
        bool split = !all_vals_;
        if (mixed_)
            split = true;
        if (split)
            batch_spmm_kernel<2, 4, 32, double><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, d_row0_, P, N, d_active_, Xi64, Yi64),
                ::pyci_gpu::note_launch();
        else
            batch_spmm_kernel<0, 4, 32, double><<<static_cast<unsigned>(blocks), 256, 0, st_>>>(d_ops_, d_row0_, P, N, d_active_, Xi64, Yi64),
                ::pyci_gpu::note_launch();
        batch_unpack_kernel<double, 4><<<gr, 256, 0, st_>>>(Yi64, N, b, AX64), ::pyci_gpu::note_launch();
        matvecs_ += static_cast<int64_t>(P) * b;
    }
    std::vector<double> S64, H64;
    if ((rc = gram<double>(X64, b, X64, b, S64)) || (rc = gram<double>(X64, b, AX64, b, H64)))
        return rc;
    for (int p = 0; p < P; ++p) {
        // Generalised b x b problem H y = e S y via S^{-1/2}.
        const int n = static_cast<int>(std::min<int64_t>(b, ops_[p]->nrow));
        std::vector<double> S(static_cast<size_t>(n) * n), H(static_cast<size_t>(n) * n), se, sv;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                S[i * n + j] = S64[(static_cast<size_t>(p) * b + i) * b + j];
                H[i * n + j] = H64[(static_cast<size_t>(p) * b + i) * b + j];
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
        // Decreasing order, ecore added (the reference's result order).
        for (int c = 0; c < b; ++c)
            evals[static_cast<size_t>(p) * b + c] = (c < n) ? e[n - 1 - c] + ecore[p] : 0.0;
    }
    PYCI_CUDA_TRY(cudaStreamSynchronize(st_));
    if (stats) {
        stats->iterations = iter + 1;
        stats->matvecs = matvecs_;
        stats->matvecs_fp64 = mixed_ ? static_cast<int64_t>(P) * b : matvecs_;
        stats->restarts = 0;
        stats->refinements = 1;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->seconds_spmm = spmm_ms_ * 1e-3;
        stats->max_residual = 0.0;
    }
    return PYCI_GPU_OK;
}

} // namespace

extern "C" int pyci_gpu_batch_solve(pyci_gpu_ctx *ctx, int64_t nprob, pyci_gpu_csr *const *ops, int64_t n,
                                    int64_t maxiter, double tol, const double *ecore, int mode, double *evals,
                                    pyci_gpu_solve_stats *stats) {
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
    const int mmax = 32;
    if (mode == PYCI_SOLVE_MIXED) {
        for (auto *c : v) {
            int rc = csr_prepare_mixed_device(c, 0);
            if (rc)
                return rc;
        }
        Batch<float> bsolve(ctx, v, static_cast<int>(n), mmax, true);
        return bsolve.run(iters, tol, ecore, evals, stats);
    }
    for (auto *c : v)
        if (!c->vals && !(c->hi && c->lo)) {
            set_error("FP64 batched solve needs FP64 values");
            return PYCI_GPU_EINVAL;
        }
    Batch<double> bsolve(ctx, v, static_cast<int>(n), mmax, false);
    return bsolve.run(iters, tol, ecore, evals, stats);
}
