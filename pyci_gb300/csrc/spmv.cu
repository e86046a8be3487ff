// Sparse matrix times a block of vectors (SpMV / SpMM) for the CI
// Hamiltonian's device CSR, replacing SparseOp::perform_op(_symm)
// (pyci/src/sparseop.cpp:96-112), which the reference evaluates with Eigen on
// one core.
//
// The product is HBM-bound: each stored entry is read once (4-byte column +
// 8- or 4-byte value) while the vector block x ([ncol][k], interleaved) is
// gathered from L2.  A group of LANES threads owns one row; lanes stream the
// row's entries with 16-byte vector loads (evict-first, so the matrix does not
// push x out of L2), each lane keeps k accumulators, and a butterfly shuffle
// reduces them.  Symmetric operators store both triangles, so no scatter or
// atomics are needed and results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "internal.h"

namespace pyci_gpu {

enum ValueKind { kF64 = 0, kF32 = 1, kSplit = 2, kSplitDF = 3 };

template<int VK>
struct Values;

template<>
struct Values<kF64> {
    typedef double acc_t;
    typedef double x_t;
    const double *v;
    __device__ __forceinline__ double at(int64_t e) const { return __ldcs(v + e); }
    __device__ __forceinline__ void quad(int64_t e, double out[4]) const {
        const double2 a = __ldcs(reinterpret_cast<const double2 *>(v + e));
        const double2 b = __ldcs(reinterpret_cast<const double2 *>(v + e + 2));
        out[0] = a.x;
        out[1] = a.y;
        out[2] = b.x;
        out[3] = b.y;
    }
};

template<>
struct Values<kF32> {
    typedef float acc_t;
    typedef float x_t;
    const float *v;
    __device__ __forceinline__ float at(int64_t e) const { return __ldcs(v + e); }
    __device__ __forceinline__ void quad(int64_t e, float out[4]) const {
        const float4 a = __ldcs(reinterpret_cast<const float4 *>(v + e));
        out[0] = a.x;
        out[1] = a.y;
        out[2] = a.z;
        out[3] = a.w;
    }
};

template<>
struct Values<kSplit> {
    typedef double acc_t;
    typedef double x_t;
    const float *hi, *lo;
    __device__ __forceinline__ double at(int64_t e) const {
        return static_cast<double>(__ldcs(hi + e)) + static_cast<double>(__ldcs(lo + e));
    }
    __device__ __forceinline__ void quad(int64_t e, double out[4]) const {
        const float4 a = __ldcs(reinterpret_cast<const float4 *>(hi + e));
        const float4 b = __ldcs(reinterpret_cast<const float4 *>(lo + e));
        out[0] = static_cast<double>(a.x) + static_cast<double>(b.x);
        out[1] = static_cast<double>(a.y) + static_cast<double>(b.y);
        out[2] = static_cast<double>(a.z) + static_cast<double>(b.z);
        out[3] = static_cast<double>(a.w) + static_cast<double>(b.w);
    }
};

// Gather one row of the interleaved vector block x (K consecutive elements).
// With VEC the row is read with 8- or 16-byte vector loads (the caller has
// checked alignment); otherwise element by element.
template<bool VEC, int K, typename XT, typename AT>
__device__ __forceinline__ void load_x(const XT *__restrict__ xr, AT out[K]) {
    constexpr int BYTES = K * static_cast<int>(sizeof(XT));
    if constexpr (VEC && BYTES % 16 == 0) {
        constexpr int NV = BYTES / 16;
        constexpr int PER = 16 / static_cast<int>(sizeof(XT));
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            if constexpr (sizeof(XT) == 4) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(xr) + v);
                out[v * PER + 0] = static_cast<AT>(q.x);
                out[v * PER + 1] = static_cast<AT>(q.y);
                out[v * PER + 2] = static_cast<AT>(q.z);
                out[v * PER + 3] = static_cast<AT>(q.w);
            } else {
                const double2 q = __ldg(reinterpret_cast<const double2 *>(xr) + v);
                out[v * PER + 0] = static_cast<AT>(q.x);
                out[v * PER + 1] = static_cast<AT>(q.y);
            }
        }
    } else if constexpr (VEC && BYTES == 8 && sizeof(XT) == 4) {
        const float2 q = __ldg(reinterpret_cast<const float2 *>(xr));
        out[0] = static_cast<AT>(q.x);
        out[1] = static_cast<AT>(q.y);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
            out[k] = static_cast<AT>(__ldg(xr + k));
    }
}

// MAP 0: each lane owns 4 consecutive entries per step (16-byte loads of
// columns and values); MAP 1: lane l owns entries l, l + LANES, ... so one
// gather instruction covers LANES consecutive columns of the sorted row,
// which share 32-byte sectors more often.  The autotuner picks per operator.
template<int VK, int K, int LANES, bool VEC, int MAP>
__global__ void __launch_bounds__(256) spmm_kernel(int64_t nrow, const int64_t *__restrict__ rowptr,
                                                   const int32_t *__restrict__ cols, Values<VK> vals,
                                                   const typename Values<VK>::x_t *__restrict__ x,
                                                   int64_t ldx,
                                                   typename Values<VK>::x_t *__restrict__ y,
                                                   int64_t ldy) {
    typedef typename Values<VK>::acc_t acc_t;
    typedef typename Values<VK>::x_t x_t;
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    for (int64_t r = group; r < nrow; r += ngroups) {
        const int64_t start = rowptr[r], end = rowptr[r + 1];
        acc_t acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            acc[k] = 0;
        acc_t xv[K];
        if (MAP == 1) {
#pragma unroll 4
            for (int64_t e = start + lane; e < end; e += LANES) {
                const int64_t c = __ldcs(cols + e);
                const acc_t v = vals.at(e);
                load_x<VEC, K>(x + c * ldx, xv);
#pragma unroll
                for (int k = 0; k < K; ++k)
                    acc[k] += v * xv[k];
            }
        } else {
        // Head: entries before the first 4-aligned index.
        const int64_t a0 = min(end, (start + 3) & ~static_cast<int64_t>(3));
        const int64_t a1 = max(a0, end & ~static_cast<int64_t>(3));
        if (start + lane < a0) {
            const int64_t e = start + lane;
            const int64_t c = __ldcs(cols + e);
            const acc_t v = vals.at(e);
            load_x<VEC, K>(x + c * ldx, xv);
#pragma unroll
            for (int k = 0; k < K; ++k)
                acc[k] += v * xv[k];
        }
        // Body: 4 entries per lane per step, 16-byte loads of columns and values.
        for (int64_t e = a0 + 4 * lane; e < a1; e += 4 * LANES) {
            const int4 c4 = __ldcs(reinterpret_cast<const int4 *>(cols + e));
            acc_t v[4];
            vals.quad(e, v);
            const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                load_x<VEC, K>(x + static_cast<int64_t>(cc[q]) * ldx, xv);
#pragma unroll
                for (int k = 0; k < K; ++k)
                    acc[k] += v[q] * xv[k];
            }
        }
        // Tail.
        if (a1 + lane < end) {
            const int64_t e = a1 + lane;
            const int64_t c = __ldcs(cols + e);
            const acc_t v = vals.at(e);
            load_x<VEC, K>(x + c * ldx, xv);
#pragma unroll
            for (int k = 0; k < K; ++k)
                acc[k] += v * xv[k];
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
            y[r * ldy + lane] = static_cast<x_t>(out);
        }
    }
}

// Column-blocked pass: only the entries of each row with c0 <= column < c1
// (found by binary search; columns are sorted within a row), lanes strided
// over them; y = (accumulate ? y : 0) + that part of H x.  Passes over
// consecutive column blocks keep the gathered slice of x inside L2 when the
// whole block of vectors does not fit.
template<int VK, int K, int LANES, bool VEC>
__global__ void __launch_bounds__(256) spmm_cb_kernel(int64_t nrow, const int64_t *__restrict__ rowptr,
                                                      const int32_t *__restrict__ cols, Values<VK> vals,
                                                      const typename Values<VK>::x_t *__restrict__ x, int64_t ldx,
                                                      typename Values<VK>::x_t *__restrict__ y, int64_t ldy,
                                                      int32_t c0, int32_t c1, bool accumulate) {
    typedef typename Values<VK>::acc_t acc_t;
    typedef typename Values<VK>::x_t x_t;
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    for (int64_t r = group; r < nrow; r += ngroups) {
        const int64_t start = rowptr[r], end = rowptr[r + 1];
        // First entry with column >= c (lower bound), for c = c0 and c1.
        auto lower = [&](int32_t c) {
            int64_t lo = start, hi = end;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (__ldg(cols + mid) < c)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            return lo;
        };
        const int64_t e0 = lower(c0), e1 = lower(c1);
        acc_t acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            acc[k] = 0;
        acc_t xv[K];
#pragma unroll 4
        for (int64_t e = e0 + lane; e < e1; e += LANES) {
            const int64_t c = __ldcs(cols + e);
            const acc_t v = vals.at(e);
            load_x<VEC, K>(x + c * ldx, xv);
#pragma unroll
            for (int k = 0; k < K; ++k)
                acc[k] += v * xv[k];
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
            x_t *yo = y + r * ldy + lane;
            *yo = accumulate ? static_cast<x_t>(static_cast<acc_t>(*yo) + out) : static_cast<x_t>(out);
        }
    }
}

// FP32 product on the SELL-32 copy.  A block of 8 warps takes 8 / SPLIT
// slices of 32 rows; the SPLIT warps of a slice split its entries into
// SPLIT consecutive ranges, and lane l of each walks row 32 s + l over its
// range (entry j of the 32 rows is one coalesced 128-byte load of columns
// and one of values).
// The slice's rows share their column blocks of x (consecutive FCI / DOCI
// rows differ in the low orbitals), so a warp's 32 gathers touch far fewer
// cache lines than the 32 gathers of one CSR row.  The next U entries'
// columns and values are loaded before the current U are gathered, so the
// matrix stream and the gathers overlap within a warp.  The SPLIT partial
// sums of a row are added in a fixed order through shared memory
// (deterministic).  SPLIT = 4 keeps the last wave of blocks short when x
// fits in L2; SPLIT = 1 keeps a slice's gathers close together in time,
// which matters when x does not fit (the autotuner picks).
template<int K, bool VEC, int SPLIT>
__global__ void __launch_bounds__(256) spmm_sell_kernel(int64_t nrow, int64_t nslice, const int64_t *__restrict__ off,
                                                        const int32_t *__restrict__ cols,
                                                        const float *__restrict__ vals, const float *__restrict__ x,
                                                        int64_t ldx, float *__restrict__ y, int64_t ldy) {
    constexpr int U = 4;
    __shared__ float part[8][K][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kPer = 8 / SPLIT; // slices per block step
    const int q = warp % SPLIT;
    for (int64_t grp = blockIdx.x; kPer * grp < nslice; grp += gridDim.x) {
        const int64_t s = kPer * grp + warp / SPLIT;
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            acc[k] = 0.0f;
        if (s < nslice) {
            const int64_t o = off[s];
            const int64_t L = (off[s + 1] - o) >> 5;
            const int64_t Lq = (L + SPLIT - 1) / SPLIT;
            const int64_t j0 = min(L, q * Lq), j1 = min(L, j0 + Lq);
            const int32_t *cp = cols + o + lane;
            const float *vp = vals + o + lane;
            float xv[K];
            int64_t j = j0;
            if (j + U <= j1) {
                int32_t c[U];
                float v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    c[u] = __ldcs(cp + 32 * (j + u));
                    v[u] = __ldcs(vp + 32 * (j + u));
                }
                for (; j + 2 * U <= j1; j += U) {
                    int32_t cn[U];
                    float vn[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        cn[u] = __ldcs(cp + 32 * (j + U + u));
                        vn[u] = __ldcs(vp + 32 * (j + U + u));
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        load_x<VEC, K>(x + static_cast<int64_t>(c[u]) * ldx, xv);
#pragma unroll
                        for (int k = 0; k < K; ++k)
                            acc[k] += v[u] * xv[k];
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        c[u] = cn[u];
                        v[u] = vn[u];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    load_x<VEC, K>(x + static_cast<int64_t>(c[u]) * ldx, xv);
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        acc[k] += v[u] * xv[k];
                }
                j += U;
            }
            for (; j < j1; ++j) {
                const int32_t c = __ldcs(cp + 32 * j);
                const float v = __ldcs(vp + 32 * j);
                load_x<VEC, K>(x + static_cast<int64_t>(c) * ldx, xv);
#pragma unroll
                for (int k = 0; k < K; ++k)
                    acc[k] += v * xv[k];
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            part[warp][k][lane] = acc[k];
        __syncthreads();
        if (q == 0 && s < nslice) {
            const int64_t r = 32 * s + lane;
            if (r < nrow) {
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    float t = part[warp][k][lane];
#pragma unroll
                    for (int w = 1; w < SPLIT; ++w)
                        t += part[warp + w][k][lane];
                    y[r * ldy + k] = t;
                }
            }
        }
        __syncthreads();
    }
}

template<int K, int SPLIT>
void launch_sell_split(const pyci_gpu_csr *csr, const void *x, int64_t ldx, void *y, int64_t ldy, cudaStream_t st) {
    constexpr int kPer = 8 / SPLIT;
    const int64_t blocks = std::max<int64_t>(
        1, std::min<int64_t>(static_cast<int64_t>(csr->ctx->num_sms) * 32, (csr->nslice + kPer - 1) / kPer));
    const size_t rowbytes = static_cast<size_t>(ldx) * sizeof(float);
    const size_t vbytes = (K * sizeof(float)) % 16 == 0 ? 16 : ((K * sizeof(float)) == 8 ? 8 : 0);
    const bool vec = vbytes && (reinterpret_cast<uintptr_t>(x) % vbytes == 0) && (rowbytes % vbytes == 0);
    if (vec)
        spmm_sell_kernel<K, true, SPLIT><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
            csr->nrow, csr->nslice, csr->sell_off, csr->sell_cols, csr->sell_vals, static_cast<const float *>(x), ldx,
            static_cast<float *>(y), ldy);
    else
        spmm_sell_kernel<K, false, SPLIT><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
            csr->nrow, csr->nslice, csr->sell_off, csr->sell_cols, csr->sell_vals, static_cast<const float *>(x), ldx,
            static_cast<float *>(y), ldy);
    ::pyci_gpu::note_launch();
}

// sub 0: 4 warps per slice; sub 1: one warp per slice.
template<int K>
void launch_sell(int sub, const pyci_gpu_csr *csr, const void *x, int64_t ldx, void *y, int64_t ldy,
                 cudaStream_t st) {
    if (sub == 1)
        launch_sell_split<K, 1>(csr, x, ldx, y, ldy, st);
    else
        launch_sell_split<K, 4>(csr, x, ldx, y, ldy, st);
}

template<int VK, int K, int LANES>
void launch_cb(const pyci_gpu_csr *csr, Values<VK> vals, const void *x, int64_t ldx, void *y, int64_t ldy,
               int nblk, cudaStream_t st) {
    typedef typename Values<VK>::x_t x_t;
    const int64_t max_blocks = static_cast<int64_t>(csr->ctx->num_sms) * 8 * 4;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(max_blocks, (csr->nrow * LANES + 255) / 256));
    const size_t rowbytes = static_cast<size_t>(ldx) * sizeof(x_t);
    const size_t vbytes = (K * sizeof(x_t)) % 16 == 0 ? 16 : ((K * sizeof(x_t)) == 8 ? 8 : 0);
    const bool vec = vbytes && (reinterpret_cast<uintptr_t>(x) % vbytes == 0) && (rowbytes % vbytes == 0);
    for (int b = 0; b < nblk; ++b) {
        const int32_t c0 = static_cast<int32_t>(csr->ncol * b / nblk), c1 = static_cast<int32_t>(csr->ncol * (b + 1) / nblk);
        if (vec)
            spmm_cb_kernel<VK, K, LANES, true><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
                csr->nrow, csr->rowptr, csr->cols, vals, static_cast<const x_t *>(x), ldx, static_cast<x_t *>(y), ldy,
                c0, c1, b > 0);
        else
            spmm_cb_kernel<VK, K, LANES, false><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
                csr->nrow, csr->rowptr, csr->cols, vals, static_cast<const x_t *>(x), ldx, static_cast<x_t *>(y), ldy,
                c0, c1, b > 0);
        ::pyci_gpu::note_launch();
    }
}

template<int VK, int K, int LANES, int MAP>
void launch_one(const pyci_gpu_csr *csr, Values<VK> vals, const void *x, int64_t ldx, void *y,
                int64_t ldy, cudaStream_t st) {
    typedef typename Values<VK>::x_t x_t;
    const int threads = 256;
    const int64_t groups_needed = csr->nrow;
    const int64_t max_blocks = static_cast<int64_t>(csr->ctx->num_sms) * 8 * 4;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(max_blocks, (groups_needed * LANES + threads - 1) / threads));
    // Vector gathers need every x row on a 16-byte (or 8-byte) boundary.
    const size_t rowbytes = static_cast<size_t>(ldx) * sizeof(x_t);
    const size_t vbytes = (K * sizeof(x_t)) % 16 == 0 ? 16 : ((K * sizeof(x_t)) == 8 ? 8 : 0);
    const bool vec = vbytes && (reinterpret_cast<uintptr_t>(x) % vbytes == 0) && (rowbytes % vbytes == 0);
    if (vec)
        spmm_kernel<VK, K, LANES, true, MAP><<<static_cast<unsigned>(blocks), threads, 0, st>>>(
            csr->nrow, csr->rowptr, csr->cols, vals, static_cast<const x_t *>(x), ldx,
            static_cast<x_t *>(y), ldy), ::pyci_gpu::note_launch();
    else
        spmm_kernel<VK, K, LANES, false, MAP><<<static_cast<unsigned>(blocks), threads, 0, st>>>(
            csr->nrow, csr->rowptr, csr->cols, vals, static_cast<const x_t *>(x), ldx,
            static_cast<x_t *>(y), ldy), ::pyci_gpu::note_launch();
}

// Tile variants: lanes per row (8, 16, 32) x entry mapping (0, 1); and, for
// the FP32 values of an operator that has one, the SELL-32 copy.
constexpr int kVariants = 6;
constexpr int kSellVariant = 0x100; // FP32: + 0 (4 warps per slice) or + 1 (one warp)
constexpr int kFxVariant = 0x200;   // implicit form of a full FullCI (fcix.cu) or DOCI (docx.cu) space

// The implicit-column form serves the FP32 products (mode 0) and the
// double-float ones (csr_spmm_df); FP64 arithmetic stays on the CSR, whose
// product this GPU's FP64 pipe already bounds.
template<int VK>
inline bool fx_usable(const pyci_gpu_csr *csr, int K) {
    return VK == kF32 && has_implicit(csr) && K <= 8;
}
inline int variant_lanes(int v) { return v % 3 == 0 ? 8 : (v % 3 == 1 ? 16 : 32); }
inline int variant_map(int v) { return v / 3; }

inline int heuristic_variant(const pyci_gpu_csr *csr);

template<int VK, int K>
void launch_variant(int v, const pyci_gpu_csr *csr, Values<VK> vals, const void *x, int64_t ldx, void *y,
                    int64_t ldy, cudaStream_t st) {
    if (v == kFxVariant) {
        if (VK == kF32 && implicit_launch(csr, 0, K, x, ldx, y, ldy, st))
            return;
        v = heuristic_variant(csr); // a cached choice from an operator of the same shape without the form
    }
    if (v == kSellVariant || v == kSellVariant + 1) {
        if constexpr (VK == kF32) {
            if (csr->sell_cols) {
                launch_sell<K>(v - kSellVariant, csr, x, ldx, y, ldy, st);
                return;
            }
        }
        // A cached choice from an operator of the same shape that had the
        // SELL copy: this one runs the row-length heuristic instead.
        v = heuristic_variant(csr);
    }
    const int nblk = v >> 4;
    v &= 15;
    if (nblk > 1) {
        // Column-blocked passes (lane-strided entries) at the variant's lanes.
        switch (variant_lanes(v)) {
        case 8: launch_cb<VK, K, 8>(csr, vals, x, ldx, y, ldy, nblk, st); break;
        case 16: launch_cb<VK, K, 16>(csr, vals, x, ldx, y, ldy, nblk, st); break;
        default: launch_cb<VK, K, 32>(csr, vals, x, ldx, y, ldy, nblk, st); break;
        }
        return;
    }
    constexpr bool kMapped = (K == 1 || K == 2 || K == 4 || K == 8);
    const int map = kMapped ? variant_map(v) : 0;
    switch (variant_lanes(v) * 2 + map) {
    case 16: launch_one<VK, K, 8, 0>(csr, vals, x, ldx, y, ldy, st); break;
    case 32: launch_one<VK, K, 16, 0>(csr, vals, x, ldx, y, ldy, st); break;
    case 64: launch_one<VK, K, 32, 0>(csr, vals, x, ldx, y, ldy, st); break;
    case 17: launch_one<VK, K, 8, kMapped ? 1 : 0>(csr, vals, x, ldx, y, ldy, st); break;
    case 33: launch_one<VK, K, 16, kMapped ? 1 : 0>(csr, vals, x, ldx, y, ldy, st); break;
    default: launch_one<VK, K, 32, kMapped ? 1 : 0>(csr, vals, x, ldx, y, ldy, st); break;
    }
}

template<int VK>
void launch_k(int v, const pyci_gpu_csr *csr, Values<VK> vals, int K, const void *x, int64_t ldx, void *y,
              int64_t ldy, cudaStream_t st) {
    switch (K) {
    case 1: launch_variant<VK, 1>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 2: launch_variant<VK, 2>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 3: launch_variant<VK, 3>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 4: launch_variant<VK, 4>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 5: launch_variant<VK, 5>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 6: launch_variant<VK, 6>(v, csr, vals, x, ldx, y, ldy, st); break;
    case 7: launch_variant<VK, 7>(v, csr, vals, x, ldx, y, ldy, st); break;
    default: launch_variant<VK, 8>(v, csr, vals, x, ldx, y, ldy, st); break;
    }
}

// Heuristic variant from the mean row length (used when tuning is off).
inline int heuristic_variant(const pyci_gpu_csr *csr) {
    return csr->spmm_lanes >= 32 ? 2 : (csr->spmm_lanes >= 16 ? 1 : 0);
}

// Tuning results shared by operators of the same shape (rows, columns,
// stored entries) in this process, so rebuilding an operator does not tune
// again.
struct TuneKey {
    int64_t nrow, ncol, nnz;
    int vk, k;
    bool operator<(const TuneKey &o) const {
        return std::tie(nrow, ncol, nnz, vk, k) < std::tie(o.nrow, o.ncol, o.nnz, o.vk, o.k);
    }
};
std::mutex g_tune_mutex;
std::map<TuneKey, int> g_tune_cache;

int tuning_cache_lookup(const pyci_gpu_csr *csr, int vk, int k) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(TuneKey{csr->nrow, csr->ncol, csr->nnz, vk, k});
    return it == g_tune_cache.end() ? -1 : it->second;
}

void tuning_cache_store(const pyci_gpu_csr *csr, int vk, int k, int v) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[TuneKey{csr->nrow, csr->ncol, csr->nnz, vk, k}] = v;
}

bool autotune_enabled() {
    static const bool on = [] {
        const char *e = std::getenv("PYCI_GPU_AUTOTUNE");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Whether PYCI_GPU_SPMM pins products to the CSR or SELL-32 kernels.
bool pinned_to_csr() {
    const char *e = std::getenv("PYCI_GPU_SPMM");
    return e && (!std::strcmp(e, "csr") || !std::strcmp(e, "sell") || !std::strcmp(e, "sell1"));
}

// PYCI_GPU_SPMM=fcix, =sell, =sell1 or =csr pins the products of an operator
// (read when it makes its first product of a kind, so a process can compare
// them): the implicit form (FP32 and double-float; full FullCI and DOCI
// spaces), the SELL-32 copy (FP32 and double-float; FP32 with 4 warps or one
// warp per slice) or the CSR heuristic (all precisions).
int forced_sell_variant(const pyci_gpu_csr *csr) {
    const char *e = std::getenv("PYCI_GPU_SPMM");
    if (!e)
        return -1;
    if (!std::strcmp(e, "fcix"))
        return has_implicit(csr) ? kFxVariant : heuristic_variant(csr);
    if (!std::strcmp(e, "sell"))
        return csr->sell_cols ? kSellVariant : heuristic_variant(csr);
    if (!std::strcmp(e, "sell1"))
        return csr->sell_cols ? kSellVariant + 1 : heuristic_variant(csr);
    if (!std::strcmp(e, "csr"))
        return heuristic_variant(csr);
    return -1;
}

// Autotuner: the first product of an operator for a (precision, width) pair
// times every tile variant (one warm-up + two timed launches each, CUDA
// events on the caller's stream) and keeps the fastest for later calls.
// Every variant computes the same y, so the tuning call's result is valid.
template<int VK>
void launch_vk(const pyci_gpu_csr *csr, Values<VK> vals, int64_t k, const void *x, void *y,
               cudaStream_t st) {
    typedef typename Values<VK>::x_t x_t;
    for (int64_t j0 = 0; j0 < k; j0 += 8) {
        const int K = static_cast<int>(std::min<int64_t>(8, k - j0));
        const void *xs = static_cast<const x_t *>(x) + j0;
        void *ys = static_cast<x_t *>(y) + j0;
        int &choice = csr->tuned[VK][K];
        if (choice < 0 && VK == kF32)
            choice = forced_sell_variant(csr);
        if (choice < 0 && VK != kF32) {
            const char *e = std::getenv("PYCI_GPU_SPMM");
            if (e && (!std::strcmp(e, "csr") || !std::strcmp(e, "sell") || !std::strcmp(e, "sell1")))
                choice = heuristic_variant(csr);
        }
        if (choice < 0)
            choice = tuning_cache_lookup(csr, VK, K);
        if (choice < 0) {
            if (!autotune_enabled() || csr->nnz < (1 << 20)) {
                choice = heuristic_variant(csr);
            } else {
                cudaEvent_t a, b;
                cudaEventCreate(&a);
                cudaEventCreate(&b);
                float best = 1e30f;
                int best_v = heuristic_variant(csr);
                for (int v = 0; v < kVariants; ++v) {
                    launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(a, st);
                    launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                    launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(b, st);
                    cudaEventSynchronize(b);
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, a, b);
                    if (ms < best) {
                        best = ms;
                        best_v = v;
                    }
                }
                const int best_csr = best_v;
                // The implicit-column form.
                if (fx_usable<VK>(csr, K)) {
                    launch_k<VK>(kFxVariant, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(a, st);
                    launch_k<VK>(kFxVariant, csr, vals, K, xs, k, ys, k, st);
                    launch_k<VK>(kFxVariant, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(b, st);
                    cudaEventSynchronize(b);
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, a, b);
                    if (ms < best) {
                        best = ms;
                        best_v = kFxVariant;
                    }
                }
                // The SELL-32 copy (FP32 values only), both splits.
                for (int sv = kSellVariant; VK == kF32 && csr->sell_cols && sv <= kSellVariant + 1; ++sv) {
                    launch_k<VK>(sv, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(a, st);
                    launch_k<VK>(sv, csr, vals, K, xs, k, ys, k, st);
                    launch_k<VK>(sv, csr, vals, K, xs, k, ys, k, st);
                    cudaEventRecord(b, st);
                    cudaEventSynchronize(b);
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, a, b);
                    if (ms < best) {
                        best = ms;
                        best_v = sv;
                    }
                }
                // Column blocks when the gathered block of vectors is larger
                // than about half the L2 (126 MB on this GPU).
                const double xbytes = static_cast<double>(csr->ncol) * K * sizeof(x_t);
                if (xbytes > 48.0 * (1 << 20) && csr->ncol < INT32_MAX) {
                    for (int nblk = 2; nblk <= 4; ++nblk) {
                        const int v = best_csr | (nblk << 4);
                        launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                        cudaEventRecord(a, st);
                        launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                        launch_k<VK>(v, csr, vals, K, xs, k, ys, k, st);
                        cudaEventRecord(b, st);
                        cudaEventSynchronize(b);
                        float ms = 0.0f;
                        cudaEventElapsedTime(&ms, a, b);
                        if (ms < best) {
                            best = ms;
                            best_v = v;
                        }
                    }
                }
                cudaEventDestroy(a);
                cudaEventDestroy(b);
                choice = best_v;
                tuning_cache_store(csr, VK, K, choice);
            }
        }
        launch_k<VK>(choice, csr, vals, K, xs, k, ys, k, st);
    }
}

// Self-adjoint product from a lower-triangle CSR (only used for operators that
// keep just the reference layout): y += L x + L^T x - D x with atomics; y must
// be zeroed first.  Equivalent to the Eigen selfadjointView<Lower> product of
// pyci/src/sparseop.cpp:106-112.
template<typename T>
__global__ void spmm_lower_kernel(int64_t nrow, const int64_t *rowptr, const int32_t *cols,
                                  const double *vals, const float *hi, const float *lo,
                                  const T *x, int k, T *y) {
    for (int64_t e0 = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e0 < nrow;
         e0 += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e0;
        for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) {
            const int64_t c = cols[e];
            const double v = vals ? vals[e] : static_cast<double>(hi[e]) + static_cast<double>(lo[e]);
            for (int j = 0; j < k; ++j) {
                atomicAdd(&y[r * k + j], static_cast<T>(v * static_cast<double>(x[c * k + j])));
                if (c != r)
                    atomicAdd(&y[c * k + j], static_cast<T>(v * static_cast<double>(x[r * k + j])));
            }
        }
    }
}

// FP64-accurate product with FP32 arithmetic only (this GPU's FP64 rate is
// a small fraction of its FP32 rate).  Values are the exact high/low split
// v = hi + lo; x arrives split the same way, row c of xs holding
// xh[c][0..K) then xl[c][0..K).  Each term
//   v x = hi xh + (hi xh - fl(hi xh)) + hi xl + lo xh  (+ lo xl, ~2^-48 |v x|)
// is formed as p = fl(hi xh), its exact rounding error e = fma(hi, xh, -p),
// and t = fma(hi, xl, fma(lo, xh, e)); p is added to a double-float sum
// (s, c) with Knuth's TwoSum (6 FP32 additions, exact), and t to c.  The
// result s + c is converted to FP64 once per row: relative error ~2^-44,
// against ~2^-53 for FP64 arithmetic, far below what the FP64 refinement of
// the eigensolver can resolve.  __fadd_rn / __fmul_rn keep the compiler from
// fusing the error-free transformations into FMAs.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float p) {
    const float u = __fadd_rn(s, p);
    const float z = __fadd_rn(u, -s);
    const float d = __fadd_rn(__fadd_rn(s, -__fadd_rn(u, -z)), __fadd_rn(p, -z));
    s = u;
    c = __fadd_rn(c, d);
}

// Split operand row c: K high parts then K low parts.
template<int K>
__device__ __forceinline__ void load_split(const float *__restrict__ xs, int64_t col, float xh[K], float xl[K]) {
    const float *xr = xs + col * (2 * K);
    if constexpr (K == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(xr));
        const float4 b = __ldg(reinterpret_cast<const float4 *>(xr) + 1);
        xh[0] = a.x, xh[1] = a.y, xh[2] = a.z, xh[3] = a.w;
        xl[0] = b.x, xl[1] = b.y, xl[2] = b.z, xl[3] = b.w;
    } else if constexpr (K == 2) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(xr));
        xh[0] = a.x, xh[1] = a.y;
        xl[0] = a.z, xl[1] = a.w;
    } else {
        const float2 a = __ldg(reinterpret_cast<const float2 *>(xr));
        xh[0] = a.x;
        xl[0] = a.y;
    }
}

// Adds (vh + vl) (xh + xl) to the double-float sums (s, c).
template<int K>
__device__ __forceinline__ void df_term(float vh, float vl, const float xh[K], const float xl[K], float s[K],
                                        float c[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float p = __fmul_rn(vh, xh[k]);
        const float err = fmaf(vh, xh[k], -p);
        const float t = fmaf(vh, xl[k], fmaf(vl, xh[k], err));
        two_sum_acc(s[k], c[k], p);
        c[k] = __fadd_rn(c[k], t);
    }
}

// MAP 1: lane l takes entries l, l + LANES, ... of the row; MAP 0: each lane
// takes 4 consecutive entries per step (16-byte loads of columns and of both
// value halves), so four independent gathers are in flight per lane.
template<int K, int LANES, int MAP>
__global__ void __launch_bounds__(256) spmm_df_kernel(int64_t nrow, const int64_t *__restrict__ rowptr,
                                                      const int32_t *__restrict__ cols, const float *__restrict__ hi,
                                                      const float *__restrict__ lo, const float *__restrict__ xs,
                                                      double *__restrict__ y) {
    const int lane = threadIdx.x % LANES;
    const int64_t group = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / LANES;
    const int64_t ngroups = (static_cast<int64_t>(gridDim.x) * blockDim.x) / LANES;
    for (int64_t r = group; r < nrow; r += ngroups) {
        const int64_t start = rowptr[r], end = rowptr[r + 1];
        float s[K], c[K], xh[K], xl[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            s[k] = c[k] = 0.0f;
        if constexpr (MAP == 1) {
            for (int64_t e = start + lane; e < end; e += LANES) {
                const int64_t col = __ldcs(cols + e);
                const float vh = __ldcs(hi + e), vl = __ldcs(lo + e);
                load_split<K>(xs, col, xh, xl);
                df_term<K>(vh, vl, xh, xl, s, c);
            }
        } else {
            // Head: entries before the first 4-aligned index; body: 4 per lane
            // per step; tail.
            const int64_t a0 = min(end, (start + 3) & ~static_cast<int64_t>(3));
            const int64_t a1 = max(a0, end & ~static_cast<int64_t>(3));
            if (start + lane < a0) {
                const int64_t e = start + lane;
                load_split<K>(xs, __ldcs(cols + e), xh, xl);
                df_term<K>(__ldcs(hi + e), __ldcs(lo + e), xh, xl, s, c);
            }
            for (int64_t e = a0 + 4 * lane; e < a1; e += 4 * LANES) {
                const int4 c4 = __ldcs(reinterpret_cast<const int4 *>(cols + e));
                const float4 h4 = __ldcs(reinterpret_cast<const float4 *>(hi + e));
                const float4 l4 = __ldcs(reinterpret_cast<const float4 *>(lo + e));
                float gh[4][K], gl[4][K];
                load_split<K>(xs, c4.x, gh[0], gl[0]);
                load_split<K>(xs, c4.y, gh[1], gl[1]);
                load_split<K>(xs, c4.z, gh[2], gl[2]);
                load_split<K>(xs, c4.w, gh[3], gl[3]);
                df_term<K>(h4.x, l4.x, gh[0], gl[0], s, c);
                df_term<K>(h4.y, l4.y, gh[1], gl[1], s, c);
                df_term<K>(h4.z, l4.z, gh[2], gl[2], s, c);
                df_term<K>(h4.w, l4.w, gh[3], gl[3], s, c);
            }
            if (a1 + lane < end) {
                const int64_t e = a1 + lane;
                load_split<K>(xs, __ldcs(cols + e), xh, xl);
                df_term<K>(__ldcs(hi + e), __ldcs(lo + e), xh, xl, s, c);
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1) {
                const float s2 = __shfl_xor_sync(0xffffffffu, s[k], o, LANES);
                const float c2 = __shfl_xor_sync(0xffffffffu, c[k], o, LANES);
                two_sum_acc(s[k], c[k], s2);
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

// Double-float product on the SELL-32 copy: lane l of the slice's warp owns
// row 32 s + l over the whole row and keeps its own double-float sums, so
// no cross-lane combination is needed.
template<int K>
__global__ void __launch_bounds__(256) spmm_df_sell_kernel(int64_t nrow, int64_t nslice,
                                                           const int64_t *__restrict__ off,
                                                           const int32_t *__restrict__ cols,
                                                           const float *__restrict__ hi, const float *__restrict__ lo,
                                                           const float *__restrict__ xs, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t s = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; s < nslice; s += nwarps) {
        const int64_t o = off[s];
        const int64_t L = (off[s + 1] - o) >> 5;
        const int32_t *cp = cols + o + lane;
        const float *hp = hi + o + lane;
        const float *lp = lo + o + lane;
        float sm[K], cm[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            sm[k] = cm[k] = 0.0f;
        int64_t j = 0;
        for (; j + 2 <= L; j += 2) {
            const int32_t c0 = __ldcs(cp + 32 * j), c1 = __ldcs(cp + 32 * (j + 1));
            const float h0 = __ldcs(hp + 32 * j), h1 = __ldcs(hp + 32 * (j + 1));
            const float l0 = __ldcs(lp + 32 * j), l1 = __ldcs(lp + 32 * (j + 1));
            float xh0[K], xl0[K], xh1[K], xl1[K];
            load_split<K>(xs, c0, xh0, xl0);
            load_split<K>(xs, c1, xh1, xl1);
            df_term<K>(h0, l0, xh0, xl0, sm, cm);
            df_term<K>(h1, l1, xh1, xl1, sm, cm);
        }
        if (j < L) {
            float xh[K], xl[K];
            load_split<K>(xs, __ldcs(cp + 32 * j), xh, xl);
            df_term<K>(__ldcs(hp + 32 * j), __ldcs(lp + 32 * j), xh, xl, sm, cm);
        }
        const int64_t r = 32 * s + lane;
        if (r < nrow) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                y[r * K + k] = static_cast<double>(sm[k]) + static_cast<double>(cm[k]);
        }
    }
}

template<int K>
void launch_df_variant(int v, const pyci_gpu_csr *csr, const float *xs, double *y, cudaStream_t st) {
    if (v == kFxVariant) {
        if (implicit_launch(csr, 2, K, xs, 2 * K, y, K, st))
            return;
        v = heuristic_variant(csr);
    }
    if (v >= kSellVariant && csr->sell_lo) {
        const int64_t blocks = std::max<int64_t>(
            1, std::min<int64_t>(static_cast<int64_t>(csr->ctx->num_sms) * 32, (csr->nslice * 32 + 255) / 256));
        spmm_df_sell_kernel<K><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
            csr->nrow, csr->nslice, csr->sell_off, csr->sell_cols, csr->sell_vals, csr->sell_lo, xs, y);
        ::pyci_gpu::note_launch();
        return;
    }
    if (v >= kSellVariant)
        v = heuristic_variant(csr);
    const int lanes = variant_lanes(v), map = variant_map(v);
    const int64_t max_blocks = static_cast<int64_t>(csr->ctx->num_sms) * 8 * 4;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(max_blocks, (csr->nrow * lanes + 255) / 256));
    const unsigned g = static_cast<unsigned>(blocks);
    const int64_t n = csr->nrow;
    switch (lanes * 2 + map) {
    case 16: spmm_df_kernel<K, 8, 0><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    case 17: spmm_df_kernel<K, 8, 1><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    case 32: spmm_df_kernel<K, 16, 0><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    case 33: spmm_df_kernel<K, 16, 1><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    case 64: spmm_df_kernel<K, 32, 0><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    default: spmm_df_kernel<K, 32, 1><<<g, 256, 0, st>>>(n, csr->rowptr, csr->cols, csr->hi, csr->lo, xs, y); break;
    }
    ::pyci_gpu::note_launch();
}

inline void launch_df(int v, const pyci_gpu_csr *csr, int K, const float *xs, double *y, cudaStream_t st) {
    if (K == 4)
        launch_df_variant<4>(v, csr, xs, y, st);
    else if (K == 2)
        launch_df_variant<2>(v, csr, xs, y, st);
    else
        launch_df_variant<1>(v, csr, xs, y, st);
}

} // namespace pyci_gpu

using namespace pyci_gpu;

// y[N][K] = (hi + lo) x for one split block xs[N][2K] (K = 1, 2 or 4), FP32
// arithmetic with double-float accumulation; the tile variant (lanes per row x
// entry mapping, as the other products) is tuned on first use.
int csr_spmm_df(const pyci_gpu_csr *csr, int K, const float *xs, double *y, cudaStream_t st) {
    if ((!csr->hi || !csr->lo) && has_implicit(csr)) {
        // Implicit form only (a full FullCI or DOCI space).
        if ((K == 1 || K == 2 || K == 4) && !pinned_to_csr() && implicit_launch(csr, 2, K, xs, 2 * K, y, K, st)) {
            csr->tuned[kSplitDF][K] = kFxVariant;
            PYCI_CUDA_TRY(cudaGetLastError());
            return PYCI_GPU_OK;
        }
        int rc = csr_ensure_split(const_cast<pyci_gpu_csr *>(csr));
        if (rc)
            return rc;
    }
    if (!csr->hi || !csr->lo) {
        set_error("split product needs pyci_gpu_csr_prepare_mixed first");
        return PYCI_GPU_EINVAL;
    }
    if (csr->lower_only || !(K == 1 || K == 2 || K == 4)) {
        set_error("double-float product: unsupported operator layout or width %d", K);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (csr->nrow == 0)
        return PYCI_GPU_OK;
    int &choice = csr->tuned[kSplitDF][K];
    if (choice < 0)
        choice = forced_sell_variant(csr);
    if (choice < 0)
        choice = tuning_cache_lookup(csr, kSplitDF, K);
    if (choice < 0) {
        if (!autotune_enabled() || csr->nnz < (1 << 20)) {
            choice = heuristic_variant(csr);
        } else {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            float best = 1e30f;
            int best_v = heuristic_variant(csr);
            for (int v = 0; v < kVariants; ++v) {
                launch_df(v, csr, K, xs, y, st);
                cudaEventRecord(a, st);
                launch_df(v, csr, K, xs, y, st);
                launch_df(v, csr, K, xs, y, st);
                cudaEventRecord(b, st);
                cudaEventSynchronize(b);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                if (ms < best) {
                    best = ms;
                    best_v = v;
                }
            }
            if (has_implicit(csr)) {
                launch_df(kFxVariant, csr, K, xs, y, st);
                cudaEventRecord(a, st);
                launch_df(kFxVariant, csr, K, xs, y, st);
                launch_df(kFxVariant, csr, K, xs, y, st);
                cudaEventRecord(b, st);
                cudaEventSynchronize(b);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                if (ms < best) {
                    best = ms;
                    best_v = kFxVariant;
                }
            }
            if (csr->sell_lo) {
                launch_df(kSellVariant, csr, K, xs, y, st);
                cudaEventRecord(a, st);
                launch_df(kSellVariant, csr, K, xs, y, st);
                launch_df(kSellVariant, csr, K, xs, y, st);
                cudaEventRecord(b, st);
                cudaEventSynchronize(b);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                if (ms < best) {
                    best = ms;
                    best_v = kSellVariant;
                }
            }
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            choice = best_v;
            tuning_cache_store(csr, kSplitDF, K, choice);
        }
    }
    launch_df(choice, csr, K, xs, y, st);
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

static int spmm_lower(const pyci_gpu_csr *csr, int precision, int64_t k, const void *x, void *y,
                      cudaStream_t st) {
    const bool f32 = (precision == PYCI_PREC_FP32);
    const size_t es = f32 ? sizeof(float) : sizeof(double);
    PYCI_CUDA_TRY(cudaMemsetAsync(y, 0, es * csr->nrow * k, st));
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((csr->nrow + 255) / 256, 65536));
    const double *vals = (precision == PYCI_PREC_FP64 && csr->vals) ? csr->vals : nullptr;
    if (f32)
        spmm_lower_kernel<float><<<blocks, 256, 0, st>>>(csr->nrow, csr->rowptr, csr->cols, nullptr,
                                                        csr->hi, csr->lo, static_cast<const float *>(x),
                                                        static_cast<int>(k), static_cast<float *>(y)), ::pyci_gpu::note_launch();
    else
        spmm_lower_kernel<double><<<blocks, 256, 0, st>>>(csr->nrow, csr->rowptr, csr->cols, vals,
                                                         csr->hi, csr->lo, static_cast<const double *>(x),
                                                         static_cast<int>(k), static_cast<double *>(y)), ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

extern "C" int pyci_gpu_csr_product_form(const pyci_gpu_csr *csr, int precision, int64_t k, int *form) {
    if (!csr || !form) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    const int K = static_cast<int>(std::min<int64_t>(std::max<int64_t>(k, 1), 8));
    int vk;
    switch (precision) {
    case PYCI_PREC_FP64: vk = csr->vals ? kF64 : kSplit; break;
    case PYCI_PREC_FP32: vk = kF32; break;
    case PYCI_PREC_FP64_SPLIT: vk = kSplit; break;
    case PYCI_PREC_FP64_DF: vk = kSplitDF; break;
    default: set_error("unknown precision %d", precision); return PYCI_GPU_EINVAL;
    }
    const int v = csr->tuned[vk][K];
    *form = v < 0 ? PYCI_FORM_UNTUNED
                  : (v == kFxVariant ? PYCI_FORM_IMPLICIT
                                     : (v >= kSellVariant && v < kFxVariant ? PYCI_FORM_SELL : PYCI_FORM_CSR));
    return PYCI_GPU_OK;
}

int csr_spmm(const pyci_gpu_csr *csr, int precision, int64_t k, const void *x, void *y,
             cudaStream_t stream) {
    if (k <= 0) {
        set_error("k must be positive");
        return PYCI_GPU_EINVAL;
    }
    if (csr->nrow == 0)
        return PYCI_GPU_OK;
    if (csr->lower_only) {
        if ((precision == PYCI_PREC_FP32 && !csr->hi) || (precision == PYCI_PREC_FP64_SPLIT && !csr->hi) ||
            (precision == PYCI_PREC_FP64 && !csr->vals && !csr->hi)) {
            set_error("operator lacks the values for this precision");
            return PYCI_GPU_EINVAL;
        }
        return spmm_lower(csr, precision, k, x, y, stream);
    }
    switch (precision) {
    case PYCI_PREC_FP64:
        if (!csr->vals && csr->deferred) {
            int rc = csr_materialize(csr);
            if (rc)
                return rc;
        }
        if (csr->vals) {
            launch_vk<kF64>(csr, Values<kF64>{csr->vals}, k, x, y, stream);
        } else if (csr->hi && csr->lo) {
            launch_vk<kSplit>(csr, Values<kSplit>{csr->hi, csr->lo}, k, x, y, stream);
        } else {
            set_error("operator has no values");
            return PYCI_GPU_EINVAL;
        }
        break;
    case PYCI_PREC_FP32:
        if (!csr->hi && has_implicit(csr)) {
            // Only the implicit form serves FP32 products (a full FullCI or
            // DOCI space): up to 8 vectors in one launch; the CSR-order split
            // is made on demand for anything else.
            if (k <= 8 && !pinned_to_csr() && implicit_launch(csr, 0, static_cast<int>(k), x, k, y, k, stream)) {
                csr->tuned[kF32][k] = kFxVariant;
                break;
            }
            int rc = csr_ensure_split(const_cast<pyci_gpu_csr *>(csr));
            if (rc)
                return rc;
        }
        if (!csr->hi) {
            set_error("FP32 product needs pyci_gpu_csr_prepare_mixed first");
            return PYCI_GPU_EINVAL;
        }
        launch_vk<kF32>(csr, Values<kF32>{csr->hi}, k, x, y, stream);
        break;
    case PYCI_PREC_FP64_SPLIT:
        if (!csr->hi && has_implicit(csr)) {
            int rc = csr_ensure_split(const_cast<pyci_gpu_csr *>(csr));
            if (rc)
                return rc;
        }
        if (!csr->hi || !csr->lo) {
            set_error("split product needs pyci_gpu_csr_prepare_mixed first");
            return PYCI_GPU_EINVAL;
        }
        launch_vk<kSplit>(csr, Values<kSplit>{csr->hi, csr->lo}, k, x, y, stream);
        break;
    default:
        set_error("unknown precision %d", precision);
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}
