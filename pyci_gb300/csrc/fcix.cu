// Implicit-column products for full FullCI spaces ("FCIX" form of the
// operator), part of SparseOp::perform_op (pyci/src/sparseop.cpp:96-112).
//
// In a full FullCI space of colex-ranked strings, determinant (a, b) is row
// a * nbeta + b, and its row holds exactly these entries
// (pyci/src/sparseop.cpp:260-427 keeps all of them for a full space):
//   A: (a, b') for b' in {b} + singles(b) + doubles(b)   (diagonal, beta excitations)
//   B: (a', b') for a' in singles(a), b' in {b} + singles(b)  (alpha singles, opposite-spin doubles)
//   C: (a', b) for a' in doubles(a)                       (alpha doubles)
// with column a' * nbeta + b'.  Every column is thus a function of small
// per-string tables, and a product streams the values only: 4 bytes per
// entry in FP32 and 8 for FP64-accurate products from the exact high/low
// split, against 8 and 12 with int32 columns.
//
// Layout.  A row is stored as its sections A, B, C; A and C are padded to a
// multiple of 4 entries and every group of B (one alpha single) to a
// multiple of 4 (padding: zero values).  Inside a section the entries follow
// the sorted target lists.  Rows are grouped by alpha string with the beta
// count padded to a multiple of 32 (nbp); lane l of slice s holds row (a, b),
// a = s / (nbp / 32), b = 32 (s mod (nbp / 32)) + l (rows with b >= nbeta
// are padding: zero values, computed with b = nbeta - 1 and not written).
// Values travel in packets of 4 consecutive entries: entry t of lane l in
// slice s sits at ((s * npk + t / 4) * 32 + l) * 4 + t mod 4, so a lane's
// 16-byte load brings 4 entries and a warp's 512 contiguous bytes.
//
// Product.  One block serves the slices of one alpha string a (or a part of
// them), one warp per slice.  Section A reads x's block of rows a * nbeta ..
// a * nbeta + nbeta - 1 and each group of section B the block of its alpha
// target: the block stages these x blocks in shared memory one at a time
// (cp.async, double-buffered, the next block in flight while the current
// group is multiplied), so the scattered beta gathers of A and B hit shared
// memory instead of missing L1 towards L2.  Section C's gathers (rows
// a' * nbeta + b for 32 consecutive b) are coalesced global loads.  Each warp
// keeps its lanes' section-B partner lists in shared memory.
//
// The build writes the values in this layout without the CSR (build.cu,
// fcix_fill_kernel); the CSR follows on first use.
//
// Tables (L1/L2-resident): atab[a] = the targets of a's singles and doubles
// (sorted), their groups' offsets in the sorted CSR row and that of a's own
// group; bfull[p][b] and bsub[p][b], the sorted
// beta lists, transposed so the 32 lanes of a slice read consecutive words,
// and bq, section A's list as 16-bit indices 4 per packet (one 8-byte load).

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>

#include "dfarith.cuh"
#include "internal.h"

namespace pyci_gpu {

struct FxArgs {
    int64_t nslice, spa, nbeta, npk;
    int ns, nd, nlb, nls, nlsp, la, lb, lc, aw;
    int parts;     // blocks per alpha string
    int xblk;      // floats of one staged x block (nbeta rows, padded to 4)
    const int32_t *atab, *bfull, *bsub;
    const ushort4 *bq; // [la / 4][nbeta]: section A's beta partners, 4 per packet (padding: b)
    const float4 *hi, *lo;
};

// Asynchronous copy of n floats from global src to shared dst by the whole
// block (16-byte pieces when both ends and n allow it, 4-byte otherwise).
__device__ __forceinline__ void fx_stage(float *dst, const float *src, int n) {
    const unsigned sbase = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    if (((reinterpret_cast<uintptr_t>(src) | sbase) & 15) == 0 && (n & 3) == 0) {
        for (int i = threadIdx.x; i < n / 4; i += blockDim.x)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sbase + 16 * i), "l"(src + 4 * i));
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sbase + 4 * i), "l"(src + i));
    }
    asm volatile("cp.async.commit_group;\n" ::);
}

__device__ __forceinline__ void fx_stage_wait() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Shared memory of one block: two staged x blocks, the alpha targets times
// nbeta (singles padded to a multiple of 4, then doubles padded to lc with
// the row's own block), and per warp its lanes' section-B partner lists
// (16-bit: nbeta < 65536; 4 consecutive positions of a lane together, so a
// packet's 4 partners are one 8-byte load).
__host__ __device__ inline int fx_up4(int v) { return (v + 3) / 4 * 4; }
__host__ __device__ inline size_t fx_smem_bytes(int xblk, int ns, int lc, int nlsp, int warps) {
    return sizeof(float) * 2 * static_cast<size_t>(xblk) + sizeof(int) * static_cast<size_t>(fx_up4(ns) + lc) +
           sizeof(uint16_t) * static_cast<size_t>(warps) * nlsp * 32;
}

// MODE 0: FP32 values, x [N][K], y [N][K] float (FP32 accumulation).
// MODE 2: double-float, xs float [N][2K] (high parts then low parts of a
// row), y double [N][K].  Block (a, h) serves slices [h spa / parts,
// (h + 1) spa / parts) of alpha string a, one warp per slice.
template<int MODE, int K>
__global__ void __launch_bounds__(512, 2) fcix_spmm_kernel(FxArgs A, const float *__restrict__ x,
                                                           void *__restrict__ yv) {
    constexpr int XW = MODE == 2 ? 2 * K : K; // floats per x row
    extern __shared__ __align__(16) unsigned char fx_dyn[];
    float *xb0 = reinterpret_cast<float *>(fx_dyn);
    float *xb1 = xb0 + A.xblk;
    const int ns4 = fx_up4(A.ns);
    int *aT = reinterpret_cast<int *>(xb1 + A.xblk);
    uint16_t *jbS = reinterpret_cast<uint16_t *>(aT + ns4 + A.lc);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nbeta = static_cast<int>(A.nbeta);
    const int64_t a = blockIdx.x / A.parts;
    const int h = static_cast<int>(blockIdx.x - a * A.parts);
    const int64_t sb = a * A.spa + h * A.spa / A.parts, se = a * A.spa + (h + 1) * A.spa / A.parts;
    const int64_t s = sb + warp;
    const bool active = s < se;
    const int bb = static_cast<int>((s - a * A.spa) * 32) + lane;
    const int b = bb < nbeta ? bb : nbeta - 1;
    const int self = static_cast<int>(a) * nbeta;
    const int32_t *arow = A.atab + a * A.aw;
    for (int i = threadIdx.x; i < ns4 + A.lc; i += blockDim.x) {
        int v = self;
        if (i < A.ns)
            v = __ldg(arow + i) * nbeta;
        else if (i >= ns4 && i - ns4 < A.nd)
            v = __ldg(arow + A.ns + (i - ns4)) * nbeta;
        aT[i] = v;
    }
    uint16_t *mj = jbS + warp * A.nlsp * 32;
    if (active)
        for (int p = 0; p < A.nlsp; ++p)
            mj[((p >> 2) * 32 + lane) * 4 + (p & 3)] =
                static_cast<uint16_t>(p < A.nls ? __ldg(A.bsub + static_cast<int64_t>(p) * nbeta + b) : b);
    fx_stage(xb0, x + static_cast<int64_t>(self) * XW, nbeta * XW);
    fx_stage_wait();
    __syncthreads();
    if (A.ns > 0)
        fx_stage(xb1, x + static_cast<int64_t>(aT[0]) * XW, nbeta * XW);
    float acc[K], cc[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
        acc[k] = cc[k] = 0.0f;
    const float4 *hp = A.hi + s * A.npk * 32 + lane;
    const float4 *lp = A.lo + s * A.npk * 32 + lane;
    // Packets are read kD at a time (all loads issued before the first is
    // used), so each warp keeps several 512-byte value loads in flight.
    constexpr int kD = 4;
    float4 vh[kD], vl[kD];
    auto load_packets = [&](int q, int qend) {
#pragma unroll
        for (int i = 0; i < kD; ++i) {
            vh[i] = q + i < qend ? __ldcs(hp + 32 * (q + i)) : make_float4(0.f, 0.f, 0.f, 0.f);
            if (MODE == 2)
                vl[i] = q + i < qend ? __ldcs(lp + 32 * (q + i)) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    // Section A: (a, every beta partner of b), x block a in xb0.
    if (active) {
        const ushort4 *tb = A.bq + b;
        for (int q0 = 0; q0 < A.la / 4; q0 += kD) {
            load_packets(q0, A.la / 4);
#pragma unroll
            for (int i = 0; i < kD; ++i) {
                if (q0 + i >= A.la / 4)
                    break;
                const float h4[4] = {vh[i].x, vh[i].y, vh[i].z, vh[i].w};
                const float l4[4] = {vl[i].x, vl[i].y, vl[i].z, vl[i].w};
                const ushort4 j4 = __ldg(tb + static_cast<int64_t>(q0 + i) * nbeta);
                const int jb[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    df_acc<MODE, K>(xb0 + jb[u] * XW, h4[u], l4[u], acc, cc);
            }
        }
    }
    // Section B: group g = alpha single g, x block of its target staged.
    const int qb = A.la / 4, gq = A.nlsp / 4;
    for (int g = 0; g < A.ns; ++g) {
        float *cur = (g & 1) ? xb0 : xb1;
        fx_stage_wait();
        __syncthreads(); // block g staged; nobody still reads the other buffer
        if (g + 1 < A.ns)
            fx_stage((g & 1) ? xb1 : xb0, x + static_cast<int64_t>(aT[g + 1]) * XW, nbeta * XW);
        if (active) {
            for (int qq0 = 0; qq0 < gq; qq0 += kD) {
                load_packets(qb + g * gq + qq0, qb + (g + 1) * gq);
#pragma unroll
                for (int i = 0; i < kD; ++i) {
                    if (qq0 + i >= gq)
                        break;
                    const float h4[4] = {vh[i].x, vh[i].y, vh[i].z, vh[i].w};
                    const float l4[4] = {vl[i].x, vl[i].y, vl[i].z, vl[i].w};
                    const ushort4 j4 = reinterpret_cast<const ushort4 *>(mj)[(qq0 + i) * 32 + lane];
                    const int jb[4] = {j4.x, j4.y, j4.z, j4.w};
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        df_acc<MODE, K>(cur + jb[u] * XW, h4[u], l4[u], acc, cc);
                }
            }
        }
    }
    // Section C: (alpha double, b), coalesced global gathers.
    if (active) {
        const int qc = (A.la + A.lb) / 4;
        for (int q0 = qc; q0 < A.npk; q0 += kD) {
            load_packets(q0, static_cast<int>(A.npk));
#pragma unroll
            for (int i = 0; i < kD; ++i) {
                if (q0 + i >= A.npk)
                    break;
                const float h4[4] = {vh[i].x, vh[i].y, vh[i].z, vh[i].w};
                const float l4[4] = {vl[i].x, vl[i].y, vl[i].z, vl[i].w};
                const int4 d4 = reinterpret_cast<const int4 *>(aT + ns4)[q0 + i - qc];
                const int col[4] = {d4.x + b, d4.y + b, d4.z + b, d4.w + b};
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    df_acc<MODE, K>(x + static_cast<int64_t>(col[u]) * XW, h4[u], l4[u], acc, cc);
            }
        }
        if (bb < nbeta) {
            const int64_t row = static_cast<int64_t>(self) + bb;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if constexpr (MODE == 0)
                    static_cast<float *>(yv)[row * K + k] = acc[k];
                else
                    static_cast<double *>(yv)[row * K + k] = static_cast<double>(acc[k]) + static_cast<double>(cc[k]);
            }
        }
    }
}

inline FxArgs fx_args(const pyci_gpu_csr *csr) {
    FxArgs A;
    A.spa = csr->fx_nbp / 32;
    A.nslice = csr->fx_nalpha * A.spa;
    A.nbeta = csr->fx_nbeta;
    A.npk = csr->fx_npk;
    A.ns = csr->fx_ns;
    A.nd = csr->fx_nd;
    A.nlb = csr->fx_nlb;
    A.nls = csr->fx_nls;
    A.nlsp = (csr->fx_nls + 3) / 4 * 4;
    A.parts = static_cast<int>((A.spa + 15) / 16);
    A.xblk = 0;
    A.la = csr->fx_la;
    A.lb = csr->fx_lb;
    A.lc = csr->fx_lc;
    A.aw = fx_atab_width(csr);
    A.atab = csr->fx_atab;
    A.bfull = csr->fx_bfull;
    A.bsub = csr->fx_bsub;
    A.bq = reinterpret_cast<const ushort4 *>(csr->fx_bq);
    A.hi = reinterpret_cast<const float4 *>(csr->fx_hi);
    A.lo = reinterpret_cast<const float4 *>(csr->fx_lo);
    return A;
}

template<int MODE, int K>
bool fx_launch_k(const pyci_gpu_csr *csr, const void *x, void *y, cudaStream_t st) {
    FxArgs A = fx_args(csr);
    constexpr int XW = MODE == 2 ? 2 * K : K;
    A.xblk = static_cast<int>((A.nbeta * XW + 3) / 4 * 4);
    const int warps = static_cast<int>((A.spa + A.parts - 1) / A.parts);
    const size_t smem = fx_smem_bytes(A.xblk, A.ns, A.lc, A.nlsp, warps);
    // Raise this instantiation's dynamic shared-memory limit once to what the
    // device allows next to its static arrays.
    static const size_t limit = [&] {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, fcix_spmm_kernel<MODE, K>);
        const size_t lim = csr->ctx->smem_optin > fa.sharedSizeBytes ? csr->ctx->smem_optin - fa.sharedSizeBytes : 0;
        cudaFuncSetAttribute(fcix_spmm_kernel<MODE, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(lim));
        return lim;
    }();
    if (smem > limit || A.nbeta >= 65536)
        return false;
    const int64_t blocks = csr->fx_nalpha * A.parts;
    fcix_spmm_kernel<MODE, K><<<static_cast<unsigned>(blocks), 32 * warps, smem, st>>>(
        A, static_cast<const float *>(x), y);
    note_launch();
    return true;
}

} // namespace pyci_gpu

using namespace pyci_gpu;

bool fcix_launch(const pyci_gpu_csr *csr, int mode, int K, const void *x, int64_t ldx, void *y, int64_t ldy,
                 cudaStream_t st) {
    if (!csr->fx_hi || !csr->fx_lo || csr->nrow >= INT32_MAX)
        return false;
    if (mode == 0) {
        // Interleaved blocks with row stride K, 16-byte aligned for K = 4, 8.
        const size_t align = (K % 4 == 0) ? 16 : (K == 2 ? 8 : 4);
        if (ldx != K || ldy != K || reinterpret_cast<uintptr_t>(x) % align)
            return false;
        switch (K) {
        case 1: return fx_launch_k<0, 1>(csr, x, y, st);
        case 2: return fx_launch_k<0, 2>(csr, x, y, st);
        case 3: return fx_launch_k<0, 3>(csr, x, y, st);
        case 4: return fx_launch_k<0, 4>(csr, x, y, st);
        case 5: return fx_launch_k<0, 5>(csr, x, y, st);
        case 6: return fx_launch_k<0, 6>(csr, x, y, st);
        case 7: return fx_launch_k<0, 7>(csr, x, y, st);
        case 8: return fx_launch_k<0, 8>(csr, x, y, st);
        default: return false;
        }
    }
    if (mode != 2 || ldx != 2 * K || ldy != K || reinterpret_cast<uintptr_t>(x) % 16)
        return false;
    switch (K) {
    case 1: return fx_launch_k<2, 1>(csr, x, y, st);
    case 2: return fx_launch_k<2, 2>(csr, x, y, st);
    case 4: return fx_launch_k<2, 4>(csr, x, y, st);
    default: return false;
    }
}
