// Tall-skinny Gram products C = A^T B of the block Davidson on the 5th-
// generation tensor cores (tcgen05, sm_103a), for FP32 vectors.
//
// A holds p <= 128 vectors and B q <= 8 vectors of N rows each, vector-major
// (element (i, r) at i * N + r).  One MMA computes a 128 x 16 tile of C over
// 8 rows: M = the A vectors (zero beyond p), N = the B vectors (zero beyond
// q), K = rows.  A CTA owns the 32-row tiles t = blockIdx.x, blockIdx.x +
// gridDim.x, ...; per tile its four warps load the vectors' 128-byte row
// segments with coalesced loads, split every value into TF32 high and low
// parts (hi = rna(x), lo = rna(x - hi)) and store both into shared memory in
// the MMA's no-swizzle K-major layout, and one thread issues 4 K-steps x
// {hi.hi, hi.lo, lo.hi} MMAs into FP32 accumulators in tensor memory.  The
// split keeps the products at ~2^-21 relative (a plain TF32 product loses
// ~2^-11), close to FP32 arithmetic.
//
// The tensor core's FP32 accumulation does not round to nearest: summing
// every tile of a CTA into one accumulator biased the diagonal of an
// orthonormal block's Gram by -3e-6 (~180 accumulations).  So each tile
// starts fresh accumulators -- the hi.hi products of K-steps 0-1 and 2-3 in
// two column ranges, the small hi.lo / lo.hi terms in a third -- and
// after the tile's MMAs complete each warp reads its 32 accumulator lanes with
// tcgen05.ld and adds them to per-thread FP32 sums (round to nearest, as in
// the CUDA-core kernel).  The CTA's partial C is written as FP64; a second
// kernel sums the partials over CTAs in FP64.
//
// Two loaders feed the same MMA stage.  For wide A blocks (p >= 96) whose
// rows are 16-byte aligned (N % 4 == 0), gram_tma_kernel streams each tile of
// A and B into a ring of shared-memory stages with TMA (cp.async.bulk.tensor,
// 128-byte swizzle, zero fill past N; up to 16 tiles in flight per CTA) and
// double-buffers the operand tiles and accumulators, and the warps split the
// landed tile into the hi/lo operand tiles (the swizzle makes both the reads
// and the writes bank-conflict-free).  Otherwise gram_tc_kernel loads each
// tile with plain coalesced loads into registers.
//
// Each MMA (128 x 16 x 8) does little work for its fixed cost, so for narrow
// blocks the product is bound by MMA latency, not by HBM: the eigensolver
// sends only its wide Gram products here and the rest to the CUDA-core kernel.
//
// The product reads every vector once and does (p x q) FMAs per row of 4(p+q)
// bytes, so at best it is HBM-bound like the CUDA-core version
// (gram_rows_kernel); the tensor cores take the multiply-adds off the FMA
// pipes.
//
// Waits on the MMA-completion mbarrier are bounded: on expiry the kernel
// records an error in g_gram_tc_error, writes NaN partials (so the caller's
// finite check fails), waits once more (bounded) for its MMAs, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "internal.h"

namespace pyci_gpu {

namespace {

constexpr int kM = 128;                          // MMA M: A vectors (padded)
constexpr int kN = 16;                           // MMA N: B vectors (padded)
constexpr int kDepth = 32;                       // rows per tile (4 MMAs of K = 8)
constexpr uint32_t kCoreK = 128;                 // bytes between core matrices along K
constexpr uint32_t kCoreMN = (kDepth / 4) * 128; // bytes between 8-row groups
constexpr uint32_t kTileA = kM * kDepth * 4;     // 16 KB
constexpr uint32_t kTileB = kN * kDepth * 4;     // 2 KB
constexpr uint32_t kTiles = 2 * kTileA + 2 * kTileB;
// Operand tiles + alignment slack, padded so at most four CTAs share an SM
// (4 x kTmemCols = the SM's 512 tensor-memory columns).
constexpr uint32_t kSmemBytes = (kTiles + 1024 > 46u * 1024u) ? kTiles + 1024 : 46u * 1024u;
constexpr uint32_t kTmemCols = 128;              // six accumulators of kN columns (power of 2)
constexpr uint32_t kWaitLimit = 1u << 22;        // mbarrier polls before giving up

// Instruction descriptor of tcgen05.mma kind::tf32: D F32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(kN >> 3) << 17) |
                            (static_cast<uint32_t>(kM >> 4) << 24);

__device__ int g_gram_tc_error = 0;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (between core matrices along K), stride byte offset (between 8-row
// groups), all >> 4; bits 46-48 hold the fixed value 0b001.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((kCoreK >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((kCoreMN >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity))
            return true;
    return false;
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x -> (hi, lo) TF32 pair, four values at a time.
__device__ __forceinline__ void split4(const float4 x, uint4 &hi, uint4 &lo) {
    hi.x = tf32_rna(x.x);
    hi.y = tf32_rna(x.y);
    hi.z = tf32_rna(x.z);
    hi.w = tf32_rna(x.w);
    lo.x = tf32_rna(x.x - __uint_as_float(hi.x));
    lo.y = tf32_rna(x.y - __uint_as_float(hi.y));
    lo.z = tf32_rna(x.z - __uint_as_float(hi.z));
    lo.w = tf32_rna(x.w - __uint_as_float(hi.w));
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// Four floats of row segment `src` (element offset e from the tile start),
// zero past N.
template<bool VEC>
__device__ __forceinline__ float4 load4(const float *__restrict__ src, int64_t r, int64_t N) {
    if constexpr (VEC) {
        // N % 4 == 0 and 16-byte aligned vectors: r < N implies r + 3 < N.
        return r < N ? __ldg(reinterpret_cast<const float4 *>(src + r)) : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        float4 v;
        v.x = r < N ? __ldg(src + r) : 0.f;
        v.y = r + 1 < N ? __ldg(src + r + 1) : 0.f;
        v.z = r + 2 < N ? __ldg(src + r + 2) : 0.f;
        v.w = r + 3 < N ? __ldg(src + r + 3) : 0.f;
        return v;
    }
}

// Read the first 8 columns of the six accumulators for this warp's 32
// lanes (rows of C) and add them to the thread's FP32 sums.  Waits for the
// tile's MMAs (mbarrier) must precede it.
__device__ __forceinline__ void drain(uint32_t tmem, int warp, float acc[8]) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    uint32_t r[6][8];
#pragma unroll
    for (int a = 0; a < 6; ++a)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(r[a][0]), "=r"(r[a][1]), "=r"(r[a][2]), "=r"(r[a][3]), "=r"(r[a][4]), "=r"(r[a][5]),
                       "=r"(r[a][6]), "=r"(r[a][7])
                     : "r"(taddr + static_cast<uint32_t>(a * 16))
                     : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float small = (__uint_as_float(r[0][j]) + __uint_as_float(r[1][j])) +
                            (__uint_as_float(r[2][j]) + __uint_as_float(r[3][j]));
        acc[j] += (__uint_as_float(r[4][j]) + __uint_as_float(r[5][j])) + small;
    }
}

// One tile's MMAs (4 K-steps x 3 terms; lo.lo, ~2^-22 of a product, is
// left out) into six accumulators of kN columns each, so that no MMA
// waits on the one before it: region 4 + k/2 takes hi.hi of K-steps k, and
// region k (0..3) takes lo.hi and hi.lo of K-step k.  Issued in two rounds
// of six independent MMAs (the first of each region restarts it), then one
// commit of all of them to `bar`.  A chain of dependent accumulations would
// expose the MMA latency on every step.

__device__ __forceinline__ void issue_tile_mmas(uint32_t tmem, uint32_t sa_hi, uint32_t sa_lo, uint32_t sb_hi,
                                                uint32_t sb_lo, uint32_t bar) {
    // 8 rows of K = 2 core matrices.
    auto d = [&](uint32_t a, int k) { return smem_desc(a + static_cast<uint32_t>(k) * 2u * kCoreK); };
    auto region = [&](int r) { return tmem + static_cast<uint32_t>(r * kN); };
#pragma unroll
    for (int k = 0; k < kDepth / 8; ++k)
        mma_tf32(region(k), d(sa_lo, k), d(sb_hi, k), 0u);
    mma_tf32(region(4), d(sa_hi, 0), d(sb_hi, 0), 0u);
    mma_tf32(region(5), d(sa_hi, 2), d(sb_hi, 2), 0u);
#pragma unroll
    for (int k = 0; k < kDepth / 8; ++k)
        mma_tf32(region(k), d(sa_hi, k), d(sb_lo, k), 1u);
    mma_tf32(region(4), d(sa_hi, 1), d(sb_hi, 1), 1u);
    mma_tf32(region(5), d(sa_hi, 3), d(sb_hi, 3), 1u);
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Write the CTA's partial C (FP64) or, after a failed wait, NaN.
__device__ __forceinline__ void write_partial(double *out, int p, int q, int warp, int lane, const float acc[8],
                                              bool failed) {
    const int i = warp * 32 + lane; // accumulator lane = row of C
    if (i < p) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (j < q)
                out[i * q + j] = failed ? __longlong_as_double(0x7ff8000000000000ll) : static_cast<double>(acc[j]);
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int32_t x, int32_t y,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Loader tasks: 8 vectors x 32 rows each (A tasks first, then the one B
// task); warp w takes tasks w, w + 4, ...; at most 16 + 1 tasks.
constexpr int kTasksPerWarp = 5;

template<bool VEC>
__global__ void __launch_bounds__(128) gram_tc_kernel(const float *__restrict__ A, int p, const float *__restrict__ B,
                                                      int q, int64_t N, double *__restrict__ partial) {
    extern __shared__ uint8_t dyn_smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    uint8_t *tiles = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~uintptr_t(1023));
    uint8_t *a_hi = tiles, *a_lo = tiles + kTileA, *b_hi = tiles + 2 * kTileA, *b_lo = b_hi + kTileB;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t bar_addr = smem_addr(&bar);

    // Padding rows (A beyond p, B beyond q) only reach discarded entries of
    // C; they are zeroed so the accumulator holds no stray NaN/Inf.
    for (uint32_t i = tid; i < kTiles / 16; i += blockDim.x)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_addr) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    const int ga = (p + 7) >> 3;
    const int ntask = ga + 1;
    const int row8 = lane & 7;   // vector within the task's group of 8
    const int chunk = lane >> 3; // 16-byte chunks `chunk` and `chunk + 4` of the 128-byte segment
    const int64_t ntiles = (N + kDepth - 1) / kDepth;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}; // row warp*32+lane of C, columns 0..7
    int it = 0;
    bool failed = false;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int64_t r0 = t * kDepth;
        float4 raw[kTasksPerWarp][2];
#pragma unroll
        for (int s = 0; s < kTasksPerWarp; ++s) {
            const int task = warp + 4 * s;
            raw[s][0] = raw[s][1] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (task < ntask) {
                const int v = (task < ga ? task : task - ga) * 8 + row8;
                if (task < ga ? v < p : v < q) {
                    const float *src = (task < ga ? A : B) + static_cast<int64_t>(v) * N;
                    raw[s][0] = load4<VEC>(src, r0 + 4 * chunk, N);
                    raw[s][1] = load4<VEC>(src, r0 + 4 * (chunk + 4), N);
                }
            }
        }
        // The previous tile's MMAs must have finished reading shared memory
        // and writing their accumulators.
        bool late = false;
        if (it > 0)
            late = !mbar_wait(bar_addr, static_cast<uint32_t>(it - 1) & 1u);
        if (__syncthreads_or(late)) {
            failed = true;
            break;
        }
        if (it > 0)
            drain(tmem, warp, acc);
#pragma unroll
        for (int s = 0; s < kTasksPerWarp; ++s) {
            const int task = warp + 4 * s;
            if (task < ntask) {
                const bool is_a = task < ga;
                const uint32_t grp = static_cast<uint32_t>(is_a ? task : task - ga);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t off = grp * kCoreMN + static_cast<uint32_t>(chunk + 4 * h) * kCoreK +
                                         static_cast<uint32_t>(row8) * 16u;
                    uint4 hi, lo;
                    split4(raw[s][h], hi, lo);
                    *reinterpret_cast<uint4 *>((is_a ? a_hi : b_hi) + off) = hi;
                    *reinterpret_cast<uint4 *>((is_a ? a_lo : b_lo) + off) = lo;
                }
            }
        }
        // Make the generic-proxy stores visible to the tensor core's reads, and
        // order this tile's MMAs after every warp's accumulator reads.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            issue_tile_mmas(tmem, smem_addr(a_hi), smem_addr(a_lo), smem_addr(b_hi), smem_addr(b_lo), bar_addr);
        }
    }

    double *out = partial + static_cast<int64_t>(blockIdx.x) * (p * q);
    if (!failed && it > 0 && __syncthreads_or(!mbar_wait(bar_addr, static_cast<uint32_t>(it - 1) & 1u)))
        failed = true;
    if (failed) {
        if (tid == 0)
            atomicExch(&g_gram_tc_error, 1);
        // Give outstanding MMAs one more bounded wait before freeing their accumulator.
        if (it > 0)
            mbar_wait(bar_addr, static_cast<uint32_t>(it - 1) & 1u);
    } else if (it > 0) {
        drain(tmem, warp, acc);
    }
    write_partial(out, p, q, warp, lane, acc, failed);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// TMA-fed version, double-buffered: tile `it` is split into operand buffer
// it % 2 and accumulated into accumulator set it % 2 (columns 64 (it % 2) +
// [0, 3 kN)), so its MMAs run while the warps split tile it + 1; tile it + 2
// waits for them.  Dynamic shared memory: two sets of hi/lo operand tiles
// (no swizzle, 1024-aligned), then `stages` raw stages of stage_bytes each
// (A's p x 32 box at 0, B's q x 32 box at b_off, 128-byte swizzled), as TMA
// lands them.
constexpr int kMaxStages = 16;
constexpr uint32_t kTmaTmemCols = 256; // two accumulator sets of 128 columns

__global__ void __launch_bounds__(128) gram_tma_kernel(const __grid_constant__ CUtensorMap mapA,
                                                       const __grid_constant__ CUtensorMap mapB, int p, int q,
                                                       int64_t N, int stages, uint32_t stage_bytes, uint32_t b_off,
                                                       double *__restrict__ partial) {
    extern __shared__ uint8_t dyn_smem[];
    __shared__ __align__(8) uint64_t full[kMaxStages];
    __shared__ __align__(8) uint64_t mma_done[2];
    __shared__ uint32_t tmem_slot;
    uint8_t *tiles = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~uintptr_t(1023));
    uint8_t *ring = tiles + 2 * kTiles;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ring_addr = smem_addr(ring);

    for (uint32_t i = tid; i < 2 * kTiles / 16; i += blockDim.x)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kTmaTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < stages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full[s])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mma_done[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mma_done[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    // This CTA's tiles: blockIdx.x + j * gridDim.x for j < mine.
    const int64_t ntiles = (N + kDepth - 1) / kDepth;
    const int64_t mine = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t tx_bytes = static_cast<uint32_t>(p + q) * (kDepth * 4);
    auto issue = [&](int64_t j) {
        const int s = static_cast<int>(j % stages);
        const uint32_t bar = smem_addr(&full[s]);
        const uint32_t dst = ring_addr + static_cast<uint32_t>(s) * stage_bytes;
        const int32_t x = static_cast<int32_t>((blockIdx.x + j * gridDim.x) * kDepth);
        mbar_expect_tx(bar, tx_bytes);
        tma_load_2d(dst, &mapA, x, 0, bar);
        tma_load_2d(dst + b_off, &mapB, x, 0, bar);
    };
    if (tid == 0)
        for (int64_t j = 0; j < stages && j < mine; ++j)
            issue(j);
    // Wait for the MMAs of tile j (the (j / 2)-th commit on mma_done[j % 2]).
    auto wait_mma = [&](int64_t j) {
        return mbar_wait(smem_addr(&mma_done[j & 1]), static_cast<uint32_t>((j >> 1) & 1));
    };

    const int ga = (p + 7) >> 3;
    const int ntask = ga + 1;
    const int row8 = lane & 7;
    const int chunk = lane >> 3;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int64_t it = 0;
    bool failed = false;
    for (; it < mine; ++it) {
        const int s = static_cast<int>(it % stages);
        const int b = static_cast<int>(it & 1);
        uint8_t *a_hi = tiles + b * kTiles, *a_lo = a_hi + kTileA, *b_hi = a_hi + 2 * kTileA, *b_lo = b_hi + kTileB;
        const uint8_t *stage = ring + static_cast<size_t>(s) * stage_bytes;
        bool late = !mbar_wait(smem_addr(&full[s]), static_cast<uint32_t>((it / stages) & 1));
        // Raw tile -> registers.
        float4 raw[kTasksPerWarp][2];
        uint32_t offs[kTasksPerWarp][2];
#pragma unroll
        for (int t = 0; t < kTasksPerWarp; ++t) {
            const int task = warp + 4 * t;
            const bool is_a = task < ga;
            const int grp = is_a ? task : task - ga;
            const int v = grp * 8 + row8;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = chunk + 4 * h;
                // Raw box: 128-byte swizzle (chunk c of row v at c ^ (v % 8));
                // operand tiles: no-swizzle core matrices.  Both mappings are
                // conflict-free for this lane layout.
                const uint32_t src = static_cast<uint32_t>(grp * 1024 + row8 * 128 + ((c ^ row8) * 16));
                offs[t][h] = static_cast<uint32_t>(grp) * kCoreMN + static_cast<uint32_t>(c) * kCoreK +
                             static_cast<uint32_t>(row8) * 16u;
                raw[t][h] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (task < ntask && (is_a ? v < p : v < q))
                    raw[t][h] = *reinterpret_cast<const float4 *>(stage + (is_a ? 0u : b_off) + src);
            }
        }
        // Tile it - 2 used this operand buffer and accumulator set.
        if (it >= 2)
            late = late || !wait_mma(it - 2);
        if (__syncthreads_or(late)) {
            failed = true;
            break;
        }
        // Every thread has read stage s: refill it with a later tile.
        if (tid == 0 && it + stages < mine)
            issue(it + stages);
        if (it >= 2)
            drain(tmem + static_cast<uint32_t>(b * 128), warp, acc);
#pragma unroll
        for (int t = 0; t < kTasksPerWarp; ++t) {
            const int task = warp + 4 * t;
            if (task < ntask) {
                const bool is_a = task < ga;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint4 hi, lo;
                    split4(raw[t][h], hi, lo);
                    *reinterpret_cast<uint4 *>((is_a ? a_hi : b_hi) + offs[t][h]) = hi;
                    *reinterpret_cast<uint4 *>((is_a ? a_lo : b_lo) + offs[t][h]) = lo;
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            issue_tile_mmas(tmem + static_cast<uint32_t>(b * 128), smem_addr(a_hi), smem_addr(a_lo),
                                  smem_addr(b_hi), smem_addr(b_lo), smem_addr(&mma_done[b]));
        }
    }

    double *out = partial + static_cast<int64_t>(blockIdx.x) * (p * q);
    if (!failed) {
        // Drain the last two tiles.
        for (int64_t j = (it >= 2 ? it - 2 : 0); j < it && !failed; ++j) {
            if (__syncthreads_or(!wait_mma(j)))
                failed = true;
            else
                drain(tmem + static_cast<uint32_t>((j & 1) * 128), warp, acc);
        }
    }
    if (failed) {
        if (tid == 0)
            atomicExch(&g_gram_tc_error, 1);
        // Bounded waits for this CTA's MMAs and TMA copies still in flight.
        for (int64_t j = (it >= 2 ? it - 2 : 0); j < it; ++j)
            wait_mma(j);
        for (int64_t j = it; j < mine && j < it + stages; ++j)
            mbar_wait(smem_addr(&full[j % stages]), static_cast<uint32_t>((j / stages) & 1));
    }
    write_partial(out, p, q, warp, lane, acc, failed);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmaTmemCols)
                     : "memory");
    }
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// Map of `rows` FP32 vectors of N elements (vector-major) with a box of
// `rows` vectors x 32 elements, 128-byte swizzle, zero fill past N.
bool encode_vectors(CUtensorMap *map, const float *base, int rows, int64_t N) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc)
        return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(N), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(N) * 4u};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(kDepth), static_cast<cuuint32_t>(rows)};
    const cuuint32_t estr[2] = {1u, 1u};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr uint32_t kTmaSmemTarget = 110 * 1024; // per CTA: two CTAs per SM
// The TMA loader pays off for wide A blocks only (measured on 10.5M-row
// vectors, q = 4..8: p = 128 2.0 ms vs 2.3 ms with direct loads; p = 64
// 1.8 ms vs 1.2 ms).
constexpr int kTmaMinP = 96;

} // namespace

unsigned launch_gram_tc(unsigned budget, cudaStream_t st, const float *A, int p, const float *B, int q, int64_t N,
                        double *partial) {
    const int64_t ntiles = (N + kDepth - 1) / kDepth;
    const bool vec = (N % 4 == 0) && (reinterpret_cast<uintptr_t>(A) % 16 == 0) &&
                     (reinterpret_cast<uintptr_t>(B) % 16 == 0);
    CUtensorMap mapA, mapB;
    if (vec && p >= kTmaMinP && N < (int64_t(1) << 31) && encode_vectors(&mapA, A, p, N) &&
        encode_vectors(&mapB, B, q, N)) {
        const uint32_t b_off = (static_cast<uint32_t>(p) * kDepth * 4 + 1023u) & ~1023u;
        const uint32_t stage_bytes = b_off + 1024u;
        const uint32_t fixed = 1024u + 2 * kTiles;
        const int stages = static_cast<int>(std::max<uint32_t>(2, std::min<uint32_t>(kMaxStages, (kTmaSmemTarget - fixed) / stage_bytes)));
        const uint32_t smem = fixed + static_cast<uint32_t>(stages) * stage_bytes;
        cudaFuncSetAttribute(gram_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        int dev = 0, sms = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        // CTAs per SM by shared memory (1 KB reserved per CTA), at most two
        // (2 x kTmaTmemCols = 512 tensor-memory columns).
        const int per_sm = std::max(1, std::min(2, smem_sm / static_cast<int>(smem + 1024)));
        const int64_t want = static_cast<int64_t>(sms) * per_sm;
        const unsigned nb = static_cast<unsigned>(
            std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(budget, want), ntiles)));
        gram_tma_kernel<<<nb, 128, smem, st>>>(mapA, mapB, p, q, N, stages, stage_bytes, b_off, partial);
        note_launch();
        return nb;
    }
    const unsigned nb = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(budget, ntiles)));
    if (vec)
        gram_tc_kernel<true><<<nb, 128, kSmemBytes, st>>>(A, p, B, q, N, partial);
    else
        gram_tc_kernel<false><<<nb, 128, kSmemBytes, st>>>(A, p, B, q, N, partial);
    note_launch();
    return nb;
}

int gram_tc_error(bool clear) {
    int v = 0;
    cudaMemcpyFromSymbol(&v, g_gram_tc_error, sizeof(int));
    if (clear && v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_gram_tc_error, &zero, sizeof(int));
    }
    return v;
}

} // namespace pyci_gpu
