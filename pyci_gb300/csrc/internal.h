// Internal host-side definitions shared by the CUDA translation units of
// libpyci_gb300.so.  Nothing here is part of the C ABI (include/pyci_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pyci_gb300.h"

class PinnedRing;

struct pyci_gpu_ctx {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    PinnedRing *ring = nullptr; // pinned staging for small uploads (created with the context)
    // Mapped pinned buffer of the eigensolver's Gram read-backs, pinned once
    // per context rather than once per solve (pinning host memory takes
    // milliseconds, at varying cost); one solve at a time holds it, others
    // pin their own.  Freed with the context.
    double *mapped_host = nullptr;
    double *mapped_dev = nullptr; // its device alias, or null
    std::atomic<bool> mapped_busy{false};
};

// Device-resident CSR of the CI Hamiltonian.
//
// Storage: rows 0..nrow-1, columns sorted ascending in each row, int32
// column indices, int64 row pointers.  For a symmetric operator both
// triangles are stored (so the SpMV is a pure gather); the reference's
// lower-triangle layout is the prefix of each row up to and including the
// diagonal, whose length is kept in lower_len.
struct pyci_gpu_csr {
    pyci_gpu_ctx *ctx = nullptr;
    int kind = 0;
    int flags = 0;
    int64_t nbasis = 0, nocc_up = 0, nocc_dn = 0;
    int64_t ndet = 0, nrow = 0, ncol = 0;
    bool symmetric = true;
    int64_t nnz = 0;      // entries stored on the device
    int64_t nnz_ref = 0;  // entries in the reference's layout
    int64_t *rowptr = nullptr;   // [nrow + 1]
    int32_t *cols = nullptr;     // [nnz]
    double *vals = nullptr;      // [nnz] FP64 values (null after prepare_mixed(drop))
    float *hi = nullptr;         // [nnz] FP32 high part (mixed precision)
    float *lo = nullptr;         // [nnz] FP32 low part: f32(v - hi)
    int32_t *lower_len = nullptr; // [nrow] reference entries per row (symmetric)
    int64_t *ref_rowptr = nullptr; // [nrow + 1] prefix sum of lower_len (symmetric)
    double *diag = nullptr;      // [nrow] diagonal (0 where absent)
    int spmm_lanes = 32;         // lanes per row suggested by the mean row length
    // SpMM tile variant chosen by the autotuner per (value kind, width k <= 8),
    // -1 until the first product with that pair.
    // Kinds: FP64, FP32, FP64 from high + low, double-float from high + low.
    mutable int tuned[4][9] = {{-1, -1, -1, -1, -1, -1, -1, -1, -1},
                               {-1, -1, -1, -1, -1, -1, -1, -1, -1},
                               {-1, -1, -1, -1, -1, -1, -1, -1, -1},
                               {-1, -1, -1, -1, -1, -1, -1, -1, -1}};
    // GenCI in the reference's own row loop (see genci_ref_* in build.cu):
    // only the reference's layout is stored; a symmetric product then
    // scatters the transpose with atomics.
    bool lower_only = false;
    // SELL-32 copy of the split operator (high and low FP32 parts), built
    // with the mixed-precision split when rows within each 32-row slice have (nearly) equal
    // lengths: entry j of slice s, lane l (row 32 s + l) at sell_off[s] + 32 j
    // + l; shorter rows padded with zero values.  One lane per row walks its
    // row while the warp's 32 rows share column blocks of x (consecutive FCI
    // rows share their alpha string), so the gathers of a warp share cache
    // lines.  Null when not built.
    int64_t nslice = 0;
    int64_t sell_nnz = 0;
    int64_t *sell_off = nullptr;  // [nslice + 1], multiples of 32
    int32_t *sell_cols = nullptr; // [sell_nnz]
    float *sell_vals = nullptr;   // [sell_nnz] high parts
    float *sell_lo = nullptr;     // [sell_nnz] low parts
    // Implicit-column form of a full FullCI space (fcix.cu): the columns of
    // row (a, b) follow from per-string tables, so products stream values
    // only.  Each row is stored as three sections: A = the alpha string
    // itself with every beta partner (sorted {b} + singles + doubles), B =
    // each alpha single with sorted {b} + beta singles (one group per
    // single), C = each alpha double with b; A, C and each group of B padded
    // to a multiple of 4 entries.  Tables and values (FP32 high and low
    // parts, in 4-entry packets) are written by the sorted FullCI build
    // (fcix_fill_kernel), the CSR on first use.  Null when the operator is
    // not a full FullCI space.
    int64_t fx_nalpha = 0, fx_nbeta = 0, fx_nbp = 0; // strings per spin; beta count padded to 32
    int64_t fx_npk = 0;           // 4-entry packets per row (padded length / 4)
    int fx_ns = 0, fx_nd = 0;     // alpha singles / doubles per alpha string
    int fx_nlb = 0, fx_nls = 0;   // beta partners in section A / per group of section B
    int fx_la = 0, fx_lb = 0, fx_lc = 0; // padded section lengths
    int32_t *fx_atab = nullptr;   // [nalpha][2 (ns + nd) + 1]: single targets, double targets,
                                  // their CSR offsets in the sorted row, the offset of section A's group
    int32_t *fx_bfull = nullptr;  // [nlb][nbeta]: sorted {b} + singles + doubles, transposed
    int32_t *fx_bsub = nullptr;   // [nls][nbeta]: sorted {b} + singles, transposed
    uint16_t *fx_bq = nullptr;    // [la / 4][nbeta][4]: section A's partners by packet (padding: b)
    float *fx_hi = nullptr;       // [nslice][npk][32][4] high parts
    float *fx_lo = nullptr;       // [nslice][npk][32][4] low parts
    // Implicit form of a full DOCI space (docx.cu): columns from each row's
    // occupation, values from the pair-integral table, so a product reads no
    // stored entries.  Null when the operator is not a full DOCI space.
    int dx_n = 0, dx_m = 0, dx_ldk = 0; // orbitals, pairs, binomial row length (m + 2)
    int64_t *dx_binom = nullptr;        // [(n + 1) * ldk]: C(o, k)
    float *dx_v = nullptr;              // [2][n][n]: v split into high and low parts
    // Deferred CSR: an operator with the implicit-column form is built
    // without its CSR entries (cols, vals null) unless PYCI_BUILD_EAGER_CSR
    // asks for them; this holds what the CSR fill needs (build.cu), and
    // csr_materialize() writes the entries on first use.  Null otherwise.
    void *deferred = nullptr;
    // prepare_mixed(drop_fp64) was asked for: FP64 values written later (a
    // deferred CSR) are freed again once the CSR-order split exists.
    bool drop_fp64 = false;
};

// Width of one alpha string's row of pyci_gpu_csr::fx_atab.
inline int fx_atab_width(const pyci_gpu_csr *c) { return 2 * (c->fx_ns + c->fx_nd) + 1; }

// Whether the operator has an implicit form (full FullCI or full DOCI space)
// that serves its FP32 and double-float products.
inline bool has_implicit(const pyci_gpu_csr *c) { return c->fx_hi || c->dx_v; }

namespace pyci_gpu {
// Kernel launches issued by this library (diagnostic counter).
void note_launch();
// Whether PYCI_GPU_SPMM pins products to the CSR or SELL-32 kernels (spmv.cu).
bool pinned_to_csr();
} // namespace pyci_gpu

// Thread-local error message.
void set_error(const char *fmt, ...);

// Map a CUDA failure to a status code and message.
int cuda_status(cudaError_t err, const char *what);

#define PYCI_CUDA_TRY(expr)                                                                        \
    do {                                                                                           \
        cudaError_t e_ = (expr);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return cuda_status(e_, #expr);                                                         \
    } while (0)

// Internal launchers (implemented in the .cu files).
int csr_build_device(pyci_gpu_ctx *ctx, pyci_gpu_csr *csr, const uint64_t *dets_host,
                     const double *one_mo, const double *two_mo, int64_t legacy_nrow,
                     int64_t legacy_ncol);
int csr_spmm(const pyci_gpu_csr *csr, int precision, int64_t k, const void *x, void *y,
             cudaStream_t stream);
// y[N][K] = (hi + lo) x with FP32 arithmetic and double-float accumulation;
// xs[N][2K] holds each row's FP32 high parts then low parts; K = 1, 2 or 4.
int csr_spmm_df(const pyci_gpu_csr *csr, int K, const float *xs, double *y, cudaStream_t stream);
void csr_release(pyci_gpu_csr *csr);
// Implicit-column form (fcix.cu).  fcix_launch runs one product on it: mode 0 FP32 (x, y
// float [N][K], K <= 8), mode 2 double-float (xs float [N][2K], y double
// [N][K], K = 1, 2, 4).  FP64 arithmetic is not offered: forming hi + lo in
// FP64 costs three FP64 instructions per entry on top of the FMA, and this
// GPU's FP64 pipe already bounds the CSR FP64 product.  Returns false when
// the operator has no values in this form or the operands do not fit it (the
// caller then uses another kernel).
bool fcix_launch(const pyci_gpu_csr *csr, int mode, int K, const void *x, int64_t ldx, void *y, int64_t ldy,
                 cudaStream_t st);
// The same on the implicit form of a full DOCI space (docx.cu).
bool docx_launch(const pyci_gpu_csr *csr, int mode, int K, const void *x, int64_t ldx, void *y, int64_t ldy,
                 cudaStream_t st);
// FP32 product on the implicit DOCI form with x as rows of K values and y
// written as K columns of nrow values (y + k * nrow); false when it does not
// apply.
bool docx_launch_columns(const pyci_gpu_csr *csr, int K, const float *x, float *y, cudaStream_t st);
// Whichever implicit form the operator has.
inline bool implicit_launch(const pyci_gpu_csr *csr, int mode, int K, const void *x, int64_t ldx, void *y,
                            int64_t ldy, cudaStream_t st) {
    return csr->dx_v ? docx_launch(csr, mode, K, x, ldx, y, ldy, st) : fcix_launch(csr, mode, K, x, ldx, y, ldy, st);
}
// Writes a deferred CSR's entries (no-op when there is nothing deferred);
// every path that reads cols or vals calls it first.  Logically const: the
// operator's contents do not change.
int csr_materialize(const pyci_gpu_csr *csr);
void csr_deferred_free(pyci_gpu_csr *csr);
int csr_export_device(const pyci_gpu_csr *csr, double *data, int64_t *indices, int64_t *indptr);
int csr_digest_device(const pyci_gpu_csr *csr, uint64_t *psum, uint64_t *pxor, double *vsum,
                      double *vabs, double *vwsum);
int csr_prepare_mixed_device(pyci_gpu_csr *csr, int drop_fp64);
int csr_ensure_split(pyci_gpu_csr *csr);
int add_all_dets_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                        int64_t nocc_dn, uint64_t *dets_host);
int davidson_solve(pyci_gpu_csr *csr, int64_t n, const double *c0, int64_t ncv, int64_t maxiter,
                   double tol, double ecore, int mode, double *evals, double *evecs,
                   pyci_gpu_solve_stats *stats);

int64_t host_binomial(int64_t n, int64_t k);

// Exclusive scan of counts[n] into out[n + 1] (out[n] = total) on `stream`.
int device_exclusive_scan(const int64_t *counts, int64_t n, int64_t *out, cudaStream_t stream);
// Device determinant hash table (build.cu): slots from the stream's pool.
int det_table_build(const uint64_t *d_dets, int64_t ndet, int nwords, cudaStream_t st, int *d_err,
                    int32_t **slots, uint64_t *mask);
// Reduced density matrices on the device (rdm.cu), pyci_gpu_compute_rdms.
// dets2 == NULL: RDMs of (dets, coeffs); otherwise transition RDMs against
// (dets2, coeffs2).
int rdm_compute_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t ndet, const uint64_t *dets,
                       const double *coeffs, int64_t ndet2, const uint64_t *dets2, const double *coeffs2,
                       double *rdm1, double *rdm2);
// Epstein-Nesbet second-order energy on the device (hci.cu), pyci_gpu_compute_enpt2.
int enpt2_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                 const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo, double energy,
                 double ecore, double eps, double *result);
// Heat-bath CI selection on the device (hci.cu), pyci_gpu_add_hci.
int hci_select_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                      const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo,
                      double eps, int flags, int64_t max_new, uint64_t *out, int64_t *n_new);

namespace pyci_gpu {
// Tensor-core Gram partials (gram_tc.cu): partial[b][i * q + j] = sum over
// the rows of CTA b of A[i][r] B[j][r], p <= 128, q <= 8, FP32 vectors with
// N rows (vector-major).  Returns the number of CTAs (partials per entry).
unsigned launch_gram_tc(unsigned budget, cudaStream_t st, const float *A, int p, const float *B, int q, int64_t N,
                        double *partial);
// Nonzero when a tensor-core Gram kernel gave up waiting for its MMAs
// (its partials are then NaN); `clear` resets the flag.
int gram_tc_error(bool clear);
// Whether the FP32 Gram products use the tensor cores (PYCI_GPU_GRAM=cuda
// selects the CUDA-core kernel instead).
bool gram_tc_enabled();
// C (host, p x q row-major) = A^T B for FP32 vectors on the device
// (method 0: CUDA cores, 1: tensor cores); pyci_gpu_gram_device.
int gram_device(pyci_gpu_ctx *ctx, int method, const float *A, int64_t p, const float *B, int64_t q, int64_t N,
                double *C);
} // namespace pyci_gpu

// Seeded perturbation of the Davidson start vectors.  Unit vectors on the
// lowest diagonal elements can all lie in one symmetry sector of H (e.g.
// symmetric under alpha <-> beta exchange), and the sector of a skipped root
// is then fed only by the corrections of roots that happen to share it: once
// those converge, the skipped root is never found.  A small deterministic
// component in every row (relative norm kGuessNoise / sqrt(3)) gives every
// sector a start, as the reference's random Lanczos start vector does.
constexpr double kGuessNoise = 1e-3;

// Uniform in [-1, 1) from (row, column) via the splitmix64 finaliser.
__host__ __device__ inline double guess_noise(uint64_t row, uint64_t col) {
    uint64_t z = row * 0x9E3779B97F4A7C15ull + (col + 1) * 0xD1B54A32D192ED03ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Asynchronous host -> device uploads of small coefficient blocks through a
// ring of pinned staging buffers.  A cudaMemcpyAsync from pageable memory
// first synchronises the stream, which would stall the GPU once per upload;
// from pinned memory it is queued like a kernel.  A slot is reused only after
// the event recorded behind its previous copy has completed.
class PinnedRing {
public:
    ~PinnedRing() {
        for (size_t i = 0; i < buf_.size(); ++i) {
            if (ev_[i]) {
                cudaEventSynchronize(ev_[i]);
                cudaEventDestroy(ev_[i]);
            }
            if (buf_[i])
                cudaFreeHost(buf_[i]);
        }
    }
    // nslot buffers of `bytes` each.
    int init(int nslot, size_t bytes) {
        bytes_ = bytes;
        buf_.assign(nslot, nullptr);
        ev_.assign(nslot, nullptr);
        for (int i = 0; i < nslot; ++i) {
            PYCI_CUDA_TRY(cudaMallocHost(&buf_[i], bytes));
            PYCI_CUDA_TRY(cudaEventCreateWithFlags(&ev_[i], cudaEventDisableTiming));
        }
        return PYCI_GPU_OK;
    }
    // dst[0..n) = src[0..n) (bytes) on stream st, asynchronously.
    int upload(void *dst, const void *src, size_t n, cudaStream_t st) {
        std::lock_guard<std::mutex> lock(mu_);
        if (buf_.empty() || n > bytes_) {
            PYCI_CUDA_TRY(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st));
            return PYCI_GPU_OK;
        }
        const int s = next_;
        next_ = (next_ + 1) % static_cast<int>(buf_.size());
        PYCI_CUDA_TRY(cudaEventSynchronize(ev_[s])); // its previous copy has been consumed
        std::memcpy(buf_[s], src, n);
        PYCI_CUDA_TRY(cudaMemcpyAsync(dst, buf_[s], n, cudaMemcpyHostToDevice, st));
        PYCI_CUDA_TRY(cudaEventRecord(ev_[s], st));
        return PYCI_GPU_OK;
    }

private:
    std::vector<void *> buf_;
    std::vector<cudaEvent_t> ev_;
    size_t bytes_ = 0;
    int next_ = 0;
    std::mutex mu_;
};
