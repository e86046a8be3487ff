// C-ABI entry points of libpyci_gb300.so (declared in include/pyci_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "internal.h"

#include <atomic>

namespace {
thread_local char g_error[1024] = "";
std::atomic<int64_t> g_launches{0};
} // namespace

namespace pyci_gpu {
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
} // namespace pyci_gpu

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t err, const char *what) {
    set_error("%s: %s", what, cudaGetErrorString(err));
    if (err == cudaErrorMemoryAllocation) {
        cudaGetLastError(); // clear the sticky-free allocation error
        return PYCI_GPU_ENOMEM;
    }
    return PYCI_GPU_ECUDA;
}

// Drops the implicit-column arrays from a handle (their memory is owned
// elsewhere or already freed).
static void fx_forget(pyci_gpu_csr *csr) {
    csr->fx_atab = csr->fx_bfull = csr->fx_bsub = nullptr;
    csr->fx_bq = nullptr;
    csr->fx_hi = csr->fx_lo = nullptr;
    csr->fx_nalpha = csr->fx_nbeta = csr->fx_nbp = csr->fx_npk = 0;
    csr->fx_ns = csr->fx_nd = csr->fx_nlb = csr->fx_nls = 0;
    csr->fx_la = csr->fx_lb = csr->fx_lc = 0;
    csr->dx_binom = nullptr;
    csr->dx_v = nullptr;
    csr->dx_n = csr->dx_m = csr->dx_ldk = 0;
}

void csr_release(pyci_gpu_csr *csr) {
    if (!csr || !csr->ctx)
        return;
    cudaStream_t st = csr->ctx->stream;
    csr_deferred_free(csr);
    void *ptrs[] = {csr->rowptr,     csr->cols,     csr->vals,     csr->hi,        csr->lo,        csr->lower_len,
                    csr->ref_rowptr, csr->diag,     csr->sell_off, csr->sell_cols, csr->sell_vals,
                    csr->sell_lo,    csr->fx_atab,  csr->fx_bfull, csr->fx_bsub,   csr->fx_hi,
                    csr->fx_lo,      csr->fx_bq,    csr->dx_binom, csr->dx_v};
    for (void *p : ptrs)
        if (p)
            cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    csr->rowptr = nullptr;
    csr->cols = nullptr;
    csr->vals = nullptr;
    csr->hi = csr->lo = nullptr;
    csr->lower_len = nullptr;
    csr->ref_rowptr = nullptr;
    csr->diag = nullptr;
    csr->sell_off = nullptr;
    csr->sell_cols = nullptr;
    csr->sell_vals = nullptr;
    csr->sell_lo = nullptr;
    csr->nslice = csr->sell_nnz = 0;
    fx_forget(csr);
}

extern "C" {

const char *pyci_gpu_last_error(void) { return g_error; }

const char *pyci_gpu_version(void) { return "pyci_gb300 0.1.0 (sm_103a)"; }

int64_t pyci_gpu_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int pyci_gpu_ctx_create(int device, pyci_gpu_ctx **out) {
    if (!out) {
        set_error("out is NULL");
        return PYCI_GPU_EINVAL;
    }
    int count = 0;
    PYCI_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) {
        set_error("device %d not present (%d devices)", device, count);
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    PYCI_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) {
        set_error("device %d (%s, sm_%d%d) is not a Blackwell GPU", device, prop.name, prop.major, prop.minor);
        return PYCI_GPU_EUNSUPPORTED;
    }
    pyci_gpu_ctx *ctx = new (std::nothrow) pyci_gpu_ctx();
    if (!ctx) {
        set_error("out of host memory");
        return PYCI_GPU_ENOMEM;
    }
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return cuda_status(e, "cudaStreamCreate");
    }
    // Keep memory released by cudaFreeAsync in the device's stream-ordered
    // pool rather than handing it back to the driver at every
    // synchronisation: each solve allocates and frees gigabytes of workspace,
    // and re-mapping it cost more than the solve's own kernels on large
    // operators.  pyci_gpu_ctx_destroy trims the pool.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    // Pinned staging for the solvers' coefficient uploads: 16 slots of 512 KB.
    ctx->ring = new (std::nothrow) PinnedRing();
    if (!ctx->ring || ctx->ring->init(16, 512 * 1024) != PYCI_GPU_OK) {
        delete ctx->ring;
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return PYCI_GPU_ENOMEM;
    }
    *out = ctx;
    return PYCI_GPU_OK;
}

int pyci_gpu_ctx_destroy(pyci_gpu_ctx *ctx) {
    if (!ctx)
        return PYCI_GPU_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete ctx->ring;
    if (ctx->mapped_host)
        cudaFreeHost(ctx->mapped_host);
    cudaStreamDestroy(ctx->stream);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess)
        cudaMemPoolTrimTo(pool, 0);
    delete ctx;
    return PYCI_GPU_OK;
}

void *pyci_gpu_ctx_stream(pyci_gpu_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

static int validate_wfn(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn) {
    // Wfn::init (pyci/src/wfn.cpp:51-57) and the subclass checks.
    if (kind != PYCI_WFN_DOCI && kind != PYCI_WFN_FULLCI && kind != PYCI_WFN_GENCI) {
        set_error("unknown wave function kind %d", kind);
        return PYCI_GPU_EINVAL;
    }
    if (nocc_dn < 0) {
        set_error("nocc_dn is < 0");
        return PYCI_GPU_EINVAL;
    }
    if (nocc_up < nocc_dn) {
        set_error("nocc_up is < nocc_dn");
        return PYCI_GPU_EINVAL;
    }
    if (nbasis < nocc_up) {
        set_error("nbasis is < nocc_up");
        return PYCI_GPU_EINVAL;
    }
    if (kind == PYCI_WFN_DOCI && nocc_up != nocc_dn) {
        set_error("nocc_up != nocc_dn");
        return PYCI_GPU_EINVAL;
    }
    if (kind == PYCI_WFN_GENCI && nocc_dn != 0) {
        set_error("nocc_dn != 0");
        return PYCI_GPU_EINVAL;
    }
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_build(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                       int64_t nocc_dn, int64_t ndet, const uint64_t *dets, int64_t nrow,
                       int64_t ncol, int symmetric, const double *one_mo, const double *two_mo,
                       int flags, pyci_gpu_csr **out) {
    if (!ctx || !out || !one_mo || !two_mo) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    if (ndet < 0) {
        set_error("ndet < 0");
        return PYCI_GPU_EINVAL;
    }
    if (nrow < 0)
        nrow = ndet;
    if (ncol < 0)
        ncol = ndet;
    if (nrow > ndet) {
        set_error("nrow (%lld) exceeds the number of determinants (%lld)", (long long)nrow, (long long)ndet);
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    pyci_gpu_csr *csr = new (std::nothrow) pyci_gpu_csr();
    if (!csr) {
        set_error("out of host memory");
        return PYCI_GPU_ENOMEM;
    }
    csr->ctx = ctx;
    csr->kind = kind;
    csr->flags = flags;
    csr->nbasis = nbasis;
    csr->nocc_up = nocc_up;
    csr->nocc_dn = nocc_dn;
    csr->ndet = ndet;
    csr->nrow = nrow;
    csr->ncol = ncol;
    csr->symmetric = symmetric != 0;
    rc = csr_build_device(ctx, csr, dets, one_mo, two_mo, 0, 0);
    if (rc) {
        csr_release(csr);
        delete csr;
        return rc;
    }
    const double avg = nrow ? static_cast<double>(csr->nnz) / nrow : 0.0;
    csr->spmm_lanes = avg >= 96 ? 32 : (avg >= 24 ? 16 : 8);
    *out = csr;
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_update(pyci_gpu_csr *csr, int64_t ndet, const uint64_t *dets,
                        const double *one_mo, const double *two_mo, int flags) {
    if (!csr || !one_mo || !two_mo) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (ndet < csr->nrow) {
        set_error("the wave function has fewer determinants than the operator has rows");
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    pyci_gpu_csr next = *csr;
    next.rowptr = nullptr;
    next.cols = nullptr;
    next.vals = nullptr;
    next.hi = next.lo = nullptr;
    next.lower_len = nullptr;
    next.ref_rowptr = nullptr;
    next.diag = nullptr;
    next.sell_off = nullptr;
    next.sell_cols = nullptr;
    next.sell_vals = nullptr;
    next.sell_lo = nullptr;
    next.nslice = next.sell_nnz = 0;
    fx_forget(&next);
    next.deferred = nullptr; // the old handle's, freed with it
    next.flags = flags;
    next.ndet = ndet;
    next.nrow = ndet;
    next.ncol = ndet;
    // Rows built before keep their old column range (pyci/src/sparseop.cpp:175-178).
    int rc = csr_build_device(csr->ctx, &next, dets, one_mo, two_mo, csr->nrow, csr->ncol);
    if (rc) {
        csr_release(&next);
        return rc;
    }
    csr_release(csr);
    const double avg = next.nrow ? static_cast<double>(next.nnz) / next.nrow : 0.0;
    next.spmm_lanes = avg >= 96 ? 32 : (avg >= 24 ? 16 : 8);
    for (auto &row : next.tuned)
        for (int &v : row)
            v = -1; // the matrix changed: tune again
    *csr = next;
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_free(pyci_gpu_csr *csr) {
    if (!csr)
        return PYCI_GPU_OK;
    cudaSetDevice(csr->ctx->device);
    csr_release(csr);
    delete csr;
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_clone(const pyci_gpu_csr *csr, pyci_gpu_csr **out) {
    if (!csr || !out) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    cudaStream_t st = csr->ctx->stream;
    // The copy gets the CSR entries: write a deferred CSR first.
    int rc0 = csr_materialize(csr);
    if (rc0)
        return rc0;
    pyci_gpu_csr *c = new (std::nothrow) pyci_gpu_csr(*csr);
    if (!c) {
        set_error("out of host memory");
        return PYCI_GPU_ENOMEM;
    }
    c->deferred = nullptr;
    c->rowptr = nullptr;
    c->cols = nullptr;
    c->vals = nullptr;
    c->hi = c->lo = nullptr;
    c->lower_len = nullptr;
    c->ref_rowptr = nullptr;
    c->diag = nullptr;
    c->sell_off = nullptr;
    c->sell_cols = nullptr;
    c->sell_vals = nullptr;
    c->sell_lo = nullptr;
    c->fx_atab = c->fx_bfull = c->fx_bsub = nullptr;
    c->fx_bq = nullptr;
    c->fx_hi = c->fx_lo = nullptr;
    c->dx_binom = nullptr;
    c->dx_v = nullptr;
    const int64_t fx_vals = csr->fx_nalpha * (csr->fx_nbp / 32) * csr->fx_npk * 128;
    struct Item {
        void *src;
        void **dst;
        size_t bytes;
    } items[] = {
        {csr->rowptr, reinterpret_cast<void **>(&c->rowptr), sizeof(int64_t) * (csr->nrow + 1)},
        {csr->cols, reinterpret_cast<void **>(&c->cols), sizeof(int32_t) * csr->nnz},
        {csr->vals, reinterpret_cast<void **>(&c->vals), sizeof(double) * csr->nnz},
        {csr->hi, reinterpret_cast<void **>(&c->hi), sizeof(float) * csr->nnz},
        {csr->lo, reinterpret_cast<void **>(&c->lo), sizeof(float) * csr->nnz},
        {csr->lower_len, reinterpret_cast<void **>(&c->lower_len), sizeof(int32_t) * csr->nrow},
        {csr->ref_rowptr, reinterpret_cast<void **>(&c->ref_rowptr), sizeof(int64_t) * (csr->nrow + 1)},
        {csr->diag, reinterpret_cast<void **>(&c->diag), sizeof(double) * csr->nrow},
        {csr->sell_off, reinterpret_cast<void **>(&c->sell_off), sizeof(int64_t) * (csr->nslice + 1)},
        {csr->sell_cols, reinterpret_cast<void **>(&c->sell_cols), sizeof(int32_t) * csr->sell_nnz},
        {csr->sell_vals, reinterpret_cast<void **>(&c->sell_vals), sizeof(float) * csr->sell_nnz},
        {csr->sell_lo, reinterpret_cast<void **>(&c->sell_lo), sizeof(float) * csr->sell_nnz},
        {csr->fx_atab, reinterpret_cast<void **>(&c->fx_atab), sizeof(int32_t) * csr->fx_nalpha * fx_atab_width(csr)},
        {csr->fx_bfull, reinterpret_cast<void **>(&c->fx_bfull), sizeof(int32_t) * csr->fx_nlb * csr->fx_nbeta},
        {csr->fx_bsub, reinterpret_cast<void **>(&c->fx_bsub), sizeof(int32_t) * csr->fx_nls * csr->fx_nbeta},
        {csr->fx_bq, reinterpret_cast<void **>(&c->fx_bq), sizeof(uint16_t) * csr->fx_la * csr->fx_nbeta},
        {csr->fx_hi, reinterpret_cast<void **>(&c->fx_hi), sizeof(float) * fx_vals},
        {csr->fx_lo, reinterpret_cast<void **>(&c->fx_lo), sizeof(float) * fx_vals},
        {csr->dx_binom, reinterpret_cast<void **>(&c->dx_binom), sizeof(int64_t) * (csr->dx_n + 1) * csr->dx_ldk},
        {csr->dx_v, reinterpret_cast<void **>(&c->dx_v), sizeof(float) * 2 * csr->dx_n * csr->dx_n},
    };
    for (auto &it : items) {
        if (!it.src)
            continue;
        cudaError_t e = cudaMallocAsync(it.dst, it.bytes ? it.bytes : 1, st);
        if (e == cudaSuccess && it.bytes)
            e = cudaMemcpyAsync(*it.dst, it.src, it.bytes, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            csr_release(c);
            delete c;
            return cuda_status(e, "clone");
        }
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        csr_release(c);
        delete c;
        return cuda_status(e, "clone");
    }
    *out = c;
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_storage(const pyci_gpu_csr *csr, int *flags) {
    if (!csr || !flags) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    *flags = (csr->vals ? PYCI_STORE_FP64 : 0) | (csr->hi && csr->lo ? PYCI_STORE_SPLIT : 0) |
             (csr->sell_cols ? PYCI_STORE_SELL : 0) | (has_implicit(csr) ? PYCI_STORE_IMPLICIT : 0) |
             (csr->deferred ? PYCI_STORE_DEFERRED : 0);
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_shape(const pyci_gpu_csr *csr, int64_t *nrow, int64_t *ncol, int64_t *size,
                       int64_t *nnz_stored) {
    if (!csr) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (nrow)
        *nrow = csr->nrow;
    if (ncol)
        *ncol = csr->ncol;
    if (size)
        *size = csr->nnz_ref;
    if (nnz_stored)
        *nnz_stored = csr->nnz;
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_export(const pyci_gpu_csr *csr, double *data, int64_t *indices, int64_t *indptr) {
    if (!csr) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    return csr_export_device(csr, data, indices, indptr);
}

int pyci_gpu_csr_get_element(const pyci_gpu_csr *csr, int64_t i, int64_t j, double *out) {
    if (!csr || !out) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (i < 0 || i >= csr->nrow) {
        set_error("row index %lld out of range", (long long)i);
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    cudaStream_t st = csr->ctx->stream;
    int rc0 = csr_materialize(csr);
    if (rc0)
        return rc0;
    int64_t ptr[2];
    int32_t len = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(ptr, csr->rowptr + i, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, st));
    if (csr->symmetric)
        PYCI_CUDA_TRY(cudaMemcpyAsync(&len, csr->lower_len + i, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    const int64_t n = csr->symmetric ? len : ptr[1] - ptr[0];
    *out = 0.0;
    if (n == 0)
        return PYCI_GPU_OK;
    std::vector<int32_t> cols(n);
    PYCI_CUDA_TRY(cudaMemcpyAsync(cols.data(), csr->cols + ptr[0], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    auto it = std::lower_bound(cols.begin(), cols.end(), j);
    if (it == cols.end() || *it != j)
        return PYCI_GPU_OK;
    const int64_t e = ptr[0] + (it - cols.begin());
    if (csr->vals) {
        PYCI_CUDA_TRY(cudaMemcpyAsync(out, csr->vals + e, sizeof(double), cudaMemcpyDeviceToHost, st));
    } else {
        float hl[2];
        PYCI_CUDA_TRY(cudaMemcpyAsync(&hl[0], csr->hi + e, sizeof(float), cudaMemcpyDeviceToHost, st));
        PYCI_CUDA_TRY(cudaMemcpyAsync(&hl[1], csr->lo + e, sizeof(float), cudaMemcpyDeviceToHost, st));
        PYCI_CUDA_TRY(cudaStreamSynchronize(st));
        *out = static_cast<double>(hl[0]) + static_cast<double>(hl[1]);
    }
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_matvec(const pyci_gpu_csr *csr, const double *x, double *y) {
    if (!csr || !x || !y) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (csr->symmetric && csr->ncol < csr->nrow) {
        set_error("symmetric operator with fewer columns than rows");
        return PYCI_GPU_ETYPE;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    cudaStream_t st = csr->ctx->stream;
    double *dx = nullptr, *dy = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&dx), sizeof(double) * std::max<int64_t>(csr->ncol, 1), st));
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&dy), sizeof(double) * std::max<int64_t>(csr->nrow, 1), st);
    if (e != cudaSuccess) {
        cudaFreeAsync(dx, st);
        return cuda_status(e, "cudaMallocAsync");
    }
    int rc = PYCI_GPU_OK;
    e = cudaMemcpyAsync(dx, x, sizeof(double) * csr->ncol, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rc = csr_spmm(csr, PYCI_PREC_FP64, 1, dx, dy, st);
        if (!rc)
            e = cudaMemcpyAsync(y, dy, sizeof(double) * csr->nrow, cudaMemcpyDeviceToHost, st);
    }
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFreeAsync(dx, st);
    cudaFreeAsync(dy, st);
    if (rc)
        return rc;
    if (e != cudaSuccess)
        return cuda_status(e, "matvec");
    if (e2 != cudaSuccess)
        return cuda_status(e2, "matvec");
    return PYCI_GPU_OK;
}

int pyci_gpu_csr_spmm_device(const pyci_gpu_csr *csr, int precision, int64_t k, const void *x,
                             void *y, void *stream) {
    if (!csr || !x || !y) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : csr->ctx->stream;
    if (precision == PYCI_PREC_FP64_DF)
        return csr_spmm_df(csr, static_cast<int>(k), static_cast<const float *>(x), static_cast<double *>(y), st);
    return csr_spmm(csr, precision, k, x, y, st);
}

int pyci_gpu_gram_device(pyci_gpu_ctx *ctx, int method, const float *A, int64_t p, const float *B, int64_t q,
                         int64_t N, double *C) {
    if (!ctx || !A || !B || !C) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (p < 0 || q < 0 || N < 0 || (method != PYCI_GRAM_CUDA_CORES && method != PYCI_GRAM_TENSOR_CORES)) {
        set_error("invalid Gram product arguments (p=%lld, q=%lld, N=%lld, method=%d)", static_cast<long long>(p),
                  static_cast<long long>(q), static_cast<long long>(N), method);
        return PYCI_GPU_EINVAL;
    }
    if (p == 0 || q == 0)
        return PYCI_GPU_OK;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    return pyci_gpu::gram_device(ctx, method, A, p, B, q, N, C);
}

int pyci_gpu_csr_prepare_mixed(pyci_gpu_csr *csr, int drop_fp64) {
    if (!csr) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    return csr_prepare_mixed_device(csr, drop_fp64);
}

int pyci_gpu_csr_solve(pyci_gpu_csr *csr, int64_t n, const double *c0, int64_t ncv,
                       int64_t maxiter, double tol, double ecore, int mode, double *evals,
                       double *evecs, pyci_gpu_solve_stats *stats) {
    if (!csr || !evals) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    // pyci/src/sparseop.cpp:116-125
    const int64_t nrow = csr->nrow;
    if ((nrow > 1 && n >= nrow) || (nrow == 1 && n > 1)) {
        set_error("cannot find >=n eigenpairs for sparse operator with n rows");
        return PYCI_GPU_EINVAL;
    }
    if (nrow != csr->ncol) {
        set_error("Can only solve sparse symmetric matrix operators");
        return PYCI_GPU_ETYPE;
    }
    if (!csr->symmetric) {
        set_error("Can only solve sparse symmetric matrix operators");
        return PYCI_GPU_ETYPE;
    }
    if (n < 1) {
        set_error("n must be >= 1");
        return PYCI_GPU_EINVAL;
    }
    if (mode != PYCI_SOLVE_FP64 && mode != PYCI_SOLVE_MIXED) {
        set_error("unknown solve mode %d", mode);
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    if (nrow == 1) {
        double h00 = 0.0;
        int rc = pyci_gpu_csr_get_element(csr, 0, 0, &h00);
        if (rc)
            return rc;
        evals[0] = h00 + ecore;
        if (evecs)
            evecs[0] = 1.0;
        if (stats)
            std::memset(stats, 0, sizeof(*stats));
        return PYCI_GPU_OK;
    }
    return davidson_solve(csr, n, c0, ncv, maxiter, tol, ecore, mode, evals, evecs, stats);
}

int pyci_gpu_csr_digest(const pyci_gpu_csr *csr, uint64_t *pattern_sum, uint64_t *pattern_xor,
                        double *value_sum, double *value_abs_sum, double *value_wsum) {
    if (!csr) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    return csr_digest_device(csr, pattern_sum, pattern_xor, value_sum, value_abs_sum, value_wsum);
}

int pyci_gpu_add_all_dets(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                          int64_t nocc_dn, uint64_t *dets) {
    if (!ctx || !dets) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    return add_all_dets_device(ctx, kind, nbasis, nocc_up, nocc_dn, dets);
}

int pyci_gpu_add_hci(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                     const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo,
                     double eps, int flags, int64_t max_new, uint64_t *out, int64_t *n_new) {
    if (!ctx || !n_new || !one_mo || !two_mo || (ndet > 0 && (!dets || !coeffs))) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (ndet < 0 || max_new < 0) {
        set_error("negative determinant count");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    return hci_select_device(ctx, kind, nbasis, nocc_up, nocc_dn, ndet, dets, coeffs, one_mo, two_mo, eps, flags,
                             max_new, out, n_new);
}

int pyci_gpu_compute_rdms(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                          int64_t ndet, const uint64_t *dets, const double *coeffs, double *rdm1, double *rdm2) {
    if (!ctx || !rdm1 || !rdm2 || (ndet > 0 && (!dets || !coeffs))) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (ndet < 0) {
        set_error("negative determinant count");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    return rdm_compute_device(ctx, kind, nbasis, ndet, dets, coeffs, 0, nullptr, nullptr, rdm1, rdm2);
}

int pyci_gpu_compute_transition_rdms(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                                     int64_t ndet1, const uint64_t *dets1, const double *coeffs1, int64_t ndet2,
                                     const uint64_t *dets2, const double *coeffs2, double *rdm1, double *rdm2) {
    if (!ctx || !rdm1 || !rdm2 || (ndet1 > 0 && (!dets1 || !coeffs1)) || (ndet2 > 0 && (!dets2 || !coeffs2))) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (ndet1 < 0 || ndet2 < 0) {
        set_error("negative determinant count");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    static const uint64_t empty = 0;
    return rdm_compute_device(ctx, kind, nbasis, ndet1, dets1, coeffs1, ndet2, dets2 ? dets2 : &empty, coeffs2, rdm1,
                              rdm2);
}

int pyci_gpu_compute_enpt2(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                           int64_t ndet, const uint64_t *dets, const double *coeffs, const double *one_mo,
                           const double *two_mo, double energy, double ecore, double eps, double *result) {
    if (!ctx || !result || !one_mo || !two_mo || (ndet > 0 && (!dets || !coeffs))) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (ndet < 0) {
        set_error("negative determinant count");
        return PYCI_GPU_EINVAL;
    }
    int rc = validate_wfn(kind, nbasis, nocc_up, nocc_dn);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaSetDevice(ctx->device));
    return enpt2_device(ctx, kind, nbasis, nocc_up, nocc_dn, ndet, dets, coeffs, one_mo, two_mo, energy, ecore, eps,
                        result);
}

} // extern "C"
