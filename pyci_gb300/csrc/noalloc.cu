// op(x) without any device allocation: pyci_gpu_csr_matvec_noalloc.
//
// pyci_gpu_csr_matvec stages x and y in device buffers it takes from the
// device's stream-ordered memory pool on every call.  Some callers cannot let
// a library allocate device memory while they run: a host application whose
// own allocator (an arena or pool it manages itself) has reserved the GPU's
// memory up front, so that an allocation made on its behalf fails or eats
// into memory the application has planned for; or a deployment that must
// know the library's whole device footprint before it starts.  This variant
// stages x and y in two file-scope device arrays instead, so a call allocates
// nothing; the operator's own arrays were allocated when it was built.  Like
// the allocating call it copies x from and y to host memory and waits for
// its stream before returning.
//
// Limits and sharing rules (also in include/pyci_gb300.h):
//   * nrow and ncol must each be <= PYCI_GPU_NOALLOC_MAX_ROWS (2^20): the
//     arrays hold 2 x 8 MiB, kept by every GPU that loads the library until
//     the process exits;
//   * every call on a device uses the same two arrays: calls that overlap on
//     the GPU (two host threads, two streams) race and may return each
//     other's results; serialise them;
//   * the first call on a device looks the arrays' device addresses up
//     (cudaGetSymbolAddress, once per device, with that device current); make
//     that first call before any stream capture begins;
//   * an operator whose CSR entries are deferred (built with the
//     implicit-column form and without PYCI_BUILD_EAGER_CSR) gets them on
//     its first FP64 product, so a first call on it allocates them.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"

namespace {

constexpr int64_t kNoAllocMaxRows = PYCI_GPU_NOALLOC_MAX_ROWS;
constexpr int kMaxDevices = 64;

// Device-side staging for x (ncol entries) and y (nrow entries).
static __device__ __align__(256) double g_noalloc_x[kNoAllocMaxRows];
static __device__ __align__(256) double g_noalloc_y[kNoAllocMaxRows];

std::mutex g_setup_mutex;
double *g_x_addr[kMaxDevices] = {};
double *g_y_addr[kMaxDevices] = {};

// Host code only sees stand-ins for g_noalloc_x/y: their device addresses
// must be looked up per device (with that device current).
int noalloc_addresses(int device, double **x, double **y) {
    if (device < 0 || device >= kMaxDevices) {
        set_error("device %d is beyond the %d devices the no-allocation path supports", device, kMaxDevices);
        return PYCI_GPU_EUNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_x_addr[device]) {
        void *px = nullptr, *py = nullptr;
        PYCI_CUDA_TRY(cudaGetSymbolAddress(&px, g_noalloc_x));
        PYCI_CUDA_TRY(cudaGetSymbolAddress(&py, g_noalloc_y));
        g_x_addr[device] = static_cast<double *>(px);
        g_y_addr[device] = static_cast<double *>(py);
    }
    *x = g_x_addr[device];
    *y = g_y_addr[device];
    return PYCI_GPU_OK;
}

} // namespace

extern "C" int pyci_gpu_csr_matvec_noalloc(const pyci_gpu_csr *csr, const double *x, double *y) {
    if (!csr || !x || !y) {
        set_error("NULL argument");
        return PYCI_GPU_EINVAL;
    }
    if (csr->nrow > kNoAllocMaxRows || csr->ncol > kNoAllocMaxRows) {
        set_error("pyci_gpu_csr_matvec_noalloc handles at most %lld rows and columns; this operator is "
                  "%lld x %lld (use pyci_gpu_csr_matvec)",
                  (long long)kNoAllocMaxRows, (long long)csr->nrow, (long long)csr->ncol);
        return PYCI_GPU_EINVAL;
    }
    if (csr->symmetric && csr->ncol < csr->nrow) {
        set_error("symmetric operator with fewer columns than rows");
        return PYCI_GPU_ETYPE;
    }
    PYCI_CUDA_TRY(cudaSetDevice(csr->ctx->device));
    double *dx = nullptr, *dy = nullptr;
    int rc = noalloc_addresses(csr->ctx->device, &dx, &dy);
    if (rc)
        return rc;
    cudaStream_t st = csr->ctx->stream;
    // x is overwritten in full (ncol entries); every row of y is written by
    // the product (the lower-layout product zeroes y itself first).
    PYCI_CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * csr->ncol, cudaMemcpyHostToDevice, st));
    rc = csr_spmm(csr, PYCI_PREC_FP64, 1, dx, dy, st);
    if (rc)
        return rc;
    PYCI_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * csr->nrow, cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    return PYCI_GPU_OK;
}
