/* pyci_gb300 -- GB300 (sm_103a) implementation of PyCI's CI hot path behind a C ABI.
 *
 * The hot path is the sparse CI Hamiltonian operator of PyCI: the CSR build
 * (pyci::SparseOp constructors and update, pyci/src/sparseop.cpp:49-71,186-201,
 * 220-502), its matrix-vector product (perform_op / perform_op_symm,
 * pyci/src/sparseop.cpp:96-112) and the lowest-eigenpair solve (solve_ci,
 * pyci/src/sparseop.cpp:114-146).  In the reference these are methods of the
 * C++ class pyci::SparseOp (pyci/include/pyci.h:621-693) bound to Python as
 * `pyci.sparse_op` (pyci/src/binding.cpp:884-1088).  Every entry point below
 * takes plain pointers and sizes; all array arguments are HOST memory unless
 * the name says `_device`.  Calls on one handle must not overlap; calls are
 * synchronous (results are on the host on return), as in the reference.
 *
 * Status codes: 0 on success, negative on failure; pyci_gpu_last_error()
 * returns the message of the calling thread's last failure.  The codes map to
 * the exceptions the reference raises for the same condition:
 *   PYCI_GPU_EINVAL  -> ValueError   (std::invalid_argument, std::domain_error)
 *   PYCI_GPU_ETYPE   -> TypeError    (pybind11::type_error)
 *   PYCI_GPU_ENOCONV -> RuntimeError ("did not converge")
 *   PYCI_GPU_ECUDA, PYCI_GPU_ENOMEM, PYCI_GPU_EUNSUPPORTED -> RuntimeError
 */
#ifndef PYCI_GB300_H
#define PYCI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYCI_GPU_OK 0
#define PYCI_GPU_EINVAL (-1)
#define PYCI_GPU_ETYPE (-2)
#define PYCI_GPU_ENOCONV (-3)
#define PYCI_GPU_ECUDA (-4)
#define PYCI_GPU_ENOMEM (-5)
#define PYCI_GPU_EUNSUPPORTED (-6)

/* Wave-function kinds (pyci/include/pyci.h:520-617). */
#define PYCI_WFN_DOCI 0   /* DOCIWfn: one spin string of nbasis spatial orbitals (pairs)  */
#define PYCI_WFN_FULLCI 1 /* FullCIWfn: alpha string then beta string, nword words each    */
#define PYCI_WFN_GENCI 2  /* GenCIWfn: one string of nbasis spin-orbitals                  */

/* Build flags. */
#define PYCI_BUILD_FULL_COLEX 0x1   /* dets are exactly add_all_dets' list; dets may be NULL */
#define PYCI_BUILD_GENCI_EXACT 0x2  /* GenCI: Slater-Condon rules over the true virtuals
                                       instead of the reference's virtual-count quirk       */
#define PYCI_BUILD_FORCE_HASH 0x4   /* look columns up in the hash table even for full spaces */
#define PYCI_BUILD_EAGER_CSR 0x8    /* write the CSR entries during the build even when the operator
                                       has the implicit-column form (by default they are written on
                                       first use: export, get_element, FP64 products, update) */

/* Solve modes. */
#define PYCI_SOLVE_FP64 0  /* FP64 CSR values, FP64 vectors, FP64 SpMM                      */
#define PYCI_SOLVE_MIXED 1 /* FP32 values/vectors/SpMM with FP64 Rayleigh-Ritz,
                              re-orthogonalisation and FP64 residual refinement           */

/* Precisions of pyci_gpu_csr_spmm_device. */
#define PYCI_PREC_FP64 0       /* values f64, x/y f64                                      */
#define PYCI_PREC_FP32 1       /* values f32 (high part), x/y f32                          */
#define PYCI_PREC_FP64_SPLIT 2 /* values f32 high + f32 low summed in f64, x/y f64         */
#define PYCI_PREC_FP64_DF 3    /* values f32 high + low, x split the same way, FP32
                                  arithmetic with double-float sums (~2^-44 relative):
                                  x f32[ncol][2k] (each row's k high parts, then its k
                                  low parts), y f64[nrow][k]; k = 1, 2 or 4            */

typedef struct pyci_gpu_ctx pyci_gpu_ctx;
typedef struct pyci_gpu_csr pyci_gpu_csr;

typedef struct pyci_gpu_solve_stats {
    int64_t iterations;   /* Davidson iterations                                  */
    int64_t matvecs;      /* vectors multiplied by H (all precisions)             */
    int64_t matvecs_fp64; /* of which in FP64 (refinement steps in mixed mode)    */
    int64_t restarts;
    int64_t refinements;
    double seconds;       /* wall time inside the solve                           */
    double seconds_spmm;  /* device time of the SpMM launches (CUDA events)       */
    double max_residual;  /* final max over roots of ||H x - theta x||, FP64      */
    int64_t host_syncs;   /* stream synchronisations (device -> host round trips) */
    double seconds_wait;  /* wall time the host spent blocked in them             */
} pyci_gpu_solve_stats;

/* Thread-local message of the last failure of the calling thread. */
const char *pyci_gpu_last_error(void);

/* Library version string. */
const char *pyci_gpu_version(void);

/* Number of CUDA kernels this library has launched since it was loaded
 * (diagnostic; no counterpart in the reference, which has no GPU code). */
int64_t pyci_gpu_kernel_launches(void);

/* Context: one CUDA device, one stream.  Replaces nothing in the reference
 * (which is host-only); every SparseOp of the reference maps to one csr
 * handle created on a context. */
int pyci_gpu_ctx_create(int device, pyci_gpu_ctx **out);
int pyci_gpu_ctx_destroy(pyci_gpu_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer (for device-pointer calls). */
void *pyci_gpu_ctx_stream(pyci_gpu_ctx *ctx);

/* Build the CI Hamiltonian in CSR form on the device.
 * Replaces SparseOp::SparseOp(ham, wfn, nrow, ncol, symmetric)
 * (pyci/src/sparseop.cpp:49-71) and the row loop it runs (update + add_row,
 * pyci/src/sparseop.cpp:186-201,220-502).
 *   kind      PYCI_WFN_*; nbasis/nocc_up/nocc_dn as in Wfn::init (pyci/src/wfn.cpp:51-70)
 *   ndet      number of determinants in the wave function
 *   dets      uint64[ndet][nwords], nwords = ceil(nbasis/64) (x2 for FULLCI), in the
 *             wave function's insertion order; may be NULL with PYCI_BUILD_FULL_COLEX
 *   nrow,ncol -1 means ndet (pyci/src/sparseop.cpp:51-52)
 *   one_mo    f64[nbasis][nbasis]; two_mo f64[nbasis]^4, physicist's notation
 *             (the arrays of pyci::SQuantOp, pyci/include/pyci.h:285-302)
 * The handle stores both triangles when symmetric (for a gather-only SpMV);
 * pyci_gpu_csr_export returns the reference's layout. */
int pyci_gpu_csr_build(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                       int64_t nocc_dn, int64_t ndet, const uint64_t *dets, int64_t nrow,
                       int64_t ncol, int symmetric, const double *one_mo, const double *two_mo,
                       int flags, pyci_gpu_csr **out);

/* Append rows [old nrow, ndet) for a grown wave function (new determinants at the end).
 * Replaces SparseOp::py_update (pyci/src/sparseop.cpp:175-178), which calls
 * update(ham, wfn, ndet, ndet, nrow).  Requires a symmetric operator. */
int pyci_gpu_csr_update(pyci_gpu_csr *csr, int64_t ndet, const uint64_t *dets,
                        const double *one_mo, const double *two_mo, int flags);

int pyci_gpu_csr_free(pyci_gpu_csr *csr);
/* Deep copy (SparseOp's copy constructor, pyci/src/sparseop.cpp:31-34). */
int pyci_gpu_csr_clone(const pyci_gpu_csr *csr, pyci_gpu_csr **out);

/* nrow, ncol, size (reference nnz: lower triangle + diagonal when symmetric)
 * and the number of entries stored on the device. */
int pyci_gpu_csr_shape(const pyci_gpu_csr *csr, int64_t *nrow, int64_t *ncol, int64_t *size,
                       int64_t *nnz_stored);

/* Copy the CSR arrays out in the reference's layout: data f64[size],
 * indices i64[size], indptr i64[nrow+1] (SparseOp::py_data/py_indices/py_indptr,
 * pyci/src/sparseop.cpp:504-514).  Any pointer may be NULL to skip it. */
int pyci_gpu_csr_export(const pyci_gpu_csr *csr, double *data, int64_t *indices, int64_t *indptr);

/* Element (i, j) of the reference's stored matrix, 0.0 when absent
 * (SparseOp::get_element, pyci/src/sparseop.cpp:89-94). */
int pyci_gpu_csr_get_element(const pyci_gpu_csr *csr, int64_t i, int64_t j, double *out);

/* y[nrow] = H x[ncol] in FP64, host buffers (SparseOp::perform_op,
 * pyci/src/sparseop.cpp:96-112; the symmetric operator applies L + L^T - D). */
int pyci_gpu_csr_matvec(const pyci_gpu_csr *csr, const double *x, double *y);

/* Largest nrow / ncol pyci_gpu_csr_matvec_noalloc accepts. */
#define PYCI_GPU_NOALLOC_MAX_ROWS (1 << 20)

/* y[nrow] = H x[ncol] in FP64 like pyci_gpu_csr_matvec, but without allocating
 * any device memory: x and y are staged in two fixed device arrays of
 * PYCI_GPU_NOALLOC_MAX_ROWS doubles each (16 MiB together) that the library
 * keeps on every GPU it is loaded on until the process exits.  No counterpart
 * in the reference (whose product runs on the host); it is for callers that
 * cannot let a library allocate device memory while they run -- a host whose
 * own allocator has reserved the GPU's memory, or one that must know the
 * library's device footprint in advance.  Returns PYCI_GPU_EINVAL when nrow
 * or ncol exceeds the maximum.  The first call on a device looks up the
 * arrays' device addresses (once per device); make it before any stream
 * capture.  All calls on a device share the arrays: calls that overlap on the
 * GPU race, so serialise them.  Synchronous, like pyci_gpu_csr_matvec.  An
 * operator built with its CSR entries deferred (PYCI_STORE_DEFERRED) gets
 * them on its first FP64 product, so a first call on it allocates them;
 * build with PYCI_BUILD_EAGER_CSR, or make one allocating call first. */
int pyci_gpu_csr_matvec_noalloc(const pyci_gpu_csr *csr, const double *x, double *y);

/* Y = H X on device buffers for k vectors stored interleaved ([ncol][k] and
 * [nrow][k], element (row, vector) at row*k + vector), on `stream` (a
 * cudaStream_t, or NULL for the context's stream).  precision PYCI_PREC_*;
 * FP32, FP64_SPLIT and FP64_DF need pyci_gpu_csr_prepare_mixed first
 * (FP64_DF uses its own operand layout, above).  Asynchronous.
 * The device form of perform_op, used by the eigensolver and benchmarks. */
int pyci_gpu_csr_spmm_device(const pyci_gpu_csr *csr, int precision, int64_t k, const void *x,
                             void *y, void *stream);

/* Gram product C = A^T B of FP32 vector blocks on the device, as the mixed-
 * precision eigensolver forms it: A holds p vectors and B q vectors of N rows,
 * vector-major (element (i, r) at i*N + r); C is f64[p][q] on the host.
 * method PYCI_GRAM_CUDA_CORES: FP32 FMAs; PYCI_GRAM_TENSOR_CORES: tcgen05
 * TF32 MMAs on high/low split operands (~2^-22 relative per product).  Partial
 * sums are added in FP64.  Synchronous.  No counterpart in the reference
 * (Spectra orthogonalises its Lanczos basis on the host); exposed so the two
 * device paths can be checked against each other. */
#define PYCI_GRAM_CUDA_CORES 0
#define PYCI_GRAM_TENSOR_CORES 1
int pyci_gpu_gram_device(pyci_gpu_ctx *ctx, int method, const float *A, int64_t p, const float *B, int64_t q,
                         int64_t N, double *C);

/* Derive the FP32 high/low value split used by the mixed-precision solve.
 * With drop_fp64 != 0 the FP64 values are freed afterwards (FP64 products then
 * use high + low, which reproduces every FP64 value to within 2^-48 relative). */
int pyci_gpu_csr_prepare_mixed(pyci_gpu_csr *csr, int drop_fp64);

/* Lowest n eigenpairs of the symmetric operator plus ecore
 * (SparseOp::solve_ci / py_solve_ci, pyci/src/sparseop.cpp:114-173).
 *   c0       optional f64[nrow] initial guess (NULL for the default guess)
 *   ncv      maximum subspace dimension (-1: default)
 *   maxiter  maximum iterations (-1: default)
 *   tol      convergence: ||H x - theta x|| <= tol * max(eps^(2/3), |theta|) per root
 *   evals    f64[n]; evecs f64[n][nrow] (eigenvector per row), or NULL to keep
 *            the eigenvectors on the device only
 * Eigenpairs are returned in decreasing order of eigenvalue, as the reference
 * returns them.  Errors: EINVAL when n >= nrow (nrow > 1), ETYPE when
 * nrow != ncol or the operator is not symmetric, ENOCONV on no convergence. */
int pyci_gpu_csr_solve(pyci_gpu_csr *csr, int64_t n, const double *c0, int64_t ncv,
                       int64_t maxiter, double tol, double ecore, int mode, double *evals,
                       double *evecs, pyci_gpu_solve_stats *stats);

/* Lowest 4 eigenpairs of each of nprob independent operators (square,
 * symmetric, built on ctx), solved together: all problems advance through one
 * block-Davidson iteration, with one SpMM launch per iteration for every
 * still-unconverged problem (replayed from a captured CUDA graph), segmented
 * Gram products, and per-problem subspace sizes, Rayleigh-Ritz and restarts.
 * No counterpart in the reference, which solves one operator at a time
 * (SparseOp::solve_ci, pyci/src/sparseop.cpp:114-146); the convergence test is
 * the one of pyci_gpu_csr_solve.  n must be 4.
 *   evals       f64[nprob][4], each problem's in decreasing order with ecore[p] added
 *   evecs       NULL, or nprob host pointers (each NULL or f64[4][nrow_p]):
 *               eigenvectors in the order of evals
 *   iterations  NULL or int64[nprob]: the iteration at which each problem converged
 * MIXED mode splits every operator's values (pyci_gpu_csr_prepare_mixed) and
 * finishes each problem with an FP64 Rayleigh-Ritz step; stats->max_residual
 * is the largest FP64 residual norm over all problems' eigenpairs. */
int pyci_gpu_batch_solve(pyci_gpu_ctx *ctx, int64_t nprob, pyci_gpu_csr *const *ops, int64_t n,
                         int64_t maxiter, double tol, const double *ecore, int mode, double *evals,
                         double *const *evecs, int64_t *iterations, pyci_gpu_solve_stats *stats);

/* Storage forms an operator holds on the device (bit flags, diagnostic; no
 * counterpart in the reference, whose operator is one host CSR):
 * PYCI_STORE_FP64 FP64 CSR values, PYCI_STORE_SPLIT the exact FP32 high/low
 * split in CSR order, PYCI_STORE_SELL the SELL-32 copy of the split,
 * PYCI_STORE_IMPLICIT the implicit-column form of a full FullCI space
 * (columns derived from per-string tables, values only), PYCI_STORE_DEFERRED
 * the CSR entries not written yet (they are written on first use). */
#define PYCI_STORE_FP64 0x1
#define PYCI_STORE_SPLIT 0x2
#define PYCI_STORE_SELL 0x4
#define PYCI_STORE_IMPLICIT 0x8
#define PYCI_STORE_DEFERRED 0x10
int pyci_gpu_csr_storage(const pyci_gpu_csr *csr, int *flags);

/* Kernel form the autotuner chose for the products of `precision` at width k
 * (diagnostic for benchmarks; no counterpart in the reference):
 * PYCI_FORM_CSR, PYCI_FORM_SELL, PYCI_FORM_IMPLICIT, or PYCI_FORM_UNTUNED
 * before the operator's first such product. */
#define PYCI_FORM_UNTUNED (-1)
#define PYCI_FORM_CSR 0
#define PYCI_FORM_SELL 1
#define PYCI_FORM_IMPLICIT 2
int pyci_gpu_csr_product_form(const pyci_gpu_csr *csr, int precision, int64_t k, int *form);

/* Order-independent digest of the reference-layout CSR, for checking
 * full-size builds against a digest computed from the reference's arrays:
 *   pattern_sum = sum over stored (i, j) of mix64(i * 2^32 + j)  (mod 2^64)
 *   pattern_xor = xor of the same terms
 *   value_sum   = sum of data, value_abs_sum = sum of |data|, value_wsum =
 *   sum of data * (1 + ((i * 31 + j * 17) mod 1024) / 1024)   (FP64)
 * where mix64 is the splitmix64 finaliser. */
int pyci_gpu_csr_digest(const pyci_gpu_csr *csr, uint64_t *pattern_sum, uint64_t *pattern_xor,
                        double *value_sum, double *value_abs_sum, double *value_wsum);

/* Generate add_all_dets' determinant list on the device (colex unranking)
 * and copy it to `dets` (uint64[ndet][nwords]).  Replaces
 * OneSpinWfn::add_all_dets / TwoSpinWfn::add_all_dets
 * (pyci/src/onespinwfn.cpp:173-217, pyci/src/twospinwfn.cpp:181-245). */
int pyci_gpu_add_all_dets(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up,
                          int64_t nocc_dn, uint64_t *dets);

/* One heat-bath CI selection step (add_hci, pyci/src/hci.cpp:240-262): the
 * determinants not among dets[ndet] that some determinant i reaches by a
 * single or double excitation with |H_ji| > eps / |coeffs[i]|, each once, in
 * first-occurrence order (i ascending, then the reference's excitation
 * order; the reference's own order follows its hash maps, its set is the
 * same).  dets in the wave function's layout (uint64[ndet][nwords],
 * nwords = ceil(nbasis / 64), doubled for FullCI); coeffs f64[ndet]; one_mo,
 * two_mo as for pyci_gpu_csr_build.  flags: PYCI_BUILD_GENCI_EXACT (GenCI
 * over the true virtual spin-orbitals; by default the reference's GenCI loop
 * with its virtual-count quirk).  *n_new receives the number of new
 * determinants; they are written to out only when out != NULL and
 * *n_new <= max_new (otherwise call again with room for *n_new).  The caller
 * appends them to its wave function. */
int pyci_gpu_add_hci(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                     const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo,
                     double eps, int flags, int64_t max_new, uint64_t *out, int64_t *n_new);

/* Epstein-Nesbet second-order energy (compute_enpt2, pyci/src/enpt2.cpp:332-375;
 * binding pyci/src/binding.cpp:1344-1375): energy + sum over determinants k
 * outside the wave function of V_k^2 / (energy - ecore - H_kk), where V_k sums
 * H_ki coeffs[i] over the excitations with |H_ki| > eps / |coeffs[i]| (the
 * selection of add_hci).  DOCI runs through its FullCI image, as the
 * reference does; GenCI is EUNSUPPORTED.  V_k is summed with FP64 atomics (the
 * reference sums in loop order), so results agree to rounding.  Writes the
 * energy to *result. */
int pyci_gpu_compute_enpt2(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                           int64_t ndet, const uint64_t *dets, const double *coeffs, const double *one_mo,
                           const double *two_mo, double energy, double ecore, double eps, double *result);

/* One- and two-particle reduced density matrices of sum_i coeffs[i] |dets[i]>
 * (compute_rdms, pyci/src/rdm.cpp:20-66 for DOCI, 269-530 for FullCI; binding
 * pyci/src/binding.cpp:1208-1291).  dets in the wave function's layout
 * (host), coeffs f64[ndet].  DOCI: rdm1 = d0 f64[n][n], rdm2 = d2 f64[n][n];
 * FullCI: rdm1 = [aa, bb] f64[2][n][n], rdm2 = [aaaa, bbbb, abab]
 * f64[3][n][n][n][n] (host).  Same terms as the reference, summed with FP64
 * atomics (entries agree to rounding).  GenCI: the spin-orbital RDMs from
 * their definition, rdm1[p][q] = <a+_p a_q> f64[n][n] and rdm2[p][q][r][s] =
 * <a+_p a+_q a_s a_r> f64[n][n][n][n] (the reference's GenCI compute_rdms,
 * pyci/src/rdm.cpp:532-632, writes past its output arrays, so its result is
 * undefined and is not reproduced). */
int pyci_gpu_compute_rdms(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                          int64_t ndet, const uint64_t *dets, const double *coeffs, double *rdm1, double *rdm2);

/* Transition RDMs between sum_i coeffs1[i] |dets1[i]> and sum_j coeffs2[j]
 * |dets2[j]> (compute_transition_rdms, pyci/src/rdm.cpp:634-902; binding
 * pyci/src/binding.cpp:1293-1340): same layouts as pyci_gpu_compute_rdms;
 * the reference's terms (each excitation of a determinant of 1 found in 2,
 * without the transposed partners), summed with FP64 atomics.  GenCI: the
 * definition-based spin-orbital forms above, <1| ... |2> with wave function 1
 * as the bra. */
int pyci_gpu_compute_transition_rdms(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                                     int64_t ndet1, const uint64_t *dets1, const double *coeffs1, int64_t ndet2,
                                     const uint64_t *dets2, const double *coeffs2, double *rdm1, double *rdm2);

#ifdef __cplusplus
}
#endif

#endif
