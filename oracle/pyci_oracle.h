/* CPU restatement of PyCI's CI hot path: determinant enumeration, the
 * Slater-Condon CSR build and the sparse matrix-vector products.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path
 * (tests, smoke check, and the timed CPU baseline); the product never links
 * or calls it.  Every function follows a reference routine, cited per
 * function in pyci_oracle.c.  Plain C11 + pthreads.
 */
#ifndef PYCI_ORACLE_H
#define PYCI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ORC_GENCI: Slater-Condon rules over the true virtual spin-orbitals.
 * ORC_GENCI_REF: the reference's GenCI row loop verbatim, including its
 * virtual-count quirk (see row_genci in pyci_oracle.c). */
enum { ORC_DOCI = 0, ORC_FULLCI = 1, ORC_GENCI = 2, ORC_GENCI_REF = 3 };

int64_t orc_binomial(int64_t n, int64_t k);
int64_t orc_nword(int64_t nbasis);
int64_t orc_rank_colex(int64_t nbasis, int64_t nocc, const uint64_t *det);
void orc_unrank_colex(int64_t nbasis, int64_t nocc, int64_t rank, int64_t *occs);
int orc_phase_single(const uint64_t *det, int64_t i, int64_t a);
int orc_phase_double(const uint64_t *det, int64_t i1, int64_t i2, int64_t a1, int64_t a2);

/* Number of determinants add_all_dets produces, or -1 on overflow. */
int64_t orc_ndet_all(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn);

/* Writes every determinant in the reference's add_all_dets order.  dets has
 * room for ndet * (nword for DOCI/GenCI, 2 * nword for FullCI) words. */
int orc_add_all_dets(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, uint64_t *dets);

/* Two-pass CSR build.  Pass 1 writes indptr[0..nrow] (row counts then the
 * prefix sum); pass 2 writes indices/data for the same rows.  Layout and
 * element order match the reference exactly (row-sorted columns; with
 * symmetric != 0, only columns < row plus the diagonal). */
int orc_csr_count(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                  const uint64_t *dets, int64_t nrow, int64_t ncol, int symmetric, int nthreads,
                  int64_t *indptr);
int orc_csr_fill(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                 const uint64_t *dets, int64_t nrow, int64_t ncol, int symmetric,
                 const double *one_mo, const double *two_mo, const double *h, const double *v,
                 const double *w, int nthreads, const int64_t *indptr, int64_t *indices,
                 double *data);

/* The same two passes for rows [row0, row1) only; indptr is local to the
 * range (row1 - row0 + 1 entries, indptr[0] = 0). */
int orc_csr_count_rows(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                       const uint64_t *dets, int64_t row0, int64_t row1, int64_t ncol, int symmetric,
                       int nthreads, int64_t *indptr);
int orc_csr_fill_rows(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                      const uint64_t *dets, int64_t row0, int64_t row1, int64_t ncol, int symmetric,
                      const double *one_mo, const double *two_mo, const double *h, const double *v,
                      const double *w, int nthreads, const int64_t *indptr, int64_t *indices,
                      double *data);

/* y = A x for a general CSR matrix. */
void orc_spmv_general(int64_t nrow, const int64_t *indptr, const int64_t *indices,
                      const double *data, const double *x, double *y, int nthreads);
/* y = (L + L^T - diag L) x for a lower-triangle CSR matrix L (nrow x nrow). */
void orc_spmv_sym_lower(int64_t nrow, const int64_t *indptr, const int64_t *indices,
                        const double *data, const double *x, double *y, int nthreads);

/* Heat-bath CI selection (add_hci): determinants not in dets[ndet] reached
 * from some determinant i by an excitation with |H_ji| > eps / |coeffs[i]|,
 * each once, in first-occurrence order.  Writes at most max_new of them to
 * out (out may be NULL) and their total count to *n_new.  kind ORC_GENCI_REF
 * follows the reference's GenCI loop (with its virtual-count quirk). */
int orc_add_hci(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                const double *coeffs, const double *one_mo, const double *two_mo, double eps, int64_t max_new,
                uint64_t *out, int64_t *n_new);

/* One- and two-particle RDMs of the wave function sum_i coeffs[i] |dets[i]>
 * (compute_rdms): DOCI rdm1 = d0 [n][n], rdm2 = d2 [n][n]; FullCI rdm1 =
 * [aa, bb] [2][n][n], rdm2 = [aaaa, bbbb, abab] [3][n][n][n][n].  Serial, in
 * the reference's summation order. */
int orc_compute_rdms(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                     const double *coeffs, double *rdm1, double *rdm2);
/* Transition RDMs <Psi_1| ... |Psi_2> (compute_transition_rdms), same layouts. */
int orc_compute_transition_rdms(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet1,
                                const uint64_t *dets1, const double *coeffs1, int64_t ndet2, const uint64_t *dets2,
                                const double *coeffs2, double *rdm1, double *rdm2);

/* Spin-orbital RDMs of a GenCI wave function from their definition:
 * rdm1[p][q] = <1| a+_p a_q |2>, rdm2[p][q][r][s] = <1| a+_p a+_q a_s a_r |2>
 * over nbasis spin orbitals (rdm1 n^2, rdm2 n^4); bra (dets1, c1), ket
 * (dets2, c2), the same wave function for compute_rdms. */
int orc_compute_rdms_genci(int64_t nbasis, int64_t ndet1, const uint64_t *dets1, const double *c1, int64_t ndet2,
                           const uint64_t *dets2, const double *c2, double *rdm1, double *rdm2);

/* Epstein-Nesbet second-order energy (compute_enpt2): energy + the sum over
 * determinants k outside the wave function of V_k^2 / (energy - ecore - H_kk),
 * V_k = sum of H_ki c_i over |H_ki| > eps / |c_i|.  DOCI through its FullCI
 * image.  Writes the energy to *result. */
int orc_compute_enpt2(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                      const double *coeffs, const double *one_mo, const double *two_mo, double energy, double ecore,
                      double eps, double *result);

#ifdef __cplusplus
}
#endif

#endif
