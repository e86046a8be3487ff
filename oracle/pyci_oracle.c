/* CPU restatement of PyCI's CI hot path (see pyci_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY -- the checker for the GPU path and the timed CPU
 * baseline.  Each routine restates the reference routine cited beside it
 * (paths relative to the PyCI source tree).  The determinant index is an
 * open-addressing table keyed on the determinant words; the reference keys a
 * hash map on a 128-bit SpookyHash of the same words
 * (pyci/src/onespinwfn.cpp:123-126), and both return the insertion index.
 *
 * Row-parallel with pthreads: the reference's sparse_op loop
 * (pyci/src/sparseop.cpp:186-201) is serial; rows are independent, so
 * splitting them over threads changes no result.
 */
#define _POSIX_C_SOURCE 200809L
#include "pyci_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define WORD_BITS 64

/* pyci/src/common.cpp:41-66 (binomial with overflow guard -> INT64_MAX). */
int64_t orc_binomial(int64_t n, int64_t k) {
    if (k < 0 || n < 0)
        return 0;
    if (k == 0)
        return 1;
    if (k == 1)
        return n;
    if (k >= n)
        return k == n;
    if (k > n / 2)
        k = n - k;
    __int128 b = 1;
    for (int64_t d = 1; d <= k; ++d) {
        b = b * (n - k + d) / d;
        if (b > INT64_MAX)
            return INT64_MAX;
    }
    return (int64_t)b;
}

/* pyci/src/common.cpp:280-282 */
int64_t orc_nword(int64_t nbasis) { return nbasis / WORD_BITS + ((nbasis % WORD_BITS) ? 1 : 0); }

/* pyci/src/common.cpp:85-97 */
static int64_t fill_occs(int64_t nword, const uint64_t *det, int64_t *occs) {
    int64_t j = 0;
    for (int64_t i = 0; i < nword; ++i) {
        uint64_t word = det[i];
        while (word) {
            int p = __builtin_ctzll(word);
            occs[j++] = p + i * WORD_BITS;
            word &= word - 1;
        }
    }
    return j;
}

/* pyci/src/common.cpp:99-113 */
static int64_t fill_virs(int64_t nword, int64_t nbasis, const uint64_t *det, int64_t *virs) {
    int64_t j = 0;
    for (int64_t i = 0; i < nword; ++i) {
        int64_t left = nbasis - i * WORD_BITS;
        uint64_t mask = (left < WORD_BITS) ? ((1ULL << left) - 1) : ~0ULL;
        uint64_t word = det[i] ^ mask;
        while (word) {
            int p = __builtin_ctzll(word);
            virs[j++] = p + i * WORD_BITS;
            word &= word - 1;
        }
    }
    return j;
}

/* pyci/src/common.cpp:124-137 (colex rank = sum over occupied p_k of C(p_k, k+1)). */
int64_t orc_rank_colex(int64_t nbasis, int64_t nocc, const uint64_t *det) {
    int64_t k = 0, rank = 0;
    for (int64_t i = 0; i < nbasis && k < nocc; ++i) {
        if (det[i / WORD_BITS] & (1ULL << (i % WORD_BITS))) {
            ++k;
            rank += orc_binomial(i, k);
        }
    }
    return rank;
}

/* pyci/src/common.cpp:139-153 */
void orc_unrank_colex(int64_t nbasis, int64_t nocc, int64_t rank, int64_t *occs) {
    for (int64_t i = 0; i < nocc; ++i) {
        int64_t j = nocc - i;
        int64_t binom = orc_binomial(nbasis, j);
        if (binom <= rank) {
            for (int64_t k = 0; k < j; ++k)
                occs[k] = k;
            break;
        }
        while (binom > rank)
            binom = orc_binomial(--nbasis, j);
        occs[j - 1] = nbasis;
        rank -= binom;
    }
}

/* pyci/src/common.cpp:155-161 */
static uint64_t mask_above(int64_t n) { return (n >= WORD_BITS - 1) ? 0ULL : ~((1ULL << (n + 1)) - 1); }
static uint64_t mask_below(int64_t m) { return (m >= WORD_BITS) ? ~0ULL : (1ULL << m) - 1; }

/* Number of occupied orbitals strictly between i and a. */
static int64_t perm_between(const uint64_t *det, int64_t i, int64_t a) {
    int64_t high = (i > a) ? i : a, low = (i > a) ? a : i;
    int64_t k = high / WORD_BITS, m = high % WORD_BITS, j = low / WORD_BITS, n = low % WORD_BITS;
    int64_t nperm = 0;
    if (j == k) {
        nperm += __builtin_popcountll(det[j] & mask_below(m) & mask_above(n));
    } else {
        nperm += __builtin_popcountll(det[j] & mask_above(n));
        nperm += __builtin_popcountll(det[k] & mask_below(m));
        for (int64_t l = j + 1; l < k; ++l)
            nperm += __builtin_popcountll(det[l]);
    }
    return nperm;
}

/* pyci/src/common.cpp:163-194 */
int orc_phase_single(const uint64_t *det, int64_t i, int64_t a) {
    return (perm_between(det, i, a) % 2) ? -1 : 1;
}

/* pyci/src/common.cpp:196-261 */
int orc_phase_double(const uint64_t *det, int64_t i1, int64_t i2, int64_t a1, int64_t a2) {
    int64_t nperm = perm_between(det, i1, a1) + perm_between(det, i2, a2);
    if ((i2 < a1) || (i1 > a2))
        ++nperm;
    return (nperm % 2) ? -1 : 1;
}

int64_t orc_ndet_all(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn) {
    int64_t a = orc_binomial(nbasis, nocc_up);
    if (kind != ORC_FULLCI)
        return (a == INT64_MAX) ? -1 : a;
    int64_t b = orc_binomial(nbasis, nocc_dn);
    if (a == INT64_MAX || b == INT64_MAX || (b && a > INT64_MAX / b))
        return -1;
    return a * b;
}

static void fill_det(int64_t nocc, const int64_t *occs, uint64_t *det) {
    for (int64_t i = 0; i < nocc; ++i)
        det[occs[i] / WORD_BITS] |= 1ULL << (occs[i] % WORD_BITS);
}

/* pyci/src/onespinwfn.cpp:173-217 and pyci/src/twospinwfn.cpp:181-245:
 * determinant r has colex rank r (one spin); for two spins, det r has
 * alpha rank r / C(n, nocc_dn) and beta rank r % C(n, nocc_dn). */
int orc_add_all_dets(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, uint64_t *dets) {
    int64_t nword = orc_nword(nbasis);
    int64_t occs[WORD_BITS * 64];
    if (nocc_up > (int64_t)(sizeof(occs) / sizeof(occs[0])))
        return -1;
    if (kind != ORC_FULLCI) {
        int64_t nd = orc_binomial(nbasis, nocc_up);
        memset(dets, 0, sizeof(uint64_t) * nword * nd);
        for (int64_t r = 0; r < nd; ++r) {
            orc_unrank_colex(nbasis, nocc_up, r, occs);
            fill_det(nocc_up, occs, dets + r * nword);
        }
        return 0;
    }
    int64_t na = orc_binomial(nbasis, nocc_up), nb = orc_binomial(nbasis, nocc_dn);
    int64_t nword2 = 2 * nword;
    memset(dets, 0, sizeof(uint64_t) * nword2 * na * nb);
    uint64_t *beta = calloc((size_t)(nb * nword), sizeof(uint64_t));
    if (!beta)
        return -1;
    for (int64_t r = 0; r < nb; ++r) {
        orc_unrank_colex(nbasis, nocc_dn, r, occs);
        fill_det(nocc_dn, occs, beta + r * nword);
    }
    uint64_t alpha[64];
    for (int64_t ra = 0; ra < na; ++ra) {
        memset(alpha, 0, sizeof(alpha));
        orc_unrank_colex(nbasis, nocc_up, ra, occs);
        fill_det(nocc_up, occs, alpha);
        for (int64_t rb = 0; rb < nb; ++rb) {
            uint64_t *d = dets + (ra * nb + rb) * nword2;
            memcpy(d, alpha, sizeof(uint64_t) * nword);
            memcpy(d + nword, beta + rb * nword, sizeof(uint64_t) * nword);
        }
    }
    free(beta);
    return 0;
}

/* ---------------- determinant -> index table ---------------- */

typedef struct {
    int64_t nwords, mask;
    int64_t *slots;
    const uint64_t *dets;
} det_index;

static uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

static uint64_t hash_det(const uint64_t *d, int64_t nwords) {
    uint64_t h = 0x84222325cbf29ce4ULL;
    for (int64_t i = 0; i < nwords; ++i)
        h = mix64(h ^ (d[i] + 0x9e3779b97f4a7c15ULL * (uint64_t)(i + 1)));
    return h;
}

static int index_build(det_index *ix, int64_t ndet, int64_t nwords, const uint64_t *dets) {
    int64_t cap = 16;
    while (cap < 2 * ndet)
        cap <<= 1;
    ix->nwords = nwords;
    ix->mask = cap - 1;
    ix->dets = dets;
    ix->slots = malloc(sizeof(int64_t) * cap);
    if (!ix->slots)
        return -1;
    for (int64_t i = 0; i < cap; ++i)
        ix->slots[i] = -1;
    for (int64_t i = 0; i < ndet; ++i) {
        int64_t s = (int64_t)(hash_det(dets + i * nwords, nwords) & (uint64_t)ix->mask);
        for (;;) {
            int64_t cur = ix->slots[s];
            if (cur < 0) {
                ix->slots[s] = i;
                break;
            }
            if (!memcmp(dets + cur * nwords, dets + i * nwords, sizeof(uint64_t) * nwords))
                break; /* duplicate: the first insertion keeps its index */
            s = (s + 1) & ix->mask;
        }
    }
    return 0;
}

static int64_t index_find(const det_index *ix, const uint64_t *d) {
    int64_t s = (int64_t)(hash_det(d, ix->nwords) & (uint64_t)ix->mask);
    for (;;) {
        int64_t cur = ix->slots[s];
        if (cur < 0)
            return -1;
        if (!memcmp(ix->dets + cur * ix->nwords, d, sizeof(uint64_t) * ix->nwords))
            return cur;
        s = (s + 1) & ix->mask;
    }
}

/* ---------------- Slater-Condon rows ---------------- */

typedef struct {
    int kind;
    int64_t nbasis, nocc_up, nocc_dn, ndet, nrow, ncol, nword;
    int symmetric;
    const uint64_t *dets;
    const double *one_mo, *two_mo, *h, *v, *w;
    const int64_t *indptr;
    int64_t *indices, *counts;
    double *data;
    det_index ix;
    int nthreads;
    int64_t row0; /* first row of the range [row0, nrow); counts/indptr are indexed from it */
} job;

typedef struct {
    int64_t n, cap;
    int64_t *col;
    double *val;
} rowbuf;

static void row_push(rowbuf *r, int64_t col, double val) {
    if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 1024;
        r->col = realloc(r->col, sizeof(int64_t) * r->cap);
        r->val = realloc(r->val, sizeof(double) * r->cap);
    }
    r->col[r->n] = col;
    r->val[r->n] = val;
    ++r->n;
}

/* Keeps a candidate column when the reference does: found, below the
 * symmetric cut-off, and inside the column range (pyci/src/sparseop.cpp:243). */
static int keep(const job *jb, int64_t idet, int64_t jdet) {
    int64_t jmin = jb->symmetric ? idet : INT64_MAX;
    return (jdet != -1) && (jdet < jmin) && (jdet < jb->ncol);
}

#define TWO(i, k, j, l) two[(i) * n3 + (k) * n2 + (j) * n1 + (l)]

/* pyci/src/sparseop.cpp:220-258 */
static void row_doci(const job *jb, int64_t idet, rowbuf *rb, int values) {
    const int64_t nw = jb->nword, n = jb->nbasis;
    uint64_t det[64];
    int64_t occs[256], virs[4096];
    memcpy(det, jb->dets + idet * nw, sizeof(uint64_t) * nw);
    int64_t no = fill_occs(nw, det, occs), nv = fill_virs(nw, n, det, virs);
    double val1 = 0.0, val2 = 0.0;
    for (int64_t i = 0; i < no; ++i) {
        int64_t k = occs[i];
        if (values) {
            val1 += jb->v[k * (n + 1)];
            val2 += jb->h[k];
            for (int64_t j = i + 1; j < no; ++j)
                val2 += jb->w[k * n + occs[j]];
        }
        for (int64_t j = 0; j < nv; ++j) {
            int64_t l = virs[j];
            det[k / WORD_BITS] &= ~(1ULL << (k % WORD_BITS));
            det[l / WORD_BITS] |= 1ULL << (l % WORD_BITS);
            int64_t jdet = index_find(&jb->ix, det);
            if (keep(jb, idet, jdet))
                row_push(rb, jdet, values ? jb->v[k * n + l] : 0.0);
            det[l / WORD_BITS] &= ~(1ULL << (l % WORD_BITS));
            det[k / WORD_BITS] |= 1ULL << (k % WORD_BITS);
        }
    }
    if (idet < jb->ncol)
        row_push(rb, idet, val1 + val2 * 2);
}

static inline void excite(uint64_t *d, int64_t i, int64_t a) {
    d[i / WORD_BITS] &= ~(1ULL << (i % WORD_BITS));
    d[a / WORD_BITS] |= 1ULL << (a % WORD_BITS);
}

/* pyci/src/sparseop.cpp:260-427 */
static void row_fullci(const job *jb, int64_t idet, rowbuf *rb, int values) {
    const int64_t nw = jb->nword, n1 = jb->nbasis, n2 = n1 * n1, n3 = n1 * n2;
    const double *one = jb->one_mo, *two = jb->two_mo;
    const uint64_t *rup = jb->dets + idet * 2 * nw, *rdn = rup + nw;
    uint64_t det[128];
    uint64_t *dup = det, *ddn = det + nw;
    int64_t ou[256], od[256], vu[4096], vd[4096];
    memcpy(det, rup, sizeof(uint64_t) * 2 * nw);
    int64_t nou = fill_occs(nw, rup, ou), nod = fill_occs(nw, rdn, od);
    int64_t nvu = fill_virs(nw, n1, rup, vu), nvd = fill_virs(nw, n1, rdn, vd);
    double val1, val2 = 0.0;
    for (int64_t i = 0; i < nou; ++i) {
        int64_t ii = ou[i];
        if (values) {
            val2 += one[(n1 + 1) * ii];
            for (int64_t k = i + 1; k < nou; ++k) {
                int64_t kk = ou[k];
                val2 += TWO(ii, kk, ii, kk) - TWO(ii, kk, kk, ii);
            }
            for (int64_t k = 0; k < nod; ++k) {
                int64_t kk = od[k];
                val2 += TWO(ii, kk, ii, kk);
            }
        }
        for (int64_t j = 0; j < nvu; ++j) {
            int64_t jj = vu[j];
            excite(dup, ii, jj);
            int64_t jdet = index_find(&jb->ix, det);
            if (keep(jb, idet, jdet)) {
                double val = 0.0;
                if (values) {
                    int sign_up = orc_phase_single(rup, ii, jj);
                    val1 = one[n1 * ii + jj];
                    for (int64_t k = 0; k < nou; ++k) {
                        int64_t kk = ou[k];
                        val1 += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                    }
                    for (int64_t k = 0; k < nod; ++k) {
                        int64_t kk = od[k];
                        val1 += TWO(ii, kk, jj, kk);
                    }
                    val = sign_up * val1;
                }
                row_push(rb, jdet, val);
            }
            int sign_up = orc_phase_single(rup, ii, jj);
            for (int64_t k = 0; k < nod; ++k) {
                int64_t kk = od[k];
                for (int64_t l = 0; l < nvd; ++l) {
                    int64_t ll = vd[l];
                    excite(ddn, kk, ll);
                    jdet = index_find(&jb->ix, det);
                    if (keep(jb, idet, jdet))
                        row_push(rb, jdet,
                                 values ? sign_up * orc_phase_single(rdn, kk, ll) * TWO(ii, kk, jj, ll)
                                        : 0.0);
                    excite(ddn, ll, kk);
                }
            }
            for (int64_t k = i + 1; k < nou; ++k) {
                int64_t kk = ou[k];
                for (int64_t l = j + 1; l < nvu; ++l) {
                    int64_t ll = vu[l];
                    excite(dup, kk, ll);
                    jdet = index_find(&jb->ix, det);
                    if (keep(jb, idet, jdet))
                        row_push(rb, jdet,
                                 values ? orc_phase_double(rup, ii, kk, jj, ll) *
                                              (TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj))
                                        : 0.0);
                    excite(dup, ll, kk);
                }
            }
            excite(dup, jj, ii);
        }
    }
    for (int64_t i = 0; i < nod; ++i) {
        int64_t ii = od[i];
        if (values) {
            val2 += one[(n1 + 1) * ii];
            for (int64_t k = i + 1; k < nod; ++k) {
                int64_t kk = od[k];
                val2 += TWO(ii, kk, ii, kk) - TWO(ii, kk, kk, ii);
            }
        }
        for (int64_t j = 0; j < nvd; ++j) {
            int64_t jj = vd[j];
            excite(ddn, ii, jj);
            int64_t jdet = index_find(&jb->ix, det);
            if (keep(jb, idet, jdet)) {
                double val = 0.0;
                if (values) {
                    val1 = one[n1 * ii + jj];
                    for (int64_t k = 0; k < nou; ++k) {
                        int64_t kk = ou[k];
                        val1 += TWO(ii, kk, jj, kk);
                    }
                    for (int64_t k = 0; k < nod; ++k) {
                        int64_t kk = od[k];
                        val1 += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                    }
                    val = orc_phase_single(rdn, ii, jj) * val1;
                }
                row_push(rb, jdet, val);
            }
            for (int64_t k = i + 1; k < nod; ++k) {
                int64_t kk = od[k];
                for (int64_t l = j + 1; l < nvd; ++l) {
                    int64_t ll = vd[l];
                    excite(ddn, kk, ll);
                    jdet = index_find(&jb->ix, det);
                    if (keep(jb, idet, jdet))
                        row_push(rb, jdet,
                                 values ? orc_phase_double(rdn, ii, kk, jj, ll) *
                                              (TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj))
                                        : 0.0);
                    excite(ddn, ll, kk);
                }
            }
            excite(ddn, jj, ii);
        }
    }
    if (idet < jb->ncol)
        row_push(rb, idet, val2);
}

/* pyci/src/sparseop.cpp:429-502.
 *
 * With kind ORC_GENCI_REF the virtual loop runs to the reference's
 * wfn.nvir = 2 * nbasis - nocc (pyci/src/wfn.cpp:62), nbasis more entries than
 * there are virtual spin-orbitals; the extra entries of the reference's
 * zero-initialised virs buffer (pyci/src/sparseop.cpp:190) are orbital 0.
 * This reproduces the reference's GenCI matrix exactly, including the
 * duplicate entries and the lost orbital-0 electron that follow.  ORC_GENCI
 * loops over the true virtual spin-orbitals only (the Slater-Condon rules). */
static void row_genci(const job *jb, int64_t idet, rowbuf *rb, int values) {
    const int64_t nw = jb->nword, n1 = jb->nbasis, n2 = n1 * n1, n3 = n1 * n2;
    const double *one = jb->one_mo, *two = jb->two_mo;
    const uint64_t *rdet = jb->dets + idet * nw;
    uint64_t det[64];
    int64_t occs[512], virs[8192];
    memcpy(det, rdet, sizeof(uint64_t) * nw);
    int64_t no = fill_occs(nw, rdet, occs), nv = fill_virs(nw, n1, rdet, virs);
    if (jb->kind == ORC_GENCI_REF) {
        int64_t nv_ref = 2 * n1 - jb->nocc_up - jb->nocc_dn;
        for (int64_t j = nv; j < nv_ref; ++j)
            virs[j] = 0;
        nv = nv_ref;
    }
    double val1, val2 = 0.0;
    for (int64_t i = 0; i < no; ++i) {
        int64_t ii = occs[i];
        if (values) {
            val2 += one[(n1 + 1) * ii];
            for (int64_t k = i + 1; k < no; ++k) {
                int64_t kk = occs[k];
                val2 += TWO(ii, kk, ii, kk) - TWO(ii, kk, kk, ii);
            }
        }
        for (int64_t j = 0; j < nv; ++j) {
            int64_t jj = virs[j];
            excite(det, ii, jj);
            int64_t jdet = index_find(&jb->ix, det);
            if (keep(jb, idet, jdet)) {
                double val = 0.0;
                if (values) {
                    val1 = one[n1 * ii + jj];
                    for (int64_t k = 0; k < no; ++k) {
                        int64_t kk = occs[k];
                        val1 += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                    }
                    val = orc_phase_single(rdet, ii, jj) * val1;
                }
                row_push(rb, jdet, val);
            }
            for (int64_t k = i + 1; k < no; ++k) {
                int64_t kk = occs[k];
                for (int64_t l = j + 1; l < nv; ++l) {
                    int64_t ll = virs[l];
                    excite(det, kk, ll);
                    jdet = index_find(&jb->ix, det);
                    if (keep(jb, idet, jdet))
                        row_push(rb, jdet,
                                 values ? orc_phase_double(rdet, ii, kk, jj, ll) *
                                              (TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj))
                                        : 0.0);
                    excite(det, ll, kk);
                }
            }
            excite(det, jj, ii);
        }
    }
    if (idet < jb->ncol)
        row_push(rb, idet, val2);
}

/* pyci/src/sparseop.cpp:214-218: sort (value, column) pairs by column. */
static void sort_row(rowbuf *rb) {
    for (int64_t a = 1; a < rb->n; ++a) {
        int64_t c = rb->col[a];
        double v = rb->val[a];
        int64_t b = a - 1;
        while (b >= 0 && rb->col[b] > c) {
            rb->col[b + 1] = rb->col[b];
            rb->val[b + 1] = rb->val[b];
            --b;
        }
        rb->col[b + 1] = c;
        rb->val[b + 1] = v;
    }
}

typedef struct {
    job *jb;
    int tid, values;
} worker_arg;

static void *worker(void *p) {
    worker_arg *wa = p;
    job *jb = wa->jb;
    rowbuf rb = {0, 0, NULL, NULL};
    const int64_t chunk = 64;
    for (int64_t start = jb->row0 + (int64_t)wa->tid * chunk; start < jb->nrow;
         start += (int64_t)jb->nthreads * chunk) {
        int64_t end = start + chunk < jb->nrow ? start + chunk : jb->nrow;
        for (int64_t idet = start; idet < end; ++idet) {
            rb.n = 0;
            if (jb->kind == ORC_DOCI)
                row_doci(jb, idet, &rb, wa->values);
            else if (jb->kind == ORC_FULLCI)
                row_fullci(jb, idet, &rb, wa->values);
            else
                row_genci(jb, idet, &rb, wa->values);
            if (!wa->values) {
                jb->counts[idet - jb->row0] = rb.n;
            } else {
                sort_row(&rb);
                int64_t off = jb->indptr[idet - jb->row0];
                memcpy(jb->indices + off, rb.col, sizeof(int64_t) * rb.n);
                memcpy(jb->data + off, rb.val, sizeof(double) * rb.n);
            }
        }
    }
    free(rb.col);
    free(rb.val);
    return NULL;
}

static int run(job *jb, int values) {
    int nt = jb->nthreads < 1 ? 1 : jb->nthreads;
    jb->nthreads = nt;
    pthread_t *th = malloc(sizeof(pthread_t) * nt);
    worker_arg *args = malloc(sizeof(worker_arg) * nt);
    if (!th || !args) {
        free(th);
        free(args);
        return -1;
    }
    for (int t = 0; t < nt; ++t) {
        args[t].jb = jb;
        args[t].tid = t;
        args[t].values = values;
        pthread_create(&th[t], NULL, worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(args);
    return 0;
}

static int job_init(job *jb, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn,
                    int64_t ndet, const uint64_t *dets, int64_t nrow, int64_t ncol, int symmetric,
                    int nthreads) {
    memset(jb, 0, sizeof(*jb));
    if (nrow > ndet || nrow < 0 || ncol < 0 || nbasis > 4096)
        return -1;
    jb->kind = kind;
    jb->nbasis = nbasis;
    jb->nocc_up = nocc_up;
    jb->nocc_dn = nocc_dn;
    jb->ndet = ndet;
    jb->nrow = nrow;
    jb->ncol = ncol;
    jb->symmetric = symmetric;
    jb->dets = dets;
    jb->nword = orc_nword(nbasis);
    jb->nthreads = nthreads;
    int64_t nwords = (kind == ORC_FULLCI) ? 2 * jb->nword : jb->nword;
    return index_build(&jb->ix, ndet, nwords, dets);
}

int orc_csr_count(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                  const uint64_t *dets, int64_t nrow, int64_t ncol, int symmetric, int nthreads,
                  int64_t *indptr) {
    job jb;
    if (job_init(&jb, kind, nbasis, nocc_up, nocc_dn, ndet, dets, nrow, ncol, symmetric, nthreads))
        return -1;
    jb.counts = indptr + 1;
    int rc = run(&jb, 0);
    free(jb.ix.slots);
    indptr[0] = 0;
    for (int64_t i = 0; i < nrow; ++i)
        indptr[i + 1] += indptr[i];
    return rc;
}

int orc_csr_fill(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                 const uint64_t *dets, int64_t nrow, int64_t ncol, int symmetric,
                 const double *one_mo, const double *two_mo, const double *h, const double *v,
                 const double *w, int nthreads, const int64_t *indptr, int64_t *indices,
                 double *data) {
    job jb;
    if (job_init(&jb, kind, nbasis, nocc_up, nocc_dn, ndet, dets, nrow, ncol, symmetric, nthreads))
        return -1;
    jb.one_mo = one_mo;
    jb.two_mo = two_mo;
    jb.h = h;
    jb.v = v;
    jb.w = w;
    jb.indptr = indptr;
    jb.indices = indices;
    jb.data = data;
    int rc = run(&jb, 1);
    free(jb.ix.slots);
    return rc;
}

/* Rows [row0, row1) of the same CSR: the count and fill passes of
 * orc_csr_count / orc_csr_fill restricted to a row range, with indptr local
 * to the range (indptr[0] = 0, row0 + r at indptr[r]).  The timed CPU
 * baseline builds one slice of a large operator per sample with these. */
int orc_csr_count_rows(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                       const uint64_t *dets, int64_t row0, int64_t row1, int64_t ncol, int symmetric,
                       int nthreads, int64_t *indptr) {
    job jb;
    if (row0 < 0 || row0 > row1 ||
        job_init(&jb, kind, nbasis, nocc_up, nocc_dn, ndet, dets, row1, ncol, symmetric, nthreads))
        return -1;
    jb.row0 = row0;
    jb.counts = indptr + 1;
    int rc = run(&jb, 0);
    free(jb.ix.slots);
    indptr[0] = 0;
    for (int64_t i = 0; i < row1 - row0; ++i)
        indptr[i + 1] += indptr[i];
    return rc;
}

int orc_csr_fill_rows(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                      const uint64_t *dets, int64_t row0, int64_t row1, int64_t ncol, int symmetric,
                      const double *one_mo, const double *two_mo, const double *h, const double *v,
                      const double *w, int nthreads, const int64_t *indptr, int64_t *indices,
                      double *data) {
    job jb;
    if (row0 < 0 || row0 > row1 ||
        job_init(&jb, kind, nbasis, nocc_up, nocc_dn, ndet, dets, row1, ncol, symmetric, nthreads))
        return -1;
    jb.row0 = row0;
    jb.one_mo = one_mo;
    jb.two_mo = two_mo;
    jb.h = h;
    jb.v = v;
    jb.w = w;
    jb.indptr = indptr;
    jb.indices = indices;
    jb.data = data;
    int rc = run(&jb, 1);
    free(jb.ix.slots);
    return rc;
}

/* ---------------- sparse matrix-vector products ---------------- */

typedef struct {
    int64_t nrow;
    const int64_t *indptr, *indices;
    const double *data, *x;
    double *y, *ybuf;
    int nthreads, tid, lower;
} spmv_arg;

static void *spmv_worker(void *p) {
    spmv_arg *a = p;
    int64_t per = (a->nrow + a->nthreads - 1) / a->nthreads;
    int64_t r0 = per * a->tid, r1 = r0 + per < a->nrow ? r0 + per : a->nrow;
    double *yt = a->lower ? a->ybuf + (int64_t)a->tid * a->nrow : NULL;
    if (yt)
        memset(yt, 0, sizeof(double) * a->nrow);
    for (int64_t i = r0; i < r1; ++i) {
        double s = 0.0;
        for (int64_t k = a->indptr[i]; k < a->indptr[i + 1]; ++k) {
            int64_t j = a->indices[k];
            s += a->data[k] * a->x[j];
            if (yt && j != i)
                yt[j] += a->data[k] * a->x[i];
        }
        a->y[i] = s;
    }
    return NULL;
}

static void spmv_run(int64_t nrow, const int64_t *indptr, const int64_t *indices,
                     const double *data, const double *x, double *y, int nthreads, int lower) {
    int nt = nthreads < 1 ? 1 : nthreads;
    if (nrow < nt)
        nt = 1;
    double *ybuf = lower ? malloc(sizeof(double) * nrow * nt) : NULL;
    pthread_t th[256];
    spmv_arg args[256];
    if (nt > 256)
        nt = 256;
    for (int t = 0; t < nt; ++t) {
        args[t] = (spmv_arg){nrow, indptr, indices, data, x, y, ybuf, nt, t, lower};
        pthread_create(&th[t], NULL, spmv_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    if (lower) {
        for (int t = 0; t < nt; ++t)
            for (int64_t i = 0; i < nrow; ++i)
                y[i] += ybuf[(int64_t)t * nrow + i];
        free(ybuf);
    }
}

/* Eigen row-major CSR times vector, as used by pyci/src/sparseop.cpp:96-104. */
void orc_spmv_general(int64_t nrow, const int64_t *indptr, const int64_t *indices,
                      const double *data, const double *x, double *y, int nthreads) {
    spmv_run(nrow, indptr, indices, data, x, y, nthreads, 0);
}

/* Eigen selfadjointView<Lower> product, pyci/src/sparseop.cpp:106-112. */
void orc_spmv_sym_lower(int64_t nrow, const int64_t *indptr, const int64_t *indices,
                        const double *data, const double *x, double *y, int nthreads) {
    spmv_run(nrow, indptr, indices, data, x, y, nthreads, 1);
}

/* ---------------- heat-bath CI determinant selection ---------------- */

typedef struct {
    int64_t n, cap, nwords;
    uint64_t *words;
} candbuf;

static int cand_push(candbuf *c, const uint64_t *d) {
    if (c->n == c->cap) {
        int64_t cap = c->cap ? 2 * c->cap : 1024;
        uint64_t *w = realloc(c->words, sizeof(uint64_t) * cap * c->nwords);
        if (!w)
            return -1;
        c->words = w;
        c->cap = cap;
    }
    memcpy(c->words + c->n * c->nwords, d, sizeof(uint64_t) * c->nwords);
    ++c->n;
    return 0;
}

/* A candidate joins when |value| > eps / |c_i| and it is not a determinant of
 * the wave function already (pyci/src/hci.cpp:37-41). */
static int hci_try(const det_index *ix, candbuf *c, const uint64_t *d, double val, double eps_i) {
    if (fabs(val) > eps_i && index_find(ix, d) == -1)
        return cand_push(c, d);
    return 0;
}

/* One determinant's candidates in the reference's loop order:
 * DOCI pyci/src/hci.cpp:21-46, FullCI 48-183, GenCI 185-238 (the GenCI
 * loop runs over 2 nbasis - nocc "virtuals", the true ones then orbital 0,
 * exactly as add_row<GenCIWfn> does; ORC_GENCI uses the true virtuals). */
static int hci_row(int kind, int64_t n1, int64_t nocc_up, int64_t nocc_dn, int64_t nword, const uint64_t *rdet,
                   const double *one, const double *two, double eps_i, const det_index *ix, candbuf *c) {
    const int64_t n2 = n1 * n1, n3 = n1 * n2;
    uint64_t det[128];
    int64_t occs[512], virs[8192];
    int rc = 0;
    if (kind == ORC_DOCI) {
        memcpy(det, rdet, sizeof(uint64_t) * nword);
        int64_t no = fill_occs(nword, rdet, occs), nv = fill_virs(nword, n1, rdet, virs);
        for (int64_t i = 0; i < no && !rc; ++i) {
            int64_t k = occs[i];
            for (int64_t j = 0; j < nv && !rc; ++j) {
                int64_t l = virs[j];
                double val = TWO(k, k, l, l); /* SQuantOp::v (pyci/src/squantop.cpp:177) */
                if (fabs(val) > eps_i) {
                    excite(det, k, l);
                    rc = hci_try(ix, c, det, val, eps_i);
                    excite(det, l, k);
                }
            }
        }
        return rc;
    }
    if (kind == ORC_FULLCI) {
        uint64_t *up = det, *dn = det + nword;
        memcpy(det, rdet, sizeof(uint64_t) * 2 * nword);
        int64_t ou[256], od[256], vu[256], vd[256];
        int64_t nou = fill_occs(nword, rdet, ou), nod = fill_occs(nword, rdet + nword, od);
        int64_t nvu = fill_virs(nword, n1, rdet, vu), nvd = fill_virs(nword, n1, rdet + nword, vd);
        for (int64_t i = 0; i < nou && !rc; ++i) {
            int64_t ii = ou[i];
            for (int64_t j = 0; j < nvu && !rc; ++j) {
                int64_t jj = vu[j];
                excite(up, ii, jj);
                double val = one[n1 * ii + jj];
                for (int64_t k = 0; k < nou; ++k) {
                    int64_t kk = ou[k];
                    val += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                }
                for (int64_t k = 0; k < nod; ++k) {
                    int64_t kk = od[k];
                    val += TWO(ii, kk, jj, kk);
                }
                rc = hci_try(ix, c, det, val, eps_i);
                for (int64_t k = 0; k < nod && !rc; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = 0; l < nvd && !rc; ++l) {
                        int64_t ll = vd[l];
                        val = TWO(ii, kk, jj, ll);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            rc = hci_try(ix, c, det, val, eps_i);
                            excite(dn, ll, kk);
                        }
                    }
                }
                for (int64_t k = i + 1; k < nou && !rc; ++k) {
                    int64_t kk = ou[k];
                    for (int64_t l = j + 1; l < nvu && !rc; ++l) {
                        int64_t ll = vu[l];
                        val = TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(up, kk, ll);
                            rc = hci_try(ix, c, det, val, eps_i);
                            excite(up, ll, kk);
                        }
                    }
                }
                excite(up, jj, ii);
            }
        }
        for (int64_t i = 0; i < nod && !rc; ++i) {
            int64_t ii = od[i];
            for (int64_t j = 0; j < nvd && !rc; ++j) {
                int64_t jj = vd[j];
                excite(dn, ii, jj);
                double val = one[n1 * ii + jj];
                for (int64_t k = 0; k < nou; ++k) {
                    int64_t kk = ou[k];
                    val += TWO(ii, kk, jj, kk);
                }
                for (int64_t k = 0; k < nod; ++k) {
                    int64_t kk = od[k];
                    val += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                }
                rc = hci_try(ix, c, det, val, eps_i);
                for (int64_t k = i + 1; k < nod && !rc; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = j + 1; l < nvd && !rc; ++l) {
                        int64_t ll = vd[l];
                        val = TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            rc = hci_try(ix, c, det, val, eps_i);
                            excite(dn, ll, kk);
                        }
                    }
                }
                excite(dn, jj, ii);
            }
        }
        return rc;
    }
    /* GenCI */
    memcpy(det, rdet, sizeof(uint64_t) * nword);
    int64_t no = fill_occs(nword, rdet, occs), nv = fill_virs(nword, n1, rdet, virs);
    if (kind == ORC_GENCI_REF) {
        int64_t nv_ref = 2 * n1 - nocc_up - nocc_dn;
        for (int64_t j = nv; j < nv_ref; ++j)
            virs[j] = 0;
        nv = nv_ref;
    }
    for (int64_t i = 0; i < no && !rc; ++i) {
        int64_t ii = occs[i];
        for (int64_t j = 0; j < nv && !rc; ++j) {
            int64_t jj = virs[j];
            excite(det, ii, jj);
            double val = one[n1 * ii + jj];
            for (int64_t k = 0; k < no; ++k) {
                int64_t kk = occs[k];
                val += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
            }
            rc = hci_try(ix, c, det, val, eps_i);
            for (int64_t k = i + 1; k < no && !rc; ++k) {
                int64_t kk = occs[k];
                for (int64_t l = j + 1; l < nv && !rc; ++l) {
                    int64_t ll = virs[l];
                    val = TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj);
                    if (fabs(val) > eps_i) {
                        excite(det, kk, ll);
                        rc = hci_try(ix, c, det, val, eps_i);
                        excite(det, ll, kk);
                    }
                }
            }
            excite(det, jj, ii);
        }
    }
    return rc;
}

/* add_hci (pyci/src/hci.cpp:240-262): every determinant not yet in the wave
 * function that some determinant i reaches by an excitation with
 * |H_ji| > eps / |c_i|.  Each new determinant is listed once, at its first
 * occurrence in the order (i ascending, the reference's loop order); the
 * reference merges its per-thread results by iterating hash maps, so its
 * order is that of its hash-map implementation while the set is the same. */
int orc_add_hci(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                const double *coeffs, const double *one_mo, const double *two_mo, double eps, int64_t max_new,
                uint64_t *out, int64_t *n_new) {
    const int64_t nword = orc_nword(nbasis);
    const int64_t nw = kind == ORC_FULLCI ? 2 * nword : nword;
    if (nword > 64 || (kind == ORC_FULLCI && nword > 4))
        return -2;
    det_index ix;
    if (index_build(&ix, ndet, nw, dets))
        return -1;
    candbuf c = {0, 0, nw, NULL};
    int rc = 0;
    for (int64_t i = 0; i < ndet && !rc; ++i) {
        const double eps_i = eps / fabs(coeffs[i]);
        rc = hci_row(kind, nbasis, nocc_up, nocc_dn, nword, dets + i * nw, one_mo, two_mo, eps_i, &ix, &c);
    }
    free(ix.slots);
    if (rc) {
        free(c.words);
        return -1;
    }
    /* First occurrence of each candidate: the table keeps the first index. */
    det_index cx;
    if (index_build(&cx, c.n, nw, c.words)) {
        free(c.words);
        return -1;
    }
    int64_t m = 0;
    for (int64_t i = 0; i < c.n; ++i) {
        if (index_find(&cx, c.words + i * nw) != i)
            continue;
        if (out && m < max_new)
            memcpy(out + m * nw, c.words + i * nw, sizeof(uint64_t) * nw);
        ++m;
    }
    *n_new = m;
    free(cx.slots);
    free(c.words);
    return 0;
}

/* ---------------- reduced density matrices ---------------- */

/* compute_rdms, pyci/src/rdm.cpp:20-66 (DOCI: rdm1 = d0, rdm2 = d2, both
 * nbasis x nbasis) and 269-530 (FullCI: rdm1 = [aa, bb] (2 n^2), rdm2 =
 * [aaaa, bbbb, abab] (3 n^4)); with tr, compute_transition_rdms
 * (pyci/src/rdm.cpp:634-902): determinants of wavefunction 1 against the
 * index of wavefunction 2, every excitation found in 2 (not only j > i), and
 * no transposed partner terms.  Serial, in the reference's loop and
 * summation order, so the sums are bit-identical to the reference's. */
static int rdms_core(int kind, int64_t nbasis, int64_t ndet, const uint64_t *dets, const double *coeffs,
                     int64_t ndet2, const uint64_t *dets2, const double *coeffs2, int tr, double *rdm1,
                     double *rdm2) {
    const int64_t nword = orc_nword(nbasis), n1 = nbasis, n2 = n1 * n1, n3 = n1 * n2, n4 = n2 * n2;
    if (kind != ORC_DOCI && kind != ORC_FULLCI)
        return -2;
    const int64_t nw = kind == ORC_FULLCI ? 2 * nword : nword;
    if (nword > 4)
        return -2;
    det_index ix;
    if (index_build(&ix, ndet2, nw, dets2))
        return -1;
#define FOUND(j) (tr ? (j) != -1 : (j) > idet)
    uint64_t det[8];
    int64_t ou[256], od[256], vu[256], vd[256];
    if (kind == ORC_DOCI) {
        double *d0 = rdm1, *d2 = rdm2;
        memset(d0, 0, sizeof(double) * n2);
        memset(d2, 0, sizeof(double) * n2);
        for (int64_t idet = 0; idet < ndet; ++idet) {
            const uint64_t *rdet = dets + idet * nw;
            memcpy(det, rdet, sizeof(uint64_t) * nw);
            int64_t no = fill_occs(nword, rdet, ou), nv = fill_virs(nword, n1, rdet, vu);
            int64_t self = tr ? index_find(&ix, det) : idet;
            const double val1 = self != -1 ? coeffs[idet] * coeffs2[self] : 0.;
            for (int64_t i = 0; i < no; ++i) {
                int64_t k = ou[i];
                d0[k * (n1 + 1)] += val1;
                for (int64_t j = i + 1; j < no; ++j) {
                    int64_t l = ou[j];
                    d2[n1 * k + l] += val1;
                    d2[n1 * l + k] += val1;
                }
                for (int64_t j = 0; j < nv; ++j) {
                    int64_t l = vu[j];
                    excite(det, k, l);
                    int64_t jdet = index_find(&ix, det);
                    excite(det, l, k);
                    if (FOUND(jdet)) {
                        const double val2 = coeffs[idet] * coeffs2[jdet];
                        d0[n1 * k + l] += val2;
                        if (!tr)
                            d0[n1 * l + k] += val2;
                    }
                }
            }
        }
        free(ix.slots);
        return 0;
    }
    double *aa = rdm1, *bb = rdm1 + n2;
    double *aaaa = rdm2, *bbbb = rdm2 + n4, *abab = rdm2 + 2 * n4;
    memset(rdm1, 0, sizeof(double) * 2 * n2);
    memset(rdm2, 0, sizeof(double) * 3 * n4);
#define R4(a, p, q, r, t) a[(p) * n3 + (q) * n2 + (r) * n1 + (t)]
    for (int64_t idet = 0; idet < ndet; ++idet) {
        const uint64_t *rup = dets + idet * nw, *rdn = rup + nword;
        uint64_t *up = det, *dn = det + nword;
        memcpy(det, rup, sizeof(uint64_t) * nw);
        int64_t nou = fill_occs(nword, rup, ou), nod = fill_occs(nword, rdn, od);
        int64_t nvu = fill_virs(nword, n1, rup, vu), nvd = fill_virs(nword, n1, rdn, vd);
        int64_t self = tr ? index_find(&ix, det) : idet;
        const double val1 = self != -1 ? coeffs[idet] * coeffs2[self] : 0.;
        for (int64_t i = 0; i < nou; ++i) {
            int64_t ii = ou[i];
            aa[(n1 + 1) * ii] += val1;
            for (int64_t k = i + 1; k < nou; ++k) {
                int64_t kk = ou[k];
                R4(aaaa, ii, kk, ii, kk) += val1;
                R4(aaaa, ii, kk, kk, ii) -= val1;
                R4(aaaa, kk, ii, ii, kk) -= val1;
                R4(aaaa, kk, ii, kk, ii) += val1;
            }
            for (int64_t k = 0; k < nod; ++k) {
                int64_t kk = od[k];
                R4(abab, ii, kk, ii, kk) += val1;
            }
            for (int64_t j = 0; j < nvu; ++j) {
                int64_t jj = vu[j];
                excite(up, ii, jj);
                const int sign_up = orc_phase_single(rup, ii, jj);
                int64_t jdet = index_find(&ix, det);
                if (FOUND(jdet)) {
                    const double val2 = coeffs[idet] * coeffs2[jdet] * sign_up;
                    aa[ii * n1 + jj] += val2;
                    if (!tr)
                        aa[jj * n1 + ii] += val2;
                    for (int64_t k = 0; k < nou; ++k) {
                        if (i == k)
                            continue;
                        int64_t kk = ou[k];
                        R4(aaaa, ii, kk, jj, kk) += val2;
                        R4(aaaa, ii, kk, kk, jj) -= val2;
                        R4(aaaa, kk, ii, kk, jj) += val2;
                        R4(aaaa, kk, ii, jj, kk) -= val2;
                        if (!tr) {
                            R4(aaaa, jj, kk, ii, kk) += val2;
                            R4(aaaa, jj, kk, kk, ii) -= val2;
                            R4(aaaa, kk, jj, ii, kk) -= val2;
                            R4(aaaa, kk, jj, kk, ii) += val2;
                        }
                    }
                    for (int64_t k = 0; k < nod; ++k) {
                        int64_t kk = od[k];
                        R4(abab, ii, kk, jj, kk) += val2;
                        if (!tr)
                            R4(abab, jj, kk, ii, kk) += val2;
                    }
                }
                for (int64_t k = 0; k < nod; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = 0; l < nvd; ++l) {
                        int64_t ll = vd[l];
                        excite(dn, kk, ll);
                        jdet = index_find(&ix, det);
                        if (FOUND(jdet)) {
                            const double val2 = coeffs[idet] * coeffs2[jdet] * sign_up * orc_phase_single(rdn, kk, ll);
                            R4(abab, ii, kk, jj, ll) += val2;
                            if (!tr)
                                R4(abab, jj, ll, ii, kk) += val2;
                        }
                        excite(dn, ll, kk);
                    }
                }
                for (int64_t k = i + 1; k < nou; ++k) {
                    int64_t kk = ou[k];
                    for (int64_t l = j + 1; l < nvu; ++l) {
                        int64_t ll = vu[l];
                        excite(up, kk, ll);
                        jdet = index_find(&ix, det);
                        if (FOUND(jdet)) {
                            const double val2 = coeffs[idet] * coeffs2[jdet] * orc_phase_double(rup, ii, kk, jj, ll);
                            R4(aaaa, ii, kk, jj, ll) += val2;
                            R4(aaaa, ii, kk, ll, jj) -= val2;
                            R4(aaaa, kk, ii, jj, ll) -= val2;
                            R4(aaaa, kk, ii, ll, jj) += val2;
                            if (!tr) {
                                R4(aaaa, jj, ll, ii, kk) += val2;
                                R4(aaaa, jj, ll, kk, ii) -= val2;
                                R4(aaaa, ll, jj, ii, kk) -= val2;
                                R4(aaaa, ll, jj, kk, ii) += val2;
                            }
                        }
                        excite(up, ll, kk);
                    }
                }
                excite(up, jj, ii);
            }
        }
        for (int64_t i = 0; i < nod; ++i) {
            int64_t ii = od[i];
            bb[(n1 + 1) * ii] += val1;
            for (int64_t k = i + 1; k < nod; ++k) {
                int64_t kk = od[k];
                R4(bbbb, ii, kk, ii, kk) += val1;
                R4(bbbb, ii, kk, kk, ii) -= val1;
                R4(bbbb, kk, ii, ii, kk) -= val1;
                R4(bbbb, kk, ii, kk, ii) += val1;
            }
            for (int64_t j = 0; j < nvd; ++j) {
                int64_t jj = vd[j];
                excite(dn, ii, jj);
                int64_t jdet = index_find(&ix, det);
                if (FOUND(jdet)) {
                    const double val2 = coeffs[idet] * coeffs2[jdet] * orc_phase_single(rdn, ii, jj);
                    bb[ii * n1 + jj] += val2;
                    if (!tr)
                        bb[jj * n1 + ii] += val2;
                    for (int64_t k = 0; k < nou; ++k) {
                        int64_t kk = ou[k];
                        R4(abab, kk, ii, kk, jj) += val2;
                        if (!tr)
                            R4(abab, kk, jj, kk, ii) += val2;
                    }
                    for (int64_t k = 0; k < nod; ++k) {
                        if (i == k)
                            continue;
                        int64_t kk = od[k];
                        R4(bbbb, ii, kk, jj, kk) += val2;
                        R4(bbbb, ii, kk, kk, jj) -= val2;
                        R4(bbbb, kk, ii, kk, jj) += val2;
                        R4(bbbb, kk, ii, jj, kk) -= val2;
                        if (!tr) {
                            R4(bbbb, jj, kk, ii, kk) += val2;
                            R4(bbbb, jj, kk, kk, ii) -= val2;
                            R4(bbbb, kk, jj, ii, kk) -= val2;
                            R4(bbbb, kk, jj, kk, ii) += val2;
                        }
                    }
                }
                for (int64_t k = i + 1; k < nod; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = j + 1; l < nvd; ++l) {
                        int64_t ll = vd[l];
                        excite(dn, kk, ll);
                        jdet = index_find(&ix, det);
                        if (FOUND(jdet)) {
                            const double val2 = coeffs[idet] * coeffs2[jdet] * orc_phase_double(rdn, ii, kk, jj, ll);
                            R4(bbbb, ii, kk, jj, ll) += val2;
                            R4(bbbb, ii, kk, ll, jj) -= val2;
                            R4(bbbb, kk, ii, jj, ll) -= val2;
                            R4(bbbb, kk, ii, ll, jj) += val2;
                            if (!tr) {
                                R4(bbbb, jj, ll, ii, kk) += val2;
                                R4(bbbb, ll, jj, ii, kk) -= val2;
                                R4(bbbb, jj, ll, kk, ii) -= val2;
                                R4(bbbb, ll, jj, kk, ii) += val2;
                            }
                        }
                        excite(dn, ll, kk);
                    }
                }
                excite(dn, jj, ii);
            }
        }
    }
#undef R4
#undef FOUND
    free(ix.slots);
    return 0;
}

/* Spin-orbital RDMs of a GenCI wave function from their definition (no
 * reference counterpart: the reference's GenCI compute_rdms,
 * pyci/src/rdm.cpp:532-632, writes past its output arrays and repeats index
 * factors, so its result is undefined):
 *   rdm1[p][q] = sum_IJ c1_I c2_J <I| a+_p a_q |J>,
 *   rdm2[p][q][r][s] = sum_IJ c1_I c2_J <I| a+_p a+_q a_s a_r |J>,
 * n = nbasis spin orbitals; (dets1, c1) the bra, (dets2, c2) the ket (the
 * same wave function for compute_rdms).  Ket-driven: every determinant J of
 * the ket, each of its diagonal, single and double excitations I found in
 * the bra, with the sign of the operator string applied to J (occupied
 * orbitals below each acted orbital) and all antisymmetric images. */

/* (-1)^(number of occupied orbitals below p). */
static int below_sign(const uint64_t *d, int64_t p) {
    int c = 0;
    for (int64_t w = 0; w < (p >> 6); ++w)
        c += __builtin_popcountll(d[w]);
    const uint64_t m = (p & 63) ? (d[p >> 6] & ((1ULL << (p & 63)) - 1)) : 0;
    c += __builtin_popcountll(m);
    return (c & 1) ? -1 : 1;
}

static void flip_bit(uint64_t *d, int64_t p) { d[p >> 6] ^= 1ULL << (p & 63); }

int orc_compute_rdms_genci(int64_t nbasis, int64_t ndet1, const uint64_t *dets1, const double *c1, int64_t ndet2,
                           const uint64_t *dets2, const double *c2, double *rdm1, double *rdm2) {
    const int64_t nword = orc_nword(nbasis), n1 = nbasis, n2 = n1 * n1, n3 = n1 * n2, n4 = n2 * n2;
    if (nword > 4)
        return -2;
    det_index ix;
    if (index_build(&ix, ndet1, nword, dets1))
        return -1;
    memset(rdm1, 0, sizeof(double) * n2);
    memset(rdm2, 0, sizeof(double) * n4);
    uint64_t det[4];
    int64_t occ[256], vir[256];
    for (int64_t jdet = 0; jdet < ndet2; ++jdet) {
        const uint64_t *kdet = dets2 + jdet * nword;
        const double cj = c2[jdet];
        const int64_t no = fill_occs(nword, kdet, occ), nv = fill_virs(nword, n1, kdet, vir);
        memcpy(det, kdet, sizeof(uint64_t) * nword);
        int64_t idet = index_find(&ix, det);
        if (idet != -1) {
            const double v = c1[idet] * cj;
            for (int64_t x = 0; x < no; ++x) {
                const int64_t p = occ[x];
                rdm1[p * (n1 + 1)] += v;
                for (int64_t y = 0; y < no; ++y) {
                    const int64_t q = occ[y];
                    if (q == p)
                        continue;
                    rdm2[p * n3 + q * n2 + p * n1 + q] += v;
                    rdm2[p * n3 + q * n2 + q * n1 + p] -= v;
                }
            }
        }
        for (int64_t x = 0; x < no; ++x) {
            const int64_t i = occ[x];
            for (int64_t y = 0; y < nv; ++y) {
                const int64_t a = vir[y];
                /* single: a+_a a_i J */
                int sg = below_sign(det, i);
                flip_bit(det, i);
                sg *= below_sign(det, a);
                flip_bit(det, a);
                idet = index_find(&ix, det);
                if (idet != -1) {
                    const double v = c1[idet] * cj * sg;
                    rdm1[a * n1 + i] += v;
                    for (int64_t z = 0; z < no; ++z) {
                        const int64_t k = occ[z];
                        if (k == i)
                            continue;
                        rdm2[a * n3 + k * n2 + i * n1 + k] += v;
                        rdm2[k * n3 + a * n2 + i * n1 + k] -= v;
                        rdm2[a * n3 + k * n2 + k * n1 + i] -= v;
                        rdm2[k * n3 + a * n2 + k * n1 + i] += v;
                    }
                }
                flip_bit(det, a);
                flip_bit(det, i);
            }
        }
        /* doubles: a+_a a+_b a_j a_i J, i < j occupied, a < b virtual */
        for (int64_t x = 0; x < no; ++x)
            for (int64_t x2 = x + 1; x2 < no; ++x2)
                for (int64_t y = 0; y < nv; ++y)
                    for (int64_t y2 = y + 1; y2 < nv; ++y2) {
                        const int64_t i = occ[x], j = occ[x2], a = vir[y], b = vir[y2];
                        int sg = below_sign(det, i);
                        flip_bit(det, i);
                        sg *= below_sign(det, j);
                        flip_bit(det, j);
                        sg *= below_sign(det, b);
                        flip_bit(det, b);
                        sg *= below_sign(det, a);
                        flip_bit(det, a);
                        idet = index_find(&ix, det);
                        if (idet != -1) {
                            const double v = c1[idet] * cj * sg;
                            rdm2[a * n3 + b * n2 + i * n1 + j] += v;
                            rdm2[b * n3 + a * n2 + i * n1 + j] -= v;
                            rdm2[a * n3 + b * n2 + j * n1 + i] -= v;
                            rdm2[b * n3 + a * n2 + j * n1 + i] += v;
                        }
                        memcpy(det, kdet, sizeof(uint64_t) * nword);
                    }
    }
    free(ix.slots);
    return 0;
}

int orc_compute_rdms(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                     const double *coeffs, double *rdm1, double *rdm2) {
    (void)nocc_up;
    (void)nocc_dn;
    return rdms_core(kind, nbasis, ndet, dets, coeffs, ndet, dets, coeffs, 0, rdm1, rdm2);
}

int orc_compute_transition_rdms(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet1,
                                const uint64_t *dets1, const double *coeffs1, int64_t ndet2, const uint64_t *dets2,
                                const double *coeffs2, double *rdm1, double *rdm2) {
    (void)nocc_up;
    (void)nocc_dn;
    return rdms_core(kind, nbasis, ndet1, dets1, coeffs1, ndet2, dets2, coeffs2, 1, rdm1, rdm2);
}

/* ---------------- Epstein-Nesbet second-order correction ---------------- */

typedef struct {
    int64_t n, cap, nwords;
    uint64_t *words;
    double *val;
} termbuf;

static int term_push(termbuf *t, const uint64_t *d, double v) {
    if (t->n == t->cap) {
        int64_t cap = t->cap ? 2 * t->cap : 1024;
        uint64_t *w = realloc(t->words, sizeof(uint64_t) * cap * t->nwords);
        double *x = realloc(t->val, sizeof(double) * cap);
        if (!w || !x) {
            free(w ? w : t->words);
            free(x ? x : t->val);
            t->words = NULL;
            t->val = NULL;
            return -1;
        }
        t->words = w;
        t->val = x;
        t->cap = cap;
    }
    memcpy(t->words + t->n * t->nwords, d, sizeof(uint64_t) * t->nwords);
    t->val[t->n++] = v;
    return 0;
}

/* FullCI diagonal element of a determinant (compute_enpt2_thread_gather,
 * pyci/src/enpt2.cpp:37-74): alpha terms with alpha-beta Coulomb, then beta. */
static double fci_diag(int64_t nword, int64_t n1, const uint64_t *det, const double *one, const double *two) {
    const int64_t n2 = n1 * n1, n3 = n1 * n2;
    int64_t ou[256], od[256];
    int64_t nou = fill_occs(nword, det, ou), nod = fill_occs(nword, det + nword, od);
    double diag = 0.0;
    for (int64_t i = 0; i < nou; ++i) {
        int64_t j = ou[i];
        diag += one[(n1 + 1) * j];
        for (int64_t k = i + 1; k < nou; ++k) {
            int64_t l = ou[k];
            diag += TWO(j, l, j, l) - TWO(j, l, l, j);
        }
        for (int64_t k = 0; k < nod; ++k) {
            int64_t l = od[k];
            diag += TWO(j, l, j, l);
        }
    }
    for (int64_t i = 0; i < nod; ++i) {
        int64_t j = od[i];
        diag += one[(n1 + 1) * j];
        for (int64_t k = i + 1; k < nod; ++k) {
            int64_t l = od[k];
            diag += TWO(j, l, j, l) - TWO(j, l, l, j);
        }
    }
    return diag;
}

/* compute_enpt2 (pyci/src/enpt2.cpp:76-197, 332-375) for FullCI
 * determinants; DOCI runs through its FullCI image (alpha = beta string),
 * as the reference does.  Every external determinant k reached from i with
 * |H_ki| > eps / |c_i| collects H_ki c_i (phase included) in loop order;
 * the result is energy + sum_k V_k^2 / (energy - ecore - H_kk). */
int orc_compute_enpt2(int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet, const uint64_t *dets,
                      const double *coeffs, const double *one_mo, const double *two_mo, double energy, double ecore,
                      double eps, double *result) {
    const int64_t nword = orc_nword(nbasis), nw = 2 * nword, n1 = nbasis, n2 = n1 * n1, n3 = n1 * n2;
    const double *one = one_mo, *two = two_mo;
    (void)nocc_up;
    (void)nocc_dn;
    if ((kind != ORC_DOCI && kind != ORC_FULLCI) || nword > 4)
        return -2;
    uint64_t *fdets = malloc(sizeof(uint64_t) * (ndet ? ndet : 1) * nw);
    if (!fdets)
        return -1;
    for (int64_t i = 0; i < ndet; ++i)
        for (int64_t w = 0; w < nword; ++w) {
            const uint64_t a = kind == ORC_DOCI ? dets[i * nword + w] : dets[i * nw + w];
            const uint64_t b = kind == ORC_DOCI ? dets[i * nword + w] : dets[i * nw + nword + w];
            fdets[i * nw + w] = a;
            fdets[i * nw + nword + w] = b;
        }
    det_index ix;
    if (index_build(&ix, ndet, nw, fdets)) {
        free(fdets);
        return -1;
    }
    termbuf t = {0, 0, nw, NULL, NULL};
    int rc = 0;
    uint64_t det[8];
    int64_t ou[256], od[256], vu[256], vd[256];
#define PUSH(v)                                                                                                        \
    do {                                                                                                               \
        if (index_find(&ix, det) == -1 && term_push(&t, det, (v)))                                                     \
            rc = -1;                                                                                                   \
    } while (0)
    for (int64_t idet = 0; idet < ndet && !rc; ++idet) {
        const uint64_t *rup = fdets + idet * nw, *rdn = rup + nword;
        uint64_t *up = det, *dn = det + nword;
        memcpy(det, rup, sizeof(uint64_t) * nw);
        const double ci = coeffs[idet], eps_i = eps / fabs(ci);
        int64_t nou = fill_occs(nword, rup, ou), nod = fill_occs(nword, rdn, od);
        int64_t nvu = fill_virs(nword, n1, rup, vu), nvd = fill_virs(nword, n1, rdn, vd);
        for (int64_t i = 0; i < nou && !rc; ++i) {
            int64_t ii = ou[i];
            for (int64_t j = 0; j < nvu && !rc; ++j) {
                int64_t jj = vu[j];
                excite(up, ii, jj);
                const int sign_up = orc_phase_single(rup, ii, jj);
                double val = one[n1 * ii + jj];
                for (int64_t k = 0; k < nou; ++k) {
                    int64_t kk = ou[k];
                    val += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                }
                for (int64_t k = 0; k < nod; ++k) {
                    int64_t kk = od[k];
                    val += TWO(ii, kk, jj, kk);
                }
                if (fabs(val) > eps_i)
                    PUSH(val * (sign_up * ci));
                for (int64_t k = 0; k < nod && !rc; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = 0; l < nvd && !rc; ++l) {
                        int64_t ll = vd[l];
                        val = TWO(ii, kk, jj, ll);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            PUSH(val * ((double)(sign_up * orc_phase_single(rdn, kk, ll)) * ci));
                            excite(dn, ll, kk);
                        }
                    }
                }
                for (int64_t k = i + 1; k < nou && !rc; ++k) {
                    int64_t kk = ou[k];
                    for (int64_t l = j + 1; l < nvu && !rc; ++l) {
                        int64_t ll = vu[l];
                        val = TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(up, kk, ll);
                            PUSH(val * (orc_phase_double(rup, ii, kk, jj, ll) * ci));
                            excite(up, ll, kk);
                        }
                    }
                }
                excite(up, jj, ii);
            }
        }
        for (int64_t i = 0; i < nod && !rc; ++i) {
            int64_t ii = od[i];
            for (int64_t j = 0; j < nvd && !rc; ++j) {
                int64_t jj = vd[j];
                excite(dn, ii, jj);
                double val = one[n1 * ii + jj];
                for (int64_t k = 0; k < nou; ++k) {
                    int64_t kk = ou[k];
                    val += TWO(ii, kk, jj, kk);
                }
                for (int64_t k = 0; k < nod; ++k) {
                    int64_t kk = od[k];
                    val += TWO(ii, kk, jj, kk) - TWO(ii, kk, kk, jj);
                }
                if (fabs(val) > eps_i)
                    PUSH(val * (orc_phase_single(rdn, ii, jj) * ci));
                for (int64_t k = i + 1; k < nod && !rc; ++k) {
                    int64_t kk = od[k];
                    for (int64_t l = j + 1; l < nvd && !rc; ++l) {
                        int64_t ll = vd[l];
                        val = TWO(ii, kk, jj, ll) - TWO(ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            PUSH(val * (orc_phase_double(rdn, ii, kk, jj, ll) * ci));
                            excite(dn, ll, kk);
                        }
                    }
                }
                excite(dn, jj, ii);
            }
        }
    }
#undef PUSH
    free(ix.slots);
    free(fdets);
    if (rc) {
        free(t.words);
        free(t.val);
        return -1;
    }
    /* Sum each determinant's contributions in loop order (the reference's
     * per-thread order with one thread), then the correction. */
    det_index cx;
    if (index_build(&cx, t.n, nw, t.words)) {
        free(t.words);
        free(t.val);
        return -1;
    }
    double *sum = calloc(t.n ? t.n : 1, sizeof(double));
    for (int64_t c = 0; c < t.n; ++c)
        sum[index_find(&cx, t.words + c * nw)] += t.val[c];
    const double e = energy - ecore;
    double correction = 0.0;
    for (int64_t c = 0; c < t.n; ++c)
        if (index_find(&cx, t.words + c * nw) == c)
            correction += sum[c] * sum[c] / (e - fci_diag(nword, n1, t.words + c * nw, one, two));
    *result = energy + correction;
    free(sum);
    free(cx.slots);
    free(t.words);
    free(t.val);
    return 0;
}
