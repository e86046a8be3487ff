// Two-pass CSR build of the CI Hamiltonian on sm_103a.
//
// Replaces the serial row loop of pyci::SparseOp (update + add_row,
// pyci/src/sparseop.cpp:186-502).  Pass 1 counts the stored entries of every
// row, an exclusive scan turns the counts into row pointers, and pass 2
// enumerates the same excitations again, evaluates the Slater-Condon matrix
// elements in FP64 with the reference's summation order, sorts each row by
// column in shared memory (bitonic network) and writes it in place.
//
// One thread block per row: its threads split the row's candidate
// excitations (singles, same-spin doubles, opposite-spin doubles) by index,
// so a row of ~1,700 entries (FCI 12 orbitals, 5+5 electrons) is generated
// by 256 threads without any per-thread list.  Columns come either from the
// colex rank of the excited determinant (when the wave function is the full
// add_all_dets space) or from the device hash table.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <mutex>
#include <new>
#include <vector>

#include "detops.cuh"
#include "internal.h"
#include "split_bits.h"

namespace pyci_gpu {

constexpr int32_t kSentinel = INT32_MAX;

struct BuildParams {
    int kind;
    int nbasis;
    int nocc_up, nocc_dn;
    int genci_exact;
    int colex;
    int symmetric;
    int64_t ndet, nrow, ncol;
    int64_t legacy_nrow, legacy_ncol;
    int64_t nbeta;          // C(nbasis, nocc_dn): FCI column = rank_a * nbeta + rank_b
    const int64_t *binom;   // [(nbasis + 1) * ldk]
    int ldk;
    DetTable table;
    const uint64_t *dets;   // [ndet * nwords] (hash mode) or null
    const double *one_mo, *two_mo, *h, *v, *w;
    int ncache;             // rank-cache entries per row (0: no cache)
    int binom_smem;         // binomial-table entries staged in shared memory (0: read from global)
    int64_t *counts;        // pass 1 output [nrow]
    const int64_t *rowptr;  // pass 2 input [nrow + 1]
    int32_t *cols;
    double *vals;
    int32_t *lower_len;
    double *diag;
    int *error;             // set to a nonzero code on an internal inconsistency
};

// Column limit of a row's own (lower / general) entries: update() keeps the
// rows built before it with their old column range (pyci/src/sparseop.cpp:175-201).
__device__ __forceinline__ int64_t row_limit(const BuildParams &p, int64_t r) {
    return (r < p.legacy_nrow) ? p.legacy_ncol : p.ncol;
}

// Whether row i stores column j (reference filters at pyci/src/sparseop.cpp:243,
// 301, 321, 343, 381, 401, 461, 483: found, j < idet when symmetric, j < ncol).
// Symmetric operators also store the mirror of every lower entry.
__device__ __forceinline__ bool keep_entry(const BuildParams &p, int64_t i, int64_t j) {
    if (j < 0)
        return false;
    if (!p.symmetric)
        return j < row_limit(p, i);
    if (j < i)
        return j < row_limit(p, i);
    if (j == i)
        return i < row_limit(p, i);
    return j < p.nrow && i < row_limit(p, j);
}

struct RowState {
    int no_a, no_b, nv_a, nv_b;
    int16_t occ_a[kMaxOcc], occ_b[kMaxOcc];
    int16_t vir_a[kMaxVir], vir_b[kMaxVir];
    uint64_t ra[4], rb[4];
};

__device__ __forceinline__ void decode_pair(int q, int &i, int &k) {
    // q = k (k - 1) / 2 + i with 0 <= i < k.
    int kk = static_cast<int>((1.0f + sqrtf(1.0f + 8.0f * static_cast<float>(q))) * 0.5f);
    while (kk * (kk - 1) / 2 > q)
        --kk;
    while ((kk + 1) * kk / 2 <= q)
        ++kk;
    k = kk;
    i = q - kk * (kk - 1) / 2;
}

__device__ __forceinline__ double two_mo_at(const double *two, int n, int i, int k, int j, int l) {
    const int64_t n1 = n, n2 = n1 * n1, n3 = n2 * n1;
    return __ldg(&two[i * n3 + k * n2 + j * n1 + l]);
}

// Load the row's determinant and occupation lists into shared memory.
template<int NW>
__device__ void load_row(const BuildParams &p, int64_t row, RowState &s) {
    if (threadIdx.x == 0) {
        uint64_t a[NW], b[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w)
            a[w] = b[w] = 0;
        if (p.kind == PYCI_WFN_FULLCI) {
            if (p.colex) {
                unrank_colex<NW>(row / p.nbeta, p.nbasis, p.nocc_up, p.binom, p.ldk, a);
                unrank_colex<NW>(row % p.nbeta, p.nbasis, p.nocc_dn, p.binom, p.ldk, b);
            } else {
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    a[w] = p.dets[row * 2 * NW + w];
                    b[w] = p.dets[row * 2 * NW + NW + w];
                }
            }
        } else {
            if (p.colex) {
                unrank_colex<NW>(row, p.nbasis, p.nocc_up, p.binom, p.ldk, a);
            } else {
#pragma unroll
                for (int w = 0; w < NW; ++w)
                    a[w] = p.dets[row * NW + w];
            }
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            s.ra[w] = a[w];
            s.rb[w] = b[w];
        }
        s.no_a = occ_list<NW>(a, s.occ_a);
        s.nv_a = vir_list<NW>(a, p.nbasis, s.vir_a);
        if (p.kind == PYCI_WFN_FULLCI) {
            s.no_b = occ_list<NW>(b, s.occ_b);
            s.nv_b = vir_list<NW>(b, p.nbasis, s.vir_b);
        } else {
            s.no_b = s.nv_b = 0;
        }
    }
    __syncthreads();
}

// Column of an excited determinant.
template<int NW>
__device__ __forceinline__ int64_t column_of(const BuildParams &p, const uint64_t *a,
                                             const uint64_t *b) {
    if (p.kind == PYCI_WFN_FULLCI) {
        if (p.colex)
            return rank_colex<NW>(a, p.binom, p.ldk) * p.nbeta + rank_colex<NW>(b, p.binom, p.ldk);
        uint64_t key[2 * NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            key[w] = a[w];
            key[NW + w] = b[w];
        }
        return p.table.find<2 * NW>(key);
    }
    if (p.colex)
        return rank_colex<NW>(a, p.binom, p.ldk);
    return p.table.find<NW>(a);
}

// Number of candidate excitations of a row (diagonal excluded).
__device__ __forceinline__ int num_candidates(const BuildParams &p, const RowState &s) {
    if (p.kind == PYCI_WFN_DOCI)
        return s.no_a * s.nv_a;
    const int sa = s.no_a * s.nv_a;
    const int da = (s.no_a * (s.no_a - 1) / 2) * (s.nv_a * (s.nv_a - 1) / 2);
    if (p.kind == PYCI_WFN_GENCI)
        return sa + da;
    const int sb = s.no_b * s.nv_b;
    const int db = (s.no_b * (s.no_b - 1) / 2) * (s.nv_b * (s.nv_b - 1) / 2);
    return sa + sb + da + db + sa * sb;
}

// One candidate excitation of a row, decoded from its index.
struct Exc {
    int type;            // kDociPair, kSingleA, kSingleB, kDoubleAA, kDoubleBB, kDoubleAB
    int ii, jj, kk, ll;  // occupied/virtual orbitals (singles: ii -> jj; doubles: ii,kk -> jj,ll)
    int sa_idx, sb_idx;  // index among the row's alpha / beta singles (opposite-spin doubles)
    int q;               // index among the row's same-spin doubles
};
enum { kDociPair = 0, kSingleA = 1, kSingleB = 2, kDoubleAA = 3, kDoubleBB = 4, kDoubleAB = 5 };

// Candidate c: singles of the first string (alpha, or the GenCI/DOCI string),
// then [FullCI] beta singles, then same-spin doubles (alpha, then beta), then
// opposite-spin doubles.  The order only fixes the index; rows are sorted.
__device__ __forceinline__ Exc decode(const BuildParams &p, const RowState &s, int c) {
    Exc e{};
    const int sa = s.no_a * s.nv_a;
    if (p.kind == PYCI_WFN_DOCI) {
        e.type = kDociPair;
        e.sa_idx = c;
        e.ii = s.occ_a[c / s.nv_a];
        e.jj = s.vir_a[c % s.nv_a];
        return e;
    }
    if (c < sa) {
        e.type = kSingleA;
        e.sa_idx = c;
        e.ii = s.occ_a[c / s.nv_a];
        e.jj = s.vir_a[c % s.nv_a];
        return e;
    }
    c -= sa;
    const int qa = s.nv_a * (s.nv_a - 1) / 2;
    const int sb = s.no_b * s.nv_b;
    if (p.kind == PYCI_WFN_FULLCI) {
        if (c < sb) {
            e.type = kSingleB;
            e.sb_idx = c;
            e.ii = s.occ_b[c / s.nv_b];
            e.jj = s.vir_b[c % s.nv_b];
            return e;
        }
        c -= sb;
    }
    const int pa = s.no_a * (s.no_a - 1) / 2;
    const int pb = s.no_b * (s.no_b - 1) / 2, qb = s.nv_b * (s.nv_b - 1) / 2;
    if (c < pa * qa || (p.kind == PYCI_WFN_FULLCI && c < pa * qa + pb * qb)) {
        const bool alpha = c < pa * qa;
        const int q = alpha ? c : c - pa * qa;
        const int qq = alpha ? qa : qb;
        int i, k, x, y;
        decode_pair(q / qq, i, k);
        decode_pair(q % qq, x, y);
        const int16_t *occ = alpha ? s.occ_a : s.occ_b;
        const int16_t *vir = alpha ? s.vir_a : s.vir_b;
        e.type = alpha ? kDoubleAA : kDoubleBB;
        e.q = q;
        e.ii = occ[i];
        e.kk = occ[k];
        e.jj = vir[x];
        e.ll = vir[y];
        return e;
    }
    c -= pa * qa + pb * qb;
    e.type = kDoubleAB;
    e.sa_idx = c / sb;
    e.sb_idx = c % sb;
    e.ii = s.occ_a[e.sa_idx / s.nv_a];
    e.jj = s.vir_a[e.sa_idx % s.nv_a];
    e.kk = s.occ_b[e.sb_idx / s.nv_b];
    e.ll = s.vir_b[e.sb_idx % s.nv_b];
    return e;
}

// Column of an excitation: from the row's rank cache (full spaces) or by
// building the excited determinant and ranking / looking it up.
template<int NW>
__device__ __forceinline__ int64_t exc_column(const BuildParams &p, const RowState &s, int64_t row,
                                              const Exc &e, const int32_t *cache) {
    if (cache) {
        const int sa = s.no_a * s.nv_a, sb = s.no_b * s.nv_b;
        const int da = (s.no_a * (s.no_a - 1) / 2) * (s.nv_a * (s.nv_a - 1) / 2);
        if (p.kind != PYCI_WFN_FULLCI)
            return (e.type == kDoubleAA) ? cache[sa + e.q] : cache[e.sa_idx];
        const int64_t ra = row / p.nbeta, rb = row % p.nbeta;
        switch (e.type) {
        case kSingleA: return cache[e.sa_idx] * p.nbeta + rb;
        case kSingleB: return ra * p.nbeta + cache[sa + e.sb_idx];
        case kDoubleAA: return cache[sa + sb + e.q] * p.nbeta + rb;
        case kDoubleBB: return ra * p.nbeta + cache[sa + sb + da + e.q];
        default: return cache[e.sa_idx] * p.nbeta + cache[sa + e.sb_idx];
        }
    }
    uint64_t a[NW], b[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        a[w] = s.ra[w];
        b[w] = s.rb[w];
    }
    switch (e.type) {
    case kDociPair:
    case kSingleA:
        flip(a, e.ii);
        flip(a, e.jj);
        break;
    case kSingleB:
        flip(b, e.ii);
        flip(b, e.jj);
        break;
    case kDoubleAA:
        flip(a, e.ii);
        flip(a, e.kk);
        flip(a, e.jj);
        flip(a, e.ll);
        break;
    case kDoubleBB:
        flip(b, e.ii);
        flip(b, e.kk);
        flip(b, e.jj);
        flip(b, e.ll);
        break;
    default:
        flip(a, e.ii);
        flip(a, e.jj);
        flip(b, e.kk);
        flip(b, e.ll);
        break;
    }
    return column_of<NW>(p, a, b);
}

// phase * v for phase = +-1, as a sign-bit flip: bit-identical to the FP64
// product and free of FP64 arithmetic (scarce on this GPU).
__device__ __forceinline__ double apply_phase(int phase, double v) {
    return __longlong_as_double(__double_as_longlong(v) ^ (static_cast<long long>(phase < 0) << 63));
}

// Matrix element of an excitation, with the formulas and summation order of
// add_row (pyci/src/sparseop.cpp:220-258 DOCI, 260-427 FullCI, 429-502 GenCI).
template<int NW>
__device__ double exc_value(const BuildParams &p, const RowState &s, const Exc &e) {
    const int n = p.nbasis;
    const double *one = p.one_mo, *two = p.two_mo;
    const int ii = e.ii, jj = e.jj, kk = e.kk, ll = e.ll;
    switch (e.type) {
    case kDociPair:
        return __ldg(&p.v[ii * n + jj]);
    case kSingleA: {
        // 1-0 excitation (or the GenCI single)
        double v1 = __ldg(&one[ii * n + jj]);
        for (int t = 0; t < s.no_a; ++t) {
            const int k2 = s.occ_a[t];
            v1 += two_mo_at(two, n, ii, k2, jj, k2) - two_mo_at(two, n, ii, k2, k2, jj);
        }
        for (int t = 0; t < s.no_b; ++t) {
            const int k2 = s.occ_b[t];
            v1 += two_mo_at(two, n, ii, k2, jj, k2);
        }
        return apply_phase(phase_single<NW>(s.ra, ii, jj), v1);
    }
    case kSingleB: {
        // 0-1 excitation
        double v1 = __ldg(&one[ii * n + jj]);
        for (int t = 0; t < s.no_a; ++t) {
            const int k2 = s.occ_a[t];
            v1 += two_mo_at(two, n, ii, k2, jj, k2);
        }
        for (int t = 0; t < s.no_b; ++t) {
            const int k2 = s.occ_b[t];
            v1 += two_mo_at(two, n, ii, k2, jj, k2) - two_mo_at(two, n, ii, k2, k2, jj);
        }
        return apply_phase(phase_single<NW>(s.rb, ii, jj), v1);
    }
    case kDoubleAA:
        return apply_phase(phase_double<NW>(s.ra, ii, kk, jj, ll),
                           two_mo_at(two, n, ii, kk, jj, ll) - two_mo_at(two, n, ii, kk, ll, jj));
    case kDoubleBB:
        return apply_phase(phase_double<NW>(s.rb, ii, kk, jj, ll),
                           two_mo_at(two, n, ii, kk, jj, ll) - two_mo_at(two, n, ii, kk, ll, jj));
    default:
        // 1-1 excitation: alpha ii -> jj, beta kk -> ll
        return apply_phase(phase_single<NW>(s.ra, ii, jj) * phase_single<NW>(s.rb, kk, ll),
                           two_mo_at(two, n, ii, kk, jj, ll));
    }
}

// Candidate c of row `row`: its column (or -1) and, when VALUES and the entry
// is kept, its matrix element.
template<int NW, bool VALUES>
__device__ __forceinline__ int64_t candidate(const BuildParams &p, const RowState &s, int64_t row, int c,
                                             double &val, const int32_t *cache) {
    const Exc e = decode(p, s, c);
    const int64_t col = exc_column<NW>(p, s, row, e, cache);
    if (VALUES && keep_entry(p, row, col))
        val = exc_value<NW>(p, s, e);
    return col;
}

// Fill the row's rank cache: the colex rank of every singly / doubly excited
// string, in decode()'s order (alpha singles, beta singles, alpha doubles,
// beta doubles; DOCI/GenCI: singles then doubles).  Full spaces only.
template<int NW>
__device__ void fill_rank_cache(const BuildParams &p, const RowState &s, const int64_t *binom, int32_t *cache) {
    const int sa = s.no_a * s.nv_a, sb = s.no_b * s.nv_b;
    const int pa = s.no_a * (s.no_a - 1) / 2, qa = s.nv_a * (s.nv_a - 1) / 2;
    const int pb = s.no_b * (s.no_b - 1) / 2, qb = s.nv_b * (s.nv_b - 1) / 2;
    const bool two = (p.kind == PYCI_WFN_FULLCI);
    const int nsingle_b = two ? sb : 0;
    const int ndouble_a = (p.kind == PYCI_WFN_DOCI) ? 0 : pa * qa;
    const int ndouble_b = two ? pb * qb : 0;
    const int total = sa + nsingle_b + ndouble_a + ndouble_b;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        uint64_t d[NW];
        const bool alpha = (t < sa) || (t >= sa + nsingle_b && t < sa + nsingle_b + ndouble_a);
#pragma unroll
        for (int w = 0; w < NW; ++w)
            d[w] = alpha ? s.ra[w] : s.rb[w];
        if (t < sa) {
            flip(d, s.occ_a[t / s.nv_a]);
            flip(d, s.vir_a[t % s.nv_a]);
        } else if (t < sa + nsingle_b) {
            const int u = t - sa;
            flip(d, s.occ_b[u / s.nv_b]);
            flip(d, s.vir_b[u % s.nv_b]);
        } else {
            const int u = alpha ? t - sa - nsingle_b : t - sa - nsingle_b - ndouble_a;
            const int qq = alpha ? qa : qb;
            const int16_t *occ = alpha ? s.occ_a : s.occ_b;
            const int16_t *vir = alpha ? s.vir_a : s.vir_b;
            int i, k, x, y;
            decode_pair(u / qq, i, k);
            decode_pair(u % qq, x, y);
            flip(d, occ[i]);
            flip(d, occ[k]);
            flip(d, vir[x]);
            flip(d, vir[y]);
        }
        int64_t r = 0;
        int cnt = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint64_t x = d[w];
            while (x) {
                const int pbit = __ffsll(static_cast<long long>(x)) - 1 + 64 * w;
                ++cnt;
                r += binom[pbit * p.ldk + cnt];
                x &= x - 1;
            }
        }
        cache[t] = static_cast<int32_t>(r);
    }
}

// Diagonal element in the reference's summation order.
__device__ double diagonal(const BuildParams &p, const RowState &s) {
    const int n = p.nbasis;
    const double *one = p.one_mo, *two = p.two_mo;
    if (p.kind == PYCI_WFN_DOCI) {
        double v1 = 0.0, v2 = 0.0;
        for (int i = 0; i < s.no_a; ++i) {
            const int k = s.occ_a[i];
            v1 += __ldg(&p.v[k * (n + 1)]);
            v2 += __ldg(&p.h[k]);
            for (int j = i + 1; j < s.no_a; ++j)
                v2 += __ldg(&p.w[k * n + s.occ_a[j]]);
        }
        return v1 + v2 * 2;
    }
    double v2 = 0.0;
    for (int i = 0; i < s.no_a; ++i) {
        const int ii = s.occ_a[i];
        v2 += __ldg(&one[(n + 1) * ii]);
        for (int k = i + 1; k < s.no_a; ++k) {
            const int kk = s.occ_a[k];
            v2 += two_mo_at(two, n, ii, kk, ii, kk) - two_mo_at(two, n, ii, kk, kk, ii);
        }
        for (int k = 0; k < s.no_b; ++k) {
            const int kk = s.occ_b[k];
            v2 += two_mo_at(two, n, ii, kk, ii, kk);
        }
    }
    for (int i = 0; i < s.no_b; ++i) {
        const int ii = s.occ_b[i];
        v2 += __ldg(&one[(n + 1) * ii]);
        for (int k = i + 1; k < s.no_b; ++k) {
            const int kk = s.occ_b[k];
            v2 += two_mo_at(two, n, ii, kk, ii, kk) - two_mo_at(two, n, ii, kk, kk, ii);
        }
    }
    return v2;
}

// Shared-memory scratch shared by both passes: [rank cache][binomial table].
struct RowScratch {
    int32_t *cache;
    const int64_t *binom;
};

__device__ __forceinline__ RowScratch setup_scratch(const BuildParams &p, unsigned char *base) {
    RowScratch r;
    r.cache = p.ncache ? reinterpret_cast<int32_t *>(base) : nullptr;
    const size_t off = (static_cast<size_t>(p.ncache) * sizeof(int32_t) + 7) & ~static_cast<size_t>(7);
    if (p.binom_smem) {
        int64_t *b = reinterpret_cast<int64_t *>(base + off);
        for (int t = threadIdx.x; t < p.binom_smem; t += blockDim.x)
            b[t] = p.binom[t];
        r.binom = b;
    } else {
        r.binom = p.binom;
    }
    return r;
}

// Pass 1: stored entries per row.
template<int NW>
__global__ void __launch_bounds__(256) count_kernel(BuildParams p, int64_t row0) {
    __shared__ RowState s;
    __shared__ int total;
    extern __shared__ __align__(16) unsigned char dyn[];
    const int64_t row = row0 + blockIdx.x;
    if (row >= p.nrow)
        return;
    if (threadIdx.x == 0)
        total = 0;
    const RowScratch sc = setup_scratch(p, dyn);
    load_row<NW>(p, row, s);
    if (sc.cache) {
        fill_rank_cache<NW>(p, s, sc.binom, sc.cache);
        __syncthreads();
    }
    const int nc = num_candidates(p, s);
    int mine = 0;
    double dummy = 0.0;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int64_t col = candidate<NW, false>(p, s, row, c, dummy, sc.cache);
        mine += keep_entry(p, row, col) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1)
        mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(&total, mine);
    __syncthreads();
    if (threadIdx.x == 0)
        p.counts[row] = total + (keep_entry(p, row, row) ? 1 : 0);
}

// Pass 2: matrix elements, in-row sort, write-out.  Dynamic shared memory
// holds `cap` (power of two >= candidates + 1) keys and values.
template<int NW>
__global__ void __launch_bounds__(256) fill_kernel(BuildParams p, int64_t row0, int cap) {
    __shared__ RowState s;
    extern __shared__ __align__(16) unsigned char smem[];
    double *sval = reinterpret_cast<double *>(smem);
    int32_t *skey = reinterpret_cast<int32_t *>(smem + sizeof(double) * cap);
    const int64_t row = row0 + blockIdx.x;
    if (row >= p.nrow)
        return;
    const RowScratch sc = setup_scratch(p, smem + (sizeof(double) + sizeof(int32_t)) * static_cast<size_t>(cap));
    load_row<NW>(p, row, s);
    if (sc.cache) {
        fill_rank_cache<NW>(p, s, sc.binom, sc.cache);
        __syncthreads();
    }
    const int nc = num_candidates(p, s);
    for (int c = threadIdx.x; c < cap; c += blockDim.x) {
        int32_t key = kSentinel;
        double val = 0.0;
        if (c < nc) {
            const int64_t col = candidate<NW, true>(p, s, row, c, val, sc.cache);
            if (keep_entry(p, row, col))
                key = static_cast<int32_t>(col);
        } else if (c == nc) {
            if (keep_entry(p, row, row)) {
                key = static_cast<int32_t>(row);
                val = diagonal(p, s);
            }
        }
        skey[c] = key;
        sval[c] = val;
    }
    __syncthreads();
    // Bitonic sort of (key, value) pairs by key, ascending.
    for (int size = 2; size <= cap; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < cap / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool up = ((lo & size) == 0);
                const int32_t klo = skey[lo], khi = skey[hi];
                if ((klo > khi) == up) {
                    skey[lo] = khi;
                    skey[hi] = klo;
                    const double vlo = sval[lo];
                    sval[lo] = sval[hi];
                    sval[hi] = vlo;
                }
            }
            __syncthreads();
        }
    }
    const int64_t start = p.rowptr[row];
    const int len = static_cast<int>(p.rowptr[row + 1] - start);
    if (threadIdx.x == 0) {
        if (len > cap || (len > 0 && skey[len - 1] == kSentinel) || (len < cap && skey[len] != kSentinel))
            atomicExch(p.error, 1);
    }
    for (int t = threadIdx.x; t < len && t < cap; t += blockDim.x) {
        const int32_t key = skey[t];
        p.cols[start + t] = key;
        p.vals[start + t] = sval[t];
        if (key == row)
            p.diag[row] = sval[t];
        const bool last_lower = (key <= row) && (t + 1 == len || skey[t + 1] > row);
        if (last_lower && p.lower_len)
            p.lower_len[row] = t + 1;
    }
    if (threadIdx.x == 0 && p.lower_len && (len == 0 || skey[0] > row))
        p.lower_len[row] = 0;
}

// Exc of a given kind and within-kind index (inverse of decode's layout).
__device__ __forceinline__ Exc make_exc(const RowState &s, int type, int i1, int i2) {
    Exc e{};
    e.type = type;
    const int qa = s.nv_a * (s.nv_a - 1) / 2, qb = s.nv_b * (s.nv_b - 1) / 2;
    int i, k, x, y;
    switch (type) {
    case kSingleA:
        e.sa_idx = i1;
        e.ii = s.occ_a[i1 / s.nv_a];
        e.jj = s.vir_a[i1 % s.nv_a];
        break;
    case kSingleB:
        e.sb_idx = i1;
        e.ii = s.occ_b[i1 / s.nv_b];
        e.jj = s.vir_b[i1 % s.nv_b];
        break;
    case kDoubleAA:
        e.q = i1;
        decode_pair(i1 / qa, i, k);
        decode_pair(i1 % qa, x, y);
        e.ii = s.occ_a[i];
        e.kk = s.occ_a[k];
        e.jj = s.vir_a[x];
        e.ll = s.vir_a[y];
        break;
    case kDoubleBB:
        e.q = i1;
        decode_pair(i1 / qb, i, k);
        decode_pair(i1 % qb, x, y);
        e.ii = s.occ_b[i];
        e.kk = s.occ_b[k];
        e.jj = s.vir_b[x];
        e.ll = s.vir_b[y];
        break;
    default: // kDoubleAB
        e.sa_idx = i1;
        e.sb_idx = i2;
        e.ii = s.occ_a[i1 / s.nv_a];
        e.jj = s.vir_a[i1 % s.nv_a];
        e.kk = s.occ_b[i2 / s.nv_b];
        e.ll = s.vir_b[i2 % s.nv_b];
        break;
    }
    return e;
}

// Exclusive prefix sum of v[0..n) in shared memory (n <= blockDim.x * 2).
__device__ void block_exclusive_scan(int *v, int *tmp, int n) {
    for (int t = threadIdx.x; t < n; t += blockDim.x)
        tmp[t] = v[t];
    __syncthreads();
    for (int off = 1; off < n; off <<= 1) {
        int a[2] = {0, 0};
        int c = 0;
        for (int t = threadIdx.x; t < n; t += blockDim.x, ++c)
            a[c] = (t >= off) ? tmp[t - off] : 0;
        __syncthreads();
        c = 0;
        for (int t = threadIdx.x; t < n; t += blockDim.x, ++c)
            tmp[t] += a[c];
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x)
        v[t] = tmp[t] - v[t];
    __syncthreads();
}

// Bitonic sort of n (power of two) int keys with int payloads.
__device__ void block_sort_pairs(int *key, int *val, int n) {
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool up = ((lo & size) == 0);
                const int klo = key[lo], khi = key[hi];
                if ((klo > khi) == up) {
                    key[lo] = khi;
                    key[hi] = klo;
                    const int v = val[lo];
                    val[lo] = val[hi];
                    val[hi] = v;
                }
            }
            __syncthreads();
        }
    }
}

constexpr int kSortedMax = 512; // max alpha (or beta) excitations + 1 per string for the table fill

// Full-space FullCI rows written directly in ascending column order.
//
// Columns are rank(a') * nbeta + rank(b'), so a row is the concatenation,
// over the row's alpha excitations a' = {a} + singles + doubles sorted by
// rank, of its beta partners sorted by rank: all of {b} + singles + doubles
// for a' = a, {b} + singles for a single, {b} for a double.  The sorted lists
// depend on one string only, so they are built once per string
// (string_tables_kernel) rather than once per row: for 12 orbitals, 5 + 5
// electrons, 792 strings serve 627,264 rows.  Only for builds that keep every
// candidate (fresh full space, nrow = ncol = ndet).
//
// Per string s of one spin (arrays [nstr][npad]):
//   key[s][i]     target string rank, ascending (INT32_MAX padding)
//   val[s][i]     type << 20 | index within its kind (type 0: s itself,
//                 1: single, 2: double; the index is the row's own
//                 occupied/virtual enumeration, as in make_exc)
//   off[s][i]     exclusive prefix of the number of beta partners of the
//                 entries before i (alpha use)
//   sub[s][c], subval[s][c]  the entries of type <= 1, in order (beta use)
//   self[s]       position of s itself in key
//   bits[s][w]    the string's occupation words (nw of them)
//   sdesc[s][i]   single i (in make_exc's enumeration): ii | jj << 8 | (phase < 0) << 16
//   dval[s][q]    the same-spin double q's matrix element (one string only:
//                 phase * (<ii kk|jj ll> - <ii kk|ll jj>), add_row's formula)
//   gmap[s][t]    alpha use: the group (position in key) that row entry t
//                 falls in, for t < glen (the uniform row length)
struct StringTables {
    int32_t *key, *val, *off, *sub, *subval, *self, *sdesc;
    uint16_t *gmap;
    uint64_t *bits;
    double *dval;
    int64_t glen;
    int npad, nw, n1, n2;
};

// One block per string of `spin` (0 alpha, 1 beta).  grp0 / grp1: beta
// partners of the alpha string itself / of an alpha single (the beta list
// length 1 + singles + doubles, and 1 + singles).  row_len: the uniform row
// length, checked on alpha tables (error 4 on a mismatch).
template<int NW>
__global__ void __launch_bounds__(256) string_tables_kernel(BuildParams p, int spin, StringTables T, int grp0,
                                                            int grp1, int64_t row_len) {
    __shared__ RowState s;
    __shared__ int key[kSortedMax], val[kSortedMax], flag[kSortedMax], tmp[kSortedMax];
    extern __shared__ __align__(16) unsigned char dyn[];
    const int64_t str = blockIdx.x;
    const RowScratch sc = setup_scratch(p, dyn);
    load_row<NW>(p, spin == 0 ? str * p.nbeta : str, s);
    fill_rank_cache<NW>(p, s, sc.binom, sc.cache);
    __syncthreads();
    const int sa = s.no_a * s.nv_a, sb = s.no_b * s.nv_b;
    const int da = (s.no_a * (s.no_a - 1) / 2) * (s.nv_a * (s.nv_a - 1) / 2);
    const int n1 = spin == 0 ? sa : sb;
    const int n2 = spin == 0 ? da : (s.no_b * (s.no_b - 1) / 2) * (s.nv_b * (s.nv_b - 1) / 2);
    const int nl = 1 + n1 + n2, npad = T.npad;
    // Rank cache layout: alpha singles, beta singles, alpha doubles, beta doubles.
    const int s_off = spin == 0 ? 0 : sa, d_off = sa + sb + (spin == 0 ? 0 : da);
    for (int t = threadIdx.x; t < npad; t += blockDim.x) {
        if (t < nl) {
            key[t] = (t == 0) ? static_cast<int>(str) : (t <= n1 ? sc.cache[s_off + t - 1] : sc.cache[d_off + t - 1 - n1]);
            val[t] = (t == 0) ? 0 : (t <= n1 ? ((1 << 20) | (t - 1)) : ((2 << 20) | (t - 1 - n1)));
        } else {
            key[t] = INT32_MAX;
            val[t] = 0;
        }
    }
    __syncthreads();
    block_sort_pairs(key, val, npad);
    int32_t *K = T.key + str * npad, *V = T.val + str * npad, *O = T.off + str * npad;
    int32_t *SK = T.sub + str * npad, *SV = T.subval + str * npad;
    // Entries of type <= 1, compacted in order.
    for (int t = threadIdx.x; t < npad; t += blockDim.x)
        flag[t] = (t < nl && (val[t] >> 20) <= 1) ? 1 : 0;
    __syncthreads();
    block_exclusive_scan(flag, tmp, npad);
    for (int t = threadIdx.x; t < npad; t += blockDim.x) {
        if (t < nl && (val[t] >> 20) <= 1) {
            SK[flag[t]] = key[t];
            SV[flag[t]] = val[t];
        }
        if (t < nl && val[t] == 0)
            T.self[str] = t;
    }
    if (threadIdx.x < T.nw)
        T.bits[str * T.nw + threadIdx.x] = spin == 0 ? s.ra[threadIdx.x] : s.rb[threadIdx.x];
    // Single descriptors and same-spin double values of this string.
    for (int i = threadIdx.x; i < n1; i += blockDim.x) {
        const Exc e = make_exc(s, spin == 0 ? kSingleA : kSingleB, i, 0);
        const int ph = phase_single<NW>(spin == 0 ? s.ra : s.rb, e.ii, e.jj);
        T.sdesc[str * T.n1 + i] = e.ii | (e.jj << 8) | ((ph < 0 ? 1 : 0) << 16);
    }
    for (int q = threadIdx.x; q < n2; q += blockDim.x)
        T.dval[str * T.n2 + q] = exc_value<NW>(p, s, make_exc(s, spin == 0 ? kDoubleAA : kDoubleBB, q, 0));
    __syncthreads();
    // Beta-partner counts along the sorted list, then their exclusive prefix.
    for (int t = threadIdx.x; t < npad; t += blockDim.x) {
        const int ty = val[t] >> 20;
        flag[t] = (t < nl) ? (ty == 0 ? grp0 : (ty == 1 ? grp1 : 1)) : 0;
    }
    __syncthreads();
    block_exclusive_scan(flag, tmp, npad);
    for (int t = threadIdx.x; t < npad; t += blockDim.x) {
        K[t] = key[t];
        V[t] = val[t];
        O[t] = flag[t];
    }
    if (T.gmap) {
        // Entry -> group map for the alpha use of this string.
        uint16_t *G = T.gmap + str * T.glen;
        for (int g = threadIdx.x; g < nl; g += blockDim.x) {
            const int ty = val[g] >> 20;
            const int64_t e = min(static_cast<int64_t>(flag[g]) + (ty == 0 ? grp0 : (ty == 1 ? grp1 : 1)), T.glen);
            for (int64_t t = flag[g]; t < e; ++t)
                G[t] = static_cast<uint16_t>(g);
        }
    }
    if (threadIdx.x == 0 && spin == 0) {
        const int ty = val[nl - 1] >> 20;
        const int64_t total = flag[nl - 1] + (ty == 0 ? grp0 : (ty == 1 ? grp1 : 1));
        if (total != row_len)
            atomicExch(p.error, 4);
    }
}

// Next set bit at or above position `from` in an NW-word string (-1: none).
template<int NW>
__device__ __forceinline__ int next_bit(const uint64_t *w, int from) {
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        if (from >= 64 * (i + 1))
            continue;
        const int sh = from - 64 * i;
        const uint64_t m = sh > 0 ? (w[i] >> sh) << sh : w[i];
        if (m)
            return 64 * i + __ffsll(static_cast<long long>(m)) - 1;
    }
    return -1;
}

// Ascending occupied and virtual orbital lists of one string, built by a
// warp: lane j tests orbital o0 + j, a ballot gives each list position.
template<int NW>
__device__ __forceinline__ void warp_lists(const uint64_t *bits, int nbasis, int16_t *occ, int16_t *vir, int &no,
                                           int &nv) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    int cno = 0, cnv = 0;
    for (int o0 = 0; o0 < nbasis; o0 += 32) {
        const int o = o0 + lane;
        const bool valid = o < nbasis;
        const bool in = valid && ((bits[o >> 6] >> (o & 63)) & 1ULL);
        const unsigned mo = __ballot_sync(0xffffffffu, in), mv = __ballot_sync(0xffffffffu, valid && !in);
        if (in && cno + __popc(mo & below) < kMaxOcc)
            occ[cno + __popc(mo & below)] = static_cast<int16_t>(o);
        else if (valid && !in && cnv + __popc(mv & below) < kMaxVir)
            vir[cnv + __popc(mv & below)] = static_cast<int16_t>(o);
        cno += __popc(mo);
        cnv += __popc(mv);
    }
    no = cno;
    nv = cnv;
}

// DOCI diagonal of every row of a full colex space, one thread per row, in
// diagonal()'s summation order: for each occupied pair k (ascending),
// v1 += v_kk, v2 += h_k, then v2 += w_kj for each later occupied j; the
// element is v1 + 2 v2.
template<int NW>
__global__ void doci_diag_kernel(BuildParams p) {
    const int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (row >= p.nrow)
        return;
    uint64_t a[NW];
    unrank_colex<NW>(row, p.nbasis, p.nocc_up, p.binom, p.ldk, a);
    const int n = p.nbasis;
    double v1 = 0.0, v2 = 0.0;
    for (int k = next_bit<NW>(a, 0); k >= 0; k = next_bit<NW>(a, k + 1)) {
        v1 += __ldg(&p.v[k * (n + 1)]);
        v2 += __ldg(&p.h[k]);
        for (int j = next_bit<NW>(a, k + 1); j >= 0; j = next_bit<NW>(a, j + 1))
            v2 += __ldg(&p.w[k * n + j]);
    }
    p.diag[row] = v1 + v2 * 2;
}

// Inclusive prefix sum of v[0..n) in shared memory by one warp (32-wide
// shuffle scans with a running carry).
__device__ __forceinline__ void warp_inclusive_scan(int *v, int n) {
    const int lane = threadIdx.x & 31;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        int x = (i < n) ? v[i] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o)
                x += y;
        }
        if (i < n)
            v[i] = x + carry;
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    __syncwarp();
}

// Full-space DOCI rows, one warp per row, each warp taking kDociRowsPerWarp
// consecutive rows (8 warps per block), with no block-wide barriers after
// the binomial table is staged.
//
// Colex order of same-size subsets is the numeric order of their bitmasks,
// so the pair moves i -> a of a string s sort by 2^a - 2^i: first every move
// with a < i, grouped by i descending and a ascending within a group; then s
// itself (the diagonal); then every move with a > i, grouped by a ascending
// and i descending within a group.  Prefix counts of the groups place any
// output position directly: lanes walk the row's positions in order (no
// sort, coalesced writes), rank each excited string (colex) and take its
// element v_ia.  Later strings of a warp's run follow by Gosper's step (next
// larger mask with the same popcount) for one-word strings.
constexpr int kDociRowsPerWarp = 4;
constexpr int kDociBinomSmem = 1024; // binomial-table entries staged in shared memory

template<int NW>
__global__ void __launch_bounds__(256) fill_doci_warp_kernel(BuildParams p, int64_t row0) {
    __shared__ int16_t occ_s[8][kMaxOcc], vir_s[8][kMaxVir];
    __shared__ int negc[8][kMaxOcc + 1], posc[8][kMaxVir + 1];
    __shared__ int64_t binom_s[kDociBinomSmem];
    const int nbin = (p.nbasis + 1) * p.ldk;
    const bool bsm = nbin <= kDociBinomSmem;
    if (bsm)
        for (int t = threadIdx.x; t < nbin; t += blockDim.x)
            binom_s[t] = p.binom[t];
    __syncthreads();
    const int64_t *binom = bsm ? binom_s : p.binom;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t first = row0 + (static_cast<int64_t>(blockIdx.x) * 8 + warp) * kDociRowsPerWarp;
    const int n = p.nbasis;
    int16_t *occ = occ_s[warp], *vir = vir_s[warp];
    int *nc_ = negc[warp], *pc_ = posc[warp];
    uint64_t bits[NW];
    for (int rr = 0; rr < kDociRowsPerWarp; ++rr) {
        const int64_t row = first + rr;
        if (row >= p.nrow)
            return;
        if (rr == 0 || NW > 1) {
#pragma unroll
            for (int w = 0; w < NW; ++w)
                bits[w] = 0;
            int64_t rank = row;
            int pp = n - 1;
            for (int j = p.nocc_up; j >= 1; --j) {
                while (pp >= 0 && binom[pp * p.ldk + j] > rank)
                    --pp;
                if (pp < 0)
                    break;
                bits[pp >> 6] |= 1ULL << (pp & 63);
                rank -= binom[pp * p.ldk + j];
                --pp;
            }
        } else {
            const uint64_t x = bits[0], c = x & (~x + 1), r = x + c;
            bits[0] = (((r ^ x) >> 2) >> (__ffsll(static_cast<long long>(c)) - 1)) | r;
        }
        int no, nv;
        __syncwarp();
        warp_lists<NW>(bits, n, occ, vir, no, nv);
        __syncwarp();
        // Group sizes: a < i moves of occupied occ[no-1-j] (descending j order):
        // virtuals below it = occ - index; a > i moves into vir[u]: occupied
        // below it = vir - index.  Slot 0 holds the exclusive start.
        for (int j = lane; j < no; j += 32) {
            const int t = no - 1 - j;
            nc_[j + 1] = occ[t] - t;
        }
        for (int u = lane; u < nv; u += 32)
            pc_[u + 1] = vir[u] - u;
        if (lane == 0)
            nc_[0] = pc_[0] = 0;
        __syncwarp();
        warp_inclusive_scan(nc_ + 1, no);
        warp_inclusive_scan(pc_ + 1, nv);
        const int nneg = nc_[no];
        const int64_t start = p.rowptr[row];
        const int len = static_cast<int>(p.rowptr[row + 1] - start);
        if (lane == 0) {
            if (len != no * nv + 1)
                atomicExch(p.error, 5);
            if (p.lower_len)
                p.lower_len[row] = nneg + 1;
        }
        for (int pos = lane; pos < len; pos += 32) {
            int32_t col;
            double val;
            if (pos == nneg) {
                col = static_cast<int32_t>(row);
                val = p.diag[row]; // doci_diag_kernel ran first
            } else {
                int ii, aa;
                if (pos < nneg) {
                    int lo = 0, hi = no - 1; // last j with nc_[j] <= pos
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (nc_[mid] <= pos)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    ii = occ[no - 1 - lo];
                    aa = vir[pos - nc_[lo]];
                } else {
                    const int q = pos - nneg - 1;
                    int lo = 0, hi = nv - 1; // last u with pc_[u] <= q
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (pc_[mid] <= q)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    aa = vir[lo];
                    const int below = pc_[lo + 1] - pc_[lo]; // occupied below aa
                    ii = occ[below - 1 - (q - pc_[lo])];
                }
                uint64_t d[NW];
#pragma unroll
                for (int w = 0; w < NW; ++w)
                    d[w] = bits[w];
                flip(d, ii);
                flip(d, aa);
                int64_t r = 0;
                int cnt = 0;
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    uint64_t x = d[w];
                    while (x) {
                        const int pb = __ffsll(static_cast<long long>(x)) - 1 + 64 * w;
                        ++cnt;
                        r += binom[pb * p.ldk + cnt];
                        x &= x - 1;
                    }
                }
                col = static_cast<int32_t>(r);
                val = __ldg(&p.v[ii * n + aa]);
            }
            p.cols[start + pos] = col;
            p.vals[start + pos] = val;
        }
        __syncwarp();
    }
}

// FullCI diagonal of every row, one thread per row, in diagonal()'s summation
// order (occupied orbitals ascending, as add_row<FullCIWfn> sums them):
// alpha i: h_ii, then (J - K) with each later alpha, then J with each beta;
// then beta i: h_ii, then (J - K) with each later beta.
template<int NW>
__global__ void fci_diag_kernel(BuildParams p, StringTables A, StringTables B) {
    const int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (row >= p.nrow)
        return;
    const int64_t ra = row / p.nbeta, rb = row % p.nbeta;
    uint64_t a[NW], b[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        a[w] = __ldg(A.bits + ra * NW + w);
        b[w] = __ldg(B.bits + rb * NW + w);
    }
    const int n = p.nbasis;
    const double *one = p.one_mo, *two = p.two_mo;
    double v2 = 0.0;
    for (int ii = next_bit<NW>(a, 0); ii >= 0; ii = next_bit<NW>(a, ii + 1)) {
        v2 += __ldg(&one[(n + 1) * ii]);
        for (int kk = next_bit<NW>(a, ii + 1); kk >= 0; kk = next_bit<NW>(a, kk + 1))
            v2 += two_mo_at(two, n, ii, kk, ii, kk) - two_mo_at(two, n, ii, kk, kk, ii);
        for (int kk = next_bit<NW>(b, 0); kk >= 0; kk = next_bit<NW>(b, kk + 1))
            v2 += two_mo_at(two, n, ii, kk, ii, kk);
    }
    for (int ii = next_bit<NW>(b, 0); ii >= 0; ii = next_bit<NW>(b, ii + 1)) {
        v2 += __ldg(&one[(n + 1) * ii]);
        for (int kk = next_bit<NW>(b, ii + 1); kk >= 0; kk = next_bit<NW>(b, kk + 1))
            v2 += two_mo_at(two, n, ii, kk, ii, kk) - two_mo_at(two, n, ii, kk, kk, ii);
    }
    p.diag[row] = v2;
}

// One warp per row (kFillRowsPerBlock rows per block), so nothing waits on a
// block-wide barrier: the warp builds the row's occupation lists from the
// string tables, computes the row's single-excitation values (O(nocc) sums
// each) on its lanes, then places every entry from the row's alpha and beta
// tables (binary search of the entry's alpha group; same-spin doubles and
// single descriptors precomputed per string) and writes columns and values
// in order.  The diagonal comes from fci_diag_kernel (one thread per row).
// Per-warp
// shared memory: RowState, the alpha group offsets (na ints), the singles
// (nsg doubles).
constexpr int kFillRowsPerBlock = 8;
constexpr int kTableMaxSingles = 2048; // alpha + beta singles per row (8 warps' shared memory stays < 160 KB)

template<int NW>
__global__ void __launch_bounds__(256) fill_fci_tables_kernel(BuildParams p, int64_t row0, StringTables A,
                                                              StringTables B, int na, int nsg) {
    extern __shared__ __align__(16) unsigned char dyn[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per_warp = (sizeof(RowState) + sizeof(double) * nsg + sizeof(int) * na + 15) & ~static_cast<size_t>(15);
    unsigned char *mine = dyn + per_warp * warp;
    RowState &s = *reinterpret_cast<RowState *>(mine);
    double *sval = reinterpret_cast<double *>(mine + sizeof(RowState));
    int *aoff = reinterpret_cast<int *>(mine + sizeof(RowState) + sizeof(double) * nsg);
    const int64_t row = row0 + static_cast<int64_t>(blockIdx.x) * kFillRowsPerBlock + warp;
    if (row >= p.nrow)
        return;
    const int64_t ra = row / p.nbeta, rb = row % p.nbeta;
    if (lane < NW) {
        s.ra[lane] = __ldg(A.bits + ra * NW + lane);
        s.rb[lane] = __ldg(B.bits + rb * NW + lane);
    }
    __syncwarp();
    {
        int no, nv;
        warp_lists<NW>(s.ra, p.nbasis, s.occ_a, s.vir_a, no, nv);
        if (lane == 0) {
            s.no_a = no;
            s.nv_a = nv;
        }
        warp_lists<NW>(s.rb, p.nbasis, s.occ_b, s.vir_b, no, nv);
        if (lane == 0) {
            s.no_b = no;
            s.nv_b = nv;
        }
    }
    const int32_t *AK = A.key + ra * A.npad, *AV = A.val + ra * A.npad, *AO = A.off + ra * A.npad;
    const int32_t *BK = B.key + rb * B.npad, *BV = B.val + rb * B.npad;
    const int32_t *SK = B.sub + rb * B.npad, *SV = B.subval + rb * B.npad;
    for (int t = lane; t < na; t += 32)
        aoff[t] = __ldg(AO + t);
    __syncwarp();
    const int sa = s.no_a * s.nv_a;
    for (int t = lane; t < nsg; t += 32)
        sval[t] = exc_value<NW>(p, s, t < sa ? make_exc(s, kSingleA, t, 0) : make_exc(s, kSingleB, t - sa, 0));
    const double dval = p.diag[row]; // fci_diag_kernel ran first
    __syncwarp();
    const int64_t start = p.rowptr[row];
    const int len = static_cast<int>(p.rowptr[row + 1] - start);
    if (lane == 0 && p.lower_len)
        p.lower_len[row] = aoff[__ldg(A.self + ra)] + __ldg(B.self + rb) + 1;
    const uint16_t *GM = A.gmap + ra * A.glen;
    const bool idx32 = p.nbasis <= 215; // n^4 < 2^31: 32-bit integral offsets
    const int nb = p.nbasis;
    for (int t = lane; t < len; t += 32) {
        const int g = __ldg(GM + t), qpos = t - aoff[g];
        const int av = __ldg(AV + g);
        const int tya = av >> 20, ia = av & ((1 << 20) - 1);
        int bk, bv;
        if (tya == 0) {
            bk = __ldg(BK + qpos);
            bv = __ldg(BV + qpos);
        } else if (tya == 1) {
            bk = __ldg(SK + qpos);
            bv = __ldg(SV + qpos);
        } else {
            bk = static_cast<int>(rb);
            bv = 0;
        }
        const int tyb = bv >> 20, ib = bv & ((1 << 20) - 1);
        const int64_t col = static_cast<int64_t>(__ldg(AK + g)) * p.nbeta + bk;
        double val;
        if (tya == 0 && tyb == 0) {
            val = dval;
        } else if (tya == 1 && tyb == 0) {
            val = sval[ia];
        } else if (tya == 0 && tyb == 1) {
            val = sval[sa + ib];
        } else if (tya == 0) {
            val = __ldg(B.dval + rb * B.n2 + ib); // beta double
        } else if (tya == 2) {
            val = __ldg(A.dval + ra * A.n2 + ia); // alpha double
        } else {
            // Opposite-spin double: alpha ii -> jj, beta kk -> ll.
            const int da = __ldg(A.sdesc + ra * A.n1 + ia), db = __ldg(B.sdesc + rb * B.n1 + ib);
            const int ii = da & 255, jj = (da >> 8) & 255, kk = db & 255, ll = (db >> 8) & 255;
            const double g2 = idx32 ? __ldg(p.two_mo + (((ii * nb + kk) * nb + jj) * nb + ll))
                                    : two_mo_at(p.two_mo, nb, ii, kk, jj, ll);
            val = apply_phase(((da ^ db) >> 16) & 1 ? -1 : 1, g2);
        }
        p.cols[start + t] = static_cast<int32_t>(col);
        p.vals[start + t] = val;
    }
}

// Tables of the implicit-column form (fcix.cu) from the string tables: per
// alpha string a, the targets of its singles and of its doubles in sorted
// order, the CSR offsets of their groups in the sorted row, and the offset of
// its own group (one thread per alpha string walks the sorted groups), plus
// adesc[a] = the string-table codes (type << 20 | index) of those singles and
// doubles in the same order, for the value fill; the beta lists (full:
// partners of the alpha string itself, sub: of an alpha single) transposed
// to [position][string].
__global__ void fcix_tables_kernel(StringTables TA, StringTables TB, int64_t nalpha, int64_t nbeta, int na, int nbl,
                                   int grp1, int ns, int nd, int la, int32_t *atab, int32_t *bfull, int32_t *bsub,
                                   uint16_t *bq, int32_t *adesc) {
    const int64_t n_f = static_cast<int64_t>(nbl) * nbeta, n_s = static_cast<int64_t>(grp1) * nbeta;
    const int64_t n_q = static_cast<int64_t>(la) * nbeta;
    const int64_t total = nalpha + n_f + n_s + n_q;
    const int w = 2 * (ns + nd) + 1;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (i < nalpha) {
            int32_t *row = atab + i * w, *code = adesc + i * (ns + nd);
            int is = 0, id = 0;
            for (int g = 0; g < na; ++g) {
                const int32_t v = TA.val[i * TA.npad + g];
                const int ty = v >> 20;
                const int32_t key = TA.key[i * TA.npad + g], off = TA.off[i * TA.npad + g];
                if (ty == 1 && is < ns) {
                    row[is] = key;
                    row[ns + nd + is] = off;
                    code[is] = v;
                    ++is;
                } else if (ty == 2 && id < nd) {
                    row[ns + id] = key;
                    row[2 * ns + nd + id] = off;
                    code[ns + id] = v;
                    ++id;
                } else if (ty == 0) {
                    row[w - 1] = off;
                }
            }
        } else if (i < nalpha + n_f) {
            const int64_t j = i - nalpha, q = j / nbeta, b = j - q * nbeta;
            bfull[j] = TB.key[b * TB.npad + q];
        } else if (i < nalpha + n_f + n_s) {
            const int64_t j = i - nalpha - n_f, q = j / nbeta, b = j - q * nbeta;
            bsub[j] = TB.sub[b * TB.npad + q];
        } else {
            // bq[(t / 4) * nbeta + b][t % 4] = partner t of b (b past the list).
            const int64_t j = i - nalpha - n_f - n_s, t = j / nbeta, b = j - t * nbeta;
            bq[((t >> 2) * nbeta + b) * 4 + (t & 3)] =
                static_cast<uint16_t>(t < nbl ? TB.key[b * TB.npad + t] : static_cast<int32_t>(b));
        }
    }
}

// Values of the implicit-column form (fcix.cu layout) of a full FullCI
// space, written without the CSR.  Block (a, h) serves slices [h spa / parts,
// (h + 1) spa / parts) of alpha string a, one warp per slice; lane l computes
// the entries of row (a, b), b = 32 (slice mod spa) + l, in the form's order
// and the warp stores each 4-entry packet's high and low parts as two
// coalesced 512-byte writes.  Every value is add_row's
// (pyci/src/sparseop.cpp:260-427) with the formulas and summation order of
// fill_fci_tables_kernel, so the form holds the exact split of the CSR
// values whenever the CSR is written.  Padding entries and the rows past
// nbeta are written as zeros.  Also writes lower_len.
//
// What depends on one string only comes from tables that
// fcix_fill_prep_kernel lays out with the beta string fastest, so the 32
// lanes of a slice read consecutive words: section A's codes and the split
// values of its beta doubles, section B's beta partner descriptors, and the
// split values of section C's alpha doubles (one per alpha string and
// double, read by the whole warp).  Section B's opposite-spin doubles
// <ii kk|jj ll> (ii -> jj the group's alpha single) come from a table of
// all (kk, ll) for the group's (ii, jj) that the block stages in shared
// memory, FP64 and split, double-buffered with one barrier per group.
struct FxFill {
    float4 *hi, *lo;
    const int32_t *atab, *adesc;
    const int32_t *acode; // [nbl][nbeta]: section A's string-table codes
    const float *ahi, *alo; // [nbl][nbeta]: split values of section A's beta doubles (0 elsewhere)
    const int32_t *bdesc; // [nlsp][nbeta]: section B partner q of b: kk n + ll | phase << 20; -1 b itself, -2 padding
    const float *chi, *clo; // [nalpha][nd]: split values of the alpha doubles in rank order
    const int32_t *spos, *sdb; // [nsb][nbeta]: section-A position and descriptor of beta single j of b
    int64_t spa, npk;
    int parts, aw, ns, nd, nbl, nls, nlsp, la, lc, nsb;
};

__global__ void fcix_fill_prep_kernel(StringTables A, StringTables B, int64_t nalpha, int nbeta, int n, int ns,
                                      int nd, int nbl, int nls, int nlsp, const int32_t *adesc, int32_t *acode,
                                      float *ahi, float *alo, int32_t *bdesc, float *chi, float *clo, int32_t *spos,
                                      int32_t *sdb) {
    const int64_t na_ = static_cast<int64_t>(nbl) * nbeta, nb_ = static_cast<int64_t>(nlsp) * nbeta;
    const int64_t total = na_ + nb_ + nalpha * nd;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (i < na_) {
            const int t = static_cast<int>(i / nbeta), b = static_cast<int>(i - static_cast<int64_t>(t) * nbeta);
            const int code = B.val[static_cast<int64_t>(b) * B.npad + t];
            float h = 0.0f, l = 0.0f;
            if ((code >> 20) == 2)
                split_hi_lo(B.dval[static_cast<int64_t>(b) * B.n2 + (code & 0xFFFFF)], h, l);
            if ((code >> 20) == 1) {
                const int j = code & 0xFFFFF;
                spos[static_cast<int64_t>(j) * nbeta + b] = t;
                sdb[static_cast<int64_t>(j) * nbeta + b] = B.sdesc[static_cast<int64_t>(b) * B.n1 + j];
            }
            acode[i] = code;
            ahi[i] = h;
            alo[i] = l;
        } else if (i < na_ + nb_) {
            const int64_t j = i - na_;
            const int q = static_cast<int>(j / nbeta), b = static_cast<int>(j - static_cast<int64_t>(q) * nbeta);
            int d = -2;
            if (q < nls) {
                const int code = B.subval[static_cast<int64_t>(b) * B.npad + q];
                if ((code >> 20) == 0) {
                    d = -1;
                } else {
                    const int db = B.sdesc[static_cast<int64_t>(b) * B.n1 + (code & 0xFFFFF)];
                    d = ((db & 255) * n + ((db >> 8) & 255)) | (((db >> 16) & 1) << 20);
                }
            }
            bdesc[j] = d;
        } else {
            const int64_t j = i - na_ - nb_, a = j / nd;
            const int dd = static_cast<int>(j - a * nd);
            const int ia = adesc[a * (ns + nd) + ns + dd] & 0xFFFFF;
            split_hi_lo(A.dval[a * A.n2 + ia], chi[j], clo[j]);
        }
    }
}

template<int NW>
__global__ void __launch_bounds__(512) fcix_fill_kernel(BuildParams p, StringTables A, StringTables B, FxFill F) {
    extern __shared__ __align__(16) unsigned char fx_smem[];
    const int n = p.nbasis, nn = n * n;
    double *pre = reinterpret_cast<double *>(fx_smem); // [ns]: one-electron term + alpha sums of a's singles
    double *t64 = pre + F.ns;                          // [2][nn]: <ii kk|jj ll> of the group's (ii, jj)
    float *thi = reinterpret_cast<float *>(t64 + 2 * nn), *tlo = thi + 2 * nn; // [2][nn]: its split
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nbeta = static_cast<int>(p.nbeta);
    const double *one = p.one_mo, *two = p.two_mo;
    const int64_t a = blockIdx.x / F.parts;
    const int h = static_cast<int>(blockIdx.x - a * F.parts);
    const int64_t sb = a * F.spa + h * F.spa / F.parts, se = a * F.spa + (h + 1) * F.spa / F.parts;
    uint64_t wa[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w)
        wa[w] = __ldg(A.bits + a * NW + w);
    const int32_t *AD = F.adesc + a * (F.ns + F.nd);
    // Alpha single g of row (a, b): one[ii][jj] + sum over a's occupied k of
    // (<ii k|jj k> - <ii k|k jj>), then (per row) + sum over b's occupied k of
    // <ii k|jj k>: the first part is the same for every b.
    for (int g = threadIdx.x; g < F.ns; g += blockDim.x) {
        const int da = __ldg(A.sdesc + a * A.n1 + (__ldg(AD + g) & 0xFFFFF));
        const int ii = da & 255, jj = (da >> 8) & 255;
        double v1 = __ldg(&one[ii * n + jj]);
        for (int k = next_bit<NW>(wa, 0); k >= 0; k = next_bit<NW>(wa, k + 1))
            v1 += two_mo_at(two, n, ii, k, jj, k) - two_mo_at(two, n, ii, k, k, jj);
        pre[g] = v1;
    }
    // Group g's integrals <ii kk|jj ll> for every (kk, ll) into buffer buf.
    auto stage = [&](int g, int buf) {
        const int da = __ldg(A.sdesc + a * A.n1 + (__ldg(AD + g) & 0xFFFFF));
        const int ii = da & 255, jj = (da >> 8) & 255;
        for (int idx = threadIdx.x; idx < nn; idx += blockDim.x) {
            const int kk = idx / n, ll = idx - kk * n;
            const double v = two_mo_at(two, n, ii, kk, jj, ll);
            t64[buf * nn + idx] = v;
            split_hi_lo(v, thi[buf * nn + idx], tlo[buf * nn + idx]);
        }
    };
    if (F.ns > 0)
        stage(0, 0);
    __syncthreads();
    const int64_t s = sb + warp;
    const bool active = s < se; // every warp takes part in the barriers below
    const int bb = active ? static_cast<int>((s - a * F.spa) * 32) + lane : 0;
    const bool valid = active && bb < nbeta;
    const int b = valid ? bb : nbeta - 1;
    const int64_t row = a * nbeta + b;
    uint64_t wb[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w)
        wb[w] = __ldg(B.bits + static_cast<int64_t>(b) * NW + w);
    float4 *hp = F.hi + (active ? s : 0) * F.npk * 32 + lane, *lp = F.lo + (active ? s : 0) * F.npk * 32 + lane;
    // One packet: entries t0 .. t0 + 3, value(t) returning (high, low).
    auto packet = [&](int t0, auto value) {
        float h4[4], l4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float2 v = value(t0 + u);
            h4[u] = valid ? v.x : 0.0f;
            l4[u] = valid ? v.y : 0.0f;
        }
        hp[32 * static_cast<int64_t>(t0 >> 2)] = make_float4(h4[0], h4[1], h4[2], h4[3]);
        lp[32 * static_cast<int64_t>(t0 >> 2)] = make_float4(l4[0], l4[1], l4[2], l4[3]);
    };
    auto split2 = [](double v) {
        float hv, lv;
        split_hi_lo(v, hv, lv);
        return make_float2(hv, lv);
    };
    if (active) {
        // Section A: the alpha string itself with every beta partner of b.
        // The beta singles sit at different positions in different lanes'
        // rows: they are written as zeros here and then one single at a time
        // in every lane (no lane waits on another lane's FP64 sums).
        const float2 dsp = split2(p.diag[row]); // fci_diag_kernel ran first
        auto value_a = [&](int t) -> float2 {
            if (t >= F.nbl)
                return make_float2(0.0f, 0.0f);
            const int64_t at = static_cast<int64_t>(t) * nbeta + b;
            const int ty = __ldg(F.acode + at) >> 20;
            if (ty == 0)
                return dsp;
            return ty == 2 ? make_float2(__ldg(F.ahi + at), __ldg(F.alo + at)) : make_float2(0.0f, 0.0f);
        };
        for (int t = 0; t < F.la; t += 4)
            packet(t, value_a);
        float *hf = reinterpret_cast<float *>(F.hi), *lf = reinterpret_cast<float *>(F.lo);
        for (int j = 0; j < F.nsb; ++j) {
            // Beta single j, ii -> jj (0-1 excitation).
            const int t = __ldg(F.spos + static_cast<int64_t>(j) * nbeta + b);
            const int db = __ldg(F.sdb + static_cast<int64_t>(j) * nbeta + b);
            const int ii = db & 255, jj = (db >> 8) & 255;
            double v1 = __ldg(&one[ii * n + jj]);
            for (int k = next_bit<NW>(wa, 0); k >= 0; k = next_bit<NW>(wa, k + 1))
                v1 += two_mo_at(two, n, ii, k, jj, k);
            for (int k = next_bit<NW>(wb, 0); k >= 0; k = next_bit<NW>(wb, k + 1))
                v1 += two_mo_at(two, n, ii, k, jj, k) - two_mo_at(two, n, ii, k, k, jj);
            if (valid) {
                const int64_t at = ((s * F.npk + (t >> 2)) * 32 + lane) * 4 + (t & 3);
                split_hi_lo(apply_phase((db >> 16) & 1 ? -1 : 1, v1), hf[at], lf[at]);
            }
        }
    }
    // Section B: each alpha single with {b} + the beta singles of b.
    int tb = F.la;
    for (int g = 0; g < F.ns; ++g, tb += F.nlsp) {
        if (g + 1 < F.ns)
            stage(g + 1, (g + 1) & 1); // last read in group g - 1, before the barrier below
        if (active) {
            const int da = __ldg(A.sdesc + a * A.n1 + (__ldg(AD + g) & 0xFFFFF));
            const int pha = (da >> 16) & 1;
            const double *T64 = t64 + (g & 1) * nn;
            const float *Th = thi + (g & 1) * nn, *Tl = tlo + (g & 1) * nn;
            // Alpha single ii -> jj (1-0 excitation), the group's entry for b
            // itself: computed in every lane, used where the partner is b.
            double v1 = pre[g];
            for (int k = next_bit<NW>(wb, 0); k >= 0; k = next_bit<NW>(wb, k + 1))
                v1 += T64[k * n + k];
            const float2 selfv = split2(apply_phase(pha ? -1 : 1, v1));
            auto value_b = [&](int t) -> float2 {
                const int d = __ldg(F.bdesc + static_cast<int64_t>(t - tb) * nbeta + b);
                if (d == -2)
                    return make_float2(0.0f, 0.0f);
                if (d == -1)
                    return selfv;
                // Opposite-spin double: alpha ii -> jj, beta kk -> ll; the
                // split of -v is (-high, -low).
                const int off = d & 0xFFFFF;
                const float hv = Th[off], lv = Tl[off];
                return ((d >> 20) ^ pha) ? make_float2(-hv, -lv) : make_float2(hv, lv);
            };
            for (int t = tb; t < tb + F.nlsp; t += 4)
                packet(t, value_b);
        }
        __syncthreads();
    }
    if (!active)
        return;
    // Section C: each alpha double with b.
    const int tc = tb;
    const float *CH = F.chi + a * F.nd, *CL = F.clo + a * F.nd;
    auto value_c = [&](int t) -> float2 {
        const int d = t - tc;
        return d < F.nd ? make_float2(__ldg(CH + d), __ldg(CL + d)) : make_float2(0.0f, 0.0f);
    };
    for (int t = tc; t < tc + F.lc; t += 4)
        packet(t, value_c);
    if (valid && p.lower_len)
        p.lower_len[row] = __ldg(F.atab + a * F.aw + F.aw - 1) + __ldg(B.self + b) + 1;
}

// Insert every determinant index into the table (linear probing).
template<int NWT>
__global__ void table_insert_kernel(int32_t *slots, uint64_t mask, const uint64_t *dets,
                                    int64_t ndet, int *error) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= ndet)
        return;
    uint64_t key[NWT];
#pragma unroll
    for (int w = 0; w < NWT; ++w)
        key[w] = dets[i * NWT + w];
    uint64_t s = hash_words(key, NWT) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        const int32_t prev = atomicCAS(&slots[s], -1, static_cast<int32_t>(i));
        if (prev == -1)
            return;
        bool eq = true;
#pragma unroll
        for (int w = 0; w < NWT; ++w)
            eq &= (dets[static_cast<int64_t>(prev) * NWT + w] == key[w]);
        if (eq) {
            // Duplicate determinant: keep the smaller (first-inserted) index.
            atomicMin(&slots[s], static_cast<int32_t>(i));
            return;
        }
        s = (s + 1) & mask;
    }
    atomicExch(error, 2);
}

// ---------------- exclusive scan of int64 counts ----------------

constexpr int kScanBlock = 1024;

__global__ void scan_block_sums(const int64_t *in, int64_t n, int64_t *sums) {
    __shared__ int64_t red[32];
    const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kScanBlock;
    int64_t v = 0;
    for (int t = threadIdx.x; t < kScanBlock; t += blockDim.x)
        if (i0 + t < n)
            v += in[i0 + t];
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0)
            sums[blockIdx.x] = v;
    }
}

// Exclusive scan of the block sums in place, single block.
__global__ void scan_sums_serial(int64_t *sums, int64_t nblocks, int64_t *total) {
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    int64_t acc = 0;
    for (int64_t b = 0; b < nblocks; ++b) {
        const int64_t v = sums[b];
        sums[b] = acc;
        acc += v;
    }
    *total = acc;
}

// out[i] = sums[block] + exclusive scan within the block; out has n + 1 slots.
__global__ void scan_apply(const int64_t *in, int64_t n, const int64_t *sums, const int64_t *total,
                           int64_t *out) {
    __shared__ int64_t buf[kScanBlock];
    const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kScanBlock;
    for (int t = threadIdx.x; t < kScanBlock; t += blockDim.x)
        buf[t] = (i0 + t < n) ? in[i0 + t] : 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t acc = sums[blockIdx.x];
        for (int t = 0; t < kScanBlock; ++t) {
            const int64_t v = buf[t];
            buf[t] = acc;
            acc += v;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kScanBlock; t += blockDim.x)
        if (i0 + t < n)
            out[i0 + t] = buf[t];
    if (blockIdx.x == 0 && threadIdx.x == 0)
        out[n] = *total;
}

// ---------------- GenCI in the reference's own row loop ----------------
//
// GenCIWfn inherits Wfn::init's nvir = 2 * nbasis - nocc (pyci/src/wfn.cpp:62),
// although nbasis already counts spin-orbitals, and add_row<GenCIWfn>
// (pyci/src/sparseop.cpp:429-502) loops j < wfn.nvir over a virs buffer whose
// entries past the true virtual count stay 0 (zero-initialised at
// pyci/src/sparseop.cpp:190).  The loop therefore also "excites" into orbital
// 0, and its excite_det restores (clear i, set a) can drop orbital 0 from the
// working determinant for the rest of the row.  These kernels replay that
// loop step by step (one thread per row) so the matrix matches the
// reference's entry for entry; PYCI_BUILD_GENCI_EXACT selects the
// Slater-Condon rules over the true virtuals instead.

__device__ __forceinline__ void excite_ref(uint64_t *det, int i, int a) {
    det[i >> 6] &= ~(1ULL << (i & 63));
    det[a >> 6] |= 1ULL << (a & 63);
}

__device__ __forceinline__ bool keep_ref(const BuildParams &p, int64_t idet, int64_t jdet) {
    const int64_t jmin = p.symmetric ? idet : INT64_MAX;
    return (jdet != -1) && (jdet < jmin) && (jdet < row_limit(p, idet));
}

// Replays one row; calls emit(col, value) for every appended entry.
template<int NW, bool VALUES, class Emit>
__device__ void genci_ref_row(const BuildParams &p, int64_t idet, Emit emit) {
    const int n = p.nbasis;
    const double *one = p.one_mo, *two = p.two_mo;
    uint64_t rdet[NW], det[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w)
        rdet[w] = det[w] = p.dets[idet * NW + w];
    int16_t occs[kMaxOcc], virs[2 * kMaxVir];
    const int no = occ_list<NW>(rdet, occs);
    const int nv_true = vir_list<NW>(rdet, n, virs);
    const int nv = 2 * n - p.nocc_up - p.nocc_dn;
    for (int j = nv_true; j < nv; ++j)
        virs[j] = 0;
    double val2 = 0.0;
    for (int i = 0; i < no; ++i) {
        const int ii = occs[i];
        if (VALUES) {
            val2 += __ldg(&one[(n + 1) * ii]);
            for (int k = i + 1; k < no; ++k) {
                const int kk = occs[k];
                val2 += two_mo_at(two, n, ii, kk, ii, kk) - two_mo_at(two, n, ii, kk, kk, ii);
            }
        }
        for (int j = 0; j < nv; ++j) {
            const int jj = virs[j];
            excite_ref(det, ii, jj);
            int64_t jdet = p.table.find<NW>(det);
            if (keep_ref(p, idet, jdet)) {
                double v = 0.0;
                if (VALUES) {
                    double v1 = __ldg(&one[n * ii + jj]);
                    for (int k = 0; k < no; ++k) {
                        const int kk = occs[k];
                        v1 += two_mo_at(two, n, ii, kk, jj, kk) - two_mo_at(two, n, ii, kk, kk, jj);
                    }
                    v = apply_phase(phase_single<NW>(rdet, ii, jj), v1);
                }
                emit(jdet, v);
            }
            for (int k = i + 1; k < no; ++k) {
                const int kk = occs[k];
                for (int l = j + 1; l < nv; ++l) {
                    const int ll = virs[l];
                    excite_ref(det, kk, ll);
                    jdet = p.table.find<NW>(det);
                    if (keep_ref(p, idet, jdet))
                        emit(jdet, VALUES ? apply_phase(phase_double<NW>(rdet, ii, kk, jj, ll),
                                                        two_mo_at(two, n, ii, kk, jj, ll) - two_mo_at(two, n, ii, kk, ll, jj))
                                          : 0.0);
                    excite_ref(det, ll, kk);
                }
            }
            excite_ref(det, jj, ii);
        }
    }
    if (idet < row_limit(p, idet))
        emit(idet, val2);
}

template<int NW>
__global__ void genci_ref_count_kernel(BuildParams p) {
    const int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (row >= p.nrow)
        return;
    int64_t cnt = 0;
    genci_ref_row<NW, false>(p, row, [&](int64_t, double) { ++cnt; });
    p.counts[row] = cnt;
}

// One block per row: thread 0 replays the row into shared memory, then the
// block sorts it by column and writes it out.
template<int NW>
__global__ void __launch_bounds__(256) genci_ref_fill_kernel(BuildParams p, int64_t row0, int cap) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *sval = reinterpret_cast<double *>(smem);
    int32_t *skey = reinterpret_cast<int32_t *>(smem + sizeof(double) * cap);
    const int64_t row = row0 + blockIdx.x;
    if (row >= p.nrow)
        return;
    for (int c = threadIdx.x; c < cap; c += blockDim.x) {
        skey[c] = kSentinel;
        sval[c] = 0.0;
    }
    __syncthreads();
    const int64_t start = p.rowptr[row];
    const int len = static_cast<int>(p.rowptr[row + 1] - start);
    if (threadIdx.x == 0) {
        int t = 0;
        genci_ref_row<NW, true>(p, row, [&](int64_t col, double v) {
            if (t < cap) {
                skey[t] = static_cast<int32_t>(col);
                sval[t] = v;
            }
            ++t;
        });
        if (t != len)
            atomicExch(p.error, 3);
    }
    __syncthreads();
    for (int size = 2; size <= cap; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < cap / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool up = ((lo & size) == 0);
                const int32_t klo = skey[lo], khi = skey[hi];
                if ((klo > khi) == up) {
                    skey[lo] = khi;
                    skey[hi] = klo;
                    const double vlo = sval[lo];
                    sval[lo] = sval[hi];
                    sval[hi] = vlo;
                }
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < len && t < cap; t += blockDim.x) {
        p.cols[start + t] = skey[t];
        p.vals[start + t] = sval[t];
        if (skey[t] == row)
            p.diag[row] = sval[t];
    }
    if (threadIdx.x == 0 && p.lower_len)
        p.lower_len[row] = len;
}

__global__ void max_kernel(const int64_t *v, int64_t n, unsigned long long *out) {
    unsigned long long m = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        m = max(m, static_cast<unsigned long long>(v[i]));
    for (int o = 16; o > 0; o >>= 1)
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(out, m);
}

// rowptr[i] = i * len (every row of a full space keeps all its candidates).
__global__ void uniform_rowptr_kernel(int64_t *rowptr, int64_t nrow, int64_t len) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i <= nrow;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        rowptr[i] = i * len;
}

__global__ void widen_kernel(const int32_t *in, int64_t *out, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = in[i];
}

} // namespace pyci_gpu

using namespace pyci_gpu;

int64_t host_binomial(int64_t n, int64_t k) {
    if (k < 0 || n < 0 || k > n)
        return 0;
    if (k == 0 || k == n)
        return 1;
    if (k > n / 2)
        k = n - k;
    __int128 b = 1;
    for (int64_t d = 1; d <= k; ++d) {
        b = b * (n - k + d) / d;
        if (b > INT64_MAX)
            return INT64_MAX;
    }
    return static_cast<int64_t>(b);
}

// Exclusive scan of counts[n] into out[n + 1] on `stream`.
int device_exclusive_scan(const int64_t *counts, int64_t n, int64_t *out, cudaStream_t stream) {
    const int64_t nblocks = (n + kScanBlock - 1) / kScanBlock;
    int64_t *sums = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(&sums, sizeof(int64_t) * (nblocks + 1), stream));
    if (nblocks > 0) {
        scan_block_sums<<<nblocks, 256, 0, stream>>>(counts, n, sums), ::pyci_gpu::note_launch();
        scan_sums_serial<<<1, 32, 0, stream>>>(sums, nblocks, sums + nblocks), ::pyci_gpu::note_launch();
        scan_apply<<<nblocks, 256, 0, stream>>>(counts, n, sums, sums + nblocks, out), ::pyci_gpu::note_launch();
    } else {
        PYCI_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int64_t), stream));
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    PYCI_CUDA_TRY(cudaFreeAsync(sums, stream));
    return PYCI_GPU_OK;
}

// Open-addressing table over ndet determinants of nwords (1, 2, 4 or 8)
// words at d_dets: *slots (2^k >= 2 ndet int32 slots, from the stream's pool;
// the caller frees it) and *mask = 2^k - 1.  Duplicates keep the smallest
// index.  Table overflow sets *d_err = 2.
int det_table_build(const uint64_t *d_dets, int64_t ndet, int nwords, cudaStream_t st, int *d_err,
                    int32_t **slots_out, uint64_t *mask_out) {
    uint64_t cap = 16;
    while (cap < static_cast<uint64_t>(2 * ndet))
        cap <<= 1;
    int32_t *slots = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(&slots, sizeof(int32_t) * cap, st));
    PYCI_CUDA_TRY(cudaMemsetAsync(slots, 0xff, sizeof(int32_t) * cap, st));
    const unsigned blocks = static_cast<unsigned>((ndet + 255) / 256);
    if (blocks) {
        switch (nwords) {
        case 1: table_insert_kernel<1><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, ndet, d_err); break;
        case 2: table_insert_kernel<2><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, ndet, d_err); break;
        case 4: table_insert_kernel<4><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, ndet, d_err); break;
        case 8: table_insert_kernel<8><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, ndet, d_err); break;
        default:
            cudaFreeAsync(slots, st);
            set_error("unsupported determinant width");
            return PYCI_GPU_EUNSUPPORTED;
        }
        ::pyci_gpu::note_launch();
        PYCI_CUDA_TRY(cudaGetLastError());
    }
    *slots_out = slots;
    *mask_out = cap - 1;
    return PYCI_GPU_OK;
}

namespace {

struct DeviceBuffers {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit DeviceBuffers(cudaStream_t st) : s(st) {}
    template<typename T>
    cudaError_t alloc(T **p, size_t count) {
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(p), sizeof(T) * (count ? count : 1), s);
        if (e == cudaSuccess)
            ptrs.push_back(*p);
        return e;
    }
    ~DeviceBuffers() {
        for (void *p : ptrs)
            cudaFreeAsync(p, s);
    }
};

int pick_nw(int64_t nbasis) {
    if (nbasis <= 64)
        return 1;
    if (nbasis <= 128)
        return 2;
    if (nbasis <= 256)
        return 4;
    return 0;
}

// Sets up the implicit-column form of a full FullCI space when its beta
// string count pads to a multiple of 32 with at most 1/4 extra rows (the
// padding rows are streamed as zeros, still fewer bytes than int32 columns):
// the tables and the value arrays (csr->fx_*), which fcix_fill_kernel then
// writes.  *adesc: the per-alpha-string codes the fill reads (the caller
// frees it).  Leaves csr->fx_hi null when the space does not qualify.
int fcix_tables(pyci_gpu_ctx *ctx, pyci_gpu_csr *csr, const StringTables &TA, const StringTables &TB, int64_t nalpha,
                int64_t nbeta, int na, int nbl, int grp1, int64_t len, int32_t **adesc) {
    cudaStream_t st = ctx->stream;
    *adesc = nullptr;
    const int64_t nbp = (nbeta + 31) / 32 * 32;
    const int ns = TA.n1, nd = TA.n2;
    if (nbeta < 32 || nbeta >= 65536 || 4 * (nbp - nbeta) > nbeta || len <= 0 || len > (1 << 20) ||
        !csr->symmetric || na != 1 + ns + nd ||
        len != static_cast<int64_t>(nbl) + static_cast<int64_t>(ns) * grp1 + nd)
        return PYCI_GPU_OK;
    auto up4 = [](int64_t v) { return (v + 3) / 4 * 4; };
    // Sections padded to multiples of 4 entries, and each group of section B
    // too (a 4-entry packet never spans two alpha targets).
    const int la = static_cast<int>(up4(nbl)), lb = static_cast<int>(ns * up4(grp1)), lc = static_cast<int>(up4(nd));
    const int w = 2 * (ns + nd) + 1;
    const size_t sa = sizeof(int32_t) * nalpha * w, sf = sizeof(int32_t) * nbl * nbeta,
                 ss = sizeof(int32_t) * grp1 * nbeta;
    const int64_t npk = (la + lb + lc) / 4;
    const size_t nval = static_cast<size_t>(nalpha) * (nbp / 32) * npk * 128;
    int32_t *atab = nullptr, *bfull = nullptr, *bsub = nullptr, *codes = nullptr;
    uint16_t *bq = nullptr;
    float *hi = nullptr, *lo = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&atab), sa, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&bfull), sf, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&bsub), ss, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&bq), sizeof(uint16_t) * la * nbeta, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&codes), sizeof(int32_t) * nalpha * std::max(ns + nd, 1), st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&hi), sizeof(float) * nval, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&lo), sizeof(float) * nval, st);
    if (e != cudaSuccess) {
        for (void *q : {static_cast<void *>(atab), static_cast<void *>(bfull), static_cast<void *>(bsub),
                        static_cast<void *>(bq), static_cast<void *>(codes), static_cast<void *>(hi),
                        static_cast<void *>(lo)})
            if (q)
                cudaFreeAsync(q, st);
        return cuda_status(e, "cudaMallocAsync (implicit-column form)");
    }
    const int64_t total = nalpha + (static_cast<int64_t>(nbl) + grp1 + la) * nbeta;
    fcix_tables_kernel<<<static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 4096)), 256, 0, st>>>(
        TA, TB, nalpha, nbeta, na, nbl, grp1, ns, nd, la, atab, bfull, bsub, bq, codes);
    ::pyci_gpu::note_launch();
    csr->fx_nalpha = nalpha;
    csr->fx_nbeta = nbeta;
    csr->fx_nbp = nbp;
    csr->fx_ns = ns;
    csr->fx_nd = nd;
    csr->fx_nlb = nbl;
    csr->fx_nls = grp1;
    csr->fx_la = la;
    csr->fx_lb = lb;
    csr->fx_lc = lc;
    csr->fx_npk = npk;
    csr->fx_atab = atab;
    csr->fx_bfull = bfull;
    csr->fx_bsub = bsub;
    csr->fx_bq = bq;
    csr->fx_hi = hi;
    csr->fx_lo = lo;
    *adesc = codes;
    return PYCI_GPU_OK;
}

// Lay out fcix_fill_kernel's per-string tables (fcix_fill_prep_kernel), then
// launch it over every slice of the implicit-column form.
template<int NW>
int fcix_fill(pyci_gpu_ctx *ctx, pyci_gpu_csr *csr, const BuildParams &p, const StringTables &TA,
              const StringTables &TB, const int32_t *adesc) {
    cudaStream_t st = ctx->stream;
    FxFill F{};
    F.hi = reinterpret_cast<float4 *>(csr->fx_hi);
    F.lo = reinterpret_cast<float4 *>(csr->fx_lo);
    F.atab = csr->fx_atab;
    F.adesc = adesc;
    F.spa = csr->fx_nbp / 32;
    F.npk = csr->fx_npk;
    F.parts = static_cast<int>((F.spa + 7) / 8); // blocks of <= 8 warps: more of them resident (registers)
    F.aw = fx_atab_width(csr);
    F.ns = csr->fx_ns;
    F.nd = csr->fx_nd;
    F.nbl = csr->fx_nlb;
    F.nls = csr->fx_nls;
    F.nlsp = (csr->fx_nls + 3) / 4 * 4;
    F.la = csr->fx_la;
    F.lc = csr->fx_lc;
    const int n = p.nbasis, nbeta = static_cast<int>(csr->fx_nbeta);
    const int warps = static_cast<int>((F.spa + F.parts - 1) / F.parts);
    const size_t smem = sizeof(double) * std::max(F.ns, 1) + static_cast<size_t>(n) * n * 2 * (sizeof(double) + 2 * sizeof(float));
    if (smem > 48 * 1024) {
        set_error("implicit-column fill: %d orbitals and %d alpha singles exceed its shared memory", n, F.ns);
        return PYCI_GPU_EUNSUPPORTED;
    }
    const int64_t na_ = static_cast<int64_t>(F.nbl) * nbeta, nb_ = static_cast<int64_t>(F.nlsp) * nbeta,
                  nc_ = csr->fx_nalpha * std::max(F.nd, 1);
    F.nsb = TB.n1;
    const int64_t ns_ = static_cast<int64_t>(std::max(F.nsb, 1)) * nbeta;
    int32_t *acode = nullptr, *bdesc = nullptr, *sps = nullptr;
    float *ahl = nullptr, *chl = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&acode), sizeof(int32_t) * na_, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&sps), sizeof(int32_t) * 2 * ns_, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&ahl), sizeof(float) * 2 * na_, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&bdesc), sizeof(int32_t) * nb_, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&chl), sizeof(float) * 2 * nc_, st);
    if (e == cudaSuccess) {
        const int64_t total = na_ + nb_ + csr->fx_nalpha * F.nd;
        fcix_fill_prep_kernel<<<static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 8192)), 256, 0, st>>>(
            TA, TB, csr->fx_nalpha, nbeta, n, F.ns, F.nd, F.nbl, F.nls, F.nlsp, adesc, acode, ahl, ahl + na_, bdesc,
            chl, chl + nc_, sps, sps + ns_);
        ::pyci_gpu::note_launch();
        F.spos = sps;
        F.sdb = sps + ns_;
        F.acode = acode;
        F.ahi = ahl;
        F.alo = ahl + na_;
        F.bdesc = bdesc;
        F.chi = chl;
        F.clo = chl + nc_;
        fcix_fill_kernel<NW><<<static_cast<unsigned>(csr->fx_nalpha * F.parts), 32 * warps, smem, st>>>(p, TA, TB, F);
        ::pyci_gpu::note_launch();
        e = cudaGetLastError();
    }
    for (void *q : {static_cast<void *>(acode), static_cast<void *>(ahl), static_cast<void *>(bdesc),
                    static_cast<void *>(chl), static_cast<void *>(sps)})
        if (q)
            cudaFreeAsync(q, st);
    if (e != cudaSuccess)
        return cuda_status(e, "implicit-column fill");
    return PYCI_GPU_OK;
}

// Device arrays of the CSR entries (int32 columns, FP64 values) for
// csr->nnz entries.
int csr_alloc_entries(pyci_gpu_csr *csr) {
    cudaStream_t st = csr->ctx->stream;
    const int64_t nnz = csr->nnz ? csr->nnz : 1;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->cols), sizeof(int32_t) * nnz, st));
    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&csr->vals), sizeof(double) * nnz, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(csr->cols, st);
        csr->cols = nullptr;
        return cuda_status(e, "cudaMallocAsync (CSR entries)");
    }
    return PYCI_GPU_OK;
}

// Reference-layout row pointers of a symmetric operator: the prefix sums of
// lower_len, and nnz_ref.
int ref_rowptr_from_lower_len(pyci_gpu_csr *csr) {
    cudaStream_t st = csr->ctx->stream;
    int64_t *lens64 = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&lens64), sizeof(int64_t) * std::max<int64_t>(csr->nrow, 1), st));
    if (csr->nrow > 0)
        widen_kernel<<<static_cast<unsigned>(std::min<int64_t>((csr->nrow + 255) / 256, 1 << 16)), 256, 0, st>>>(
            csr->lower_len, lens64, csr->nrow), ::pyci_gpu::note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&csr->ref_rowptr), sizeof(int64_t) * (csr->nrow + 1), st);
    int rc = e == cudaSuccess ? device_exclusive_scan(lens64, csr->nrow, csr->ref_rowptr, st)
                              : cuda_status(e, "reference row pointers");
    if (!rc) {
        e = cudaMemcpyAsync(&csr->nnz_ref, csr->ref_rowptr + csr->nrow, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            rc = cuda_status(e, "reference row pointers");
    }
    cudaFreeAsync(lens64, st);
    return rc;
}

// The sorted FullCI row fill over every row (the diagonal must be in p.diag).
template<int NW>
int launch_fci_fill(pyci_gpu_ctx *ctx, const BuildParams &p, const StringTables &TA, const StringTables &TB, int na,
                    int nsg) {
    cudaStream_t st = ctx->stream;
    const size_t per_warp = (sizeof(RowState) + sizeof(double) * nsg + sizeof(int) * na + 15) & ~static_cast<size_t>(15);
    const size_t dsm = per_warp * kFillRowsPerBlock;
    if (dsm > 48 * 1024)
        PYCI_CUDA_TRY(cudaFuncSetAttribute(fill_fci_tables_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(dsm)));
    const int64_t rows_per_launch = (static_cast<int64_t>(1) << 20) * kFillRowsPerBlock;
    for (int64_t r0 = 0; r0 < p.nrow; r0 += rows_per_launch) {
        const int64_t nr = (p.nrow - r0 < rows_per_launch) ? p.nrow - r0 : rows_per_launch;
        const unsigned nb = static_cast<unsigned>((nr + kFillRowsPerBlock - 1) / kFillRowsPerBlock);
        fill_fci_tables_kernel<NW><<<nb, 32 * kFillRowsPerBlock, dsm, st>>>(p, r0, TA, TB, na, nsg),
            ::pyci_gpu::note_launch();
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

// The full-DOCI row fill over every row (the diagonal must be in p.diag).
template<int NW>
int launch_doci_fill(pyci_gpu_ctx *ctx, const BuildParams &p) {
    const int64_t rows_per_block = 8 * kDociRowsPerWarp;
    const int64_t rows_per_launch = static_cast<int64_t>(1) << 30;
    for (int64_t r0 = 0; r0 < p.nrow; r0 += rows_per_launch) {
        const int64_t nr = std::min<int64_t>(p.nrow - r0, rows_per_launch);
        fill_doci_warp_kernel<NW><<<static_cast<unsigned>((nr + rows_per_block - 1) / rows_per_block), 256, 0,
                                    ctx->stream>>>(p, r0),
            ::pyci_gpu::note_launch();
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

// What a row fill needs to write the CSR later: the build's parameters and
// device copies of what they point to (FullCI: the string tables and the
// integrals; DOCI: the binomial table, the pair integrals and an error flag).
struct DeferredCsr {
    BuildParams p{};
    StringTables TA{}, TB{};
    int kind = 0, na = 0, nsg = 0, nw = 1;
    std::vector<void *> mem; // device arrays owned here
};

// Keeps the string tables (taking the arrays in `mem`) so that
// csr_materialize can write the CSR; the caller has written the
// implicit-column form and the diagonal.
int defer_csr(pyci_gpu_csr *csr, const BuildParams &p, const StringTables &TA, const StringTables &TB, int na,
              int nsg, int nw, std::vector<void *> &mem) {
    cudaStream_t st = csr->ctx->stream;
    DeferredCsr *d = new (std::nothrow) DeferredCsr();
    if (!d) {
        set_error("out of host memory");
        return PYCI_GPU_ENOMEM;
    }
    const int64_t n = p.nbasis, n2 = n * n, n4 = n2 * n2;
    double *one = nullptr, *two = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&one), sizeof(double) * n2, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&two), sizeof(double) * n4, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(one, p.one_mo, sizeof(double) * n2, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(two, p.two_mo, sizeof(double) * n4, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        if (one)
            cudaFreeAsync(one, st);
        if (two)
            cudaFreeAsync(two, st);
        delete d;
        return cuda_status(e, "deferred CSR (integrals)");
    }
    d->p = p;
    d->p.one_mo = one;
    d->p.two_mo = two;
    // Only the tables, the integrals and the row arrays serve the sorted fill.
    d->p.binom = nullptr;
    d->p.dets = nullptr;
    d->p.h = d->p.v = d->p.w = nullptr;
    d->p.counts = nullptr;
    d->p.error = nullptr;
    d->p.cols = nullptr;
    d->p.vals = nullptr;
    d->p.lower_len = nullptr;
    d->TA = TA;
    d->TB = TB;
    d->kind = PYCI_WFN_FULLCI;
    d->na = na;
    d->nsg = nsg;
    d->nw = nw;
    d->mem = mem;
    d->mem.push_back(one);
    d->mem.push_back(two);
    mem.clear();
    csr->deferred = d;
    return PYCI_GPU_OK;
}

// Keeps what fill_doci_warp_kernel reads (the diagonal is written) so that
// csr_materialize can write the CSR of a full DOCI space.
int defer_csr_doci(pyci_gpu_csr *csr, const BuildParams &p, int nw) {
    cudaStream_t st = csr->ctx->stream;
    DeferredCsr *d = new (std::nothrow) DeferredCsr();
    if (!d) {
        set_error("out of host memory");
        return PYCI_GPU_ENOMEM;
    }
    const int64_t n = p.nbasis, nb = (n + 1) * p.ldk;
    int64_t *binom = nullptr;
    double *v = nullptr;
    int *err = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&binom), sizeof(int64_t) * nb, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&v), sizeof(double) * n * n, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&err), sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(binom, p.binom, sizeof(int64_t) * nb, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(v, p.v, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e != cudaSuccess) {
        for (void *q : {static_cast<void *>(binom), static_cast<void *>(v), static_cast<void *>(err)})
            if (q)
                cudaFreeAsync(q, st);
        delete d;
        return cuda_status(e, "deferred CSR (DOCI tables)");
    }
    d->p = p;
    d->p.binom = binom;
    d->p.v = v;
    d->p.error = err;
    d->p.one_mo = d->p.two_mo = d->p.h = d->p.w = nullptr;
    d->p.dets = nullptr;
    d->p.counts = nullptr;
    d->p.cols = nullptr;
    d->p.vals = nullptr;
    d->p.lower_len = nullptr;
    d->kind = PYCI_WFN_DOCI;
    d->nw = nw;
    d->mem = {binom, v, err};
    csr->deferred = d;
    return PYCI_GPU_OK;
}

} // namespace

void csr_deferred_free(pyci_gpu_csr *csr) {
    if (!csr || !csr->deferred)
        return;
    auto *d = static_cast<DeferredCsr *>(csr->deferred);
    for (void *m : d->mem)
        cudaFreeAsync(m, csr->ctx->stream);
    delete d;
    csr->deferred = nullptr;
}

int csr_materialize(const pyci_gpu_csr *ccsr) {
    pyci_gpu_csr *csr = const_cast<pyci_gpu_csr *>(ccsr);
    if (!csr || !csr->deferred)
        return PYCI_GPU_OK;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (!csr->deferred)
        return PYCI_GPU_OK;
    auto *d = static_cast<DeferredCsr *>(csr->deferred);
    int rc = csr_alloc_entries(csr);
    if (rc)
        return rc;
    BuildParams p = d->p;
    p.rowptr = csr->rowptr;
    p.diag = csr->diag;
    p.cols = csr->cols;
    p.vals = csr->vals;
    if (d->kind == PYCI_WFN_DOCI) {
        // The DOCI fill also writes lower_len; the reference-layout row
        // pointers follow from it.
        p.lower_len = csr->lower_len;
        switch (d->nw) {
        case 1: rc = launch_doci_fill<1>(csr->ctx, p); break;
        case 2: rc = launch_doci_fill<2>(csr->ctx, p); break;
        default: rc = launch_doci_fill<4>(csr->ctx, p); break;
        }
        if (!rc && csr->symmetric && !csr->ref_rowptr)
            rc = ref_rowptr_from_lower_len(csr);
        int herr = 0;
        if (!rc) {
            cudaError_t e = cudaMemcpyAsync(&herr, p.error, sizeof(int), cudaMemcpyDeviceToHost, csr->ctx->stream);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(csr->ctx->stream);
            if (e != cudaSuccess)
                rc = cuda_status(e, "deferred CSR");
            else if (herr) {
                set_error("internal inconsistency in the CSR build (code %d)", herr);
                rc = PYCI_GPU_ECUDA;
            }
        }
    } else {
        p.lower_len = nullptr; // written with the implicit-column form
        switch (d->nw) {
        case 1: rc = launch_fci_fill<1>(csr->ctx, p, d->TA, d->TB, d->na, d->nsg); break;
        case 2: rc = launch_fci_fill<2>(csr->ctx, p, d->TA, d->TB, d->na, d->nsg); break;
        default: rc = launch_fci_fill<4>(csr->ctx, p, d->TA, d->TB, d->na, d->nsg); break;
        }
    }
    if (rc) {
        cudaFreeAsync(csr->cols, csr->ctx->stream);
        cudaFreeAsync(csr->vals, csr->ctx->stream);
        csr->cols = nullptr;
        csr->vals = nullptr;
        return rc;
    }
    csr_deferred_free(csr);
    return PYCI_GPU_OK;
}

namespace {

template<int NW>
int run_build(pyci_gpu_ctx *ctx, BuildParams &p, pyci_gpu_csr *csr, int cap, int64_t uniform_len,
              bool sorted_fci, bool warp_doci) {
    cudaStream_t st = ctx->stream;
    const int64_t chunk = 1 << 20; // rows per launch (grid.x limit is generous; keeps launches short)
    // Shared-memory scratch: rank cache + binomial table (see setup_scratch).
    const size_t scratch = ((static_cast<size_t>(p.ncache) * sizeof(int32_t) + 7) & ~static_cast<size_t>(7)) +
                           static_cast<size_t>(p.binom_smem) * sizeof(int64_t);
    if (scratch > 48 * 1024)
        PYCI_CUDA_TRY(cudaFuncSetAttribute(count_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(scratch)));
    if (uniform_len > 0) {
        // Full space, fresh build, nrow = ncol = ndet: every candidate and the
        // diagonal are kept, so every row has the same length.
        uniform_rowptr_kernel<<<static_cast<unsigned>(std::min<int64_t>((p.nrow + 256) / 256, 1 << 16)), 256, 0, st>>>(
            csr->rowptr, p.nrow, uniform_len), ::pyci_gpu::note_launch();
    } else {
        for (int64_t r0 = 0; r0 < p.nrow; r0 += chunk) {
            const int64_t nb = (p.nrow - r0 < chunk) ? p.nrow - r0 : chunk;
            count_kernel<NW><<<static_cast<unsigned>(nb), 256, scratch, st>>>(p, r0), ::pyci_gpu::note_launch();
        }
        PYCI_CUDA_TRY(cudaGetLastError());
        int rc = device_exclusive_scan(p.counts, p.nrow, csr->rowptr, st);
        if (rc)
            return rc;
    }
    int64_t nnz = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(&nnz, csr->rowptr + p.nrow, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    csr->nnz = nnz;
    PYCI_CUDA_TRY(cudaMemsetAsync(csr->diag, 0, sizeof(double) * (p.nrow ? p.nrow : 1), st));
    p.rowptr = csr->rowptr;
    p.diag = csr->diag;
    p.lower_len = csr->lower_len;
    if (!sorted_fci && !warp_doci) {
        int rc = csr_alloc_entries(csr);
        if (rc)
            return rc;
        p.cols = csr->cols;
        p.vals = csr->vals;
    }
    if (warp_doci) {
        // Full DOCI space: thread-per-row diagonal, then one warp per row
        // (on first use when the implicit DOCI form serves the products).
        doci_diag_kernel<NW><<<static_cast<unsigned>((p.nrow + 255) / 256), 256, 0, st>>>(p), ::pyci_gpu::note_launch();
        if (csr->dx_v && !(csr->flags & PYCI_BUILD_EAGER_CSR))
            return defer_csr_doci(csr, p, NW);
        int rc = csr_alloc_entries(csr);
        if (rc)
            return rc;
        p.cols = csr->cols;
        p.vals = csr->vals;
        return launch_doci_fill<NW>(ctx, p);
    }
    if (sorted_fci) {
        // Per-string tables (alpha and beta; one set when both spins have the
        // same electron count), then the row fill.
        const int64_t nstr_a = p.nrow / p.nbeta, nstr_b = p.nbeta;
        const int no_a = static_cast<int>(p.nocc_up), no_b = static_cast<int>(p.nocc_dn);
        const int nv_a = p.nbasis - no_a, nv_b = p.nbasis - no_b;
        const int na = 1 + no_a * nv_a + (no_a * (no_a - 1) / 2) * (nv_a * (nv_a - 1) / 2);
        const int nbl = 1 + no_b * nv_b + (no_b * (no_b - 1) / 2) * (nv_b * (nv_b - 1) / 2);
        const int grp1 = 1 + no_b * nv_b;
        auto pad = [](int n) {
            int q = 2;
            while (q < n)
                q <<= 1;
            return q;
        };
        const bool shared = (no_a == no_b);
        StringTables TA{}, TB{};
        TA.npad = pad(na);
        TB.npad = pad(nbl);
        TA.nw = TB.nw = NW;
        TA.n1 = no_a * nv_a;
        TA.n2 = (no_a * (no_a - 1) / 2) * (nv_a * (nv_a - 1) / 2);
        TB.n1 = no_b * nv_b;
        TB.n2 = (no_b * (no_b - 1) / 2) * (nv_b * (nv_b - 1) / 2);
        std::vector<void *> mem;
        auto make = [&](StringTables &T, int64_t nstr) -> int {
            int32_t **arrs[] = {&T.key, &T.val, &T.off, &T.sub, &T.subval};
            for (int32_t **a : arrs) {
                PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(a), sizeof(int32_t) * nstr * T.npad, st));
                mem.push_back(*a);
            }
            PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&T.self), sizeof(int32_t) * nstr, st));
            mem.push_back(T.self);
            PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&T.bits), sizeof(uint64_t) * nstr * NW, st));
            mem.push_back(T.bits);
            PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&T.sdesc), sizeof(int32_t) * nstr * std::max(T.n1, 1), st));
            mem.push_back(T.sdesc);
            PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&T.dval), sizeof(double) * nstr * std::max(T.n2, 1), st));
            mem.push_back(T.dval);
            return PYCI_GPU_OK;
        };
        int rc = make(TA, nstr_a);
        if (!rc && !shared)
            rc = make(TB, nstr_b);
        TA.glen = uniform_len;
        if (!rc) {
            const cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&TA.gmap),
                                                  sizeof(uint16_t) * nstr_a * uniform_len, st);
            if (e != cudaSuccess)
                rc = cuda_status(e, "cudaMallocAsync (string tables)");
            else
                mem.push_back(TA.gmap);
        }
        if (!shared && !rc) {
            string_tables_kernel<NW><<<static_cast<unsigned>(nstr_a), 256, scratch, st>>>(p, 0, TA, nbl, grp1, uniform_len),
                ::pyci_gpu::note_launch();
            string_tables_kernel<NW><<<static_cast<unsigned>(nstr_b), 256, scratch, st>>>(p, 1, TB, nbl, grp1, uniform_len),
                ::pyci_gpu::note_launch();
        } else if (!rc) {
            // Same string space for both spins: the alpha tables (offsets for
            // alpha use, type <= 1 lists for beta use) serve both.
            string_tables_kernel<NW><<<static_cast<unsigned>(nstr_a), 256, scratch, st>>>(p, 0, TA, nbl, grp1, uniform_len),
                ::pyci_gpu::note_launch();
            TB = TA;
        }
        int32_t *adesc = nullptr;
        if (!rc)
            rc = fcix_tables(ctx, csr, TA, TB, nstr_a, nstr_b, na, nbl, grp1, uniform_len, &adesc);
        if (!rc) {
            fci_diag_kernel<NW><<<static_cast<unsigned>((p.nrow + 255) / 256), 256, 0, st>>>(p, TA, TB),
                ::pyci_gpu::note_launch();
            if (csr->fx_hi)
                rc = fcix_fill<NW>(ctx, csr, p, TA, TB, adesc);
        }
        if (adesc)
            cudaFreeAsync(adesc, st);
        const int nsg = no_a * nv_a + no_b * nv_b;
        if (!rc && csr->fx_hi && !(csr->flags & PYCI_BUILD_EAGER_CSR)) {
            // The implicit-column form serves the products: the CSR is written
            // on first use (csr_materialize), from these tables.
            rc = defer_csr(csr, p, TA, TB, na, nsg, NW, mem);
            if (!rc)
                return PYCI_GPU_OK;
        }
        if (!rc) {
            rc = csr_alloc_entries(csr);
            p.cols = csr->cols;
            p.vals = csr->vals;
        }
        if (!rc) {
            p.lower_len = csr->fx_hi ? nullptr : csr->lower_len; // written by the implicit-column fill
            rc = launch_fci_fill<NW>(ctx, p, TA, TB, na, nsg);
        }
        for (void *m : mem)
            cudaFreeAsync(m, st);
        if (rc)
            return rc;
        PYCI_CUDA_TRY(cudaGetLastError());
        return PYCI_GPU_OK;
    }
    const size_t smem = static_cast<size_t>(cap) * (sizeof(double) + sizeof(int32_t)) + scratch;
    if (smem > 48 * 1024) {
        if (smem > ctx->smem_optin) {
            set_error("a row has %d candidate entries, more than shared memory holds", cap);
            return PYCI_GPU_EUNSUPPORTED;
        }
        PYCI_CUDA_TRY(cudaFuncSetAttribute(fill_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem)));
    }
    const int threads = cap >= 512 ? 256 : (cap >= 256 ? 128 : 64);
    for (int64_t r0 = 0; r0 < p.nrow; r0 += chunk) {
        const int64_t nb = (p.nrow - r0 < chunk) ? p.nrow - r0 : chunk;
        fill_kernel<NW><<<static_cast<unsigned>(nb), threads, smem, st>>>(p, r0, cap), ::pyci_gpu::note_launch();
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

template<int NW>
int run_build_genci_ref(pyci_gpu_ctx *ctx, BuildParams &p, pyci_gpu_csr *csr) {
    cudaStream_t st = ctx->stream;
    if (p.nrow > 0)
        genci_ref_count_kernel<NW><<<static_cast<unsigned>((p.nrow + 127) / 128), 128, 0, st>>>(p), ::pyci_gpu::note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    int rc = device_exclusive_scan(p.counts, p.nrow, csr->rowptr, st);
    if (rc)
        return rc;
    unsigned long long *d_max = nullptr;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&d_max), sizeof(unsigned long long), st));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), st));
    if (p.nrow > 0)
        max_kernel<<<static_cast<unsigned>(std::min<int64_t>((p.nrow + 255) / 256, 1024)), 256, 0, st>>>(p.counts, p.nrow, d_max), ::pyci_gpu::note_launch();
    unsigned long long maxlen = 0;
    int64_t nnz = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(&maxlen, d_max, sizeof(maxlen), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(&nnz, csr->rowptr + p.nrow, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFreeAsync(d_max, st);
    csr->nnz = nnz;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->cols), sizeof(int32_t) * (nnz ? nnz : 1), st));
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->vals), sizeof(double) * (nnz ? nnz : 1), st));
    PYCI_CUDA_TRY(cudaMemsetAsync(csr->diag, 0, sizeof(double) * (p.nrow ? p.nrow : 1), st));
    p.rowptr = csr->rowptr;
    p.cols = csr->cols;
    p.vals = csr->vals;
    p.diag = csr->diag;
    p.lower_len = csr->lower_len;
    int cap = 2;
    while (static_cast<unsigned long long>(cap) < maxlen)
        cap <<= 1;
    const size_t smem = static_cast<size_t>(cap) * (sizeof(double) + sizeof(int32_t));
    if (smem > ctx->smem_optin) {
        set_error("a GenCI row has %llu entries, more than shared memory holds", maxlen);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (smem > 48 * 1024)
        PYCI_CUDA_TRY(cudaFuncSetAttribute(genci_ref_fill_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem)));
    const int64_t chunk = 1 << 20;
    for (int64_t r0 = 0; r0 < p.nrow; r0 += chunk) {
        const int64_t nb = std::min(chunk, p.nrow - r0);
        genci_ref_fill_kernel<NW><<<static_cast<unsigned>(nb), 128, smem, st>>>(p, r0, cap), ::pyci_gpu::note_launch();
    }
    PYCI_CUDA_TRY(cudaGetLastError());
    return PYCI_GPU_OK;
}

} // namespace

int csr_build_device(pyci_gpu_ctx *ctx, pyci_gpu_csr *csr, const uint64_t *dets_host,
                     const double *one_mo, const double *two_mo, int64_t legacy_nrow,
                     int64_t legacy_ncol) {
    cudaStream_t st = ctx->stream;
    const int64_t n = csr->nbasis;
    const int nw = pick_nw(n);
    if (nw == 0) {
        set_error("nbasis = %lld exceeds the 256 orbitals the GPU build supports", (long long)n);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (csr->nocc_up > kMaxOcc || csr->nocc_dn > kMaxOcc || n - csr->nocc_dn > kMaxVir) {
        set_error("occupation numbers exceed the GPU build's limits (%d occupied)", kMaxOcc);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (csr->ndet >= INT32_MAX || csr->ncol >= INT32_MAX) {
        set_error("more than 2^31 - 1 determinants is not supported");
        return PYCI_GPU_EUNSUPPORTED;
    }
    const bool genci_ref = (csr->kind == PYCI_WFN_GENCI) && !(csr->flags & PYCI_BUILD_GENCI_EXACT);
    const bool colex = (csr->flags & PYCI_BUILD_FULL_COLEX) && !(csr->flags & PYCI_BUILD_FORCE_HASH) && !genci_ref;
    csr->lower_only = genci_ref && csr->symmetric;
    if (genci_ref && dets_host == nullptr && csr->ndet > 0) {
        set_error("the reference GenCI row loop needs the determinant array");
        return PYCI_GPU_EINVAL;
    }
    if (!colex && dets_host == nullptr && csr->ndet > 0) {
        set_error("determinant array is required unless the wave function is the full space");
        return PYCI_GPU_EINVAL;
    }
    const int kind = csr->kind;
    const int64_t nwords = (kind == PYCI_WFN_FULLCI ? 2 : 1) * static_cast<int64_t>(nw);
    const int64_t host_nword = (n + 63) / 64;

    DeviceBuffers tmp(st);
    BuildParams p{};
    p.kind = kind;
    p.nbasis = static_cast<int>(n);
    p.nocc_up = static_cast<int>(csr->nocc_up);
    p.nocc_dn = static_cast<int>(csr->nocc_dn);
    p.genci_exact = (csr->flags & PYCI_BUILD_GENCI_EXACT) ? 1 : 0;
    p.colex = colex ? 1 : 0;
    p.symmetric = csr->symmetric ? 1 : 0;
    p.ndet = csr->ndet;
    p.nrow = csr->nrow;
    p.ncol = csr->ncol;
    p.legacy_nrow = legacy_nrow;
    p.legacy_ncol = legacy_ncol;
    p.nbeta = (kind == PYCI_WFN_FULLCI) ? host_binomial(n, csr->nocc_dn) : 1;

    // Binomial table C(m, k), m <= nbasis, k <= max occupation + 1.
    const int ldk = static_cast<int>(std::max(csr->nocc_up, csr->nocc_dn) + 2);
    std::vector<int64_t> binom((n + 1) * ldk);
    for (int64_t m = 0; m <= n; ++m)
        for (int k = 0; k < ldk; ++k)
            binom[m * ldk + k] = host_binomial(m, k);
    int64_t *d_binom = nullptr;
    PYCI_CUDA_TRY(tmp.alloc(&d_binom, binom.size()));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_binom, binom.data(), sizeof(int64_t) * binom.size(),
                                  cudaMemcpyHostToDevice, st));
    p.binom = d_binom;
    p.ldk = ldk;

    // Integrals and the seniority-zero h, v, w (pyci/src/squantop.cpp:175-182).
    const int64_t n2 = n * n, n4 = n2 * n2;
    double *d_one = nullptr, *d_two = nullptr, *d_h = nullptr, *d_v = nullptr, *d_w = nullptr;
    std::vector<float> dx_v; // DOCI: v split into high and low parts (the implicit form's table)
    PYCI_CUDA_TRY(tmp.alloc(&d_one, n2));
    PYCI_CUDA_TRY(tmp.alloc(&d_two, n4));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_one, one_mo, sizeof(double) * n2, cudaMemcpyHostToDevice, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_two, two_mo, sizeof(double) * n4, cudaMemcpyHostToDevice, st));
    if (kind == PYCI_WFN_DOCI) {
        std::vector<double> h(n), v(n2), w(n2);
        for (int64_t i = 0; i < n; ++i) {
            h[i] = one_mo[i * (n + 1)];
            for (int64_t j = 0; j < n; ++j) {
                v[i * n + j] = two_mo[i * n * n2 + i * n2 + j * n + j];
                w[i * n + j] = two_mo[i * n * n2 + j * n2 + i * n + j] * 2 - two_mo[i * n * n2 + j * n2 + j * n + i];
            }
        }
        PYCI_CUDA_TRY(tmp.alloc(&d_h, n));
        PYCI_CUDA_TRY(tmp.alloc(&d_v, n2));
        PYCI_CUDA_TRY(tmp.alloc(&d_w, n2));
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_h, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_v, v.data(), sizeof(double) * n2, cudaMemcpyHostToDevice, st));
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_w, w.data(), sizeof(double) * n2, cudaMemcpyHostToDevice, st));
        dx_v.resize(2 * n2);
        for (int64_t i = 0; i < n2; ++i)
            split_hi_lo(v[i], dx_v[i], dx_v[n2 + i]);
        // The host vectors die at scope end: wait for the copies.
        PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    }
    p.one_mo = d_one;
    p.two_mo = d_two;
    p.h = d_h;
    p.v = d_v;
    p.w = d_w;

    int *d_err = nullptr;
    PYCI_CUDA_TRY(tmp.alloc(&d_err, 1));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    p.error = d_err;

    // Determinants (repacked to nw words per string) and the hash table.
    if (!colex) {
        std::vector<uint64_t> packed(static_cast<size_t>(csr->ndet * nwords), 0ULL);
        const int nstr = (kind == PYCI_WFN_FULLCI) ? 2 : 1;
        for (int64_t i = 0; i < csr->ndet; ++i)
            for (int sidx = 0; sidx < nstr; ++sidx)
                for (int64_t w = 0; w < host_nword; ++w)
                    packed[i * nwords + sidx * nw + w] = dets_host[(i * nstr + sidx) * host_nword + w];
        uint64_t *d_dets = nullptr;
        PYCI_CUDA_TRY(tmp.alloc(&d_dets, packed.size()));
        PYCI_CUDA_TRY(cudaMemcpyAsync(d_dets, packed.data(), sizeof(uint64_t) * packed.size(),
                                      cudaMemcpyHostToDevice, st));
        uint64_t cap = 16;
        while (cap < static_cast<uint64_t>(2 * csr->ndet))
            cap <<= 1;
        int32_t *slots = nullptr;
        PYCI_CUDA_TRY(tmp.alloc(&slots, cap));
        PYCI_CUDA_TRY(cudaMemsetAsync(slots, 0xff, sizeof(int32_t) * cap, st));
        const unsigned blocks = static_cast<unsigned>((csr->ndet + 255) / 256);
        if (blocks) {
            switch (nwords) {
            case 1: table_insert_kernel<1><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, csr->ndet, d_err), ::pyci_gpu::note_launch(); break;
            case 2: table_insert_kernel<2><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, csr->ndet, d_err), ::pyci_gpu::note_launch(); break;
            case 4: table_insert_kernel<4><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, csr->ndet, d_err), ::pyci_gpu::note_launch(); break;
            case 8: table_insert_kernel<8><<<blocks, 256, 0, st>>>(slots, cap - 1, d_dets, csr->ndet, d_err), ::pyci_gpu::note_launch(); break;
            default: set_error("unsupported determinant width"); return PYCI_GPU_EUNSUPPORTED;
            }
            PYCI_CUDA_TRY(cudaGetLastError());
        }
        p.dets = d_dets;
        p.table = DetTable{slots, d_dets, cap - 1, static_cast<int>(nwords)};
        // `packed` must outlive the copy.
        PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    }

    // Candidate capacity: largest row, rounded up to a power of two.
    int64_t no_a = csr->nocc_up, no_b = (kind == PYCI_WFN_FULLCI) ? csr->nocc_dn : 0;
    int64_t nv_a = n - no_a, nv_b = (kind == PYCI_WFN_FULLCI) ? n - no_b : 0;
    int64_t ncand;
    if (kind == PYCI_WFN_DOCI) {
        ncand = no_a * nv_a;
    } else {
        const int64_t sa = no_a * nv_a, sb = no_b * nv_b;
        const int64_t da = (no_a * (no_a - 1) / 2) * (nv_a * (nv_a - 1) / 2);
        const int64_t db = (no_b * (no_b - 1) / 2) * (nv_b * (nv_b - 1) / 2);
        ncand = sa + sb + da + db + sa * sb;
    }
    int64_t cap = 2;
    while (cap < ncand + 1)
        cap <<= 1;
    if (cap > (1 << 22)) {
        set_error("rows with %lld candidate excitations are not supported", (long long)ncand);
        return PYCI_GPU_EUNSUPPORTED;
    }

    // Rank cache (full spaces): every row has the same number of excitations.
    p.ncache = 0;
    if (colex) {
        const int64_t pa = no_a * (no_a - 1) / 2, qa = nv_a * (nv_a - 1) / 2;
        const int64_t pb = no_b * (no_b - 1) / 2, qb = nv_b * (nv_b - 1) / 2;
        int64_t nc = no_a * nv_a;
        if (kind == PYCI_WFN_FULLCI)
            nc += no_b * nv_b + pa * qa + pb * qb;
        else if (kind == PYCI_WFN_GENCI)
            nc += pa * qa;
        if (nc * static_cast<int64_t>(sizeof(int32_t)) <= 64 * 1024)
            p.ncache = static_cast<int>(nc);
    }
    p.binom_smem = (binom.size() * sizeof(int64_t) <= 16 * 1024) ? static_cast<int>(binom.size()) : 0;

    int64_t *d_counts = nullptr;
    PYCI_CUDA_TRY(tmp.alloc(&d_counts, csr->nrow));
    p.counts = d_counts;
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->rowptr), sizeof(int64_t) * (csr->nrow + 1), st));
    PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->diag), sizeof(double) * (csr->nrow ? csr->nrow : 1), st));
    if (csr->symmetric) {
        PYCI_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(&csr->lower_len), sizeof(int32_t) * (csr->nrow ? csr->nrow : 1), st));
        PYCI_CUDA_TRY(cudaMemsetAsync(csr->lower_len, 0, sizeof(int32_t) * (csr->nrow ? csr->nrow : 1), st));
    }

    int rc;
    if (genci_ref) {
        switch (nw) {
        case 1: rc = run_build_genci_ref<1>(ctx, p, csr); break;
        case 2: rc = run_build_genci_ref<2>(ctx, p, csr); break;
        default: rc = run_build_genci_ref<4>(ctx, p, csr); break;
        }
    } else {
        const bool uniform = colex && legacy_nrow == 0 && csr->nrow == csr->ndet && csr->ncol == csr->ndet;
        const int64_t ulen = uniform ? ncand + 1 : 0;
        const int64_t na = 1 + no_a * nv_a + (no_a * (no_a - 1) / 2) * (nv_a * (nv_a - 1) / 2);
        const int64_t nbb = 1 + no_b * nv_b + (no_b * (no_b - 1) / 2) * (nv_b * (nv_b - 1) / 2);
        const bool warp_doci = uniform && kind == PYCI_WFN_DOCI && no_a <= kMaxOcc && nv_a <= kMaxVir &&
                               !(csr->flags & PYCI_BUILD_FORCE_HASH);
        const bool sorted_fci = uniform && kind == PYCI_WFN_FULLCI && p.ncache > 0 && na <= kSortedMax &&
                                nbb <= kSortedMax && no_a * nv_a + no_b * nv_b <= kTableMaxSingles &&
                                !(csr->flags & PYCI_BUILD_FORCE_HASH);
        // Implicit form of a full DOCI space (docx.cu): the binomial table and
        // the split pair integrals; products then read no stored entries.
        if (warp_doci && csr->symmetric && n <= 64 && !dx_v.empty()) {
            const size_t nb = binom.size();
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&csr->dx_binom), sizeof(int64_t) * nb, st);
            if (e == cudaSuccess)
                e = cudaMallocAsync(reinterpret_cast<void **>(&csr->dx_v), sizeof(float) * dx_v.size(), st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(csr->dx_binom, binom.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(csr->dx_v, dx_v.data(), sizeof(float) * dx_v.size(), cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess)
                return cuda_status(e, "implicit DOCI tables");
            csr->dx_n = static_cast<int>(n);
            csr->dx_m = static_cast<int>(csr->nocc_up);
            csr->dx_ldk = ldk;
        }
        switch (nw) {
        case 1: rc = run_build<1>(ctx, p, csr, static_cast<int>(cap), ulen, sorted_fci, warp_doci); break;
        case 2: rc = run_build<2>(ctx, p, csr, static_cast<int>(cap), ulen, sorted_fci, warp_doci); break;
        default: rc = run_build<4>(ctx, p, csr, static_cast<int>(cap), ulen, sorted_fci, warp_doci); break;
        }
    }
    if (rc)
        return rc;

    // Reference-layout row pointers (symmetric: prefix sums of lower_len).
    // A deferred DOCI operator gets them with its entries; its pattern is
    // symmetric, so the reference's count is the lower triangle + diagonal.
    if (csr->symmetric && csr->deferred && kind == PYCI_WFN_DOCI) {
        csr->nnz_ref = (csr->nnz - csr->nrow) / 2 + csr->nrow;
    } else if (csr->symmetric) {
        rc = ref_rowptr_from_lower_len(csr);
        if (rc)
            return rc;
    } else {
        csr->nnz_ref = csr->nnz;
    }
    int herr = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
        set_error("internal inconsistency in the CSR build (code %d)", herr);
        return PYCI_GPU_ECUDA;
    }
    return PYCI_GPU_OK;
}

