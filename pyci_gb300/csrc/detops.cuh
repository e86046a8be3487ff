// Device-side determinant primitives: occupation lists, Slater-Condon phases,
// colex ranking/unranking and the determinant -> index hash table.
//
// Determinants are bit strings of 64-bit words (bit p of word p/64 set when
// orbital p is occupied), the layout of pyci::Wfn (pyci/include/pyci.h:306-330).
#pragma once

#include <cstdint>

namespace pyci_gpu {

constexpr int kMaxOcc = 64;   // occupied orbitals per spin string
constexpr int kMaxVir = 256;  // virtual orbitals per spin string

// Bits strictly between orbitals i and a (exclusive), summed over NW words.
// Same count as the masks of phase_single_det (pyci/src/common.cpp:163-194).
template<int NW>
__device__ __forceinline__ int perm_between(const uint64_t *det, int i, int a) {
    int lo = i < a ? i : a, hi = i < a ? a : i;
    int n = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        int s = lo + 1 - 64 * w, e = hi - 1 - 64 * w;
        if (s < 0)
            s = 0;
        if (e > 63)
            e = 63;
        if (s <= e) {
            uint64_t m = (~0ULL >> (63 - e)) & (~0ULL << s);
            n += __popcll(det[w] & m);
        }
    }
    return n;
}

// pyci/src/common.cpp:163-194
template<int NW>
__device__ __forceinline__ int phase_single(const uint64_t *det, int i, int a) {
    return (perm_between<NW>(det, i, a) & 1) ? -1 : 1;
}

// pyci/src/common.cpp:196-261 (both excitations measured on the reference
// determinant, plus one transposition when the pairs do not nest).
template<int NW>
__device__ __forceinline__ int phase_double(const uint64_t *det, int i1, int i2, int a1, int a2) {
    int n = perm_between<NW>(det, i1, a1) + perm_between<NW>(det, i2, a2);
    if ((i2 < a1) || (i1 > a2))
        ++n;
    return (n & 1) ? -1 : 1;
}

__device__ __forceinline__ void flip(uint64_t *det, int p) { det[p >> 6] ^= 1ULL << (p & 63); }

// Ascending occupied / virtual orbital lists of one spin string
// (pyci/src/common.cpp:85-113).  Returns the count.
template<int NW>
__device__ __forceinline__ int occ_list(const uint64_t *det, int16_t *out) {
    int j = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint64_t x = det[w];
        while (x && j < kMaxOcc) {
            int p = __ffsll(static_cast<long long>(x)) - 1;
            out[j++] = static_cast<int16_t>(p + 64 * w);
            x &= x - 1;
        }
    }
    return j;
}

template<int NW>
__device__ __forceinline__ int vir_list(const uint64_t *det, int nbasis, int16_t *out) {
    int j = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        int left = nbasis - 64 * w;
        if (left <= 0)
            break;
        uint64_t mask = left >= 64 ? ~0ULL : ((1ULL << left) - 1);
        uint64_t x = ~det[w] & mask;
        while (x) {
            int p = __ffsll(static_cast<long long>(x)) - 1;
            out[j++] = static_cast<int16_t>(p + 64 * w);
            x &= x - 1;
        }
    }
    return j;
}

// Colex rank: sum over the t-th occupied orbital p_t (t = 1, 2, ...) of
// C(p_t, t) (pyci/src/common.cpp:124-137).  binom[n * ldk + k] = C(n, k).
template<int NW>
__device__ __forceinline__ int64_t rank_colex(const uint64_t *det, const int64_t *binom, int ldk) {
    int64_t r = 0;
    int t = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint64_t x = det[w];
        while (x) {
            int p = __ffsll(static_cast<long long>(x)) - 1 + 64 * w;
            ++t;
            r += __ldg(&binom[p * ldk + t]);
            x &= x - 1;
        }
    }
    return r;
}

// Inverse of rank_colex (pyci/src/common.cpp:139-153): sets nocc bits of det.
template<int NW>
__device__ __forceinline__ void unrank_colex(int64_t rank, int nbasis, int nocc,
                                             const int64_t *binom, int ldk, uint64_t *det) {
#pragma unroll
    for (int w = 0; w < NW; ++w)
        det[w] = 0;
    int p = nbasis - 1;
    for (int j = nocc; j >= 1; --j) {
        while (p >= 0 && __ldg(&binom[p * ldk + j]) > rank)
            --p;
        if (p < 0)
            return;
        det[p >> 6] |= 1ULL << (p & 63);
        rank -= __ldg(&binom[p * ldk + j]);
        --p;
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

__device__ __forceinline__ uint64_t hash_words(const uint64_t *w, int n) {
    uint64_t h = 0x84222325cbf29ce4ULL;
    for (int i = 0; i < n; ++i)
        h = mix64(h ^ (w[i] + 0x9e3779b97f4a7c15ULL * static_cast<uint64_t>(i + 1)));
    return h;
}

// Open-addressing table of determinant indices (int32, -1 = empty), keyed on
// the determinant words stored in `dets` (nwords per determinant).  Plays the
// role of the reference's hash map from determinant to insertion index
// (pyci/src/onespinwfn.cpp:123-126, pyci/src/twospinwfn.cpp:129-132).
struct DetTable {
    const int32_t *slots;
    const uint64_t *dets;
    uint64_t mask;
    int nwords;

    template<int NWT>
    __device__ __forceinline__ int64_t find(const uint64_t *key) const {
        uint64_t s = hash_words(key, NWT) & mask;
        for (uint64_t probe = 0; probe <= mask; ++probe) {
            int32_t idx = __ldg(&slots[s]);
            if (idx < 0)
                return -1;
            const uint64_t *d = dets + static_cast<int64_t>(idx) * NWT;
            bool eq = true;
#pragma unroll
            for (int i = 0; i < NWT; ++i)
                eq &= (__ldg(&d[i]) == key[i]);
            if (eq)
                return idx;
            s = (s + 1) & mask;
        }
        return -1;
    }
};

} // namespace pyci_gpu
