// Heat-bath CI determinant selection on the device, replacing add_hci
// (pyci/src/hci.cpp:240-262), which runs the loops of hci_thread_add_dets
// (DOCI 21-46, FullCI 48-183, GenCI 185-238) on host threads.
//
// A candidate determinant is reached from determinant i by a single or double
// excitation whose matrix element satisfies |H_ji| > eps / |c_i|; it is new
// when the wave function does not contain it.  One thread per determinant
// replays the reference's loops (same excitation order, same FP64 sums for
// the single-excitation elements, the threshold compared the same way), in
// two passes: count the new candidates of each determinant, then, after a
// prefix sum, write them.  The written list is in (i ascending, loop order),
// so a candidate's position is its first-occurrence rank; a hash table over
// the list keeps the smallest position of every distinct determinant, and a
// compaction of those positions gives each new determinant once, in
// first-occurrence order.  (The reference merges per-thread hash maps, so its
// order of the new determinants follows its hash map; the set is the same.)
//
// GenCI: by default the reference's own loop, including its virtual-count
// quirk (Wfn::init sets nvir = 2 nbasis - nocc for a spin-orbital basis, so
// the loop also "excites" into orbital 0 and its excite/restore pairs can
// drop orbital 0 from the working determinant; it then adds determinants
// with one electron too few).  PYCI_BUILD_GENCI_EXACT loops over the true
// virtual spin-orbitals instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "detops.cuh"
#include "internal.h"

namespace pyci_gpu {

namespace {

struct HciParams {
    int kind;
    int genci_ref;
    int n, nocc_up, nocc_dn;
    int64_t ndet;
    const uint64_t *dets; // [ndet][words per determinant]
    const double *coeffs, *one, *two;
    double eps;
    DetTable table;          // the wave function's determinants
    int64_t *counts;         // count pass: new candidates per determinant
    const int64_t *offsets;  // fill pass: prefix sum of counts
    uint64_t *cand;          // fill pass: candidate determinants
};

__device__ __forceinline__ double two_at(const double *two, int n, int i, int k, int j, int l) {
    return __ldg(&two[((static_cast<int64_t>(i) * n + k) * n + j) * n + l]);
}

// excite_det (pyci/src/common.cpp:284-287): clear i, set a.
__device__ __forceinline__ void excite(uint64_t *det, int i, int a) {
    det[i >> 6] &= ~(1ULL << (i & 63));
    det[a >> 6] |= 1ULL << (a & 63);
}

// Candidates of determinant idet in the reference's loop order; emit(det)
// for each one that passes the threshold and is not in the table.  NW words
// per spin string; NWD words per determinant (2 NW for FullCI).
template<int NW, int NWD, class Emit>
__device__ void hci_row(const HciParams &p, int64_t idet, Emit emit) {
    const int n = p.n;
    const double *one = p.one, *two = p.two;
    const double eps_i = p.eps / fabs(p.coeffs[idet]);
    uint64_t det[NWD];
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        det[w] = p.dets[idet * NWD + w];
    auto visit = [&](double val) {
        if (fabs(val) > eps_i && p.table.find<NWD>(det) < 0)
            emit(det);
    };
    if (p.kind == PYCI_WFN_DOCI) {
        // pyci/src/hci.cpp:31-45; v[k][l] = two_mo[k][k][l][l] (pyci/src/squantop.cpp:177).
        int16_t occ[kMaxOcc], vir[kMaxVir];
        const int no = occ_list<NW>(det, occ), nv = vir_list<NW>(det, n, vir);
        for (int i = 0; i < no; ++i) {
            const int k = occ[i];
            for (int j = 0; j < nv; ++j) {
                const int l = vir[j];
                const double val = two_at(two, n, k, k, l, l);
                if (fabs(val) > eps_i) {
                    excite(det, k, l);
                    visit(val);
                    excite(det, l, k);
                }
            }
        }
        return;
    }
    if (p.kind == PYCI_WFN_FULLCI) {
        // pyci/src/hci.cpp:60-182.
        uint64_t *up = det, *dn = det + NW;
        int16_t ou[kMaxOcc], od[kMaxOcc], vu[kMaxVir], vd[kMaxVir];
        const int nou = occ_list<NW>(up, ou), nod = occ_list<NW>(dn, od);
        const int nvu = vir_list<NW>(up, n, vu), nvd = vir_list<NW>(dn, n, vd);
        for (int i = 0; i < nou; ++i) {
            const int ii = ou[i];
            for (int j = 0; j < nvu; ++j) {
                const int jj = vu[j];
                excite(up, ii, jj);
                double val = __ldg(&one[n * ii + jj]);
                for (int k = 0; k < nou; ++k) {
                    const int kk = ou[k];
                    val += two_at(two, n, ii, kk, jj, kk) - two_at(two, n, ii, kk, kk, jj);
                }
                for (int k = 0; k < nod; ++k) {
                    const int kk = od[k];
                    val += two_at(two, n, ii, kk, jj, kk);
                }
                visit(val);
                for (int k = 0; k < nod; ++k) {
                    const int kk = od[k];
                    for (int l = 0; l < nvd; ++l) {
                        const int ll = vd[l];
                        val = two_at(two, n, ii, kk, jj, ll);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            visit(val);
                            excite(dn, ll, kk);
                        }
                    }
                }
                for (int k = i + 1; k < nou; ++k) {
                    const int kk = ou[k];
                    for (int l = j + 1; l < nvu; ++l) {
                        const int ll = vu[l];
                        val = two_at(two, n, ii, kk, jj, ll) - two_at(two, n, ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(up, kk, ll);
                            visit(val);
                            excite(up, ll, kk);
                        }
                    }
                }
                excite(up, jj, ii);
            }
        }
        for (int i = 0; i < nod; ++i) {
            const int ii = od[i];
            for (int j = 0; j < nvd; ++j) {
                const int jj = vd[j];
                excite(dn, ii, jj);
                double val = __ldg(&one[n * ii + jj]);
                for (int k = 0; k < nou; ++k) {
                    const int kk = ou[k];
                    val += two_at(two, n, ii, kk, jj, kk);
                }
                for (int k = 0; k < nod; ++k) {
                    const int kk = od[k];
                    val += two_at(two, n, ii, kk, jj, kk) - two_at(two, n, ii, kk, kk, jj);
                }
                visit(val);
                for (int k = i + 1; k < nod; ++k) {
                    const int kk = od[k];
                    for (int l = j + 1; l < nvd; ++l) {
                        const int ll = vd[l];
                        val = two_at(two, n, ii, kk, jj, ll) - two_at(two, n, ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            visit(val);
                            excite(dn, ll, kk);
                        }
                    }
                }
                excite(dn, jj, ii);
            }
        }
        return;
    }
    // GenCI, pyci/src/hci.cpp:196-237.
    int16_t occ[kMaxOcc], vir[2 * kMaxVir];
    const int no = occ_list<NW>(det, occ);
    int nv = vir_list<NW>(det, n, vir);
    if (p.genci_ref) {
        const int nv_ref = 2 * n - p.nocc_up - p.nocc_dn;
        for (int j = nv; j < nv_ref; ++j)
            vir[j] = 0;
        nv = nv_ref;
    }
    for (int i = 0; i < no; ++i) {
        const int ii = occ[i];
        for (int j = 0; j < nv; ++j) {
            const int jj = vir[j];
            excite(det, ii, jj);
            double val = __ldg(&one[n * ii + jj]);
            for (int k = 0; k < no; ++k) {
                const int kk = occ[k];
                val += two_at(two, n, ii, kk, jj, kk) - two_at(two, n, ii, kk, kk, jj);
            }
            visit(val);
            for (int k = i + 1; k < no; ++k) {
                const int kk = occ[k];
                for (int l = j + 1; l < nv; ++l) {
                    const int ll = vir[l];
                    val = two_at(two, n, ii, kk, jj, ll) - two_at(two, n, ii, kk, ll, jj);
                    if (fabs(val) > eps_i) {
                        excite(det, kk, ll);
                        visit(val);
                        excite(det, ll, kk);
                    }
                }
            }
            excite(det, jj, ii);
        }
    }
}

template<int NW, int NWD>
__global__ void __launch_bounds__(128) hci_count_kernel(HciParams p) {
    const int64_t idet = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (idet >= p.ndet)
        return;
    int64_t cnt = 0;
    hci_row<NW, NWD>(p, idet, [&](const uint64_t *) { ++cnt; });
    p.counts[idet] = cnt;
}

template<int NW, int NWD>
__global__ void __launch_bounds__(128) hci_fill_kernel(HciParams p) {
    const int64_t idet = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (idet >= p.ndet)
        return;
    uint64_t *out = p.cand + p.offsets[idet] * NWD;
    const int64_t cap = p.offsets[idet + 1] - p.offsets[idet];
    int64_t cnt = 0;
    hci_row<NW, NWD>(p, idet, [&](const uint64_t *d) {
        if (cnt < cap) {
#pragma unroll
            for (int w = 0; w < NWD; ++w)
                out[cnt * NWD + w] = d[w];
        }
        ++cnt;
    });
}

// keep[c] = 1 when candidate c is the first occurrence of its determinant
// (the table over the candidates keeps the smallest index).
template<int NWD>
__global__ void first_occurrence_kernel(DetTable t, int64_t ncand, int64_t *keep) {
    const int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (c >= ncand)
        return;
    uint64_t d[NWD];
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        d[w] = t.dets[c * NWD + w];
    keep[c] = (t.find<NWD>(d) == c) ? 1 : 0;
}

template<int NWD>
__global__ void compact_kernel(const uint64_t *cand, int64_t ncand, const int64_t *keep, const int64_t *pos,
                               uint64_t *out) {
    const int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (c >= ncand || !keep[c])
        return;
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        out[pos[c] * NWD + w] = cand[c * NWD + w];
}

struct Pool {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit Pool(cudaStream_t st) : s(st) {}
    template<typename T>
    cudaError_t alloc(T **p, size_t count) {
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(p), sizeof(T) * (count ? count : 1), s);
        if (e == cudaSuccess)
            ptrs.push_back(*p);
        return e;
    }
    void adopt(void *p) { ptrs.push_back(p); }
    ~Pool() {
        for (void *p : ptrs)
            cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
    }
};

template<int NW, int NWD>
int run_select(cudaStream_t st, HciParams p, int64_t host_nword, int nstr, int64_t max_new, uint64_t *out,
               int64_t *n_new, Pool &pool) {
    const unsigned blocks = static_cast<unsigned>((p.ndet + 127) / 128);
    int64_t *counts = nullptr, *offsets = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&counts, p.ndet));
    PYCI_CUDA_TRY(pool.alloc(&offsets, p.ndet + 1));
    p.counts = counts;
    hci_count_kernel<NW, NWD><<<blocks, 128, 0, st>>>(p), note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    int rc = device_exclusive_scan(counts, p.ndet, offsets, st);
    if (rc)
        return rc;
    int64_t ncand = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(&ncand, offsets + p.ndet, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    if (ncand >= INT32_MAX) {
        set_error("heat-bath CI step with %lld candidates exceeds the device table's 2^31 - 1 entries",
                  static_cast<long long>(ncand));
        return PYCI_GPU_EUNSUPPORTED;
    }
    *n_new = 0;
    if (ncand == 0)
        return PYCI_GPU_OK;
    uint64_t *cand = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&cand, static_cast<size_t>(ncand) * NWD));
    p.offsets = offsets;
    p.cand = cand;
    hci_fill_kernel<NW, NWD><<<blocks, 128, 0, st>>>(p), note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    // First occurrences, in candidate order.
    int *d_err = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&d_err, 1));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    int32_t *slots = nullptr;
    uint64_t mask = 0;
    if ((rc = det_table_build(cand, ncand, NWD, st, d_err, &slots, &mask)))
        return rc;
    pool.adopt(slots);
    int64_t *keep = nullptr, *pos = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&keep, ncand));
    PYCI_CUDA_TRY(pool.alloc(&pos, ncand + 1));
    const unsigned cblocks = static_cast<unsigned>((ncand + 255) / 256);
    first_occurrence_kernel<NWD><<<cblocks, 256, 0, st>>>(DetTable{slots, cand, mask, NWD}, ncand, keep),
        note_launch();
    if ((rc = device_exclusive_scan(keep, ncand, pos, st)))
        return rc;
    int64_t m = 0;
    int err = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(&m, pos + ncand, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    if (err) {
        set_error("device determinant table overflow");
        return PYCI_GPU_ECUDA;
    }
    *n_new = m;
    if (m == 0 || !out || m > max_new)
        return PYCI_GPU_OK;
    uint64_t *uniq = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&uniq, static_cast<size_t>(m) * NWD));
    compact_kernel<NWD><<<cblocks, 256, 0, st>>>(cand, ncand, keep, pos, uniq), note_launch();
    std::vector<uint64_t> packed(static_cast<size_t>(m) * NWD);
    PYCI_CUDA_TRY(cudaMemcpyAsync(packed.data(), uniq, sizeof(uint64_t) * packed.size(), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    // Device strings hold NW words; the caller's hold host_nword (<= NW).
    for (int64_t d = 0; d < m; ++d)
        for (int s = 0; s < nstr; ++s)
            for (int64_t w = 0; w < host_nword; ++w)
                out[(d * nstr + s) * host_nword + w] = packed[d * NWD + s * NW + w];
    return PYCI_GPU_OK;
}

} // namespace

} // namespace pyci_gpu

using namespace pyci_gpu;

int hci_select_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                      const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo,
                      double eps, int flags, int64_t max_new, uint64_t *out, int64_t *n_new) {
    cudaStream_t st = ctx->stream;
    const int64_t n = nbasis;
    const int nw = n <= 64 ? 1 : (n <= 128 ? 2 : (n <= 256 ? 4 : 0));
    if (nw == 0) {
        set_error("nbasis = %lld exceeds the 256 orbitals the GPU path supports", static_cast<long long>(n));
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (nocc_up > kMaxOcc || nocc_dn > kMaxOcc || (kind == PYCI_WFN_GENCI && nocc_up + nocc_dn > kMaxOcc)) {
        set_error("occupation numbers exceed the GPU path's limits (%d occupied)", kMaxOcc);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (ndet >= INT32_MAX) {
        set_error("more than 2^31 - 1 determinants is not supported");
        return PYCI_GPU_EUNSUPPORTED;
    }
    *n_new = 0;
    if (ndet == 0)
        return PYCI_GPU_OK;
    const int nstr = kind == PYCI_WFN_FULLCI ? 2 : 1;
    const int64_t host_nword = (n + 63) / 64;
    const int nwd = nstr * nw;
    Pool pool(st);
    // Determinants repacked to nw words per string, and their table.
    std::vector<uint64_t> packed(static_cast<size_t>(ndet) * nwd, 0ULL);
    for (int64_t i = 0; i < ndet; ++i)
        for (int s = 0; s < nstr; ++s)
            for (int64_t w = 0; w < host_nword; ++w)
                packed[i * nwd + s * nw + w] = dets[(i * nstr + s) * host_nword + w];
    uint64_t *d_dets = nullptr;
    double *d_coef = nullptr, *d_one = nullptr, *d_two = nullptr;
    int *d_err = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&d_dets, packed.size()));
    PYCI_CUDA_TRY(pool.alloc(&d_coef, ndet));
    PYCI_CUDA_TRY(pool.alloc(&d_one, n * n));
    PYCI_CUDA_TRY(pool.alloc(&d_two, n * n * n * n));
    PYCI_CUDA_TRY(pool.alloc(&d_err, 1));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_dets, packed.data(), sizeof(uint64_t) * packed.size(), cudaMemcpyHostToDevice, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_coef, coeffs, sizeof(double) * ndet, cudaMemcpyHostToDevice, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_one, one_mo, sizeof(double) * n * n, cudaMemcpyHostToDevice, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(d_two, two_mo, sizeof(double) * n * n * n * n, cudaMemcpyHostToDevice, st));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    int32_t *slots = nullptr;
    uint64_t mask = 0;
    int rc = det_table_build(d_dets, ndet, nwd, st, d_err, &slots, &mask);
    if (rc)
        return rc;
    pool.adopt(slots);
    PYCI_CUDA_TRY(cudaStreamSynchronize(st)); // `packed` must outlive its copy

    HciParams p{};
    p.kind = kind;
    p.genci_ref = (kind == PYCI_WFN_GENCI) && !(flags & PYCI_BUILD_GENCI_EXACT);
    p.n = static_cast<int>(n);
    p.nocc_up = static_cast<int>(nocc_up);
    p.nocc_dn = static_cast<int>(nocc_dn);
    p.ndet = ndet;
    p.dets = d_dets;
    p.coeffs = d_coef;
    p.one = d_one;
    p.two = d_two;
    p.eps = eps;
    p.table = DetTable{slots, d_dets, mask, nwd};
    switch (nwd) {
    case 1: rc = run_select<1, 1>(st, p, host_nword, nstr, max_new, out, n_new, pool); break;
    case 2: rc = kind == PYCI_WFN_FULLCI ? run_select<1, 2>(st, p, host_nword, nstr, max_new, out, n_new, pool)
                                         : run_select<2, 2>(st, p, host_nword, nstr, max_new, out, n_new, pool);
        break;
    case 4: rc = kind == PYCI_WFN_FULLCI ? run_select<2, 4>(st, p, host_nword, nstr, max_new, out, n_new, pool)
                                         : run_select<4, 4>(st, p, host_nword, nstr, max_new, out, n_new, pool);
        break;
    default: rc = run_select<4, 8>(st, p, host_nword, nstr, max_new, out, n_new, pool); break;
    }
    return rc;
}
