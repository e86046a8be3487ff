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
// The same loops drive the Epstein-Nesbet second-order correction
// (compute_enpt2, pyci/src/enpt2.cpp:76-375): the FullCI excitations and
// thresholds of add_hci, with each external determinant k collecting
// H_ki c_i (phase included; DOCI through its FullCI image, as the reference
// does).  The candidate list is filled with those values; a table over the
// list maps every candidate to its determinant's first occurrence, the values
// are summed there with FP64 atomics, and each distinct k adds
// V_k^2 / (E - H_kk) to the correction.
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
    double *cand_val;        // ENPT2 fill pass: H_ki c_i of each candidate
};

__device__ __forceinline__ double two_at(const double *two, int n, int i, int k, int j, int l) {
    return __ldg(&two[((static_cast<int64_t>(i) * n + k) * n + j) * n + l]);
}

// excite_det (pyci/src/common.cpp:284-287): clear i, set a.
__device__ __forceinline__ void excite(uint64_t *det, int i, int a) {
    det[i >> 6] &= ~(1ULL << (i & 63));
    det[a >> 6] |= 1ULL << (a & 63);
}

// Candidates of determinant idet in the reference's loop order; emit(det, v)
// for each one that passes the threshold and is not in the table.  With
// VALUES (FullCI only), v = H_ki c_i with the excitation's phase, multiplied
// in the reference's order (pyci/src/enpt2.cpp:120-236); otherwise v = 0.
// NW words per spin string; NWD words per determinant (2 NW for FullCI).
template<int NW, int NWD, bool VALUES, class Emit>
__device__ void hci_row(const HciParams &p, int64_t idet, Emit emit) {
    const int n = p.n;
    const double *one = p.one, *two = p.two;
    const double ci = p.coeffs[idet];
    const double eps_i = p.eps / fabs(ci);
    uint64_t det[NWD], rdet[NWD];
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        det[w] = rdet[w] = p.dets[idet * NWD + w];
    // factor(): the phase times c_i, evaluated only for an emitted candidate.
    auto visit = [&](double val, auto factor) {
        if (fabs(val) > eps_i && p.table.find<NWD>(det) < 0)
            emit(det, VALUES ? val * factor() : 0.0);
    };
    auto none = [] { return 0.0; };
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
                    visit(val, none);
                    excite(det, l, k);
                }
            }
        }
        return;
    }
    if (p.kind == PYCI_WFN_FULLCI) {
        // pyci/src/hci.cpp:60-182.
        uint64_t *up = det, *dn = det + NW;
        const uint64_t *rup = rdet, *rdn = rdet + NW;
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
                visit(val, [&] { return phase_single<NW>(rup, ii, jj) * ci; });
                for (int k = 0; k < nod; ++k) {
                    const int kk = od[k];
                    for (int l = 0; l < nvd; ++l) {
                        const int ll = vd[l];
                        val = two_at(two, n, ii, kk, jj, ll);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            visit(val, [&] {
                                return static_cast<double>(phase_single<NW>(rup, ii, jj) * phase_single<NW>(rdn, kk, ll)) * ci;
                            });
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
                            visit(val, [&] { return phase_double<NW>(rup, ii, kk, jj, ll) * ci; });
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
                visit(val, [&] { return phase_single<NW>(rdn, ii, jj) * ci; });
                for (int k = i + 1; k < nod; ++k) {
                    const int kk = od[k];
                    for (int l = j + 1; l < nvd; ++l) {
                        const int ll = vd[l];
                        val = two_at(two, n, ii, kk, jj, ll) - two_at(two, n, ii, kk, ll, jj);
                        if (fabs(val) > eps_i) {
                            excite(dn, kk, ll);
                            visit(val, [&] { return phase_double<NW>(rdn, ii, kk, jj, ll) * ci; });
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
            visit(val, none);
            for (int k = i + 1; k < no; ++k) {
                const int kk = occ[k];
                for (int l = j + 1; l < nv; ++l) {
                    const int ll = vir[l];
                    val = two_at(two, n, ii, kk, jj, ll) - two_at(two, n, ii, kk, ll, jj);
                    if (fabs(val) > eps_i) {
                        excite(det, kk, ll);
                        visit(val, none);
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
    hci_row<NW, NWD, false>(p, idet, [&](const uint64_t *, double) { ++cnt; });
    p.counts[idet] = cnt;
}

template<int NW, int NWD, bool VALUES>
__global__ void __launch_bounds__(128) hci_fill_kernel(HciParams p) {
    const int64_t idet = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (idet >= p.ndet)
        return;
    const int64_t base = p.offsets[idet];
    uint64_t *out = p.cand + base * NWD;
    const int64_t cap = p.offsets[idet + 1] - base;
    int64_t cnt = 0;
    hci_row<NW, NWD, VALUES>(p, idet, [&](const uint64_t *d, double v) {
        if (cnt < cap) {
#pragma unroll
            for (int w = 0; w < NWD; ++w)
                out[cnt * NWD + w] = d[w];
            if (VALUES)
                p.cand_val[base + cnt] = v;
        }
        ++cnt;
    });
}

// ENPT2: sum each candidate's value at its determinant's first occurrence.
template<int NWD>
__global__ void enpt2_accumulate_kernel(DetTable t, int64_t ncand, const double *val, double *sum) {
    const int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (c >= ncand)
        return;
    uint64_t d[NWD];
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        d[w] = t.dets[c * NWD + w];
    const int64_t rep = t.find<NWD>(d);
    if (rep >= 0)
        atomicAdd(&sum[rep], val[c]);
}

// FullCI diagonal element (compute_enpt2_thread_gather, pyci/src/enpt2.cpp:37-74):
// alpha terms with the alpha-beta Coulomb terms, then the beta terms.
template<int NW>
__device__ double fci_diag(const uint64_t *det, int n, const double *one, const double *two) {
    int16_t ou[kMaxOcc], od[kMaxOcc];
    const int nou = occ_list<NW>(det, ou), nod = occ_list<NW>(det + NW, od);
    double diag = 0.0;
    for (int i = 0; i < nou; ++i) {
        const int j = ou[i];
        diag += __ldg(&one[(n + 1) * j]);
        for (int k = i + 1; k < nou; ++k) {
            const int l = ou[k];
            diag += two_at(two, n, j, l, j, l) - two_at(two, n, j, l, l, j);
        }
        for (int k = 0; k < nod; ++k) {
            const int l = od[k];
            diag += two_at(two, n, j, l, j, l);
        }
    }
    for (int i = 0; i < nod; ++i) {
        const int j = od[i];
        diag += __ldg(&one[(n + 1) * j]);
        for (int k = i + 1; k < nod; ++k) {
            const int l = od[k];
            diag += two_at(two, n, j, l, j, l) - two_at(two, n, j, l, l, j);
        }
    }
    return diag;
}

// partial[block] = sum over the block's first occurrences c of
// sum[c]^2 / (e - H_cc).
template<int NW, int NWD>
__global__ void __launch_bounds__(256) enpt2_terms_kernel(DetTable t, int64_t ncand, const int64_t *keep,
                                                          const double *sum, int n, const double *one,
                                                          const double *two, double e, double *partial) {
    double acc = 0.0;
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < ncand;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (!keep[c])
            continue;
        const double v = sum[c];
        acc += v * v / (e - fci_diag<NW>(t.dets + c * NWD, n, one, two));
    }
    __shared__ double red[8];
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
            s += red[w];
        partial[blockIdx.x] = s;
    }
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
    hci_fill_kernel<NW, NWD, false><<<blocks, 128, 0, st>>>(p), note_launch();
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

template<int NW, int NWD>
int run_enpt2(cudaStream_t st, HciParams p, double e, int num_sms, double *correction, Pool &pool) {
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
    *correction = 0.0;
    if (ncand == 0)
        return PYCI_GPU_OK;
    if (ncand >= INT32_MAX) {
        set_error("ENPT2 with %lld external terms exceeds the device table's 2^31 - 1 entries",
                  static_cast<long long>(ncand));
        return PYCI_GPU_EUNSUPPORTED;
    }
    uint64_t *cand = nullptr;
    double *val = nullptr, *sum = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&cand, static_cast<size_t>(ncand) * NWD));
    PYCI_CUDA_TRY(pool.alloc(&val, ncand));
    PYCI_CUDA_TRY(pool.alloc(&sum, ncand));
    PYCI_CUDA_TRY(cudaMemsetAsync(sum, 0, sizeof(double) * ncand, st));
    p.offsets = offsets;
    p.cand = cand;
    p.cand_val = val;
    hci_fill_kernel<NW, NWD, true><<<blocks, 128, 0, st>>>(p), note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    int *d_err = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&d_err, 1));
    PYCI_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    int32_t *slots = nullptr;
    uint64_t mask = 0;
    if ((rc = det_table_build(cand, ncand, NWD, st, d_err, &slots, &mask)))
        return rc;
    pool.adopt(slots);
    const DetTable t{slots, cand, mask, NWD};
    int64_t *keep = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&keep, ncand));
    const unsigned cblocks = static_cast<unsigned>((ncand + 255) / 256);
    first_occurrence_kernel<NWD><<<cblocks, 256, 0, st>>>(t, ncand, keep), note_launch();
    enpt2_accumulate_kernel<NWD><<<cblocks, 256, 0, st>>>(t, ncand, val, sum), note_launch();
    const unsigned tblocks = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(num_sms * 4, cblocks)));
    double *partial = nullptr;
    PYCI_CUDA_TRY(pool.alloc(&partial, tblocks));
    enpt2_terms_kernel<NW, NWD><<<tblocks, 256, 0, st>>>(t, ncand, keep, sum, p.n, p.one, p.two, e, partial),
        note_launch();
    PYCI_CUDA_TRY(cudaGetLastError());
    std::vector<double> host(tblocks);
    int err = 0;
    PYCI_CUDA_TRY(cudaMemcpyAsync(host.data(), partial, sizeof(double) * tblocks, cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PYCI_CUDA_TRY(cudaStreamSynchronize(st));
    if (err) {
        set_error("device determinant table overflow");
        return PYCI_GPU_ECUDA;
    }
    double c = 0.0;
    for (double x : host)
        c += x;
    *correction = c;
    return PYCI_GPU_OK;
}

} // namespace

} // namespace pyci_gpu

using namespace pyci_gpu;

int enpt2_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t nocc_up, int64_t nocc_dn, int64_t ndet,
                 const uint64_t *dets, const double *coeffs, const double *one_mo, const double *two_mo, double energy,
                 double ecore, double eps, double *result) {
    cudaStream_t st = ctx->stream;
    const int64_t n = nbasis;
    const int nw = n <= 64 ? 1 : (n <= 128 ? 2 : (n <= 256 ? 4 : 0));
    if (nw == 0) {
        set_error("nbasis = %lld exceeds the 256 orbitals the GPU path supports", static_cast<long long>(n));
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (kind != PYCI_WFN_DOCI && kind != PYCI_WFN_FULLCI) {
        set_error("compute_enpt2 on the GPU supports DOCI and FullCI wave functions");
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (nocc_up > kMaxOcc || nocc_dn > kMaxOcc) {
        set_error("occupation numbers exceed the GPU path's limits (%d occupied)", kMaxOcc);
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (ndet >= INT32_MAX) {
        set_error("more than 2^31 - 1 determinants is not supported");
        return PYCI_GPU_EUNSUPPORTED;
    }
    *result = energy;
    if (ndet == 0)
        return PYCI_GPU_OK;
    // FullCI image (a DOCI determinant is its string in both spins,
    // FullCIWfn(const DOCIWfn &), pyci/src/fullciwfn.cpp:26-35), nw words per string.
    const int64_t host_nword = (n + 63) / 64;
    const int nwd = 2 * nw;
    std::vector<uint64_t> packed(static_cast<size_t>(ndet) * nwd, 0ULL);
    for (int64_t i = 0; i < ndet; ++i)
        for (int s = 0; s < 2; ++s)
            for (int64_t w = 0; w < host_nword; ++w)
                packed[i * nwd + s * nw + w] =
                    kind == PYCI_WFN_DOCI ? dets[i * host_nword + w] : dets[(i * 2 + s) * host_nword + w];
    Pool pool(st);
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
    p.kind = PYCI_WFN_FULLCI;
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
    double correction = 0.0;
    const double e = energy - ecore;
    switch (nw) {
    case 1: rc = run_enpt2<1, 2>(st, p, e, ctx->num_sms, &correction, pool); break;
    case 2: rc = run_enpt2<2, 4>(st, p, e, ctx->num_sms, &correction, pool); break;
    default: rc = run_enpt2<4, 8>(st, p, e, ctx->num_sms, &correction, pool); break;
    }
    if (rc == PYCI_GPU_OK) {
        int err = 0;
        PYCI_CUDA_TRY(cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            set_error("device determinant table overflow");
            return PYCI_GPU_ECUDA;
        }
        *result = energy + correction;
    }
    return rc;
}

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
