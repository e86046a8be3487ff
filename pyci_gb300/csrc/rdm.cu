// One- and two-particle reduced density matrices of a CI vector on the
// device, replacing compute_rdms (pyci/src/rdm.cpp:20-66 for DOCI, 269-530
// for FullCI), which walks the determinants serially on the host.
//
// One thread per determinant i replays the reference's loops: the diagonal
// terms c_i^2, and for every single / double excitation that reaches a
// determinant j > i of the wave function (table lookup on the determinant
// words) the terms c_i c_j (phase) with their transposed partners, added to
// the RDM arrays in device memory with FP64 atomics.  The set of terms and
// each term's value are the reference's; only the order of the FP64 sums
// differs (atomics), so entries agree to rounding (~1e-16 relative).
//
// Transition RDMs (compute_transition_rdms, pyci/src/rdm.cpp:634-902) run
// the same loops over wave function 1 with lookups in wave function 2: the
// diagonal terms use c1_i c2_(i in 2), every excitation found in 2 counts
// (not only j > i), and the transposed partner terms are not added.
//
// Layouts (as pyci.compute_rdms returns them): DOCI d0 = rdm1 [n][n],
// d2 = rdm2 [n][n]; FullCI rdm1 = [aa, bb] [2][n][n], rdm2 = [aaaa, bbbb,
// abab] [3][n][n][n][n]; GenCI (definition-based, rdm_genci_kernel) rdm1
// [n][n], rdm2 [n][n][n][n] over spin orbitals.
#include <cuda_runtime.h>

#include <vector>

#include "detops.cuh"
#include "internal.h"

namespace pyci_gpu {

namespace {

struct RdmParams {
    int kind;
    int n;
    int64_t ndet;
    const uint64_t *dets;
    const double *coeffs;
    DetTable table;          // lookups: wave function 2 (the wave function itself unless transition)
    const double *coeffs2;   // coefficients of the table's wave function
    double *rdm1, *rdm2;
};

__device__ __forceinline__ void add(double *a, int64_t idx, double v) { atomicAdd(a + idx, v); }

template<int NW, int NWD, bool TR>
__global__ void __launch_bounds__(128) rdm_kernel(RdmParams p) {
    const int64_t idet = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (idet >= p.ndet)
        return;
    const int64_t n1 = p.n, n2 = n1 * n1, n3 = n1 * n2, n4 = n2 * n2;
    uint64_t det[NWD], rdet[NWD];
#pragma unroll
    for (int w = 0; w < NWD; ++w)
        det[w] = rdet[w] = p.dets[idet * NWD + w];
    const double ci = p.coeffs[idet];
    auto find = [&]() { return p.table.find<NWD>(det); };
    const int64_t self = TR ? find() : idet;
    const double val1 = self != -1 ? ci * p.coeffs2[self] : 0.0;
    // The reference's partner test: j > i for the RDMs, found for transition RDMs.
    auto hit = [&](int64_t j) { return TR ? j != -1 : j > idet; };
    auto flip = [&](uint64_t *d, int a) { d[a >> 6] ^= 1ULL << (a & 63); };
    if (p.kind == PYCI_WFN_DOCI) {
        // pyci/src/rdm.cpp:33-64.
        double *d0 = p.rdm1, *d2 = p.rdm2;
        int16_t occ[kMaxOcc], vir[kMaxVir];
        const int no = occ_list<NW>(det, occ), nv = vir_list<NW>(det, p.n, vir);
        for (int i = 0; i < no; ++i) {
            const int k = occ[i];
            add(d0, k * (n1 + 1), val1);
            for (int j = i + 1; j < no; ++j) {
                const int l = occ[j];
                add(d2, n1 * k + l, val1);
                add(d2, n1 * l + k, val1);
            }
            for (int j = 0; j < nv; ++j) {
                const int l = vir[j];
                flip(det, k);
                flip(det, l);
                const int64_t jdet = find();
                flip(det, l);
                flip(det, k);
                if (hit(jdet)) {
                    const double val2 = ci * p.coeffs2[jdet];
                    add(d0, n1 * k + l, val2);
                    if (!TR)
                        add(d0, n1 * l + k, val2);
                }
            }
        }
        return;
    }
    // FullCI, pyci/src/rdm.cpp:295-528.
    double *aa = p.rdm1, *bb = p.rdm1 + n2;
    double *aaaa = p.rdm2, *bbbb = p.rdm2 + n4, *abab = p.rdm2 + 2 * n4;
    auto at = [&](int64_t a, int64_t b, int64_t c, int64_t d) { return a * n3 + b * n2 + c * n1 + d; };
    uint64_t *up = det, *dn = det + NW;
    const uint64_t *rup = rdet, *rdn = rdet + NW;
    int16_t ou[kMaxOcc], od[kMaxOcc], vu[kMaxVir], vd[kMaxVir];
    const int nou = occ_list<NW>(rup, ou), nod = occ_list<NW>(rdn, od);
    const int nvu = vir_list<NW>(rup, p.n, vu), nvd = vir_list<NW>(rdn, p.n, vd);
    // Same-spin terms of one spin block (s = 0: alpha, 1: beta); `other`
    // lists the opposite spin's occupied orbitals.
    for (int s = 0; s < 2; ++s) {
        const int16_t *oc = s ? od : ou, *vc = s ? vd : vu, *oo = s ? ou : od;
        const int no = s ? nod : nou, nv = s ? nvd : nvu, nother = s ? nou : nod;
        uint64_t *mine = s ? dn : up;
        const uint64_t *rmine = s ? rdn : rup;
        double *one = s ? bb : aa, *same = s ? bbbb : aaaa;
        for (int i = 0; i < no; ++i) {
            const int ii = oc[i];
            add(one, (n1 + 1) * ii, val1);
            for (int k = i + 1; k < no; ++k) {
                const int kk = oc[k];
                add(same, at(ii, kk, ii, kk), val1);
                add(same, at(ii, kk, kk, ii), -val1);
                add(same, at(kk, ii, ii, kk), -val1);
                add(same, at(kk, ii, kk, ii), val1);
            }
            if (s == 0) {
                for (int k = 0; k < nod; ++k)
                    add(abab, at(ii, od[k], ii, od[k]), val1);
            }
            for (int j = 0; j < nv; ++j) {
                const int jj = vc[j];
                flip(mine, ii);
                flip(mine, jj);
                const double sign = phase_single<NW>(rmine, ii, jj);
                int64_t jdet = find();
                if (hit(jdet)) {
                    const double val2 = ci * p.coeffs2[jdet] * sign;
                    add(one, ii * n1 + jj, val2);
                    if (!TR)
                        add(one, jj * n1 + ii, val2);
                    for (int k = 0; k < no; ++k) {
                        if (k == i)
                            continue;
                        const int kk = oc[k];
                        add(same, at(ii, kk, jj, kk), val2);
                        add(same, at(ii, kk, kk, jj), -val2);
                        add(same, at(kk, ii, kk, jj), val2);
                        add(same, at(kk, ii, jj, kk), -val2);
                        if (!TR) {
                            add(same, at(jj, kk, ii, kk), val2);
                            add(same, at(jj, kk, kk, ii), -val2);
                            add(same, at(kk, jj, ii, kk), -val2);
                            add(same, at(kk, jj, kk, ii), val2);
                        }
                    }
                    for (int k = 0; k < nother; ++k) {
                        const int kk = oo[k];
                        if (s == 0) {
                            add(abab, at(ii, kk, jj, kk), val2);
                            if (!TR)
                                add(abab, at(jj, kk, ii, kk), val2);
                        } else {
                            add(abab, at(kk, ii, kk, jj), val2);
                            if (!TR)
                                add(abab, at(kk, jj, kk, ii), val2);
                        }
                    }
                }
                if (s == 0) {
                    // alpha-beta doubles: the alpha single ii -> jj with a beta single.
                    for (int k = 0; k < nod; ++k) {
                        const int kk = od[k];
                        for (int l = 0; l < nvd; ++l) {
                            const int ll = vd[l];
                            flip(dn, kk);
                            flip(dn, ll);
                            jdet = find();
                            if (hit(jdet)) {
                                const double val2 = ci * p.coeffs2[jdet] * sign * phase_single<NW>(rdn, kk, ll);
                                add(abab, at(ii, kk, jj, ll), val2);
                                if (!TR)
                                    add(abab, at(jj, ll, ii, kk), val2);
                            }
                            flip(dn, ll);
                            flip(dn, kk);
                        }
                    }
                }
                for (int k = i + 1; k < no; ++k) {
                    const int kk = oc[k];
                    for (int l = j + 1; l < nv; ++l) {
                        const int ll = vc[l];
                        flip(mine, kk);
                        flip(mine, ll);
                        jdet = find();
                        if (hit(jdet)) {
                            const double val2 = ci * p.coeffs2[jdet] * phase_double<NW>(rmine, ii, kk, jj, ll);
                            add(same, at(ii, kk, jj, ll), val2);
                            add(same, at(ii, kk, ll, jj), -val2);
                            add(same, at(kk, ii, jj, ll), -val2);
                            add(same, at(kk, ii, ll, jj), val2);
                            if (!TR) {
                                add(same, at(jj, ll, ii, kk), val2);
                                add(same, at(jj, ll, kk, ii), -val2);
                                add(same, at(ll, jj, ii, kk), -val2);
                                add(same, at(ll, jj, kk, ii), val2);
                            }
                        }
                        flip(mine, ll);
                        flip(mine, kk);
                    }
                }
                flip(mine, jj);
                flip(mine, ii);
            }
        }
    }
}

// GenCI spin-orbital RDMs from their definition (no reference counterpart:
// the reference's GenCI compute_rdms, pyci/src/rdm.cpp:532-632, writes past
// its output arrays and repeats index factors).  One thread per ket
// determinant J (wave function p.dets / p.coeffs) walks its diagonal, single
// and double excitations I, looks I up in the bra (p.table / p.coeffs2) and
// adds c_I c_J <I| a+_p a_q |J> and c_I c_J <I| a+_p a+_q a_s a_r |J> with
// every antisymmetric image (rdm1 [n][n], rdm2 [n][n][n][n]).  The sign of an
// operator string is (-1) to the number of occupied orbitals below each
// acted orbital, applied right to left.
template<int NW>
__device__ __forceinline__ int below_sign(const uint64_t *d, int p) {
    int c = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        if (64 * (w + 1) <= p)
            c += __popcll(d[w]);
        else if (64 * w < p)
            c += __popcll(d[w] & ((1ULL << (p - 64 * w)) - 1));
    }
    return (c & 1) ? -1 : 1;
}

template<int NW>
__global__ void __launch_bounds__(128) rdm_genci_kernel(RdmParams p) {
    const int64_t jdet = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (jdet >= p.ndet)
        return;
    const int64_t n1 = p.n, n2 = n1 * n1, n3 = n1 * n2;
    uint64_t det[NW], kdet[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w)
        det[w] = kdet[w] = p.dets[jdet * NW + w];
    const double cj = p.coeffs[jdet];
    auto flip = [&](uint64_t *d, int a) { d[a >> 6] ^= 1ULL << (a & 63); };
    int16_t occ[kMaxOcc], vir[kMaxVir];
    const int no = occ_list<NW>(det, occ), nv = vir_list<NW>(det, p.n, vir);
    double *r1 = p.rdm1, *r2 = p.rdm2;
    int64_t idet = p.table.find<NW>(det);
    if (idet != -1) {
        const double v = p.coeffs2[idet] * cj;
        for (int x = 0; x < no; ++x) {
            const int q0 = occ[x];
            add(r1, q0 * (n1 + 1), v);
            for (int y = 0; y < no; ++y) {
                const int q1 = occ[y];
                if (q1 == q0)
                    continue;
                add(r2, q0 * n3 + q1 * n2 + q0 * n1 + q1, v);
                add(r2, q0 * n3 + q1 * n2 + q1 * n1 + q0, -v);
            }
        }
    }
    for (int x = 0; x < no; ++x) {
        const int i = occ[x];
        for (int y = 0; y < nv; ++y) {
            const int a = vir[y];
            int sg = below_sign<NW>(det, i);
            flip(det, i);
            sg *= below_sign<NW>(det, a);
            flip(det, a);
            idet = p.table.find<NW>(det);
            if (idet != -1) {
                const double v = p.coeffs2[idet] * cj * sg;
                add(r1, a * n1 + i, v);
                for (int z = 0; z < no; ++z) {
                    const int k = occ[z];
                    if (k == i)
                        continue;
                    add(r2, a * n3 + k * n2 + i * n1 + k, v);
                    add(r2, k * n3 + a * n2 + i * n1 + k, -v);
                    add(r2, a * n3 + k * n2 + k * n1 + i, -v);
                    add(r2, k * n3 + a * n2 + k * n1 + i, v);
                }
            }
            flip(det, a);
            flip(det, i);
        }
    }
    for (int x = 0; x < no; ++x)
        for (int x2 = x + 1; x2 < no; ++x2)
            for (int y = 0; y < nv; ++y)
                for (int y2 = y + 1; y2 < nv; ++y2) {
                    const int i = occ[x], j = occ[x2], a = vir[y], b = vir[y2];
                    int sg = below_sign<NW>(det, i);
                    flip(det, i);
                    sg *= below_sign<NW>(det, j);
                    flip(det, j);
                    sg *= below_sign<NW>(det, b);
                    flip(det, b);
                    sg *= below_sign<NW>(det, a);
                    flip(det, a);
                    idet = p.table.find<NW>(det);
                    if (idet != -1) {
                        const double v = p.coeffs2[idet] * cj * sg;
                        add(r2, a * n3 + b * n2 + i * n1 + j, v);
                        add(r2, b * n3 + a * n2 + i * n1 + j, -v);
                        add(r2, a * n3 + b * n2 + j * n1 + i, -v);
                        add(r2, b * n3 + a * n2 + j * n1 + i, v);
                    }
#pragma unroll
                    for (int w = 0; w < NW; ++w)
                        det[w] = kdet[w];
                }
}

template<bool TR>
void launch_rdm(int nwd, int kind, unsigned blocks, cudaStream_t st, const RdmParams &p) {
    switch (nwd) {
    case 1: rdm_kernel<1, 1, TR><<<blocks, 128, 0, st>>>(p); break;
    case 2:
        if (kind == PYCI_WFN_FULLCI)
            rdm_kernel<1, 2, TR><<<blocks, 128, 0, st>>>(p);
        else
            rdm_kernel<2, 2, TR><<<blocks, 128, 0, st>>>(p);
        break;
    case 4:
        if (kind == PYCI_WFN_FULLCI)
            rdm_kernel<2, 4, TR><<<blocks, 128, 0, st>>>(p);
        else
            rdm_kernel<4, 4, TR><<<blocks, 128, 0, st>>>(p);
        break;
    default: rdm_kernel<4, 8, TR><<<blocks, 128, 0, st>>>(p); break;
    }
}

void launch_rdm_genci(int nw, unsigned blocks, cudaStream_t st, const RdmParams &p) {
    switch (nw) {
    case 1: rdm_genci_kernel<1><<<blocks, 128, 0, st>>>(p); break;
    case 2: rdm_genci_kernel<2><<<blocks, 128, 0, st>>>(p); break;
    default: rdm_genci_kernel<4><<<blocks, 128, 0, st>>>(p); break;
    }
}

} // namespace

} // namespace pyci_gpu

using namespace pyci_gpu;

int rdm_compute_device(pyci_gpu_ctx *ctx, int kind, int64_t nbasis, int64_t ndet, const uint64_t *dets,
                       const double *coeffs, int64_t ndet2, const uint64_t *dets2, const double *coeffs2,
                       double *rdm1, double *rdm2) {
    const bool tr = dets2 != nullptr;
    cudaStream_t st = ctx->stream;
    const int64_t n = nbasis;
    const int nw = n <= 64 ? 1 : (n <= 128 ? 2 : (n <= 256 ? 4 : 0));
    if (nw == 0) {
        set_error("nbasis = %lld exceeds the 256 orbitals the GPU path supports", static_cast<long long>(n));
        return PYCI_GPU_EUNSUPPORTED;
    }
    if (kind != PYCI_WFN_DOCI && kind != PYCI_WFN_FULLCI && kind != PYCI_WFN_GENCI) {
        set_error("compute_rdms on the GPU supports DOCI, FullCI and (definition-based) GenCI wave functions");
        return PYCI_GPU_EUNSUPPORTED;
    }
    const bool genci = kind == PYCI_WFN_GENCI;
    if (ndet >= INT32_MAX || ndet2 >= INT32_MAX) {
        set_error("more than 2^31 - 1 determinants is not supported");
        return PYCI_GPU_EUNSUPPORTED;
    }
    const int nstr = kind == PYCI_WFN_FULLCI ? 2 : 1;
    const int64_t n2 = n * n;
    const int64_t len1 = (kind == PYCI_WFN_FULLCI ? 2 : 1) * n2;
    const int64_t len2 = kind == PYCI_WFN_FULLCI ? 3 * n2 * n2 : (genci ? n2 * n2 : n2);
    const int64_t host_nword = (n + 63) / 64;
    const int nwd = nstr * nw;
    std::vector<void *> bufs;
    auto release = [&]() {
        for (void *b : bufs)
            cudaFreeAsync(b, st);
        cudaStreamSynchronize(st);
    };
    auto alloc = [&](void **p, size_t bytes) {
        cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 1, st);
        if (e == cudaSuccess)
            bufs.push_back(*p);
        return e;
    };
    // Determinants of both wave functions (the second only for transition
    // RDMs), repacked to nw words per string.
    const int64_t nall = ndet + (tr ? ndet2 : 0);
    std::vector<uint64_t> packed(static_cast<size_t>(nall) * nwd, 0ULL);
    for (int64_t i = 0; i < nall; ++i) {
        const uint64_t *src = i < ndet ? dets + i * nstr * host_nword : dets2 + (i - ndet) * nstr * host_nword;
        for (int s = 0; s < nstr; ++s)
            for (int64_t w = 0; w < host_nword; ++w)
                packed[i * nwd + s * nw + w] = src[s * host_nword + w];
    }
    uint64_t *d_dets = nullptr;
    double *d_coef = nullptr, *d_r1 = nullptr, *d_r2 = nullptr;
    int *d_err = nullptr;
    cudaError_t e = cudaSuccess;
    if ((e = alloc(reinterpret_cast<void **>(&d_dets), sizeof(uint64_t) * packed.size())) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void **>(&d_coef), sizeof(double) * nall)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void **>(&d_r1), sizeof(double) * len1)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void **>(&d_r2), sizeof(double) * len2)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void **>(&d_err), sizeof(int))) != cudaSuccess) {
        release();
        return cuda_status(e, "cudaMallocAsync (RDM workspace)");
    }
    int32_t *slots = nullptr;
    uint64_t mask = 0;
    int rc = PYCI_GPU_OK;
    do {
        if ((e = cudaMemcpyAsync(d_dets, packed.data(), sizeof(uint64_t) * packed.size(), cudaMemcpyHostToDevice,
                                 st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_coef, coeffs, sizeof(double) * ndet, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (tr && ndet2 > 0 &&
             (e = cudaMemcpyAsync(d_coef + ndet, coeffs2, sizeof(double) * ndet2, cudaMemcpyHostToDevice, st)) !=
                 cudaSuccess) ||
            (e = cudaMemsetAsync(d_r1, 0, sizeof(double) * len1, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_r2, 0, sizeof(double) * len2, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_err, 0, sizeof(int), st)) != cudaSuccess) {
            rc = cuda_status(e, "RDM upload");
            break;
        }
        // The lookup table covers wave function 2 (itself unless transition).
        const uint64_t *tdets = tr ? d_dets + ndet * nwd : d_dets;
        const int64_t tndet = tr ? ndet2 : ndet;
        if ((rc = det_table_build(tdets, tndet, nwd, st, d_err, &slots, &mask)))
            break;
        bufs.push_back(slots);
        RdmParams p{};
        p.kind = kind;
        p.n = static_cast<int>(n);
        p.ndet = ndet;
        p.dets = d_dets;
        p.coeffs = d_coef;
        p.table = DetTable{slots, tdets, mask, nwd};
        p.coeffs2 = tr ? d_coef + ndet : d_coef;
        p.rdm1 = d_r1;
        p.rdm2 = d_r2;
        if (genci) {
            // Ket-driven: threads over wave function 2 (the wave function
            // itself for compute_rdms), lookups in wave function 1 (the bra).
            p.ndet = tr ? ndet2 : ndet;
            p.dets = tr ? d_dets + ndet * nwd : d_dets;
            p.coeffs = tr ? d_coef + ndet : d_coef;
            p.coeffs2 = d_coef;
            if (tr) {
                int32_t *slots1 = nullptr;
                uint64_t mask1 = 0;
                if ((rc = det_table_build(d_dets, ndet, nwd, st, d_err, &slots1, &mask1)))
                    break;
                bufs.push_back(slots1);
                p.table = DetTable{slots1, d_dets, mask1, nwd};
            }
        }
        const unsigned blocks = static_cast<unsigned>((p.ndet + 127) / 128);
        if (blocks) {
            if (genci)
                launch_rdm_genci(nwd, blocks, st, p);
            else if (tr)
                launch_rdm<true>(nwd, kind, blocks, st, p);
            else
                launch_rdm<false>(nwd, kind, blocks, st, p);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) {
                rc = cuda_status(e, "RDM kernel");
                break;
            }
        }
        int err = 0;
        if ((e = cudaMemcpyAsync(rdm1, d_r1, sizeof(double) * len1, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(rdm2, d_r2, sizeof(double) * len2, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            rc = cuda_status(e, "RDM download");
            break;
        }
        if (err) {
            set_error("device determinant table overflow");
            rc = PYCI_GPU_ECUDA;
        }
    } while (false);
    release();
    return rc;
}
