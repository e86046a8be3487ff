// Host side of pyci_gb300: a pybind11 module with the class and method names,
// keyword names, defaults and error types of the reference's `pyci._pyci`
// module (pyci/src/binding.cpp:29-1088) for the CI hot path --
// secondquant_op, the DOCI / FullCI / GenCI wave functions and sparse_op.
// Determinant sets live on the host (as in the reference); every sparse_op
// operation goes through the C ABI of libpyci_gb300.so (include/pyci_gb300.h),
// which runs on the GPU.  There is no CPU implementation of the operator: a
// missing or unusable GPU raises RuntimeError.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <memory>
#include <mutex>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "pyci_gb300.h"

namespace py = pybind11;

namespace {

typedef uint64_t ulong_t;
template<typename T>
using Array = py::array_t<T, py::array::c_style | py::array::forcecast>;

long g_threads = 1;

// ---------------------------------------------------------------- errors

[[noreturn]] void raise_status(int rc) {
    const std::string msg = pyci_gpu_last_error();
    switch (rc) {
    case PYCI_GPU_EINVAL:
        throw std::invalid_argument(msg);
    case PYCI_GPU_ETYPE:
        throw py::type_error(msg);
    default:
        throw std::runtime_error(msg);
    }
}

inline void check(int rc) {
    if (rc != PYCI_GPU_OK)
        raise_status(rc);
}

// One context (device 0 unless PYCI_GPU_DEVICE is set) shared by all operators.
std::shared_ptr<pyci_gpu_ctx> default_ctx() {
    static std::mutex mu;
    static std::shared_ptr<pyci_gpu_ctx> ctx;
    std::lock_guard<std::mutex> lock(mu);
    if (!ctx) {
        const char *env = std::getenv("PYCI_GPU_DEVICE");
        const int dev = env ? std::atoi(env) : 0;
        pyci_gpu_ctx *raw = nullptr;
        const int rc = pyci_gpu_ctx_create(dev, &raw);
        if (rc != PYCI_GPU_OK)
            throw std::runtime_error(std::string("pyci_gb300 needs a CUDA GPU: ") + pyci_gpu_last_error());
        ctx.reset(raw, [](pyci_gpu_ctx *c) { pyci_gpu_ctx_destroy(c); });
    }
    return ctx;
}

// --------------------------------------------------------------- combinatorics

long binomial(long n, long k) {
    if (k < 0 || n < 0 || k > n)
        return 0;
    if (k == 0 || k == n)
        return 1;
    if (k > n / 2)
        k = n - k;
    __int128 b = 1;
    for (long d = 1; d <= k; ++d) {
        b = b * (n - k + d) / d;
        if (b > static_cast<__int128>(INT64_MAX))
            return INT64_MAX;
    }
    return static_cast<long>(b);
}

long nword_det(long n) { return n / 64 + ((n % 64) ? 1 : 0); }

void fill_det(long nocc, const long *occs, ulong_t *det) {
    for (long i = 0; i < nocc; ++i)
        det[occs[i] / 64] |= 1ULL << (occs[i] % 64);
}

long fill_occs(long nword, const ulong_t *det, long *occs) {
    long j = 0;
    for (long i = 0; i < nword; ++i) {
        ulong_t w = det[i];
        while (w) {
            occs[j++] = __builtin_ctzll(w) + i * 64;
            w &= w - 1;
        }
    }
    return j;
}

long fill_virs(long nword, long nbasis, const ulong_t *det, long *virs) {
    long j = 0;
    for (long i = 0; i < nword; ++i) {
        const long left = nbasis - i * 64;
        const ulong_t mask = left >= 64 ? ~0ULL : ((1ULL << left) - 1);
        ulong_t w = ~det[i] & mask;
        while (w) {
            virs[j++] = __builtin_ctzll(w) + i * 64;
            w &= w - 1;
        }
    }
    return j;
}

// pyci/src/common.cpp:115-122
void next_colex(long *idx) {
    long i = 0;
    while (idx[i + 1] - idx[i] == 1) {
        idx[i] = i;
        ++i;
    }
    ++(idx[i]);
}

// pyci/src/common.cpp:139-153
void unrank_colex(long nbasis, long nocc, long rank, long *occs) {
    for (long i = 0; i < nocc; ++i) {
        const long j = nocc - i;
        long b = binomial(nbasis, j);
        if (b <= rank) {
            for (long k = 0; k < j; ++k)
                occs[k] = k;
            break;
        }
        while (b > rank)
            b = binomial(--nbasis, j);
        occs[j - 1] = nbasis;
        rank -= b;
    }
}

void fill_hartreefock_det(long nocc, ulong_t *det) {
    long i = 0;
    while (nocc >= 64) {
        det[i++] = ~0ULL;
        nocc -= 64;
    }
    if (nocc)
        det[i] = (1ULL << nocc) - 1;
}

// --------------------------------------------------------------- det index

// Open-addressing map from determinant words to insertion index.
class DetIndex {
public:
    void clear() {
        slots_.clear();
        count_ = 0;
    }
    bool built() const { return !slots_.empty(); }

    long find(const std::vector<ulong_t> &dets, long nw, const ulong_t *d) const {
        if (slots_.empty())
            return -1;
        size_t s = hash(d, nw) & mask_;
        for (;;) {
            const long idx = slots_[s];
            if (idx < 0)
                return -1;
            if (!std::memcmp(&dets[idx * nw], d, sizeof(ulong_t) * nw))
                return idx;
            s = (s + 1) & mask_;
        }
    }

    // Insert index i whose words are already at dets[i * nw].
    void insert(const std::vector<ulong_t> &dets, long nw, long i) {
        if (2 * (count_ + 1) > static_cast<long>(slots_.size()))
            rehash(dets, nw, std::max<size_t>(16, slots_.size() * 2));
        place(dets, nw, i);
        ++count_;
    }

    void rebuild(const std::vector<ulong_t> &dets, long nw, long ndet) {
        size_t cap = 16;
        while (cap < static_cast<size_t>(2 * ndet + 2))
            cap <<= 1;
        slots_.assign(cap, -1);
        mask_ = cap - 1;
        count_ = 0;
        for (long i = 0; i < ndet; ++i) {
            place(dets, nw, i);
            ++count_;
        }
    }

private:
    static size_t hash(const ulong_t *d, long nw) {
        uint64_t h = 0x84222325cbf29ce4ULL;
        for (long i = 0; i < nw; ++i) {
            uint64_t x = h ^ (d[i] + 0x9e3779b97f4a7c15ULL * static_cast<uint64_t>(i + 1));
            x ^= x >> 30;
            x *= 0xbf58476d1ce4e5b9ULL;
            x ^= x >> 27;
            x *= 0x94d049bb133111ebULL;
            x ^= x >> 31;
            h = x;
        }
        return static_cast<size_t>(h);
    }
    void place(const std::vector<ulong_t> &dets, long nw, long i) {
        size_t s = hash(&dets[i * nw], nw) & mask_;
        while (slots_[s] >= 0)
            s = (s + 1) & mask_;
        slots_[s] = i;
    }
    void rehash(const std::vector<ulong_t> &dets, long nw, size_t cap) {
        slots_.assign(cap, -1);
        mask_ = cap - 1;
        const long n = count_;
        count_ = 0;
        for (long i = 0; i < n; ++i) {
            place(dets, nw, i);
            ++count_;
        }
    }
    std::vector<long> slots_;
    size_t mask_ = 0;
    long count_ = 0;
};

// --------------------------------------------------------------- Hamiltonian

// pyci::SQuantOp (pyci/include/pyci.h:285-302, pyci/src/squantop.cpp).
struct SQuantOp {
    long nbasis = 0;
    double ecore = 0.0;
    Array<double> one_mo, two_mo, h, v, w;

    void derive() {
        // pyci/src/squantop.cpp:175-182
        const long n1 = nbasis, n2 = n1 * n1, n3 = n2 * n1;
        h = Array<double>(n1);
        v = Array<double>({n1, n1});
        w = Array<double>({n1, n1});
        const double *two = two_mo.data();
        const double *one = one_mo.data();
        double *ph = h.mutable_data(), *pv = v.mutable_data(), *pw = w.mutable_data();
        long k = 0, l = 0;
        for (long i = 0; i != n1; ++i) {
            ph[k++] = one[i * (n1 + 1)];
            for (long j = 0; j != n1; ++j) {
                pv[l] = two[i * n3 + i * n2 + j * n1 + j];
                pw[l++] = two[i * n3 + j * n2 + i * n1 + j] * 2 - two[i * n3 + j * n2 + j * n1 + i];
            }
        }
    }

    SQuantOp(double e, Array<double> mo1, Array<double> mo2) : ecore(e), one_mo(mo1), two_mo(mo2) {
        if (mo1.ndim() != 2 || mo1.shape(0) != mo1.shape(1))
            throw std::invalid_argument("one_mo must be a square matrix");
        nbasis = mo1.shape(0);
        if (mo2.ndim() != 4 || mo2.shape(0) != nbasis || mo2.shape(1) != nbasis || mo2.shape(2) != nbasis ||
            mo2.shape(3) != nbasis)
            throw std::invalid_argument("two_mo must have shape (n, n, n, n)");
        derive();
    }

    // FCIDUMP reader (pyci/src/squantop.cpp:79-161).
    explicit SQuantOp(const std::string &filename) {
        std::ifstream f(filename);
        if (f.fail())
            throw std::ios_base::failure("Failed to read the FCIDUMP file " + filename);
        std::string header, line;
        bool ended = false;
        while (std::getline(f, line)) {
            if (line.find("&END") != std::string::npos || line.find("/") != std::string::npos) {
                ended = true;
                break;
            }
            header += " " + line;
        }
        if (!ended || f.eof())
            throw std::ios_base::failure("FCIDUMP has the wrong header");
        std::smatch m;
        if (!std::regex_search(header, m, std::regex(R"(NORB[ ]*=[ ]*(\d+))")))
            throw std::invalid_argument("NORB is not found.");
        nbasis = std::stol(m[1]);
        if (std::regex_search(header, m, std::regex(R"(UHF[ ]*=[ .]*(FALSE|TRUE|false|true))"))) {
            std::string u = m[1];
            std::transform(u.begin(), u.end(), u.begin(), ::tolower);
            if (u == "true")
                throw std::runtime_error("Unrestricted FCIDUMP not implemented");
        }
        const long n1 = nbasis, n2 = n1 * n1, n3 = n2 * n1;
        one_mo = Array<double>({n1, n1});
        two_mo = Array<double>({n1, n1, n1, n1});
        double *one = one_mo.mutable_data(), *two = two_mo.mutable_data();
        std::fill(one, one + n2, 0.0);
        std::fill(two, two + n3 * n1, 0.0);
        ecore = 0.0;
        double x;
        long i, j, k, l;
        while (f >> x >> i >> j >> k >> l) {
            if (i && j && k && l) {
                --i, --j, --k, --l;
                two[i * n3 + k * n2 + j * n1 + l] = x;
                two[k * n3 + i * n2 + l * n1 + j] = x;
                two[j * n3 + k * n2 + i * n1 + l] = x;
                two[i * n3 + l * n2 + j * n1 + k] = x;
                two[j * n3 + l * n2 + i * n1 + k] = x;
                two[l * n3 + j * n2 + k * n1 + i] = x;
                two[k * n3 + j * n2 + l * n1 + i] = x;
                two[l * n3 + i * n2 + k * n1 + j] = x;
            } else if (i && j) {
                --i, --j;
                one[i * n1 + j] = x;
                one[j * n1 + i] = x;
            } else {
                ecore = x;
            }
        }
        derive();
    }

    // FCIDUMP writer (pyci/src/squantop.cpp:185-223).
    void to_file(const std::string &filename, long nelec, long ms2, double tol) const {
        const long n1 = nbasis, n2 = n1 * n1, n3 = n2 * n1;
        std::ofstream f(filename);
        if (f.fail())
            throw std::ios_base::failure("Failed to open the FCIDUMP file " + filename);
        f << "&FCIDUMP\nNORB=" << nbasis << ",\nNELEC=" << nelec << ",\nMS2=" << ms2
          << ",\nUHF=.FALSE.,\nORBSYM=";
        for (long i = 0; i != nbasis; ++i)
            f << "1,";
        f << "\nISYM=1,\n&END\n";
        const double *two = two_mo.data(), *one = one_mo.data();
        for (long i = 0; i != nbasis; ++i)
            for (long j = 0; j <= i; ++j)
                for (long k = 0; k != nbasis; ++k)
                    for (long l = 0; l <= k; ++l)
                        if ((i * (i + 1)) / 2 + j >= (k * (k + 1)) / 2 + l) {
                            const double val = two[i * n3 + k * n2 + j * n1 + l];
                            if (std::abs(val) > tol)
                                f << std::setw(28) << std::setprecision(20) << std::scientific << val << ' '
                                  << i + 1 << ' ' << j + 1 << ' ' << k + 1 << ' ' << l + 1 << "\n";
                        }
        for (long i = 0; i != nbasis; ++i)
            for (long j = 0; j <= i; ++j) {
                const double val = one[i * n1 + j];
                if (std::abs(val) > tol)
                    f << std::setw(28) << std::setprecision(20) << std::scientific << val << ' ' << i + 1
                      << ' ' << j + 1 << " 0 0\n";
            }
        f << std::setw(28) << std::setprecision(20) << std::scientific << ecore << " 0 0 0 0\n";
    }
};

// --------------------------------------------------------------- wave functions

// pyci::Wfn (pyci/include/pyci.h:306-330, pyci/src/wfn.cpp).
struct Wfn {
    long nbasis = 0, nocc = 0, nocc_up = 0, nocc_dn = 0, nvir = 0, nvir_up = 0, nvir_dn = 0;
    long ndet = 0, nword = 0, nword2 = 0, maxrank_up = 0, maxrank_dn = 0;
    std::vector<ulong_t> dets;
    mutable DetIndex index;
    mutable bool index_valid = false;
    bool full_colex = false; // dets are exactly add_all_dets' list

    virtual ~Wfn() = default;
    virtual long words() const = 0; // words per determinant
    virtual int kind() const = 0;

    void init(long nb, long nu, long nd) {
        // pyci/src/wfn.cpp:51-70
        if (nd < 0)
            throw std::domain_error("nocc_dn is < 0");
        if (nu < nd)
            throw std::domain_error("nocc_up is < nocc_dn");
        if (nb < nu)
            throw std::domain_error("nbasis is < nocc_up");
        nbasis = nb;
        nocc = nu + nd;
        nocc_up = nu;
        nocc_dn = nd;
        nvir = nb * 2 - nu - nd;
        nvir_up = nb - nu;
        nvir_dn = nb - nd;
        ndet = 0;
        nword = nword_det(nb);
        nword2 = nword * 2;
        maxrank_up = binomial(nb, nu);
        maxrank_dn = binomial(nb, nd);
    }

    long length() const { return ndet; }

    void ensure_index() const {
        if (!index_valid) {
            index.rebuild(dets, words(), ndet);
            index_valid = true;
        }
    }

    long index_det(const ulong_t *d) const {
        ensure_index();
        return index.find(dets, words(), d);
    }

    long add_det(const ulong_t *d) {
        const long nw = words();
        ensure_index();
        if (index.find(dets, nw, d) >= 0)
            return -1;
        dets.insert(dets.end(), d, d + nw);
        index.insert(dets, nw, ndet);
        full_colex = false;
        return ndet++;
    }

    void reserve(long n) { dets.reserve(static_cast<size_t>(n * words())); }
    void squeeze() { dets.shrink_to_fit(); }

    void to_file(const std::string &filename) const {
        // pyci/src/onespinwfn.cpp:78-90, pyci/src/twospinwfn.cpp:81-93
        std::ofstream file(filename, std::ios::out | std::ios::binary);
        bool ok = file.write(reinterpret_cast<const char *>(&ndet), sizeof(long)) &&
                  file.write(reinterpret_cast<const char *>(&nbasis), sizeof(long)) &&
                  file.write(reinterpret_cast<const char *>(&nocc_up), sizeof(long)) &&
                  file.write(reinterpret_cast<const char *>(&nocc_dn), sizeof(long)) &&
                  file.write(reinterpret_cast<const char *>(dets.data()), sizeof(ulong_t) * ndet * words());
        if (!ok)
            throw std::ios_base::failure("error writing file");
    }

    void read_file(const std::string &filename, bool two_spin) {
        std::ifstream file(filename, std::ios::in | std::ios::binary);
        long n, nb, nu, nd;
        if (!(file.read(reinterpret_cast<char *>(&n), sizeof(long)) &&
              file.read(reinterpret_cast<char *>(&nb), sizeof(long)) &&
              file.read(reinterpret_cast<char *>(&nu), sizeof(long)) &&
              file.read(reinterpret_cast<char *>(&nd), sizeof(long))))
            throw std::ios_base::failure("error in file");
        const long nw = nword_det(nb) * (two_spin ? 2 : 1);
        std::vector<ulong_t> buf(static_cast<size_t>(n * nw));
        if (!file.read(reinterpret_cast<char *>(buf.data()), sizeof(ulong_t) * n * nw))
            throw std::ios_base::failure("error in file");
        init(nb, nu, nd);
        dets = std::move(buf);
        ndet = n;
        index_valid = false;
        full_colex = false;
    }

    // Replace the contents with `n` determinants (duplicates keep their first index).
    void assign_dets(const ulong_t *src, long n) {
        const long nw = words();
        dets.clear();
        ndet = 0;
        index.clear();
        index.rebuild(dets, nw, 0);
        index_valid = true;
        full_colex = false;
        for (long i = 0; i < n; ++i) {
            // The reference overwrites the dict entry for repeated dets but keeps
            // every row (pyci/src/onespinwfn.cpp:52-58); keep every row too.
            dets.insert(dets.end(), src + i * nw, src + (i + 1) * nw);
            ++ndet;
        }
        index_valid = false;
    }
};

struct OneSpinWfn : Wfn {
    long words() const override { return nword; }

    // pyci/src/onespinwfn.cpp:173-217
    void add_all_dets(long nthread) {
        if (maxrank_up == INT64_MAX)
            throw std::domain_error("cannot generate > 2 ** 63 determinants");
        if (nthread == -1)
            nthread = g_threads;
        nthread = std::max(1L, nthread);
        const long nd = maxrank_up;
        while (nthread > 1 && (nd + nthread - 1) / nthread < 1024)
            nthread /= 2;
        dets.assign(static_cast<size_t>(nd * nword), 0ULL);
        auto work = [&](long start, long end) {
            std::vector<long> occs(nocc_up + 1);
            unrank_colex(nbasis, nocc_up, start, occs.data());
            occs[nocc_up] = nbasis + 1;
            for (long i = start; i < end; ++i) {
                fill_det(nocc_up, occs.data(), &dets[i * nword]);
                next_colex(occs.data());
            }
        };
        std::vector<std::thread> th;
        for (long t = 0; t < nthread; ++t) {
            const long s = nd * t / nthread, e = nd * (t + 1) / nthread;
            th.emplace_back(work, s, e);
        }
        for (auto &x : th)
            x.join();
        ndet = nd;
        index_valid = false;
        full_colex = true;
    }

    // pyci/src/onespinwfn.cpp:219-244 (same insertion order).
    void add_excited_dets(const ulong_t *rdet, long e) {
        const long no = binomial(nocc_up, e), nv = binomial(nvir_up, e);
        std::vector<ulong_t> det(nword);
        std::vector<long> occs(nocc_up), virs(nvir_up), oi(e + 1), vi(e + 1);
        fill_occs(nword, rdet, occs.data());
        fill_virs(nword, nbasis, rdet, virs.data());
        for (long k = 0; k < e; ++k)
            vi[k] = k;
        vi[e] = nvir_up + 1;
        for (long i = 0; i < nv; ++i) {
            for (long k = 0; k < e; ++k)
                oi[k] = k;
            oi[e] = nocc_up + 1;
            for (long j = 0; j < no; ++j) {
                std::memcpy(det.data(), rdet, sizeof(ulong_t) * nword);
                for (long k = 0; k < e; ++k) {
                    const long a = occs[oi[k]], b = virs[vi[k]];
                    det[a / 64] &= ~(1ULL << (a % 64));
                    det[b / 64] |= 1ULL << (b % 64);
                }
                add_det(det.data());
                next_colex(oi.data());
            }
            next_colex(vi.data());
        }
    }
};

struct TwoSpinWfn : Wfn {
    long words() const override { return nword2; }

    // pyci/src/twospinwfn.cpp:181-245: det i = (alpha rank i / maxrank_dn, beta rank i % maxrank_dn).
    void add_all_dets(long nthread) {
        if (nthread == -1)
            nthread = g_threads;
        nthread = std::max(1L, nthread);
        if (maxrank_dn && maxrank_up > INT64_MAX / maxrank_dn)
            throw std::domain_error("cannot generate > 2 ** 63 determinants");
        const long nd = maxrank_up * maxrank_dn;
        while (nthread > 1 && (nd + nthread - 1) / nthread < 1024)
            nthread /= 2;
        dets.assign(static_cast<size_t>(nd * nword2), 0ULL);
        std::vector<ulong_t> beta(static_cast<size_t>(maxrank_dn * nword), 0ULL);
        {
            std::vector<long> occs(nocc_dn + 1);
            unrank_colex(nbasis, nocc_dn, 0, occs.data());
            occs[nocc_dn] = nbasis + 1;
            for (long i = 0; i < maxrank_dn; ++i) {
                fill_det(nocc_dn, occs.data(), &beta[i * nword]);
                next_colex(occs.data());
            }
        }
        auto work = [&](long start, long end) {
            std::vector<long> occs(nocc_up + 1);
            std::vector<ulong_t> a(nword);
            unrank_colex(nbasis, nocc_up, start, occs.data());
            occs[nocc_up] = nbasis + 1;
            for (long i = start; i < end; ++i) {
                std::fill(a.begin(), a.end(), 0ULL);
                fill_det(nocc_up, occs.data(), a.data());
                for (long j = 0; j < maxrank_dn; ++j) {
                    ulong_t *d = &dets[(i * maxrank_dn + j) * nword2];
                    std::memcpy(d, a.data(), sizeof(ulong_t) * nword);
                    std::memcpy(d + nword, &beta[j * nword], sizeof(ulong_t) * nword);
                }
                next_colex(occs.data());
            }
        };
        std::vector<std::thread> th;
        for (long t = 0; t < nthread; ++t)
            th.emplace_back(work, maxrank_up * t / nthread, maxrank_up * (t + 1) / nthread);
        for (auto &x : th)
            x.join();
        ndet = nd;
        index_valid = false;
        full_colex = true;
    }
};

struct DOCIWfn final : OneSpinWfn {
    int kind() const override { return PYCI_WFN_DOCI; }
    void check() const {
        if (nocc_up != nocc_dn)
            throw std::invalid_argument("nocc_up != nocc_dn");
    }
};

struct FullCIWfn final : TwoSpinWfn {
    int kind() const override { return PYCI_WFN_FULLCI; }
};

struct GenCIWfn final : OneSpinWfn {
    int kind() const override { return PYCI_WFN_GENCI; }
    void check() const {
        if (nocc_dn)
            throw std::invalid_argument("nocc_dn != 0");
    }
};

// ---------------------------------------------------------------- heat-bath CI

// add_hci (pyci/src/hci.cpp:240-262, binding pyci/src/binding.cpp:1147-1181):
// one selection step on the device, then the new determinants are appended
// to the wave function in first-occurrence order.  Returns how many were
// added.  nthread is accepted for the reference's signature (the device
// needs no host threads).
long add_hci(const SQuantOp &ham, Wfn &wfn, Array<double> coeffs, double eps, int flags) {
    if (ham.nbasis != wfn.nbasis)
        throw std::invalid_argument("Hamiltonian and wave function have different nbasis");
    if (coeffs.size() < wfn.ndet)
        throw std::invalid_argument("coeffs has fewer entries than the wave function has determinants");
    const long nw = wfn.words();
    auto ctx = default_ctx();
    // A step adds at most ~(connections per determinant) x ndet; a buffer of
    // 16 ndet avoids the second call (a full recount) in practice.
    int64_t cap = std::max<int64_t>(1 << 16, 16 * wfn.ndet), n_new = 0;
    std::vector<ulong_t> out;
    for (;;) {
        out.assign(static_cast<size_t>(cap * nw), 0);
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_add_hci(ctx.get(), wfn.kind(), wfn.nbasis, wfn.nocc_up, wfn.nocc_dn, wfn.ndet,
                                   wfn.ndet ? wfn.dets.data() : nullptr, coeffs.data(), ham.one_mo.data(),
                                   ham.two_mo.data(), eps, flags, cap, out.data(), &n_new));
        }
        if (n_new <= cap)
            break;
        cap = n_new;
    }
    const long before = wfn.ndet;
    for (int64_t i = 0; i < n_new; ++i)
        wfn.add_det(&out[static_cast<size_t>(i * nw)]);
    return wfn.ndet - before;
}

// compute_rdms (pyci/src/rdm.cpp:1011-1055): DOCI (d0, d2), FullCI
// (rdm1 [2, n, n], rdm2 [3, n, n, n, n]) on the device.
// GenCI (genci_exact=True only): the spin-orbital RDMs from their
// definition, rdm1 [n, n] = <a+_p a_q>, rdm2 [n, n, n, n] = <a+_p a+_q a_s a_r>
// (the reference's GenCI compute_rdms writes past its output arrays, so its
// result is undefined and is not reproduced).
static void require_genci_exact(const Wfn &wfn, bool exact) {
    if (wfn.kind() == PYCI_WFN_GENCI && !exact)
        throw std::invalid_argument("RDMs of a GenCI wave function: the reference's result is undefined (it writes "
                                    "past its output arrays); pass genci_exact=True for the RDMs from their "
                                    "definition");
}

py::tuple compute_rdms(const Wfn &wfn, Array<double> coeffs, bool genci_exact = false) {
    require_genci_exact(wfn, genci_exact);
    if (coeffs.size() < wfn.ndet)
        throw std::invalid_argument("coeffs has fewer entries than the wave function has determinants");
    const long n = wfn.nbasis;
    const bool fci = wfn.kind() == PYCI_WFN_FULLCI, gen = wfn.kind() == PYCI_WFN_GENCI;
    Array<double> r1 = fci ? Array<double>({2L, n, n}) : Array<double>({n, n});
    Array<double> r2 = fci ? Array<double>(std::vector<long>{3L, n, n, n, n})
                           : (gen ? Array<double>(std::vector<long>{n, n, n, n}) : Array<double>({n, n}));
    auto ctx = default_ctx();
    const double *c = coeffs.data();
    double *p1 = r1.mutable_data(), *p2 = r2.mutable_data();
    {
        py::gil_scoped_release nogil;
        check(pyci_gpu_compute_rdms(ctx.get(), wfn.kind(), wfn.nbasis, wfn.nocc_up, wfn.nocc_dn, wfn.ndet,
                                    wfn.ndet ? wfn.dets.data() : nullptr, c, p1, p2));
    }
    return py::make_tuple(r1, r2);
}

// compute_enpt2 (pyci/src/enpt2.cpp:332-375, binding pyci/src/binding.cpp:1344-1375):
// Epstein-Nesbet second-order energy on the device.  nthread is accepted for
// the reference's signature.
double compute_enpt2(const SQuantOp &ham, const Wfn &wfn, Array<double> coeffs, double energy, double eps) {
    if (ham.nbasis != wfn.nbasis)
        throw std::invalid_argument("Hamiltonian and wave function have different nbasis");
    if (coeffs.size() < wfn.ndet)
        throw std::invalid_argument("coeffs has fewer entries than the wave function has determinants");
    auto ctx = default_ctx();
    double out = 0.0;
    const double *c = coeffs.data();
    {
        py::gil_scoped_release nogil;
        check(pyci_gpu_compute_enpt2(ctx.get(), wfn.kind(), wfn.nbasis, wfn.nocc_up, wfn.nocc_dn, wfn.ndet,
                                     wfn.ndet ? wfn.dets.data() : nullptr, c, ham.one_mo.data(), ham.two_mo.data(),
                                     energy, ham.ecore, eps, &out));
    }
    return out;
}

// compute_transition_rdms (pyci/src/rdm.cpp:634-902, 1057-1080): same
// layouts as compute_rdms, between two wave functions of the same space.
py::tuple compute_transition_rdms(const Wfn &w1, const Wfn &w2, Array<double> c1, Array<double> c2,
                                  bool genci_exact = false) {
    if (w1.kind() != w2.kind() || w1.nbasis != w2.nbasis || w1.nocc_up != w2.nocc_up || w1.nocc_dn != w2.nocc_dn)
        throw std::invalid_argument("the two wave functions describe different spaces");
    require_genci_exact(w1, genci_exact);
    if (c1.size() < w1.ndet || c2.size() < w2.ndet)
        throw std::invalid_argument("a coefficient vector has fewer entries than its wave function has determinants");
    const long n = w1.nbasis;
    const bool fci = w1.kind() == PYCI_WFN_FULLCI, gen = w1.kind() == PYCI_WFN_GENCI;
    Array<double> r1 = fci ? Array<double>({2L, n, n}) : Array<double>({n, n});
    Array<double> r2 = fci ? Array<double>(std::vector<long>{3L, n, n, n, n})
                           : (gen ? Array<double>(std::vector<long>{n, n, n, n}) : Array<double>({n, n}));
    auto ctx = default_ctx();
    const double *p1c = c1.data(), *p2c = c2.data();
    double *p1 = r1.mutable_data(), *p2 = r2.mutable_data();
    {
        py::gil_scoped_release nogil;
        check(pyci_gpu_compute_transition_rdms(ctx.get(), w1.kind(), n, w1.nocc_up, w1.nocc_dn, w1.ndet,
                                               w1.ndet ? w1.dets.data() : nullptr, p1c, w2.ndet,
                                               w2.ndet ? w2.dets.data() : nullptr, p2c, p1, p2));
    }
    return py::make_tuple(r1, r2);
}

// ---------------------------------------------------------------- numpy views

Array<ulong_t> one_det(const Wfn &w, long i, bool two) {
    if (i < 0 || i >= w.ndet)
        throw py::index_error("determinant index out of range");
    if (!two) {
        Array<ulong_t> a(w.nword);
        std::memcpy(a.mutable_data(), &w.dets[i * w.nword], sizeof(ulong_t) * w.nword);
        return a;
    }
    Array<ulong_t> a({2L, w.nword});
    std::memcpy(a.mutable_data(), &w.dets[i * w.nword2], sizeof(ulong_t) * w.nword2);
    return a;
}

void fix_range(const Wfn &w, long &start, long &end) {
    // pyci/src/onespinwfn.cpp:267-276
    if (start == -1) {
        start = 0;
        if (end == -1)
            end = w.ndet;
    } else if (end == -1) {
        end = start;
        start = 0;
    }
}

Array<ulong_t> to_det_array_one(const Wfn &w, long start, long end) {
    fix_range(w, start, end);
    Array<ulong_t> a({end - start, w.nword});
    if (end > start)
        std::memcpy(a.mutable_data(), &w.dets[start * w.nword], sizeof(ulong_t) * (end - start) * w.nword);
    return a;
}

Array<ulong_t> to_det_array_two(const Wfn &w, long start, long end) {
    fix_range(w, start, end);
    Array<ulong_t> a({end - start, 2L, w.nword});
    // The reference offsets the copy by start * nword (pyci/src/twospinwfn.cpp:112).
    if (end > start)
        std::memcpy(a.mutable_data(), &w.dets[start * w.nword], sizeof(ulong_t) * (end - start) * w.nword2);
    return a;
}

Array<long> to_occ_array_one(const Wfn &w, long start, long end) {
    fix_range(w, start, end);
    Array<long> a({end - start, w.nocc_up});
    long *p = a.mutable_data();
    for (long i = start; i < end; ++i)
        fill_occs(w.nword, &w.dets[i * w.nword], p + (i - start) * w.nocc_up);
    return a;
}

Array<long> to_occ_array_two(const Wfn &w, long start, long end) {
    fix_range(w, start, end);
    Array<long> a({end - start, 2L, w.nocc_up});
    long *p = a.mutable_data();
    std::fill(p, p + (end - start) * 2 * w.nocc_up, 0L);
    for (long i = start; i < end; ++i) {
        fill_occs(w.nword, &w.dets[i * w.nword2], p + (i - start) * 2 * w.nocc_up);
        fill_occs(w.nword, &w.dets[i * w.nword2 + w.nword], p + (i - start) * 2 * w.nocc_up + w.nocc_up);
    }
    return a;
}

void from_det_array(Wfn &w, Array<ulong_t> arr) {
    const long n = arr.ndim() ? arr.shape(0) : 0;
    if (arr.size() != n * w.words())
        throw std::invalid_argument("determinant array has the wrong shape");
    w.assign_dets(arr.data(), n);
}

void from_occ_array_one(Wfn &w, Array<long> arr) {
    const long n = arr.ndim() ? arr.shape(0) : 0;
    std::vector<ulong_t> buf(static_cast<size_t>(n * w.nword), 0ULL);
    const long *p = arr.data();
    for (long i = 0; i < n; ++i)
        fill_det(w.nocc_up, p + i * w.nocc_up, &buf[i * w.nword]);
    w.assign_dets(buf.data(), n);
}

void from_occ_array_two(Wfn &w, Array<long> arr) {
    // pyci/src/twospinwfn.cpp:61-77 (rows of [2][nocc_up]).
    const long n = arr.ndim() ? arr.shape(0) : 0;
    std::vector<ulong_t> buf(static_cast<size_t>(n * w.nword2), 0ULL);
    const long *p = arr.data();
    long j = 0;
    for (long i = 0; i < n; ++i) {
        fill_det(w.nocc_up, p + j, &buf[i * w.nword2]);
        j += w.nocc_up;
        fill_det(w.nocc_dn, p + j, &buf[i * w.nword2 + w.nword]);
        j += w.nocc_up;
    }
    w.assign_dets(buf.data(), n);
}

// ---------------------------------------------------------------- sparse_op

struct CsrDeleter {
    void operator()(pyci_gpu_csr *c) const { pyci_gpu_csr_free(c); }
};

struct SparseOp {
    long nrow = 0, ncol = 0, size = 0;
    double ecore = 0.0;
    bool symmetric = true;
    py::tuple shape;
    std::shared_ptr<pyci_gpu_ctx> ctx;
    std::shared_ptr<pyci_gpu_csr> csr;
    py::dict last_stats;
    int genci_flags = 0;

    SparseOp(const SQuantOp &ham, const Wfn &wfn, long rows, long cols, bool symm, int extra_flags)
        : ecore(ham.ecore), symmetric(symm) {
        if (ham.nbasis != wfn.nbasis)
            throw std::invalid_argument("Hamiltonian and wave function have different nbasis");
        ctx = default_ctx();
        genci_flags = extra_flags;
        int flags = extra_flags;
        if (wfn.full_colex)
            flags |= PYCI_BUILD_FULL_COLEX;
        pyci_gpu_csr *raw = nullptr;
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_csr_build(ctx.get(), wfn.kind(), wfn.nbasis, wfn.nocc_up, wfn.nocc_dn, wfn.ndet,
                                     wfn.ndet ? wfn.dets.data() : nullptr, rows, cols, symm ? 1 : 0,
                                     ham.one_mo.data(), ham.two_mo.data(), flags, &raw));
        }
        csr.reset(raw, CsrDeleter());
        refresh();
    }

    void refresh() {
        int64_t r, c, s, stored;
        check(pyci_gpu_csr_shape(csr.get(), &r, &c, &s, &stored));
        nrow = r;
        ncol = c;
        size = s;
        shape = py::make_tuple(nrow, ncol);
    }

    void update(const SQuantOp &ham, const Wfn &wfn) {
        int flags = genci_flags;
        if (wfn.full_colex)
            flags |= PYCI_BUILD_FULL_COLEX;
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_csr_update(csr.get(), wfn.ndet, wfn.ndet ? wfn.dets.data() : nullptr,
                                      ham.one_mo.data(), ham.two_mo.data(), flags));
        }
        refresh();
    }

    Array<double> matvec(Array<double> x) const {
        if (x.size() != ncol)
            throw std::invalid_argument("x has the wrong length");
        Array<double> y(nrow);
        const double *px = x.data();
        double *py_ = y.mutable_data();
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_csr_matvec(csr.get(), px, py_));
        }
        return y;
    }

    Array<double> matvec_out(Array<double> x, Array<double> out) const {
        if (x.size() != ncol || out.size() != nrow)
            throw std::invalid_argument("x or out has the wrong length");
        const double *px = x.data();
        double *py_ = out.mutable_data();
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_csr_matvec(csr.get(), px, py_));
        }
        return out;
    }

    double get_element(long i, long j) const {
        double v = 0.0;
        check(pyci_gpu_csr_get_element(csr.get(), i, j, &v));
        return v;
    }

    py::tuple solve(long n, py::object c0, long ncv, long maxiter, double tol, const std::string &mode) {
        int m;
        if (mode == "fp64")
            m = PYCI_SOLVE_FP64;
        else if (mode == "mixed")
            m = PYCI_SOLVE_MIXED;
        else
            throw std::invalid_argument("mode must be 'fp64' or 'mixed'");
        Array<double> evals(n);
        Array<double> evecs({n, nrow});
        Array<double> c0a;
        const double *pc0 = nullptr;
        if (!c0.is_none()) {
            c0a = c0.cast<Array<double>>();
            if (c0a.size() != nrow)
                throw std::invalid_argument("c0 has the wrong length");
            pc0 = c0a.data();
        }
        pyci_gpu_solve_stats st{};
        double *pe = evals.mutable_data(), *pv = evecs.mutable_data();
        {
            py::gil_scoped_release nogil;
            check(pyci_gpu_csr_solve(csr.get(), n, pc0, ncv, maxiter, tol, ecore, m, pe, pv, &st));
        }
        py::dict d;
        d["iterations"] = st.iterations;
        d["matvecs"] = st.matvecs;
        d["matvecs_fp64"] = st.matvecs_fp64;
        d["restarts"] = st.restarts;
        d["refinements"] = st.refinements;
        d["seconds"] = st.seconds;
        d["seconds_spmm"] = st.seconds_spmm;
        d["host_syncs"] = st.host_syncs;
        d["seconds_wait"] = st.seconds_wait;
        d["max_residual"] = st.max_residual;
        d["mode"] = mode;
        last_stats = d;
        return py::make_tuple(evals, evecs);
    }

    Array<double> data() const {
        Array<double> a(size);
        check(pyci_gpu_csr_export(csr.get(), a.mutable_data(), nullptr, nullptr));
        return a;
    }
    Array<long> indices() const {
        Array<long> a(size);
        check(pyci_gpu_csr_export(csr.get(), nullptr, reinterpret_cast<int64_t *>(a.mutable_data()), nullptr));
        return a;
    }
    Array<long> indptr() const {
        Array<long> a(nrow + 1);
        check(pyci_gpu_csr_export(csr.get(), nullptr, nullptr, reinterpret_cast<int64_t *>(a.mutable_data())));
        return a;
    }
};

} // namespace

PYBIND11_MODULE(_pyci, m) {
    m.doc() = "pyci_gb300 host module: PyCI's sparse_op on GB300 (sm_103a)";
    m.attr("__version__") = "0.6.1+gb300";
    m.attr("c_long") = py::dtype::of<long>();
    m.attr("c_ulong") = py::dtype::of<unsigned long>();
    m.attr("c_double") = py::dtype::of<double>();
    if (const char *env = std::getenv("PYCI_NUM_THREADS"))
        g_threads = std::max(1L, std::atol(env));

    py::register_exception_translator([](std::exception_ptr p) {
        try {
            if (p)
                std::rethrow_exception(p);
        } catch (const std::domain_error &e) {
            PyErr_SetString(PyExc_ValueError, e.what());
        } catch (const std::ios_base::failure &e) {
            PyErr_SetString(PyExc_RuntimeError, e.what());
        }
    });

    py::class_<SQuantOp> sq(m, "secondquant_op");
    sq.def_readonly("nbasis", &SQuantOp::nbasis);
    sq.def_readonly("ecore", &SQuantOp::ecore);
    sq.def_readonly("one_mo", &SQuantOp::one_mo);
    sq.def_readonly("two_mo", &SQuantOp::two_mo);
    sq.def_readonly("h", &SQuantOp::h);
    sq.def_readonly("v", &SQuantOp::v);
    sq.def_readonly("w", &SQuantOp::w);
    sq.def(py::init<const std::string &>(), py::arg("filename"));
    sq.def(py::init<double, Array<double>, Array<double>>(), py::arg("ecore"), py::arg("one_mo"), py::arg("two_mo"));
    sq.def("to_file", &SQuantOp::to_file, py::arg("filename"), py::arg("nelec") = 0, py::arg("ms2") = 0,
           py::arg("tol") = 0.0);

    py::class_<Wfn> wf(m, "wavefunction");
    wf.def_readonly("nbasis", &Wfn::nbasis);
    wf.def_readonly("nocc", &Wfn::nocc);
    wf.def_readonly("nocc_up", &Wfn::nocc_up);
    wf.def_readonly("nocc_dn", &Wfn::nocc_dn);
    wf.def_readonly("nvir", &Wfn::nvir);
    wf.def_readonly("nvir_up", &Wfn::nvir_up);
    wf.def_readonly("nvir_dn", &Wfn::nvir_dn);
    wf.def("__len__", &Wfn::length);
    wf.def("squeeze", &Wfn::squeeze);
    wf.def("reserve", &Wfn::reserve, py::arg("n"));
    wf.def("to_file", &Wfn::to_file, py::arg("filename"));

    py::class_<OneSpinWfn, Wfn> one(m, "one_spin_wfn");
    one.def("__getitem__", [](const OneSpinWfn &w, long i) { return one_det(w, i, false); }, py::arg("index"));
    one.def("to_det_array", [](const OneSpinWfn &w, long lo, long hi) { return to_det_array_one(w, lo, hi); },
            py::arg("low") = -1, py::arg("high") = -1);
    one.def("to_occ_array", [](const OneSpinWfn &w, long lo, long hi) { return to_occ_array_one(w, lo, hi); },
            py::arg("low") = -1, py::arg("high") = -1);
    one.def("index_det", [](const OneSpinWfn &w, Array<ulong_t> d) {
        if (d.size() != w.nword)
            throw std::invalid_argument("determinant has the wrong length");
        return w.index_det(d.data());
    }, py::arg("det"));
    one.def("add_det", [](OneSpinWfn &w, Array<ulong_t> d) {
        if (d.size() != w.nword)
            throw std::invalid_argument("determinant has the wrong length");
        return w.add_det(d.data());
    }, py::arg("det"));
    one.def("add_occs", [](OneSpinWfn &w, Array<long> o) {
        std::vector<ulong_t> d(w.nword, 0ULL);
        fill_det(w.nocc_up, o.data(), d.data());
        return w.add_det(d.data());
    }, py::arg("occs"));
    one.def("add_hartreefock_det", [](OneSpinWfn &w) {
        std::vector<ulong_t> d(w.nword, 0ULL);
        fill_hartreefock_det(w.nocc_up, d.data());
        w.add_det(d.data());
    });
    one.def("add_all_dets", &OneSpinWfn::add_all_dets, py::arg("nthread") = -1);
    one.def("add_excited_dets", [](OneSpinWfn &w, long exc, py::object ref) {
        std::vector<ulong_t> r(w.nword, 0ULL);
        if (ref.is_none()) {
            fill_hartreefock_det(w.nocc_up, r.data());
        } else {
            Array<ulong_t> a = ref.cast<Array<ulong_t>>();
            std::memcpy(r.data(), a.data(), sizeof(ulong_t) * w.nword);
        }
        const long before = w.ndet;
        w.add_excited_dets(r.data(), exc);
        return w.ndet - before;
    }, py::arg("exc"), py::arg("ref") = py::none());
    one.def("add_dets_from_wfn", [](OneSpinWfn &w, const OneSpinWfn &o) {
        for (long i = 0; i < o.ndet; ++i)
            w.add_det(&o.dets[i * o.nword]);
    }, py::arg("wfn"));

    py::class_<TwoSpinWfn, Wfn> two(m, "two_spin_wfn");
    two.def("__getitem__", [](const TwoSpinWfn &w, long i) { return one_det(w, i, true); }, py::arg("index"));
    two.def("to_det_array", [](const TwoSpinWfn &w, long lo, long hi) { return to_det_array_two(w, lo, hi); },
            py::arg("low") = -1, py::arg("high") = -1);
    two.def("to_occ_array", [](const TwoSpinWfn &w, long lo, long hi) { return to_occ_array_two(w, lo, hi); },
            py::arg("low") = -1, py::arg("high") = -1);
    two.def("index_det", [](const TwoSpinWfn &w, Array<ulong_t> d) {
        if (d.size() != w.nword2)
            throw std::invalid_argument("determinant has the wrong length");
        return w.index_det(d.data());
    }, py::arg("det"));
    two.def("add_det", [](TwoSpinWfn &w, Array<ulong_t> d) {
        if (d.size() != w.nword2)
            throw std::invalid_argument("determinant has the wrong length");
        return w.add_det(d.data());
    }, py::arg("det"));
    two.def("add_occs", [](TwoSpinWfn &w, Array<long> o) {
        std::vector<ulong_t> d(w.nword2, 0ULL);
        fill_det(w.nocc_up, o.data(), d.data());
        fill_det(w.nocc_dn, o.data() + w.nocc_up, d.data() + w.nword);
        return w.add_det(d.data());
    }, py::arg("occs"));
    two.def("add_hartreefock_det", [](TwoSpinWfn &w) {
        std::vector<ulong_t> d(w.nword2, 0ULL);
        fill_hartreefock_det(w.nocc_up, d.data());
        fill_hartreefock_det(w.nocc_dn, d.data() + w.nword);
        w.add_det(d.data());
    });
    two.def("add_all_dets", &TwoSpinWfn::add_all_dets, py::arg("nthread") = -1);
    two.def("add_excited_dets", [](TwoSpinWfn &w, long exc, py::object ref) {
        // pyci/src/twospinwfn.cpp:247-265 and 320-341
        std::vector<ulong_t> r(w.nword2, 0ULL);
        if (ref.is_none()) {
            fill_hartreefock_det(w.nocc_up, r.data());
            fill_hartreefock_det(w.nocc_dn, r.data() + w.nword);
        } else {
            Array<ulong_t> a = ref.cast<Array<ulong_t>>();
            std::memcpy(r.data(), a.data(), sizeof(ulong_t) * w.nword2);
        }
        const long before = w.ndet;
        const long maxup = std::min(w.nocc_up, w.nvir_up), maxdn = std::min(w.nocc_dn, w.nvir_dn);
        long a = std::min(exc, maxup), b = exc - a;
        while (a >= 0 && b <= maxdn) {
            if (a == 0 && b == 0) {
                w.add_det(r.data());
            } else {
                DOCIWfn up, dn; // plain one-spin strings
                up.init(w.nbasis, w.nocc_up, w.nocc_up);
                dn.init(w.nbasis, w.nocc_dn, w.nocc_dn);
                up.add_excited_dets(r.data(), a);
                dn.add_excited_dets(r.data() + w.nword, b);
                std::vector<ulong_t> d(w.nword2);
                for (long i = 0; i < up.ndet; ++i) {
                    std::memcpy(d.data(), &up.dets[i * w.nword], sizeof(ulong_t) * w.nword);
                    for (long j = 0; j < dn.ndet; ++j) {
                        std::memcpy(d.data() + w.nword, &dn.dets[j * w.nword], sizeof(ulong_t) * w.nword);
                        w.add_det(d.data());
                    }
                }
            }
            --a;
            ++b;
        }
        return w.ndet - before;
    }, py::arg("exc"), py::arg("ref") = py::none());
    two.def("add_dets_from_wfn", [](TwoSpinWfn &w, const TwoSpinWfn &o) {
        for (long i = 0; i < o.ndet; ++i)
            w.add_det(&o.dets[i * o.nword2]);
    }, py::arg("wfn"));

    py::class_<DOCIWfn, OneSpinWfn> doci(m, "doci_wfn");
    doci.def(py::init([](const DOCIWfn &o) { return DOCIWfn(o); }), py::arg("wfn"));
    doci.def(py::init([](const std::string &f) {
        DOCIWfn w;
        w.read_file(f, false);
        w.check();
        return w;
    }), py::arg("filename"));
    doci.def(py::init([](long nb, long nu, long nd) {
        DOCIWfn w;
        w.init(nb, nu, nd);
        w.check();
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"));
    doci.def(py::init([](long nb, long nu, long nd, py::array arr) {
        DOCIWfn w;
        w.init(nb, nu, nd);
        w.check();
        if (py::isinstance<py::array_t<ulong_t>>(arr) || arr.dtype().kind() == 'u')
            from_det_array(w, arr.cast<Array<ulong_t>>());
        else
            from_occ_array_one(w, arr.cast<Array<long>>());
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"), py::arg("array"));

    py::class_<FullCIWfn, TwoSpinWfn> fci(m, "fullci_wfn");
    fci.def(py::init([](const DOCIWfn &o) {
        // pyci/src/fullciwfn.cpp:26-35
        FullCIWfn w;
        w.init(o.nbasis, o.nocc_up, o.nocc_dn);
        std::vector<ulong_t> buf(static_cast<size_t>(o.ndet * w.nword2));
        for (long i = 0; i < o.ndet; ++i) {
            std::memcpy(&buf[i * w.nword2], &o.dets[i * o.nword], sizeof(ulong_t) * o.nword);
            std::memcpy(&buf[i * w.nword2 + w.nword], &o.dets[i * o.nword], sizeof(ulong_t) * o.nword);
        }
        w.assign_dets(buf.data(), o.ndet);
        return w;
    }), py::arg("wfn"));
    fci.def(py::init([](const FullCIWfn &o) { return FullCIWfn(o); }), py::arg("wfn"));
    fci.def(py::init([](const std::string &f) {
        FullCIWfn w;
        w.read_file(f, true);
        return w;
    }), py::arg("filename"));
    fci.def(py::init([](long nb, long nu, long nd) {
        FullCIWfn w;
        w.init(nb, nu, nd);
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"));
    fci.def(py::init([](long nb, long nu, long nd, py::array arr) {
        FullCIWfn w;
        w.init(nb, nu, nd);
        if (arr.dtype().kind() == 'u')
            from_det_array(w, arr.cast<Array<ulong_t>>());
        else
            from_occ_array_two(w, arr.cast<Array<long>>());
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"), py::arg("array"));

    py::class_<GenCIWfn, OneSpinWfn> gen(m, "genci_wfn");
    auto genci_from_fullci = [](const FullCIWfn &o) {
        // pyci/src/genciwfn.cpp:31-44, including its filling of the beta
        // occupations from the alpha word (genciwfn.cpp:37).
        GenCIWfn w;
        w.init(o.nbasis * 2, o.nocc, 0);
        std::vector<ulong_t> buf(static_cast<size_t>(o.ndet * o.nword2), 0ULL);
        std::vector<long> occs(o.nocc);
        for (long i = 0; i < o.ndet; ++i) {
            fill_occs(o.nword, &o.dets[i * o.nword2], occs.data());
            fill_occs(o.nword, &o.dets[i * o.nword2], occs.data() + o.nocc_up);
            for (long j = 0; j < o.nocc_dn; ++j)
                occs[o.nocc_up + j] += o.nbasis;
            fill_det(o.nocc, occs.data(), &buf[i * o.nword2]);
        }
        // GenCIWfn's nword (for 2 * nbasis spin-orbitals) may differ from
        // FullCIWfn's nword2; repack.
        std::vector<ulong_t> packed(static_cast<size_t>(o.ndet * w.nword), 0ULL);
        for (long i = 0; i < o.ndet; ++i)
            for (long k = 0; k < std::min(w.nword, o.nword2); ++k)
                packed[i * w.nword + k] = buf[i * o.nword2 + k];
        w.assign_dets(packed.data(), o.ndet);
        return w;
    };
    gen.def(py::init([genci_from_fullci](const DOCIWfn &d) {
        FullCIWfn f;
        f.init(d.nbasis, d.nocc_up, d.nocc_dn);
        std::vector<ulong_t> buf(static_cast<size_t>(d.ndet * f.nword2));
        for (long i = 0; i < d.ndet; ++i) {
            std::memcpy(&buf[i * f.nword2], &d.dets[i * d.nword], sizeof(ulong_t) * d.nword);
            std::memcpy(&buf[i * f.nword2 + f.nword], &d.dets[i * d.nword], sizeof(ulong_t) * d.nword);
        }
        f.assign_dets(buf.data(), d.ndet);
        return genci_from_fullci(f);
    }), py::arg("wfn"));
    gen.def(py::init(genci_from_fullci), py::arg("wfn"));
    gen.def(py::init([](const GenCIWfn &o) { return GenCIWfn(o); }), py::arg("wfn"));
    gen.def(py::init([](const std::string &f) {
        GenCIWfn w;
        w.read_file(f, false);
        w.check();
        return w;
    }), py::arg("filename"));
    gen.def(py::init([](long nb, long nu, long nd) {
        GenCIWfn w;
        w.init(nb, nu, nd);
        w.check();
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"));
    gen.def(py::init([](long nb, long nu, long nd, py::array arr) {
        GenCIWfn w;
        w.init(nb, nu, nd);
        w.check();
        if (arr.dtype().kind() == 'u')
            from_det_array(w, arr.cast<Array<ulong_t>>());
        else
            from_occ_array_one(w, arr.cast<Array<long>>());
        return w;
    }), py::arg("nbasis"), py::arg("nocc_up"), py::arg("nocc_dn"), py::arg("array"));

    py::class_<SparseOp> sp(m, "sparse_op");
    sp.def_readonly("ecore", &SparseOp::ecore);
    sp.def_readonly("symmetric", &SparseOp::symmetric);
    sp.def_readonly("size", &SparseOp::size);
    sp.def_readonly("shape", &SparseOp::shape);
    sp.def_property_readonly("dtype", [](const SparseOp &) { return py::dtype::of<double>(); });
    sp.def_readonly("solve_stats", &SparseOp::last_stats);
    sp.def(py::init([](const SQuantOp &h, const DOCIWfn &w, long nr, long nc, bool s) {
        return SparseOp(h, w, nr, nc, s, 0);
    }), py::arg("ham"), py::arg("wfn"), py::arg("nrow") = -1, py::arg("ncol") = -1, py::arg("symmetric") = true);
    sp.def(py::init([](const SQuantOp &h, const FullCIWfn &w, long nr, long nc, bool s) {
        return SparseOp(h, w, nr, nc, s, 0);
    }), py::arg("ham"), py::arg("wfn"), py::arg("nrow") = -1, py::arg("ncol") = -1, py::arg("symmetric") = true);
    sp.def(py::init([](const SQuantOp &h, const GenCIWfn &w, long nr, long nc, bool s, bool exact) {
        return SparseOp(h, w, nr, nc, s, exact ? PYCI_BUILD_GENCI_EXACT : 0);
    }), py::arg("ham"), py::arg("wfn"), py::arg("nrow") = -1, py::arg("ncol") = -1, py::arg("symmetric") = true,
        py::arg("genci_exact") = false);
    sp.def("update", [](SparseOp &o, const SQuantOp &h, const DOCIWfn &w) { o.update(h, w); }, py::arg("ham"), py::arg("wfn"));
    sp.def("update", [](SparseOp &o, const SQuantOp &h, const FullCIWfn &w) { o.update(h, w); }, py::arg("ham"), py::arg("wfn"));
    sp.def("update", [](SparseOp &o, const SQuantOp &h, const GenCIWfn &w) { o.update(h, w); }, py::arg("ham"), py::arg("wfn"));
    sp.def("__call__", &SparseOp::matvec, py::arg("x"));
    sp.def("__call__", &SparseOp::matvec_out, py::arg("x"), py::arg("out"));
    sp.def("matvec", &SparseOp::matvec, py::arg("x"));
    sp.def("matvec", &SparseOp::matvec_out, py::arg("x"), py::arg("out"));
    sp.def("get_element", &SparseOp::get_element, py::arg("i"), py::arg("j"));
    sp.def("solve", &SparseOp::solve, py::arg("n") = 1, py::arg("c0") = py::none(), py::arg("ncv") = -1,
           py::arg("maxiter") = -1, py::arg("tol") = 1.0e-12, py::arg("mode") = "fp64");
    sp.def("reserve", [](SparseOp &, long) {}, py::arg("n"));
    sp.def("squeeze", [](SparseOp &) {});
    sp.def("data", &SparseOp::data);
    sp.def("indices", &SparseOp::indices);
    sp.def("indptr", &SparseOp::indptr);

    m.def("add_hci", [](const SQuantOp &h, DOCIWfn &w, Array<double> c, double eps, long) {
        return add_hci(h, w, c, eps, 0);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("eps") = 1.0e-5, py::arg("nthread") = -1);
    m.def("add_hci", [](const SQuantOp &h, FullCIWfn &w, Array<double> c, double eps, long) {
        return add_hci(h, w, c, eps, 0);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("eps") = 1.0e-5, py::arg("nthread") = -1);
    m.def("add_hci", [](const SQuantOp &h, GenCIWfn &w, Array<double> c, double eps, long, bool exact) {
        return add_hci(h, w, c, eps, exact ? PYCI_BUILD_GENCI_EXACT : 0);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("eps") = 1.0e-5, py::arg("nthread") = -1,
        py::arg("genci_exact") = false);
    m.def("compute_rdms", [](const DOCIWfn &w, Array<double> c) { return compute_rdms(w, c); }, py::arg("wfn"),
          py::arg("coeffs"));
    m.def("compute_rdms", [](const FullCIWfn &w, Array<double> c) { return compute_rdms(w, c); }, py::arg("wfn"),
          py::arg("coeffs"));
    m.def("compute_rdms", [](const GenCIWfn &w, Array<double> c, bool exact) { return compute_rdms(w, c, exact); },
          py::arg("wfn"), py::arg("coeffs"), py::arg("genci_exact") = false);
    m.def("compute_enpt2", [](const SQuantOp &h, const DOCIWfn &w, Array<double> c, double e, double eps, long) {
        return compute_enpt2(h, w, c, e, eps);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("energy"), py::arg("eps") = 1.0e-5,
          py::arg("nthread") = -1);
    m.def("compute_enpt2", [](const SQuantOp &h, const FullCIWfn &w, Array<double> c, double e, double eps, long) {
        return compute_enpt2(h, w, c, e, eps);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("energy"), py::arg("eps") = 1.0e-5,
          py::arg("nthread") = -1);
    m.def("compute_enpt2", [](const SQuantOp &h, const GenCIWfn &w, Array<double> c, double e, double eps, long) {
        return compute_enpt2(h, w, c, e, eps);
    }, py::arg("ham"), py::arg("wfn"), py::arg("coeffs"), py::arg("energy"), py::arg("eps") = 1.0e-5,
          py::arg("nthread") = -1);
    m.def("compute_transition_rdms", [](const DOCIWfn &w1, const DOCIWfn &w2, Array<double> c1, Array<double> c2) {
        return compute_transition_rdms(w1, w2, c1, c2);
    }, py::arg("wfn1"), py::arg("wfn2"), py::arg("coeffs1"), py::arg("coeffs2"));
    m.def("compute_transition_rdms", [](const FullCIWfn &w1, const FullCIWfn &w2, Array<double> c1, Array<double> c2) {
        return compute_transition_rdms(w1, w2, c1, c2);
    }, py::arg("wfn1"), py::arg("wfn2"), py::arg("coeffs1"), py::arg("coeffs2"));
    m.def("compute_transition_rdms", [](const GenCIWfn &w1, const GenCIWfn &w2, Array<double> c1, Array<double> c2,
                                        bool exact) { return compute_transition_rdms(w1, w2, c1, c2, exact); },
          py::arg("wfn1"), py::arg("wfn2"), py::arg("coeffs1"), py::arg("coeffs2"), py::arg("genci_exact") = false);
    m.def("get_num_threads", []() { return g_threads; });
    m.def("set_num_threads", [](long n) { g_threads = std::max(1L, n); }, py::arg("n"));
    m.def("popcnt", [](Array<ulong_t> d) {
        long c = 0;
        for (long i = 0; i < d.size(); ++i)
            c += __builtin_popcountll(d.data()[i]);
        return c;
    }, py::arg("det"));
    m.def("ctz", [](Array<ulong_t> d) {
        for (long i = 0; i < d.size(); ++i)
            if (d.data()[i])
                return static_cast<long>(__builtin_ctzll(d.data()[i]) + i * 64);
        return 0L;
    }, py::arg("det"));
    m.def("gpu_version", []() { return std::string(pyci_gpu_version()); });
}
