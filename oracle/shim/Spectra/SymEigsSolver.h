// Stand-in for Spectra::SymEigsSolver as used in pyci/src/sparseop.cpp:127-146.
//
// Test infrastructure only.  Spectra (cloned unpinned by the reference
// Makefile) is unavailable offline, so this header implements the same
// contract -- the nev algebraically smallest eigenpairs of a symmetric
// operator from a Krylov space of dimension ncv -- with a thick-restart
// Lanczos iteration (Wu & Simon, SIAM J. Matrix Anal. Appl. 22 (2000) 602),
// which is mathematically equivalent to Spectra's implicitly restarted Lanczos.
// Convergence test as documented by Spectra: residual norm of each wanted Ritz
// pair <= tol * max(eps^(2/3), |theta|).  Results are returned in decreasing
// order, Spectra's default sorting rule for compute().
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <vector>

#include <Eigen/Core>

namespace Spectra {

enum class SortRule { LargestMagn, LargestAlge, SmallestMagn, SmallestAlge };

enum class CompInfo { Successful, NotComputed, NotConverging, NumericalIssue };

// Cyclic Jacobi eigen-decomposition of a dense symmetric n x n matrix `a`
// (row-major, destroyed).  Eigenvalues ascending; eigenvectors column-major.
inline void shim_jacobi_eigh(long n, std::vector<double> &a, std::vector<double> &evals,
                             std::vector<double> &evecs) {
    std::vector<double> v(n * n, 0.0);
    for (long i = 0; i < n; ++i)
        v[i * n + i] = 1.0; // row-major while rotating
    double scale = 0.0;
    for (long i = 0; i < n * n; ++i)
        scale += a[i] * a[i];
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (long p = 0; p < n; ++p)
            for (long q = p + 1; q < n; ++q)
                off += a[p * n + q] * a[p * n + q];
        if (off <= 1e-32 * scale || off == 0.0)
            break;
        for (long p = 0; p < n; ++p) {
            for (long q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0)
                    continue;
                const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double t = ((theta >= 0.0) ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (long k = 0; k < n; ++k) {
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (long k = 0; k < n; ++k) {
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                for (long k = 0; k < n; ++k) {
                    const double vkp = v[k * n + p], vkq = v[k * n + q];
                    v[k * n + p] = c * vkp - s * vkq;
                    v[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    std::vector<long> order(n);
    for (long i = 0; i < n; ++i)
        order[i] = i;
    std::sort(order.begin(), order.end(),
              [&](long x, long y) { return a[x * n + x] < a[y * n + y]; });
    evals.resize(n);
    evecs.resize(n * n);
    for (long c = 0; c < n; ++c) {
        evals[c] = a[order[c] * n + order[c]];
        for (long r = 0; r < n; ++r)
            evecs[c * n + r] = v[r * n + order[c]];
    }
}

template<typename OpType>
class SymEigsSolver {
public:
    SymEigsSolver(OpType &op, long nev, long ncv)
        : op_(op), n_(op.rows()), nev_(nev), ncv_(std::min(ncv, op.rows())),
          info_(CompInfo::NotComputed) {
        if (nev_ < 1 || nev_ > n_ - 1)
            throw std::invalid_argument("nev must satisfy 1 <= nev <= n - 1");
        if (ncv_ <= nev_ && ncv_ < n_)
            throw std::invalid_argument("ncv must satisfy nev < ncv <= n");
    }

    void init(const double *v0) { start_.assign(v0, v0 + n_); }

    void init() {
        start_.resize(n_);
        std::uint64_t s = 0x2545f4914f6cdd1dULL;
        for (long i = 0; i < n_; ++i) {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            start_[i] = static_cast<double>(s >> 11) * (1.0 / 9007199254740992.0) - 0.5;
        }
    }

    long compute(SortRule rule, long maxit, double tol) {
        if (rule != SortRule::SmallestAlge)
            throw std::invalid_argument("only SmallestAlge is supported");
        const long n = n_, m = ncv_;
        const double eps23 = std::pow(std::numeric_limits<double>::epsilon(), 2.0 / 3.0);
        std::vector<double> V(n * m, 0.0), T(m * m, 0.0), w(n), f(n);
        std::vector<double> theta, Y;
        double fnorm = 0.0;
        if (start_.empty())
            init();
        copy_normalized(start_.data(), &V[0]);
        long k = 0;
        info_ = CompInfo::NotConverging;
        for (long iter = 0; iter < maxit; ++iter) {
            for (long j = k; j < m; ++j) {
                op_.perform_op(&V[j * n], w.data());
                for (long i = 0; i < m; ++i)
                    T[i * m + j] = T[j * m + i] = (i < k && j < k) ? T[i * m + j] : 0.0;
                for (int pass = 0; pass < 2; ++pass) {
                    for (long i = 0; i <= j; ++i) {
                        const double c = dot(&V[i * n], w.data());
                        T[i * m + j] += c;
                        axpy(-c, &V[i * n], w.data());
                    }
                }
                for (long i = 0; i < j; ++i)
                    T[j * m + i] = T[i * m + j];
                const double beta = std::sqrt(dot(w.data(), w.data()));
                if (j + 1 < m) {
                    if (beta > 1e-13 * scale_of(T, m, j)) {
                        for (long r = 0; r < n; ++r)
                            V[(j + 1) * n + r] = w[r] / beta;
                    } else {
                        fresh_direction(V, j + 1);
                    }
                } else {
                    f = w;
                    fnorm = beta;
                }
            }
            std::vector<double> Tc(T);
            shim_jacobi_eigh(m, Tc, theta, Y);
            long nconv = 0;
            for (long i = 0; i < nev_; ++i) {
                const double res = fnorm * std::fabs(Y[i * m + (m - 1)]);
                if (res <= tol * std::max(eps23, std::fabs(theta[i])))
                    ++nconv;
            }
            const bool done = (nconv >= nev_) || (m >= n);
            long p = done ? nev_ : std::min(nev_ + std::min(nconv, (m - nev_) / 2), m - 1);
            if (p < 1)
                p = 1;
            std::vector<double> U(n * p, 0.0);
            for (long c = 0; c < p; ++c)
                for (long i = 0; i < m; ++i)
                    axpy(Y[c * m + i], &V[i * n], &U[c * n]);
            if (done) {
                // Selection picks the nev smallest; Spectra's default sorting
                // rule for the result (LargestAlge) then lists them in
                // decreasing order, which pyci's test_odometer relies on.
                evals_.resize(nev_);
                evecs_ = Eigen::MatrixXd(n, nev_);
                for (long c = 0; c < nev_; ++c) {
                    const long src = nev_ - 1 - c;
                    evals_[c] = theta[src];
                    for (long r = 0; r < n; ++r)
                        evecs_(r, c) = U[src * n + r];
                }
                info_ = CompInfo::Successful;
                return nconv;
            }
            std::fill(T.begin(), T.end(), 0.0);
            for (long c = 0; c < p; ++c) {
                std::copy(&U[c * n], &U[c * n] + n, &V[c * n]);
                T[c * m + c] = theta[c];
            }
            if (fnorm > 0.0) {
                for (long r = 0; r < n; ++r)
                    V[p * n + r] = f[r] / fnorm;
            } else {
                fresh_direction(V, p);
            }
            k = p;
        }
        return 0;
    }

    CompInfo info() const { return info_; }

    Eigen::VectorXd eigenvalues() const {
        Eigen::VectorXd out(static_cast<long>(evals_.size()));
        for (long i = 0; i < static_cast<long>(evals_.size()); ++i)
            out[i] = evals_[i];
        return out;
    }

    Eigen::MatrixXd eigenvectors() const { return evecs_; }

private:
    double dot(const double *a, const double *b) const {
        double s = 0.0;
        for (long i = 0; i < n_; ++i)
            s += a[i] * b[i];
        return s;
    }

    void axpy(double a, const double *x, double *y) const {
        for (long i = 0; i < n_; ++i)
            y[i] += a * x[i];
    }

    static double scale_of(const std::vector<double> &T, long m, long j) {
        double s = 0.0;
        for (long i = 0; i <= j; ++i)
            s = std::max(s, std::fabs(T[i * m + i]));
        return std::max(s, 1e-300);
    }

    void copy_normalized(const double *src, double *dst) const {
        const double nrm = std::sqrt(dot(src, src));
        for (long i = 0; i < n_; ++i)
            dst[i] = src[i] / nrm;
    }

    // Fill column j of V with a unit vector orthogonal to columns 0..j-1.
    void fresh_direction(std::vector<double> &V, long j) {
        std::uint64_t s = 0x9e3779b97f4a7c15ULL + static_cast<std::uint64_t>(j) * 7919ULL;
        double *v = &V[j * n_];
        for (int attempt = 0; attempt < 8; ++attempt) {
            for (long i = 0; i < n_; ++i) {
                s ^= s << 13;
                s ^= s >> 7;
                s ^= s << 17;
                v[i] = static_cast<double>(s >> 11) * (1.0 / 9007199254740992.0) - 0.5;
            }
            for (int pass = 0; pass < 2; ++pass)
                for (long i = 0; i < j; ++i)
                    axpy(-dot(&V[i * n_], v), &V[i * n_], v);
            const double nrm = std::sqrt(dot(v, v));
            if (nrm > 1e-8) {
                for (long i = 0; i < n_; ++i)
                    v[i] /= nrm;
                return;
            }
        }
        throw std::runtime_error("could not extend the Krylov basis");
    }

    OpType &op_;
    long n_, nev_, ncv_;
    CompInfo info_;
    std::vector<double> start_, evals_;
    Eigen::MatrixXd evecs_;
};

} // namespace Spectra
