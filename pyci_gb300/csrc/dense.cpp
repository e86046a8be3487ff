// Householder tridiagonalisation + implicit QL for small symmetric matrices.
#include "dense.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace pyci_gpu {

namespace {
// sqrt(a^2 + b^2) without intermediate overflow or underflow (scaled by the
// larger magnitude); cheaper than std::hypot's correctly rounded version,
// which dominated the QL sweeps.
inline double pythag(double a, double b) {
    const double x = std::fabs(a), y = std::fabs(b);
    const double hi = x > y ? x : y, lo = x > y ? y : x;
    if (hi == 0.0)
        return 0.0;
    const double t = lo / hi;
    return hi * std::sqrt(1.0 + t * t);
}
} // namespace

bool symmetric_eigen(int m, const std::vector<double> &a_in, std::vector<double> &evals,
                     std::vector<double> &evecs) {
    const int n = m;
    std::vector<double> A(a_in.begin(), a_in.begin() + static_cast<size_t>(n) * n);
    // QT = Q^T: row r of QT is column r of Q, so reflections and rotations
    // update contiguous rows.
    std::vector<double> QT(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i)
        QT[i * n + i] = 1.0;
    // Symmetrise against round-off in the input.
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j)
            A[i * n + j] = A[j * n + i] = 0.5 * (A[i * n + j] + A[j * n + i]);

    // Householder reduction: A <- H A H with H = I - 2 v v^T, v supported on
    // rows k+1..n-1, chosen to zero A[k+2.., k]; only the trailing block
    // A[k+1.., k+1..] and column/row k change.
    std::vector<double> v(n), p(n), w(n);
    for (int k = 0; k + 2 < n; ++k) {
        const int k1 = k + 1;
        double norm = 0.0;
        for (int i = k1; i < n; ++i)
            norm += A[i * n + k] * A[i * n + k];
        norm = std::sqrt(norm);
        if (norm == 0.0)
            continue;
        const double x0 = A[k1 * n + k];
        const double alpha = (x0 > 0.0) ? -norm : norm;
        for (int i = k1; i < n; ++i)
            v[i] = A[i * n + k];
        v[k1] -= alpha;
        double vn = 0.0;
        for (int i = k1; i < n; ++i)
            vn += v[i] * v[i];
        vn = std::sqrt(vn);
        if (vn == 0.0)
            continue;
        for (int i = k1; i < n; ++i)
            v[i] /= vn;
        // Column / row k: H x = alpha e_1.
        A[k1 * n + k] = A[k * n + k1] = alpha;
        for (int i = k1 + 1; i < n; ++i)
            A[i * n + k] = A[k * n + i] = 0.0;
        // Trailing block B: p = B v, K = v^T p, B -= 2 v p^T + 2 p v^T - 4 K v v^T.
        double K = 0.0;
        for (int i = k1; i < n; ++i) {
            const double *row = &A[i * n];
            double sum = 0.0;
            for (int j = k1; j < n; ++j)
                sum += row[j] * v[j];
            p[i] = sum;
            K += v[i] * sum;
        }
        for (int i = k1; i < n; ++i) {
            double *row = &A[i * n];
            const double vi = v[i], pi = p[i], c4 = 4.0 * K * vi;
            for (int j = k1; j < n; ++j)
                row[j] += -2.0 * vi * p[j] - 2.0 * pi * v[j] + c4 * v[j];
        }
        // Q <- Q H, i.e. QT[k1..] -= 2 v (v^T QT[k1..]).
        std::fill(w.begin(), w.end(), 0.0);
        for (int j = k1; j < n; ++j) {
            const double *row = &QT[j * n];
            const double vj = v[j];
            for (int c = 0; c < n; ++c)
                w[c] += vj * row[c];
        }
        for (int j = k1; j < n; ++j) {
            double *row = &QT[j * n];
            const double vj2 = 2.0 * v[j];
            for (int c = 0; c < n; ++c)
                row[c] -= vj2 * w[c];
        }
    }
    std::vector<double> d(n), e(n, 0.0);
    for (int i = 0; i < n; ++i)
        d[i] = A[i * n + i];
    for (int i = 0; i + 1 < n; ++i)
        e[i] = A[(i + 1) * n + i];

    // Implicit QL with shifts on (d, e); e[i] couples d[i] and d[i + 1].
    const double eps = std::numeric_limits<double>::epsilon();
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        for (;;) {
            int mm = l;
            for (; mm + 1 < n; ++mm) {
                const double dd = std::fabs(d[mm]) + std::fabs(d[mm + 1]);
                if (std::fabs(e[mm]) <= eps * dd)
                    break;
            }
            if (mm == l)
                break;
            if (++iter > 200)
                return false;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = pythag(g, 1.0);
            g = d[mm] - d[l] + e[l] / (g + std::copysign(r, g));
            double s = 1.0, c = 1.0, pp = 0.0;
            int i = mm - 1;
            bool underflow = false;
            for (; i >= l; --i) {
                double f = s * e[i];
                const double b = c * e[i];
                r = pythag(f, g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= pp;
                    e[mm] = 0.0;
                    underflow = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - pp;
                r = (d[i] - g) * s + 2.0 * c * b;
                pp = s * r;
                d[i + 1] = g + pp;
                g = c * r - b;
                double *qa = &QT[i * n], *qb = &QT[(i + 1) * n];
                for (int k = 0; k < n; ++k) {
                    const double x = qb[k], y = qa[k];
                    qb[k] = s * y + c * x;
                    qa[k] = c * y - s * x;
                }
            }
            if (underflow)
                continue;
            d[l] -= pp;
            e[l] = g;
            e[mm] = 0.0;
        }
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return d[x] < d[y]; });
    evals.resize(n);
    evecs.assign(static_cast<size_t>(n) * n, 0.0);
    for (int c = 0; c < n; ++c) {
        evals[c] = d[order[c]];
        const double *col = &QT[static_cast<size_t>(order[c]) * n];
        for (int r = 0; r < n; ++r)
            evecs[r * n + c] = col[r];
    }
    return true;
}

} // namespace pyci_gpu
