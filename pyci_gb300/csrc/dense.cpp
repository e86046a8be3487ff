// Householder tridiagonalisation + implicit QL for small symmetric matrices.
#include "dense.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace pyci_gpu {

bool symmetric_eigen(int m, const std::vector<double> &a_in, std::vector<double> &evals,
                     std::vector<double> &evecs) {
    const int n = m;
    std::vector<double> A(a_in.begin(), a_in.begin() + static_cast<size_t>(n) * n);
    std::vector<double> Q(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i)
        Q[i * n + i] = 1.0;
    // Symmetrise against round-off in the input.
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j)
            A[i * n + j] = A[j * n + i] = 0.5 * (A[i * n + j] + A[j * n + i]);

    // Householder reduction: A <- H A H with H = I - 2 v v^T, v supported on
    // rows k+1..n-1, chosen to zero A[k+2.., k].
    std::vector<double> v(n), p(n), qv(n);
    for (int k = 0; k + 2 < n; ++k) {
        double norm = 0.0;
        for (int i = k + 1; i < n; ++i)
            norm += A[i * n + k] * A[i * n + k];
        norm = std::sqrt(norm);
        if (norm == 0.0)
            continue;
        const double x0 = A[(k + 1) * n + k];
        const double alpha = (x0 > 0.0) ? -norm : norm;
        std::fill(v.begin(), v.end(), 0.0);
        for (int i = k + 1; i < n; ++i)
            v[i] = A[i * n + k];
        v[k + 1] -= alpha;
        double vn = 0.0;
        for (int i = k + 1; i < n; ++i)
            vn += v[i] * v[i];
        vn = std::sqrt(vn);
        if (vn == 0.0)
            continue;
        for (int i = k + 1; i < n; ++i)
            v[i] /= vn;
        // p = A v ; K = v^T p ; A -= 2 v p^T + 2 p v^T - 4 K v v^T
        double K = 0.0;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j)
                s += A[i * n + j] * v[j];
            p[i] = s;
        }
        for (int i = k + 1; i < n; ++i)
            K += v[i] * p[i];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                A[i * n + j] += -2.0 * v[i] * p[j] - 2.0 * p[i] * v[j] + 4.0 * K * v[i] * v[j];
        // Q <- Q H
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j)
                s += Q[i * n + j] * v[j];
            qv[i] = s;
        }
        for (int i = 0; i < n; ++i)
            for (int j = k + 1; j < n; ++j)
                Q[i * n + j] -= 2.0 * qv[i] * v[j];
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
            double r = std::hypot(g, 1.0);
            g = d[mm] - d[l] + e[l] / (g + std::copysign(r, g));
            double s = 1.0, c = 1.0, pp = 0.0;
            int i = mm - 1;
            bool underflow = false;
            for (; i >= l; --i) {
                double f = s * e[i];
                const double b = c * e[i];
                r = std::hypot(f, g);
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
                for (int k = 0; k < n; ++k) {
                    f = Q[k * n + i + 1];
                    Q[k * n + i + 1] = s * Q[k * n + i] + c * f;
                    Q[k * n + i] = c * Q[k * n + i] - s * f;
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
        for (int r = 0; r < n; ++r)
            evecs[r * n + c] = Q[r * n + order[c]];
    }
    return true;
}

} // namespace pyci_gpu
