// Small dense symmetric eigensolver for the Rayleigh-Ritz step of the
// Davidson iteration (host, FP64).
#pragma once

#include <cstdint>
#include <vector>

namespace pyci_gpu {

// Eigen-decomposition of the symmetric m x m matrix `a` (row-major; only
// read).  Householder reduction to tridiagonal form followed by the implicit
// QL iteration with Wilkinson shifts.  Eigenvalues ascending in `evals`;
// eigenvector c in column c of `evecs` (row-major m x m: evecs[r * m + c]).
// Returns false if the QL iteration fails to converge.
bool symmetric_eigen(int m, const std::vector<double> &a, std::vector<double> &evals,
                     std::vector<double> &evecs);

} // namespace pyci_gpu
