// Stand-in for Spectra::SparseSymMatProd as used in pyci/src/sparseop.cpp:127:
// y = A x for the self-adjoint matrix whose lower triangle is stored in a
// row-major CSR map.  Test infrastructure only.
#pragma once

#include <Eigen/Core>
#include <Eigen/SparseCore>

namespace Spectra {

template<typename T, int UpLo, int Opt, typename Index>
class SparseSymMatProd {
public:
    typedef Eigen::Map<const Eigen::SparseMatrix<T, Opt, Index>> MapType;

    explicit SparseSymMatProd(const MapType &m) : mat(m) {}

    long rows() const { return mat.rows(); }
    long cols() const { return mat.cols(); }

    void perform_op(const T *x, T *y) const {
        Eigen::LowerSelfAdjointTimesVector<T, Index> e{mat.a, x};
        Eigen::csr_apply(e, y);
    }

private:
    MapType mat;
};

} // namespace Spectra
