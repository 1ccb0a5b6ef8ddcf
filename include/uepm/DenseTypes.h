// DenseTypes.h -- the dense vector / matrix types of the Hamiltonian's eigen results. With Eigen on the
// include path they are Eigen::VectorXd and Eigen::MatrixXcd, exactly the reference's types
// (src/EPP/Hamiltonian.h:18-21); without Eigen, minimal column-major stand-ins with the members the
// reference's callers use (operator(), rows(), cols(), size(), col()).
#pragma once

#include <complex>
#include <cstddef>
#include <vector>

#if defined(UEPM_USE_EIGEN) || __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
namespace uepm::pseudopotential {
using RealVector    = Eigen::VectorXd;
using ComplexMatrix = Eigen::MatrixXcd;
using ComplexVector = Eigen::VectorXcd;
}  // namespace uepm::pseudopotential
#else
namespace uepm::pseudopotential {

class RealVector {
 public:
    RealVector() = default;
    explicit RealVector(std::ptrdiff_t n) : v_((size_t)n) {}
    void           resize(std::ptrdiff_t n) { v_.resize((size_t)n); }
    std::ptrdiff_t size() const { return (std::ptrdiff_t)v_.size(); }
    std::ptrdiff_t rows() const { return size(); }
    double&        operator()(std::ptrdiff_t i) { return v_[(size_t)i]; }
    double         operator()(std::ptrdiff_t i) const { return v_[(size_t)i]; }
    double&        operator[](std::ptrdiff_t i) { return v_[(size_t)i]; }
    double         operator[](std::ptrdiff_t i) const { return v_[(size_t)i]; }
    double*        data() { return v_.data(); }
    const double*  data() const { return v_.data(); }

 private:
    std::vector<double> v_;
};

using ComplexVector = std::vector<std::complex<double>>;

class ComplexMatrix {
 public:
    ComplexMatrix() = default;
    ComplexMatrix(std::ptrdiff_t r, std::ptrdiff_t c) : r_(r), c_(c), v_((size_t)(r * c)) {}
    void resize(std::ptrdiff_t r, std::ptrdiff_t c) {
        r_ = r;
        c_ = c;
        v_.assign((size_t)(r * c), {});
    }
    std::ptrdiff_t              rows() const { return r_; }
    std::ptrdiff_t              cols() const { return c_; }
    std::ptrdiff_t              size() const { return r_ * c_; }
    std::complex<double>&       operator()(std::ptrdiff_t i, std::ptrdiff_t j) { return v_[(size_t)(j * r_ + i)]; }
    const std::complex<double>& operator()(std::ptrdiff_t i, std::ptrdiff_t j) const { return v_[(size_t)(j * r_ + i)]; }
    // copy of column j (band j)
    ComplexVector col(std::ptrdiff_t j) const {
        return ComplexVector(v_.begin() + j * r_, v_.begin() + (j + 1) * r_);
    }
    std::complex<double>*       data() { return v_.data(); }
    const std::complex<double>* data() const { return v_.data(); }

 private:
    std::ptrdiff_t                    r_ = 0, c_ = 0;
    std::vector<std::complex<double>> v_;
};

}  // namespace uepm::pseudopotential
#endif
