// matrix.h - the few dense-matrix operations the reference's programs perform on spectra read
// from CSV files (cpp_simulations/*: `Eigen::MatrixXd m = SourceHelpers::readCSV(path);
// m.col(0) = m.col(0).array() * 1000; Eigen::VectorXd e = m.col(0);`), so that they build
// without Eigen.  With Eigen present (EIGEN_WORLD_VERSION defined) the aliases are not made.
#pragma once
#include <cstddef>
#include <stdexcept>
#include <vector>

namespace midsx {

class Matrix;

// An element-wise view of a column (Eigen's .array()): scaled by a number, assigned back.
class ColumnArray {
public:
    explicit ColumnArray(std::vector<double> v) : v_(std::move(v)) {}
    ColumnArray operator*(double s) const {
        std::vector<double> r(v_);
        for (double& x : r) x *= s;
        return ColumnArray(std::move(r));
    }
    ColumnArray operator/(double s) const { return *this * (1.0 / s); }
    const std::vector<double>& values() const { return v_; }
    operator std::vector<double>() const { return v_; }

private:
    std::vector<double> v_;
};

inline ColumnArray operator*(double s, const ColumnArray& a) { return a * s; }

// Column c of a Matrix, writable.
class MatrixColumn {
public:
    MatrixColumn(Matrix& m, int c) : m_(m), c_(c) {}
    inline std::vector<double> values() const;
    ColumnArray array() const { return ColumnArray(values()); }
    inline MatrixColumn& operator=(const ColumnArray& a);
    inline MatrixColumn& operator=(const std::vector<double>& v);
    operator std::vector<double>() const { return values(); }
    inline double operator[](std::ptrdiff_t r) const;
    inline std::ptrdiff_t size() const;

private:
    Matrix& m_;
    int c_;
};

// Row-major dense matrix of doubles.
class Matrix {
public:
    Matrix() = default;
    Matrix(std::ptrdiff_t rows, std::ptrdiff_t cols) : rows_(rows), cols_(cols), a_(size_t(rows * cols), 0.0) {}
    // rows of equal length (SourceHelpers::readCSV)
    explicit Matrix(const std::vector<std::vector<double>>& rows) {
        rows_ = std::ptrdiff_t(rows.size());
        cols_ = rows.empty() ? 0 : std::ptrdiff_t(rows[0].size());
        a_.reserve(size_t(rows_ * cols_));
        for (const auto& r : rows) {
            if (std::ptrdiff_t(r.size()) != cols_) throw std::invalid_argument("rows of unequal length");
            a_.insert(a_.end(), r.begin(), r.end());
        }
    }
    std::ptrdiff_t rows() const { return rows_; }
    std::ptrdiff_t cols() const { return cols_; }
    double& operator()(std::ptrdiff_t r, std::ptrdiff_t c) { return a_.at(size_t(r * cols_ + c)); }
    double operator()(std::ptrdiff_t r, std::ptrdiff_t c) const { return a_.at(size_t(r * cols_ + c)); }
    MatrixColumn col(int c) {
        if (c < 0 || c >= cols_) throw std::out_of_range("column index");
        return MatrixColumn(*this, c);
    }
    std::vector<double> col(int c) const {
        if (c < 0 || c >= cols_) throw std::out_of_range("column index");
        std::vector<double> v(static_cast<size_t>(rows_));
        for (std::ptrdiff_t r = 0; r < rows_; ++r) v[size_t(r)] = (*this)(r, c);
        return v;
    }
    operator std::vector<std::vector<double>>() const {
        std::vector<std::vector<double>> out(static_cast<size_t>(rows_));
        for (std::ptrdiff_t r = 0; r < rows_; ++r)
            out[size_t(r)].assign(a_.begin() + r * cols_, a_.begin() + (r + 1) * cols_);
        return out;
    }

private:
    std::ptrdiff_t rows_ = 0, cols_ = 0;
    std::vector<double> a_;
};

inline std::vector<double> MatrixColumn::values() const { return static_cast<const Matrix&>(m_).col(c_); }
inline MatrixColumn& MatrixColumn::operator=(const std::vector<double>& v) {
    if (std::ptrdiff_t(v.size()) != m_.rows()) throw std::invalid_argument("column length");
    for (std::ptrdiff_t r = 0; r < m_.rows(); ++r) m_(r, c_) = v[size_t(r)];
    return *this;
}
inline MatrixColumn& MatrixColumn::operator=(const ColumnArray& a) { return *this = a.values(); }
inline double MatrixColumn::operator[](std::ptrdiff_t r) const { return static_cast<const Matrix&>(m_)(r, c_); }
inline std::ptrdiff_t MatrixColumn::size() const { return m_.rows(); }

}  // namespace midsx

#if !defined(EIGEN_WORLD_VERSION) && !defined(MIDSX_NO_EIGEN_ALIAS)
namespace Eigen {
using MatrixXd = ::midsx::Matrix;
using VectorXd = std::vector<double>;
}  // namespace Eigen
#endif
