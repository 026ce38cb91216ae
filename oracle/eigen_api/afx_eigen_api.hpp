// Minimal stand-in for the part of the Eigen 3 API that AeroFLEX's rans
// headers call (test infrastructure only).
//
// It lets the UNMODIFIED reference headers (src/rans/include/rans/{core,mesh,
// physics,solver,multigrid,post}.h) compile where Eigen is not installed, so
// that the reference's own code runs here as the oracle's pin.  It is not
// Eigen: every class is written for this project from the documented
// behaviour of the calls the headers make, and nothing else is provided.
//
// Arithmetic semantics, and where they could differ from a real Eigen build:
// - Dense expressions are evaluated eagerly, one IEEE operation per
//   coefficient in the order the expression is written.  Real Eigen fuses the
//   same expression lazily into one loop; per coefficient the operations and
//   their order are the same, so coefficient-wise results are identical
//   (both builds without FMA contraction: -ffp-contract=off).
// - Reductions (norm(), small dense products) sum in index order.  Real
//   Eigen may sum vectorised partial sums (packets) instead, so norm() and the
//   least-squares products are not pinned to Eigen's own order.
// - Sparse matrix times dense vector accumulates each row in ascending column
//   order, as a compressed-column (or compressed-row) product does.
// - Storage starts zeroed (Eigen leaves it uninitialised; the oracle makes the
//   same choice).
// - GMRES and IncompleteLUT are a right-preconditioned restarted GMRES(30)
//   and an ILU(0) factorisation on the matrix's own pattern (fill factor and
//   drop tolerance are accepted and not used).  Their iterates are not
//   Eigen's; a converged implicit solution is the same fixed point.
// - Only the pieces the rans headers use exist; a header built with
//   RANS_MATRIX_FREE, RANS_SPARSELU or RANS_BICGSTAB does not compile.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;
const int Dynamic = -1;

enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
enum StorageOptions { ColMajor = 0, RowMajor = 1 };

inline int nbThreads() { return 1; }

class DenseView;

// Column-major dense matrix of doubles, sized at run time.  A vector is a
// matrix with one column.
class Dense {
public:
    Dense() {}
    Dense(Index r, Index c) : r_(r), c_(c), v_((size_t)(r * c), 0.0) {}
    Dense(const DenseView& b);

    Index rows() const { return r_; }
    Index cols() const { return c_; }
    Index size() const { return r_ * c_; }
    double* data() { return v_.data(); }
    const double* data() const { return v_.data(); }

    double& operator()(Index i) { return v_[(size_t)i]; }
    double operator()(Index i) const { return v_[(size_t)i]; }
    double& operator()(Index i, Index j) { return v_[(size_t)(i + j * r_)]; }
    double operator()(Index i, Index j) const { return v_[(size_t)(i + j * r_)]; }
    double& operator[](Index i) { return v_[(size_t)i]; }
    double operator[](Index i) const { return v_[(size_t)i]; }
    double& coeffRef(Index i) { return v_[(size_t)i]; }
    double& coeffRef(Index i, Index j) { return (*this)(i, j); }
    double coeff(Index i) const { return v_[(size_t)i]; }
    double coeff(Index i, Index j) const { return (*this)(i, j); }

    void resize(Index n) { resize(n, 1); }
    void resize(Index r, Index c) {
        if (r == r_ && c == c_) return;
        r_ = r;
        c_ = c;
        v_.assign((size_t)(r * c), 0.0);
    }
    void setZero() { std::fill(v_.begin(), v_.end(), 0.0); }

    DenseView segment(Index start, Index n) const;
    DenseView block(Index i, Index j, Index nr, Index nc) const;
    DenseView col(Index j) const;

    Dense transpose() const {
        Dense t(c_, r_);
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) t(j, i) = (*this)(i, j);
        return t;
    }

    // Inverse of a 2x2 matrix by the adjugate over the determinant (the only
    // size the rans headers invert: the least-squares normal matrix).
    Dense inverse() const {
        if (r_ != 2 || c_ != 2) throw std::logic_error("eigen_api: inverse() is provided for 2x2 matrices only");
        const double a = (*this)(0, 0), b = (*this)(0, 1), c = (*this)(1, 0), d = (*this)(1, 1);
        const double det = a * d - b * c;
        const double inv = 1.0 / det;
        Dense r(2, 2);
        r(0, 0) = d * inv;
        r(0, 1) = -b * inv;
        r(1, 0) = -c * inv;
        r(1, 1) = a * inv;
        return r;
    }

    double squaredNorm() const {
        double s = 0.0;
        for (double x : v_) s += x * x;
        return s;
    }
    double norm() const { return std::sqrt(squaredNorm()); }

    Dense cwiseProduct(const Dense& o) const {
        same_shape(o);
        Dense r(r_, c_);
        for (size_t i = 0; i < v_.size(); ++i) r.v_[i] = v_[i] * o.v_[i];
        return r;
    }

    Dense& operator+=(const Dense& o) {
        same_shape(o);
        for (size_t i = 0; i < v_.size(); ++i) v_[i] += o.v_[i];
        return *this;
    }
    Dense& operator-=(const Dense& o) {
        same_shape(o);
        for (size_t i = 0; i < v_.size(); ++i) v_[i] -= o.v_[i];
        return *this;
    }
    Dense& operator*=(double s) {
        for (double& x : v_) x *= s;
        return *this;
    }
    Dense& operator/=(double s) {
        for (double& x : v_) x /= s;
        return *this;
    }

    void same_shape(const Dense& o) const {
        if (o.r_ != r_ || o.c_ != c_) throw std::logic_error("eigen_api: operand sizes differ");
    }

protected:
    Index r_ = 0, c_ = 0;
    std::vector<double> v_;
};

// A rectangular window into a Dense (segment, block, col).  Assigning to it
// writes the coefficients of the underlying matrix.
class DenseView {
public:
    DenseView(double* p, Index r, Index c, Index ld) : p_(p), r_(r), c_(c), ld_(ld) {}
    Index rows() const { return r_; }
    Index cols() const { return c_; }
    Index size() const { return r_ * c_; }
    double& operator()(Index i, Index j) const { return p_[i + j * ld_]; }
    double& operator()(Index i) const { return c_ == 1 ? p_[i] : p_[i * ld_]; }
    double& coeffRef(Index i) const { return (*this)(i); }

    DenseView& operator=(const Dense& d) {
        if (d.rows() != r_ || d.cols() != c_) throw std::logic_error("eigen_api: block assignment sizes differ");
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) (*this)(i, j) = d(i, j);
        return *this;
    }
    DenseView& operator=(const DenseView& b) { return *this = Dense(b); }
    DenseView& operator*=(double s) {
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) (*this)(i, j) *= s;
        return *this;
    }
    DenseView& operator/=(double s) {
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) (*this)(i, j) /= s;
        return *this;
    }
    DenseView& operator+=(const Dense& d) {
        if (d.rows() != r_ || d.cols() != c_) throw std::logic_error("eigen_api: operand sizes differ");
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) (*this)(i, j) += d(i, j);
        return *this;
    }
    DenseView& operator-=(const Dense& d) {
        if (d.rows() != r_ || d.cols() != c_) throw std::logic_error("eigen_api: operand sizes differ");
        for (Index j = 0; j < c_; ++j)
            for (Index i = 0; i < r_; ++i) (*this)(i, j) -= d(i, j);
        return *this;
    }
    Dense cwiseProduct(const Dense& o) const { return Dense(*this).cwiseProduct(o); }
    double norm() const { return Dense(*this).norm(); }

private:
    double* p_;
    Index r_, c_, ld_;
};

inline Dense::Dense(const DenseView& b) : r_(b.rows()), c_(b.cols()), v_((size_t)(b.rows() * b.cols())) {
    for (Index j = 0; j < c_; ++j)
        for (Index i = 0; i < r_; ++i) (*this)(i, j) = b(i, j);
}

inline DenseView Dense::segment(Index start, Index n) const {
    if (start < 0 || n < 0 || start + n > size()) throw std::out_of_range("eigen_api: segment out of range");
    return DenseView(const_cast<double*>(v_.data()) + start, n, 1, n);
}
inline DenseView Dense::block(Index i, Index j, Index nr, Index nc) const {
    if (i < 0 || j < 0 || i + nr > r_ || j + nc > c_) throw std::out_of_range("eigen_api: block out of range");
    return DenseView(const_cast<double*>(v_.data()) + i + j * r_, nr, nc, r_);
}
inline DenseView Dense::col(Index j) const { return block(0, j, r_, 1); }

inline Dense operator+(const Dense& a, const Dense& b) {
    Dense r(a);
    r += b;
    return r;
}
inline Dense operator-(const Dense& a, const Dense& b) {
    Dense r(a);
    r -= b;
    return r;
}
inline Dense operator-(const Dense& a) {
    Dense r(a.rows(), a.cols());
    for (Index i = 0; i < a.size(); ++i) r(i) = -a(i);
    return r;
}
inline Dense operator*(const Dense& a, double s) {
    Dense r(a.rows(), a.cols());
    for (Index i = 0; i < a.size(); ++i) r(i) = a(i) * s;
    return r;
}
inline Dense operator*(double s, const Dense& a) {
    Dense r(a.rows(), a.cols());
    for (Index i = 0; i < a.size(); ++i) r(i) = s * a(i);
    return r;
}
inline Dense operator/(const Dense& a, double s) {
    Dense r(a.rows(), a.cols());
    for (Index i = 0; i < a.size(); ++i) r(i) = a(i) / s;
    return r;
}
// Matrix product; each coefficient sums its terms in index order.
inline Dense operator*(const Dense& a, const Dense& b) {
    if (a.cols() != b.rows()) throw std::logic_error("eigen_api: product sizes differ");
    Dense r(a.rows(), b.cols());
    for (Index j = 0; j < b.cols(); ++j)
        for (Index i = 0; i < a.rows(); ++i) {
            double s = 0.0;
            for (Index k = 0; k < a.cols(); ++k) s += a(i, k) * b(k, j);
            r(i, j) = s;
        }
    return r;
}

// Matrix<double, R, C>: the fixed- and run-time-sized types the headers name
// (VectorXd, MatrixXd, Vector2d, Matrix2d).  A fixed size is the default
// size; all of them share Dense's storage and arithmetic.
template <typename Scalar, int R, int C, int Options = 0, int MaxR = R, int MaxC = C>
class Matrix : public Dense {
    static_assert(sizeof(Scalar) == sizeof(double), "eigen_api: double only");

public:
    Matrix() : Dense(R < 0 ? 0 : R, C < 0 ? 0 : C) {}
    explicit Matrix(Index n) : Dense(C == 1 ? n : 1, C == 1 ? 1 : n) {}
    Matrix(Index r, Index c) : Dense(r, c) {}
    Matrix(const Dense& d) : Dense(d) { check(); }
    Matrix(const DenseView& b) : Dense(b) { check(); }
    Matrix& operator=(const Dense& d) {
        Dense::operator=(d);
        check();
        return *this;
    }
    Matrix& operator=(const DenseView& b) { return *this = Dense(b); }

    static Matrix Zero() { return Matrix(); }
    static Matrix Zero(Index n) { return Matrix(n); }
    static Matrix Zero(Index r, Index c) { return Matrix(r, c); }

private:
    void check() const {
        if ((R >= 0 && rows() != R) || (C >= 0 && cols() != C))
            throw std::logic_error("eigen_api: size does not fit a fixed-size matrix");
    }
};

typedef Matrix<double, Dynamic, 1> VectorXd;
typedef Matrix<double, Dynamic, Dynamic> MatrixXd;
typedef Matrix<double, 2, 1> Vector2d;
typedef Matrix<double, 2, 2> Matrix2d;
typedef Matrix<double, 4, 1> Vector4d;
typedef Matrix<double, 4, 4> Matrix4d;

// ------------------------------------------------------------------ sparse
template <typename Scalar>
class Triplet {
public:
    Triplet(Index r = 0, Index c = 0, Scalar v = Scalar(0)) : r_(r), c_(c), v_(v) {}
    Index row() const { return r_; }
    Index col() const { return c_; }
    Scalar value() const { return v_; }

private:
    Index r_, c_;
    Scalar v_;
};

// Compressed sparse matrix (rows or columns outer, per Options).  The
// pattern is set by setFromTriplets (duplicates summed); coeffRef on an
// entry outside the pattern inserts it.
template <typename Scalar, int Options = ColMajor, typename StorageIndex = int>
class SparseMatrix {
public:
    SparseMatrix() {}
    SparseMatrix(Index r, Index c) { resize(r, c); }

    Index rows() const { return r_; }
    Index cols() const { return c_; }
    Index outerSize() const { return row_major() ? r_ : c_; }
    Index nonZeros() const { return (Index)inner_.size(); }
    static constexpr bool row_major() { return (Options & RowMajor) != 0; }

    void resize(Index r, Index c) {
        r_ = r;
        c_ = c;
        outer_.assign((size_t)outerSize() + 1, 0);
        inner_.clear();
        val_.clear();
    }
    void setZero() { std::fill(val_.begin(), val_.end(), Scalar(0)); }
    void makeCompressed() {}

    template <typename It>
    void setFromTriplets(It begin, It end) {
        const Index no = outerSize();
        std::vector<std::vector<std::pair<Index, Scalar>>> lists((size_t)no);
        for (It it = begin; it != end; ++it) {
            const Index o = row_major() ? it->row() : it->col();
            const Index in = row_major() ? it->col() : it->row();
            if (it->row() < 0 || it->row() >= r_ || it->col() < 0 || it->col() >= c_)
                throw std::out_of_range("eigen_api: triplet out of range");
            lists[(size_t)o].push_back({in, it->value()});
        }
        outer_.assign((size_t)no + 1, 0);
        inner_.clear();
        val_.clear();
        for (Index o = 0; o < no; ++o) {
            auto& l = lists[(size_t)o];
            std::stable_sort(l.begin(), l.end(),
                             [](const std::pair<Index, Scalar>& a, const std::pair<Index, Scalar>& b) {
                                 return a.first < b.first;
                             });
            for (size_t k = 0; k < l.size(); ++k) {
                if (k > 0 && l[k].first == l[k - 1].first) {
                    val_.back() += l[k].second;
                } else {
                    inner_.push_back(l[k].first);
                    val_.push_back(l[k].second);
                }
            }
            outer_[(size_t)o + 1] = (Index)inner_.size();
        }
    }

    Scalar& coeffRef(Index i, Index j) {
        const Index o = row_major() ? i : j, in = row_major() ? j : i;
        auto b = inner_.begin() + outer_[(size_t)o], e = inner_.begin() + outer_[(size_t)o + 1];
        auto it = std::lower_bound(b, e, in);
        const size_t pos = (size_t)(it - inner_.begin());
        if (it != e && *it == in) return val_[pos];
        inner_.insert(inner_.begin() + (std::ptrdiff_t)pos, in);
        val_.insert(val_.begin() + (std::ptrdiff_t)pos, Scalar(0));
        for (size_t k = (size_t)o + 1; k < outer_.size(); ++k) ++outer_[k];
        return val_[pos];
    }
    Scalar coeff(Index i, Index j) const {
        const Index o = row_major() ? i : j, in = row_major() ? j : i;
        auto b = inner_.begin() + outer_[(size_t)o], e = inner_.begin() + outer_[(size_t)o + 1];
        auto it = std::lower_bound(b, e, in);
        return (it != e && *it == in) ? val_[(size_t)(it - inner_.begin())] : Scalar(0);
    }

    // Compressed-row copy (row pointers, column indices ascending, values).
    void to_csr(std::vector<Index>& ptr, std::vector<Index>& col, std::vector<Scalar>& val) const {
        if (row_major()) {
            ptr = outer_;
            col = inner_;
            val = val_;
            return;
        }
        ptr.assign((size_t)r_ + 1, 0);
        for (Index in : inner_) ++ptr[(size_t)in + 1];
        for (Index i = 0; i < r_; ++i) ptr[(size_t)i + 1] += ptr[(size_t)i];
        col.assign(inner_.size(), 0);
        val.assign(inner_.size(), Scalar(0));
        std::vector<Index> fill(ptr.begin(), ptr.end() - 1);
        for (Index j = 0; j < c_; ++j)
            for (Index k = outer_[(size_t)j]; k < outer_[(size_t)j + 1]; ++k) {
                const Index i = inner_[(size_t)k];
                col[(size_t)fill[(size_t)i]] = j;
                val[(size_t)fill[(size_t)i]++] = val_[(size_t)k];
            }
    }

    // y = A x, each row accumulated in ascending column order.
    friend Dense operator*(const SparseMatrix& A, const Dense& x) {
        if (x.rows() != A.c_ || x.cols() != 1) throw std::logic_error("eigen_api: sparse product sizes differ");
        Dense y(A.r_, 1);
        if (row_major()) {
            for (Index i = 0; i < A.r_; ++i) {
                double s = 0.0;
                for (Index k = A.outer_[(size_t)i]; k < A.outer_[(size_t)i + 1]; ++k)
                    s += A.val_[(size_t)k] * x(A.inner_[(size_t)k]);
                y(i) = s;
            }
        } else {
            for (Index j = 0; j < A.c_; ++j) {
                const double xj = x(j);
                for (Index k = A.outer_[(size_t)j]; k < A.outer_[(size_t)j + 1]; ++k)
                    y(A.inner_[(size_t)k]) += A.val_[(size_t)k] * xj;
            }
        }
        return y;
    }

private:
    Index r_ = 0, c_ = 0;
    std::vector<Index> outer_{0};
    std::vector<Index> inner_;
    std::vector<Scalar> val_;
};

// ----------------------------------------------------- iterative solvers
class IdentityPreconditioner {
public:
    template <typename M>
    IdentityPreconditioner& compute(const M&) { return *this; }
    Dense solve(const Dense& b) const { return b; }
    ComputationInfo info() const { return Success; }
};

// ILU(0): incomplete LU on the pattern of A (Saad, Iterative Methods for
// Sparse Linear Systems, 2nd ed., Algorithm 10.4, IKJ order).  The fill
// factor and drop tolerance of an ILUT are accepted and not used.
template <typename Scalar>
class IncompleteLUT {
public:
    void setFillfactor(int f) { fill_ = f; }
    void setDroptol(double t) { droptol_ = t; }

    template <typename M>
    IncompleteLUT& compute(const M& A) {
        A.to_csr(ptr_, col_, val_);
        const Index n = A.rows();
        diag_.assign((size_t)n, -1);
        info_ = Success;
        for (Index i = 0; i < n; ++i)
            for (Index k = ptr_[(size_t)i]; k < ptr_[(size_t)i + 1]; ++k)
                if (col_[(size_t)k] == i) diag_[(size_t)i] = k;
        std::vector<Index> where((size_t)n, -1);
        for (Index i = 0; i < n; ++i) {
            if (diag_[(size_t)i] < 0) {
                info_ = NumericalIssue;
                return *this;
            }
            for (Index k = ptr_[(size_t)i]; k < ptr_[(size_t)i + 1]; ++k) where[(size_t)col_[(size_t)k]] = k;
            for (Index k = ptr_[(size_t)i]; k < ptr_[(size_t)i + 1] && col_[(size_t)k] < i; ++k) {
                const Index p = col_[(size_t)k];
                const Scalar piv = val_[(size_t)diag_[(size_t)p]];
                if (piv == Scalar(0)) {
                    info_ = NumericalIssue;
                    return *this;
                }
                const Scalar lik = val_[(size_t)k] / piv;
                val_[(size_t)k] = lik;
                for (Index kk = diag_[(size_t)p] + 1; kk < ptr_[(size_t)p + 1]; ++kk) {
                    const Index w = where[(size_t)col_[(size_t)kk]];
                    if (w >= 0) val_[(size_t)w] -= lik * val_[(size_t)kk];
                }
            }
            for (Index k = ptr_[(size_t)i]; k < ptr_[(size_t)i + 1]; ++k) where[(size_t)col_[(size_t)k]] = -1;
            if (val_[(size_t)diag_[(size_t)i]] == Scalar(0)) info_ = NumericalIssue;
        }
        return *this;
    }

    Dense solve(const Dense& b) const {
        const Index n = (Index)diag_.size();
        Dense x(b);
        for (Index i = 0; i < n; ++i) {
            double s = x(i);
            for (Index k = ptr_[(size_t)i]; k < diag_[(size_t)i]; ++k) s -= val_[(size_t)k] * x(col_[(size_t)k]);
            x(i) = s;
        }
        for (Index i = n - 1; i >= 0; --i) {
            double s = x(i);
            for (Index k = diag_[(size_t)i] + 1; k < ptr_[(size_t)i + 1]; ++k) s -= val_[(size_t)k] * x(col_[(size_t)k]);
            x(i) = s / val_[(size_t)diag_[(size_t)i]];
        }
        return x;
    }
    ComputationInfo info() const { return info_; }

private:
    int fill_ = 10;
    double droptol_ = 0.0;
    ComputationInfo info_ = Success;
    std::vector<Index> ptr_, col_, diag_;
    std::vector<Scalar> val_;
};

// Restarted GMRES(m) with right preconditioning (Saad, Algorithm 9.5),
// modified Gram-Schmidt and Givens rotations; zero initial guess; stops when
// ||b - A x|| <= tol ||b||.
template <typename MatrixType, typename Preconditioner>
class GMRES {
public:
    void setTolerance(double t) { tol_ = t; }
    void setMaxIterations(Index n) { max_it_ = n; }
    void set_restart(int m) { restart_ = m; }
    Preconditioner& preconditioner() { return pre_; }
    Index iterations() const { return its_; }
    double error() const { return err_; }
    ComputationInfo info() const { return info_; }

    GMRES& compute(const MatrixType& A) {
        A_ = &A;
        pre_.compute(A);
        info_ = pre_.info();
        return *this;
    }

    Matrix<double, Dynamic, 1> solve(const Dense& b) {
        const Index n = b.rows();
        Dense x(n, 1);
        its_ = 0;
        err_ = 0.0;
        if (!A_) {
            info_ = InvalidInput;
            return x;
        }
        if (pre_.info() != Success) {
            info_ = NumericalIssue;
            return x;
        }
        const double bn = b.norm();
        if (bn == 0.0) {
            info_ = Success;
            return x;
        }
        const int m = restart_;
        std::vector<Dense> V;
        std::vector<double> H((size_t)(m + 1) * m), cs((size_t)m), sn((size_t)m), g((size_t)m + 1);
        auto h = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
        info_ = NoConvergence;
        while (its_ < max_it_) {
            Dense r = b - (*A_) * x;
            double beta = r.norm();
            err_ = beta / bn;
            if (err_ <= tol_) {
                info_ = Success;
                break;
            }
            V.assign(1, r / beta);
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            int k = 0;
            for (; k < m && its_ < max_it_; ++k) {
                ++its_;
                Dense w = (*A_) * pre_.solve(V[(size_t)k]);
                for (int i = 0; i <= k; ++i) {
                    double d = 0.0;
                    for (Index t = 0; t < n; ++t) d += w(t) * V[(size_t)i](t);
                    h(i, k) = d;
                    for (Index t = 0; t < n; ++t) w(t) -= d * V[(size_t)i](t);
                }
                const double hn = w.norm();
                h(k + 1, k) = hn;
                for (int i = 0; i < k; ++i) {
                    const double a = cs[(size_t)i] * h(i, k) + sn[(size_t)i] * h(i + 1, k);
                    h(i + 1, k) = -sn[(size_t)i] * h(i, k) + cs[(size_t)i] * h(i + 1, k);
                    h(i, k) = a;
                }
                const double den = std::sqrt(h(k, k) * h(k, k) + h(k + 1, k) * h(k + 1, k));
                cs[(size_t)k] = den == 0.0 ? 1.0 : h(k, k) / den;
                sn[(size_t)k] = den == 0.0 ? 0.0 : h(k + 1, k) / den;
                h(k, k) = den;
                h(k + 1, k) = 0.0;
                g[(size_t)k + 1] = -sn[(size_t)k] * g[(size_t)k];
                g[(size_t)k] = cs[(size_t)k] * g[(size_t)k];
                err_ = std::fabs(g[(size_t)k + 1]) / bn;
                if (hn == 0.0 || err_ <= tol_) {
                    ++k;
                    break;
                }
                V.push_back(w / hn);
            }
            // x += M^-1 V y, with H y = g (upper triangular, k x k)
            std::vector<double> y((size_t)k);
            for (int i = k - 1; i >= 0; --i) {
                double s = g[(size_t)i];
                for (int j = i + 1; j < k; ++j) s -= h(i, j) * y[(size_t)j];
                y[(size_t)i] = s / h(i, i);
            }
            Dense u(n, 1);
            for (int j = 0; j < k; ++j)
                for (Index t = 0; t < n; ++t) u(t) += y[(size_t)j] * V[(size_t)j](t);
            x += pre_.solve(u);
            if (err_ <= tol_) {
                info_ = Success;
                break;
            }
        }
        return x;
    }

private:
    const MatrixType* A_ = nullptr;
    Preconditioner pre_;
    double tol_ = 1e-12;
    Index max_it_ = 1000;
    int restart_ = 30;
    Index its_ = 0;
    double err_ = 0.0;
    ComputationInfo info_ = Success;
};

}  // namespace Eigen
