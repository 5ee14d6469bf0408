// CPU FP64 CSR backend for the reference's own solver templates -- TEST INFRASTRUCTURE ONLY.
//
// utopia's solvers (ConjugateGradient, Multigrid, Chebyshev3level, Jacobi, PointJacobi,
// PowerMethod, MPRGP, ProjectedGaussSeidel, ...) are templates over a backend satisfying
// utopia::Traits (utopia/utopia_core/utopia_Traits.hpp:12-21,306-386).  Their numeric kernels
// normally come from PETSc, which is not available here.  This header is a small serial
// backend (Backend = HOMEMADE) whose vector and CSR matrix implement the L1 interfaces
// (utopia/utopia_core/interfaces/utopia_{Vector,Matrix,Tensor,BLAS_Operands,Operator}.hpp)
// with plain loops that restate the PETSc kernels the solvers call:
//   MatMult            y_i = sum_k a_ik x_k in CSR order  (utopia_petsc_Matrix.cpp:1358)
//   MatMultAdd         z = y + A x                        (utopia_petsc_Matrix.cpp:1400-1404)
//   VecDot / VecNorm   sums in fixed blocks of 8192 entries, then the block sums in order
//                      (the summation order of the restated oracle, so that the two agree
//                      bit for bit and a difference isolates the solver logic)
//   VecAXPY            y_i += a x_i                       (utopia_petsc_Vector.cpp:671)
//   MatGetDiagonal     0 where a row stores no diagonal   (utopia_petsc_Matrix.cpp:756)
//   MatTranspose, MatPtAP with the full symbolic structure (utopia_petsc_Eval_Multiply.cpp:12-61)
// The reference's templates are compiled unchanged against it (oracle/ref/ref_solvers.cpp).
#pragma once

#include <algorithm>
#include <cmath>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "utopia_Base.hpp"
#include "utopia_DeviceView.hpp"
#include "utopia_RangeDevice.hpp"
#include "utopia_Core.hpp"

#include "utopia_BLAS_Operands.hpp"
#include "utopia_BackendInfo.hpp"
#include "utopia_Communicator.hpp"
#include "utopia_Comparable.hpp"
#include "utopia_Constructible.hpp"
#include "utopia_Device.hpp"
#include "utopia_ElementWiseOperand.hpp"
#include "utopia_Interfaces.hpp"
#include "utopia_Layout.hpp"
#include "utopia_Matrix.hpp"
#include "utopia_Normed.hpp"
#include "utopia_Operator.hpp"
#include "utopia_Reducible.hpp"
#include "utopia_Select.hpp"
#include "utopia_Transformable.hpp"
#include "utopia_Vector.hpp"
#include "utopia_Wrapper.hpp"

#include "utopia_LinearSolver.hpp"
#include "utopia_RowView.hpp"

#include <algorithm>
#include <cmath>
#include <iostream>
#include <limits>
#include <memory>
#include <vector>

namespace utopia {

class RefVector;
class RefMatrix;

// index sets of this backend (Selectable)
using RefIndexSet = std::vector<SizeType>;

class RefTraits {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using LocalSizeType = utopia::SizeType;
    using Matrix = RefMatrix;
    using SparseMatrix = RefMatrix;
    using Vector = RefVector;
    using IndexSet = RefIndexSet;
    using IndexArray = std::vector<int>;
    using ScalarArray = std::vector<double>;
    using Communicator = SelfCommunicator;
    using Device = utopia::Device<HOMEMADE>;
    using Layout = utopia::Layout<SelfCommunicator, 1, SizeType>;
    using MatrixLayout = utopia::Layout<SelfCommunicator, 2, SizeType>;

    enum { Backend = HOMEMADE };

    static BackendInfo &backend_info() {
        static BackendInfo instance_("ref_cpu");
        return instance_;
    }
    static constexpr SizeType decide() { return INVALID_INDEX; }
    static constexpr SizeType determine() { return INVALID_INDEX; }
};

UTOPIA_MAKE_TRAITS_SPARSE(RefMatrix, RefTraits, 2);
UTOPIA_MAKE_TRAITS(RefVector, RefTraits, 1);

namespace ref {
constexpr SizeType kBlock = 8192;

inline double blocked_dot(SizeType n, const double *a, const double *b) {
    double total = 0.0;
    for (SizeType s = 0; s < n; s += kBlock) {
        const SizeType e = std::min(n, s + kBlock);
        double part = 0.0;
        for (SizeType i = s; i < e; ++i) part += a[i] * b[i];
        total += part;
    }
    return total;
}
}  // namespace ref

// ------------------------------------------------------------------------------------
class RefVector final : public DistributedVector<double, SizeType>,
                        public Normed<double>,
                        public Transformable<double>,
                        public Reducible<double>,
                        public ElementWiseOperand<double>,
                        public Constructible<RefVector>,
                        public ElementWiseOperand<RefVector>,
                        public Comparable<RefVector>,
                        public BLAS1Tensor<RefVector>,
                        public Tensor<RefVector, 1>,
                        public Selectable<RefVector, 1> {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using Layout = RefTraits::Layout;
    using Super = utopia::Tensor<RefVector, 1>;
    using Super::Super;

    template <class Expr>
    RefVector(const Expression<Expr> &expr) {
        Super::construct_eval(expr.derived());
    }
    template <class Expr>
    inline RefVector &operator=(const Expression<Expr> &expr) {
        Super::assign_eval(expr.derived());
        return *this;
    }
    void assign(const RefVector &other) override { copy(other); }
    void assign(RefVector &&other) override { v_ = std::move(other.v_); }

    RefVector() = default;
    explicit RefVector(const Layout &l, const Scalar &val = 0.0) { values(l, val); }
    RefVector(const RefVector &o) : v_(o.v_) {}
    RefVector(RefVector &&o) : v_(std::move(o.v_)) {}
    RefVector &operator=(const RefVector &o) {
        if (this != &o) copy(o);
        return *this;
    }
    RefVector &operator=(RefVector &&o) {
        if (this != &o) v_ = std::move(o.v_);
        return *this;
    }

    // storage access for the driver
    std::vector<double> &data() { return v_; }
    const std::vector<double> &data() const { return v_; }
    double *ptr() { return v_.data(); }
    const double *ptr() const { return v_.data(); }

    // locks are no-ops
    void read_lock() override {}
    void write_lock(WriteMode) override {}
    void read_unlock() override {}
    void write_unlock(WriteMode) override {}
    void read_and_write_lock(WriteMode) override {}
    void read_and_write_unlock(WriteMode) override {}

    void set(const SizeType &i, const Scalar &value) override { v_[size_t(i)] = value; }
    void add(const SizeType &i, const Scalar &value) override { v_[size_t(i)] += value; }
    Scalar get(const SizeType &i) const override { return v_[size_t(i)]; }
    void c_set(const SizeType &i, const Scalar &value) override { set(i, value); }
    void c_add(const SizeType &i, const Scalar &value) override { add(i, value); }
    inline Scalar l_get(const SizeType &i) const { return v_[size_t(i)]; }
    inline void l_set(const SizeType &i, const Scalar &value) { v_[size_t(i)] = value; }
    inline void l_add(const SizeType &i, const Scalar &value) { v_[size_t(i)] += value; }

    void describe() const override {
        for (double e : v_) std::cout << e << " ";
        std::cout << "\n";
    }
    bool empty() const override { return v_.empty(); }
    void clear() override { v_.clear(); }
    void set(const Scalar &val) override { std::fill(v_.begin(), v_.end(), val); }
    SizeType size() const override { return SizeType(v_.size()); }
    SizeType local_size() const override { return SizeType(v_.size()); }
    Range range() const override { return Range(0, size()); }
    const SelfCommunicator &comm() const override { return comm_; }

    // BLAS1
    void swap(RefVector &x) override { std::swap(v_, x.v_); }
    void scale(const Scalar &a) override {
        for (double &e : v_) e *= a;
    }
    void copy(const RefVector &x) override { v_ = x.v_; }
    void axpy(const Scalar &a, const RefVector &x) override {
        const size_t n = v_.size();
        for (size_t i = 0; i < n; ++i) v_[i] += a * x.v_[i];
    }
    Scalar dot(const RefVector &o) const override { return ref::blocked_dot(size(), ptr(), o.ptr()); }

    // Normed
    Scalar norm2() const override { return std::sqrt(ref::blocked_dot(size(), ptr(), ptr())); }
    Scalar norm1() const override {
        double s = 0;
        for (double e : v_) s += std::abs(e);
        return s;
    }
    Scalar norm_infty() const override {
        double m = 0;
        for (double e : v_) m = std::max(m, std::abs(e));
        return m;
    }

    // Reducible
    Scalar reduce(const Plus &) const override { return sum(); }
    Scalar reduce(const Min &) const override { return min(); }
    Scalar reduce(const Max &) const override { return max(); }
    Scalar sum() const override {
        double s = 0;
        for (double e : v_) s += e;
        return s;
    }
    Scalar min() const override {
        double m = std::numeric_limits<double>::max();
        for (double e : v_) m = std::min(m, e);
        return m;
    }
    Scalar max() const override {
        double m = -std::numeric_limits<double>::max();
        for (double e : v_) m = std::max(m, e);
        return m;
    }

    // element-wise
    void e_mul(const RefVector &o) override {
        for (size_t i = 0; i < v_.size(); ++i) v_[i] *= o.v_[i];
    }
    void e_div(const RefVector &o) override {
        for (size_t i = 0; i < v_.size(); ++i) v_[i] /= o.v_[i];
    }
    void e_min(const RefVector &o) override {
        for (size_t i = 0; i < v_.size(); ++i) v_[i] = std::min(o.v_[i], v_[i]);
    }
    void e_max(const RefVector &o) override {
        for (size_t i = 0; i < v_.size(); ++i) v_[i] = std::max(o.v_[i], v_[i]);
    }
    void e_mul(const Scalar &a) override { scale(a); }
    void e_div(const Scalar &a) override {
        for (double &e : v_) e /= a;
    }
    void e_min(const Scalar &a) override {
        for (double &e : v_) e = std::min(a, e);
    }
    void e_max(const Scalar &a) override {
        for (double &e : v_) e = std::max(a, e);
    }

    // Transformable
    template <class Op>
    void each(const Op &op) {
        for (double &e : v_) e = op.apply(e);
    }
    void transform(const Sqrt &op) override { each(op); }
    void transform(const Pow2 &op) override { each(op); }
    void transform(const Log &op) override { each(op); }
    void transform(const Exp &op) override { each(op); }
    void transform(const Cos &op) override { each(op); }
    void transform(const Sin &op) override { each(op); }
    void transform(const Abs &op) override { each(op); }
    void transform(const Pow &op) override { each(op); }
    void transform(const Reciprocal<double> &op) override { each(op); }
    void transform(const Minus &) override {
        for (double &e : v_) e = -e;
    }
    template <class F>
    void transform_values(F f) {
        for (double &e : v_) e = f(e);
    }

    // Constructible
    void values(const Layout &l, const Scalar &val) override { v_.assign(size_t(l.size()), val); }
    void zeros(const Layout &l) override { values(l, 0.0); }

    bool equals(const RefVector &o, const Scalar &tol = 0.0) const override {
        if (o.size() != size()) return false;
        for (size_t i = 0; i < v_.size(); ++i)
            if (std::abs(v_[i] - o.v_[i]) > tol) return false;
        return true;
    }

    void select(const RefIndexSet &index, RefVector &result) const override {
        result.v_.resize(index.size());
        for (size_t i = 0; i < index.size(); ++i) result.v_[i] = v_[size_t(index[i])];
    }

    bool has_nan_or_inf() const {
        for (double e : v_)
            if (!std::isfinite(e)) return true;
        return false;
    }
    inline bool is_alias(const RefVector &o) const { return this == &o; }
    std::string get_class() const override { return "RefVector"; }
    void shift(const Scalar &a) {
        for (double &e : v_) e += a;
    }

private:
    std::vector<double> v_;
    SelfCommunicator comm_;
};

// ------------------------------------------------------------------------------------
class RefMatrix final : public DistributedSparseMatrix<double, SizeType>,
                        public Normed<double>,
                        public Transformable<double>,
                        public SparseConstructible<RefMatrix>,
                        public BLAS1Tensor<RefMatrix>,
                        public BLAS2Matrix<RefMatrix, RefVector>,
                        public BLAS3Matrix<RefMatrix>,
                        public Comparable<RefMatrix>,
                        public Operator<RefVector>,
                        public Tensor<RefMatrix, 2>,
                        public Selectable<RefMatrix, 2> {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using MatrixLayout = RefTraits::MatrixLayout;
    using Super = utopia::Tensor<RefMatrix, 2>;
    using Super::Super;
    using BLAS2Matrix<RefMatrix, RefVector>::multiply;
    using BLAS3Matrix<RefMatrix>::multiply;
    using BLAS3Matrix<RefMatrix>::transpose_multiply;
    // y = A^T x (MatMultTranspose, PetscMatrix::transpose_multiply, utopia_petsc_Matrix.cpp:1368-1380)
    void transpose_multiply(const RefVector &x, RefVector &y) const override { gemv(true, 1.0, x, 0.0, y); }
    void transpose_multiply(const Scalar &alpha, const RefVector &x, RefVector &y) const override {
        gemv(true, alpha, x, 0.0, y);
    }

    template <class Expr>
    RefMatrix(const Expression<Expr> &expr) {
        Super::construct_eval(expr.derived());
    }
    template <class Expr>
    inline RefMatrix &operator=(const Expression<Expr> &expr) {
        Super::assign_eval(expr.derived());
        return *this;
    }
    void assign(const RefMatrix &o) override { copy(o); }
    void assign(RefMatrix &&o) override { steal(o); }

    RefMatrix() = default;
    RefMatrix(const RefMatrix &o) { copy(o); }
    RefMatrix(RefMatrix &&o) { steal(o); }
    RefMatrix &operator=(const RefMatrix &o) {
        if (this != &o) copy(o);
        return *this;
    }
    RefMatrix &operator=(RefMatrix &&o) {
        if (this != &o) steal(o);
        return *this;
    }

    // CSR arrays (int32 column indices, FP64 values, columns ascending per row)
    SizeType nrows = 0, ncols = 0;
    std::vector<int> rowptr{0}, colidx;
    std::vector<double> vals;

    void from_csr(SizeType m, SizeType n, const int *rp, const int *ci, const double *v) {
        nrows = m;
        ncols = n;
        rowptr.assign(rp, rp + m + 1);
        colidx.assign(ci, ci + rp[m]);
        vals.assign(v, v + rp[m]);
    }
    SizeType nnz() const { return SizeType(colidx.size()); }

    // locks are no-ops
    void read_lock() override {}
    void write_lock(WriteMode) override {}
    void read_unlock() override {}
    void write_unlock(WriteMode) override {}
    void read_and_write_lock(WriteMode) {}
    void read_and_write_unlock(WriteMode) {}

    Scalar get(const SizeType &i, const SizeType &j) const {
        for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
            if (colidx[size_t(k)] == j) return vals[size_t(k)];
        return 0.0;
    }
    // structural entries only (a CSR pattern is fixed once assembled)
    void set(const SizeType &i, const SizeType &j, const Scalar &value) override { *find(i, j) = value; }
    void add(const SizeType &i, const SizeType &j, const Scalar &value) override { *find(i, j) += value; }
    void c_set(const SizeType &i, const SizeType &j, const Scalar &value) override { set(i, j, value); }
    void c_add(const SizeType &i, const SizeType &j, const Scalar &value) override { add(i, j, value); }
    void set(const Scalar &val) { std::fill(vals.begin(), vals.end(), val); }

    void describe() const override {
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                std::cout << i << " " << colidx[size_t(k)] << " " << vals[size_t(k)] << "\n";
    }
    bool empty() const override { return nrows == 0 && ncols == 0; }
    void clear() override {
        nrows = ncols = 0;
        rowptr.assign(1, 0);
        colidx.clear();
        vals.clear();
    }
    SizeType rows() const override { return nrows; }
    SizeType cols() const override { return ncols; }
    SizeType local_rows() const override { return nrows; }
    SizeType local_cols() const override { return ncols; }
    Range row_range() const override { return Range(0, nrows); }
    Range col_range() const override { return Range(0, ncols); }
    Size size() const override { return {nrows, ncols}; }
    Size local_size() const override { return {nrows, ncols}; }
    const SelfCommunicator &comm() const override { return comm_; }
    bool is_alias(const RefMatrix &o) const { return this == &o; }
    std::string get_class() const override { return "RefMatrix"; }

    // Normed
    Scalar norm2() const override {  // Frobenius
        double s = 0;
        for (double v : vals) s += v * v;
        return std::sqrt(s);
    }
    Scalar norm1() const override {
        std::vector<double> c(size_t(ncols), 0.0);
        for (SizeType k = 0; k < nnz(); ++k) c[size_t(colidx[size_t(k)])] += std::abs(vals[size_t(k)]);
        return c.empty() ? 0.0 : *std::max_element(c.begin(), c.end());
    }
    Scalar norm_infty() const override {
        double m = 0;
        for (SizeType i = 0; i < nrows; ++i) {
            double s = 0;
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k) s += std::abs(vals[size_t(k)]);
            m = std::max(m, s);
        }
        return m;
    }

    // Transformable (stored values)
    template <class Op>
    void each(const Op &op) {
        for (double &e : vals) e = op.apply(e);
    }
    void transform(const Sqrt &op) override { each(op); }
    void transform(const Pow2 &op) override { each(op); }
    void transform(const Log &op) override { each(op); }
    void transform(const Exp &op) override { each(op); }
    void transform(const Cos &op) override { each(op); }
    void transform(const Sin &op) override { each(op); }
    void transform(const Abs &op) override { each(op); }
    void transform(const Pow &op) override { each(op); }
    void transform(const Reciprocal<double> &op) override { each(op); }
    void transform(const Minus &) override {
        for (double &e : vals) e = -e;
    }
    // f(value) -> value on every stored entry
    template <class F>
    void transform_values(F f) {
        for (double &e : vals) e = f(e);
    }
    // f(i, j, value) on every stored entry, rows in order
    template <class F>
    void read(F f) const {
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k) f(i, SizeType(colidx[size_t(k)]), vals[size_t(k)]);
    }
    bool write(const std::string &) const { return false; }

    // SparseConstructible
    void sparse(const MatrixLayout &l, const SizeType &, const SizeType &) override {
        nrows = l.size(0);
        ncols = l.size(1);
        rowptr.assign(size_t(nrows) + 1, 0);
        colidx.clear();
        vals.clear();
    }
    void identity(const MatrixLayout &l, const Scalar &d = 1.0) override {
        nrows = l.size(0);
        ncols = l.size(1);
        const SizeType m = std::min(nrows, ncols);
        rowptr.assign(size_t(nrows) + 1, 0);
        for (SizeType i = 0; i < nrows; ++i) rowptr[size_t(i) + 1] = rowptr[size_t(i)] + (i < m ? 1 : 0);
        colidx.resize(size_t(m));
        vals.assign(size_t(m), d);
        for (SizeType i = 0; i < m; ++i) colidx[size_t(i)] = int(i);
    }

    // BLAS1 on the stored values (same pattern)
    void swap(RefMatrix &o) override {
        std::swap(nrows, o.nrows);
        std::swap(ncols, o.ncols);
        rowptr.swap(o.rowptr);
        colidx.swap(o.colidx);
        vals.swap(o.vals);
    }
    void scale(const Scalar &a) override {
        for (double &v : vals) v *= a;
    }
    void copy(const RefMatrix &o) override {
        nrows = o.nrows;
        ncols = o.ncols;
        rowptr = o.rowptr;
        colidx = o.colidx;
        vals = o.vals;
    }
    void axpy(const Scalar &a, const RefMatrix &x) override;
    Scalar dot(const RefMatrix &o) const override {
        double s = 0;
        for (size_t k = 0; k < vals.size(); ++k) s += vals[k] * o.vals[k];
        return s;
    }

    // BLAS2: y := alpha op(A) x + beta y, MatMult order (row sums in CSR order)
    void gemv(const bool transpose, const Scalar &alpha, const RefVector &x, const Scalar &beta,
              RefVector &y) const override;
    void multiply(const RefVector &x, RefVector &y) const override;
    void multiply_add(const Scalar &alpha, const RefVector &x, const Scalar &beta, RefVector &y) const override {
        gemv(false, alpha, x, beta, y);
    }

    // Operator
    bool apply(const RefVector &rhs, RefVector &sol) const override {
        multiply(rhs, sol);
        return true;
    }

    // BLAS3
    void transpose(RefMatrix &C) const override;
    void multiply(const Scalar &alpha, const RefMatrix &B, RefMatrix &C) const override;
    void multiply(const bool transpose_A, const bool transpose_B, const RefMatrix &B, RefMatrix &C) const override;

    // diagonal access (MatGetDiagonal / diag(v) / shift)
    void build_diag(RefVector &d) const {
        d.values(RefTraits::Layout(comm_, nrows, nrows), 0.0);
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                if (colidx[size_t(k)] == i) d.set(i, vals[size_t(k)]);
    }
    void diag(const RefVector &d) {
        const SizeType n = d.size();
        nrows = ncols = n;
        rowptr.resize(size_t(n) + 1);
        colidx.resize(size_t(n));
        vals.resize(size_t(n));
        for (SizeType i = 0; i <= n; ++i) rowptr[size_t(i)] = int(i);
        for (SizeType i = 0; i < n; ++i) {
            colidx[size_t(i)] = int(i);
            vals[size_t(i)] = d.get(i);
        }
    }
    void shift_diag(const Scalar &a) {
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                if (colidx[size_t(k)] == i) vals[size_t(k)] += a;
    }
    void shift_diag(const RefVector &d) {
        if (empty()) {  // an empty matrix becomes diag(d) (PetscMatrix::shift_diag, utopia_petsc_Matrix.cpp:1783-1789)
            diag(d);
            return;
        }
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                if (colidx[size_t(k)] == i) vals[size_t(k)] += d.get(i);
    }

    bool equals(const RefMatrix &o, const Scalar &tol = 0.0) const override {
        if (o.nrows != nrows || o.ncols != ncols || o.rowptr != rowptr || o.colidx != colidx) return false;
        for (size_t k = 0; k < vals.size(); ++k)
            if (std::abs(vals[k] - o.vals[k]) > tol) return false;
        return true;
    }
    void select(const RefIndexSet &, const RefIndexSet &, RefMatrix &) const override {
        throw std::runtime_error("RefMatrix::select is not provided by this backend");
    }

    // P^T A P with the full symbolic structure (MatPtAP)
    static void ptap(const RefMatrix &A, const RefMatrix &P, RefMatrix &C);

    bool is_sparse() const { return true; }
    bool has_nan_or_inf() const {
        for (double v : vals)
            if (!std::isfinite(v)) return true;
        return false;
    }

private:
    SelfCommunicator comm_;
    double *find(SizeType i, SizeType j) {
        for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
            if (colidx[size_t(k)] == j) return &vals[size_t(k)];
        throw std::runtime_error("RefMatrix: entry outside the sparsity pattern");
    }
    void steal(RefMatrix &o) {
        nrows = o.nrows;
        ncols = o.ncols;
        rowptr = std::move(o.rowptr);
        colidx = std::move(o.colidx);
        vals = std::move(o.vals);
    }
};

// ------------------------------------------------------------------------------------
inline void RefMatrix::gemv(const bool transpose_, const Scalar &alpha, const RefVector &x, const Scalar &beta,
                            RefVector &y) const {
    if (y.is_alias(x)) {
        RefVector t(x);
        gemv(transpose_, alpha, t, beta, y);
        return;
    }
    const SizeType m = transpose_ ? ncols : nrows;
    if (y.size() != m) y.values(RefTraits::Layout(comm_, m, m), 0.0);
    if (!transpose_) {
        for (SizeType i = 0; i < nrows; ++i) {
            double s = 0;
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                s += vals[size_t(k)] * x.l_get(colidx[size_t(k)]);
            y.l_set(i, beta == 0.0 ? alpha * s : alpha * s + beta * y.l_get(i));
        }
    } else {
        std::vector<double> t(size_t(ncols), 0.0);
        for (SizeType i = 0; i < nrows; ++i)
            for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k)
                t[size_t(colidx[size_t(k)])] += vals[size_t(k)] * x.l_get(i);
        for (SizeType j = 0; j < ncols; ++j) y.l_set(j, beta == 0.0 ? alpha * t[size_t(j)] : alpha * t[size_t(j)] + beta * y.l_get(j));
    }
}

inline void RefMatrix::multiply(const RefVector &x, RefVector &y) const {
    if (y.is_alias(x)) {  // y = A y: multiply a copy (as PetscMatrix::multiply does)
        RefVector t(x);
        multiply(t, y);
        return;
    }
    if (y.size() != nrows) y.values(RefTraits::Layout(comm_, nrows, nrows), 0.0);
    for (SizeType i = 0; i < nrows; ++i) {
        double s = 0;
        for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k) s += vals[size_t(k)] * x.l_get(colidx[size_t(k)]);
        y.l_set(i, s);
    }
}

inline void RefMatrix::transpose(RefMatrix &T) const {
    RefMatrix R;
    R.nrows = ncols;
    R.ncols = nrows;
    R.rowptr.assign(size_t(ncols) + 1, 0);
    for (int c : colidx) R.rowptr[size_t(c) + 1]++;
    for (SizeType j = 0; j < ncols; ++j) R.rowptr[size_t(j) + 1] += R.rowptr[size_t(j)];
    R.colidx.resize(colidx.size());
    R.vals.resize(vals.size());
    std::vector<int> pos(R.rowptr.begin(), R.rowptr.end() - 1);
    for (SizeType i = 0; i < nrows; ++i)
        for (int k = rowptr[size_t(i)]; k < rowptr[size_t(i) + 1]; ++k) {
            const int p = pos[size_t(colidx[size_t(k)])]++;
            R.colidx[size_t(p)] = int(i);
            R.vals[size_t(p)] = vals[size_t(k)];
        }
    T = std::move(R);
}

namespace ref {
// C = A B keeping every structurally produced entry, columns ascending, products summed
// in A-row order
inline void spgemm(const RefMatrix &A, const RefMatrix &B, RefMatrix &C) {
    RefMatrix R;
    R.nrows = A.nrows;
    R.ncols = B.ncols;
    R.rowptr.assign(size_t(A.nrows) + 1, 0);
    std::vector<SizeType> mark(size_t(B.ncols), -1);
    std::vector<double> acc(size_t(B.ncols), 0.0);
    std::vector<int> cols;
    for (SizeType i = 0; i < A.nrows; ++i) {
        cols.clear();
        for (int ka = A.rowptr[size_t(i)]; ka < A.rowptr[size_t(i) + 1]; ++ka) {
            const int j = A.colidx[size_t(ka)];
            const double a = A.vals[size_t(ka)];
            for (int kb = B.rowptr[size_t(j)]; kb < B.rowptr[size_t(j) + 1]; ++kb) {
                const int c = B.colidx[size_t(kb)];
                if (mark[size_t(c)] != i) {
                    mark[size_t(c)] = i;
                    acc[size_t(c)] = 0.0;
                    cols.push_back(c);
                }
                acc[size_t(c)] += a * B.vals[size_t(kb)];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int c : cols) {
            R.colidx.push_back(c);
            R.vals.push_back(acc[size_t(c)]);
        }
        R.rowptr[size_t(i) + 1] = int(R.colidx.size());
    }
    C = std::move(R);
}
}  // namespace ref

inline void RefMatrix::multiply(const Scalar &alpha, const RefMatrix &B, RefMatrix &C) const {
    ref::spgemm(*this, B, C);
    if (alpha != 1.0) C.scale(alpha);
}

inline void RefMatrix::multiply(const bool tA, const bool tB, const RefMatrix &B, RefMatrix &C) const {
    RefMatrix At, Bt;
    if (tA) transpose(At);
    if (tB) B.transpose(Bt);
    ref::spgemm(tA ? At : *this, tB ? Bt : B, C);
}

inline void RefMatrix::ptap(const RefMatrix &A, const RefMatrix &P, RefMatrix &C) {
    RefMatrix R, AP;
    P.transpose(R);
    ref::spgemm(A, P, AP);
    ref::spgemm(R, AP, C);
}

inline void RefMatrix::axpy(const Scalar &a, const RefMatrix &x) {
    if (x.rowptr == rowptr && x.colidx == colidx) {
        for (size_t k = 0; k < vals.size(); ++k) vals[k] += a * x.vals[k];
        return;
    }
    // union pattern
    RefMatrix R;
    R.nrows = nrows;
    R.ncols = ncols;
    R.rowptr.assign(size_t(nrows) + 1, 0);
    for (SizeType i = 0; i < nrows; ++i) {
        int p = rowptr[size_t(i)], q = x.rowptr[size_t(i)];
        const int pe = rowptr[size_t(i) + 1], qe = x.rowptr[size_t(i) + 1];
        while (p < pe || q < qe) {
            const int cp = p < pe ? colidx[size_t(p)] : std::numeric_limits<int>::max();
            const int cq = q < qe ? x.colidx[size_t(q)] : std::numeric_limits<int>::max();
            if (cp == cq) {
                R.colidx.push_back(cp);
                R.vals.push_back(vals[size_t(p++)] + a * x.vals[size_t(q++)]);
            } else if (cp < cq) {
                R.colidx.push_back(cp);
                R.vals.push_back(vals[size_t(p++)]);
            } else {
                R.colidx.push_back(cq);
                R.vals.push_back(a * x.vals[size_t(q++)]);
            }
        }
        R.rowptr[size_t(i) + 1] = int(R.colidx.size());
    }
    *this = std::move(R);
}

// ------------------------------------------------------------------------------------
// MatPtAP: transpose(P) * A * P evaluated as one triple product (the pattern the PETSc
// backend matches in utopia/backend/petsc/eval/utopia_petsc_Eval_Multiply.hpp)
template <class M1, class M2, class Traits_>
class Eval<Multiply<Multiply<Transposed<M1>, M2>, M1>, Traits_, HOMEMADE> {
public:
    using Expr = utopia::Multiply<Multiply<Transposed<M1>, M2>, M1>;
    using Result = EXPR_TYPE(Traits_, Expr);

    inline static Result apply(const Expr &expr) {
        Result result;
        apply(expr, result);
        return result;
    }
    inline static void apply(const Expr &expr, Result &result) {
        RefMatrix::ptap(Eval<M2, Traits_>::apply(expr.left().right()), Eval<M1, Traits_>::apply(expr.right()),
                        result);
    }
};


// row access of the CSR backend (used by ProjectedGaussSeidel::step)
template <class Tensor>
class RowView<Tensor, 2, FillType::SPARSE, HOMEMADE> {
public:
    using SizeType = typename utopia::Traits<Tensor>::SizeType;
    using Scalar = typename utopia::Traits<Tensor>::Scalar;

    inline RowView(Tensor &t, const SizeType row) : t_(t), row_(row) {}
    inline SizeType n_values() const { return t_.rowptr[size_t(row_) + 1] - t_.rowptr[size_t(row_)]; }
    inline SizeType col(const SizeType index) const { return t_.colidx[size_t(t_.rowptr[size_t(row_)] + index)]; }
    inline Scalar get(const SizeType index) const { return t_.vals[size_t(t_.rowptr[size_t(row_)] + index)]; }

private:
    Tensor &t_;
    SizeType row_;
};

// dense Cholesky direct solver for the coarse level
class RefCholesky final : public LinearSolver<RefMatrix, RefVector> {
public:
    RefCholesky *clone() const override { return new RefCholesky(*this); }
    void update(const std::shared_ptr<const RefMatrix> &op) override {
        LinearSolver<RefMatrix, RefVector>::update(op);
        const RefMatrix &A = *op;
        n_ = A.nrows;
        L_.assign(size_t(n_ * n_), 0.0);
        for (SizeType i = 0; i < n_; ++i)
            for (int k = A.rowptr[size_t(i)]; k < A.rowptr[size_t(i) + 1]; ++k)
                L_[size_t(i * n_ + A.colidx[size_t(k)])] = A.vals[size_t(k)];
        ok_ = true;
        for (SizeType j = 0; j < n_ && ok_; ++j) {
            double s = L_[size_t(j * n_ + j)];
            for (SizeType k = 0; k < j; ++k) s -= L_[size_t(j * n_ + k)] * L_[size_t(j * n_ + k)];
            if (!(s > 0.0)) {
                ok_ = false;
                break;
            }
            const double ljj = std::sqrt(s);
            L_[size_t(j * n_ + j)] = ljj;
            for (SizeType i = j + 1; i < n_; ++i) {
                double t = L_[size_t(i * n_ + j)];
                for (SizeType k = 0; k < j; ++k) t -= L_[size_t(i * n_ + k)] * L_[size_t(j * n_ + k)];
                L_[size_t(i * n_ + j)] = t / ljj;
            }
        }
    }
    bool apply(const RefVector &b, RefVector &x) override {
        if (!ok_) throw std::runtime_error("coarse operator is not SPD");
        if (x.size() != n_) x.zeros(RefTraits::Layout(SelfCommunicator(), n_, n_));
        std::vector<double> y(static_cast<size_t>(n_), 0.0);
        for (SizeType i = 0; i < n_; ++i) {
            double s = b.get(i);
            for (SizeType k = 0; k < i; ++k) s -= L_[size_t(i * n_ + k)] * y[size_t(k)];
            y[size_t(i)] = s / L_[size_t(i * n_ + i)];
        }
        for (SizeType i = n_ - 1; i >= 0; --i) {
            double s = y[size_t(i)];
            for (SizeType k = i + 1; k < n_; ++k) s -= L_[size_t(k * n_ + i)] * x.get(k);
            x.set(i, s / L_[size_t(i * n_ + i)]);
        }
        return true;
    }

private:
    SizeType n_ = 0;
    std::vector<double> L_;
    bool ok_ = false;
};

}  // namespace utopia
