/* A utopia backend on this library: CudaTraits (Backend = CUDA), CuVector and CuMatrix.
 *
 * utopia's solvers are templates over a backend that satisfies utopia::Traits
 * (utopia/utopia_core/utopia_Traits.hpp:12-21,306-386; the id CUDA = 100 at :16 is reserved for
 * it).  With this header, the reference's own ConjugateGradient, Multigrid (+ IPRTransfer,
 * MultiLevelMask, Galerkin assembly), Chebyshev3level / PowerMethod, Jacobi, PointJacobi,
 * InvDiagPreconditioner, MPRGP and ProjectedGaussSeidel compile unchanged as
 * Solver<utopia::CuMatrix, utopia::CuVector>: every vector and matrix lives in GPU memory as a
 * ugpu_vec / ugpu_mat and the L1 interfaces (utopia/utopia_core/interfaces/utopia_{Vector,
 * Matrix,Tensor,BLAS_Operands,Normed,Reducible,Transformable,ElementWiseOperand,Operator}.hpp)
 * are one C-ABI call each:
 *   axpy / scale / copy / set        ugpu_axpby, ugpu_vec_copy, ugpu_vec_set
 *   dot / norm2 / dots(...)          ugpu_dot, ugpu_norm2, ugpu_dots (EvalDots specialisation)
 *   reduce / norm1 / norm_infty      ugpu_vec_reduce
 *   transform / e_mul ... e_max      ugpu_vec_transform, ugpu_pointwise
 *   y = A x, b - A x                 ugpu_spmv, ugpu_residual (Eval<ResidualExpr> specialisation)
 *   transpose, A*B, ptap(A, P)       ugpu_transpose, ugpu_spgemm, ugpu_ptap (triple-product Eval)
 *   diag(A)                          ugpu_diag
 * Element-wise host code of the templates (Read/Write locks, get/set, RowView, the
 * UTOPIA_LAMBDA loops of device views, which are host lambdas in the reference's
 * configuration) works on a host mirror with an offload flag, as PETSc's CUDA vectors do for
 * VecGetArray: the mirror is downloaded on first host access, a written mirror is uploaded
 * before the next device operation reads the vector, and a device write invalidates it.
 *
 * Host C++ only (g++ or nvcc); link against libugpu.so.  One process, one GPU: the vectors
 * and matrices share one ugpu context (utopia::cuda::context(), created on device 0 or on
 * the device named by UTOPIA_CUDA_DEVICE, or the one passed to utopia::cuda::set_context).
 * Include it after utopia's headers are on the include path; solver headers after it.
 */
#ifndef UTOPIA_CUDA_BACKEND_HPP
#define UTOPIA_CUDA_BACKEND_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ugpu.h"

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
#include "utopia_RowView.hpp"
#include "utopia_Select.hpp"
#include "utopia_Transformable.hpp"
#include "utopia_Vector.hpp"
#include "utopia_Wrapper.hpp"

#include "utopia_Eval_Residual.hpp"
#include "utopia_LinearSolver.hpp"

namespace utopia {

namespace cuda {

inline ugpu_ctx *&context_slot() {
    static ugpu_ctx *ctx = nullptr;
    return ctx;
}

// Throws std::runtime_error with the library's message when rc != 0.
inline void check(int rc, const char *what) {
    if (rc == 0) return;
    std::string msg = std::string("utopia CUDA backend: ") + what + ": ";
    const char *e = ugpu_last_error(context_slot());
    msg += e ? e : "error";
    throw std::runtime_error(msg);
}

// The shared context (created on first use).
inline ugpu_ctx *context() {
    ugpu_ctx *&c = context_slot();
    if (!c) {
        const char *dev = std::getenv("UTOPIA_CUDA_DEVICE");
        ugpu_ctx *made = nullptr;
        const int rc = ugpu_create(dev ? std::atoi(dev) : 0, &made);
        if (rc != 0) {
            const char *e = ugpu_last_error(nullptr);
            throw std::runtime_error(std::string("utopia CUDA backend: no device context: ") + (e ? e : "error"));
        }
        c = made;
    }
    return c;
}

// Use an existing context (for example the one an application already created).
inline void set_context(ugpu_ctx *ctx) { context_slot() = ctx; }

}  // namespace cuda

class CuVector;
class CuMatrix;
using CuIndexSet = std::vector<SizeType>;

class CudaTraits {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using LocalSizeType = utopia::SizeType;
    using Matrix = CuMatrix;
    using SparseMatrix = CuMatrix;
    using Vector = CuVector;
    using IndexSet = CuIndexSet;
    using IndexArray = std::vector<int>;
    using ScalarArray = std::vector<double>;
    using Communicator = SelfCommunicator;
    using Device = utopia::Device<CUDA>;
    using Layout = utopia::Layout<SelfCommunicator, 1, SizeType>;
    using MatrixLayout = utopia::Layout<SelfCommunicator, 2, SizeType>;

    enum { Backend = CUDA };

    static BackendInfo &backend_info() {
        static BackendInfo instance_("cuda");
        return instance_;
    }
    static constexpr SizeType decide() { return INVALID_INDEX; }
    static constexpr SizeType determine() { return INVALID_INDEX; }
};

UTOPIA_MAKE_TRAITS_SPARSE(CuMatrix, CudaTraits, 2);
UTOPIA_MAKE_TRAITS(CuVector, CudaTraits, 1);

// ------------------------------------------------------------------------------------
// CuVector: an FP64 ugpu_vec with a host mirror for element access
class CuVector final : public DistributedVector<double, SizeType>,
                       public Normed<double>,
                       public Transformable<double>,
                       public Reducible<double>,
                       public ElementWiseOperand<double>,
                       public Constructible<CuVector>,
                       public ElementWiseOperand<CuVector>,
                       public Comparable<CuVector>,
                       public BLAS1Tensor<CuVector>,
                       public Tensor<CuVector, 1>,
                       public Selectable<CuVector, 1> {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using Layout = CudaTraits::Layout;
    using Super = utopia::Tensor<CuVector, 1>;
    using Super::Super;

    template <class Expr>
    CuVector(const Expression<Expr> &expr) {
        Super::construct_eval(expr.derived());
    }
    template <class Expr>
    inline CuVector &operator=(const Expression<Expr> &expr) {
        Super::assign_eval(expr.derived());
        return *this;
    }
    void assign(const CuVector &other) override { copy(other); }
    void assign(CuVector &&other) override { steal(other); }

    CuVector() = default;
    explicit CuVector(const Layout &l, const Scalar &val = 0.0) { values(l, val); }
    CuVector(const CuVector &o) { copy(o); }
    CuVector(CuVector &&o) { steal(o); }
    CuVector &operator=(const CuVector &o) {
        if (this != &o) copy(o);
        return *this;
    }
    CuVector &operator=(CuVector &&o) {
        if (this != &o) steal(o);
        return *this;
    }
    ~CuVector() override { release(); }

    // ---- access to the device vector (device state made current first)
    ugpu_vec *raw() const {
        flush();
        return h_;
    }
    // called after a device operation wrote the vector
    void device_written() { mirror_ = kNone; }

    // host data in and out (synchronous)
    void upload(const std::vector<double> &host) {
        resize(SizeType(host.size()));
        if (n_) cuda::check(ugpu_vec_upload(h_, host.data()), "vector upload");
        device_written();
    }
    std::vector<double> download() const {
        ensure_mirror();
        return host_;
    }

    // ---- locks: host element access goes through the mirror
    void read_lock() override { ensure_mirror(); }
    void write_lock(WriteMode) override { ensure_mirror(); }
    void read_unlock() override {}
    void write_unlock(WriteMode) override {}
    void read_and_write_lock(WriteMode) override { ensure_mirror(); }
    void read_and_write_unlock(WriteMode) override {}

    void set(const SizeType &i, const Scalar &value) override {
        ensure_mirror();
        host_[size_t(i)] = value;
        mirror_ = kDirty;
    }
    void add(const SizeType &i, const Scalar &value) override {
        ensure_mirror();
        host_[size_t(i)] += value;
        mirror_ = kDirty;
    }
    Scalar get(const SizeType &i) const override {
        ensure_mirror();
        return host_[size_t(i)];
    }
    void c_set(const SizeType &i, const Scalar &value) override { set(i, value); }
    void c_add(const SizeType &i, const Scalar &value) override { add(i, value); }
    inline Scalar l_get(const SizeType &i) const { return get(i); }
    inline void l_set(const SizeType &i, const Scalar &value) { set(i, value); }
    inline void l_add(const SizeType &i, const Scalar &value) { add(i, value); }

    void describe() const override {
        for (double e : download()) std::cout << e << " ";
        std::cout << "\n";
    }
    bool empty() const override { return h_ == nullptr; }
    void clear() override { release(); }
    void set(const Scalar &val) override {
        if (!n_) return;
        cuda::check(ugpu_vec_set(h_, val), "vector set");
        device_written();
    }
    SizeType size() const override { return n_; }
    SizeType local_size() const override { return n_; }
    Range range() const override { return Range(0, n_); }
    const SelfCommunicator &comm() const override { return comm_; }

    // ---- BLAS1
    void swap(CuVector &x) override {
        std::swap(h_, x.h_);
        std::swap(n_, x.n_);
        std::swap(host_, x.host_);
        std::swap(mirror_, x.mirror_);
    }
    void scale(const Scalar &a) override { transform_op(UGPU_TR_SCALE, a); }
    void copy(const CuVector &x) override {
        if (this == &x) return;
        resize(x.n_);
        if (n_) cuda::check(ugpu_vec_copy(x.raw(), raw()), "vector copy");
        device_written();
    }
    void axpy(const Scalar &a, const CuVector &x) override {
        if (!n_) return;
        cuda::check(ugpu_axpby(a, x.raw(), 1.0, raw()), "axpy");
        device_written();
    }
    Scalar dot(const CuVector &o) const override {
        double r = 0;
        if (n_) cuda::check(ugpu_dot(raw(), o.raw(), &r), "dot");
        return r;
    }

    // ---- Normed / Reducible
    Scalar norm2() const override {
        double r = 0;
        if (n_) cuda::check(ugpu_norm2(raw(), &r), "norm2");
        return r;
    }
    Scalar norm1() const override { return reduce_op(UGPU_RED_ASUM); }
    Scalar norm_infty() const override { return reduce_op(UGPU_RED_AMAX); }
    Scalar reduce(const Plus &) const override { return reduce_op(UGPU_RED_SUM); }
    Scalar reduce(const Min &) const override { return reduce_op(UGPU_RED_MIN); }
    Scalar reduce(const Max &) const override { return reduce_op(UGPU_RED_MAX); }
    Scalar sum() const override { return reduce_op(UGPU_RED_SUM); }
    Scalar min() const override { return reduce_op(UGPU_RED_MIN); }
    Scalar max() const override { return reduce_op(UGPU_RED_MAX); }

    // ---- element-wise
    void e_mul(const CuVector &o) override { pointwise(UGPU_EMUL, o); }
    void e_div(const CuVector &o) override { pointwise(UGPU_EDIV, o); }
    void e_min(const CuVector &o) override { pointwise(UGPU_EMIN, o); }
    void e_max(const CuVector &o) override { pointwise(UGPU_EMAX, o); }
    void e_mul(const Scalar &a) override { scale(a); }
    void e_div(const Scalar &a) override { transform_op(UGPU_TR_SCALE, 1.0 / a); }
    void e_min(const Scalar &a) override { pointwise(UGPU_EMIN, constant(a)); }
    void e_max(const Scalar &a) override { pointwise(UGPU_EMAX, constant(a)); }

    // ---- Transformable
    void transform(const Sqrt &) override { transform_op(UGPU_TR_SQRT, 0); }
    void transform(const Pow2 &) override { transform_op(UGPU_TR_POW2, 0); }
    void transform(const Log &) override { transform_op(UGPU_TR_LOG, 0); }
    void transform(const Exp &) override { transform_op(UGPU_TR_EXP, 0); }
    void transform(const Cos &) override { transform_op(UGPU_TR_COS, 0); }
    void transform(const Sin &) override { transform_op(UGPU_TR_SIN, 0); }
    void transform(const Abs &) override { transform_op(UGPU_TR_ABS, 0); }
    void transform(const Minus &) override { transform_op(UGPU_TR_MINUS, 0); }
    void transform(const Pow &p) override { transform_op(UGPU_TR_POW, p.a_); }
    void transform(const Reciprocal<double> &r) override { transform_op(UGPU_TR_RECIPROCAL, r.numerator()); }
    template <class F>
    void transform_values(F f) {  // host functor on the mirror
        ensure_mirror();
        for (double &e : host_) e = f(e);
        mirror_ = kDirty;
    }
    void shift(const Scalar &a) { transform_op(UGPU_TR_SHIFT, a); }

    // ---- Constructible
    void values(const Layout &l, const Scalar &val) override {
        resize(l.size());
        set(val);
    }
    void zeros(const Layout &l) override { values(l, 0.0); }

    bool equals(const CuVector &o, const Scalar &tol = 0.0) const override {
        if (o.size() != size()) return false;
        const auto a = download(), b = o.download();
        for (size_t i = 0; i < a.size(); ++i)
            if (std::abs(a[i] - b[i]) > tol) return false;
        return true;
    }
    void select(const CuIndexSet &index, CuVector &result) const override {
        const auto a = download();
        std::vector<double> out(index.size());
        for (size_t i = 0; i < index.size(); ++i) out[i] = a[size_t(index[i])];
        result.upload(out);
    }
    bool has_nan_or_inf() const {
        const double s = reduce_op(UGPU_RED_SUM);
        return !std::isfinite(s) || !std::isfinite(reduce_op(UGPU_RED_AMAX));
    }
    inline bool is_alias(const CuVector &o) const { return this == &o; }
    std::string get_class() const override { return "CuVector"; }

private:
    enum : int { kNone = 0, kValid = 1, kDirty = 2 };
    ugpu_vec *h_ = nullptr;
    SizeType n_ = 0;
    mutable std::vector<double> host_;
    mutable int mirror_ = kNone;
    SelfCommunicator comm_;

    void release() {
        if (h_) ugpu_vec_destroy(h_);
        h_ = nullptr;
        n_ = 0;
        host_.clear();
        mirror_ = kNone;
    }
    void steal(CuVector &o) {
        release();
        std::swap(h_, o.h_);
        std::swap(n_, o.n_);
        std::swap(host_, o.host_);
        std::swap(mirror_, o.mirror_);
    }
    void resize(SizeType n) {
        if (h_ && n == n_) return;
        release();
        cuda::check(ugpu_vec_create(cuda::context(), n, UGPU_F64, &h_), "vector create");
        n_ = n;
    }
    // a written mirror goes to the device before the device reads the vector
    void flush() const {
        if (mirror_ == kDirty) {
            cuda::check(ugpu_vec_upload(h_, host_.data()), "vector upload");
            mirror_ = kValid;
        }
    }
    void ensure_mirror() const {
        if (mirror_ != kNone || !h_) return;
        host_.resize(size_t(n_));
        if (n_) cuda::check(ugpu_vec_download(h_, host_.data()), "vector download");
        mirror_ = kValid;
    }
    Scalar reduce_op(int op) const {
        double r = 0;
        if (n_) cuda::check(ugpu_vec_reduce(raw(), op, &r), "reduce");
        return r;
    }
    void transform_op(int op, double param) {
        if (!n_) return;
        cuda::check(ugpu_vec_transform(raw(), op, param), "transform");
        device_written();
    }
    void pointwise(int op, const CuVector &o) {
        if (!n_) return;
        cuda::check(ugpu_pointwise(op, raw(), o.raw(), raw()), "pointwise");
        device_written();
    }
    CuVector constant(Scalar a) const {
        CuVector c;
        c.values(Layout(comm_, n_, n_), a);
        return c;
    }
};

// ------------------------------------------------------------------------------------
// CuMatrix: an FP64 CSR ugpu_mat (sliced-ELL SpMV layout built by the library)
class CuMatrix final : public DistributedSparseMatrix<double, SizeType>,
                       public Normed<double>,
                       public Transformable<double>,
                       public SparseConstructible<CuMatrix>,
                       public BLAS1Tensor<CuMatrix>,
                       public BLAS2Matrix<CuMatrix, CuVector>,
                       public BLAS3Matrix<CuMatrix>,
                       public Comparable<CuMatrix>,
                       public Operator<CuVector>,
                       public Tensor<CuMatrix, 2>,
                       public Selectable<CuMatrix, 2> {
public:
    using Scalar = double;
    using SizeType = utopia::SizeType;
    using MatrixLayout = CudaTraits::MatrixLayout;
    using Super = utopia::Tensor<CuMatrix, 2>;
    using Super::Super;
    using BLAS2Matrix<CuMatrix, CuVector>::multiply;
    using BLAS3Matrix<CuMatrix>::multiply;

    template <class Expr>
    CuMatrix(const Expression<Expr> &expr) {
        Super::construct_eval(expr.derived());
    }
    template <class Expr>
    inline CuMatrix &operator=(const Expression<Expr> &expr) {
        Super::assign_eval(expr.derived());
        return *this;
    }
    void assign(const CuMatrix &o) override { copy(o); }
    void assign(CuMatrix &&o) override { steal(o); }

    CuMatrix() = default;
    CuMatrix(const CuMatrix &o) { copy(o); }
    CuMatrix(CuMatrix &&o) { steal(o); }
    CuMatrix &operator=(const CuMatrix &o) {
        if (this != &o) copy(o);
        return *this;
    }
    CuMatrix &operator=(CuMatrix &&o) {
        if (this != &o) steal(o);
        return *this;
    }
    ~CuMatrix() override { release(); }

    // CSR from host arrays (copied to the device): int32 indices, FP64 values, ascending columns
    void from_csr(SizeType m, SizeType n, const int *rp, const int *ci, const double *v) {
        release();
        cuda::check(ugpu_csr_create(cuda::context(), m, n, rp[m], reinterpret_cast<const int32_t *>(rp),
                                    reinterpret_cast<const int32_t *>(ci), v, &h_),
                    "CSR create");
        nrows_ = m;
        ncols_ = n;
    }
    // adopt a matrix the library created
    void adopt(ugpu_mat *h) {
        release();
        h_ = h;
        int64_t m = 0, n = 0, nnz = 0;
        int dt = 0;
        cuda::check(ugpu_mat_info(h_, &m, &n, &nnz, &dt), "matrix info");
        nrows_ = m;
        ncols_ = n;
    }
    ugpu_mat *raw() const {
        flush();
        return h_;
    }
    SizeType nnz() const {
        int64_t m = 0, n = 0, z = 0;
        int dt = 0;
        if (h_) cuda::check(ugpu_mat_info(h_, &m, &n, &z, &dt), "matrix info");
        return z;
    }

    // host CSR mirror (RowView, read, transform_values, get)
    const std::vector<int> &host_rowptr() const {
        ensure_mirror();
        return rp_;
    }
    const std::vector<int> &host_colidx() const {
        ensure_mirror();
        return ci_;
    }
    const std::vector<double> &host_values() const {
        ensure_mirror();
        return v_;
    }

    void read_lock() override { ensure_mirror(); }
    void write_lock(WriteMode) override { ensure_mirror(); }
    void read_unlock() override {}
    void write_unlock(WriteMode) override {}
    void read_and_write_lock(WriteMode) { ensure_mirror(); }
    void read_and_write_unlock(WriteMode) {}

    Scalar get(const SizeType &i, const SizeType &j) const {
        ensure_mirror();
        for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k)
            if (ci_[size_t(k)] == j) return v_[size_t(k)];
        return 0.0;
    }
    void set(const SizeType &i, const SizeType &j, const Scalar &value) override { *find(i, j) = value; }
    void add(const SizeType &i, const SizeType &j, const Scalar &value) override { *find(i, j) += value; }
    void c_set(const SizeType &i, const SizeType &j, const Scalar &value) override { set(i, j, value); }
    void c_add(const SizeType &i, const SizeType &j, const Scalar &value) override { add(i, j, value); }
    void set(const Scalar &val) {
        ensure_mirror();
        std::fill(v_.begin(), v_.end(), val);
        dirty_ = true;
    }

    void describe() const override {
        ensure_mirror();
        for (SizeType i = 0; i < nrows_; ++i)
            for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k)
                std::cout << i << " " << ci_[size_t(k)] << " " << v_[size_t(k)] << "\n";
    }
    bool empty() const override { return h_ == nullptr; }
    void clear() override { release(); }
    SizeType rows() const override { return nrows_; }
    SizeType cols() const override { return ncols_; }
    SizeType local_rows() const override { return nrows_; }
    SizeType local_cols() const override { return ncols_; }
    Range row_range() const override { return Range(0, nrows_); }
    Range col_range() const override { return Range(0, ncols_); }
    Size size() const override { return {nrows_, ncols_}; }
    Size local_size() const override { return {nrows_, ncols_}; }
    const SelfCommunicator &comm() const override { return comm_; }
    bool is_alias(const CuMatrix &o) const { return this == &o; }
    std::string get_class() const override { return "CuMatrix"; }
    bool is_sparse() const { return true; }

    // ---- Normed (on the stored values)
    Scalar norm2() const override {
        double s = 0;
        for (double v : host_values()) s += v * v;
        return std::sqrt(s);
    }
    Scalar norm1() const override {
        ensure_mirror();
        std::vector<double> c(size_t(ncols_), 0.0);
        for (size_t k = 0; k < ci_.size(); ++k) c[size_t(ci_[k])] += std::abs(v_[k]);
        return c.empty() ? 0.0 : *std::max_element(c.begin(), c.end());
    }
    Scalar norm_infty() const override {
        ensure_mirror();
        double m = 0;
        for (SizeType i = 0; i < nrows_; ++i) {
            double s = 0;
            for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k) s += std::abs(v_[size_t(k)]);
            m = std::max(m, s);
        }
        return m;
    }

    // ---- Transformable (stored values)
    template <class F>
    void transform_values(F f) {
        ensure_mirror();
        for (double &e : v_) e = f(e);
        dirty_ = true;
    }
    template <class F>
    void read(F f) const {
        ensure_mirror();
        for (SizeType i = 0; i < nrows_; ++i)
            for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k) f(i, SizeType(ci_[size_t(k)]), v_[size_t(k)]);
    }
    bool write(const std::string &path) const {
        return h_ && ugpu_petsc_write_mat(raw(), path.c_str()) == 0;
    }
    template <class Op>
    void each(const Op &op) {
        transform_values([&op](double v) { return op.apply(v); });
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
        transform_values([](double v) { return -v; });
    }

    // ---- SparseConstructible
    void sparse(const MatrixLayout &l, const SizeType &, const SizeType &) override {
        std::vector<int> rp(size_t(l.size(0)) + 1, 0), ci(1, 0);
        std::vector<double> v(1, 0.0);
        from_csr(l.size(0), l.size(1), rp.data(), ci.data(), v.data());
    }
    void identity(const MatrixLayout &l, const Scalar &d = 1.0) override {
        const SizeType m = l.size(0), n = l.size(1), k = std::min(m, n);
        std::vector<int> rp(static_cast<size_t>(m) + 1, 0), ci(static_cast<size_t>(k));
        std::vector<double> v(size_t(k), d);
        for (SizeType i = 0; i < m; ++i) rp[size_t(i) + 1] = rp[size_t(i)] + (i < k ? 1 : 0);
        for (SizeType i = 0; i < k; ++i) ci[size_t(i)] = int(i);
        from_csr(m, n, rp.data(), ci.data(), v.data());
    }

    // ---- BLAS1 on the values (same pattern)
    void swap(CuMatrix &o) override {
        std::swap(h_, o.h_);
        std::swap(nrows_, o.nrows_);
        std::swap(ncols_, o.ncols_);
        std::swap(rp_, o.rp_);
        std::swap(ci_, o.ci_);
        std::swap(v_, o.v_);
        std::swap(mirrored_, o.mirrored_);
        std::swap(dirty_, o.dirty_);
        std::swap(t_, o.t_);
    }
    void scale(const Scalar &a) override {
        transform_values([a](double v) { return v * a; });
    }
    void copy(const CuMatrix &o) override {
        if (this == &o) return;
        if (!o.h_) {
            release();
            return;
        }
        o.ensure_mirror();
        from_csr(o.nrows_, o.ncols_, o.rp_.data(), o.ci_.data(), o.v_.data());
    }
    void axpy(const Scalar &a, const CuMatrix &x) override {
        ensure_mirror();
        x.ensure_mirror();
        if (x.rp_ == rp_ && x.ci_ == ci_) {
            for (size_t k = 0; k < v_.size(); ++k) v_[k] += a * x.v_[k];
            dirty_ = true;
            return;
        }
        // union of the two patterns (MatAXPY with DIFFERENT_NONZERO_PATTERN), rebuilt on the device
        std::vector<int> rp(static_cast<size_t>(nrows_) + 1, 0), ci;
        std::vector<double> v;
        for (SizeType i = 0; i < nrows_; ++i) {
            int p = rp_[size_t(i)], q = x.rp_[size_t(i)];
            const int pe = rp_[size_t(i) + 1], qe = x.rp_[size_t(i) + 1];
            while (p < pe || q < qe) {
                const int cp = p < pe ? ci_[size_t(p)] : std::numeric_limits<int>::max();
                const int cq = q < qe ? x.ci_[size_t(q)] : std::numeric_limits<int>::max();
                if (cp == cq) {
                    ci.push_back(cp);
                    v.push_back(v_[size_t(p++)] + a * x.v_[size_t(q++)]);
                } else if (cp < cq) {
                    ci.push_back(cp);
                    v.push_back(v_[size_t(p++)]);
                } else {
                    ci.push_back(cq);
                    v.push_back(a * x.v_[size_t(q++)]);
                }
            }
            rp[size_t(i) + 1] = int(ci.size());
        }
        if (ci.empty()) ci.push_back(0), v.push_back(0.0);  // valid pointers for an empty pattern
        const SizeType m = nrows_, n = ncols_;
        from_csr(m, n, rp.data(), ci.data(), v.data());
    }
    Scalar dot(const CuMatrix &o) const override {
        ensure_mirror();
        o.ensure_mirror();
        double s = 0;
        for (size_t k = 0; k < v_.size(); ++k) s += v_[k] * o.v_[k];
        return s;
    }

    // ---- BLAS2
    void multiply(const CuVector &x, CuVector &y) const override {
        if (y.is_alias(x)) {  // y = A y: multiply a copy (as PetscMatrix::multiply does)
            CuVector t(x);
            multiply(t, y);
            return;
        }
        if (y.size() != nrows_) y.zeros(CudaTraits::Layout(comm_, nrows_, nrows_));
        cuda::check(ugpu_spmv(raw(), x.raw(), y.raw()), "SpMV");
        y.device_written();
    }
    void gemv(const bool transpose_, const Scalar &alpha, const CuVector &x, const Scalar &beta,
              CuVector &y) const override {
        const CuMatrix &op = transpose_ ? transposed() : *this;
        CuVector t;
        op.multiply(x, t);
        if (beta == 0.0) {
            t.scale(alpha);
            y = std::move(t);
        } else {
            y.scale(beta);
            y.axpy(alpha, t);
        }
    }
    void multiply_add(const Scalar &alpha, const CuVector &x, const Scalar &beta, CuVector &y) const override {
        if (alpha == 1.0 && beta == 1.0 && !y.is_alias(x)) {  // MatMultAdd
            cuda::check(ugpu_spmv_add(raw(), x.raw(), y.raw(), y.raw()), "SpMV add");
            y.device_written();
            return;
        }
        gemv(false, alpha, x, beta, y);
    }
    bool apply(const CuVector &rhs, CuVector &sol) const override {
        multiply(rhs, sol);
        return true;
    }

    // ---- BLAS3
    void transpose(CuMatrix &C) const override {
        ugpu_mat *t = nullptr;
        cuda::check(ugpu_transpose(raw(), &t), "transpose");
        C.adopt(t);
    }
    void multiply(const Scalar &alpha, const CuMatrix &B, CuMatrix &C) const override {
        ugpu_mat *c = nullptr;
        cuda::check(ugpu_spgemm(raw(), B.raw(), &c), "SpGEMM");
        C.adopt(c);
        if (alpha != 1.0) C.scale(alpha);
    }
    void multiply(const bool tA, const bool tB, const CuMatrix &B, CuMatrix &C) const override {
        const CuMatrix &a = tA ? transposed() : *this;
        const CuMatrix &b = tB ? B.transposed() : B;
        a.multiply(1.0, b, C);
    }
    // MatPtAP with the full symbolic structure
    static void ptap(const CuMatrix &A, const CuMatrix &P, CuMatrix &C) {
        ugpu_mat *c = nullptr;
        cuda::check(ugpu_ptap(A.raw(), P.raw(), &c), "PtAP");
        C.adopt(c);
    }

    // ---- diagonal
    void build_diag(CuVector &d) const {
        if (d.size() != nrows_) d.zeros(CudaTraits::Layout(comm_, nrows_, nrows_));
        cuda::check(ugpu_diag(raw(), d.raw()), "diag");
        d.device_written();
    }
    void diag(const CuVector &d) {
        const auto v = d.download();
        const SizeType n = SizeType(v.size());
        std::vector<int> rp(static_cast<size_t>(n) + 1), ci(static_cast<size_t>(n));
        for (SizeType i = 0; i <= n; ++i) rp[size_t(i)] = int(i);
        for (SizeType i = 0; i < n; ++i) ci[size_t(i)] = int(i);
        from_csr(n, n, rp.data(), ci.data(), v.data());
    }
    void shift_diag(const Scalar &a) {
        ensure_mirror();
        for (SizeType i = 0; i < nrows_; ++i)
            for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k)
                if (ci_[size_t(k)] == i) v_[size_t(k)] += a;
        dirty_ = true;
    }

    bool equals(const CuMatrix &o, const Scalar &tol = 0.0) const override {
        ensure_mirror();
        o.ensure_mirror();
        if (o.nrows_ != nrows_ || o.ncols_ != ncols_ || o.rp_ != rp_ || o.ci_ != ci_) return false;
        for (size_t k = 0; k < v_.size(); ++k)
            if (std::abs(v_[k] - o.v_[k]) > tol) return false;
        return true;
    }
    void select(const CuIndexSet &, const CuIndexSet &, CuMatrix &) const override {
        throw std::runtime_error("CuMatrix::select is not provided by this backend");
    }
    bool has_nan_or_inf() const {
        for (double v : host_values())
            if (!std::isfinite(v)) return true;
        return false;
    }

private:
    ugpu_mat *h_ = nullptr;
    SizeType nrows_ = 0, ncols_ = 0;
    mutable std::vector<int> rp_, ci_;
    mutable std::vector<double> v_;
    mutable bool mirrored_ = false;
    mutable bool dirty_ = false;
    mutable std::shared_ptr<CuMatrix> t_;  // cached transpose for transposed products
    SelfCommunicator comm_;

    void release() {
        if (h_) ugpu_mat_destroy(h_);
        h_ = nullptr;
        nrows_ = ncols_ = 0;
        rp_.clear();
        ci_.clear();
        v_.clear();
        mirrored_ = dirty_ = false;
        t_.reset();
    }
    void steal(CuMatrix &o) {
        release();
        swap(o);
    }
    void ensure_mirror() const {
        if (mirrored_ || !h_) return;
        const SizeType z = nnz();
        rp_.resize(size_t(nrows_) + 1);
        ci_.resize(size_t(z));
        v_.resize(size_t(z));
        cuda::check(ugpu_csr_download(h_, reinterpret_cast<int32_t *>(rp_.data()),
                                      reinterpret_cast<int32_t *>(ci_.data()), v_.data()),
                    "CSR download");
        mirrored_ = true;
    }
    // written values go to the device (same pattern) before the device reads the matrix
    void flush() const {
        if (!dirty_) return;
        cuda::check(ugpu_mat_update_values(h_, v_.data()), "matrix values update");
        dirty_ = false;
        t_.reset();
    }
    double *find(SizeType i, SizeType j) {
        ensure_mirror();
        for (int k = rp_[size_t(i)]; k < rp_[size_t(i) + 1]; ++k)
            if (ci_[size_t(k)] == j) {
                dirty_ = true;
                return &v_[size_t(k)];
            }
        throw std::runtime_error("CuMatrix: entry outside the sparsity pattern");
    }
    const CuMatrix &transposed() const {
        flush();
        if (!t_) {
            t_ = std::make_shared<CuMatrix>();
            transpose(*t_);
        }
        return *t_;
    }
};

// ------------------------------------------------------------------------------------
// backend evaluations

// row access through the host mirror (ProjectedGaussSeidel::step)
template <class Tensor>
class RowView<Tensor, 2, FillType::SPARSE, CUDA> {
public:
    using SizeType = typename utopia::Traits<Tensor>::SizeType;
    using Scalar = typename utopia::Traits<Tensor>::Scalar;

    inline RowView(Tensor &t, const SizeType row)
        : rp_(t.host_rowptr()), ci_(t.host_colidx()), v_(t.host_values()), row_(row) {}
    inline SizeType n_values() const { return rp_[size_t(row_) + 1] - rp_[size_t(row_)]; }
    inline SizeType col(const SizeType index) const { return ci_[size_t(rp_[size_t(row_)] + index)]; }
    inline Scalar get(const SizeType index) const { return v_[size_t(rp_[size_t(row_)] + index)]; }

private:
    const std::vector<int> &rp_;
    const std::vector<int> &ci_;
    const std::vector<double> &v_;
    SizeType row_;
};

// r = b - A x in one pass (ugpu_residual)
template <class Traits_>
class Eval<ResidualExpr<CuMatrix, CuVector, CuVector>, Traits_, CUDA> {
public:
    using Expr = utopia::ResidualExpr<CuMatrix, CuVector, CuVector>;
    using Result = CuVector;

    UTOPIA_EVAL_APPLY_TO_TEMPORARY(Expr, Result)

    inline static void apply(const Expr &expr, Result &result) {
        const CuMatrix &a = expr.right().left().derived();
        const CuVector &x = expr.right().right().derived();
        const CuVector &b = expr.left().derived();
        if (result.is_alias(x) || result.is_alias(b)) {
            CuVector t;
            apply(expr, t);
            result = std::move(t);
            return;
        }
        if (result.size() != a.rows()) result.zeros(CudaTraits::Layout(SelfCommunicator(), a.rows(), a.rows()));
        cuda::check(ugpu_residual(a.raw(), b.raw(), x.raw(), result.raw()), "residual");
        result.device_written();
    }
};

// transpose(P) * A * P as one Galerkin product (MatPtAP)
template <class M1, class M2, class Traits_>
class Eval<Multiply<Multiply<Transposed<M1>, M2>, M1>, Traits_, CUDA> {
public:
    using Expr = utopia::Multiply<Multiply<Transposed<M1>, M2>, M1>;
    using Result = EXPR_TYPE(Traits_, Expr);

    inline static Result apply(const Expr &expr) {
        Result result;
        apply(expr, result);
        return result;
    }
    inline static void apply(const Expr &expr, Result &result) {
        CuMatrix::ptap(Eval<M2, Traits_>::apply(expr.left().right()), Eval<M1, Traits_>::apply(expr.right()), result);
    }
};

// fused dots (VecMDot): one reduction pass for 2 or 3 pairs
template <>
class EvalDots<CuVector, CUDA> {
public:
    using Scalar = double;

    static void apply(const CuVector &v1, const std::vector<std::shared_ptr<CuVector>> &vs, std::vector<Scalar> &r) {
        r.resize(vs.size());
        for (size_t i = 0; i < vs.size(); ++i) r[i] = v1.dot(*vs[i]);
    }
    static void apply(const CuVector &v1, const std::vector<CuVector> &vs, std::vector<Scalar> &r) {
        r.resize(vs.size());
        for (size_t i = 0; i < vs.size(); ++i) r[i] = v1.dot(vs[i]);
    }
    static void apply(const CuVector &a1, const CuVector &b1, Scalar &r1, const CuVector &a2, const CuVector &b2,
                      Scalar &r2) {
        const ugpu_vec *a[2] = {a1.raw(), a2.raw()}, *b[2] = {b1.raw(), b2.raw()};
        double out[2] = {0, 0};
        if (a1.size()) cuda::check(ugpu_dots(2, a, b, out), "dots");
        r1 = out[0];
        r2 = out[1];
    }
    static void apply(const CuVector &a1, const CuVector &b1, Scalar &r1, const CuVector &a2, const CuVector &b2,
                      Scalar &r2, const CuVector &a3, const CuVector &b3, Scalar &r3) {
        const ugpu_vec *a[3] = {a1.raw(), a2.raw(), a3.raw()}, *b[3] = {b1.raw(), b2.raw(), b3.raw()};
        double out[3] = {0, 0, 0};
        if (a1.size()) cuda::check(ugpu_dots(3, a, b, out), "dots");
        r1 = out[0];
        r2 = out[1];
        r3 = out[2];
    }
};

// Dense Cholesky direct solver on the GPU for small (coarse-level) operators: the place the
// reference's tests give PETSc's Factorization (utopia/backend/petsc/solvers/linear/
// utopia_petsc_Factorization.hpp), e.g. Multigrid<CuMatrix, CuVector>(smoother, coarse).
class CuCholesky final : public LinearSolver<CuMatrix, CuVector> {
public:
    CuCholesky() = default;
    CuCholesky(const CuCholesky &) {}
    ~CuCholesky() override {
        if (s_) ugpu_solver_destroy(s_);
    }
    CuCholesky *clone() const override { return new CuCholesky(); }
    void update(const std::shared_ptr<const CuMatrix> &op) override {
        LinearSolver<CuMatrix, CuVector>::update(op);
        if (!s_) cuda::check(ugpu_solver_create(cuda::context(), UGPU_SOLVER_CHOLESKY, &s_), "Cholesky create");
        cuda::check(ugpu_solver_update(s_, op->raw()), "Cholesky factorisation");
    }
    bool apply(const CuVector &rhs, CuVector &x) override {
        if (x.size() != rhs.size()) x.zeros(layout(rhs));
        cuda::check(ugpu_solver_apply(s_, rhs.raw(), x.raw()), "Cholesky solve");
        x.device_written();
        return true;
    }

private:
    ugpu_solver *s_ = nullptr;
};

}  // namespace utopia

#endif  // UTOPIA_CUDA_BACKEND_HPP
