// ShiftedPenaltyQPSolver (utopia/solvers/nonlinear/constrained/penalty/
// utopia_ShiftedPenaltyQPSolver_impl.hpp:87-156) with the ShiftedPenalty term
// (utopia/solvers/nonlinear/constrained/penalty/utopia_ShiftedPenalty.hpp), the solver of the
// reference's qp_solve app (utopia/apps/qp_solve/utopia_qp_solve.cpp:61-107).
//
// One iteration, all on the device:
//   g = A x - b (the residual product, negated where it is used)
//   w = x, or O^T (T x) with a transformation (the constraint space)
//   ShiftedPenalty::update_shift_aux (:348-463) on w, one fused kernel that also writes the
//   penalty gradient -p dps (:32-50) and the Hessian diagonal active p (:52-75), both multiplied
//   by the selection (Penalty::apply_selection) and mapped by the scaling matrix; p grows by
//   penalty_parameter_factor up to penalty_parameter_max before the kernel (update_shift)
//   c = the gradient, or T^T (O gc) with a transformation (gradient, :283-330)
//   rhs = -(g + c)
//   H = A + diag(h), or A + T^T (O^T diag(h) O) T (hessian, :181-237; the app's transform_matrix):
//   the union structure of A and the penalty term is built once (MatAXPY with a different
//   pattern), the Galerkin products keep their structure, and every iteration only recomputes
//   values and refreshes the sliced-ELL layout
//   c = 0; solve H c = rhs; x += c; stop on check_convergence(it, 1, 1, ||c||).
// The constraint is the upper bound: update() fills a missing one with the largest double
// (VariableBoundSolverInterface::init_memory -> BoxConstraints::fill_empty_bounds), so
// update_shift_aux always takes its upper-bound branch and a lower bound is never enforced.
// The inner solver is CG + Jacobi to linear_rtol * ||rhs|| (H is symmetric positive definite)
// unless one is set through ugpu_solver_set_preconditioner (the reference's linear_solver slot).
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "abi_util.cuh"
#include "solver.cuh"

namespace ugpu {
namespace {

#define PEN_LOOP(i, n) \
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

// ---- C = A + B for CSR matrices with ascending columns (union structure, built once) ----

__device__ __forceinline__ int32_t merged_count(const int32_t *ca, int32_t a, int32_t ae, const int32_t *cb, int32_t b,
                                                int32_t be) {
    int32_t k = 0;
    while (a < ae || b < be) {
        const int32_t x = a < ae ? ca[a] : INT32_MAX;
        const int32_t y = b < be ? cb[b] : INT32_MAX;
        a += x <= y;
        b += y <= x;
        ++k;
    }
    return k;
}

__global__ void k_add_count(int64_t n, const int32_t *ra, const int32_t *ca, const int32_t *rb, const int32_t *cb,
                            int64_t *cnt) {
    PEN_LOOP(i, n) cnt[i] = merged_count(ca, ra[i], ra[i + 1], cb, rb[i], rb[i + 1]);
}

__global__ void k_add_structure(int64_t n, const int32_t *ra, const int32_t *ca, const int32_t *rb, const int32_t *cb,
                                const int64_t *pos, int32_t *rc, int32_t *cc) {
    PEN_LOOP(i, n) {
        int32_t a = ra[i], ae = ra[i + 1], b = rb[i], be = rb[i + 1];
        int64_t k = pos[i];
        rc[i] = int32_t(k);
        if (i == n - 1) rc[n] = int32_t(pos[n]);
        while (a < ae || b < be) {
            const int32_t x = a < ae ? ca[a] : INT32_MAX;
            const int32_t y = b < be ? cb[b] : INT32_MAX;
            cc[k++] = x < y ? x : y;
            a += x <= y;
            b += y <= x;
        }
    }
}

// values: a + b where both have the entry, else the one that has it (MatAXPY with alpha 1)
__global__ void k_add_values(int64_t n, const int32_t *ra, const int32_t *ca, const double *va, const int32_t *rb,
                             const int32_t *cb, const double *vb, const int32_t *rc, double *vc) {
    PEN_LOOP(i, n) {
        int32_t a = ra[i], ae = ra[i + 1], b = rb[i], be = rb[i + 1];
        int32_t k = rc[i];
        while (a < ae || b < be) {
            const int32_t x = a < ae ? ca[a] : INT32_MAX;
            const int32_t y = b < be ? cb[b] : INT32_MAX;
            vc[k++] = x == y ? va[a] + vb[b] : (x < y ? va[a] : vb[b]);
            a += x <= y;
            b += y <= x;
        }
    }
}

__global__ void k_identity_structure(int64_t n, int32_t *rp, int32_t *ci) {
    PEN_LOOP(i, n) {
        rp[i] = int32_t(i);
        ci[i] = int32_t(i);
        if (i == n - 1) rp[n] = int32_t(n);
    }
}

// ---- the penalty terms ----

// update_shift_aux (upper-bound branch) + penalty_gradient + penalty_hessian + apply_selection,
// for constraint-space position w: d = ub - w; dps = d + s; active = dps <= 0; s = active dps;
// dps = active (d + s); gradient 0 - p dps; Hessian diagonal active p
__global__ void k_penalty_terms(int64_t m, const double *__restrict__ w, const double *__restrict__ ub, double p,
                                const double *__restrict__ sel, double *__restrict__ shift, double *__restrict__ gc,
                                double *__restrict__ h) {
    PEN_LOOP(i, m) {
        const double di = ub[i] - w[i];
        double si = shift[i];
        double dps = di + si;
        const double a = dps <= 0.0 ? 1.0 : 0.0;
        si = a * dps;
        dps = a * (di + si);
        shift[i] = si;
        double g = 0.0 - p * dps;
        double hh = a * p;
        if (sel) {
            g = sel[i] * g;
            hh = sel[i] * hh;
        }
        gc[i] = g;
        h[i] = hh;
    }
}

// rhs = -((A x - b) + (0 + c)) with r = b - A x
__global__ void k_penalty_rhs(int64_t n, const double *__restrict__ r, const double *__restrict__ c,
                              double *__restrict__ rhs) {
    PEN_LOOP(i, n) rhs[i] = -((-r[i]) + (0.0 + c[i]));
}

class ShiftedPenalty final : public Solver {
public:
    explicit ShiftedPenalty(Context *c) : Solver(c, UGPU_SOLVER_SHIFTED_PENALTY) {
        // ShiftedPenalty defaults (utopia_ShiftedPenalty.hpp:581-584); penalty_parameter_max 0
        // takes penalty_parameter, as ShiftedPenalty::read does
        prm["penalty_parameter"] = 1e4;
        prm["penalty_parameter_max"] = 0;
        prm["penalty_parameter_factor"] = 1.5;
        prm["zero_shift_on_reset"] = 1;
        prm["linear_rtol"] = 1e-12;
        prm["linear_max_it"] = 10000;
    }

    void set_preconditioner(Solver *s) override { user_linear_ = s; }
    void set_box(const Vec *lb, const Vec *ub) override {
        for (const Vec *v : {lb, ub})
            UGPU_CHECK(!v || v->dtype == UGPU_F64, UGPU_ERR_ARG, "box constraints must be FP64 vectors");
        lb_ = lb;
        ub_ = ub;
    }

    void set_transform(const Mat *T, const Mat *O) {
        UGPU_CHECK((T == nullptr) == (O == nullptr), UGPU_ERR_ARG, "ShiftedPenalty: both T and O, or neither");
        if (T) {
            UGPU_CHECK(T->nrows == T->ncols && O->nrows == O->ncols && T->nrows == O->nrows && T->vdtype == UGPU_F64 &&
                           O->vdtype == UGPU_F64,
                       UGPU_ERR_ARG, "ShiftedPenalty: square FP64 transformation matrices of one size");
            Tt_ = transpose(*T);
            Ot_ = transpose(*O);
        } else {
            Tt_.reset();
            Ot_.reset();
        }
        T_ = T;
        O_ = O;
        invalidate();
    }
    void set_selection(const Vec *sel) {
        UGPU_CHECK(!sel || sel->dtype == UGPU_F64, UGPU_ERR_ARG, "ShiftedPenalty: FP64 selection vector");
        sel_ = sel;
    }
    void set_scaling(const Mat *S) {
        UGPU_CHECK(!S || (S->nrows == S->ncols && S->vdtype == UGPU_F64), UGPU_ERR_ARG,
                   "ShiftedPenalty: square FP64 scaling matrix");
        S_ = S;
    }

    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG,
                   "ShiftedPenalty: square FP64 operator required");
        op = A;
        invalidate();
        const int64_t n = A->nrows;
        const size_t b = sizeof(double) * size_t(std::max<int64_t>(n, 1));
        for (Buffer *w : {&res_, &rhs_, &corr_, &w_, &gc_, &gs_, &t1_, &t2_}) w->alloc(b);
        if (shift_n_ != n) {
            shift_.alloc(b);
            UGPU_CUDA(cudaMemsetAsync(shift_.ptr, 0, b, ctx->stream));  // reset_buffers: a new shift is zero
            shift_n_ = n;
        }
        if (!user_linear_ && !linear_) {
            linear_ = make_cg(ctx);
            jacobi_ = make_invdiag(ctx);
            linear_->set_preconditioner(jacobi_.get());
        }
    }

    void apply(const Vec &bv, Vec &xv) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "ShiftedPenalty: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(bv.n == n && xv.n == n && bv.dtype == UGPU_F64 && xv.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "ShiftedPenalty: FP64 vectors of the operator's size required");
        UGPU_CHECK((!ub_ || ub_->n == n) && (!lb_ || lb_->n == n) && (!sel_ || sel_->n == n), UGPU_ERR_ARG,
                   "ShiftedPenalty: bound / selection size mismatch");
        UGPU_CHECK(!T_ || T_->nrows == n, UGPU_ERR_ARG, "ShiftedPenalty: transformation size mismatch");
        UGPU_CHECK(!S_ || S_->nrows == n, UGPU_ERR_ARG, "ShiftedPenalty: scaling matrix size mismatch");
        const double t0 = now_s();
        const int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        const double *ub = ub_ ? ub_->as<double>() : nullptr;
        if (!ub) {  // fill_empty_bounds
            ubfill_.alloc(sizeof(double) * size_t(std::max<int64_t>(n, 1)));
            enq_set(*ctx, UGPU_F64, n, DBL_MAX, ubfill_.ptr, nullptr);
            ub = ubfill_.as<double>();
        }
        const double *sel = sel_ ? sel_->as<double>() : nullptr;
        double *x = xv.as<double>();
        if (get("zero_shift_on_reset") != 0)  // ShiftedPenalty::reset
            UGPU_CUDA(cudaMemsetAsync(shift_.ptr, 0, sizeof(double) * size_t(n), ctx->stream));
        const double p0 = get("penalty_parameter");
        const double pmax = get("penalty_parameter_max") != 0 ? get("penalty_parameter_max") : p0;
        const double factor = get("penalty_parameter_factor");
        double p = p0;
        build_structures();
        Solver *lin = user_linear_ ? user_linear_ : linear_.get();
        const int g = stream_grid(*ctx, n);
        Vec rv, cv;
        rv.ctx = cv.ctx = ctx;
        rv.n = cv.n = n;
        rv.dtype = cv.dtype = UGPU_F64;
        rv.buf.borrow(rhs_.ptr, sizeof(double) * size_t(n));
        cv.buf.borrow(corr_.ptr, sizeof(double) * size_t(n));
        double *c = corr_.as<double>();
        int64_t lin_its = 0;
        const int64_t max_it = int64_t(get("max_it"));
        for (int64_t it = 1; it <= max_it; ++it) {
            spmv(*op, x, res_.as<double>(), bv.as<double>());  // r = b - A x
            const double *w = x;
            if (T_) {
                spmv(*T_, x, t1_.as<double>());
                spmv(*Ot_, t1_.as<double>(), w_.as<double>());
                w = w_.as<double>();
            }
            p = std::min(pmax, factor * p);  // update_shift
            double *gc = gc_.as<double>(), *h = D_->vals.as<double>();
            k_penalty_terms<<<g, kBlock, 0, ctx->stream>>>(n, w, ub, p, sel, shift_.as<double>(), gc, h);
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
            if (S_) {  // scaling_matrix()->apply: gc = S gc, h = S h
                spmv(*S_, gc, gs_.as<double>());
                gc = gs_.as<double>();
                spmv(*S_, h, t2_.as<double>());
                enq_copy(*ctx, UGPU_F64, n, t2_.ptr, h, nullptr);
            }
            const double *cg = gc;  // the gradient in the problem space
            if (T_) {
                spmv(*O_, gc, t1_.as<double>());
                spmv(*Tt_, t1_.as<double>(), t2_.as<double>());
                cg = t2_.as<double>();
            }
            k_penalty_rhs<<<g, kBlock, 0, ctx->stream>>>(n, res_.as<double>(), cg, rhs_.as<double>());
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
            assemble_hessian();
            enq_set(*ctx, UGPU_F64, n, 0.0, c, nullptr);
            if (!user_linear_) {
                lin->set("atol", get("linear_rtol") * norm(rhs_.as<double>(), n));
                lin->set("max_it", get("linear_max_it"));
            }
            lin->update(H_.get());
            lin->apply(rv, cv);
            lin_its += lin->st.iterates;
            enq_axpy(*ctx, UGPU_F64, n, 1.0, c, x, nullptr);  // x += c
            const double norm_c = norm(c, n);
            if (check_convergence(it, 1, 1, norm_c)) break;
        }
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        st.converged = st.reason > 0 ? 1 : 0;
        st.spmv_count = lin_its;  // inner iterations
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

private:
    const Mat *T_ = nullptr, *O_ = nullptr, *S_ = nullptr;
    const Vec *sel_ = nullptr, *lb_ = nullptr, *ub_ = nullptr;
    std::unique_ptr<Mat> Tt_, Ot_;
    std::unique_ptr<Mat> D_;        // diag(h): identity structure, values = the Hessian diagonal
    std::unique_ptr<Mat> Pen_, H_;  // T^T (O^T D O) T (with a transformation) and H = A + penalty
    std::unique_ptr<Mat> tmp_;      // O^T D O
    std::shared_ptr<PtapPlan> plan1_, plan2_;
    Buffer res_, rhs_, corr_, w_, gc_, gs_, t1_, t2_, shift_, ubfill_;
    int64_t shift_n_ = -1;
    Solver *user_linear_ = nullptr;
    std::unique_ptr<Solver> linear_, jacobi_;

    void invalidate() {
        D_.reset();
        Pen_.reset();
        H_.reset();
        tmp_.reset();
        plan1_.reset();
        plan2_.reset();
    }

    void spmv(const Mat &M, const double *xin, double *y, const double *b = nullptr) {
        SpmvArgs a;
        a.x = xin;
        a.y = y;
        a.v = b;
        a.vec_dtype = UGPU_F64;
        a.epilogue = b ? EPI_RESIDUAL : EPI_STORE;
        launch_spmv(*ctx, M, a);
    }

    double norm(const double *v, int64_t n) {
        DotArgs d{};
        d.a[0] = d.b[0] = v;
        d.dtype_a[0] = d.dtype_b[0] = UGPU_F64;
        d.nd = 1;
        double o = 0;
        host_dots(*ctx, n, d, &o);
        return std::sqrt(o);
    }

    // D, the Galerkin plans and H's union structure, once per operator / transformation
    void build_structures() {
        if (H_) return;
        const int64_t n = op->nrows;
        D_ = make_csr_device(*ctx, n, n, n, UGPU_F64);
        if (n) {
            k_identity_structure<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, D_->rowptr.as<int32_t>(),
                                                                                  D_->colidx.as<int32_t>());
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
        }
        enq_set(*ctx, UGPU_F64, n, 0.0, D_->vals.ptr, nullptr);
        finalize_matrix(*D_);
        const Mat *pen = D_.get();
        if (T_) {
            tmp_ = ptap_with_plan(*D_, *O_, plan1_);  // O^T D O
            Pen_ = ptap_with_plan(*tmp_, *T_, plan2_);  // T^T (O^T D O) T
            pen = Pen_.get();
        }
        // union structure of A and the penalty term
        Buffer cnt, pos;
        cnt.alloc(sizeof(int64_t) * std::max<int64_t>(n, 1));
        pos.alloc(sizeof(int64_t) * (n + 1));
        const int g = stream_grid(*ctx, n);
        int64_t nnz = 0;
        if (n) {
            k_add_count<<<g, kBlock, 0, ctx->stream>>>(n, op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(),
                                                       pen->rowptr.as<int32_t>(), pen->colidx.as<int32_t>(),
                                                       cnt.as<int64_t>());
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
            nnz = device_exclusive_scan(*ctx, cnt.as<int64_t>(), pos.as<int64_t>(), n);
        }
        UGPU_CHECK(nnz < (int64_t(1) << 31), UGPU_ERR_ARG, "ShiftedPenalty: int32 entry count exceeded");
        H_ = make_csr_device(*ctx, n, n, nnz, UGPU_F64);
        if (n) {
            k_add_structure<<<g, kBlock, 0, ctx->stream>>>(n, op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(),
                                                           pen->rowptr.as<int32_t>(), pen->colidx.as<int32_t>(),
                                                           pos.as<int64_t>(), H_->rowptr.as<int32_t>(),
                                                           H_->colidx.as<int32_t>());
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
        } else {
            UGPU_CUDA(cudaMemsetAsync(H_->rowptr.ptr, 0, sizeof(int32_t), ctx->stream));
        }
        add_values(*pen);
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        finalize_matrix(*H_);
    }

    void add_values(const Mat &pen) {
        const int64_t n = op->nrows;
        if (!n) return;
        k_add_values<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
            n, op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(), op->vals.as<double>(), pen.rowptr.as<int32_t>(),
            pen.colidx.as<int32_t>(), pen.vals.as<double>(), H_->rowptr.as<int32_t>(), H_->vals.as<double>());
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
    }

    // H = A + penalty Hessian for the current diagonal D (values only)
    void assemble_hessian() {
        const Mat *pen = D_.get();
        if (T_) {
            UGPU_CHECK(ptap_numeric(*D_, *O_, *tmp_, *plan1_, false) && ptap_numeric(*tmp_, *T_, *Pen_, *plan2_, false),
                       UGPU_ERR_STATE, "ShiftedPenalty: the transformation changed structure; set it again");
            pen = Pen_.get();
        }
        add_values(*pen);
        refresh_values(*H_);
    }
};

}  // namespace

std::unique_ptr<Solver> make_shifted_penalty(Context *c) { return std::make_unique<ShiftedPenalty>(c); }

namespace {
ShiftedPenalty *as_penalty(ugpu_solver *s) {
    auto p = dynamic_cast<ShiftedPenalty *>(s->impl.get());
    UGPU_CHECK(p, UGPU_ERR_ARG, "not a shifted-penalty QP solver");
    return p;
}
}  // namespace

}  // namespace ugpu

using namespace ugpu;

extern "C" int ugpu_penalty_set_transform(ugpu_solver *s, const ugpu_mat *T, const ugpu_mat *O) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    as_penalty(s)->set_transform(T ? &T->impl : nullptr, O ? &O->impl : nullptr);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

extern "C" int ugpu_penalty_set_selection(ugpu_solver *s, const ugpu_vec *selection) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    as_penalty(s)->set_selection(selection ? &selection->impl : nullptr);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

extern "C" int ugpu_penalty_set_scaling_matrix(ugpu_solver *s, const ugpu_mat *S) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    as_penalty(s)->set_scaling(S ? &S->impl : nullptr);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}
