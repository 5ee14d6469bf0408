// MonotoneMultigrid (utopia/solvers/multilevel/utopia_MonotoneMultigrid.hpp:33-377) on the GPU:
// a box-constrained QP solver whose fine level is smoothed by projected Gauss-Seidel and whose
// coarse correction runs a linear multigrid on the Galerkin operator of a truncated transfer.
//
//   update(A):  PGS set-up on A; P_t = P (the fine transfer); A_H = P_t^T A P_t with
//               fix_semidefinite_operator; the linear multigrid (or the dense coarse solver
//               when P is the only transfer) set up on A_H.
//   step:       pre_smoothing_steps PGS steps;
//               active set (ActiveSet::determine, utopia_ActiveSet.hpp:47-84):
//                   a_i = x_i <= lb_i + tol || x_i >= ub_i - tol;
//               if it changed: P_t = P with the active rows zeroed (IPTruncatedTransfer::
//                   truncate_interpolation, utopia_IPTruncatedTransfer.hpp:203-223; the
//                   structure is kept) and A_H and the multigrid below it rebuilt;
//               x += P_t MG(P_t^T (b - A x)) (coarse_space_it cycles from zero);
//               post_smoothing_steps PGS steps.
//   apply:      for it = 1 .. max_it-1: step; stop on check_convergence(it, ||P(x - g) - x||, 1,
//               ||x - x_old||) with g = A x - b (criticality_measure_inf; ||g|| when a bound
//               is missing).
//
// The fine smoother is the multicolour PGS (rows of one colour relaxed in parallel); the
// linear multigrid below the truncated level is this library's Multigrid (Jacobi,
// Chebyshev3level or PointJacobi smoothing, no masks, fix_semidefinite_operators on).
// Per iteration the host reads the number of active-set changes and the two norms.
#include <cfloat>
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {

#define MMG_LOOP(i, n) \
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

// ActiveSet::determine: the indicator and the number of entries that changed
__global__ void k_mmg_active(int64_t n, const double *__restrict__ x, const double *__restrict__ lb,
                             const double *__restrict__ ub, double tol, int32_t *__restrict__ active,
                             unsigned int *changed) {
    unsigned int cnt = 0;
    MMG_LOOP(i, n) {
        const double xi = x[i];
        const int32_t a = (xi <= lb[i] + tol || xi >= ub[i] - tol) ? 1 : 0;
        cnt += (a != active[i]);
        active[i] = a;
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(changed, cnt);
}

// truncate_interpolation: the rows of active fine dofs zeroed, every other value copied
__global__ void k_mmg_truncate(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ active,
                               const double *__restrict__ src, double *__restrict__ dst) {
    MMG_LOOP(i, n) {
        const bool a = active[i] != 0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) dst[k] = a ? 0.0 : src[k];
    }
}

// help = P(x + r) - x (r = b - A x = -g) and dx = x - x_old
__global__ void k_mmg_measure(int64_t n, const double *__restrict__ x, const double *__restrict__ r,
                              const double *__restrict__ lb, const double *__restrict__ ub,
                              const double *__restrict__ xold, double *__restrict__ help, double *__restrict__ dx) {
    MMG_LOOP(i, n) {
        const double xi = x[i];
        const double y = xi + r[i];
        help[i] = ((lb[i] >= y) ? lb[i] : ((ub[i] <= y) ? ub[i] : y)) - xi;
        dx[i] = xi - xold[i];
    }
}

}  // namespace

class MonotoneMultigrid final : public Solver {
public:
    explicit MonotoneMultigrid(Context *c) : Solver(c, UGPU_SOLVER_MONOTONE_MG) {
        prm["pre_smoothing_steps"] = 3;   // utopia_MultiLevelBase.hpp:35-42
        prm["post_smoothing_steps"] = 3;
        prm["n_local_sweeps"] = 3;        // ProjectedGaussSeidel(): n_local_sweeps_(3)
        prm["use_symmetric_sweep"] = 1;
        prm["smoother"] = 1;              // linear multigrid: 0 Jacobi, 1 Chebyshev3level, 2 PointJacobi
        prm["omega"] = 1.0;
        prm["active_set_tol"] = 0;        // ActiveSet: tol_{0}
        prm["coarse_space_it"] = 1;       // coarse_space_it_{1}
        prm["use_coarse_space"] = 1;      // use_coarse_space_{true}
        prm["galerkin_assemblies"] = 0;   // read-only: truncated Galerkin assemblies of the last apply()
        prm["n_active"] = 0;              // read-only: size of the active set after the last apply()
    }

    void set_box(const Vec *lb, const Vec *ub) override {
        for (const Vec *v : {lb, ub})
            UGPU_CHECK(!v || v->dtype == UGPU_F64, UGPU_ERR_ARG, "box constraints must be FP64 vectors");
        lb_ = lb;
        ub_ = ub;
        if (pgs_) pgs_->set_box(lb, ub);
    }

    // set_transfer_operators: interpolations coarse -> fine; the last one is the fine-level
    // transfer that gets truncated, the others go to the linear multigrid
    void set_transfers(const std::vector<const Mat *> &P) {
        UGPU_CHECK(!P.empty(), UGPU_ERR_ARG, "MonotoneMultigrid: at least one transfer operator");
        std::vector<std::unique_ptr<Mat>> copy;
        for (auto *p : P) {
            UGPU_CHECK(p && p->vdtype == UGPU_F64, UGPU_ERR_ARG, "transfer operators must be FP64 matrices");
            copy.push_back(cast_matrix(*p, UGPU_F64));
        }
        for (size_t i = 1; i < copy.size(); ++i)
            UGPU_CHECK(copy[i]->ncols == copy[i - 1]->nrows, UGPU_ERR_ARG,
                       "interpolation operators do not chain (coarse -> fine order)");
        P_ = std::move(copy);
        mg_.reset();
        ready_ = false;
    }

    int n_levels() const { return mg_ ? mg_n_levels(mg_.get()) + 1 : 2; }

    std::unique_ptr<Mat> level_matrix(int l) const {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "MonotoneMultigrid: update() first");
        const int L = n_levels();
        UGPU_CHECK(l >= 0 && l < L, UGPU_ERR_ARG, "level out of range");
        if (l == L - 1) return cast_matrix(*op, UGPU_F64);
        if (l == L - 2) return cast_matrix(*AH_, UGPU_F64);
        return mg_level_matrix(mg_.get(), l);
    }

    std::vector<int32_t> active_set() const {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "MonotoneMultigrid: update() first");
        std::vector<int32_t> h(size_t(op->nrows));
        if (op->nrows)
            UGPU_CUDA(cudaMemcpy(h.data(), active_.ptr, sizeof(int32_t) * op->nrows, cudaMemcpyDeviceToHost));
        return h;
    }

    // MonotoneMultigrid::update (:135-154) with init_memory and galerkin_assembly
    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG,
                   "MonotoneMultigrid: square FP64 operator");
        UGPU_CHECK(!P_.empty(), UGPU_ERR_STATE, "MonotoneMultigrid: set the transfer operators first");
        const Mat &I = *P_.back();
        UGPU_CHECK(I.nrows == A->nrows, UGPU_ERR_ARG, "fine transfer rows do not match the operator");
        op = A;
        const int64_t n = A->nrows, nc = I.ncols;
        if (!pgs_) pgs_ = make_pgs(ctx);
        pgs_->set("n_local_sweeps", get("n_local_sweeps"));
        pgs_->set("use_symmetric_sweep", get("use_symmetric_sweep"));
        pgs_->set_box(lb_, ub_);
        pgs_->update(A);
        active_.alloc(sizeof(int32_t) * std::max<int64_t>(n, 1));
        UGPU_CUDA(cudaMemsetAsync(active_.ptr, 0, active_.bytes, ctx->stream));
        cnt_.alloc(sizeof(unsigned int));
        for (Buffer *b : {&r_, &help_, &dx_, &xold_, &corr_}) b->alloc(sizeof(double) * std::max<int64_t>(n, 1));
        for (Vec *v : {&rc_, &cc_}) {
            v->ctx = ctx;
            v->n = nc;
            v->dtype = UGPU_F64;
            v->buf.alloc(sizeof(double) * std::max<int64_t>(nc, 1));
        }
        It_ = cast_matrix(I, UGPU_F64);  // no truncation until the active set first changes
        AH_.reset();
        Rt_.reset();
        galerkin();
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        ready_ = true;
    }

    void apply(const Vec &b, Vec &x) override;

private:
    std::vector<std::unique_ptr<Mat>> P_;  // interpolations coarse -> fine (deep copies)
    std::unique_ptr<Mat> It_, Rt_, AH_;   // truncated fine transfer, its transpose, the Galerkin operator
    std::unique_ptr<Solver> pgs_, mg_;
    DenseCholesky chol_;                   // coarse solve when the fine transfer is the only one
    const Vec *lb_ = nullptr, *ub_ = nullptr;
    Buffer lbfill_, ubfill_, active_, cnt_, r_, help_, dx_, xold_, corr_, rt_perm_;
    Vec rc_, cc_;
    bool ready_ = false;
    int64_t assemblies_ = 0;

    // galerkin_assembly (:212-227): A_H = P_t^T A P_t, fix_semidefinite_operator, then the
    // linear multigrid (which assembles the levels below with the same fix) or the direct
    // solver.  Truncation only changes values, so after the first assembly every product
    // (A_H, the levels below it, P_t^T) is recomputed in place on its kept structure.
    void galerkin() {
        const bool numeric = AH_ && AH_->ptap_plan && ptap_numeric(*op, *It_, *AH_, *AH_->ptap_plan, false);
        std::unique_ptr<Mat> fresh;
        if (!numeric) {
            std::shared_ptr<PtapPlan> plan;
            fresh = ptap_with_plan(*op, *It_, plan);
            fresh->ptap_plan = std::move(plan);
        }
        Mat &AH = numeric ? *AH_ : *fresh;
        fix_semidefinite_operator(*ctx, AH);
        if (P_.size() == 1) {
            UGPU_CHECK(chol_.factor(AH), UGPU_ERR_NOT_SPD, "MonotoneMultigrid: coarse operator is not SPD");
        } else {
            if (!mg_) {
                mg_ = make_multigrid(ctx);
                std::vector<const Mat *> rest;
                for (size_t i = 0; i + 1 < P_.size(); ++i) rest.push_back(P_[i].get());
                mg_set_transfers(mg_.get(), rest);
            }
            for (const char *k : {"pre_smoothing_steps", "post_smoothing_steps", "smoother", "omega"})
                mg_->set(k, get(k));
            mg_->set("fix_semidefinite_operators", 1);  // MonotoneMultigrid(): algo_.fix_semidefinite_operators(true)
            mg_->set("must_generate_masks", 0);         // algo_.must_generate_masks(false)
            mg_->set("keep_galerkin_structure", 1);
            mg_->update(&AH);
        }
        if (!numeric) AH_ = std::move(fresh);  // the multigrid keeps a pointer to this operator
        // P_t^T: values gathered from P_t through the transpose's entry permutation
        if (Rt_ && Rt_->nnz == It_->nnz) {
            gather_values(*ctx, It_->nnz, It_->vals.as<double>(), rt_perm_.as<int64_t>(), Rt_->vals.as<double>());
            refresh_values(*Rt_);
        } else {
            Rt_ = transpose_with_perm(*It_, rt_perm_, true);
        }
        ++assemblies_;
    }

    void bounds(int64_t n, const double **lb, const double **ub) {
        UGPU_CHECK(!lb_ || lb_->n == n, UGPU_ERR_ARG, "lower bound size mismatch");
        UGPU_CHECK(!ub_ || ub_->n == n, UGPU_ERR_ARG, "upper bound size mismatch");
        if (!lb_) {
            lbfill_.alloc(sizeof(double) * std::max<int64_t>(n, 1));
            enq_set(*ctx, UGPU_F64, n, -DBL_MAX, lbfill_.ptr, nullptr);
        }
        if (!ub_) {
            ubfill_.alloc(sizeof(double) * std::max<int64_t>(n, 1));
            enq_set(*ctx, UGPU_F64, n, DBL_MAX, ubfill_.ptr, nullptr);
        }
        *lb = lb_ ? lb_->as<double>() : lbfill_.as<double>();
        *ub = ub_ ? ub_->as<double>() : ubfill_.as<double>();
    }

    void step(const Vec &b, Vec &x, const double *lb, const double *ub);
    void measure(const Vec &b, const Vec &x, const double *lb, const double *ub, double *g_norm, double *x_diff);
};

// r = b - A x; ||P(x - g) - x|| (||g|| without both bounds) and ||x - x_old||
void MonotoneMultigrid::measure(const Vec &b, const Vec &x, const double *lb, const double *ub, double *g_norm,
                                double *x_diff) {
    const int64_t n = op->nrows;
    SpmvArgs a;
    a.x = x.data();
    a.v = b.data();
    a.y = r_.ptr;
    a.vec_dtype = UGPU_F64;
    a.epilogue = EPI_RESIDUAL;
    launch_spmv(*ctx, *op, a);
    k_mmg_measure<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, x.as<double>(), r_.as<double>(), lb, ub,
                                                                     xold_.as<double>(), help_.as<double>(),
                                                                     dx_.as<double>());
    ctx->launches++;
    DotArgs d{};
    d.nd = 2;
    d.a[0] = d.b[0] = (lb_ && ub_) ? help_.as<double>() : r_.as<double>();
    d.a[1] = d.b[1] = dx_.as<double>();
    d.dtype_a[0] = d.dtype_b[0] = d.dtype_a[1] = d.dtype_b[1] = UGPU_F64;
    double out[2];
    host_dots(*ctx, n, d, out);
    *g_norm = std::sqrt(out[0]);
    *x_diff = std::sqrt(out[1]);
}

// MonotoneMultigrid::step (:238-319)
void MonotoneMultigrid::step(const Vec &b, Vec &x, const double *lb, const double *ub) {
    const int64_t n = op->nrows, nc = rc_.n;
    pgs_->smooth(b, x, int(get("pre_smoothing_steps")));
    if (get("use_coarse_space") != 0) {
        UGPU_CUDA(cudaMemsetAsync(cnt_.ptr, 0, sizeof(unsigned int), ctx->stream));
        k_mmg_active<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
            n, x.as<double>(), lb, ub, get("active_set_tol"), active_.as<int32_t>(), cnt_.as<unsigned int>());
        ctx->launches++;
        unsigned int changed = 0;
        UGPU_CUDA(cudaMemcpyAsync(&changed, cnt_.ptr, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        if (changed) {
            const Mat &I = *P_.back();
            k_mmg_truncate<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
                n, I.rowptr.as<int32_t>(), active_.as<int32_t>(), I.vals.as<double>(), It_->vals.as<double>());
            ctx->launches++;
            refresh_values(*It_);
            galerkin();
        }
        // r = b - A x; r_H = P_t^T r
        SpmvArgs a;
        a.x = x.data();
        a.v = b.data();
        a.y = r_.ptr;
        a.vec_dtype = UGPU_F64;
        a.epilogue = EPI_RESIDUAL;
        launch_spmv(*ctx, *op, a);
        SpmvArgs rs;
        rs.x = r_.ptr;
        rs.y = rc_.data();
        rs.vec_dtype = UGPU_F64;
        rs.epilogue = EPI_STORE;
        launch_spmv(*ctx, *Rt_, rs);
        // coarse_space_step (:229-236) from c_H = 0
        const int csi = int(get("coarse_space_it"));
        if (!mg_) {
            chol_.solve(rc_.data(), UGPU_F64, cc_.data(), UGPU_F64, nullptr);
        } else if (csi == 1) {
            mg_->pc_enqueue(rc_.data(), cc_.data(), nullptr);  // one cycle from zero
        } else {
            enq_set(*ctx, UGPU_F64, nc, 0.0, cc_.data(), nullptr);
            mg_->set("max_it", csi);
            mg_->apply(rc_, cc_);
        }
        // x += P_t c_H
        SpmvArgs ip;
        ip.x = cc_.data();
        ip.y = corr_.ptr;
        ip.vec_dtype = UGPU_F64;
        ip.epilogue = EPI_STORE;
        launch_spmv(*ctx, *It_, ip);
        enq_axpy(*ctx, UGPU_F64, n, 1.0, corr_.ptr, x.data(), nullptr);
    }
    pgs_->smooth(b, x, int(get("post_smoothing_steps")));
}

// MonotoneMultigrid::apply (:158-202)
void MonotoneMultigrid::apply(const Vec &b, Vec &x) {
    UGPU_CHECK(ready_, UGPU_ERR_STATE, "MonotoneMultigrid: update() first");
    const int64_t n = op->nrows;
    UGPU_CHECK(b.n == n && x.n == n && b.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG,
               "MonotoneMultigrid: FP64 vectors of the operator size");
    const double t0 = now_s();
    const int64_t l0 = ctx->launches;
    st = ugpu_solution_status{};
    assemblies_ = 0;
    const double *lb, *ub;
    bounds(n, &lb, &ub);
    enq_copy(*ctx, UGPU_F64, n, x.data(), xold_.ptr, nullptr);
    double g_norm = 0, x_diff = 0;
    measure(b, x, lb, ub, &g_norm, &x_diff);
    const int64_t max_it = int64_t(get("max_it"));
    bool converged = false;
    for (int64_t it = 1; it < max_it && !converged; ++it) {
        step(b, x, lb, ub);
        measure(b, x, lb, ub, &g_norm, &x_diff);
        converged = check_convergence(it, g_norm, 1, x_diff);
        if (!converged) enq_copy(*ctx, UGPU_F64, n, x.data(), xold_.ptr, nullptr);
    }
    UGPU_LAUNCH_CHECK();
    UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!converged) {  // the loop ran out at it == max_it without a test that says so
        st.iterates = std::max<int64_t>(max_it - 1, 0);
        st.gradient_norm = g_norm;
        st.relative_gradient_norm = 1;
        st.step_norm = x_diff;
        st.reason = UGPU_DIVERGED_MAX_IT;
    }
    st.converged = st.reason > 0 ? 1 : 0;
    st.execution_time = now_s() - t0;
    st.kernel_launches = ctx->launches - l0;
    prm["galerkin_assemblies"] = double(assemblies_);
    int64_t na = 0;
    for (int32_t v : active_set()) na += v;
    prm["n_active"] = double(na);
}

std::unique_ptr<Solver> make_monotone_mg(Context *c) { return std::make_unique<MonotoneMultigrid>(c); }

bool mmg_set_transfers(Solver *s, const std::vector<const Mat *> &P) {
    auto m = dynamic_cast<MonotoneMultigrid *>(s);
    if (!m) return false;
    m->set_transfers(P);
    return true;
}

int mmg_n_levels(const Solver *s) {
    auto m = dynamic_cast<const MonotoneMultigrid *>(s);
    return m ? m->n_levels() : -1;
}

std::unique_ptr<Mat> mmg_level_matrix(const Solver *s, int l) {
    auto m = dynamic_cast<const MonotoneMultigrid *>(s);
    return m ? m->level_matrix(l) : nullptr;
}

}  // namespace ugpu

using namespace ugpu;

extern "C" {

int ugpu_mmg_active_set(const ugpu_solver *s, int32_t *indicator, int64_t *n_active) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    auto m = dynamic_cast<const MonotoneMultigrid *>(s->impl.get());
    UGPU_CHECK(m, UGPU_ERR_ARG, "not a monotone multigrid solver");
    auto h = m->active_set();
    int64_t na = 0;
    for (int32_t v : h) na += v;
    if (indicator && !h.empty()) std::copy(h.begin(), h.end(), indicator);
    if (n_active) *n_active = na;
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

}  // extern "C"
