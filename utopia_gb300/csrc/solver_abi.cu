// C ABI of the solver layer and the dense coarse solver as a stand-alone solver kind.
#include <cstring>

#include "abi_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {
// Dense Cholesky as a LinearSolver (the Factorization role of the coarse level)
class CholeskySolver final : public Solver {
public:
    explicit CholeskySolver(Context *c) : Solver(c, UGPU_SOLVER_CHOLESKY) {}
    DenseCholesky chol;
    void update(const Mat *A) override {
        op = A;
        UGPU_CHECK(chol.factor(*A), UGPU_ERR_NOT_SPD, "matrix is not symmetric positive definite");
    }
    void apply(const Vec &b, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "update() first");
        UGPU_CHECK(b.n == op->nrows && x.n == op->nrows && b.dtype == x.dtype, UGPU_ERR_ARG, "size/dtype mismatch");
        UGPU_CHECK(b.data() != x.data(), UGPU_ERR_ARG, "x must not alias b");
        chol.solve(b.data(), b.dtype, x.data(), x.dtype, nullptr);
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        st = ugpu_solution_status{};
        st.converged = 1;
        st.reason = UGPU_CONVERGED_FNORM_ABS;
    }
    void pc_enqueue(const void *r, void *z, const int *done) override { chol.solve(r, UGPU_F64, z, UGPU_F64, done); }
};
}  // namespace

std::unique_ptr<Solver> make_cholesky(Context *c) { return std::make_unique<CholeskySolver>(c); }

}  // namespace ugpu

using namespace ugpu;

extern "C" {

int ugpu_solver_create(ugpu_ctx *ctx, int kind, ugpu_solver **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    auto s = std::make_unique<ugpu_solver>();
    Context *c = &ctx->impl;
    switch (kind) {
        case UGPU_SOLVER_CG: s->impl = make_cg(c); break;
        case UGPU_SOLVER_MULTIGRID: s->impl = make_multigrid(c); break;
        case UGPU_SOLVER_INVDIAG: s->impl = make_invdiag(c); break;
        case UGPU_SOLVER_MPRGP: s->impl = make_mprgp(c); break;
        case UGPU_SOLVER_PGS: s->impl = make_pgs(c); break;
        case UGPU_SOLVER_CHOLESKY: s->impl = make_cholesky(c); break;
        case UGPU_SOLVER_AMG: s->impl = make_amg(c); break;
        case UGPU_SOLVER_BICGSTAB: s->impl = make_bicgstab(c); break;
        case UGPU_SOLVER_SSNEWTON: s->impl = make_ssnewton(c); break;
        case UGPU_SOLVER_MONOTONE_MG: s->impl = make_monotone_mg(c); break;
        case UGPU_SOLVER_SHIFTED_PENALTY: s->impl = make_shifted_penalty(c); break;
        default: throw Error(UGPU_ERR_ARG, "unknown solver kind");
    }
    *out = s.release();
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_solver_destroy(ugpu_solver *s) {
    UGPU_ABI_BEGIN
    delete s;
    UGPU_ABI_END(nullptr)
}

int ugpu_solver_set(ugpu_solver *s, const char *key, double value) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(key);
    s->impl->set(key, value);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_solver_get(const ugpu_solver *s, const char *key, double *value) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(key);
    UGPU_REQUIRE(value);
    *value = s->impl->get(key);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_solver_set_preconditioner(ugpu_solver *s, ugpu_solver *prec) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    s->impl->set_preconditioner(prec ? prec->impl.get() : nullptr);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_mg_set_transfer_operators(ugpu_solver *mg, int n, const ugpu_mat *const *interpolations) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(mg);
    UGPU_CHECK(n >= 1 && interpolations, UGPU_ERR_ARG, "at least one interpolation operator");
    std::vector<const Mat *> P;
    for (int i = 0; i < n; ++i) {
        UGPU_CHECK(interpolations[i], UGPU_ERR_ARG, "null interpolation operator");
        P.push_back(&interpolations[i]->impl);
    }
    mg_set_transfers(mg->impl.get(), P);
    UGPU_ABI_END(mg ? mg->impl->ctx : nullptr)
}

int ugpu_mg_level_matrix(const ugpu_solver *mg, int l, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(mg);
    UGPU_REQUIRE(out);
    auto M = mg_level_matrix(mg->impl.get(), l);
    auto h = new ugpu_mat;
    h->impl = std::move(*M);
    *out = h;
    UGPU_ABI_END(mg ? mg->impl->ctx : nullptr)
}

int ugpu_mg_n_levels(const ugpu_solver *mg, int *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(mg);
    UGPU_REQUIRE(out);
    *out = mg_n_levels(mg->impl.get());
    UGPU_ABI_END(mg ? mg->impl->ctx : nullptr)
}

int ugpu_mg_eigs(const ugpu_solver *mg, int l, double *eig_max, double *eig_min) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(mg);
    UGPU_REQUIRE(eig_max);
    UGPU_REQUIRE(eig_min);
    mg_eigs(mg->impl.get(), l, eig_max, eig_min);
    UGPU_ABI_END(mg ? mg->impl->ctx : nullptr)
}

int ugpu_mg_vcycle(ugpu_solver *mg, const ugpu_vec *r, ugpu_vec *z) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(mg);
    UGPU_REQUIRE(r);
    UGPU_REQUIRE(z);
    auto &S = *mg->impl;
    UGPU_CHECK(S.op, UGPU_ERR_STATE, "multigrid: update() first");
    UGPU_CHECK(r->impl.n == S.op->nrows && z->impl.n == S.op->nrows, UGPU_ERR_ARG, "size mismatch");
    UGPU_CHECK(r->impl.dtype == S.pc_dtype() && z->impl.dtype == S.pc_dtype(), UGPU_ERR_ARG,
               "V-cycle vectors must have the multigrid's working dtype");
    mg_n_levels(&S);  // type check
    S.pc_enqueue(r->impl.data(), z->impl.data(), nullptr);
    UGPU_CUDA(cudaStreamSynchronize(S.ctx->stream));
    UGPU_ABI_END(mg ? mg->impl->ctx : nullptr)
}

int ugpu_solver_update(ugpu_solver *s, const ugpu_mat *A) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(A);
    s->impl->update(&A->impl);
    UGPU_CUDA(cudaStreamSynchronize(s->impl->ctx->stream));
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_solver_apply(ugpu_solver *s, const ugpu_vec *rhs, ugpu_vec *x) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(rhs);
    UGPU_REQUIRE(x);
    s->impl->apply(rhs->impl, x->impl);
    s->impl->ctx->check_kernel_flags();
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_solver_solve(ugpu_solver *s, const ugpu_mat *A, const ugpu_vec *b, ugpu_vec *x) {
    int rc = ugpu_solver_update(s, A);
    if (rc != UGPU_OK) return rc;
    return ugpu_solver_apply(s, b, x);
}

int ugpu_qp_set_box_constraints(ugpu_solver *s, const ugpu_vec *lb, const ugpu_vec *ub) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    s->impl->set_box(lb ? &lb->impl : nullptr, ub ? &ub->impl : nullptr);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

int ugpu_solver_status(const ugpu_solver *s, ugpu_solution_status *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(out);
    *out = s->impl->st;
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

}  // extern "C"
