// The reference's own solver templates instantiated over the CPU backend of
// utopia_ref_backend.hpp -- TEST INFRASTRUCTURE ONLY (the oracle's pin).
//
// Compiled from the reference checkout's headers, unchanged, by oracle/__init__.py
// (build_ref) into oracle/_ref/libutopia_ref.so, with a C API that mirrors the restated
// oracle's (liboracle.so) so that the tests can run both on the same inputs:
//   ConjugateGradient (utopia/solvers/smoothers/utopia_ConjugateGradient_impl.hpp:90-294)
//   InvDiagPreconditioner (utopia/solvers/preconditioners/utopia_TrivialPreconditioners.hpp:20-56)
//   Multigrid + IPRTransfer + MultiLevelMask + Galerkin assembly
//     (utopia/solvers/multilevel/utopia_Multigrid.hpp:162-367, utopia_LinearMultiLevel.hpp:201-226)
//   Chebyshev3level + PowerMethod, Jacobi, PointJacobi (utopia/solvers/smoothers/, eigensolvers/)
//   MPRGP (utopia/solvers/nonlinear/constrained/quadratic_programming/utopia_MPRGP.hpp:57-387)
//   ProjectedGaussSeidel (.../utopia_ProjectedGaussSeidel.hpp:71-112,197-318)
//   ShiftedPenaltyQPSolver + ShiftedPenalty (utopia/solvers/nonlinear/constrained/penalty/), with
//     the qp_solve app's transformation (utopia/apps/qp_solve/utopia_qp_solve.cpp:68-88)
// The coarse-level direct solver is a dense Cholesky (the reference's tests pass PETSc's
// Factorization there), with the restated oracle's arithmetic order.
#include "utopia_ref_backend.hpp"

#include "utopia_Chebyshev3level.hpp"
#include "utopia_ConjugateGradient.hpp"
#include "utopia_ConjugateGradient_impl.hpp"
#include "utopia_IPRTransfer.hpp"
#include "utopia_Jacobi.hpp"
#include "utopia_MPRGP.hpp"
#include "utopia_Multigrid.hpp"
#include "utopia_PointJacobi.hpp"
#include "utopia_ProjectedGaussSeidel.hpp"
#include "utopia_TrivialPreconditioners.hpp"
#include "utopia_ShiftedPenaltyQPSolver_impl.hpp"
#include "utopia_TransformedBoxConstraints.hpp"
#include "utopia_InputParameters.hpp"

#include <cstdint>
#include <cstdlib>


using namespace utopia;

namespace {

using MG = Multigrid<RefMatrix, RefVector>;

struct MgHandle {
    std::shared_ptr<RefMatrix> A;
    std::vector<std::shared_ptr<RefMatrix>> P;
    std::shared_ptr<MG> mg;
};

RefVector make_vec(int64_t n, const double *v) {
    RefVector x(RefTraits::Layout(SelfCommunicator(), n, n), 0.0);
    if (v) std::copy(v, v + n, x.data().begin());
    return x;
}

// ConjugateGradient whose absolute tolerance is rel * ||b|| of each system it solves (a
// LinearSolver that forwards to the reference's CG, which is final)
class RelTolCG final : public LinearSolver<RefMatrix, RefVector> {
public:
    std::shared_ptr<ConjugateGradient<RefMatrix, RefVector>> cg = std::make_shared<ConjugateGradient<RefMatrix, RefVector>>();
    double rel = 1e-12;
    void update(const std::shared_ptr<const RefMatrix> &op) override {
        LinearSolver<RefMatrix, RefVector>::update(op);
        cg->update(op);
    }
    bool apply(const RefVector &b, RefVector &x) override {
        cg->atol(rel * norm2(b));
        return cg->apply(b, x);
    }
    RelTolCG *clone() const override { return new RelTolCG(*this); }
};

}  // namespace

extern "C" {

struct ref_status {
    int64_t iterates;
    double gradient_norm;
    double relative_gradient_norm;
    double step_norm;
    int32_t reason;
    int32_t converged;
    int64_t spmv_count;
};

static void fill_status(const SolutionStatus &s, bool converged, ref_status *st) {
    st->iterates = s.iterates;
    st->gradient_norm = s.gradient_norm;
    st->relative_gradient_norm = s.relative_gradient_norm;
    st->step_norm = s.step_norm;
    st->reason = s.reason;
    st->converged = converged ? 1 : 0;
    st->spmv_count = 0;
}

void *ref_csr_create(int64_t n, int64_t m, const int32_t *rp, const int32_t *ci, const double *v) {
    auto *A = new RefMatrix();
    A->from_csr(n, m, rp, ci, v);
    return A;
}
void ref_csr_free(void *h) { delete static_cast<RefMatrix *>(h); }
int64_t ref_csr_nnz(const void *h) { return static_cast<const RefMatrix *>(h)->nnz(); }
int64_t ref_csr_rows(const void *h) { return static_cast<const RefMatrix *>(h)->nrows; }
void ref_csr_arrays(const void *h, int32_t *rp, int32_t *ci, double *v) {
    const RefMatrix &A = *static_cast<const RefMatrix *>(h);
    std::copy(A.rowptr.begin(), A.rowptr.end(), rp);
    std::copy(A.colidx.begin(), A.colidx.end(), ci);
    std::copy(A.vals.begin(), A.vals.end(), v);
}

// smoother: 0 Jacobi, 1 Chebyshev3level, 2 PointJacobi.  The rand() stream used by
// PowerMethod's start vectors is reseeded with 1 (a fresh process) at every set-up.
void *ref_mg_create(const void *hA, int nP, const void *const *hP, int smoother, int pre, int post,
                    int fix_semidefinite) {
    try {
        auto *h = new MgHandle();
        h->A = std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hA));
        for (int k = 0; k < nP; ++k) h->P.push_back(std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hP[k])));
        std::shared_ptr<IterativeSolver<RefMatrix, RefVector>> sm;
        if (smoother == 0)
            sm = std::make_shared<Jacobi<RefMatrix, RefVector>>();
        else if (smoother == 1)
            sm = std::make_shared<Chebyshev3level<RefMatrix, RefVector>>();
        else
            sm = std::make_shared<PointJacobi<RefMatrix, RefVector>>();
        h->mg = std::make_shared<MG>(sm, std::make_shared<RefCholesky>());
        h->mg->set_transfer_operators(h->P);
        h->mg->pre_smoothing_steps(pre);
        h->mg->post_smoothing_steps(post);
        h->mg->fix_semidefinite_operators(fix_semidefinite != 0);
        h->mg->must_generate_masks(true);
        h->mg->max_it(1);
        h->mg->mg_type(1);
        std::srand(1);
        h->mg->update(h->A);
        return h;
    } catch (...) {
        return nullptr;
    }
}
void ref_mg_free(void *h) { delete static_cast<MgHandle *>(h); }
int ref_mg_levels(const void *h) { return int(static_cast<const MgHandle *>(h)->mg->n_levels()); }
const void *ref_mg_level_matrix(void *h, int l) { return &static_cast<MgHandle *>(h)->mg->level(l).A(); }

// Multigrid::apply as a stand-alone solver
int ref_mg_solve(void *h, const double *rhs, double *x, double atol, double rtol, int64_t max_it, ref_status *st) {
    try {
        auto &m = *static_cast<MgHandle *>(h);
        const int64_t n = m.A->nrows;
        RefVector b = make_vec(n, rhs), xv = make_vec(n, x);
        m.mg->atol(atol);
        m.mg->rtol(rtol);
        m.mg->max_it(max_it);
        m.mg->apply(b, xv);
        std::copy(xv.data().begin(), xv.data().end(), x);
        const auto &s = m.mg->solution_status();
        fill_status(s, s.reason > 0, st);
        m.mg->max_it(1);
        return 0;
    } catch (...) {
        return -1;
    }
}

// precond: 0 none, 1 InvDiagPreconditioner, 2 the multigrid handle (as preconditioner)
int ref_cg_solve(const void *hA, const double *b, double *x, int precond, void *hmg, double atol, double rtol,
                 double stol, int64_t max_it, ref_status *st) {
    try {
        // with the multigrid preconditioner, the operator is the one the hierarchy keeps (the
        // solver stores a non-owning reference to the operator it is updated with)
        auto A = precond == 2 ? static_cast<MgHandle *>(hmg)->A
                              : std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hA));
        const int64_t n = A->nrows;
        RefVector bv = make_vec(n, b), xv = make_vec(n, x);
        ConjugateGradient<RefMatrix, RefVector> cg;
        cg.atol(atol);
        cg.rtol(rtol);
        cg.stol(stol);
        cg.max_it(max_it);
        if (precond == 1) cg.set_preconditioner(std::make_shared<InvDiagPreconditioner<RefMatrix, RefVector>>());
        if (precond == 2) {
            auto &m = *static_cast<MgHandle *>(hmg);
            m.mg->max_it(1);
            cg.set_preconditioner(m.mg);
            // CG's update() refreshes its preconditioner; the hierarchy is rebuilt with the
            // same rand() stream as at creation
            std::srand(1);
        }
        const bool ok = cg.solve(*A, bv, xv);
        std::copy(xv.data().begin(), xv.data().end(), x);
        fill_status(cg.solution_status(), ok, st);
        return 0;
    } catch (...) {
        return -1;
    }
}

// MPRGP with lower/upper bounds (nullptr: unbounded on that side)
int ref_mprgp_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x, double atol,
                    double rtol, int64_t max_it, ref_status *st) {
    try {
        auto A = std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hA));
        const int64_t n = A->nrows;
        RefVector bv = make_vec(n, b), xv = make_vec(n, x);
        MPRGP<RefMatrix, RefVector> qp;
        qp.atol(atol);
        qp.rtol(rtol);
        qp.max_it(max_it);
        auto l = std::make_shared<RefVector>(make_vec(n, lb));
        auto u = std::make_shared<RefVector>(make_vec(n, ub));
        qp.set_box_constraints(BoxConstraints<RefVector>(lb ? l : nullptr, ub ? u : nullptr));
        const bool ok = qp.solve(*A, bv, xv);
        std::copy(xv.data().begin(), xv.data().end(), x);
        fill_status(qp.solution_status(), ok, st);
        return 0;
    } catch (...) {
        return -1;
    }
}

// ProjectedGaussSeidel (lexicographic, n_local_sweeps, symmetric), stop on ||x - x_old|| <= stol
int ref_pgs_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x, double stol,
                  int64_t max_it, int n_local_sweeps, int symmetric, ref_status *st) {
    try {
        auto A = std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hA));
        const int64_t n = A->nrows;
        RefVector bv = make_vec(n, b), xv = make_vec(n, x);
        ProjectedGaussSeidel<RefMatrix, RefVector> pgs;
        pgs.stol(stol);
        pgs.max_it(max_it);
        pgs.n_local_sweeps(n_local_sweeps);
        pgs.use_symmetric_sweep(symmetric != 0);
        auto l = std::make_shared<RefVector>(make_vec(n, lb));
        auto u = std::make_shared<RefVector>(make_vec(n, ub));
        pgs.set_box_constraints(BoxConstraints<RefVector>(lb ? l : nullptr, ub ? u : nullptr));
        const bool ok = pgs.solve(*A, bv, xv);
        std::copy(xv.data().begin(), xv.data().end(), x);
        fill_status(pgs.solution_status(), ok, st);
        return 0;
    } catch (...) {
        return -1;
    }
}

// ShiftedPenaltyQPSolver with the upper bound (else the lower bound) as its constraint.  Inner
// solves: the reference's ConjugateGradient + InvDiagPreconditioner stopped at
// linear_rtol * ||rhs|| of each system (the rule the restated oracle and the GPU solver use).
// T/O: the transformation (both or neither), S: a scaling matrix, selection: a 0/1 vector (any
// may be null).  n_solves consecutive solves by the same solver object, each from the previous
// x (the shift carries over unless zero_shift_on_reset); the status is the last one's.
int ref_penalty_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x,
                      const double *selection, const void *hT, const void *hO, const void *hS, double penalty,
                      double penalty_max, double factor, int zero_shift, int n_solves, double stol, int64_t max_it,
                      double linear_rtol, int64_t linear_max_it, ref_status *st) {
    try {
        auto A = std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hA));
        const int64_t n = A->nrows;
        RefVector bv = make_vec(n, b), xv = make_vec(n, x);
        auto lin = std::make_shared<RelTolCG>();
        lin->rel = linear_rtol;
        lin->cg->max_it(linear_max_it);
        lin->cg->set_preconditioner(std::make_shared<InvDiagPreconditioner<RefMatrix, RefVector>>());
        ShiftedPenaltyQPSolver<RefMatrix, RefVector> qp(lin);
        auto params = param_list(param("penalty_parameter", penalty), param("penalty_parameter_max", penalty_max),
                                 param("penalty_parameter_factor", factor),
                                 param("zero_shift_on_reset", zero_shift != 0));
        qp.read(params);
        qp.stol(stol);
        qp.max_it(max_it);
        auto l = std::make_shared<RefVector>(make_vec(n, lb));
        auto u = std::make_shared<RefVector>(make_vec(n, ub));
        qp.set_box_constraints(BoxConstraints<RefVector>(lb ? l : nullptr, ub ? u : nullptr));
        if (selection) qp.set_selection(std::make_shared<RefVector>(make_vec(n, selection)));
        if (hS) qp.set_scaling_matrix(std::make_shared<RefMatrix>(*static_cast<const RefMatrix *>(hS)));
        RefMatrix T, O;
        if (hT && hO) {
            T = *static_cast<const RefMatrix *>(hT);
            O = *static_cast<const RefMatrix *>(hO);
            auto tr = std::make_shared<PrototypeTransformation<RefMatrix, RefVector>>();
            tr->fun_transform_position = [&](const RefVector &in, RefVector &out) {
                RefVector t = T * in;
                out = transpose(O) * t;
            };
            tr->fun_inverse_transform_direction = [&](const RefVector &in, RefVector &out) {
                RefVector t = O * in;
                out = transpose(T) * t;
            };
            tr->fun_transform_matrix = [&](const RefMatrix &D, RefMatrix &out) {
                RefMatrix t = transpose(O) * D * O;
                out = transpose(T) * t * T;
            };
            qp.set_transform(tr);
        }
        bool ok = false;
        for (int k = 0; k < n_solves; ++k) ok = qp.solve(*A, bv, xv);
        std::copy(xv.data().begin(), xv.data().end(), x);
        fill_status(qp.solution_status(), ok, st);
        return 0;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
