// Host-side solver classes mirroring the reference's solver hierarchy.
//
//   Solver            ~ IterativeSolver / LinearSolver (utopia/solvers/linear/utopia_IterativeSolver.hpp,
//                       utopia_LinearSolver.hpp): tolerances, check_convergence, SolutionStatus
//   InvDiag           ~ InvDiagPreconditioner (utopia/solvers/preconditioners/utopia_TrivialPreconditioners.hpp)
//   Multigrid         ~ Multigrid + LinearMultiLevel + IPRTransfer + MultiLevelMask + smoothers
//   ConjugateGradient ~ ConjugateGradient (utopia/solvers/smoothers/utopia_ConjugateGradient_impl.hpp)
//   Mprgp, Pgs        ~ MPRGP, ProjectedGaussSeidel (utopia/solvers/nonlinear/constrained/quadratic_programming/)
//
// Solvers used as preconditioners expose pc_enqueue(): a stream-ordered, graph-
// capturable "z = M^{-1} r" from a zero initial guess whose kernels all test a device
// flag (`done`) and do nothing once the outer iteration has stopped.
#pragma once
#include <chrono>
#include <functional>
#include <map>
#include <string>

#include "internal.cuh"

namespace ugpu {

struct Solver {
    Context *ctx = nullptr;
    int kind = 0;
    std::map<std::string, double> prm;
    ugpu_solution_status st{};
    const Mat *op = nullptr;

    Solver(Context *c, int k) : ctx(c), kind(k) {
        // IterativeSolver defaults, utopia/solvers/linear/utopia_IterativeSolver.hpp:226-229
        prm["atol"] = 1e-9;
        prm["rtol"] = 1e-9;
        prm["stol"] = 1e-11;
        prm["max_it"] = 1000;
        prm["verbose"] = 0;
    }
    virtual ~Solver() = default;

    double get(const std::string &k) const {
        auto it = prm.find(k);
        UGPU_CHECK(it != prm.end(), UGPU_ERR_ARG, "unknown parameter: " + k);
        return it->second;
    }
    virtual void set(const std::string &k, double v) {
        UGPU_CHECK(prm.count(k), UGPU_ERR_ARG, "unknown parameter: " + k);
        prm[k] = v;
    }
    virtual void update(const Mat *A) = 0;
    virtual void apply(const Vec &b, Vec &x) = 0;
    virtual void set_preconditioner(Solver *) {
        throw Error(UGPU_ERR_UNSUPPORTED, "this solver takes no preconditioner");
    }

    // preconditioner interface
    virtual int pc_dtype() const { return UGPU_F64; }
    virtual void pc_enqueue(const void * /*r*/, void * /*z*/, const int * /*done*/) {
        throw Error(UGPU_ERR_UNSUPPORTED, "this solver cannot be used as a preconditioner");
    }
    // the outer iteration's dots of z = M^{-1} r with FP64 vectors a, b (b may be null), for a
    // preconditioner that can compute them in the kernel that writes z
    struct FinalDots {
        const double *a = nullptr, *b = nullptr;
        double *partials = nullptr, *out = nullptr;
        unsigned int *counter = nullptr;
    };
    // A preconditioner whose first step from zero is x1 = w .* r can take x1 from the kernel of its
    // caller that forms r: *w = the weights (pc_dtype(), fine-level size) and *x1 = the buffer to
    // write into, or both null when it cannot.
    virtual void pc_prescale(const void **w, void **x1) {
        *w = nullptr;
        *x1 = nullptr;
    }
    // pc_enqueue after the caller wrote x1 = w .* r (pc_prescale) for this r
    virtual void pc_enqueue_prescaled(const void *r, void *z, const int *done) { pc_enqueue(r, z, done); }
    // pc_enqueue, with out[0] = (z, a) [, out[1] = (z, b)] computed by its last kernel; returns false
    // (and computes no dot) where the preconditioner cannot do that
    virtual bool pc_enqueue_dots(const void *r, void *z, const int *done, const FinalDots & /*fd*/) {
        pc_enqueue(r, z, done);
        return false;
    }
    virtual void set_box(const Vec *, const Vec *) {
        throw Error(UGPU_ERR_UNSUPPORTED, "this solver takes no box constraints");
    }
    // Smoother::smooth with sweeps(s): s steps of the solver's iteration, no stopping test
    virtual void smooth(const Vec & /*b*/, Vec & /*x*/, int /*sweeps*/) {
        throw Error(UGPU_ERR_UNSUPPORTED, "this solver cannot be used as a smoother");
    }

    // IterativeSolver::check_convergence (utopia_IterativeSolver.hpp:148-191), host form
    bool check_convergence(int64_t it, double g, double r, double s) {
        bool conv = false;
        int reason = 0;
        if (g <= get("atol")) { reason = UGPU_CONVERGED_FNORM_ABS; conv = true; }
        if (s <= get("stol")) { reason = UGPU_CONVERGED_SNORM_RELATIVE; conv = true; }
        if (r <= get("rtol")) { reason = UGPU_CONVERGED_FNORM_RELATIVE; conv = true; }
        if (it >= int64_t(get("max_it"))) { reason = UGPU_DIVERGED_MAX_IT; conv = true; }
        if (conv) {
            st.iterates = it;
            st.gradient_norm = g;
            st.relative_gradient_norm = r;
            st.step_norm = s;
            st.reason = reason;
        }
        return conv;
    }
};

// device-flag-predicated elementwise kernels used by the solvers (solver_kernels.cu)
void enq_scale_into(Context &c, int dt, int64_t n, const void *w, const void *r, void *out, const int *done);
void enq_neg_copy(Context &c, int dt, int64_t n, const void *r, void *rr, void *p, const int *done);
void enq_axpy(Context &c, int dt, int64_t n, double alpha, const void *x, void *y, const int *done);
void enq_set(Context &c, int dt, int64_t n, double v, void *y, const int *done);
void enq_convert(Context &c, int sdt, const void *src, int ddt, void *dst, int64_t n, const int *done);
void enq_copy(Context &c, int dt, int64_t n, const void *src, void *dst, const int *done);

// A whole solve as one graph launch (loop.cu): WHILE(!*done) { body }
struct DeviceLoop {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Buffer state;          // [0] body executions, [1] cap overrun flag
    int64_t kernels = 0;   // kernels per body execution (instrumentation)
    ~DeviceLoop();
    void reset();
    bool built() const { return exec != nullptr; }
    void build(Context &ctx, const std::function<void()> &body, const int *done, int cap);
    int run(Context &ctx);
};

std::unique_ptr<Solver> make_cg(Context *c);
std::unique_ptr<Solver> make_multigrid(Context *c);
std::unique_ptr<Solver> make_invdiag(Context *c);
std::unique_ptr<Solver> make_cholesky(Context *c);
std::unique_ptr<Solver> make_mprgp(Context *c);
std::unique_ptr<Solver> make_pgs(Context *c);
std::unique_ptr<Solver> make_amg(Context *c);
std::unique_ptr<Solver> make_bicgstab(Context *c);
std::unique_ptr<Solver> make_ssnewton(Context *c);
std::unique_ptr<Solver> make_monotone_mg(Context *c);
std::unique_ptr<Solver> make_shifted_penalty(Context *c);
// the multigrid inside an algebraic multigrid solver (any other solver: itself)
const Solver *amg_multigrid(const Solver *s);

// multigrid introspection for the ABI
int mg_n_levels(const Solver *s);
std::unique_ptr<Mat> mg_level_matrix(const Solver *s, int l);
void mg_eigs(const Solver *s, int l, double *emax, double *emin);
void mg_set_transfers(Solver *s, const std::vector<const Mat *> &P);
// LinearMultiLevel::fix_semidefinite_operator: diagonal entries with |a_ii| < 1e-12 get +1
void fix_semidefinite_operator(Context &ctx, Mat &J);
// the monotone multigrid's counterparts (false / -1 / null: s is not a monotone multigrid)
bool mmg_set_transfers(Solver *s, const std::vector<const Mat *> &P);
int mmg_n_levels(const Solver *s);
std::unique_ptr<Mat> mmg_level_matrix(const Solver *s, int l);

inline double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace ugpu

struct ugpu_solver {
    std::unique_ptr<ugpu::Solver> impl;
};
