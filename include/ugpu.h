/* ugpu.h -- C ABI of the GB300 (sm_103a) backend for utopia's sparse-solver hot path.
 *
 * Every entry point returns an int status: UGPU_OK (0) on success, a negative
 * UGPU_ERR_* code otherwise; ugpu_last_error(ctx) gives the message.  No C++
 * exception crosses this boundary.  Handles own their device memory unless they
 * were created by a *_wrap_* call (borrowed memory is never freed).  All work is
 * issued on the context's stream; calls that return host scalars synchronise.
 * One context per host thread (the reference's solvers are single-threaded host
 * code; MPI ranks map to separate processes).
 *
 * Each declaration names the reference interface it replaces (paths relative to
 * the utopia repository).
 */
#ifndef UGPU_H
#define UGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define UGPU_API __attribute__((visibility("default")))
#else
#define UGPU_API
#endif

/* status codes */
#define UGPU_OK 0
#define UGPU_ERR_CUDA (-1)
#define UGPU_ERR_ARG (-2)
#define UGPU_ERR_ALLOC (-3)
#define UGPU_ERR_NOT_SPD (-4)
#define UGPU_ERR_STATE (-5)
#define UGPU_ERR_UNSUPPORTED (-6)
#define UGPU_ERR_INTERNAL (-7)

/* element types */
#define UGPU_F64 0
#define UGPU_F32 1
#define UGPU_BF16 2

/* matrix layouts used by the SpMV family */
#define UGPU_FORMAT_CSR 0
#define UGPU_FORMAT_SELL 1

/* pointwise ops */
#define UGPU_EMUL 0 /* out = a .* b */
#define UGPU_EDIV 1 /* out = a ./ b */
#define UGPU_EMIN 2
#define UGPU_EMAX 3

/* vector reductions (ugpu_vec_reduce) */
#define UGPU_RED_SUM 0  /* sum_i v_i       (Reducible::reduce(Plus)) */
#define UGPU_RED_MIN 1  /* min_i v_i       (Reducible::reduce(Min)) */
#define UGPU_RED_MAX 2  /* max_i v_i       (Reducible::reduce(Max)) */
#define UGPU_RED_ASUM 3 /* sum_i |v_i|     (Normed::norm1) */
#define UGPU_RED_AMAX 4 /* max_i |v_i|     (Normed::norm_infty) */

/* element-wise transforms (ugpu_vec_transform) */
#define UGPU_TR_SQRT 0
#define UGPU_TR_POW2 1
#define UGPU_TR_LOG 2
#define UGPU_TR_EXP 3
#define UGPU_TR_COS 4
#define UGPU_TR_SIN 5
#define UGPU_TR_ABS 6
#define UGPU_TR_MINUS 7
#define UGPU_TR_POW 8        /* v^param */
#define UGPU_TR_RECIPROCAL 9 /* param / v */
#define UGPU_TR_SHIFT 10     /* v + param */
#define UGPU_TR_SCALE 11     /* v * param */

/* index sets of a box-constrained iterate (ugpu_active_set_compact) */
#define UGPU_SET_ACTIVE 0 /* |l_i - x_i| < 1e-14 or |u_i - x_i| < 1e-14 (MPRGP::get_beta's chopped set) */
#define UGPU_SET_FREE 1   /* l_i < x_i < u_i                            (MPRGP::get_fi's free set) */

/* solver kinds */
#define UGPU_SOLVER_CG 1          /* utopia::ConjugateGradient */
#define UGPU_SOLVER_MULTIGRID 2   /* utopia::Multigrid */
#define UGPU_SOLVER_INVDIAG 3     /* utopia::InvDiagPreconditioner */
#define UGPU_SOLVER_MPRGP 4       /* utopia::MPRGP */
#define UGPU_SOLVER_PGS 5         /* utopia::ProjectedGaussSeidel */
#define UGPU_SOLVER_CHOLESKY 6    /* dense coarse-level direct solver (utopia::Factorization) */
#define UGPU_SOLVER_AMG 7         /* utopia::AlgebraicMultigrid with utopia::Agglomerate */
#define UGPU_SOLVER_BICGSTAB 8    /* utopia::BiCGStab (utopia/solvers/smoothers/utopia_BiCGStab_impl.hpp:44-250); an
                                   * FP64 preconditioner is applied from a zero initial guess */
#define UGPU_SOLVER_SSNEWTON 9    /* utopia::SemismoothNewton (quadratic_programming/utopia_SemismoothNewton_impl.hpp:
                                   * 74-207); box constraints by ugpu_qp_set_box_constraints; the inner linear solver
                                   * is BiCGStab + Jacobi to linear_rtol * ||residual|| unless one is set through
                                   * ugpu_solver_set_preconditioner */
#define UGPU_SOLVER_MONOTONE_MG 10 /* utopia::MonotoneMultigrid (utopia/solvers/multilevel/utopia_MonotoneMultigrid.hpp:
                                   * 33-377): box constraints by ugpu_qp_set_box_constraints, interpolations by
                                   * ugpu_mg_set_transfer_operators (coarse -> fine; the last one is the fine-level
                                   * transfer truncated on the active set) */

#define UGPU_SOLVER_SHIFTED_PENALTY 11 /* utopia::ShiftedPenaltyQPSolver (penalty/utopia_ShiftedPenaltyQPSolver_impl.hpp:
                                   * 87-156) with utopia::ShiftedPenalty: the upper bound of ugpu_qp_set_box_constraints
                                   * is the constraint (a missing one is the largest double, as
                                   * fill_empty_bounds makes it, and a lower bound is inert); keys penalty_parameter,
                                   * penalty_parameter_max (0: = penalty_parameter), penalty_parameter_factor,
                                   * zero_shift_on_reset, linear_rtol, linear_max_it; the inner solver is CG + Jacobi
                                   * to linear_rtol * ||rhs|| unless one is set through ugpu_solver_set_preconditioner */

/* convergence reasons (utopia/solvers/utopia_ConvergenceReason.hpp) */
#define UGPU_CONVERGED_FNORM_ABS 2
#define UGPU_CONVERGED_FNORM_RELATIVE 3
#define UGPU_CONVERGED_SNORM_RELATIVE 4
#define UGPU_DIVERGED_MAX_IT (-5)
#define UGPU_DIVERGED_NAN (-6)
#define UGPU_DIVERGED_INDEFINITE (-8)

typedef struct ugpu_ctx ugpu_ctx;
typedef struct ugpu_vec ugpu_vec;
typedef struct ugpu_mat ugpu_mat;
typedef struct ugpu_solver ugpu_solver;

/* SolutionStatus (utopia/solvers/utopia_SolutionStatus.hpp) plus GPU counters */
typedef struct ugpu_solution_status {
    int64_t iterates;
    double gradient_norm;
    double relative_gradient_norm;
    double step_norm;
    int32_t reason;
    int32_t converged;
    int64_t spmv_count;     /* operator applications of the outer solver */
    double execution_time;  /* seconds, host wall clock of apply() */
    int64_t kernel_launches;
} ugpu_solution_status;

/* ---------------------------------------------------------------- context ---- */
/* Replaces the PETSc/MPI initialisation of utopia::Utopia::Init (utopia/utopia_Instance.cpp). */
UGPU_API int ugpu_create(int device, ugpu_ctx **out);
UGPU_API int ugpu_destroy(ugpu_ctx *ctx);
UGPU_API const char *ugpu_last_error(const ugpu_ctx *ctx);
UGPU_API int ugpu_synchronize(ugpu_ctx *ctx);
/* kernels launched through this context so far (instrumentation) */
UGPU_API int ugpu_launch_count(const ugpu_ctx *ctx, int64_t *out);
/* the context's CUDA stream (cudaStream_t) for callers that interleave their own work */
UGPU_API int ugpu_stream(const ugpu_ctx *ctx, void **out);
/* FP64 arithmetic rate of the context's GPU, measured (no counterpart in the reference: the
 * denominator of FP64-pipe fractions).  kind 0: FMA chains on every thread (DFMA); kind 1: the
 * FP64 tensor path (mma.sync m8n8k4).  *flops_per_s: the best of three timed launches of about
 * 10 ms each, after one warm-up, on the context's stream (synchronising). */
UGPU_API int ugpu_fp64_rate(ugpu_ctx *ctx, int kind, double *flops_per_s);

/* ---------------------------------------------------------------- vectors ---- */
/* Replaces PetscVector construction/zeros/values/wrap
 * (utopia/backend/petsc/utopia_petsc_Vector.hpp:39-52; utopia/utopia_core/interfaces/utopia_Vector.hpp:21-94). */
UGPU_API int ugpu_vec_create(ugpu_ctx *ctx, int64_t n, int dtype, ugpu_vec **out);
/* borrowed device memory (cf. PetscVector::wrap with a no-op deleter,
 * utopia/plug_in_and_out/isolver/utopia_isolver_lsolve.cpp:155-161) */
UGPU_API int ugpu_vec_wrap_device(ugpu_ctx *ctx, void *device_ptr, int64_t n, int dtype, ugpu_vec **out);
UGPU_API int ugpu_vec_destroy(ugpu_vec *v);
UGPU_API int ugpu_vec_size(const ugpu_vec *v, int64_t *n, int *dtype);
UGPU_API int ugpu_vec_device_ptr(const ugpu_vec *v, void **out);
/* host array of the vector's dtype (synchronous) */
UGPU_API int ugpu_vec_upload(ugpu_vec *v, const void *host);
UGPU_API int ugpu_vec_download(const ugpu_vec *v, void *host);
/* Vector::set(value) (utopia/utopia_core/interfaces/utopia_Vector.hpp) */
UGPU_API int ugpu_vec_set(ugpu_vec *v, double value);
/* y = x with dtype conversion (assignment `y = x`) */
UGPU_API int ugpu_vec_copy(const ugpu_vec *x, ugpu_vec *y);

/* ---------------------------------------------------------------- BLAS 1 ---- */
/* BLAS1Tensor axpy / scale (utopia/utopia_core/interfaces/utopia_BLAS_Operands.hpp:10-54; PETSc VecAXPY
 * utopia/backend/petsc/utopia_petsc_Vector.cpp:671): y = alpha*x + beta*y */
UGPU_API int ugpu_axpby(double alpha, const ugpu_vec *x, double beta, ugpu_vec *y);
/* dot (VecDot, utopia_petsc_Vector.cpp:59): FP64 accumulation, deterministic order */
UGPU_API int ugpu_dot(const ugpu_vec *a, const ugpu_vec *b, double *out);
/* fused dots (utopia::dots, utopia/utopia_core/expressions/utopia_DotVecVecs.hpp:86-130; VecMDot) */
UGPU_API int ugpu_dots(int k, const ugpu_vec *const *a, const ugpu_vec *const *b, double *out);
/* norm2 (VecNorm, utopia/backend/petsc/utopia_petsc_Vector.hpp:303) */
UGPU_API int ugpu_norm2(const ugpu_vec *a, double *out);
/* e_mul/e_div/e_min/e_max (utopia/utopia_core/interfaces/utopia_ElementWiseOperand.hpp:6-12) */
UGPU_API int ugpu_pointwise(int op, const ugpu_vec *a, const ugpu_vec *b, ugpu_vec *out);
/* e_pseudo_inv (utopia/utopia_core/utopia_ElementWisePseudoInverse.hpp:20-65) */
UGPU_API int ugpu_pseudo_inverse(const ugpu_vec *in, ugpu_vec *out, double tol);
/* Reducible::reduce(Plus/Min/Max) and Normed::norm1/norm_infty
 * (utopia/utopia_core/interfaces/utopia_Reducible.hpp:13-15, utopia_Normed.hpp:12-13; PETSc VecSum,
 * VecMin, VecMax, VecNorm(NORM_1/NORM_INFINITY)); op = UGPU_RED_*, FP64 result, fixed order for sums.
 * An empty vector gives 0. */
UGPU_API int ugpu_vec_reduce(const ugpu_vec *v, int op, double *out);
/* Transformable::transform (utopia/utopia_core/interfaces/utopia_Transformable.hpp:13-23; PETSc
 * VecSqrtAbs/VecLog/VecExp/VecAbs/VecScale/VecShift/VecReciprocal): v = f(v), op = UGPU_TR_*,
 * param for POW, RECIPROCAL, SHIFT and SCALE. */
UGPU_API int ugpu_vec_transform(ugpu_vec *v, int op, double param);
/* Allocation-free fused dots (no counterpart in the reference).  For callers that cannot
 * allocate device memory -- host codes whose device memory belongs to their own pool or
 * memory space, and hot loops that cannot afford cudaFree's device-wide synchronisation.
 * Same deterministic result as ugpu_dots: out[i] = sum_j a[i][j] * b[i][j] (FP64
 * accumulation) for i < k, written to the DEVICE array d_out on `stream` (no context,
 * no synchronisation).  a, b: host arrays of k device pointers; dtype_a/dtype_b: their
 * element types.  Scratch is a fixed 38.9 KB device array inside the library (held by
 * every GPU that loads it until exit): k is limited to 8 pairs, larger k is rejected
 * with UGPU_ERR_ARG.  Each call looks up the array's device address in the current
 * context; the first call in a context also loads the library's device module, so make
 * that first call before any stream capture.  All calls share the one array, so
 * calls that overlap on the GPU (different streams, or several host threads) race. */
UGPU_API int ugpu_dots_noalloc(int k, const void *const *a, const void *const *b, const int *dtype_a,
                               const int *dtype_b, int64_t n, double *d_out, void *stream);
/* multi_min (utopia/utopia_core/eval/utopia_MultiReduce.hpp:14-24), FP64 vectors */
UGPU_API int ugpu_multi_min(const ugpu_vec *a, const ugpu_vec *b, double *out);

/* ---------------------------------------------------------------- matrices ---- */
/* CSR from host arrays (copied): PetscMatrix from CRS (utopia_isolver_lsolve.cpp:75-89 wraps
 * rowptr/colidx/values).  int32 indices, FP64 values. */
UGPU_API int ugpu_csr_create(ugpu_ctx *ctx, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t *rowptr,
                             const int32_t *colidx, const double *values, ugpu_mat **out);
/* CSR from device arrays of the same layout (copied) */
UGPU_API int ugpu_csr_create_device(ugpu_ctx *ctx, int64_t nrows, int64_t ncols, int64_t nnz,
                                    const int32_t *rowptr, const int32_t *colidx, const double *values,
                                    ugpu_mat **out);
UGPU_API int ugpu_mat_destroy(ugpu_mat *A);
UGPU_API int ugpu_mat_info(const ugpu_mat *A, int64_t *nrows, int64_t *ncols, int64_t *nnz, int *value_dtype);
/* structure and values back to host (values converted to FP64) */
UGPU_API int ugpu_csr_download(const ugpu_mat *A, int32_t *rowptr, int32_t *colidx, double *values);
/* overwrite the values of an existing pattern (host FP64 array, length nnz) */
UGPU_API int ugpu_mat_update_values(ugpu_mat *A, const double *values);
/* value-precision copy (FP64 -> FP32 / BF16 storage) for the mixed-precision hierarchy */
UGPU_API int ugpu_mat_cast(const ugpu_mat *A, int value_dtype, ugpu_mat **out);
/* choose the SpMV layout: UGPU_FORMAT_CSR or UGPU_FORMAT_SELL (sliced ELL, the default) */
UGPU_API int ugpu_mat_set_format(ugpu_mat *A, int format);
/* sliced-ELL statistics: slices, stored slots (incl. padding), diagonal-keyed slices */
UGPU_API int ugpu_mat_sell_info(const ugpu_mat *A, int64_t *nslices, int64_t *nstored, int64_t *ndiag_slices,
                                int *rows_per_slice);
/* sliced-ELL layout: *interleaved = 1 when lane l of a slice's warp owns rows l + 32 r (FP32 / BF16
 * operators whose slices are all keyed; their products run through the shared-memory staged kernel
 * when the vectors are 16-byte aligned), 0 when it owns R consecutive rows; *anchored_slices = slices
 * keyed by col - (first column of the row) (transfer operators).  Either pointer may be NULL.  No
 * counterpart in the reference (a layout query of this backend). */
UGPU_API int ugpu_mat_sell_layout(const ugpu_mat *A, int *interleaved, int64_t *anchored_slices);
/* diag(A) (MatGetDiagonal, utopia/backend/petsc/utopia_petsc_Matrix.cpp:756) */
UGPU_API int ugpu_diag(const ugpu_mat *A, ugpu_vec *d);
/* explicit transpose (BLAS3Matrix::transpose, utopia_BLAS_Operands.hpp:135-171; used by IPRTransfer
 * utopia/solvers/multilevel/transfer/utopia_IPRTransfer.hpp:28-39) */
UGPU_API int ugpu_transpose(const ugpu_mat *A, ugpu_mat **out);
/* C = A*B, full symbolic structure (MatMatMult; utopia/utopia_core/eval/utopia_Eval_Multiply.hpp:10-102) */
UGPU_API int ugpu_spgemm(const ugpu_mat *A, const ugpu_mat *B, ugpu_mat **out);
/* Galerkin product Ac = P^T A P (utopia::ptap -> MatPtAP,
 * utopia/backend/petsc/eval/utopia_petsc_Eval_Multiply.cpp:12-61) */
UGPU_API int ugpu_ptap(const ugpu_mat *A, const ugpu_mat *P, ugpu_mat **out);
/* PetscEvalTripleMatrixProduct::ptap(result, A, P, reuse)
 * (utopia/backend/petsc/eval/utopia_petsc_Eval_Multiply.cpp:9-50, MatPtAP's MatReuse):
 * reuse = 0 (MAT_INITIAL_MATRIX): *out = P^T A P, a new matrix that keeps its product structure;
 * reuse = 1 (MAT_REUSE_MATRIX): *out holds a product of an earlier reuse = 0 call; its values are
 * recomputed in place for the current values of A and P (UGPU_ERR_ARG if the structure of A or P
 * is no longer the one the product was formed from; a digest of rowptr/colidx is compared). */
UGPU_API int ugpu_ptap_reuse(const ugpu_mat *A, const ugpu_mat *P, int reuse, ugpu_mat **out);

/* ---------------------------------------------------------------- SpMV family ---- */
/* y = A x (MatMult, utopia/backend/petsc/utopia_petsc_Matrix.cpp:1358; Operator::apply
 * utopia/utopia_core/interfaces/utopia_Operator.hpp:47).  x, y: FP64 or FP32 (both the same). */
UGPU_API int ugpu_spmv(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y);
/* y = A x + v (MatMultAdd, utopia_petsc_Matrix.cpp:1400-1404); y may alias v */
UGPU_API int ugpu_spmv_add(const ugpu_mat *A, const ugpu_vec *x, const ugpu_vec *v, ugpu_vec *y);
/* y = A x and dot[0] = (x, y) in FP64 from the same kernel (the fused product and dot of CG's
 * `Ap = A p; alpha = rho / dot(p, Ap)`, utopia_ConjugateGradient_impl.hpp:225-230).  dot: an FP64
 * vector of at least one entry; the scalar stays on the device (asynchronous, like every vector
 * operation of the stream).  The dot is a fixed-order two-stage reduction: repeated calls give
 * identical bits.  A square operator. */
UGPU_API int ugpu_spmv_dot(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y, ugpu_vec *dot);
/* Test of the staged product's bounded waits (no counterpart in the reference): y = A x through
 * the shared-memory staged kernel (FP32 / BF16 operator, FP32 vectors) with every wait for a
 * stage's copies limited to spin_cycles (1 .. 1e8) and, in the first CTA's first warp, no copy
 * issued for its first slice, so that wait runs out.  The kernel then records the context's error
 * flag, lets its other copies land and returns; the next synchronising call (ugpu_synchronize)
 * returns UGPU_ERR_CUDA and clears the flag, and the context stays usable.  *launched = 0 when the
 * operator does not take the staged kernel (nothing runs). */
UGPU_API int ugpu_test_staged_wait_timeout(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y, int64_t spin_cycles,
                                           int *launched);
/* r = b - A x (Eval_Residual, utopia/utopia_core/eval/utopia_Eval_Residual.hpp:19-38), one pass */
UGPU_API int ugpu_residual(const ugpu_mat *A, const ugpu_vec *b, const ugpu_vec *x, ugpu_vec *r);
/* fused Jacobi sweep x_out = x + omega * d^+ (b - A x) (utopia/solvers/smoothers/utopia_Jacobi.hpp:131-141
 * with the relaxation omega; omega = 1 is the reference); x_out must not alias x */
UGPU_API int ugpu_jacobi_sweep(const ugpu_mat *A, const ugpu_vec *b, const ugpu_vec *x, double omega,
                               ugpu_vec *x_out);

/* ---------------------------------------------------------------- solvers ---- */
/* Solvers mirror the reference classes.  Parameters use the reference's Configurable::read key
 * names (utopia/solvers/linear/utopia_IterativeSolver.hpp:34-43 atol, rtol, stol, max_it, verbose;
 * utopia/solvers/multilevel/utopia_MultiLevelBase.hpp:46-54 pre_smoothing_steps,
 * post_smoothing_steps; utopia/solvers/multilevel/utopia_LinearMultiLevel.hpp:37-44
 * must_generate_masks; utopia/solvers/smoothers/utopia_Chebyshev3level.hpp:39-56 scale_max_eig,
 * scale_min_eig, power_method_tol, power_method_max_it; utopia/solvers/nonlinear/constrained/
 * quadratic_programming/utopia_MPRGP.hpp:29-35 eig_comp_tol, power_method_max_it;
 * utopia_ProjectedGaussSeidel.hpp:34-41 use_symmetric_sweep, n_local_sweeps) plus the
 * backend's own keys: "smoother" (0 Jacobi, 1 Chebyshev3level, 2 PointJacobi), "omega",
 * "precision" (UGPU_F64 / UGPU_F32 / UGPU_BF16 level storage of the multigrid; the coarse solve
 * stays FP64 unless "coarse_fp32" = 1 applies an FP32 copy of the coarse inverse), "flexible"
 * (flexible CG outer iteration), "fix_semidefinite_operators", "keep_galerkin_structure" (1: the
 * Galerkin products keep their structure and an update with an operator of the same structure
 * recomputes values only), "rand_seed" (power-method start vectors), "use_graphs" (1: a solve is
 * one CUDA graph launch), "projected_gradient_stop" (PGS), "reset_initial_guess"; read-only
 * results: "lambda_max" (MPRGP), "galerkin_assemblies", "n_active" (monotone multigrid).  The
 * algebraic, BiCGStab, semismooth Newton and monotone multigrid keys are listed with their kinds. */
UGPU_API int ugpu_solver_create(ugpu_ctx *ctx, int kind, ugpu_solver **out);
UGPU_API int ugpu_solver_destroy(ugpu_solver *s);
UGPU_API int ugpu_solver_set(ugpu_solver *s, const char *key, double value);
UGPU_API int ugpu_solver_get(const ugpu_solver *s, const char *key, double *value);
/* PreconditionedSolver::set_preconditioner (utopia/solvers/linear/utopia_PreconditionedSolver.hpp:13-92);
 * the preconditioner handle is borrowed and must outlive the solver */
UGPU_API int ugpu_solver_set_preconditioner(ugpu_solver *s, ugpu_solver *prec);
/* LinearMultiLevel::set_transfer_operators, interpolation operators ordered coarse -> fine
 * (utopia_LinearMultiLevel.hpp:58-79); the matrices are copied */
UGPU_API int ugpu_mg_set_transfer_operators(ugpu_solver *mg, int n, const ugpu_mat *const *interpolations);
/* Galerkin operator of level l (0 = coarsest, after the std::reverse of
 * utopia_LinearMultiLevel.hpp:224), returned as a new FP64 CSR copy */
UGPU_API int ugpu_mg_level_matrix(const ugpu_solver *mg, int l, ugpu_mat **out);
UGPU_API int ugpu_mg_n_levels(const ugpu_solver *mg, int *out);
/* Chebyshev eigen-bounds of level l (Chebyshev3level::init_eigs, utopia_Chebyshev3level.hpp:118-121) */
UGPU_API int ugpu_mg_eigs(const ugpu_solver *mg, int l, double *eig_max, double *eig_min);
/* one V-cycle z = M^{-1} r from a zero initial guess (Multigrid::apply with max_it 1) */
UGPU_API int ugpu_mg_vcycle(ugpu_solver *mg, const ugpu_vec *r, ugpu_vec *z);
/* update(op): LinearSolver::update (utopia/solvers/linear/utopia_LinearSolver.hpp:70-73).  The
 * matrix is borrowed and must stay alive while the solver uses it. */
UGPU_API int ugpu_solver_update(ugpu_solver *s, const ugpu_mat *A);
/* apply(rhs, x): LinearSolver::apply / Multigrid::apply / ConjugateGradient::solve(op, b, x) with the
 * stored operator; x holds the initial guess on entry */
UGPU_API int ugpu_solver_apply(ugpu_solver *s, const ugpu_vec *rhs, ugpu_vec *x);
/* solve(A, b, x) = update(A) + apply(b, x) (OperatorBasedLinearSolver::solve,
 * utopia/solvers/linear/utopia_MatrixFreeLinearSolver.hpp:54-57) */
UGPU_API int ugpu_solver_solve(ugpu_solver *s, const ugpu_mat *A, const ugpu_vec *b, ugpu_vec *x);
/* QPSolver::set_box_constraints (utopia/solvers/nonlinear/constrained/quadratic_programming/
 * utopia_QPSolver.hpp:14-139); NULL bound = unbounded (fill_empty_bounds,
 * utopia/solvers/nonlinear/constrained/utopia_BoxConstraints.hpp:281) */
UGPU_API int ugpu_qp_set_box_constraints(ugpu_solver *s, const ugpu_vec *lb, const ugpu_vec *ub);
UGPU_API int ugpu_solver_status(const ugpu_solver *s, ugpu_solution_status *out);
/* colouring used by the multicolour projected Gauss-Seidel sweep (greedy first-fit in index
 * order; red-black (x + y) mod 2 on the 5-point grid).  The reference sweeps rows
 * lexicographically (utopia_ProjectedGaussSeidel.hpp:213-254); colour may be NULL. */
UGPU_API int ugpu_pgs_colouring(const ugpu_solver *pgs, int32_t *colour, int *ncolours);
/* Aggregation of level `level` of an algebraic multigrid (0 = the fine operator's): parent[i] = the
 * aggregate of row i, -2 for excluded Dirichlet rows (Agglomerate::create_transfer_matrix,
 * utopia/solvers/multilevel/agglomerate/utopia_Agglomerate.hpp:51-186); *n rows, *n_coarse aggregates.
 * The algebraic multigrid (UGPU_SOLVER_AMG, utopia/solvers/multilevel/utopia_AlgebraicMultigrid.hpp:16-177)
 * takes the keys n_levels (reference default 2; 0 = coarsen until at most max_coarse_rows rows or until a
 * level shrinks by less than 4:3), bmax,
 * weight, use_additive_correction and every multigrid key; the ugpu_mg_* queries accept it. */
UGPU_API int ugpu_amg_parent(const ugpu_solver *amg, int level, int32_t *parent, int64_t *n, int64_t *n_coarse);

/* The monotone multigrid (UGPU_SOLVER_MONOTONE_MG): keys pre_smoothing_steps, post_smoothing_steps
 * (PGS steps on the fine level and smoothing steps of the linear multigrid), n_local_sweeps,
 * use_symmetric_sweep, smoother, omega, active_set_tol (ActiveSet tol), coarse_space_it,
 * use_coarse_space; read-only galerkin_assemblies and n_active.  ugpu_mg_n_levels / ugpu_mg_level_matrix
 * see the fine operator as the finest level and the truncated Galerkin operator below it.
 * ugpu_mmg_active_set: the active-set indicator (ActiveSet::indicator, 0/1 per fine dof, n
 * entries; may be NULL) and its size after the last update/apply. */
UGPU_API int ugpu_mmg_active_set(const ugpu_solver *mmg, int32_t *indicator, int64_t *n_active);

/* The shifted-penalty QP solver's optional terms (ShiftedPenaltyQPSolver::set_transform,
 * set_selection, set_scaling_matrix; utopia_ShiftedPenaltyQPSolver.hpp:17-53, utopia_Penalty.hpp:
 * 49-55).  Transformation: square T and O of the operator's size; the constraint acts on
 * O^T (T x), directions map back by T^T (O v) and the penalty Hessian diag(h) by T^T (O^T diag(h) O) T
 * (the qp_solve app's PrototypeTransformation, utopia/apps/qp_solve/utopia_qp_solve.cpp:68-88).
 * Selection: the penalty gradient and Hessian are multiplied by it entrywise.  Scaling: S maps both.
 * NULL clears a term; the solver keeps the pointers (the caller keeps the objects alive). */
UGPU_API int ugpu_penalty_set_transform(ugpu_solver *s, const ugpu_mat *T, const ugpu_mat *O);
UGPU_API int ugpu_penalty_set_selection(ugpu_solver *s, const ugpu_vec *selection);
UGPU_API int ugpu_penalty_set_scaling_matrix(ugpu_solver *s, const ugpu_mat *S);

/* ---------------------------------------------------------------- files ---- */
/* PETSc binary matrices and vectors (utopia::read / write over MatLoad / VecLoad, used for the
 * reference's inputs in utopia/data and by utopia/apps/ls_solve/utopia_ls_solve.cpp:117-133).  Layout
 * (big endian, 32-bit indices): Mat = classid 1211216, M, N, nnz, row lengths, column indices,
 * float64 values; Vec = classid 1211214, N, float64 values.  Rows must have ascending columns. */
UGPU_API int ugpu_petsc_read_mat(ugpu_ctx *ctx, const char *path, ugpu_mat **out);
UGPU_API int ugpu_petsc_read_vec(ugpu_ctx *ctx, const char *path, ugpu_vec **out);
UGPU_API int ugpu_petsc_write_mat(const ugpu_mat *A, const char *path);
UGPU_API int ugpu_petsc_write_vec(const ugpu_vec *x, const char *path);
/* Raw CRS directory (rowptr.raw, colidx.raw, values.raw; native endianness) as read by the reference's
 * qp_solve inputs (utopia/data/test/qpsolve.yaml:13-35): index_bytes 4 or 8, value_bytes 8 or 4,
 * ncols 0 = square.  Raw vectors: one native array of value_bytes elements (written as float64). */
UGPU_API int ugpu_raw_crs_read(ugpu_ctx *ctx, const char *dir, int index_bytes, int value_bytes, int64_t ncols,
                               ugpu_mat **out);
UGPU_API int ugpu_raw_vec_read(ugpu_ctx *ctx, const char *path, int value_bytes, ugpu_vec **out);
UGPU_API int ugpu_raw_vec_write(const ugpu_vec *x, const char *path);

/* ---------------------------------------------------------------- differentiable solve ---- */
/* No reference counterpart (utopia/differentiable/ is symbolic autodiff of expressions, not an
 * adjoint solver).  A graph with per-edge log-conductances theta:
 *   A(theta) = sum_e exp(theta_e) (e_src - e_dst)(e_src - e_dst)^T + diag(boundary).
 * edge_of_pos[k] names the edge of CSR entry k of A's pattern (-1 on the diagonal).  The
 * adjoint of x = A^{-1} b reuses the forward solver (A is symmetric): lambda = A^{-1} dL/dx,
 * dL/db = lambda, dL/dtheta_e = -exp(theta_e)(lambda_src - lambda_dst)(x_src - x_dst),
 * dL/dA_ij = -lambda_i x_j. */
typedef struct ugpu_graph ugpu_graph;
UGPU_API int ugpu_graph_create(ugpu_ctx *ctx, int64_t n, int64_t E, const int32_t *src, const int32_t *dst,
                               int64_t nnz, const int32_t *edge_of_pos, const double *boundary, ugpu_graph **out);
UGPU_API int ugpu_graph_destroy(ugpu_graph *g);
/* write A(theta) into the values of A (FP64, the n x n pattern edge_of_pos describes); theta FP32 or FP64 */
UGPU_API int ugpu_graph_assemble(ugpu_graph *g, const ugpu_vec *theta, ugpu_mat *A);
/* grad (dtype of theta) = dL/dtheta from lambda and x (FP64) */
UGPU_API int ugpu_graph_edge_grad(ugpu_graph *g, const ugpu_vec *theta, const ugpu_vec *lam, const ugpu_vec *x,
                                  ugpu_vec *grad);
/* gvals[k] = -lambda_i x_j for every CSR entry k = (i, j) of A (FP64, length nnz) */
UGPU_API int ugpu_pattern_grad(const ugpu_mat *A, const ugpu_vec *lam, const ugpu_vec *x, ugpu_vec *gvals);

/* ---------------------------------------------------------------- box constraints ---- */
/* project(lb, ub, x) (utopia/solvers/nonlinear/constrained/utopia_VariableBoundSolverInterface.hpp:134-155) */
UGPU_API int ugpu_project(const ugpu_vec *lb, const ugpu_vec *ub, ugpu_vec *x);
/* Active-set compaction (the predicates of MPRGP::get_beta / get_fi,
 * utopia/solvers/nonlinear/constrained/quadratic_programming/utopia_MPRGP.hpp:266-348): the indices i
 * of x in the set `which` (UGPU_SET_ACTIVE or UGPU_SET_FREE), ascending, written to the DEVICE int32
 * array `indices` (capacity n; may be NULL to count only), their number to *count (synchronous).
 * lb / ub may be NULL (unbounded side). */
UGPU_API int ugpu_active_set_compact(const ugpu_vec *x, const ugpu_vec *lb, const ugpu_vec *ub, int which,
                                     int32_t *indices, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif /* UGPU_H */
