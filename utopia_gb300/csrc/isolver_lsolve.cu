// The isolver linear-solver plugin (include/isolver_lsolve.h) over the libugpu C ABI.
//
// The reference's plugin (utopia/plug_in_and_out/isolver/utopia_isolver_lsolve.cpp:42-220)
// wraps the caller's CRS arrays and vectors in backend objects without copying and calls
// LinearSolver::update / apply.  Here the backend is one GPU: update_* copies the CRS matrix
// to the device (a later call with the same pattern arrays only refreshes the values), and
// apply copies rhs and the initial guess in and the solution out.  The solver is
// ConjugateGradient + InvDiagPreconditioner, the reference plugin's ConjugateGradient
// configuration (utopia_isolver_lsolve.cpp:19-22).
#include <cstdlib>

#include "../../include/isolver_lsolve.h"
#include "../../include/ugpu.h"

namespace {

struct Operator {
    ugpu_mat *mat = nullptr;
    const isolver_idx_t *rowptr = nullptr;  // pattern of the last upload (pointer identity)
    const isolver_idx_t *colidx = nullptr;
    int64_t n = 0, nnz = 0;
};

struct LSolve {
    ugpu_ctx *ctx = nullptr;
    ugpu_solver *cg = nullptr;
    ugpu_solver *jacobi = nullptr;
    Operator A, P;
    ugpu_vec *b = nullptr, *x = nullptr;
    int64_t n = 0;
};

LSolve *get(const isolver_lsolve_t *info) {
    return info ? static_cast<LSolve *>(info->private_data) : nullptr;
}

void release(LSolve *s) {
    if (!s) return;
    if (s->b) ugpu_vec_destroy(s->b);
    if (s->x) ugpu_vec_destroy(s->x);
    if (s->A.mat) ugpu_mat_destroy(s->A.mat);
    if (s->P.mat) ugpu_mat_destroy(s->P.mat);
    if (s->cg) ugpu_solver_destroy(s->cg);
    if (s->jacobi) ugpu_solver_destroy(s->jacobi);
    if (s->ctx) ugpu_destroy(s->ctx);
    delete s;
}

// copies (or refreshes the values of) one operator
int upload(LSolve *s, Operator &op, ptrdiff_t n_local, ptrdiff_t n_global, const isolver_idx_t *rowptr,
           const isolver_idx_t *colidx, const isolver_scalar_t *values) {
    if (!s) return UGPU_ERR_STATE;
    if (n_local != n_global || n_global < 0 || !rowptr) return UGPU_ERR_UNSUPPORTED;  // one process
    const int64_t n = n_global, nnz = rowptr[n];
    if (op.mat && op.rowptr == rowptr && op.colidx == colidx && op.n == n && op.nnz == nnz)
        return ugpu_mat_update_values(op.mat, values);
    if (op.mat) ugpu_mat_destroy(op.mat);
    op = Operator{};
    int rc = ugpu_csr_create(s->ctx, n, n, nnz, rowptr, colidx, values, &op.mat);
    if (rc != UGPU_OK) {
        op.mat = nullptr;
        return rc;
    }
    op.rowptr = rowptr;
    op.colidx = colidx;
    op.n = n;
    op.nnz = nnz;
    return UGPU_OK;
}

int ensure_vectors(LSolve *s, int64_t n) {
    if (s->b && s->n == n) return UGPU_OK;
    if (s->b) ugpu_vec_destroy(s->b);
    if (s->x) ugpu_vec_destroy(s->x);
    s->b = s->x = nullptr;
    int rc = ugpu_vec_create(s->ctx, n, UGPU_F64, &s->b);
    if (rc == UGPU_OK) rc = ugpu_vec_create(s->ctx, n, UGPU_F64, &s->x);
    s->n = (rc == UGPU_OK) ? n : 0;
    return rc;
}

int set_param(const isolver_lsolve_t *info, const char *key, double v) {
    LSolve *s = get(info);
    return s ? ugpu_solver_set(s->cg, key, v) : UGPU_ERR_STATE;
}

}  // namespace

extern "C" {

int isolver_lsolve_init(isolver_lsolve_t *info) {
    if (!info) return UGPU_ERR_ARG;
    info->private_data = nullptr;
    const char *dev = std::getenv("UGPU_DEVICE");
    auto *s = new LSolve();
    int rc = ugpu_create(dev ? std::atoi(dev) : 0, &s->ctx);
    if (rc == UGPU_OK) rc = ugpu_solver_create(s->ctx, UGPU_SOLVER_CG, &s->cg);
    if (rc == UGPU_OK) rc = ugpu_solver_create(s->ctx, UGPU_SOLVER_INVDIAG, &s->jacobi);
    if (rc == UGPU_OK) rc = ugpu_solver_set_preconditioner(s->cg, s->jacobi);
    if (rc != UGPU_OK) {
        release(s);
        return rc;
    }
    info->private_data = s;
    return UGPU_OK;
}

int isolver_lsolve_update_crs(const isolver_lsolve_t *info, const ptrdiff_t n_local, const ptrdiff_t n_global,
                              const isolver_idx_t *const rowptr, const isolver_idx_t *const colidx,
                              const isolver_scalar_t *const values) {
    LSolve *s = get(info);
    if (!s) return UGPU_ERR_STATE;
    int rc = upload(s, s->A, n_local, n_global, rowptr, colidx, values);
    if (rc == UGPU_OK) rc = ensure_vectors(s, n_global);
    if (rc == UGPU_OK) rc = ugpu_solver_update(s->cg, s->A.mat);  // also updates the Jacobi preconditioner
    return rc;
}

int isolver_lsolve_update_with_preconditioner_crs(const isolver_lsolve_t *info, const ptrdiff_t n_local,
                                                  const ptrdiff_t n_global, const isolver_idx_t *const rowptr,
                                                  const isolver_idx_t *const colidx,
                                                  const isolver_scalar_t *const values,
                                                  const isolver_idx_t *const prec_rowptr,
                                                  const isolver_idx_t *const prec_colidx,
                                                  const isolver_scalar_t *const prec_values) {
    LSolve *s = get(info);
    if (!s) return UGPU_ERR_STATE;
    int rc = upload(s, s->A, n_local, n_global, rowptr, colidx, values);
    if (rc == UGPU_OK) rc = upload(s, s->P, n_local, n_global, prec_rowptr, prec_colidx, prec_values);
    if (rc == UGPU_OK) rc = ensure_vectors(s, n_global);
    if (rc == UGPU_OK) rc = ugpu_solver_update(s->cg, s->A.mat);
    if (rc == UGPU_OK) rc = ugpu_solver_update(s->jacobi, s->P.mat);  // preconditioner from the second matrix
    return rc;
}

int isolver_lsolve_apply(const isolver_lsolve_t *info, const isolver_scalar_t *const rhs, isolver_scalar_t *const x) {
    LSolve *s = get(info);
    if (!s || !s->A.mat) return UGPU_ERR_STATE;
    if (!rhs || !x) return UGPU_ERR_ARG;
    int rc = ugpu_vec_upload(s->b, rhs);
    if (rc == UGPU_OK) rc = ugpu_vec_upload(s->x, x);
    if (rc == UGPU_OK) rc = ugpu_solver_apply(s->cg, s->b, s->x);
    if (rc == UGPU_OK) rc = ugpu_vec_download(s->x, x);
    return rc;
}

int isolver_lsolve_set_max_iterations(const isolver_lsolve_t *info, const int max_it) {
    return set_param(info, "max_it", double(max_it));
}

int isolver_lsolve_set_atol(const isolver_lsolve_t *info, const isolver_scalar_t atol) {
    return set_param(info, "atol", atol);
}

int isolver_lsolve_set_stol(const isolver_lsolve_t *info, const isolver_scalar_t stol) {
    return set_param(info, "stol", stol);
}

int isolver_lsolve_set_rtol(const isolver_lsolve_t *info, const isolver_scalar_t rtol) {
    return set_param(info, "rtol", rtol);
}

int isolver_lsolve_set_verbosity(const isolver_lsolve_t *info, const int verbosity_level) {
    return set_param(info, "verbose", verbosity_level > 0 ? 1.0 : 0.0);
}

int isolver_lsolve_destroy(isolver_lsolve_t *info) {
    if (!info) return UGPU_ERR_ARG;
    release(get(info));
    info->private_data = nullptr;
    return UGPU_OK;
}

}  // extern "C"
