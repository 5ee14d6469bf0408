/* isolver linear-solver plugin interface, served by libugpu on one GB300.
 *
 * The reference implements these ten entry points in
 * utopia/plug_in_and_out/isolver/utopia_isolver_lsolve.cpp:42-220 against the header
 * isolver_lsolve.h of the external isolver project, which is not part of the reference
 * tree.  The types below restate what those call sites use: the handle carries a
 * communicator and an opaque private_data pointer; CRS indices are isolver_idx_t and
 * values isolver_scalar_t; every function returns 0 on success.
 *
 * Here: one process, one GPU (UGPU_DEVICE, default 0).  comm is not used and n_local must
 * equal n_global.  The CRS arrays, rhs and x are host memory owned by the caller (as in the
 * reference, "Resources are freed outside!"); update_* copies the matrix to the device, and
 * a later update_* with the same rowptr/colidx pointers and sizes only refreshes the values.
 * The solver is ConjugateGradient with the InvDiag (Jacobi) preconditioner, the reference's
 * ConjugateGradient branch (utopia_isolver_lsolve.cpp:19-22); it stops on ||r|| <= atol or
 * max_it, as utopia's CG does.  The UTOPIA_LINEAR_SOLVER_CONFIG file is not read.  A failing
 * call returns a negative libugpu status code (include/ugpu.h). */
#ifndef ISOLVER_LSOLVE_H
#define ISOLVER_LSOLVE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ISOLVER_EXPORT
#if defined(__GNUC__)
#define ISOLVER_EXPORT __attribute__((visibility("default")))
#else
#define ISOLVER_EXPORT
#endif
#endif

typedef int isolver_idx_t;       /* CRS row pointers and column indices (int32, as libugpu's CSR) */
typedef double isolver_scalar_t; /* matrix, rhs and solution values */
typedef void *isolver_comm_t;    /* communicator slot; unused by the single-GPU plugin */

typedef struct {
    isolver_comm_t comm;
    void *private_data;
} isolver_lsolve_t;

/* creates the solver in info->private_data */
int ISOLVER_EXPORT isolver_lsolve_init(isolver_lsolve_t *info);
/* the operator (utopia_isolver_lsolve.cpp:68-91) */
int ISOLVER_EXPORT isolver_lsolve_update_crs(const isolver_lsolve_t *info, const ptrdiff_t n_local,
                                             const ptrdiff_t n_global, const isolver_idx_t *const rowptr,
                                             const isolver_idx_t *const colidx,
                                             const isolver_scalar_t *const values);
/* the operator and a separate matrix for the preconditioner (:93-139): the Jacobi preconditioner
 * takes its diagonal from the second matrix */
int ISOLVER_EXPORT isolver_lsolve_update_with_preconditioner_crs(
    const isolver_lsolve_t *info, const ptrdiff_t n_local, const ptrdiff_t n_global,
    const isolver_idx_t *const rowptr, const isolver_idx_t *const colidx, const isolver_scalar_t *const values,
    const isolver_idx_t *const prec_rowptr, const isolver_idx_t *const prec_colidx,
    const isolver_scalar_t *const prec_values);
/* x = A^{-1} rhs with x as the initial guess (:141-162) */
int ISOLVER_EXPORT isolver_lsolve_apply(const isolver_lsolve_t *info, const isolver_scalar_t *const rhs,
                                        isolver_scalar_t *const x);
/* solver parameters (:164-201) */
int ISOLVER_EXPORT isolver_lsolve_set_max_iterations(const isolver_lsolve_t *info, const int max_it);
int ISOLVER_EXPORT isolver_lsolve_set_atol(const isolver_lsolve_t *info, const isolver_scalar_t atol);
int ISOLVER_EXPORT isolver_lsolve_set_stol(const isolver_lsolve_t *info, const isolver_scalar_t stol);
int ISOLVER_EXPORT isolver_lsolve_set_rtol(const isolver_lsolve_t *info, const isolver_scalar_t rtol);
int ISOLVER_EXPORT isolver_lsolve_set_verbosity(const isolver_lsolve_t *info, const int verbosity_level);
/* frees the solver and the device copies (:212-220) */
int ISOLVER_EXPORT isolver_lsolve_destroy(isolver_lsolve_t *info);

#ifdef __cplusplus
}
#endif

#endif /* ISOLVER_LSOLVE_H */
