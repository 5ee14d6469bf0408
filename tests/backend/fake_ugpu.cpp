// A CPU stand-in for the part of the C ABI (include/ugpu.h) that include/utopia_cuda_backend.hpp
// calls -- TEST INFRASTRUCTURE ONLY.
//
// It lets tests/test_cuda_backend.py run the reference's solver templates over the CUDA
// backend's classes without a GPU, to check the backend header's own logic (host mirrors and
// their offload flags, aliasing, the residual / triple-product / fused-dot specialisations)
// against the same templates over the CPU backend of oracle/ref/.  Every entry point restates
// the operation with the arithmetic order of that backend (row-ordered CSR sums, dots summed in
// fixed 8192-entry blocks, P^T A P as R (A P) with full structure, dense Cholesky), so the two
// runs agree bit for bit.  The GPU library itself is checked against the oracle by the -m gpu
// tests; this file is never linked into it.
#include "ugpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

struct ugpu_ctx {
    int device = 0;
};
struct ugpu_vec {
    std::vector<double> v;
};
struct ugpu_mat {
    int64_t m = 0, n = 0;
    std::vector<int32_t> rp, ci;
    std::vector<double> v;
};
struct ugpu_solver {
    int64_t n = 0;
    std::vector<double> L;
};

namespace {
std::string g_error;

int fail(const char *what) {
    g_error = what;
    return -2;
}

double blocked_dot(const std::vector<double> &a, const std::vector<double> &b) {
    const size_t n = a.size();
    double total = 0.0;
    for (size_t s = 0; s < n; s += 8192) {
        const size_t e = std::min(n, s + 8192);
        double part = 0.0;
        for (size_t i = s; i < e; ++i) part += a[i] * b[i];
        total += part;
    }
    return total;
}

void matvec(const ugpu_mat &A, const std::vector<double> &x, std::vector<double> &y) {
    std::vector<double> out(size_t(A.m));
    for (int64_t i = 0; i < A.m; ++i) {
        double s = 0;
        for (int32_t k = A.rp[size_t(i)]; k < A.rp[size_t(i) + 1]; ++k) s += A.v[size_t(k)] * x[size_t(A.ci[size_t(k)])];
        out[size_t(i)] = s;
    }
    y.swap(out);
}

ugpu_mat transpose(const ugpu_mat &A) {
    ugpu_mat T;
    T.m = A.n;
    T.n = A.m;
    T.rp.assign(size_t(A.n) + 1, 0);
    for (int32_t c : A.ci) T.rp[size_t(c) + 1]++;
    for (int64_t j = 0; j < A.n; ++j) T.rp[size_t(j) + 1] += T.rp[size_t(j)];
    T.ci.resize(A.ci.size());
    T.v.resize(A.v.size());
    std::vector<int32_t> pos(T.rp.begin(), T.rp.end() - 1);
    for (int64_t i = 0; i < A.m; ++i)
        for (int32_t k = A.rp[size_t(i)]; k < A.rp[size_t(i) + 1]; ++k) {
            const int32_t p = pos[size_t(A.ci[size_t(k)])]++;
            T.ci[size_t(p)] = int32_t(i);
            T.v[size_t(p)] = A.v[size_t(k)];
        }
    return T;
}

ugpu_mat spgemm(const ugpu_mat &A, const ugpu_mat &B) {
    ugpu_mat C;
    C.m = A.m;
    C.n = B.n;
    C.rp.assign(size_t(A.m) + 1, 0);
    std::vector<int64_t> mark(size_t(B.n), -1);
    std::vector<double> acc(size_t(B.n), 0.0);
    std::vector<int32_t> cols;
    for (int64_t i = 0; i < A.m; ++i) {
        cols.clear();
        for (int32_t ka = A.rp[size_t(i)]; ka < A.rp[size_t(i) + 1]; ++ka) {
            const int32_t j = A.ci[size_t(ka)];
            const double a = A.v[size_t(ka)];
            for (int32_t kb = B.rp[size_t(j)]; kb < B.rp[size_t(j) + 1]; ++kb) {
                const int32_t c = B.ci[size_t(kb)];
                if (mark[size_t(c)] != i) {
                    mark[size_t(c)] = i;
                    acc[size_t(c)] = 0.0;
                    cols.push_back(c);
                }
                acc[size_t(c)] += a * B.v[size_t(kb)];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int32_t c : cols) {
            C.ci.push_back(c);
            C.v.push_back(acc[size_t(c)]);
        }
        C.rp[size_t(i) + 1] = int32_t(C.ci.size());
    }
    return C;
}
}  // namespace

extern "C" {

int ugpu_create(int device, ugpu_ctx **out) {
    *out = new ugpu_ctx{device};
    return 0;
}
int ugpu_destroy(ugpu_ctx *ctx) {
    delete ctx;
    return 0;
}
const char *ugpu_last_error(const ugpu_ctx *) { return g_error.c_str(); }

int ugpu_vec_create(ugpu_ctx *, int64_t n, int dtype, ugpu_vec **out) {
    if (dtype != UGPU_F64) return fail("FP64 only");
    *out = new ugpu_vec{std::vector<double>(size_t(n), 0.0)};
    return 0;
}
int ugpu_vec_destroy(ugpu_vec *v) {
    delete v;
    return 0;
}
int ugpu_vec_upload(ugpu_vec *v, const void *host) {
    std::memcpy(v->v.data(), host, v->v.size() * sizeof(double));
    return 0;
}
int ugpu_vec_download(const ugpu_vec *v, void *host) {
    std::memcpy(host, v->v.data(), v->v.size() * sizeof(double));
    return 0;
}
int ugpu_vec_set(ugpu_vec *v, double value) {
    std::fill(v->v.begin(), v->v.end(), value);
    return 0;
}
int ugpu_vec_copy(const ugpu_vec *x, ugpu_vec *y) {
    y->v = x->v;
    return 0;
}
int ugpu_axpby(double alpha, const ugpu_vec *x, double beta, ugpu_vec *y) {
    for (size_t i = 0; i < y->v.size(); ++i) {
        const double xi = x->v[i];
        y->v[i] = (beta == 0.0) ? alpha * xi : (beta == 1.0 ? y->v[i] + alpha * xi : alpha * xi + beta * y->v[i]);
    }
    return 0;
}
int ugpu_dot(const ugpu_vec *a, const ugpu_vec *b, double *out) {
    *out = blocked_dot(a->v, b->v);
    return 0;
}
int ugpu_dots(int k, const ugpu_vec *const *a, const ugpu_vec *const *b, double *out) {
    for (int i = 0; i < k; ++i) out[i] = blocked_dot(a[i]->v, b[i]->v);
    return 0;
}
int ugpu_norm2(const ugpu_vec *a, double *out) {
    *out = std::sqrt(blocked_dot(a->v, a->v));
    return 0;
}
int ugpu_pointwise(int op, const ugpu_vec *a, const ugpu_vec *b, ugpu_vec *out) {
    for (size_t i = 0; i < a->v.size(); ++i) {
        const double x = a->v[i], y = b->v[i];
        out->v[i] = op == UGPU_EMUL ? x * y : op == UGPU_EDIV ? x / y : op == UGPU_EMIN ? std::min(y, x) : std::max(y, x);
    }
    return 0;
}
int ugpu_vec_reduce(const ugpu_vec *v, int op, double *out) {
    double r = (op == UGPU_RED_SUM || op == UGPU_RED_ASUM) ? 0.0 : (op == UGPU_RED_MIN ? 1.7976931348623157e308 : -1.7976931348623157e308);
    for (double x : v->v) {
        if (op == UGPU_RED_SUM) r += x;
        if (op == UGPU_RED_ASUM) r += std::abs(x);
        if (op == UGPU_RED_MIN) r = std::min(r, x);
        if (op == UGPU_RED_MAX) r = std::max(r, x);
        if (op == UGPU_RED_AMAX) r = std::max(r, std::abs(x));
    }
    *out = v->v.empty() ? 0.0 : r;
    return 0;
}
int ugpu_vec_transform(ugpu_vec *v, int op, double p) {
    for (double &x : v->v) {
        switch (op) {
            case UGPU_TR_SQRT: x = std::sqrt(x); break;
            case UGPU_TR_POW2: x = x * x; break;
            case UGPU_TR_LOG: x = std::log(x); break;
            case UGPU_TR_EXP: x = std::exp(x); break;
            case UGPU_TR_COS: x = std::cos(x); break;
            case UGPU_TR_SIN: x = std::sin(x); break;
            case UGPU_TR_ABS: x = std::abs(x); break;
            case UGPU_TR_MINUS: x = -x; break;
            case UGPU_TR_POW: x = std::pow(x, p); break;
            case UGPU_TR_RECIPROCAL: x = p / x; break;
            case UGPU_TR_SHIFT: x = x + p; break;
            default: x = x * p; break;
        }
    }
    return 0;
}

int ugpu_csr_create(ugpu_ctx *, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t *rowptr,
                    const int32_t *colidx, const double *values, ugpu_mat **out) {
    auto *A = new ugpu_mat;
    A->m = nrows;
    A->n = ncols;
    A->rp.assign(rowptr, rowptr + nrows + 1);
    A->ci.assign(colidx, colidx + nnz);
    A->v.assign(values, values + nnz);
    *out = A;
    return 0;
}
int ugpu_mat_destroy(ugpu_mat *A) {
    delete A;
    return 0;
}
int ugpu_mat_info(const ugpu_mat *A, int64_t *nrows, int64_t *ncols, int64_t *nnz, int *value_dtype) {
    *nrows = A->m;
    *ncols = A->n;
    *nnz = int64_t(A->ci.size());
    *value_dtype = UGPU_F64;
    return 0;
}
int ugpu_csr_download(const ugpu_mat *A, int32_t *rowptr, int32_t *colidx, double *values) {
    std::copy(A->rp.begin(), A->rp.end(), rowptr);
    std::copy(A->ci.begin(), A->ci.end(), colidx);
    std::copy(A->v.begin(), A->v.end(), values);
    return 0;
}
int ugpu_mat_update_values(ugpu_mat *A, const double *values) {
    std::copy(values, values + A->v.size(), A->v.begin());
    return 0;
}
int ugpu_spmv(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y) {
    matvec(*A, x->v, y->v);
    return 0;
}
int ugpu_spmv_add(const ugpu_mat *A, const ugpu_vec *x, const ugpu_vec *v, ugpu_vec *y) {
    std::vector<double> t;
    matvec(*A, x->v, t);
    for (size_t i = 0; i < t.size(); ++i) t[i] = v->v[i] + t[i];
    y->v.swap(t);
    return 0;
}
int ugpu_residual(const ugpu_mat *A, const ugpu_vec *b, const ugpu_vec *x, ugpu_vec *r) {
    std::vector<double> t;
    matvec(*A, x->v, t);
    for (size_t i = 0; i < t.size(); ++i) t[i] = b->v[i] - t[i];
    r->v.swap(t);
    return 0;
}
int ugpu_diag(const ugpu_mat *A, ugpu_vec *d) {
    std::fill(d->v.begin(), d->v.end(), 0.0);
    for (int64_t i = 0; i < A->m; ++i)
        for (int32_t k = A->rp[size_t(i)]; k < A->rp[size_t(i) + 1]; ++k)
            if (A->ci[size_t(k)] == i) d->v[size_t(i)] = A->v[size_t(k)];
    return 0;
}
int ugpu_transpose(const ugpu_mat *A, ugpu_mat **out) {
    *out = new ugpu_mat(transpose(*A));
    return 0;
}
int ugpu_spgemm(const ugpu_mat *A, const ugpu_mat *B, ugpu_mat **out) {
    *out = new ugpu_mat(spgemm(*A, *B));
    return 0;
}
int ugpu_ptap(const ugpu_mat *A, const ugpu_mat *P, ugpu_mat **out) {
    const ugpu_mat R = transpose(*P);
    *out = new ugpu_mat(spgemm(R, spgemm(*A, *P)));
    return 0;
}
int ugpu_petsc_write_mat(const ugpu_mat *, const char *) { return fail("not provided"); }

// dense Cholesky (the only solver kind the backend header creates)
int ugpu_solver_create(ugpu_ctx *, int kind, ugpu_solver **out) {
    if (kind != UGPU_SOLVER_CHOLESKY) return fail("only the Cholesky solver is provided");
    *out = new ugpu_solver;
    return 0;
}
int ugpu_solver_destroy(ugpu_solver *s) {
    delete s;
    return 0;
}
int ugpu_solver_update(ugpu_solver *s, const ugpu_mat *A) {
    const int64_t n = A->m;
    s->n = n;
    s->L.assign(size_t(n * n), 0.0);
    std::vector<double> &L = s->L;
    for (int64_t i = 0; i < n; ++i)
        for (int32_t k = A->rp[size_t(i)]; k < A->rp[size_t(i) + 1]; ++k) L[size_t(i * n + A->ci[size_t(k)])] = A->v[size_t(k)];
    for (int64_t j = 0; j < n; ++j) {
        double d = L[size_t(j * n + j)];
        for (int64_t k = 0; k < j; ++k) d -= L[size_t(j * n + k)] * L[size_t(j * n + k)];
        if (!(d > 0.0)) return fail("not SPD");
        const double ljj = std::sqrt(d);
        L[size_t(j * n + j)] = ljj;
        for (int64_t i = j + 1; i < n; ++i) {
            double t = L[size_t(i * n + j)];
            for (int64_t k = 0; k < j; ++k) t -= L[size_t(i * n + k)] * L[size_t(j * n + k)];
            L[size_t(i * n + j)] = t / ljj;
        }
    }
    return 0;
}
int ugpu_solver_apply(ugpu_solver *s, const ugpu_vec *rhs, ugpu_vec *x) {
    const int64_t n = s->n;
    const std::vector<double> &L = s->L;
    std::vector<double> y(static_cast<size_t>(n), 0.0);
    for (int64_t i = 0; i < n; ++i) {
        double t = rhs->v[size_t(i)];
        for (int64_t k = 0; k < i; ++k) t -= L[size_t(i * n + k)] * y[size_t(k)];
        y[size_t(i)] = t / L[size_t(i * n + i)];
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        double t = y[size_t(i)];
        for (int64_t k = i + 1; k < n; ++k) t -= L[size_t(k * n + i)] * x->v[size_t(k)];
        x->v[size_t(i)] = t / L[size_t(i * n + i)];
    }
    return 0;
}

}  // extern "C"
