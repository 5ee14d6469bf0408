// BiCGStab (utopia/solvers/smoothers/utopia_BiCGStab_impl.hpp:44-250), preconditioned and
// unpreconditioned, on the GPU.
//
// The reference's loop branches on its dots every iteration (breakdown tests, omega, the norm
// checks); here each dot is one fixed-order device reduction read back by the host, and the
// vector updates of an iteration are fused into three kernels:
//   p = r + beta (p - omega v);   h = x + alpha q, s = r - alpha v;   x = h + omega z, r = s - omega t
// (q = y = M p for the preconditioned form, q = p otherwise; z = M s or s).  The operation order
// per element follows the reference expressions.  FP64 throughout; a preconditioner must work in
// FP64 vectors.
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {

__global__ void k_bicg_p(int64_t n, const double *__restrict__ r, const double *__restrict__ v, double beta,
                         double omega, double *__restrict__ p) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        p[i] = r[i] + beta * (p[i] - omega * v[i]);
}

__global__ void k_bicg_hs(int64_t n, const double *__restrict__ x, const double *__restrict__ q,
                          const double *__restrict__ r, const double *__restrict__ v, double alpha,
                          double *__restrict__ h, double *__restrict__ s) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        h[i] = x[i] + alpha * q[i];
        s[i] = r[i] - alpha * v[i];
    }
}

__global__ void k_bicg_xr(int64_t n, const double *__restrict__ h, const double *__restrict__ z,
                          const double *__restrict__ s, const double *__restrict__ t, double omega,
                          double *__restrict__ x, double *__restrict__ r) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        x[i] = h[i] + omega * z[i];
        r[i] = s[i] - omega * t[i];
    }
}

}  // namespace

class BiCGStab final : public Solver {
public:
    explicit BiCGStab(Context *c) : Solver(c, UGPU_SOLVER_BICGSTAB) {}

    void set_preconditioner(Solver *p) override {
        UGPU_CHECK(!p || p->pc_dtype() == UGPU_F64, UGPU_ERR_UNSUPPORTED,
                   "BiCGStab: the preconditioner must work in FP64");
        pc_ = p;
    }

    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols, UGPU_ERR_ARG, "BiCGStab: square operator required");
        op = A;
        if (pc_) pc_->update(A);
        const size_t b = sizeof(double) * size_t(std::max<int64_t>(A->nrows, 1));
        for (Buffer *w : {&r_, &r0_, &p_, &v_, &h_, &y_, &s_, &t_, &z_, &kt_}) w->alloc(b);
    }

    void apply(const Vec &b, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "BiCGStab: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(b.n == n && x.n == n && b.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "BiCGStab: FP64 vectors of the operator's size required");
        if (pc_) UGPU_CHECK(pc_->pc_dtype() == UGPU_F64, UGPU_ERR_UNSUPPORTED, "BiCGStab: FP64 preconditioner");
        const double t0 = now_s();
        const int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        double *X = x.as<double>();
        const double *B = b.as<double>();
        double *r = r_.as<double>(), *r0 = r0_.as<double>(), *p = p_.as<double>(), *v = v_.as<double>();
        double *h = h_.as<double>(), *y = y_.as<double>(), *s = s_.as<double>(), *t = t_.as<double>();
        double *z = z_.as<double>(), *kt = kt_.as<double>();
        const int g = stream_grid(*ctx, n);
        int64_t spmvs = 0;
        auto spmv = [&](const double *in, double *out) {
            SpmvArgs a;
            a.x = in;
            a.y = out;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_STORE;
            launch_spmv(*ctx, *op, a);
            ++spmvs;
        };
        auto dots = [&](std::initializer_list<std::pair<const double *, const double *>> pairs, double *out) {
            DotArgs d{};
            int k = 0;
            for (auto &pr : pairs) {
                d.a[k] = pr.first;
                d.b[k] = pr.second;
                d.dtype_a[k] = d.dtype_b[k] = UGPU_F64;
                ++k;
            }
            d.nd = k;
            host_dots(*ctx, n, d, out);
        };
        // z = M in, from a zero initial guess (as the preconditioner of CG)
        auto precond = [&](const double *in, double *out) { pc_->pc_enqueue(in, out, nullptr); };
        // p and v start at zero (init_memory, utopia_BiCGStab_impl.hpp:27-38)
        enq_set(*ctx, UGPU_F64, n, 0.0, p, nullptr);
        enq_set(*ctx, UGPU_F64, n, 0.0, v, nullptr);
        double rho = 1, rho_old = 1, alpha = 1, omega = 1, beta = 1;
        // r = b - A x; r0 = r
        {
            SpmvArgs a;
            a.x = X;
            a.v = B;
            a.y = r;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_RESIDUAL;
            launch_spmv(*ctx, *op, a);
            ++spmvs;
            enq_copy(*ctx, UGPU_F64, n, r, r0, nullptr);
        }
        int64_t it = 0;
        bool converged = false;
        double r_norm = 1e10, out[2];
        while (!converged) {
            dots({{r0, r}}, out);
            rho = out[0];
            if (!pc_ && rho == 0.) {  // unpreconditioned form: `if (rho == 0.) { converged = true; break; }`
                converged = true;
                break;
            }
            beta = (rho / rho_old) * (alpha / omega);
            k_bicg_p<<<g, kBlock, 0, ctx->stream>>>(n, r, v, beta, omega, p);
            ctx->launches++;
            const double *q = p;
            if (pc_) {
                precond(p, y);
                q = y;
            }
            spmv(q, v);
            dots({{r0, v}}, out);
            const double r0v = out[0];
            if (pc_ && r0v == 0.0) {  // preconditioned breakdown branch: residual of x and a norm of s
                SpmvArgs a;
                a.x = X;
                a.v = B;
                a.y = r;
                a.vec_dtype = UGPU_F64;
                a.epilogue = EPI_RESIDUAL;
                launch_spmv(*ctx, *op, a);
                ++spmvs;
                dots({{s, s}}, out);
                r_norm = std::sqrt(out[0]);
                converged = check_convergence(it, r_norm, 1, 1);
                break;
            }
            alpha = rho / r0v;
            k_bicg_hs<<<g, kBlock, 0, ctx->stream>>>(n, X, q, r, v, alpha, h, s);
            ctx->launches++;
            if (pc_) {
                dots({{s, s}}, out);
                r_norm = std::sqrt(out[0]);
                converged = check_convergence(it, r_norm, 1, 1);
                if (converged) {
                    // ||s|| met the test: return h = x + alpha y, the iterate s belongs to (the
                    // reference breaks here leaving x one half-step behind)
                    enq_copy(*ctx, UGPU_F64, n, h, X, nullptr);
                    break;
                }
            }
            const double *zz = s;
            if (pc_) {
                precond(s, z);
                zz = z;
            }
            spmv(zz, t);
            if (pc_) {
                precond(t, kt);
                dots({{z, kt}, {kt, kt}}, out);
            } else {
                dots({{t, s}, {t, t}}, out);
            }
            omega = out[0] / out[1];
            if (std::isnan(omega) || (!pc_ && std::isinf(omega))) {
                if (!pc_) {
                    dots({{s, s}}, out);
                    r_norm = std::sqrt(out[0]);
                    converged = check_convergence(it, r_norm, 1, 1);
                }
                break;
            }
            k_bicg_xr<<<g, kBlock, 0, ctx->stream>>>(n, h, zz, s, t, omega, X, r);
            ctx->launches++;
            rho_old = rho;
            dots({{r, r}}, out);
            r_norm = std::sqrt(out[0]);
            converged = check_convergence(it, r_norm, 1, 1);
            it++;
        }
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        if (st.reason == 0) {  // left by a breakdown (rho == 0 or a NaN omega), not by check_convergence
            st.iterates = it;
            st.gradient_norm = r_norm;
            if (converged) st.reason = UGPU_CONVERGED_FNORM_ABS;
            else if (std::isnan(omega)) st.reason = UGPU_DIVERGED_NAN;
        }
        st.converged = st.reason > 0 ? 1 : 0;
        st.spmv_count = spmvs;
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

private:
    Solver *pc_ = nullptr;
    Buffer r_, r0_, p_, v_, h_, y_, s_, t_, z_, kt_;
};

std::unique_ptr<Solver> make_bicgstab(Context *c) { return std::make_unique<BiCGStab>(c); }

}  // namespace ugpu
