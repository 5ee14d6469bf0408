// Conjugate gradient on the GPU with device-resident scalars.
//
// Mirrors ConjugateGradient::preconditioned_solve / unpreconditioned_solve
// (utopia/solvers/smoothers/utopia_ConjugateGradient_impl.hpp:90-294) and adds the
// flexible form (Notay's FCG(1): alpha = (p,r)/(p,Ap), beta = -(z,Ap)/(p,Ap)) used as
// the FP64 outer iteration of the mixed-precision multigrid preconditioner.
//
// The reference evaluates alpha, beta and the stopping test on the host after every
// dot.  Here the dots finish in the last CTA of the kernel that produces them, the
// scalars live in device memory, and a device flag stops every later kernel of the
// iteration.  The host launches a CUDA graph of `graph_batch` iterations and reads the
// flag once per batch, so the iteration count and the stopping iterate are exactly
// those of the per-iteration loop.
//
// Per iteration (Jacobi preconditioner): 2 kernels
//   K1  p = z + beta p ; Ap = A p ; (p,Ap)                       [SpMV, fused]
//   K2  alpha ; x += alpha p ; r -= alpha Ap ; ||r|| ; z = D^+ r ; (z,r) ; beta ; stop test
// With a multigrid preconditioner: K1, K2 (without z), the V-cycle, and
//   K3  (z,r) [and (z,Ap)] ; beta ; max_it test
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

struct CgDev {
    double rz;      // (r, z) of the current iterate
    double pAp;     // (p, Ap)
    double pr;      // (p, r)            (flexible form)
    double beta;
    double rnorm;
    double alpha;
    double gnorm;   // ||r|| at the stop
    long long it;   // the reference's `it`
    long long iterates;
    int done;
    int reason;
    int converged;
    int pad;
};

namespace {

enum CgMode : int { CG_PLAIN = 0, CG_JACOBI = 1, CG_GENERIC = 2 };

__device__ __forceinline__ void cg_stop(CgDev *d, int reason, int converged) {
    d->done = 1;
    d->reason = reason;
    d->converged = converged;
    d->iterates = d->it;
    d->gnorm = d->rnorm;
}

// K2: alpha, x/r update, ||r||^2 [, z = dinv .* r, (z,r)] [, r32 = (float) r]
template <int MODE, bool R32>
__global__ void __launch_bounds__(kBlock) k_cg_update(int64_t n, double *__restrict__ x, const double *__restrict__ p,
                                                      double *__restrict__ r, const double *__restrict__ Ap,
                                                      const double *__restrict__ dinv, double *__restrict__ z,
                                                      float *__restrict__ r32, CgDev *dev, double *partials,
                                                      unsigned int *counter, double atol, long long max_it,
                                                      int flexible) {
    if (dev->done) return;
    if (MODE == CG_PLAIN && dev->pAp == 0.0) {
        // `if (dot_pq == 0.) { converged = true; break; }`
        if (blockIdx.x == 0 && threadIdx.x == 0) cg_stop(dev, UGPU_CONVERGED_FNORM_ABS, 1);
        return;
    }
    const double num = flexible ? dev->pr : dev->rz;
    const double alpha = num / dev->pAp;
    if (isinf(alpha) || isnan(alpha)) {
        // `if (std::isinf(alpha) || std::isnan(alpha)) { stop = check_convergence(...); break; }`
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            bool conv = dev->rnorm <= atol || dev->it >= max_it;
            cg_stop(dev, conv ? (dev->rnorm <= atol ? UGPU_CONVERGED_FNORM_ABS : UGPU_DIVERGED_MAX_IT)
                              : UGPU_DIVERGED_NAN,
                    dev->rnorm <= atol);
        }
        return;
    }
    double a0 = 0.0, a1 = 0.0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        x[i] = x[i] + alpha * p[i];
        double ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        a0 = fma(ri, ri, a0);
        if constexpr (MODE == CG_JACOBI) {
            double zi = dinv[i] * ri;
            z[i] = zi;
            a1 = fma(zi, ri, a1);
        }
        if constexpr (R32) r32[i] = float(ri);
    }
    double acc[2] = {a0, a1};
    const int nd = (MODE == CG_JACOBI) ? 2 : 1;
    block_reduce_store<2>(acc, nd, partials, gridDim.x, blockIdx.x);
    double sums[2];
    if (finish_last_block(nd, partials, gridDim.x, sums, counter) && threadIdx.x == 0) {
        const double rnorm = sqrt(sums[0]);
        dev->rnorm = rnorm;
        dev->alpha = alpha;
        if constexpr (MODE == CG_PLAIN) {
            // rho_1 = rho; r_norm = norm2(r); converged = check_convergence(it, r_norm, 1, 1); it++;
            // next: rho = dot(r, r); if (rho == 0) converged; beta = rho / rho_1
            const bool conv = rnorm <= atol || dev->it >= max_it;
            if (conv) {
                cg_stop(dev, rnorm <= atol ? UGPU_CONVERGED_FNORM_ABS : UGPU_DIVERGED_MAX_IT, 1);
            } else {
                dev->it += 1;
                if (sums[0] == 0.0) {
                    cg_stop(dev, UGPU_CONVERGED_FNORM_ABS, 1);
                } else {
                    dev->beta = sums[0] / dev->rz;
                    dev->rz = sums[0];
                }
            }
        } else {
            if (rnorm <= atol) {
                cg_stop(dev, UGPU_CONVERGED_FNORM_ABS, 1);
            } else if constexpr (MODE == CG_JACOBI) {
                dev->beta = sums[1] / dev->rz;
                dev->rz = sums[1];
                if (dev->it >= max_it) cg_stop(dev, UGPU_DIVERGED_MAX_IT, 0);
                else dev->it += 1;
            }
        }
    }
}

// K3: (z, r) [and (z, Ap)] of the preconditioned residual; z may arrive in FP32
// (mixed form) and is then widened into z64 for the next direction update.
template <class ZT>
__global__ void __launch_bounds__(kBlock) k_cg_zdots(int64_t n, const ZT *__restrict__ zin, double *__restrict__ z64,
                                                     const double *__restrict__ r, const double *__restrict__ q,
                                                     CgDev *dev, double *partials, unsigned int *counter,
                                                     long long max_it, int flexible) {
    if (dev->done) return;
    double a0 = 0.0, a1 = 0.0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double zi = double(zin[i]);
        if constexpr (!std::is_same<ZT, double>::value) z64[i] = zi;
        a0 = fma(zi, r[i], a0);
        if (flexible) a1 = fma(zi, q[i], a1);
    }
    double acc[2] = {a0, a1};
    const int nd = flexible ? 2 : 1;
    block_reduce_store<2>(acc, nd, partials, gridDim.x, blockIdx.x);
    double sums[2];
    if (finish_last_block(nd, partials, gridDim.x, sums, counter) && threadIdx.x == 0) {
        if (flexible) {
            dev->beta = -sums[1] / dev->pAp;
        } else {
            dev->beta = sums[0] / dev->rz;
        }
        dev->rz = sums[0];
        if (dev->it >= max_it) cg_stop(dev, UGPU_DIVERGED_MAX_IT, 0);
        else dev->it += 1;
    }
}

__global__ void k_cg_init(CgDev *dev, double rz, double rnorm, long long it0) {
    dev->rz = rz;
    dev->pAp = 0;
    dev->pr = 0;
    dev->beta = 0;
    dev->rnorm = rnorm;
    dev->alpha = 0;
    dev->gnorm = rnorm;
    dev->it = it0;
    dev->iterates = it0;
    dev->done = 0;
    dev->reason = 0;
    dev->converged = 0;
}

}  // namespace

// InvDiagPreconditioner (utopia/solvers/preconditioners/utopia_TrivialPreconditioners.hpp:20-56):
// d = e_pseudo_inv(diag(A)) with tol = machine epsilon; apply: z = d .* r
class InvDiag final : public Solver {
public:
    explicit InvDiag(Context *c) : Solver(c, UGPU_SOLVER_INVDIAG) {}
    Buffer d;
    void update(const Mat *A) override {
        op = A;
        Mat &M = const_cast<Mat &>(*A);
        ensure_diag(M);
        d.alloc(sizeof(double) * std::max<int64_t>(A->nrows, 1));
        Vec din, dout;
        din.ctx = dout.ctx = ctx;
        din.n = dout.n = A->nrows;
        din.buf.borrow(M.diag.ptr, M.diag.bytes);
        dout.buf.borrow(d.ptr, d.bytes);
        launch_pseudo_inverse(*ctx, din, dout, std::numeric_limits<double>::epsilon());
    }
    void apply(const Vec &b, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "update() first");
        UGPU_CHECK(b.dtype == UGPU_F64 && x.dtype == UGPU_F64 && b.n == op->nrows && x.n == op->nrows, UGPU_ERR_ARG,
                   "InvDiag: FP64 vectors of the operator size");
        enq_scale_into(*ctx, UGPU_F64, b.n, d.ptr, b.data(), x.data(), nullptr);
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    void pc_enqueue(const void *r, void *z, const int *done) override {
        enq_scale_into(*ctx, UGPU_F64, op->nrows, d.ptr, r, z, done);
    }
};

class ConjugateGradient final : public Solver {
public:
    explicit ConjugateGradient(Context *c) : Solver(c, UGPU_SOLVER_CG) {
        prm["reset_initial_guess"] = 0;
        prm["flexible"] = 0;
        prm["graph_batch"] = 8;
        prm["use_graphs"] = 1;
        prm["format"] = -1;  // -1: the matrix's own SpMV layout
    }
    ~ConjugateGradient() override { drop_graph(); }

    void set_preconditioner(Solver *p) override {
        pc_ = p;
        drop_graph();
    }

    void set(const std::string &k, double v) override {
        Solver::set(k, v);
        drop_graph();
    }

    // PreconditionedSolver::update propagates the operator to the preconditioner
    // (utopia/solvers/linear/utopia_PreconditionedSolver.hpp:37-46)
    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG, "CG: square FP64 operator");
        op = A;
        if (pc_) pc_->update(A);
        const int64_t n = A->nrows;
        const size_t b = sizeof(double) * std::max<int64_t>(n, 1);
        r_.alloc(b);
        z_.alloc(b);
        p_[0].alloc(b);
        p_[1].alloc(b);
        Ap_.alloc(b);
        r32_.release();
        z32_.release();
        if (pc_ && pc_->pc_dtype() == UGPU_F32) {
            r32_.alloc(sizeof(float) * std::max<int64_t>(n, 1));
            z32_.alloc(sizeof(float) * std::max<int64_t>(n, 1));
        }
        dev_.alloc(sizeof(CgDev));
        part_.alloc(sizeof(double) * 6 * std::max(kSpmvDotGrid, kRedBlocks));  // 3 regions x 2 dots
        cnt_.alloc(sizeof(unsigned int) * 8);
        UGPU_CUDA(cudaMemsetAsync(cnt_.ptr, 0, cnt_.bytes, ctx->stream));
        if (!host_dev_) UGPU_CUDA(cudaMallocHost(&host_dev_, sizeof(CgDev)));
        drop_graph();
    }

    void apply(const Vec &b, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "CG: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(b.dtype == UGPU_F64 && x.dtype == UGPU_F64 && b.n == n && x.n == n, UGPU_ERR_ARG,
                   "CG: FP64 vectors of the operator size");
        double t0 = now_s();
        int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        if (get("reset_initial_guess") != 0) enq_set(*ctx, UGPU_F64, n, 0.0, x.data(), nullptr);
        mode_ = !pc_ ? CG_PLAIN : (dynamic_cast<InvDiag *>(pc_) ? CG_JACOBI : CG_GENERIC);
        flexible_ = get("flexible") != 0 && mode_ != CG_PLAIN;
        // r = b - A x
        {
            SpmvArgs a;
            a.x = x.data();
            a.v = b.data();
            a.y = r_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_RESIDUAL;
            launch_spmv(*ctx, *op, a);
        }
        // z = M r (z = r for the unpreconditioned form); rz = (r, z)
        double rz = 0.0, rr = 0.0;
        if (mode_ == CG_PLAIN) {
            enq_copy(*ctx, UGPU_F64, n, r_.ptr, z_.ptr, nullptr);
        } else {
            precondition(nullptr);
        }
        {
            DotArgs d{};
            d.nd = 2;
            d.a[0] = r_.ptr;
            d.b[0] = z_.ptr;
            d.a[1] = r_.ptr;
            d.b[1] = r_.ptr;
            d.dtype_a[0] = d.dtype_b[0] = d.dtype_a[1] = d.dtype_b[1] = UGPU_F64;
            double out[2];
            host_dots(*ctx, n, d, out);
            rz = out[0];
            rr = out[1];
        }
        // unpreconditioned form starts with r_norm = norm2(r); the preconditioned one with 9e9
        const double rnorm0 = (mode_ == CG_PLAIN) ? std::sqrt(rr) : 9e9;
        UGPU_CUDA(cudaMemsetAsync(p_[0].ptr, 0, p_[0].bytes, ctx->stream));
        UGPU_CUDA(cudaMemsetAsync(p_[1].ptr, 0, p_[1].bytes, ctx->stream));
        // the unpreconditioned loop starts at it = 1 (utopia_ConjugateGradient_impl.hpp:128)
        k_cg_init<<<1, 1, 0, ctx->stream>>>(dev_.as<CgDev>(), rz, rnorm0, mode_ == CG_PLAIN ? 1 : 0);
        ctx->launches++;
        if (mode_ == CG_PLAIN && rr == 0.0) {
            // `rho = dot(r, r); if (rho == 0.) { converged = true; break; }`
            finish(x, t0, l0, /*done_now=*/true, rnorm0);
            return;
        }
        const int64_t max_it = int64_t(get("max_it"));
        const bool graphs = get("use_graphs") != 0;
        int batch = std::max(2, int(get("graph_batch")));
        batch += batch & 1;  // even: the direction buffers alternate per iteration
        int64_t launched = 0;
        const int64_t limit = max_it + 2 * batch + 2;
        while (true) {
            if (graphs) {
                ensure_graph(batch, x.data());
                UGPU_CUDA(cudaGraphLaunch(exec_, ctx->stream));
                ctx->launches += graph_kernels_;
            } else {
                for (int k = 0; k < batch; ++k) iteration(k & 1, x.data());
            }
            launched += batch;
            UGPU_CUDA(cudaMemcpyAsync(host_dev_, dev_.ptr, sizeof(CgDev), cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
            if (host_dev_->done) break;
            UGPU_CHECK(launched <= limit, UGPU_ERR_INTERNAL, "CG: stop flag never set");
        }
        finish(x, t0, l0, false, 0);
    }

private:
    Solver *pc_ = nullptr;
    int mode_ = CG_PLAIN;
    bool flexible_ = false;
    Buffer r_, z_, p_[2], Ap_, r32_, z32_, dev_, part_, cnt_;
    CgDev *host_dev_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int graph_batch_ = 0;
    int64_t graph_kernels_ = 0;
    const void *graph_x_ = nullptr;

    void drop_graph() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
        exec_ = nullptr;
        graph_ = nullptr;
        graph_batch_ = 0;
    }

    void ensure_graph(int batch, void *x) {
        if (exec_ && graph_batch_ == batch && graph_x_ == x) return;
        drop_graph();
        int64_t l0 = ctx->launches;
        UGPU_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        try {
            for (int k = 0; k < batch; ++k) iteration(k & 1, x);
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(ctx->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        UGPU_CUDA(cudaStreamEndCapture(ctx->stream, &graph_));
        UGPU_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
        graph_kernels_ = ctx->launches - l0;
        ctx->launches = l0;
        graph_batch_ = batch;
        graph_x_ = x;
    }

    void precondition(const int *done) {
        const int64_t n = op->nrows;
        if (pc_->pc_dtype() == UGPU_F32) {
            pc_->pc_enqueue(r32_.ptr ? (done ? r32_.ptr : to32(n)) : nullptr, z32_.ptr, done);
            if (!done) enq_convert(*ctx, UGPU_F32, z32_.ptr, UGPU_F64, z_.ptr, n, nullptr);
        } else {
            pc_->pc_enqueue(r_.ptr, z_.ptr, done);
        }
    }

    void *to32(int64_t n) {
        enq_convert(*ctx, UGPU_F64, r_.ptr, UGPU_F32, r32_.ptr, n, nullptr);
        return r32_.ptr;
    }

    // one iteration; `par` selects which direction buffer holds the previous p
    void iteration(int par, void *x) {
        const int64_t n = op->nrows;
        CgDev *dev = dev_.as<CgDev>();
        const int *done = &dev->done;
        double *pin = p_[par].as<double>(), *pout = p_[par ^ 1].as<double>();
        double *part = part_.as<double>();
        unsigned int *cnt = cnt_.as<unsigned int>();
        // K1: p = z + beta p ; Ap = A p ; (p, Ap) [, (p, r)]
        {
            SpmvArgs a;
            a.x = (mode_ == CG_PLAIN) ? r_.ptr : z_.ptr;  // plain CG: p = r + beta p
            a.p = pin;
            a.pout = pout;
            a.beta_ptr = &dev->beta;
            a.y = Ap_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_STORE;
            a.dot_partials = part;
            a.dot_out = &dev->pAp;
            a.dot_counter = cnt + 0;
            if (flexible_) a.dv = r_.ptr;
            a.done = done;
            launch_spmv(*ctx, *op, a);
        }
        // K2
        {
            const bool r32 = mode_ == CG_GENERIC && pc_->pc_dtype() == UGPU_F32;
            const double atol = get("atol");
            const long long max_it = (long long)get("max_it");
            const int g = reduce_grid(n);
            const double *dinv = (mode_ == CG_JACOBI) ? static_cast<InvDiag *>(pc_)->d.as<double>() : nullptr;
#define UGPU_CG_UPD(M, R)                                                                                          \
    k_cg_update<M, R><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<double *>(x), pout, r_.as<double>(),             \
                                                     Ap_.as<double>(), dinv, z_.as<double>(), r32_.as<float>(), dev,  \
                                                     part + 2 * kSpmvDotGrid, cnt + 1, atol, max_it, int(flexible_))
            if (mode_ == CG_PLAIN) UGPU_CG_UPD(CG_PLAIN, false);
            else if (mode_ == CG_JACOBI) UGPU_CG_UPD(CG_JACOBI, false);
            else if (r32) UGPU_CG_UPD(CG_GENERIC, true);
            else UGPU_CG_UPD(CG_GENERIC, false);
#undef UGPU_CG_UPD
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
        }
        if (mode_ == CG_PLAIN || mode_ == CG_JACOBI) return;
        // z = M r, then K3
        const bool f32 = pc_->pc_dtype() == UGPU_F32;
        pc_->pc_enqueue(f32 ? r32_.ptr : r_.ptr, f32 ? z32_.ptr : z_.ptr, done);
        const int g = reduce_grid(n);
        const long long max_it = (long long)get("max_it");
        if (f32)
            k_cg_zdots<float><<<g, kBlock, 0, ctx->stream>>>(n, z32_.as<float>(), z_.as<double>(), r_.as<double>(),
                                                             Ap_.as<double>(), dev, part + 4 * kSpmvDotGrid, cnt + 2,
                                                             max_it, int(flexible_));
        else
            k_cg_zdots<double><<<g, kBlock, 0, ctx->stream>>>(n, z_.as<double>(), nullptr, r_.as<double>(),
                                                              Ap_.as<double>(), dev, part + 4 * kSpmvDotGrid, cnt + 2,
                                                              max_it, int(flexible_));
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
    }

    void finish(Vec &x, double t0, int64_t l0, bool done_now, double rnorm0) {
        (void)x;
        if (done_now) {
            st.iterates = 0;
            st.gradient_norm = rnorm0;
            st.reason = UGPU_CONVERGED_FNORM_ABS;
            st.converged = 1;
        } else {
            st.iterates = host_dev_->iterates;
            st.gradient_norm = host_dev_->gnorm;
            st.reason = host_dev_->reason;
            st.converged = host_dev_->converged;
        }
        st.relative_gradient_norm = 1;
        st.step_norm = 1;
        st.spmv_count = st.iterates + 2;
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }
};

std::unique_ptr<Solver> make_cg(Context *c) { return std::make_unique<ConjugateGradient>(c); }
std::unique_ptr<Solver> make_invdiag(Context *c) { return std::make_unique<InvDiag>(c); }

}  // namespace ugpu
