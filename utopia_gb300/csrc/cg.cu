// Conjugate gradient on the GPU with device-resident scalars.
//
// Mirrors ConjugateGradient::preconditioned_solve / unpreconditioned_solve
// (utopia/solvers/smoothers/utopia_ConjugateGradient_impl.hpp:90-294) and adds the
// flexible form (Notay's FCG(1): alpha = (p,r)/(p,Ap), beta = -(z,Ap)/(p,Ap)) used as
// the FP64 outer iteration of the mixed-precision multigrid preconditioner; (p,r) follows
// the scalar recurrence (p',r') = (z,r') + beta ((p,r) - alpha (p,Ap)) instead of a dot.
//
// The reference evaluates alpha, beta and the stopping test on the host after every
// dot.  Here the dots finish in the last CTA of the kernel that produces them, the
// scalars live in device memory, and a device flag stops every later kernel.  The
// whole solve is one CUDA graph launch: a conditional WHILE node re-runs the captured
// iteration until the flag is set (use_graphs = 0 runs the same kernels eagerly with a
// host check after every iteration), so the iteration count and the stopping iterate
// are exactly those of the per-iteration loop.
//
// Per iteration (Jacobi preconditioner): 3 kernels
//   K0  p = z + beta p
//   K1  Ap = A p ; (p,Ap)                                          [SpMV + last-CTA dot]
//   K2  alpha ; x += alpha p ; r -= alpha Ap ; ||r|| ; z = D^+ r ; (z,r) ; beta ; stop test
// With a multigrid preconditioner: K0, K1, K2 (without z), the V-cycle, and
//   K3  (z,r) [and (z,Ap)] ; beta ; max_it test
// Where the V-cycle ends in a Jacobi / PointJacobi sweep and fold_dots = 1, that sweep computes
// (z,r) [and (z,Ap)] as it writes z, and K3 shrinks to one thread that closes the iteration: z
// is not read back.  Off by default: measured at 192^3 (mixed form), the BF16 sweep with the two
// FP64 dots took 96 us against 42 us without them, more than the separate K3 (48 us) it replaces.
// (K0 is not folded into the SpMV: gathering z and p per nonzero doubles the FP64 FMAs of
// the product, and FP64 FMA throughput, not HBM, then bounds it on GB300.)
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

__device__ __forceinline__ double2 ld2(const double *p, int64_t j) { return reinterpret_cast<const double2 *>(p)[j]; }
__device__ __forceinline__ void st2(double *p, int64_t j, double2 v) { reinterpret_cast<double2 *>(p)[j] = v; }
inline bool al16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

__device__ __forceinline__ void cg_stop(CgDev *d, int reason, int converged) {
    d->done = 1;
    d->reason = reason;
    d->converged = converged;
    d->iterates = d->it;
    d->gnorm = d->rnorm;
}

// K2: alpha, x/r update, ||r||^2 [, z = dinv .* r, (z,r)] [, r32 = (float) r] [, x1 = pw .* r (in the
// preconditioner's precision: its first Jacobi iterate, pc_prescale)]
template <int MODE, bool R32>
__global__ void __launch_bounds__(kBlock) k_cg_update(int64_t n, double *__restrict__ x, const double *__restrict__ p,
                                                      double *__restrict__ r, const double *__restrict__ Ap,
                                                      const double *__restrict__ dinv, double *__restrict__ z,
                                                      float *__restrict__ r32, const void *__restrict__ pw,
                                                      void *__restrict__ px1, CgDev *dev, double *partials,
                                                      unsigned int *counter, double atol, long long max_it,
                                                      int flexible, int vec) {
    using PT = typename std::conditional<R32, float, double>::type;
    const PT *w1 = static_cast<const PT *>(pw);
    PT *x1 = static_cast<PT *>(px1);
    if (dev->done) return;
    if (MODE == CG_PLAIN && dev->pAp == 0.0) {
        // `if (dot_pq == 0.) { converged = true; break; }`
        if (blockIdx.x == 0 && threadIdx.x == 0) cg_stop(dev, UGPU_CONVERGED_FNORM_ABS, 1);
        return;
    }
    // alpha from one thread per CTA (a division per thread would cost the FP64 pipe about 8
    // operations per thread)
    __shared__ double s_alpha;
    if (threadIdx.x == 0) s_alpha = (flexible ? dev->pr : dev->rz) / dev->pAp;
    __syncthreads();
    const double alpha = s_alpha;
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
    auto one = [&](int64_t i) {
        x[i] = x[i] + alpha * p[i];
        double ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        a0 = fma(ri, ri, a0);
        if constexpr (MODE == CG_JACOBI) {
            double zi = dinv[i] * ri;
            z[i] = zi;
            a1 = fma(zi, ri, a1);
        }
        if constexpr (R32) {
            const float rf = d2f_bits(ri);
            r32[i] = rf;
            if (x1) x1[i] = w1[i] * rf;
        } else {
            if (x1) x1[i] = w1[i] * ri;
        }
    };
    const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int64_t nth = int64_t(gridDim.x) * blockDim.x;
    if (vec) {
        // pairs of elements as 16-byte loads and stores
        const int64_t n2 = n >> 1;
#pragma unroll 4
        for (int64_t j = tid; j < n2; j += nth) {
            const double2 xv = ld2(x, j), pv = ld2(p, j), rv = ld2(r, j), qv = ld2(Ap, j);
            const double r0 = rv.x - alpha * qv.x, r1 = rv.y - alpha * qv.y;
            st2(x, j, make_double2(xv.x + alpha * pv.x, xv.y + alpha * pv.y));
            st2(r, j, make_double2(r0, r1));
            a0 = fma(r0, r0, a0);
            a0 = fma(r1, r1, a0);
            if constexpr (MODE == CG_JACOBI) {
                const double2 dv = ld2(dinv, j);
                const double z0 = dv.x * r0, z1 = dv.y * r1;
                st2(z, j, make_double2(z0, z1));
                a1 = fma(z0, r0, a1);
                a1 = fma(z1, r1, a1);
            }
            if constexpr (R32) {
                const float2 rf = make_float2(d2f_bits(r0), d2f_bits(r1));
                reinterpret_cast<float2 *>(r32)[j] = rf;
                if (x1) {
                    const float2 wv = reinterpret_cast<const float2 *>(w1)[j];
                    reinterpret_cast<float2 *>(x1)[j] = make_float2(wv.x * rf.x, wv.y * rf.y);
                }
            } else {
                if (x1) {
                    const double2 wv = ld2(w1, j);
                    st2(x1, j, make_double2(wv.x * r0, wv.y * r1));
                }
            }
        }
        if ((n & 1) && tid == 0) one(n - 1);
    } else {
        for (int64_t i = tid; i < n; i += nth) one(i);
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

// beta and the max_it test from sums = {(z, r) [, (z, Ap)]}
__device__ __forceinline__ void cg_zclose(CgDev *dev, const double *sums, long long max_it, int flexible) {
    if (flexible) {
        // (p_new, r) without a dot over p: p_new = z + beta p and, after r -= alpha Ap,
        // (p, r) = (p, r)_old - alpha (p, Ap)
        const double beta = -sums[1] / dev->pAp;
        dev->beta = beta;
        dev->pr = sums[0] + beta * (dev->pr - dev->alpha * dev->pAp);
    } else {
        dev->beta = sums[0] / dev->rz;
    }
    dev->rz = sums[0];
    if (dev->it >= max_it) cg_stop(dev, UGPU_DIVERGED_MAX_IT, 0);
    else dev->it += 1;
}

// K3: (z, r) [and (z, Ap)] of the preconditioned residual; z may arrive in FP32
// (mixed form).
template <class ZT>
__global__ void __launch_bounds__(kBlock) k_cg_zdots(int64_t n, const ZT *__restrict__ zin,
                                                     const double *__restrict__ r, const double *__restrict__ q,
                                                     CgDev *dev, double *partials, unsigned int *counter,
                                                     long long max_it, int flexible, int vec) {
    if (dev->done) return;
    double a0 = 0.0, a1 = 0.0;
    const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int64_t nth = int64_t(gridDim.x) * blockDim.x;
    auto one = [&](int64_t i) {
        double zi = cvt<double>(zin[i]);
        a0 = fma(zi, r[i], a0);
        if (flexible) a1 = fma(zi, q[i], a1);
    };
    if (vec) {
        const int64_t n2 = n >> 1;
#pragma unroll 4
        for (int64_t j = tid; j < n2; j += nth) {
            double z0, z1;
            if constexpr (sizeof(ZT) == 4) {
                const float2 t = reinterpret_cast<const float2 *>(zin)[j];
                z0 = f2d_bits(t.x);
                z1 = f2d_bits(t.y);
            } else {
                const double2 t = ld2(reinterpret_cast<const double *>(zin), j);
                z0 = t.x;
                z1 = t.y;
            }
            const double2 rv = ld2(r, j);
            a0 = fma(z0, rv.x, a0);
            a0 = fma(z1, rv.y, a0);
            if (flexible) {
                const double2 qv = ld2(q, j);
                a1 = fma(z0, qv.x, a1);
                a1 = fma(z1, qv.y, a1);
            }
        }
        if ((n & 1) && tid == 0) one(n - 1);
    } else {
        for (int64_t i = tid; i < n; i += nth) one(i);
    }
    double acc[2] = {a0, a1};
    const int nd = flexible ? 2 : 1;
    block_reduce_store<2>(acc, nd, partials, gridDim.x, blockIdx.x);
    double sums[2];
    if (finish_last_block(nd, partials, gridDim.x, sums, counter) && threadIdx.x == 0)
        cg_zclose(dev, sums, max_it, flexible);
}

// K3 when the preconditioner's last kernel computed (z, r) [and (z, Ap)] into sums
__global__ void k_cg_zfinish(CgDev *dev, const double *sums, long long max_it, int flexible) {
    if (dev->done) return;
    const double s[2] = {sums[0], flexible ? sums[1] : 0.0};
    cg_zclose(dev, s, max_it, flexible);
}

// K0: p = z + beta p (z in FP64 or, for the mixed form, FP32)
template <class ZT>
__global__ void __launch_bounds__(kBlock) k_cg_pupdate(int64_t n, const ZT *__restrict__ z, double *__restrict__ p,
                                                       const CgDev *dev, int vec) {
    if (dev->done) return;
    const double beta = dev->beta;
    const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int64_t nth = int64_t(gridDim.x) * blockDim.x;
    if (vec) {
        const int64_t n2 = n >> 1;
#pragma unroll 4
        for (int64_t j = tid; j < n2; j += nth) {
            double z0, z1;
            if constexpr (sizeof(ZT) == 4) {
                const float2 t = reinterpret_cast<const float2 *>(z)[j];
                z0 = f2d_bits(t.x);
                z1 = f2d_bits(t.y);
            } else {
                const double2 t = ld2(reinterpret_cast<const double *>(z), j);
                z0 = t.x;
                z1 = t.y;
            }
            const double2 pv = ld2(p, j);
            st2(p, j, make_double2(z0 + beta * pv.x, z1 + beta * pv.y));
        }
        if ((n & 1) && tid == 0) p[n - 1] = cvt<double>(z[n - 1]) + beta * p[n - 1];
    } else {
        for (int64_t i = tid; i < n; i += nth) p[i] = cvt<double>(z[i]) + beta * p[i];
    }
}

__global__ void k_cg_init(CgDev *dev, double rz, double rnorm, long long it0) {
    dev->rz = rz;
    dev->pAp = 0;
    dev->pr = rz;  // flexible form: p = z at the start, so (p, r) = (z, r)
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
        prm["use_graphs"] = 1;  // 1: the solve is one graph launch (conditional WHILE node)
        prm["fold_dots"] = 0;   // 1: the preconditioner's last kernel computes (z,r) [and (z,Ap)]
    }

    void set_preconditioner(Solver *p) override {
        pc_ = p;
        loop_.reset();
    }

    void set(const std::string &k, double v) override {
        Solver::set(k, v);
        loop_.reset();
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
        p_.alloc(b);
        Ap_.alloc(b);
        r32_.release();
        z32_.release();
        if (pc_ && pc_->pc_dtype() == UGPU_F32) {
            r32_.alloc(sizeof(float) * std::max<int64_t>(n, 1));
            z32_.alloc(sizeof(float) * std::max<int64_t>(n, 1));
        }
        dev_.alloc(sizeof(CgDev));
        // 4 regions x 2 dots: K1, K2, K3 (or the folded dots' partials), the folded dots' sums
        part_.alloc(sizeof(double) * 8 * std::max(kSpmvDotGrid, kRedBlocks));
        cnt_.alloc(sizeof(unsigned int) * 8);
        UGPU_CUDA(cudaMemsetAsync(cnt_.ptr, 0, cnt_.bytes, ctx->stream));
        if (!host_dev_) UGPU_CUDA(cudaMallocHost(&host_dev_, sizeof(CgDev)));
        loop_.reset();
    }

    ~ConjugateGradient() override {
        if (host_dev_) cudaFreeHost(host_dev_);
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
        const int mode = !pc_ ? CG_PLAIN : (dynamic_cast<InvDiag *>(pc_) ? CG_JACOBI : CG_GENERIC);
        const bool flexible = get("flexible") != 0 && mode != CG_PLAIN;
        if (mode != mode_ || flexible != flexible_) loop_.reset();
        mode_ = mode;
        flexible_ = flexible;
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
        // z = M r (the unpreconditioned form uses r itself); rz = (r, z)
        if (mode_ != CG_PLAIN) {
            if (pc_->pc_dtype() == UGPU_F32) {
                enq_convert(*ctx, UGPU_F64, r_.ptr, UGPU_F32, r32_.ptr, n, nullptr);
                pc_->pc_enqueue(r32_.ptr, z32_.ptr, nullptr);
            } else {
                pc_->pc_enqueue(r_.ptr, z_.ptr, nullptr);
            }
        }
        double rz, rr;
        {
            DotArgs d{};
            d.nd = 2;
            d.a[0] = r_.ptr;
            d.b[0] = (mode_ == CG_PLAIN) ? r_.ptr : (z32_.ptr ? z32_.ptr : z_.ptr);
            d.a[1] = r_.ptr;
            d.b[1] = r_.ptr;
            d.dtype_a[0] = d.dtype_a[1] = d.dtype_b[1] = UGPU_F64;
            d.dtype_b[0] = (mode_ != CG_PLAIN && z32_.ptr) ? UGPU_F32 : UGPU_F64;
            double out[2];
            host_dots(*ctx, n, d, out);
            rz = out[0];
            rr = out[1];
        }
        // the unpreconditioned form starts with r_norm = norm2(r); the preconditioned one with 9e9
        const double rnorm0 = (mode_ == CG_PLAIN) ? std::sqrt(rr) : 9e9;
        UGPU_CUDA(cudaMemsetAsync(p_.ptr, 0, p_.bytes, ctx->stream));  // p = z + 0 * 0 = z first
        // the unpreconditioned loop starts at it = 1 (utopia_ConjugateGradient_impl.hpp:128)
        k_cg_init<<<1, 1, 0, ctx->stream>>>(dev_.as<CgDev>(), rz, rnorm0, mode_ == CG_PLAIN ? 1 : 0);
        ctx->launches++;
        if (mode_ == CG_PLAIN && rr == 0.0) {
            // `rho = dot(r, r); if (rho == 0.) { converged = true; break; }`
            finish(t0, l0, /*done_now=*/true, rnorm0);
            return;
        }
        const int64_t max_it = int64_t(get("max_it"));
        if (get("use_graphs") != 0) {
            if (!loop_.built() || graph_x_ != x.data()) {
                loop_.build(*ctx, [&] { iteration(x.data()); }, &dev_.as<CgDev>()->done,
                            int(std::min<int64_t>(max_it + 8, 1 << 30)));
                graph_x_ = x.data();
            }
            loop_.run(*ctx);
            UGPU_CUDA(cudaMemcpyAsync(host_dev_, dev_.ptr, sizeof(CgDev), cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        } else {
            const int64_t limit = max_it + 8;
            for (int64_t k = 0;; ++k) {
                iteration(x.data());
                UGPU_CUDA(cudaMemcpyAsync(host_dev_, dev_.ptr, sizeof(CgDev), cudaMemcpyDeviceToHost, ctx->stream));
                UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
                if (host_dev_->done) break;
                UGPU_CHECK(k <= limit, UGPU_ERR_INTERNAL, "CG: stop flag never set");
            }
        }
        UGPU_CHECK(host_dev_->done, UGPU_ERR_INTERNAL, "CG: loop ended without the stop flag");
        finish(t0, l0, false, 0);
    }

private:
    Solver *pc_ = nullptr;
    int mode_ = -1;
    bool flexible_ = false;
    Buffer r_, z_, p_, Ap_, r32_, z32_, dev_, part_, cnt_;
    CgDev *host_dev_ = nullptr;
    DeviceLoop loop_;
    const void *graph_x_ = nullptr;

    // one iteration of ConjugateGradient::preconditioned_solve (or unpreconditioned_solve)
    void iteration(void *x) {
        const int64_t n = op->nrows;
        CgDev *dev = dev_.as<CgDev>();
        double *part = part_.as<double>();
        unsigned int *cnt = cnt_.as<unsigned int>();
        const int g = reduce_grid(n);
        const bool f32 = mode_ == CG_GENERIC && pc_->pc_dtype() == UGPU_F32;
        // K0: p = z + beta p   (plain CG: p = r + beta p)
        // the solver's own vectors are cudaMalloc'd; only x may be caller memory
        const int vec = al16(x) ? 1 : 0;
        // K0 reduces nothing, so it is not tied to the reductions' fixed grid: full occupancy
        const int gp = int(std::max<int64_t>(1, std::min<int64_t>((n / 2 + kBlock - 1) / kBlock,
                                                                  int64_t(ctx->sms) * 8)));
        if (f32)
            k_cg_pupdate<float><<<gp, kBlock, 0, ctx->stream>>>(n, z32_.as<float>(), p_.as<double>(), dev, 1);
        else
            k_cg_pupdate<double><<<gp, kBlock, 0, ctx->stream>>>(n, (mode_ == CG_PLAIN) ? r_.as<double>()
                                                                                       : z_.as<double>(),
                                                                p_.as<double>(), dev, 1);
        ctx->launches++;
        bool prescaled = false;  // K2 wrote the preconditioner's first iterate
        // K1: Ap = A p ; (p, Ap) [, (p, r)]
        {
            SpmvArgs a;
            a.x = p_.ptr;
            a.y = Ap_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_STORE;
            a.dot_partials = part;
            a.dot_out = &dev->pAp;
            a.dot_counter = cnt + 0;
            a.done = &dev->done;
            launch_spmv(*ctx, *op, a);
        }
        // K2
        {
            const double atol = get("atol");
            const long long max_it = (long long)get("max_it");
            const double *dinv = (mode_ == CG_JACOBI) ? static_cast<InvDiag *>(pc_)->d.as<double>() : nullptr;
            // the preconditioner's first iterate x1 = w .* r, formed here where r is (pc_prescale)
            const void *pw = nullptr;
            void *px1 = nullptr;
            if (mode_ == CG_GENERIC && get("fold_dots") == 0) pc_->pc_prescale(&pw, &px1);
            prescaled = px1 != nullptr;
#define UGPU_CG_UPD(M, R)                                                                                          \
    k_cg_update<M, R><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<double *>(x), p_.as<double>(), r_.as<double>(), \
                                                     Ap_.as<double>(), dinv, z_.as<double>(), r32_.as<float>(), pw,   \
                                                     px1, dev, part + 2 * kSpmvDotGrid, cnt + 1, atol, max_it,       \
                                                     int(flexible_), vec)
            if (mode_ == CG_PLAIN) UGPU_CG_UPD(CG_PLAIN, false);
            else if (mode_ == CG_JACOBI) UGPU_CG_UPD(CG_JACOBI, false);
            else if (f32) UGPU_CG_UPD(CG_GENERIC, true);
            else UGPU_CG_UPD(CG_GENERIC, false);
#undef UGPU_CG_UPD
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
        }
        if (mode_ != CG_GENERIC) return;
        // z = M r, then K3
        const long long max_it = (long long)get("max_it");
        void *z = f32 ? z32_.ptr : z_.ptr;
        if (prescaled) {
            pc_->pc_enqueue_prescaled(f32 ? r32_.ptr : r_.ptr, z, &dev->done);
        } else if (get("fold_dots") != 0) {
            FinalDots fd;
            fd.a = r_.as<double>();
            fd.b = flexible_ ? Ap_.as<double>() : nullptr;
            fd.partials = part + 4 * kSpmvDotGrid;
            fd.out = part + 6 * kSpmvDotGrid;
            fd.counter = cnt + 3;
            if (pc_->pc_enqueue_dots(f32 ? r32_.ptr : r_.ptr, z, &dev->done, fd)) {
                k_cg_zfinish<<<1, 1, 0, ctx->stream>>>(dev, fd.out, max_it, int(flexible_));
                ctx->launches++;
                UGPU_LAUNCH_CHECK();
                return;
            }
        } else {
            pc_->pc_enqueue(f32 ? r32_.ptr : r_.ptr, z, &dev->done);
        }
        if (f32)
            k_cg_zdots<float><<<g, kBlock, 0, ctx->stream>>>(n, z32_.as<float>(), r_.as<double>(), Ap_.as<double>(),
                                                             dev, part + 4 * kSpmvDotGrid, cnt + 2, max_it,
                                                             int(flexible_), 1);
        else
            k_cg_zdots<double><<<g, kBlock, 0, ctx->stream>>>(n, z_.as<double>(), r_.as<double>(), Ap_.as<double>(),
                                                              dev, part + 4 * kSpmvDotGrid, cnt + 2, max_it,
                                                              int(flexible_), 1);
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
    }

    void finish(double t0, int64_t l0, bool done_now, double rnorm0) {
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
