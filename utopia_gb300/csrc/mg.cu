// Geometric/Galerkin multigrid on the GPU.
//
// Mirrors utopia::Multigrid (utopia/solvers/multilevel/utopia_Multigrid.hpp), its base
// LinearMultiLevel (utopia/solvers/multilevel/utopia_LinearMultiLevel.hpp), the
// IPRTransfer (utopia/solvers/multilevel/transfer/utopia_IPRTransfer.hpp), the masks
// (utopia/solvers/multilevel/utopia_MultiLevelMask.hpp) and the smoothers Jacobi,
// PointJacobi and Chebyshev3level (utopia/solvers/smoothers/).  Level 0 is the coarsest
// level, as after the std::reverse of LinearMultiLevel::galerkin_assembly.
//
// Precision: "precision" = UGPU_F64 (plain form: everything FP64), UGPU_F32 or UGPU_BF16
// (mixed form: level matrices and transfers stored in FP32 or BF16, vectors and
// accumulation in FP32; the Galerkin products, the eigen-estimates and the coarse
// Cholesky stay FP64).
#include <algorithm>
#include <cmath>
#include <limits>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {

// glibc rand() (TYPE_3 additive feedback, degree 31, separation 3) for the PowerMethod
// start vector v_i = rand()/RAND_MAX + 1 (utopia/solvers/eigensolvers/utopia_PowerMethod.hpp:99-106),
// restated so the sequence does not depend on other rand() users in the process.
struct GlibcRand {
    uint32_t ring[31];
    int f = 3, b = 0;
    explicit GlibcRand(uint32_t seed) {
        if (seed == 0) seed = 1;
        int64_t word = seed;
        ring[0] = seed;
        for (int k = 1; k < 31; ++k) {
            int64_t hi = word / 127773, lo = word % 127773;
            word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            ring[k] = uint32_t(word);
        }
        for (int k = 0; k < 310; ++k) next();
    }
    int32_t next() {
        ring[f] += ring[b];
        int32_t out = int32_t(ring[f] >> 1);
        f = (f + 1) % 31;
        b = (b + 1) % 31;
        return out;
    }
};

// MultiLevelMask::generate_mask_from_matrix: m_i = 0 if row i has an off-diagonal |a| > tol, else 1
template <class V>
__global__ void k_mask_fine(const int32_t *rp, const int32_t *ci, const V *cv, int64_t n, double tol, double *m) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double v = 1.0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] != i && fabs(cvt<double>(cv[k])) > tol) v = 0.0;
        m[i] = v;
    }
}

// IPRTransfer::boolean_restrict_or: m_c = min(1, R_bool m_f)
__global__ void k_mask_restrict(const int32_t *rp, const int32_t *ci, const double *cv, int64_t n, double tol,
                                const double *mf, double *mc) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) s += (fabs(cv[k]) > tol ? 1.0 : 0.0) * mf[ci[k]];
        mc[i] = s > 1.0 ? 1.0 : s;
    }
}

// mask = |m - 1|, counts the zeros
template <class T>
__global__ void k_mask_final(const double *m, int64_t n, T *out, unsigned long long *zeros) {
    unsigned long long z = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double v = fabs(m[i] - 1.0);
        out[i] = T(v);
        z += (v == 0.0);
    }
    atomicAdd(zeros, z);
}

// PowerMethod loop body (utopia_PowerMethod.hpp:122-146) after y = A v and dot = (y, y):
// lambda = ||y||, it++, stop when |lambda_old - lambda| < tol or it > max_it.  A call after the
// stop only sets `skip` (the rescaling of the iteration that stopped still runs).
__global__ void k_pm_check(double *st, int *done, long long *it, double tol, long long max_it) {
    if (done[0]) {
        done[1] = 1;
        return;
    }
    const double lambda = sqrt(st[0]);
    st[1] = lambda;
    *it += 1;
    if (fabs(st[2] - lambda) < tol || *it > max_it) done[0] = 1;
    st[2] = lambda;
}

// v = (1 / ||v||) v with ||v||^2 in dot[0] (the start vector's normalisation)
__global__ void k_pm_normalise(int64_t n, const double *dot, double *__restrict__ v) {
    const double s = 1. / sqrt(dot[0]);
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = s * v[i];
}

// v = (1 / lambda) y
__global__ void k_pm_scale(int64_t n, const double *__restrict__ y, const double *lambda, const int *skip,
                           double *__restrict__ v) {
    if (*skip) return;
    const double s = 1. / *lambda;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = s * y[i];
}

// LinearMultiLevel::fix_semidefinite_operator: diagonal entries with |a_ii| < 1e-12 get +1
__global__ void k_fix_semidefinite(const int32_t *rp, const int32_t *ci, double *cv, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i && fabs(cv[k]) < 1e-12) cv[k] += 1.0;
}

// PointJacobi::update: LU = A - diag(A) (diagonal entries set to 0, structure kept)
__global__ void k_zero_diag(const int32_t *rp, const int32_t *ci, double *cv, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i) cv[k] = 0.0;
}

// smoother weights from the FP64 diagonal
//   mode 0 (Jacobi):      w = omega * (|d| > 0 ? 1/d : 0)         (e_pseudo_inv with tol 0)
//   mode 1 (PointJacobi): w = 1/d, with 0 replaced by 1            (check_indef)
template <class T>
__global__ void k_weights(const double *d, int64_t n, double omega, int mode, T *w) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double v;
        if (mode == 0) {
            v = fabs(d[i]) > 0.0 ? 1.0 / d[i] : 0.0;
            v = omega * v;
        } else {
            v = 1.0 / d[i];
            if (v == 0.0) v = 1.0;
        }
        w[i] = T(v);
    }
}

struct Level {
    const Mat *A64 = nullptr;           // FP64 operator (the fine one is borrowed)
    std::unique_ptr<Mat> A64own;
    std::unique_ptr<Mat> Awork;         // storage-precision copy for the mixed form
    std::unique_ptr<Mat> LU;            // PointJacobi off-diagonal part
    const Mat *A() const { return Awork ? Awork.get() : A64; }
    int64_t n = 0;
    Buffer w;      // smoother weights (vector dtype)
    Buffer mask;   // restriction mask (vector dtype); unused if all ones
    bool has_mask = false;
    double emax = 0, emin = 0;
    std::vector<double> cheb_alpha, cheb_beta;
    Buffer r, c, c2, rR, p0, p1, rr;  // work vectors (vector dtype)
    Buffer x1;  // the first Jacobi iterate w .* r from zero, written by the kernel that forms r
};

// power-method scratch of one level
struct PmScratch {
    Buffer v, w, st, part, cnt;  // st: [0] dot, [1] lambda, [2] lambda_old; int done, int skip, int64 it
};

struct Transfer {
    std::unique_ptr<Mat> P64, R64;    // FP64 interpolation and explicit restriction R = P^T
    std::unique_ptr<Mat> Pw, Rw;      // storage-precision copies
    const Mat *P() const { return Pw ? Pw.get() : P64.get(); }
    const Mat *R() const { return Rw ? Rw.get() : R64.get(); }
};

class Multigrid final : public Solver {
public:
    ~Multigrid() override {
        if (!pm_streams_.empty() || pm_fork_) cudaStreamSynchronize(ctx->stream);
        for (auto st : pm_streams_) cudaStreamDestroy(st);
        if (pm_fork_) cudaEventDestroy(pm_fork_);
        if (pm_join_) cudaEventDestroy(pm_join_);
    }
    explicit Multigrid(Context *c) : Solver(c, UGPU_SOLVER_MULTIGRID) {
        prm["pre_smoothing_steps"] = 3;   // utopia_MultiLevelBase.hpp:35-42
        prm["post_smoothing_steps"] = 3;
        prm["smoother"] = 1;              // 0 Jacobi, 1 Chebyshev3level, 2 PointJacobi
        prm["omega"] = 1.0;
        prm["precision"] = UGPU_F64;
        prm["must_generate_masks"] = 1;   // Multigrid forces masks on, utopia_Multigrid.hpp:76
        prm["fix_semidefinite_operators"] = 0;
        prm["keep_galerkin_structure"] = 0;  // 1: products keep their structure; an operator with the
                                              // structure of the last one only recomputes values
        prm["scale_max_eig"] = 1.2;       // utopia_Chebyshev3level.hpp:183
        prm["scale_min_eig"] = 0.06;
        prm["power_method_tol"] = 1e-2;   // utopia_PowerMethod.hpp:150-151
        prm["power_method_max_it"] = 30;
        prm["rand_seed"] = 1;
        prm["mg_type"] = 1;               // V-cycle
        prm["coarse_fp32"] = 0;           // mixed form: 1 applies an FP32 copy of the coarse inverse
        prm["x1_from_producer"] = 1;      // 1: the kernel forming a level's r also writes w .* r (uses_x1)
    }

    void set_transfers(const std::vector<const Mat *> &P) {
        transfers_.clear();
        for (auto *p : P) {
            UGPU_CHECK(p && p->vdtype == UGPU_F64, UGPU_ERR_ARG, "transfer operators must be FP64 matrices");
            Transfer t;
            t.P64 = cast_matrix(*p, UGPU_F64);  // deep copy
            t.R64 = transpose(*t.P64);          // IPRTransfer: R = transpose(I)
            transfers_.push_back(std::move(t));
        }
        ready_ = false;
    }

    int n_levels() const { return int(levels_.size()); }
    const Level &level(int l) const { return levels_.at(l); }

    // Multigrid::update(op): IterativeSolver::update + galerkin_assembly + smoothers + coarse solver
    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols, UGPU_ERR_ARG, "multigrid: square operator required");
        UGPU_CHECK(A->vdtype == UGPU_F64, UGPU_ERR_ARG, "multigrid: FP64 fine operator required");
        UGPU_CHECK(!transfers_.empty(), UGPU_ERR_STATE, "Provide interpolation operators first");
        op = A;
        vdt_ = (int(get("precision")) == UGPU_F64) ? UGPU_F64 : UGPU_F32;
        const int sdt = int(get("precision"));
        const int L = int(transfers_.size()) + 1;
        const bool keep = get("keep_galerkin_structure") != 0;
        const bool fix = get("fix_semidefinite_operators") != 0;
        // an operator with the structure of the last one: only the values of the Galerkin
        // products are recomputed, in place
        bool numeric = keep && ready_ && int(levels_.size()) == L;
        if (numeric) {
            levels_[L - 1].A64 = A;
            for (int l = L - 2; l >= 0 && numeric; --l) {
                Level &c = levels_[l];
                numeric = c.A64own && c.A64own->ptap_plan &&
                          ptap_numeric(*levels_[l + 1].A64, *transfers_[l].P64, *c.A64own, *c.A64own->ptap_plan,
                                       false);
                if (!numeric) break;
                if (fix) fix_semidefinite_operator(*ctx, *c.A64own);
                else refresh_values(*c.A64own);
            }
        }
        if (!numeric) {
            // galerkin_assembly (utopia_LinearMultiLevel.hpp:201-226): fine first, then reverse
            std::vector<Level> lev(L);
            lev[0].A64 = A;
            for (int i = 1; i < L; ++i) {
                const Transfer &t = transfers_[L - 1 - i];
                UGPU_CHECK(t.P64->nrows == lev[i - 1].A64->nrows, UGPU_ERR_ARG,
                           "interpolation operator rows do not match the finer level");
                if (keep) {
                    std::shared_ptr<PtapPlan> plan;
                    lev[i].A64own = ptap_with_plan(*lev[i - 1].A64, *t.P64, plan);
                    lev[i].A64own->ptap_plan = std::move(plan);
                } else {
                    lev[i].A64own = ptap(*lev[i - 1].A64, *t.P64);
                }
                if (fix) fix_semidefinite_operator(*ctx, *lev[i].A64own);
                lev[i].A64 = lev[i].A64own.get();
            }
            std::reverse(lev.begin(), lev.end());
            // a re-assembly with unchanged level sizes keeps the work buffers (no free / malloc)
            for (int l = 0; l < L && l < int(levels_.size()); ++l) {
                if (levels_[l].n != lev[l].A64->nrows) continue;
                Level &o = levels_[l];
                for (auto pr : {std::make_pair(&o.r, &lev[l].r), std::make_pair(&o.c, &lev[l].c),
                                std::make_pair(&o.c2, &lev[l].c2), std::make_pair(&o.rR, &lev[l].rR),
                                std::make_pair(&o.p0, &lev[l].p0), std::make_pair(&o.p1, &lev[l].p1),
                                std::make_pair(&o.rr, &lev[l].rr), std::make_pair(&o.w, &lev[l].w)})
                    *pr.second = std::move(*pr.first);
            }
            levels_ = std::move(lev);
        }
        for (auto &l : levels_) l.n = l.A64->nrows;
        // storage-precision copies of operators and transfers
        for (int l = 0; l < L; ++l) {
            if (sdt != UGPU_F64) levels_[l].Awork = cast_matrix(*levels_[l].A64, sdt);
        }
        for (auto &t : transfers_) {
            if (sdt != UGPU_F64) {
                t.Pw = cast_matrix(*t.P64, sdt);
                t.Rw = cast_matrix(*t.R64, sdt);
            } else {
                t.Pw.reset();
                t.Rw.reset();
            }
        }
        make_masks();
        // Multigrid::update(): smoothers of levels 1..L-1 in order, then the coarse solver
        GlibcRand rng(uint32_t(get("rand_seed")));
        const int sm = int(get("smoother"));
        for (int l = 1; l < L; ++l) setup_smoother(l, sm);
        if (sm == 1) {
            power_methods(rng);
            for (int l = 1; l < L; ++l) chebyshev_coefficients(levels_[l]);
        }
        UGPU_CHECK(coarse_.factor(*levels_[0].A64), UGPU_ERR_NOT_SPD,
                   "coarse operator is not symmetric positive definite");
        // the mixed V-cycle's coarse solve stays FP64 (FP64 inverse, FP64 accumulation) unless
        // coarse_fp32 asks for the FP32 copy of the inverse
        if (vdt_ == UGPU_F32 && get("coarse_fp32") != 0) coarse_.make_fp32_inverse();
        const size_t vs = dtype_size(vdt_);
        for (size_t k = 0; k < levels_.size(); ++k) {
            Level &l = levels_[k];
            size_t b = vs * std::max<int64_t>(l.n, 1);
            for (Buffer *q : {&l.r, &l.c, &l.c2, &l.rR, &l.p0, &l.p1, &l.rr}) q->ensure(b);
            if (uses_x1(int(k))) l.x1.ensure(b);
        }
        f64_r_.ensure(sizeof(double) * std::max<int64_t>(A->nrows, 1));
        f64_z_.ensure(sizeof(double) * std::max<int64_t>(A->nrows, 1));
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        ready_ = true;
    }

    int pc_dtype() const override { return vdt_; }

    // one V-cycle from zero: z = M^{-1} r (vectors of pc_dtype(), fine-level size)
    void pc_enqueue(const void *r, void *z, const int *done) override {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "multigrid: update() first");
        cycle(n_levels() - 1, r, z, done);
    }

    // The Jacobi / PointJacobi pre-smoothing from zero starts with x1 = w .* r.  Rather than a
    // product whose every gather forms w_j r_j, the kernel that forms r writes x1 beside it (the
    // restriction for the coarser levels, the caller's residual update for the fine one) and the
    // sweeps start from the stored x1, as the reference's Jacobi does (in the fused form the
    // compiler may contract the row's own w_i r_i into the epilogue's FMA: a different rounding).
    bool uses_x1(int l) const {
        return l >= 1 && get("x1_from_producer") != 0 && int(get("smoother")) != 1 &&
               int(get("pre_smoothing_steps")) >= 2;
    }
    void pc_prescale(const void **w, void **x1) override {
        const int top = n_levels() - 1;
        const bool ok = ready_ && top >= 1 && uses_x1(top) && levels_[size_t(top)].x1.ptr;
        *w = ok ? levels_[size_t(top)].w.ptr : nullptr;
        *x1 = ok ? levels_[size_t(top)].x1.ptr : nullptr;
    }
    void pc_enqueue_prescaled(const void *r, void *z, const int *done) override {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "multigrid: update() first");
        top_x1_ = true;
        cycle(n_levels() - 1, r, z, done);
        top_x1_ = false;
    }

    // the V-cycle with the outer iteration's dots of z computed by the last fine-level
    // post-smoothing sweep (Jacobi / PointJacobi smoothing with at least one post sweep and a
    // coarse level); other configurations run the plain cycle
    bool pc_enqueue_dots(const void *r, void *z, const int *done, const FinalDots &fd) override {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "multigrid: update() first");
        if (int(get("smoother")) == 1 || int(get("post_smoothing_steps")) < 1 || n_levels() < 2) {
            cycle(n_levels() - 1, r, z, done);
            return false;
        }
        fd_ = &fd;
        fd_used_ = false;
        cycle(n_levels() - 1, r, z, done);
        fd_ = nullptr;
        UGPU_CHECK(fd_used_, UGPU_ERR_INTERNAL, "multigrid: the final dots were not attached");
        return true;
    }

    // Multigrid::apply as a stand-alone solver (utopia_Multigrid.hpp:162-238)
    void apply(const Vec &rhs, Vec &x) override {
        UGPU_CHECK(ready_, UGPU_ERR_STATE, "multigrid: update() first");
        UGPU_CHECK(rhs.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG, "multigrid: FP64 rhs and x");
        const int64_t n = op->nrows;
        UGPU_CHECK(rhs.n == n && x.n == n, UGPU_ERR_ARG, "multigrid: size mismatch");
        double t0 = now_s();
        int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        double *res = f64_r_.as<double>();
        auto residual = [&]() {
            SpmvArgs a;
            a.x = x.data();
            a.v = rhs.data();
            a.y = res;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_RESIDUAL;
            launch_spmv(*ctx, *op, a);
            DotArgs d{};
            d.nd = 1;
            d.a[0] = d.b[0] = res;
            d.dtype_a[0] = d.dtype_b[0] = UGPU_F64;
            double v;
            host_dots(*ctx, n, d, &v);
            return std::sqrt(v);
        };
        double r_norm = residual(), r0 = r_norm;
        int64_t it = 1;
        bool conv = false;
        Buffer r32, z32;
        if (vdt_ == UGPU_F32) {
            r32.alloc(sizeof(float) * std::max<int64_t>(n, 1));
            z32.alloc(sizeof(float) * std::max<int64_t>(n, 1));
        }
        while (!conv) {
            if (vdt_ == UGPU_F64) {
                cycle(n_levels() - 1, res, f64_z_.ptr, nullptr);
            } else {
                enq_convert(*ctx, UGPU_F64, res, UGPU_F32, r32.ptr, n, nullptr);
                cycle(n_levels() - 1, r32.ptr, z32.ptr, nullptr);
                enq_convert(*ctx, UGPU_F32, z32.ptr, UGPU_F64, f64_z_.ptr, n, nullptr);
            }
            enq_axpy(*ctx, UGPU_F64, n, 1.0, f64_z_.ptr, x.data(), nullptr);
            r_norm = residual();
            conv = check_convergence(it, r_norm, r_norm / r0, 1);
            it++;
        }
        st.converged = st.reason > 0;
        st.spmv_count = it;
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

    void eigs(int l, double *emax, double *emin) const {
        *emax = levels_.at(l).emax;
        *emin = levels_.at(l).emin;
    }

private:
    std::vector<Transfer> transfers_;
    std::vector<Level> levels_;
    DenseCholesky coarse_;
    int vdt_ = UGPU_F64;
    bool ready_ = false;
    Buffer f64_r_, f64_z_;
    std::vector<PmScratch> pm_;            // power-method scratch per level
    std::vector<cudaStream_t> pm_streams_;  // one stream per level for the concurrent power methods
    cudaEvent_t pm_fork_ = nullptr, pm_join_ = nullptr;

    void make_masks() {
        const int L = n_levels();
        for (auto &l : levels_) l.has_mask = false;
        if (get("must_generate_masks") == 0) return;
        const double tol = std::numeric_limits<double>::epsilon() * 1e6;
        std::vector<Buffer> m(L);
        for (int l = 0; l < L; ++l) m[l].alloc(sizeof(double) * std::max<int64_t>(levels_[l].n, 1));
        const Mat &Af = *levels_[L - 1].A64;
        k_mask_fine<double><<<stream_grid(*ctx, Af.nrows), kBlock, 0, ctx->stream>>>(
            Af.rowptr.as<int32_t>(), Af.colidx.as<int32_t>(), Af.vals.as<double>(), Af.nrows, tol,
            m[L - 1].as<double>());
        ctx->launches++;
        for (int l = L - 1; l > 0; --l) {
            const Mat &R = *transfers_[l - 1].R64;
            k_mask_restrict<<<stream_grid(*ctx, R.nrows), kBlock, 0, ctx->stream>>>(
                R.rowptr.as<int32_t>(), R.colidx.as<int32_t>(), R.vals.as<double>(), R.nrows, tol, m[l].as<double>(),
                m[l - 1].as<double>());
            ctx->launches++;
        }
        Buffer zeros;
        zeros.alloc(sizeof(unsigned long long));
        for (int l = 0; l < L; ++l) {
            auto &lv = levels_[l];
            lv.mask.alloc(dtype_size(vdt_) * std::max<int64_t>(lv.n, 1));
            UGPU_CUDA(cudaMemsetAsync(zeros.ptr, 0, sizeof(unsigned long long), ctx->stream));
            if (vdt_ == UGPU_F64)
                k_mask_final<double><<<stream_grid(*ctx, lv.n), kBlock, 0, ctx->stream>>>(
                    m[l].as<double>(), lv.n, lv.mask.as<double>(), zeros.as<unsigned long long>());
            else
                k_mask_final<float><<<stream_grid(*ctx, lv.n), kBlock, 0, ctx->stream>>>(
                    m[l].as<double>(), lv.n, lv.mask.as<float>(), zeros.as<unsigned long long>());
            ctx->launches++;
            unsigned long long hz = 0;
            UGPU_CUDA(cudaMemcpyAsync(&hz, zeros.ptr, sizeof(hz), cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
            lv.has_mask = hz > 0;  // an all-ones mask is skipped (multiplying by 1 is exact)
        }
        UGPU_LAUNCH_CHECK();
    }

    void setup_smoother(int l, int sm) {
        Level &lv = levels_[l];
        Mat &A64 = const_cast<Mat &>(*lv.A64);
        ensure_diag(A64);
        lv.w.ensure(dtype_size(vdt_) * std::max<int64_t>(lv.n, 1));
        int g = stream_grid(*ctx, lv.n);
        if (sm == 0 || sm == 2) {
            int mode = (sm == 0) ? 0 : 1;
            if (vdt_ == UGPU_F64)
                k_weights<double><<<g, kBlock, 0, ctx->stream>>>(A64.diag.as<double>(), lv.n, get("omega"), mode,
                                                                 lv.w.as<double>());
            else
                k_weights<float><<<g, kBlock, 0, ctx->stream>>>(A64.diag.as<double>(), lv.n, get("omega"), mode,
                                                                lv.w.as<float>());
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
            if (sm == 2) {
                auto lu = cast_matrix(A64, UGPU_F64);
                k_zero_diag<<<g, kBlock, 0, ctx->stream>>>(lu->rowptr.as<int32_t>(), lu->colidx.as<int32_t>(),
                                                           lu->vals.as<double>(), lu->nrows);
                ctx->launches++;
                finalize_matrix(*lu);
                int sdt = int(get("precision"));
                lv.LU = (sdt == UGPU_F64) ? std::move(lu) : cast_matrix(*lu, sdt);
            }
        }
    }

    // Chebyshev3level::solve recurrence coefficients (utopia_Chebyshev3level.hpp:138-156)
    void chebyshev_coefficients(Level &lv) {
        const int nu = std::max(int(get("pre_smoothing_steps")), int(get("post_smoothing_steps")));
        const double avg = (lv.emax + lv.emin) / 2.0, dif = (lv.emax - lv.emin) / 2.0;
        lv.cheb_alpha.assign(std::max(nu, 1), 0.0);
        lv.cheb_beta.assign(std::max(nu, 1), 0.0);
        double alpha = 1.0 / avg;
        lv.cheb_alpha[0] = alpha;
        for (int k = 1; k < nu; ++k) {
            double da = dif * alpha;
            double beta = (k == 1 ? 0.5 : 0.25) * da * da;
            alpha = 1.0 / (avg - (beta / alpha));
            lv.cheb_beta[k] = beta;
            lv.cheb_alpha[k] = alpha;
        }
    }

    // PowerMethod::get_max_eig / compute_max_eig (utopia_PowerMethod.hpp:95-146) in FP64 for every
    // smoothed level; Chebyshev3level::init_eigs scales the result (utopia_Chebyshev3level.hpp:118-121).
    // The start vectors are drawn from the rand() sequence in level order (as the reference's
    // levels are updated one after the other); the levels' iterations are independent, so they
    // run concurrently on one stream per level (each with its own reduction scratch), joined
    // back into the context's stream before the estimates are read.
    void power_methods(GlibcRand &rng) {
        const int L = n_levels();
        const double tol = get("power_method_tol");
        const long long max_it = (long long)get("power_method_max_it");
        std::vector<std::vector<double>> h(L);
        for (int l = 1; l < L; ++l) {
            h[l].resize(size_t(levels_[l].n));
            for (auto &x : h[l]) x = (double(rng.next()) / 2147483647.0) + 1;
        }
        if (pm_.size() < size_t(L)) pm_.resize(L);
        while (pm_streams_.size() < size_t(L)) {
            cudaStream_t st;
            UGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            pm_streams_.push_back(st);
        }
        if (!pm_fork_) {
            UGPU_CUDA(cudaEventCreateWithFlags(&pm_fork_, cudaEventDisableTiming));
            UGPU_CUDA(cudaEventCreateWithFlags(&pm_join_, cudaEventDisableTiming));
        }
        cudaStream_t main = ctx->stream;
        struct Restore {  // the context's stream is switched per level below
            Context *c;
            cudaStream_t s;
            const std::vector<cudaStream_t> *level_streams;
            int started = 0;  // level streams holding work the main stream has not joined
            ~Restore() {
                // on an exception part-way through, later work on the main stream must not
                // run beside unfinished power-method kernels: wait for the started levels
                for (int l = 1; l <= started; ++l) cudaStreamSynchronize((*level_streams)[size_t(l)]);
                c->stream = s;
            }
        } restore{ctx, main, &pm_streams_};
        for (int l = 1; l < L; ++l) {
            const int64_t n = levels_[l].n;
            PmScratch &ps = pm_[l];
            ps.v.ensure(sizeof(double) * std::max<int64_t>(n, 1));
            ps.w.ensure(sizeof(double) * std::max<int64_t>(n, 1));
            ps.st.ensure(3 * sizeof(double) + 2 * sizeof(int) + sizeof(long long));
            ps.part.ensure(sizeof(double) * kRedBlocks);
            if (!ps.cnt.ptr) {  // reduction tickets; the last CTA of every reduction resets its ticket
                ps.cnt.alloc(sizeof(unsigned int) * 4);
                UGPU_CUDA(cudaMemsetAsync(ps.cnt.ptr, 0, ps.cnt.bytes, main));
            }
        }
        UGPU_CUDA(cudaEventRecord(pm_fork_, main));
        for (int l = 1; l < L; ++l) {
            const Level &lv = levels_[l];
            const int64_t n = lv.n;
            PmScratch &ps = pm_[l];
            UGPU_CUDA(cudaStreamWaitEvent(pm_streams_[l], pm_fork_, 0));
            restore.started = l;
            ctx->stream = pm_streams_[l];
            double *dst = ps.st.as<double>();
            int *done = reinterpret_cast<int *>(dst + 3);
            long long *itp = reinterpret_cast<long long *>(done + 2);
            const double *v = ps.v.as<double>(), *w = ps.w.as<double>();
            UGPU_CUDA(cudaMemsetAsync(ps.st.ptr, 0, ps.st.bytes, ctx->stream));
            if (n) UGPU_CUDA(cudaMemcpyAsync(ps.v.ptr, h[l].data(), sizeof(double) * n, cudaMemcpyHostToDevice,
                                             ctx->stream));
            DotArgs d{};
            d.nd = 1;
            d.dtype_a[0] = d.dtype_b[0] = UGPU_F64;
            // v = v / ||v||
            d.a[0] = d.b[0] = v;
            launch_dots_into(*ctx, n, d, dst, ps.part.as<double>(), ps.cnt.as<unsigned int>());
            const int g = stream_grid(*ctx, n);
            k_pm_normalise<<<g, kBlock, 0, ctx->stream>>>(n, dst, ps.v.as<double>());
            ctx->launches++;
            // the iterations run without host round trips: a device flag set by the stop test
            // predicates the later products, and `skip` the later rescalings
            for (long long k = 0; k <= max_it + 1; ++k) {
                SpmvArgs a;
                a.x = v;
                a.y = ps.w.ptr;
                a.vec_dtype = UGPU_F64;
                a.done = done;
                launch_spmv(*ctx, *lv.A64, a);
                d.a[0] = d.b[0] = w;
                launch_dots_into(*ctx, n, d, dst, ps.part.as<double>(), ps.cnt.as<unsigned int>());
                k_pm_check<<<1, 1, 0, ctx->stream>>>(dst, done, itp, tol, max_it);
                k_pm_scale<<<g, kBlock, 0, ctx->stream>>>(n, w, dst + 1, done + 1, ps.v.as<double>());
                ctx->launches += 2;
            }
            UGPU_LAUNCH_CHECK();
            UGPU_CUDA(cudaEventRecord(pm_join_, ctx->stream));
            UGPU_CUDA(cudaStreamWaitEvent(main, pm_join_, 0));
        }
        restore.started = 0;  // every level stream is joined into the main stream
        ctx->stream = main;
        std::vector<double> hs(size_t(L) * 3);
        std::vector<int> hd(size_t(L), 1);
        for (int l = 1; l < L; ++l) {
            UGPU_CUDA(cudaMemcpyAsync(&hs[size_t(l) * 3], pm_[l].st.ptr, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                      main));
            UGPU_CUDA(cudaMemcpyAsync(&hd[size_t(l)], pm_[l].st.as<double>() + 3, sizeof(int), cudaMemcpyDeviceToHost,
                                      main));
        }
        UGPU_CUDA(cudaStreamSynchronize(main));
        for (int l = 1; l < L; ++l) {
            UGPU_CHECK(hd[size_t(l)] == 1, UGPU_ERR_INTERNAL, "power method: the stop test never held");
            Level &lv = levels_[l];
            lv.emax = get("scale_max_eig") * hs[size_t(l) * 3 + 1];
            lv.emin = get("scale_min_eig") * lv.emax;
        }
    }

    const FinalDots *fd_ = nullptr;  // set while pc_enqueue_dots runs its cycle
    bool fd_used_ = false;
    bool top_x1_ = false;  // set while pc_enqueue_prescaled runs its cycle: the fine level's x1 is valid

    // ---------------------------------------------------------------- cycle ----
    void spmv(const Mat &A, SpmvArgs a, const int *done) {
        a.vec_dtype = vdt_;
        a.done = done;
        launch_spmv(*ctx, A, a);
    }

    // smoothing sweeps of Jacobi / PointJacobi from the iterate in bufs[cur]; returns the
    // buffer index holding the result.  from_zero: the iterate is zero, so the first sweep
    // is x1 = w .* rhs and is folded into the second (its product gathers w .* rhs).
    // fd: the outer iteration's dots, computed by the last sweep (post-smoothing only)
    // x1: the first iterate w .* rhs, already formed (from_zero, nu >= 2)
    int jacobi_sweeps(Level &lv, int sm, const void *rhs, void *bufs[2], int cur, int nu, bool from_zero,
                      const int *done, const FinalDots *fd = nullptr, const void *x1 = nullptr) {
        const Mat &Aop = (sm == 2) ? *lv.LU : *lv.A();
        const int epi = (sm == 2) ? EPI_PJACOBI : EPI_JACOBI;
        int s = 0;
        if (from_zero && nu >= 2 && x1) {
            SpmvArgs a;  // x2 = x1 + w .* (rhs - A x1)
            a.x = x1;
            a.v = rhs;
            a.w = lv.w.ptr;
            a.y = bufs[cur];
            a.epilogue = epi;
            spmv(Aop, a, done);
            s = 2;
        } else if (from_zero && nu >= 1) {
            if (nu == 1) {
                // Jacobi: x = 0 + w .* (rhs - A*0); PointJacobi: x = w .* (rhs - LU*0)
                enq_scale_into(*ctx, vdt_, lv.n, lv.w.ptr, rhs, bufs[cur], done);
                return cur;
            }
            SpmvArgs a;
            a.xmode = 2;  // x1 = w .* rhs on the fly; x2 = x1 + w .* (rhs - A x1)
            a.v = rhs;
            a.w = lv.w.ptr;
            a.y = bufs[cur];
            a.epilogue = epi;
            spmv(Aop, a, done);
            s = 2;
        }
        for (; s < nu; ++s) {
            SpmvArgs a;
            a.x = bufs[cur];
            a.v = rhs;
            a.w = lv.w.ptr;
            a.y = bufs[cur ^ 1];
            a.epilogue = epi;
            if (fd && s == nu - 1) {
                a.fa = fd->a;
                a.fb = fd->b;
                a.fpart = fd->partials;
                a.fout = fd->out;
                a.fcnt = fd->counter;
                fd_used_ = true;
            }
            spmv(Aop, a, done);
            cur ^= 1;
        }
        return cur;
    }

    int jacobi_swaps(int nu, bool from_zero) const {
        if (nu <= 0) return 0;
        return from_zero ? std::max(nu - 2, 0) : nu;
    }

    // Chebyshev3level::smooth(rhs, x) with nu iterations, x updated in place.
    void chebyshev(Level &lv, const void *rhs, void *x, int nu, bool from_zero, const int *done) {
        if (nu <= 0) return;
        void *p[2] = {lv.p0.ptr, lv.p1.ptr};
        if (from_zero) {
            // r = A*0 - b = -b ; p = -1 * r
            enq_neg_copy(*ctx, vdt_, lv.n, rhs, lv.rr.ptr, p[0], done);
        } else {
            SpmvArgs a;
            a.x = x;
            a.v = rhs;
            a.vout = lv.rr.ptr;
            a.y = p[0];
            a.epilogue = EPI_CHEB0;
            spmv(*lv.A(), a, done);
        }
        int cur = 0;
        for (int k = 1; k < nu; ++k) {
            SpmvArgs a;
            a.x = p[cur];
            a.vout = lv.rr.ptr;
            a.x2 = x;
            a.y = p[cur ^ 1];
            a.s0 = lv.cheb_alpha[k - 1];
            a.s1 = lv.cheb_beta[k];
            a.s2 = lv.cheb_alpha[k];
            a.s3 = (k == 1) ? lv.cheb_alpha[0] : 0.0;
            a.x2_zero = (k == 1 && from_zero) ? 1 : 0;  // x = 0 + alpha_0 p_0 + alpha_1 p_1
            a.epilogue = EPI_CHEB;
            spmv(*lv.A(), a, done);
            cur ^= 1;
        }
        if (nu == 1) {
            if (from_zero) enq_set(*ctx, vdt_, lv.n, 0.0, x, done);
            enq_axpy(*ctx, vdt_, lv.n, lv.cheb_alpha[0], p[0], x, done);
        }
    }

    // Multigrid::standard_cycle (utopia_Multigrid.hpp:252-367), V-cycle, c from zero.
    void cycle(int l, const void *r, void *c_out, const int *done) {
        if (l == 0) {
            coarse_.solve(r, vdt_, c_out, vdt_, done);
            return;
        }
        Level &lv = levels_[l];
        Level &lc = levels_[l - 1];
        const Transfer &t = transfers_[l - 1];
        const int sm = int(get("smoother"));
        const int pre = int(get("pre_smoothing_steps")), post = int(get("post_smoothing_steps"));
        void *c;
        int cur = 0;
        void *bufs[2] = {c_out, lv.c2.ptr};
        if (sm == 1) {
            c = c_out;
            if (pre <= 0) enq_set(*ctx, vdt_, lv.n, 0.0, c, done);
            chebyshev(lv, r, c, pre, true, done);
        } else {
            const int swaps = jacobi_swaps(pre, true) + jacobi_swaps(post, false);
            cur = swaps & 1;  // start so that the last sweep lands in c_out
            if (pre <= 0) enq_set(*ctx, vdt_, lv.n, 0.0, bufs[cur], done);
            const bool x1_ok = uses_x1(l) && lv.x1.ptr && (l < n_levels() - 1 || top_x1_);
            cur = jacobi_sweeps(lv, sm, r, bufs, cur, pre, true, done, nullptr, x1_ok ? lv.x1.ptr : nullptr);
            c = bufs[cur];
        }
        // r_R = r - A c ; r_{l-1} = mask .* (R r_R)
        {
            SpmvArgs a;
            a.x = c;
            a.v = r;
            a.y = lv.rR.ptr;
            a.epilogue = EPI_RESIDUAL;
            spmv(*lv.A(), a, done);
        }
        {
            SpmvArgs a;
            a.x = lv.rR.ptr;
            a.y = lc.r.ptr;
            if (lc.has_mask) {
                a.w = lc.mask.ptr;
                a.epilogue = EPI_SCALE;
            }
            if (uses_x1(l - 1) && lc.x1.ptr) {  // the coarser level's first Jacobi iterate
                a.sw_out = lc.x1.ptr;
                a.sw = lc.w.ptr;
                a.epilogue = lc.has_mask ? EPI_SCALE_SW : EPI_STORE_SW;
            }
            spmv(*t.R(), a, done);
        }
        cycle(l - 1, lc.r.ptr, lc.c.ptr, done);
        // c += I c_{l-1}
        {
            SpmvArgs a;
            a.x = lc.c.ptr;
            a.v = c;
            a.y = c;
            a.epilogue = EPI_ADD;
            spmv(*t.P(), a, done);
        }
        if (sm == 1) {
            chebyshev(lv, r, c, post, false, done);
        } else {
            cur = jacobi_sweeps(lv, sm, r, bufs, cur, post, false, done, l == n_levels() - 1 ? fd_ : nullptr);
            UGPU_CHECK(bufs[cur] == c_out, UGPU_ERR_INTERNAL, "multigrid: smoother buffer bookkeeping");
        }
    }
};

}  // namespace

std::unique_ptr<Solver> make_multigrid(Context *c) { return std::make_unique<Multigrid>(c); }

void fix_semidefinite_operator(Context &ctx, Mat &J) {
    UGPU_CHECK(J.vdtype == UGPU_F64, UGPU_ERR_ARG, "fix_semidefinite_operator: FP64 operator");
    k_fix_semidefinite<<<stream_grid(ctx, J.nrows), kBlock, 0, ctx.stream>>>(
        J.rowptr.as<int32_t>(), J.colidx.as<int32_t>(), J.vals.as<double>(), J.nrows);
    ctx.launches++;
    refresh_values(J);
}

int mg_n_levels(const Solver *s) {
    if (int k = mmg_n_levels(s); k >= 0) return k;
    auto m = dynamic_cast<const Multigrid *>(amg_multigrid(s));
    UGPU_CHECK(m, UGPU_ERR_ARG, "not a multigrid solver");
    return m->n_levels();
}

std::unique_ptr<Mat> mg_level_matrix(const Solver *s, int l) {
    if (auto M = mmg_level_matrix(s, l)) return M;
    auto m = dynamic_cast<const Multigrid *>(amg_multigrid(s));
    UGPU_CHECK(m, UGPU_ERR_ARG, "not a multigrid solver");
    UGPU_CHECK(l >= 0 && l < m->n_levels(), UGPU_ERR_ARG, "level out of range");
    return cast_matrix(*m->level(l).A64, UGPU_F64);
}

void mg_eigs(const Solver *s, int l, double *emax, double *emin) {
    auto m = dynamic_cast<const Multigrid *>(amg_multigrid(s));
    UGPU_CHECK(m, UGPU_ERR_ARG, "not a multigrid solver");
    UGPU_CHECK(l >= 0 && l < m->n_levels(), UGPU_ERR_ARG, "level out of range");
    m->eigs(l, emax, emin);
}

void mg_set_transfers(Solver *s, const std::vector<const Mat *> &P) {
    if (mmg_set_transfers(s, P)) return;
    auto m = dynamic_cast<Multigrid *>(s);
    UGPU_CHECK(m, UGPU_ERR_ARG, "not a multigrid solver");
    m->set_transfers(P);
}

}  // namespace ugpu
