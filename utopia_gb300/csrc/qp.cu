// Box-constrained QP solvers: MPRGP and multicolour projected Gauss-Seidel.
//
// MPRGP mirrors utopia::MPRGP::solve (non-Hardik variant, no preconditioner;
// utopia/solvers/nonlinear/constrained/quadratic_programming/utopia_MPRGP.hpp:57-262) with
// get_fi / get_beta / get_alpha_f (:266-348) and its power method (:351-387).  The
// branch decisions of every iteration (proportional vs proportioning, CG vs expansion
// step, negative curvature, convergence) are taken on the device by the last CTA of
// the kernel that produces the deciding dots; the kernels of the branches that are
// not taken return at once, so a batch of iterations runs without host round trips.
//
// ProjectedGaussSeidel mirrors utopia::ProjectedGaussSeidel::apply/step
// (utopia_ProjectedGaussSeidel.hpp:71-112,197-318) with the lexicographic row loop
// replaced by a multicolour sweep: rows of one colour are relaxed in parallel, colours
// in order (then in reverse order for the symmetric sweep).  The colouring is the
// greedy first-fit colouring in index order (red-black for the 5-point grid), computed
// on the device by dependency rounds that reproduce the sequential result exactly.
#include <climits>
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {

#define QP_LOOP(i, n) \
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

struct QpDev {
    double qa0, qa1;              // the iteration's product s -> A s: (s, A s), (s, g); s = p or beta
    double neg_bsc;               // -beta_sc of the pending direction p = fi - beta_sc p (0: p = fi)
    unsigned long long amin;      // key (qp_key) of alpha_f = min step bound, reset after each use
    double alpha_cg, alpha_f, beta_sc;
    double beta_beta, fi_fi, gnorm, gnorm0;
    long long it, iterates;
    int done, reason, converged;
    int gate_cg, gate_prop, gate_exp;   // branch of the current iteration
    int step;                           // 0: CG step, 1: expansion step
};

// the predicates of MPRGP / VariableBoundSolverInterface with their comparisons on the integer
// pipes (device_util.cuh: exact for non-NaN bounds and iterates)
__device__ __forceinline__ double proj(double l, double u, double x) {
    const long long xk = dkey(x);
    return (dkey(l) >= xk) ? l : ((dkey(u) <= xk) ? u : x);
}
__device__ __forceinline__ double phi(double l, double u, double x, double g) { return (dlt(l, x) && dlt(x, u)) ? g : 0.0; }
// (|l - x| < 1e-14) ? min(0, g) : ((|u - x| < 1e-14) ? max(0, g) : 0)
__device__ __forceinline__ double chopped(double l, double u, double x, double g) {
    if (dabs_lt(l - x, 1e-14)) return dmin0(g);
    return dabs_lt(u - x, 1e-14) ? dmax0(g) : 0.0;
}

__device__ __forceinline__ void qp_stop(QpDev *d, int reason, int converged) {
    d->done = 1;
    d->reason = reason;
    d->converged = converged;
    d->iterates = d->it;
}

// initial: x = P(x); (then g = A x - b by SpMV); this kernel: fi, beta, p = fi, dots
__global__ void k_qp_project(int64_t n, const double *lb, const double *ub, double *x) {
    QP_LOOP(i, n) x[i] = proj(lb[i], ub[i], x[i]);
}

// the iteration's direction: p = fi - beta_sc p after a CG step, p = fi otherwise (neg_bsc = 0)
__global__ void __launch_bounds__(kBlock) k_mprgp_direction(int64_t n, double *p, const double *fi,
                                                           const QpDev *dev) {
    if (dev->done) return;
    const double nb = dev->neg_bsc;
    const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int64_t nth = int64_t(gridDim.x) * blockDim.x;
    const int64_t n2 = n >> 1;
    double2 *p2 = reinterpret_cast<double2 *>(p);
    const double2 *f2 = reinterpret_cast<const double2 *>(fi);
#pragma unroll 4
    for (int64_t j = tid; j < n2; j += nth) {
        const double2 pv = p2[j], fv = f2[j];
        p2[j] = make_double2(fma(nb, pv.x, fv.x), fma(nb, pv.y, fv.y));
    }
    if ((n & 1) && tid == 0) p[n - 1] = fma(nb, p[n - 1], fi[n - 1]);
}

// convergence test of the iteration that ends with the three dots s = {(beta, beta), (fi, fi),
// (gp, gp)} (check_convergence(it, gnorm, gnorm / gnorm0, 1)) and the next branch
__device__ __forceinline__ void mprgp_close_iteration(QpDev *dev, const double *s, double atol, double rtol,
                                                      long long max_it) {
    dev->beta_beta = s[0];
    dev->fi_fi = s[1];
    const double gnorm = sqrt(s[2]);
    dev->gnorm = gnorm;
    if (dev->it == 0) dev->gnorm0 = gnorm;
    dev->it += 1;
    const double rel = gnorm / dev->gnorm0;
    int reason = 0;
    if (gnorm <= atol) reason = UGPU_CONVERGED_FNORM_ABS;
    if (rel <= rtol) reason = UGPU_CONVERGED_FNORM_RELATIVE;
    if (dev->it >= max_it) reason = UGPU_DIVERGED_MAX_IT;
    if (reason) qp_stop(dev, reason, reason > 0);
    const int cgpath = s[0] <= s[1];  // beta_beta <= gamma^2 fi_fi, gamma = 1
    dev->gate_cg = cgpath;
    dev->gate_prop = !cgpath;
}

// One MPRGP iteration after its product (utopia_MPRGP.hpp:125-258).  The product kernel before it
// took s (p on the CG path, beta on the proportioning path) and formed q = A s, the dots
// qa0 = (s, q), qa1 = (s, g) and, on the CG path, the step bound alpha_f.  Every CTA takes the
// same decisions from those scalars:
//   negative curvature (qa0 <= 0)       -> stop
//   CG path, alpha_cg <= alpha_f (CG)   -> x -= alpha_cg p, g -= alpha_cg Ap, next fi, beta, dots;
//                                          p = fi - beta_sc p (beta_sc = (fi, Ap) / pAp) is formed by
//                                          the next iteration's direction kernel
//   CG path, expansion                  -> x = P(x - alpha_f p - alpha_bar phi(x - alpha_f p,
//                                          g - alpha_f Ap)); g = A x - b and the rest follow in
//                                          the gated product and closing kernels
//   proportioning path                  -> x -= alpha beta, g -= alpha A beta, p = fi
// and the last CTA closes the iteration (convergence, next branch, beta_sc, alpha_f reset).
__global__ void __launch_bounds__(kBlock) k_mprgp_step(int64_t n, double *x, double *g, const double *p,
                                                      double *fi, double *beta, const double *q,
                                                      const double *lb, const double *ub, double alpha_bar,
                                                      QpDev *dev, double *partials, unsigned int *counter,
                                                      double atol, double rtol, long long max_it) {
    if (dev->done) return;
    const int cg = dev->gate_cg;
    const double a0 = dev->qa0, a1 = dev->qa1;
    if (a0 <= 0.0) {
        // `if (pAp <= 0.0) return true;` / `if (beta_Abeta <= 0.0) return true;` (negative curvature)
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            qp_stop(dev, UGPU_DIVERGED_INDEFINITE, 1);
            dev->gate_exp = 0;
        }
        return;
    }
    // the step length and branch, from one thread per CTA (an FP64 division per thread would cost
    // the FP64 pipe about one operation per row)
    __shared__ double s_alpha;
    __shared__ int s_step;
    if (threadIdx.x == 0) {
        if (cg) {
            const double alpha_cg = a1 / a0;
            const double alpha_f = qp_unkey(dev->amin);
            const int st = (alpha_cg <= alpha_f) ? 0 : 1;
            s_alpha = st == 0 ? alpha_cg : alpha_f;
            s_step = st;
            if (blockIdx.x == 0) {
                dev->alpha_cg = alpha_cg;
                dev->alpha_f = alpha_f;
                dev->step = st;
                dev->gate_exp = st;
            }
        } else {
            s_alpha = a1 / a0;
            s_step = 0;
            if (blockIdx.x == 0) {
                dev->step = 0;
                dev->gate_exp = 0;
            }
        }
    }
    __syncthreads();
    const double alpha = s_alpha;
    const int step = s_step;
    double acc_fq = 0, acc_bb = 0, acc_ff = 0, acc_gg = 0;
    QP_LOOP(i, n) {
        const double l = lb[i], u = ub[i], xi = x[i], gi = g[i], qi = q[i];
        if (cg) {
            const double pn = p[i];  // the direction the product used
            const double xn = xi - alpha * pn;
            const double gn = gi - alpha * qi;
            if (step == 0) {
                x[i] = xn;
                g[i] = gn;
                const double f = phi(l, u, xn, gn);
                const double b = chopped(l, u, xn, gn);
                fi[i] = f;
                beta[i] = b;
                const double gp = f + b;
                acc_fq = fma(f, qi, acc_fq);
                acc_bb = fma(b, b, acc_bb);
                acc_ff = fma(f, f, acc_ff);
                acc_gg = fma(gp, gp, acc_gg);
            } else {
                x[i] = proj(l, u, xn - alpha_bar * phi(l, u, xn, gn));
            }
        } else {
            const double xn = xi - alpha * beta[i];
            const double gn = gi - alpha * qi;
            x[i] = xn;
            g[i] = gn;
            const double f = phi(l, u, xn, gn);
            const double b = chopped(l, u, xn, gn);
            fi[i] = f;
            beta[i] = b;
            const double gp = f + b;
            acc_bb = fma(b, b, acc_bb);
            acc_ff = fma(f, f, acc_ff);
            acc_gg = fma(gp, gp, acc_gg);
        }
    }
    double a[4] = {acc_fq, acc_bb, acc_ff, acc_gg};
    block_reduce_store<4>(a, 4, partials, gridDim.x, blockIdx.x);
    double s[4];
    if (finish_last_block(4, partials, gridDim.x, s, counter) && threadIdx.x == 0) {
        dev->amin = qp_key(DBL_MAX_D);
        if (cg && step == 1) return;  // expansion: closed by the gated product and closing kernels
        const double bsc = cg ? s[0] / a0 : 0.0;
        dev->beta_sc = bsc;
        dev->neg_bsc = -bsc;
        mprgp_close_iteration(dev, s + 1, atol, rtol, max_it);
    }
}

// fi = phi(x, g), beta, p = fi, the three dots and the next branch: the start of the solve
// (first = 1, no convergence test), and the end of an expansion step (first = 0: runs only when
// the step kernel chose the expansion, after g = A x - b)
__global__ void __launch_bounds__(kBlock) k_mprgp_final(int64_t n, const double *x, const double *g, double *p,
                                                       double *fi_out, double *beta, const double *lb,
                                                       const double *ub, QpDev *dev, double *partials,
                                                       unsigned int *counter, double atol, double rtol,
                                                       long long max_it, int first) {
    if (dev->done) return;
    if (!first && !dev->gate_exp) return;
    double a0 = 0, a1 = 0, a2 = 0;
    QP_LOOP(i, n) {
        const double l = lb[i], u = ub[i], xi = x[i], gi = g[i];
        const double fi = phi(l, u, xi, gi);
        const double bi = chopped(l, u, xi, gi);
        beta[i] = bi;
        p[i] = fi;
        fi_out[i] = fi;
        const double gp = fi + bi;
        a0 = fma(bi, bi, a0);
        a1 = fma(fi, fi, a1);
        a2 = fma(gp, gp, a2);
    }
    double a[3] = {a0, a1, a2};
    block_reduce_store<3>(a, 3, partials, gridDim.x, blockIdx.x);
    double s[3];
    if (finish_last_block(3, partials, gridDim.x, s, counter) && threadIdx.x == 0) {
        dev->neg_bsc = 0.0;
        dev->gate_exp = 0;
        dev->step = 0;
        if (first) {
            dev->beta_beta = s[0];
            dev->fi_fi = s[1];
            const int cgpath = s[0] <= s[1];
            dev->gate_cg = cgpath;
            dev->gate_prop = !cgpath;
        } else {
            mprgp_close_iteration(dev, s, atol, rtol, max_it);
        }
    }
}

// active-set compaction: flag[i] = row i is in the set, then the indices in ascending order
__global__ void k_set_flags(int64_t n, const double *x, const double *lb, const double *ub, int which,
                            int64_t *flag) {
    QP_LOOP(i, n) {
        const double l = lb ? lb[i] : -DBL_MAX_D, u = ub ? ub[i] : DBL_MAX_D, xi = x[i];
        const bool in = which == UGPU_SET_FREE ? (dlt(l, xi) && dlt(xi, u))
                                               : (dabs_lt(l - xi, 1e-14) || dabs_lt(u - xi, 1e-14));
        flag[i] = in ? 1 : 0;
    }
}
__global__ void k_set_scatter(int64_t n, const int64_t *flag, const int64_t *pos, int32_t *idx) {
    QP_LOOP(i, n) if (flag[i]) idx[pos[i]] = int32_t(i);
}

__global__ void k_qp_init(QpDev *d) {
    QpDev z{};
    z.gnorm = -1;
    z.gnorm0 = -1;
    z.amin = qp_key(DBL_MAX_D);
    *d = z;
}

// ------------------------------------------------------------------ PGS -------------
// multicolour projected sweep over the rows of one colour: c_i = clamp(dinv_i s_i, lo_i, hi_i) with
// s_i = r_i - sum_{j != i} a_ij c_j and the step bounds lo = lb - x, hi = ub - x of the current
// iterate (computed once per step); the clamp compares on the integer pipes
__global__ void __launch_bounds__(kBlock) k_pgs_colour(const int32_t *rows, int64_t nrows_c, const int32_t *rp,
                                                      const int32_t *ci, const double *cv, const double *r,
                                                      const double *dinv, const double *lo, const double *hi,
                                                      double *c, const int *done) {
    if (*done) return;
    QP_LOOP(q, nrows_c) {
        const int32_t i = rows[q];
        double s = r[i];
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int32_t j = ci[k];
            if (j != i) s -= cv[k] * c[j];
        }
        // fmax(fmin(v, hi), lo)
        double v = dinv[i] * s;
        const double h = hi[i], l = lo[i];
        v = dlt(h, v) ? h : v;
        v = dlt(v, l) ? l : v;
        c[i] = v;
    }
}

// The same sweep over a colour-sliced layout: the rows of one colour in ascending order, their
// off-diagonal entries slot-major (entry k of the colour's row q at k m + q: every slot is one
// coalesced load over the colour's rows), padded with (the row itself, 0), which subtracts an
// exact zero; the diagonal inverses, r and the step bounds compacted per colour (r_c, lo_c and
// hi_c start at the colour's first position), so only c is gathered.  Same operations in the same
// order as k_pgs_colour.
__global__ void __launch_bounds__(kBlock) k_pgs_colour_sliced(const int32_t *rows, int64_t m, int w,
                                                             const int32_t *cols, const double *vals,
                                                             const double *dinv_c, const double *r_c,
                                                             const double *lo_c, const double *hi_c, double *c,
                                                             const int *done) {
    if (*done) return;
    QP_LOOP(q, m) {
        const int32_t i = rows[q];
        double s = r_c[q];
        for (int k = 0; k < w; ++k) s -= vals[k * m + q] * c[cols[k * m + q]];
        double v = dinv_c[q] * s;
        const double h = hi_c[q], l = lo_c[q];
        v = dlt(h, v) ? h : v;
        v = dlt(v, l) ? l : v;
        c[i] = v;
    }
}

// the most off-diagonal entries of a row (the colour-sliced layout's width)
__global__ void k_pgs_max_row(const int32_t *rp, const int32_t *ci, int64_t n, unsigned int *mx) {
    unsigned int v = 0;
    QP_LOOP(i, n) {
        unsigned int k = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; ++e) k += ci[e] != int32_t(i) ? 1u : 0u;
        v = max(v, k);
    }
    v = __reduce_max_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) atomicMax(mx, v);
}

// the colour-sliced layout of one colour (k_pgs_colour_sliced), from the CSR rows (w the most
// off-diagonal entries of a row, so they always fit; shorter rows pad with zero entries), and
// each row's colour-ordered position
__global__ void k_pgs_slice_colour(const int32_t *rows, int64_t m, int64_t off, int w, const int32_t *rp,
                                   const int32_t *ci, const double *cv, const double *dinv, int32_t *cols,
                                   double *vals, double *dinv_c, int32_t *pos) {
    QP_LOOP(q, m) {
        const int32_t i = rows[q];
        pos[i] = int32_t(off + q);  // the row's colour-ordered position
        int k = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; ++e) {
            if (ci[e] == i) continue;
            cols[k * m + q] = ci[e];
            vals[k * m + q] = cv[e];
            ++k;
        }
        for (; k < w; ++k) {
            cols[k * m + q] = i;
            vals[k * m + q] = 0.0;
        }
        dinv_c[q] = dinv[i];
    }
}

// the step bounds lo = lb - x, hi = ub - x (smoothing steps; the solver's steps get them from
// the projected-gradient kernel)
__global__ void __launch_bounds__(kBlock) k_pgs_bounds(int64_t n, const double *x, const double *lb,
                                                      const double *ub, const double *r, double *lo, double *hi,
                                                      const int32_t *pos, double *r_c, const int *done) {
    if (*done) return;
    QP_LOOP(i, n) {
        const double xi = x[i];
        const int64_t j = pos ? int64_t(pos[i]) : i;
        lo[j] = lb[i] - xi;
        hi[j] = ub[i] - xi;
        if (pos) r_c[j] = r[i];
    }
}

struct PgsDev {
    double diff, pgnorm;
    long long it, iterates;
    int done, reason, converged, pad;
};

// x += c; ||x_new - x_old||; convergence (stol on the step, or atol on the projected gradient)
__global__ void __launch_bounds__(kBlock) k_pgs_finish(int64_t n, double *__restrict__ x,
                                                      const double *__restrict__ c, PgsDev *dev, double *partials,
                                                      unsigned int *counter, double stol, long long max_it,
                                                      int pg_stop) {
    if (dev->done) return;
    double acc = 0;
#pragma unroll 4
    QP_LOOP(i, n) {
        const double xo = x[i];
        const double xn = xo + c[i];
        x[i] = xn;
        const double d = xn - xo;
        acc = fma(d, d, acc);
    }
    double a[1] = {acc};
    block_reduce_store<1>(a, 1, partials, gridDim.x, blockIdx.x);
    double s[1];
    if (finish_last_block(1, partials, gridDim.x, s, counter) && threadIdx.x == 0) {
        const double diff = sqrt(s[0]);
        dev->diff = diff;
        // check_convergence(iteration, 1, 1, diff): stol on the step, then max_it
        int reason = 0;
        if (!pg_stop && diff <= stol) reason = UGPU_CONVERGED_SNORM_RELATIVE;
        if (dev->it >= max_it) reason = UGPU_DIVERGED_MAX_IT;
        if (reason) {
            dev->done = 1;
            dev->reason = reason;
            dev->converged = reason > 0;
            dev->iterates = dev->it;
        }
        dev->it += 1;
    }
}

// projected-gradient norm || P(x - g) - x || with g = -r (r = b - A x); optional stop test; the
// step's bounds lo = lb - x, hi = ub - x
// (pos: with the colour-sliced layout, lo, hi and a copy of r go to the rows' colour-ordered
// positions pos[i], where the colour passes read them contiguously; null: natural order, no copy)
__global__ void __launch_bounds__(kBlock) k_pgs_pgnorm(int64_t n, const double *x, const double *r, const double *lb,
                                                      const double *ub, double *lo, double *hi, const int32_t *pos,
                                                      double *r_c, PgsDev *dev, double *partials,
                                                      unsigned int *counter, double atol, int pg_stop) {
    if (dev->done) return;
    double acc = 0;
    QP_LOOP(i, n) {
        const double xi = x[i];
        const double l = lb[i], u = ub[i], ri = r[i];
        const double d = proj(l, u, xi + ri) - xi;
        acc = fma(d, d, acc);
        const int64_t j = pos ? int64_t(pos[i]) : i;
        lo[j] = l - xi;
        hi[j] = u - xi;
        if (pos) r_c[j] = ri;
    }
    double a[1] = {acc};
    block_reduce_store<1>(a, 1, partials, gridDim.x, blockIdx.x);
    double s[1];
    if (finish_last_block(1, partials, gridDim.x, s, counter) && threadIdx.x == 0) {
        const double pg = sqrt(s[0]);
        dev->pgnorm = pg;
        if (pg_stop && pg <= atol) {
            dev->done = 1;
            dev->reason = UGPU_CONVERGED_FNORM_ABS;
            dev->converged = 1;
            dev->iterates = dev->it;
        }
    }
}

// greedy colouring by dependency rounds: row i takes the smallest colour not used by its
// lower-index neighbours once all of them are coloured (the sequential first-fit result)
__global__ void k_colour_round(const int32_t *rp, const int32_t *ci, int64_t n, int *colour, unsigned int *left) {
    unsigned int mine = 0;
    QP_LOOP(i, n) {
        if (colour[i] >= 0) continue;
        unsigned long long used = 0;
        bool ready = true;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int32_t j = ci[k];
            if (j >= i) continue;
            const int cj = atomicAdd(&colour[j], 0);
            if (cj < 0) {
                ready = false;
                break;
            }
            if (cj < 64) used |= 1ull << cj;
        }
        if (!ready) {
            mine++;
            continue;
        }
        int cc = 0;
        while (cc < 63 && (used >> cc) & 1ull) ++cc;
        atomicExch(&colour[i], cc);
    }
    if (mine) atomicAdd(left, mine);
}

__global__ void k_colour_flags(const int *colour, int64_t n, int c, int64_t *flag) {
    QP_LOOP(i, n) flag[i] = (colour[i] == c) ? 1 : 0;
}

__global__ void k_colour_scatter(const int *colour, const int64_t *pos, int64_t n, int c, int32_t *rows) {
    QP_LOOP(i, n) if (colour[i] == c) rows[pos[i]] = int32_t(i);
}

__global__ void k_recip(int64_t n, const double *d, double *out) {
    QP_LOOP(i, n) out[i] = 1. / d[i];
}

__global__ void k_fill(int64_t n, double v, double *out) {
    QP_LOOP(i, n) out[i] = v;
}

}  // namespace

// ======================================================================================
class QpBase : public Solver {
public:
    QpBase(Context *c, int k) : Solver(c, k) {}
    void set_box(const Vec *lb, const Vec *ub) override {
        for (const Vec *v : {lb, ub})
            UGPU_CHECK(!v || v->dtype == UGPU_F64, UGPU_ERR_ARG, "box constraints must be FP64 vectors");
        lb_ = lb;
        ub_ = ub;
    }

protected:
    const Vec *lb_ = nullptr, *ub_ = nullptr;
    Buffer lbfill_, ubfill_;

    struct LoopKey {
        const void *p[4] = {nullptr, nullptr, nullptr, nullptr};
        double s = 0;
    };

    // run the solve as one device loop (rebuilt when the captured pointers change), or
    // eagerly with a host check per iteration; dev/host: the solver's device state
    template <class Body>
    void run_loop(DeviceLoop &loop, LoopKey &key, std::initializer_list<const void *> ptrs, double s, Body body,
                  const int *done, Buffer &dev, void *host, size_t bytes) {
        const int64_t max_it = int64_t(get("max_it"));
        if (get("use_graphs") != 0) {
            LoopKey k;
            int i = 0;
            for (auto *q : ptrs) k.p[i++] = q;
            k.s = s;
            if (!loop.built() || !std::equal(k.p, k.p + 4, key.p) || k.s != key.s) {
                // two iterations per body: the loop's tail kernel and conditional evaluation come once
                // per two iterations (every kernel is gated on the stop flag, so an iteration after the
                // stop does nothing); measured 3 % per MPRGP / PGS iteration at 1024^2
                loop.build(*ctx, [&] { body(); body(); }, done, int(std::min<int64_t>(max_it + 8, 1 << 30)));
                key = k;
            }
            loop.run(*ctx);
            UGPU_CUDA(cudaMemcpyAsync(host, dev.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        } else {
            for (int64_t it = 0;; ++it) {
                body();
                UGPU_CUDA(cudaMemcpyAsync(host, dev.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
                UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
                if (*static_cast<const int *>(static_cast<const void *>(static_cast<const char *>(host) +
                                                                        (reinterpret_cast<const char *>(done) -
                                                                         static_cast<const char *>(dev.ptr)))))
                    break;
                UGPU_CHECK(it <= max_it + 8, UGPU_ERR_INTERNAL, "stop flag never set");
            }
        }
    }

    // BoxConstraints::fill_empty_bounds: missing bounds become -+max double
    void bounds(int64_t n, const double **lb, const double **ub) {
        UGPU_CHECK(!lb_ || lb_->n == n, UGPU_ERR_ARG, "lower bound size mismatch");
        UGPU_CHECK(!ub_ || ub_->n == n, UGPU_ERR_ARG, "upper bound size mismatch");
        if (!lb_) {
            lbfill_.alloc(sizeof(double) * std::max<int64_t>(n, 1));
            k_fill<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, -DBL_MAX_D, lbfill_.as<double>());
            ctx->launches++;
        }
        if (!ub_) {
            ubfill_.alloc(sizeof(double) * std::max<int64_t>(n, 1));
            k_fill<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, DBL_MAX_D, ubfill_.as<double>());
            ctx->launches++;
        }
        *lb = lb_ ? lb_->as<double>() : lbfill_.as<double>();
        *ub = ub_ ? ub_->as<double>() : ubfill_.as<double>();
    }
};

class Mprgp final : public QpBase {
public:
    explicit Mprgp(Context *c) : QpBase(c, UGPU_SOLVER_MPRGP) {
        prm["eig_comp_tol"] = 1e-1;        // MPRGP(): eps_eig_est_(1e-1), power_method_max_it_(10)
        prm["power_method_max_it"] = 10;
        prm["use_graphs"] = 1;             // 1: the solve is one graph launch (conditional WHILE node)
        prm["lambda_max"] = 0;             // read-only: the power-method estimate of the last apply()
    }
    ~Mprgp() override {
        if (host_) cudaFreeHost(host_);
    }
    void set(const std::string &k, double v) override {
        Solver::set(k, v);
        loop_.reset();
    }
    double lambda_max = 0;

    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG, "MPRGP: square FP64 operator");
        op = A;
        const size_t b = sizeof(double) * std::max<int64_t>(A->nrows, 1);
        for (Buffer *v : {&fi_, &beta_, &p_, &Ap_, &g_, &h1_, &h2_}) v->alloc(b);
        dev_.alloc(sizeof(QpDev));
        part_.alloc(sizeof(double) * 8 * std::max(kSpmvDotGrid, kRedBlocks));
        cnt_.alloc(sizeof(unsigned int) * 8);
        UGPU_CUDA(cudaMemsetAsync(cnt_.ptr, 0, cnt_.bytes, ctx->stream));
        if (!host_) UGPU_CUDA(cudaMallocHost(&host_, sizeof(QpDev)));
        loop_.reset();
    }

    void apply(const Vec &rhs, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "MPRGP: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(rhs.n == n && x.n == n && rhs.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "MPRGP: FP64 vectors of the operator size");
        double t0 = now_s();
        int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        const double *lb, *ub;
        bounds(n, &lb, &ub);
        lambda_max = power_method();
        prm["lambda_max"] = lambda_max;
        alpha_bar_ = 1.95 / lambda_max;
        k_qp_project<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, lb, ub, x.as<double>());
        ctx->launches++;
        {   // g = A x - b
            SpmvArgs a;
            a.x = x.data();
            a.v = rhs.data();
            a.y = g_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_SUB;
            launch_spmv(*ctx, *op, a);
        }
        k_qp_init<<<1, 1, 0, ctx->stream>>>(dev_.as<QpDev>());
        ctx->launches++;
        // fi, beta, p = fi, (beta,beta), (fi,fi) and the first branch
        final_kernel(x.as<double>(), lb, ub, 1);
        rhs_ = rhs.as<double>();
        run_loop(loop_, key_, {x.data(), lb, ub, rhs_}, alpha_bar_, [&] { iteration(x.as<double>(), lb, ub); },
                 &dev_.as<QpDev>()->done, dev_, host_, sizeof(QpDev));
        st.iterates = host_->iterates;
        st.gradient_norm = host_->gnorm;
        st.relative_gradient_norm = host_->gnorm0 > 0 ? host_->gnorm / host_->gnorm0 : 1;
        st.step_norm = 1;
        st.reason = host_->reason;
        st.converged = host_->converged;
        st.spmv_count = host_->it;
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

private:
    Buffer fi_, beta_, p_, Ap_, g_, h1_, h2_, dev_, part_, cnt_;
    QpDev *host_ = nullptr;
    double alpha_bar_ = 1;
    const double *rhs_ = nullptr;
    DeviceLoop loop_;
    LoopKey key_;

    void final_kernel(double *x, const double *lb, const double *ub, int first) {
        const int64_t n = op->nrows;
        k_mprgp_final<<<reduce_grid(n), kBlock, 0, ctx->stream>>>(
            n, x, g_.as<double>(), p_.as<double>(), fi_.as<double>(), beta_.as<double>(), lb, ub, dev_.as<QpDev>(),
            part_.as<double>() + 6 * kSpmvDotGrid, cnt_.as<unsigned int>() + 3, get("atol"), get("rtol"),
            (long long)get("max_it"), first);
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
    }

    // one MPRGP iteration: the direction p = fi - beta_sc p; the product of p (CG path) or beta
    // (proportioning path, chosen on the device) with its two dots and, on the CG path, the step
    // bound alpha_f; the step kernel; and, after an expansion step only, g = A x - b and the closing
    // kernel
    void iteration(double *x, const double *lb, const double *ub) {
        const int64_t n = op->nrows;
        QpDev *dev = dev_.as<QpDev>();
        double *part = part_.as<double>();
        unsigned int *cnt = cnt_.as<unsigned int>();
        {   // p = fi - beta_sc p (or fi)
            const int gp = int(std::max<int64_t>(1, std::min<int64_t>((n / 2 + kBlock - 1) / kBlock,
                                                                      int64_t(ctx->sms) * 8)));
            k_mprgp_direction<<<gp, kBlock, 0, ctx->stream>>>(n, p_.as<double>(), fi_.as<double>(), dev);
            ctx->launches++;
            UGPU_LAUNCH_CHECK();
        }
        {
            SpmvArgs a;
            a.xmode = 3;
            a.x = p_.ptr;
            a.xalt = beta_.ptr;
            a.qmode = &dev->gate_cg;
            a.qx = x;
            a.qlb = lb;
            a.qub = ub;
            a.qmin = &dev->amin;
            a.y = Ap_.ptr;
            a.vec_dtype = UGPU_F64;
            a.dot_partials = part;
            a.dv = g_.ptr;
            a.dot_out = &dev->qa0;
            a.dot_counter = cnt + 0;
            a.done = &dev->done;
            launch_spmv(*ctx, *op, a);
        }
        k_mprgp_step<<<reduce_grid(n), kBlock, 0, ctx->stream>>>(
            n, x, g_.as<double>(), p_.as<double>(), fi_.as<double>(), beta_.as<double>(), Ap_.as<double>(), lb, ub,
            alpha_bar_, dev, part + 2 * kSpmvDotGrid, cnt + 4, get("atol"), get("rtol"), (long long)get("max_it"));
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
        {   // g = A x - b   [expansion step only]
            SpmvArgs a;
            a.x = x;
            a.v = rhs_;
            a.y = g_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_SUB;
            a.done = &dev->done;
            a.gate = &dev->gate_exp;
            launch_spmv(*ctx, *op, a);
        }
        final_kernel(x, lb, ub, 0);
    }

    // MPRGP::power_method (utopia_MPRGP.hpp:351-387)
    double power_method() {
        const int64_t n = op->nrows;
        Vec f1, f2, fi;
        for (Vec *v : {&f1, &f2, &fi}) {
            v->ctx = ctx;
            v->n = n;
        }
        f1.buf.borrow(h1_.ptr, h1_.bytes);
        f2.buf.borrow(h2_.ptr, h2_.bytes);
        fi.buf.borrow(fi_.ptr, fi_.bytes);
        launch_set(*ctx, f2, 1.0);
        auto dot = [&](const Vec &a, const Vec &b) {
            DotArgs d{};
            d.nd = 1;
            d.a[0] = a.data();
            d.b[0] = b.data();
            double v;
            host_dots(*ctx, n, d, &v);
            return v;
        };
        const double eps = get("eig_comp_tol");
        const int64_t max_it = int64_t(get("power_method_max_it"));
        double lambda = 0, lambda_old;
        int64_t it = 0;
        bool conv = false;
        while (!conv) {
            launch_convert(*ctx, f2.data(), UGPU_F64, f1.data(), UGPU_F64, n);  // help_f1 = help_f2
            SpmvArgs a;
            a.x = f1.data();
            a.y = f2.data();
            a.vec_dtype = UGPU_F64;
            launch_spmv(*ctx, *op, a);
            double s = 1.0 / std::sqrt(dot(f2, f2));
            launch_axpby(*ctx, n, s, f2, 0.0, f2);
            lambda_old = lambda;
            a.x = f2.data();
            a.y = f1.data();
            launch_spmv(*ctx, *op, a);
            lambda = dot(f2, f1);
            launch_convert(*ctx, f2.data(), UGPU_F64, fi.data(), UGPU_F64, n);
            launch_axpby(*ctx, n, -1.0, f1, 1.0, fi);  // fi = help_f2 - help_f1
            double gnorm = std::sqrt(dot(fi, fi));
            conv = (gnorm < eps) || (std::fabs(lambda_old - lambda) < eps) || it > max_it;
            it++;
        }
        return lambda;
    }
};

class Pgs final : public QpBase {
public:
    explicit Pgs(Context *c) : QpBase(c, UGPU_SOLVER_PGS) {
        prm["n_local_sweeps"] = 3;          // ProjectedGaussSeidel(): n_local_sweeps_(3)
        prm["use_symmetric_sweep"] = 1;
        prm["projected_gradient_stop"] = 0; // 1: stop on ||P(x - g) - x|| <= atol instead of the step
        prm["use_graphs"] = 1;              // 1: the solve is one graph launch (conditional WHILE node)
    }
    ~Pgs() override {
        if (host_) cudaFreeHost(host_);
    }
    void set(const std::string &k, double v) override {
        Solver::set(k, v);
        loop_.reset();
    }
    int ncolours = 0;
    std::vector<int64_t> colour_count;
    Buffer colour;  // int per row

    // ProjectedGaussSeidel::update -> init: d = diag(A), d_inv = 1/d; plus the colouring
    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG, "PGS: square FP64 operator");
        op = A;
        const int64_t n = A->nrows;
        Mat &M = const_cast<Mat &>(*A);
        ensure_diag(M);
        dinv_.alloc(sizeof(double) * std::max<int64_t>(n, 1));
        k_recip<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(n, M.diag.as<double>(), dinv_.as<double>());
        ctx->launches++;
        for (Buffer *v : {&r_, &c_, &lo_, &hi_}) v->alloc(sizeof(double) * std::max<int64_t>(n, 1));
        dev_.alloc(sizeof(PgsDev));
        part_.alloc(sizeof(double) * 2 * kRedBlocks);
        cnt_.alloc(sizeof(unsigned int) * 4);
        UGPU_CUDA(cudaMemsetAsync(cnt_.ptr, 0, cnt_.bytes, ctx->stream));
        if (!host_) UGPU_CUDA(cudaMallocHost(&host_, sizeof(PgsDev)));
        make_colouring();
        loop_.reset();
    }

    void apply(const Vec &rhs, Vec &x) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "PGS: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(rhs.n == n && x.n == n && rhs.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "PGS: FP64 vectors of the operator size");
        double t0 = now_s();
        int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        const double *lb, *ub;
        bounds(n, &lb, &ub);
        UGPU_CUDA(cudaMemsetAsync(dev_.ptr, 0, sizeof(PgsDev), ctx->stream));
        run_loop(loop_, key_, {x.data(), lb, ub, rhs.data()}, 0.0,
                 [&] { step(rhs.as<double>(), x.as<double>(), lb, ub, false); }, &dev_.as<PgsDev>()->done, dev_, host_,
                 sizeof(PgsDev));
        st.iterates = host_->iterates;
        st.gradient_norm = host_->pgnorm;
        st.step_norm = host_->diff;
        st.relative_gradient_norm = 1;
        st.reason = host_->reason;
        st.converged = host_->converged;
        st.spmv_count = host_->it;
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

    // ProjectedGaussSeidel::smooth with bounds (utopia_ProjectedGaussSeidel.hpp:52-69): `sweeps`
    // steps, no stopping test
    void smooth(const Vec &rhs, Vec &x, int sweeps) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "PGS: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(rhs.n == n && x.n == n && rhs.dtype == UGPU_F64 && x.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "PGS: FP64 vectors of the operator size");
        const double *lb, *ub;
        bounds(n, &lb, &ub);
        UGPU_CUDA(cudaMemsetAsync(dev_.ptr, 0, sizeof(PgsDev), ctx->stream));
        for (int s = 0; s < sweeps; ++s) step(rhs.as<double>(), x.as<double>(), lb, ub, true);
    }

    std::vector<int32_t> download_colouring() const {
        std::vector<int32_t> h(op->nrows);
        if (op->nrows)
            UGPU_CUDA(cudaMemcpy(h.data(), colour.ptr, sizeof(int32_t) * op->nrows, cudaMemcpyDeviceToHost));
        return h;
    }

private:
    Buffer dinv_, r_, c_, lo_, hi_, dev_, part_, cnt_, rows_;
    bool sliced_ = false;  // the colour passes read the colour-sliced layout
    int sliced_w_ = 0;
    Buffer slice_cols_, slice_vals_, dinv_c_, pos_, r_c_;  // layout, diagonal inverses, positions, r copy
    std::vector<int64_t> colour_off_;
    PgsDev *host_ = nullptr;
    DeviceLoop loop_;
    LoopKey key_;

    void make_colouring() {
        const int64_t n = op->nrows;
        colour.alloc(sizeof(int) * std::max<int64_t>(n, 1));
        UGPU_CUDA(cudaMemsetAsync(colour.ptr, 0xff, sizeof(int) * std::max<int64_t>(n, 1), ctx->stream));
        Buffer left;
        left.alloc(sizeof(unsigned int));
        unsigned int h = 1;
        int64_t rounds = 0;
        while (h && n) {
            UGPU_CUDA(cudaMemsetAsync(left.ptr, 0, sizeof(unsigned int), ctx->stream));
            for (int q = 0; q < 16; ++q) {
                k_colour_round<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
                    op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(), n, colour.as<int>(), left.as<unsigned int>());
                ctx->launches++;
            }
            UGPU_CUDA(cudaMemcpyAsync(&h, left.ptr, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
            rounds += 16;
            UGPU_CHECK(rounds <= 16 * (n + 16), UGPU_ERR_INTERNAL, "colouring did not finish");
        }
        UGPU_LAUNCH_CHECK();
        // colour-sorted row lists (ascending rows within a colour)
        std::vector<int32_t> hc(n);
        if (n) UGPU_CUDA(cudaMemcpy(hc.data(), colour.ptr, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        ncolours = 0;
        for (auto v : hc) ncolours = std::max(ncolours, v + 1);
        UGPU_CHECK(ncolours <= 63, UGPU_ERR_UNSUPPORTED, "PGS: more than 63 colours");
        rows_.alloc(sizeof(int32_t) * std::max<int64_t>(n, 1));
        Buffer flag, pos;
        flag.alloc(sizeof(int64_t) * std::max<int64_t>(n, 1));
        pos.alloc(sizeof(int64_t) * (n + 1));
        colour_off_.assign(ncolours + 1, 0);
        colour_count.assign(ncolours, 0);
        for (int c = 0; c < ncolours; ++c) {
            k_colour_flags<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(colour.as<int>(), n, c,
                                                                            flag.as<int64_t>());
            int64_t cnt = device_exclusive_scan(*ctx, flag.as<int64_t>(), pos.as<int64_t>(), n);
            k_colour_scatter<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
                colour.as<int>(), pos.as<int64_t>(), n, c, rows_.as<int32_t>() + colour_off_[c]);
            ctx->launches += 2;
            colour_count[c] = cnt;
            colour_off_[c + 1] = colour_off_[c] + cnt;
        }
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        // colour-sliced copies of the rows (off-diagonal entries slot-major per colour), when the
        // widest row keeps the padding small
        unsigned int hmax = 0;
        if (n) {
            Buffer mx;
            mx.alloc(sizeof(unsigned int));
            UGPU_CUDA(cudaMemsetAsync(mx.ptr, 0, sizeof(unsigned int), ctx->stream));
            k_pgs_max_row<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(op->rowptr.as<int32_t>(),
                                                                            op->colidx.as<int32_t>(), n,
                                                                            mx.as<unsigned int>());
            ctx->launches++;
            UGPU_CUDA(cudaMemcpyAsync(&hmax, mx.ptr, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        sliced_w_ = int(std::max(hmax, 1u));
        sliced_ = n > 0 && hmax <= 32;
        slice_cols_.release();
        slice_vals_.release();
        if (sliced_) {
            const size_t slots = size_t(sliced_w_) * size_t(n);
            slice_cols_.alloc(sizeof(int32_t) * slots);
            slice_vals_.alloc(sizeof(double) * slots);
            dinv_c_.alloc(sizeof(double) * size_t(n));
            pos_.alloc(sizeof(int32_t) * size_t(n));
            r_c_.alloc(sizeof(double) * size_t(n));
            for (int c = 0; c < ncolours; ++c) {
                const int64_t m = colour_count[c];
                if (!m) continue;
                const size_t base = size_t(sliced_w_) * size_t(colour_off_[c]);
                k_pgs_slice_colour<<<stream_grid(*ctx, m), kBlock, 0, ctx->stream>>>(
                    rows_.as<int32_t>() + colour_off_[c], m, colour_off_[c], sliced_w_, op->rowptr.as<int32_t>(),
                    op->colidx.as<int32_t>(), op->vals.as<double>(), dinv_.as<double>(),
                    slice_cols_.as<int32_t>() + base, slice_vals_.as<double>() + base,
                    dinv_c_.as<double>() + colour_off_[c], pos_.as<int32_t>());
                ctx->launches++;
            }
            UGPU_LAUNCH_CHECK();
        }
    }

    // The colour passes of one step: n_local_sweeps forward sweeps over the colours, each followed
    // by a backward one when symmetric.  A pass over colour k reads only the corrections of the
    // other colours, so a pass that repeats the one before it (the turn of a symmetric sweep, the
    // start of the next sweep) recomputes the same values and is dropped; empty colours too.
    std::vector<int> colour_passes() const {
        const int sweeps = int(get("n_local_sweeps"));
        const bool sym = get("use_symmetric_sweep") != 0;
        std::vector<int> seq;
        auto push = [&](int c) {
            if (colour_count[c] == 0) return;
            if (!seq.empty() && seq.back() == c) return;
            seq.push_back(c);
        };
        for (int il = 0; il < sweeps; ++il) {
            for (int c = 0; c < ncolours; ++c) push(c);
            if (sym)
                for (int c = ncolours - 1; c >= 0; --c) push(c);
        }
        return seq;
    }

    // ProjectedGaussSeidel::step (utopia_ProjectedGaussSeidel.hpp:197-318), multicolour
    // smoothing: no projected-gradient norm and no stopping test
    void step(const double *b, double *x, const double *lb, const double *ub, bool smoothing) {
        const int64_t n = op->nrows;
        PgsDev *dev = dev_.as<PgsDev>();
        const int pg_stop = !smoothing && get("projected_gradient_stop") != 0;
        {   // r = b - A x
            SpmvArgs a;
            a.x = x;
            a.v = b;
            a.y = r_.ptr;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_RESIDUAL;
            a.done = &dev->done;
            launch_spmv(*ctx, *op, a);
        }
        if (!smoothing) {
            k_pgs_pgnorm<<<reduce_grid(n), kBlock, 0, ctx->stream>>>(
                n, x, r_.as<double>(), lb, ub, lo_.as<double>(), hi_.as<double>(),
                sliced_ ? pos_.as<int32_t>() : nullptr, r_c_.as<double>(), dev, part_.as<double>(),
                cnt_.as<unsigned int>() + 0, get("atol"), pg_stop);
        } else {
            k_pgs_bounds<<<stream_grid(*ctx, n), kBlock, 0, ctx->stream>>>(
                n, x, lb, ub, r_.as<double>(), lo_.as<double>(), hi_.as<double>(),
                sliced_ ? pos_.as<int32_t>() : nullptr, r_c_.as<double>(), &dev->done);
        }
        ctx->launches++;
        enq_set(*ctx, UGPU_F64, n, 0.0, c_.ptr, &dev->done);
        for (int c : colour_passes()) {
            const int64_t m = colour_count[c];
            if (sliced_) {
                const size_t base = size_t(sliced_w_) * size_t(colour_off_[c]);
                const int64_t o = colour_off_[c];
                k_pgs_colour_sliced<<<stream_grid(*ctx, m), kBlock, 0, ctx->stream>>>(
                    rows_.as<int32_t>() + o, m, sliced_w_, slice_cols_.as<int32_t>() + base,
                    slice_vals_.as<double>() + base, dinv_c_.as<double>() + o, r_c_.as<double>() + o,
                    lo_.as<double>() + o, hi_.as<double>() + o, c_.as<double>(), &dev->done);
            } else {
                k_pgs_colour<<<stream_grid(*ctx, m), kBlock, 0, ctx->stream>>>(
                    rows_.as<int32_t>() + colour_off_[c], m, op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(),
                    op->vals.as<double>(), r_.as<double>(), dinv_.as<double>(), lo_.as<double>(),
                    hi_.as<double>(), c_.as<double>(), &dev->done);
            }
            ctx->launches++;
        }
        k_pgs_finish<<<reduce_grid(n), kBlock, 0, ctx->stream>>>(n, x, c_.as<double>(), dev,
                                                                 part_.as<double>() + kRedBlocks,
                                                                 cnt_.as<unsigned int>() + 1,
                                                                 smoothing ? -1.0 : get("stol"),
                                                                 smoothing ? LLONG_MAX : (long long)get("max_it"),
                                                                 pg_stop);
        ctx->launches++;
        UGPU_LAUNCH_CHECK();
    }
};

// ======================================================================================
// SemismoothNewton (utopia/solvers/nonlinear/constrained/quadratic_programming/
// utopia_SemismoothNewton_impl.hpp:74-207): primal-dual active-set Newton for
// min 1/2 x'Ax - b'x, lb <= x <= ub.  Per iteration: d_lb = x + lambda - lb, d_ub = x + lambda - ub;
// i is active at the lower (upper) bound when d_lb <= 0 (d_ub >= 0), its residual entry becomes
// lb_i - x_i (ub_i - x_i) and its row of A the identity row (set_zero_rows(mat, active, 1));
// solve mat c = residual, x += c; stop when the active set repeats (after the first
// iteration) or on ||c|| <= stol / max_it; residual = b - A x, lambda = active .* residual.
// The inner solver defaults to BiCGStab + Jacobi (the active rows make mat nonsymmetric), run
// to ||r|| <= linear_rtol * ||residual||; a caller-set solver (set_preconditioner slot) replaces it.
namespace {

__global__ void k_ssn_active(int64_t n, const double *__restrict__ x, const double *__restrict__ lam,
                             const double *__restrict__ lb, const double *__restrict__ ub, double *__restrict__ res,
                             double *__restrict__ active, int *changed) {
    int cnt = 0;
    QP_LOOP(i, n) {
        const bool prev = active[i] != 0.0;
        const double d_lb = x[i] + lam[i] - lb[i];
        const double d_ub = x[i] + lam[i] - ub[i];
        const bool alb = d_lb <= 0.0, aub = d_ub >= 0.0;
        const bool act = alb || aub;
        res[i] = alb ? (lb[i] - x[i]) : (aub ? (ub[i] - x[i]) : res[i]);
        active[i] = act ? 1.0 : 0.0;
        cnt += (prev != act);
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(changed, cnt);
}

__global__ void k_ssn_rows(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                           const double *__restrict__ a, const double *__restrict__ active, double *__restrict__ out) {
    QP_LOOP(i, n) {
        const bool act = active[i] != 0.0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) out[k] = act ? (ci[k] == i ? 1.0 : 0.0) : a[k];
    }
}

__global__ void k_ssn_lambda(int64_t n, const double *__restrict__ active, const double *__restrict__ res,
                             double *__restrict__ lam) {
    QP_LOOP(i, n) lam[i] = active[i] * res[i];
}

}  // namespace

class SemismoothNewton final : public QpBase {
public:
    explicit SemismoothNewton(Context *c) : QpBase(c, UGPU_SOLVER_SSNEWTON) {
        prm["linear_rtol"] = 1e-12;
        prm["linear_max_it"] = 10000;
    }

    void set_preconditioner(Solver *s) override { user_linear_ = s; }

    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols && A->vdtype == UGPU_F64, UGPU_ERR_ARG,
                   "SemismoothNewton: square FP64 operator required");
        op = A;
        mat_ = cast_matrix(*A, UGPU_F64);  // details_->mat = *op
        const size_t b = sizeof(double) * size_t(std::max<int64_t>(A->nrows, 1));
        for (Buffer *w : {&res_, &lam_, &active_, &corr_}) w->alloc(b);
        changed_.alloc(sizeof(int));
        if (!user_linear_ && !linear_) {
            linear_ = make_bicgstab(ctx);
            jacobi_ = make_invdiag(ctx);
            linear_->set_preconditioner(jacobi_.get());
        }
    }

    void apply(const Vec &bv, Vec &xv) override {
        UGPU_CHECK(op, UGPU_ERR_STATE, "SemismoothNewton: update() first");
        const int64_t n = op->nrows;
        UGPU_CHECK(bv.n == n && xv.n == n && bv.dtype == UGPU_F64 && xv.dtype == UGPU_F64, UGPU_ERR_ARG,
                   "SemismoothNewton: FP64 vectors of the operator's size required");
        const double t0 = now_s();
        const int64_t l0 = ctx->launches;
        st = ugpu_solution_status{};
        const double *lb, *ub;
        bounds(n, &lb, &ub);
        double *x = xv.as<double>(), *res = res_.as<double>(), *lam = lam_.as<double>();
        double *act = active_.as<double>(), *c = corr_.as<double>();
        Solver *lin = user_linear_ ? user_linear_ : linear_.get();
        const int g = stream_grid(*ctx, n);
        auto residual = [&]() {  // res = b - A x
            SpmvArgs a;
            a.x = x;
            a.v = bv.data();
            a.y = res;
            a.vec_dtype = UGPU_F64;
            a.epilogue = EPI_RESIDUAL;
            launch_spmv(*ctx, *op, a);
        };
        auto norm = [&](const double *v) {
            DotArgs d{};
            d.a[0] = d.b[0] = v;
            d.dtype_a[0] = d.dtype_b[0] = UGPU_F64;
            d.nd = 1;
            double o = 0;
            host_dots(*ctx, n, d, &o);
            return std::sqrt(o);
        };
        enq_set(*ctx, UGPU_F64, n, 0.0, lam, nullptr);
        enq_set(*ctx, UGPU_F64, n, 0.0, act, nullptr);  // Details::init: active zeroed
        residual();
        int64_t it = 0, lin_its = 0;
        bool converged = false;
        double norm_c = 0;
        Vec rv, cv;
        rv.ctx = cv.ctx = ctx;
        rv.n = cv.n = n;
        rv.dtype = cv.dtype = UGPU_F64;
        rv.buf.borrow(res, sizeof(double) * size_t(n));
        cv.buf.borrow(c, sizeof(double) * size_t(n));
        while (!converged) {
            UGPU_CUDA(cudaMemsetAsync(changed_.ptr, 0, sizeof(int), ctx->stream));
            k_ssn_active<<<g, kBlock, 0, ctx->stream>>>(n, x, lam, lb, ub, res, act, changed_.as<int>());
            k_ssn_rows<<<g, kBlock, 0, ctx->stream>>>(n, op->rowptr.as<int32_t>(), op->colidx.as<int32_t>(),
                                                      op->vals.as<double>(), act, mat_->vals.as<double>());
            ctx->launches += 2;
            UGPU_LAUNCH_CHECK();
            int changed = 0;
            UGPU_CUDA(cudaMemcpyAsync(&changed, changed_.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            refresh_values(*mat_);  // new values: refresh the sliced-ELL copy
            UGPU_CUDA(cudaStreamSynchronize(ctx->stream));  // `changed` is read below
            enq_set(*ctx, UGPU_F64, n, 0.0, c, nullptr);
            if (!user_linear_) {
                lin->set("atol", get("linear_rtol") * norm(res));
                lin->set("max_it", get("linear_max_it"));
            }
            lin->update(mat_.get());
            lin->apply(rv, cv);
            lin_its += lin->st.iterates;
            UGPU_CHECK(lin->st.converged, UGPU_ERR_INTERNAL,
                       "SemismoothNewton: unable to solve the linear system for the subgradient");
            enq_axpy(*ctx, UGPU_F64, n, 1.0, c, x, nullptr);  // x += correction
            norm_c = norm(c);
            ++it;
            if (it > 1 && !changed) {
                converged = true;
                st.iterates = it;
                st.step_norm = norm_c;
                st.reason = UGPU_CONVERGED_SNORM_RELATIVE;
            } else {
                converged = check_convergence(it, 1, 1, norm_c);
            }
            residual();
            k_ssn_lambda<<<g, kBlock, 0, ctx->stream>>>(n, act, res, lam);
            ctx->launches++;
        }
        UGPU_CUDA(cudaStreamSynchronize(ctx->stream));
        st.converged = st.reason > 0 ? 1 : 0;
        st.spmv_count = lin_its;  // inner iterations
        st.execution_time = now_s() - t0;
        st.kernel_launches = ctx->launches - l0;
    }

private:
    std::unique_ptr<Mat> mat_;
    Buffer res_, lam_, active_, corr_, changed_;
    Solver *user_linear_ = nullptr;
    std::unique_ptr<Solver> linear_, jacobi_;
};

std::unique_ptr<Solver> make_ssnewton(Context *c) { return std::make_unique<SemismoothNewton>(c); }

std::unique_ptr<Solver> make_mprgp(Context *c) { return std::make_unique<Mprgp>(c); }
std::unique_ptr<Solver> make_pgs(Context *c) { return std::make_unique<Pgs>(c); }

// indices of the active (chopped) or free set of x in [lb, ub], ascending, into a device array;
// returns their number (synchronous)
int64_t active_set_compact(Context &ctx, int64_t n, const double *x, const double *lb, const double *ub, int which,
                           int32_t *idx) {
    if (n == 0) return 0;
    Buffer flag, pos;
    flag.alloc(sizeof(int64_t) * n);
    pos.alloc(sizeof(int64_t) * (n + 1));  // the scan also writes the total at pos[n]
    const int g = stream_grid(ctx, n);
    k_set_flags<<<g, kBlock, 0, ctx.stream>>>(n, x, lb, ub, which, flag.as<int64_t>());
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    const int64_t cnt = device_exclusive_scan(ctx, flag.as<int64_t>(), pos.as<int64_t>(), n);
    if (idx && cnt) {
        k_set_scatter<<<g, kBlock, 0, ctx.stream>>>(n, flag.as<int64_t>(), pos.as<int64_t>(), idx);
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    return cnt;
}

std::vector<int32_t> pgs_colouring(const Solver *s, int *ncolours) {
    auto p = dynamic_cast<const Pgs *>(s);
    UGPU_CHECK(p, UGPU_ERR_ARG, "not a projected Gauss-Seidel solver");
    UGPU_CHECK(p->op, UGPU_ERR_STATE, "update() first");
    *ncolours = p->ncolours;
    return p->download_colouring();
}

}  // namespace ugpu

using namespace ugpu;

extern "C" int ugpu_pgs_colouring(const ugpu_solver *s, int32_t *colour, int *ncolours) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(s);
    UGPU_REQUIRE(ncolours);
    auto v = pgs_colouring(s->impl.get(), ncolours);
    if (colour) std::copy(v.begin(), v.end(), colour);
    UGPU_ABI_END(s ? s->impl->ctx : nullptr)
}

extern "C" int ugpu_active_set_compact(const ugpu_vec *x, const ugpu_vec *lb, const ugpu_vec *ub, int which,
                                       int32_t *indices, int64_t *count) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(count);
    UGPU_CHECK(which == UGPU_SET_ACTIVE || which == UGPU_SET_FREE, UGPU_ERR_ARG, "active_set_compact: which");
    UGPU_CHECK(x->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "active_set_compact: FP64 vectors");
    const int64_t n = x->impl.n;
    UGPU_CHECK(n < (int64_t(1) << 31), UGPU_ERR_ARG, "active_set_compact: int32 indices");
    for (const ugpu_vec *b : {lb, ub})
        UGPU_CHECK(!b || (b->impl.n == n && b->impl.dtype == UGPU_F64), UGPU_ERR_ARG,
                   "active_set_compact: bounds of the vector's size, FP64");
    *count = active_set_compact(*x->impl.ctx, n, x->impl.as<double>(), lb ? lb->impl.as<double>() : nullptr,
                                ub ? ub->impl.as<double>() : nullptr, which, indices);
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}
