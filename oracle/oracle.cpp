// CPU oracle for the utopia sparse-solver hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++ over FP64 CSR arrays, the algorithms of the
// reference's solver templates and the PETSc kernels they call.  It is the
// checker for the GPU library (tests, smoke() and the CPU-baseline leg of the
// benchmark load it); the GPU library never links or calls it.
//
// The restatement is pinned against the reference itself: oracle/ref/ compiles
// the reference's own solver templates, unchanged, over a CPU CSR backend that
// restates the PETSc kernels they call (PETSc 3.20.2 is not available), and
// tests/test_oracle_ref.py checks that both agree bit for bit (iterations,
// solutions, Galerkin operators, active sets) on the workloads' problems.
//
// Reduction order: every dot / norm sums fixed blocks of ORACLE_BLK entries in
// index order and then the block partials in order, so results do not depend on
// the OpenMP thread count.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int64_t ORACLE_BLK = 8192;

// ------------------------------------------------------------------------------------
// bf16 storage helpers (round to nearest even), used by the mixed-precision restatement
// ------------------------------------------------------------------------------------
struct bf16 {
    uint16_t bits;
};
inline float bf16_to_float(bf16 h) {
    uint32_t u = uint32_t(h.bits) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline bf16 float_to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return bf16{uint16_t((u >> 16) | 0x40)};  // NaN
    uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    return bf16{uint16_t(u >> 16)};
}
template <class V>
inline double to_d(V v) { return double(v); }
template <>
inline double to_d<bf16>(bf16 v) { return double(bf16_to_float(v)); }
template <class V>
inline float to_f(V v) { return float(v); }
template <>
inline float to_f<bf16>(bf16 v) { return bf16_to_float(v); }
template <class V>
inline V from_d(double d) { return V(d); }
template <>
inline bf16 from_d<bf16>(double d) { return float_to_bf16(float(d)); }

// ------------------------------------------------------------------------------------
// glibc rand() restatement (TYPE_3 additive feedback generator, degree 31, separation 3)
// Used for PowerMethod's initial vector, utopia/solvers/eigensolvers/utopia_PowerMethod.hpp:99-106
// (std::rand() / RAND_MAX + 1 in index order).
// ------------------------------------------------------------------------------------
struct GlibcRand {
    int32_t r[34];
    int i = 0;  // ring position
    uint32_t ring[31];
    int f = 3, b = 0;
    explicit GlibcRand(uint32_t seed = 1) {
        if (seed == 0) seed = 1;
        int32_t s[31];
        s[0] = int32_t(seed);
        int64_t word = seed;
        for (int k = 1; k < 31; ++k) {
            int64_t hi = word / 127773, lo = word % 127773;
            word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            s[k] = int32_t(word);
        }
        for (int k = 0; k < 31; ++k) ring[k] = uint32_t(s[k]);
        f = 3;
        b = 0;
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

// ------------------------------------------------------------------------------------
// CSR container
// ------------------------------------------------------------------------------------
template <class V>
struct CsrT {
    int64_t n = 0, m = 0;
    std::vector<int32_t> rp, ci;
    std::vector<V> v;
    int64_t nnz() const { return int64_t(ci.size()); }
};
using Csr = CsrT<double>;

template <class V>
CsrT<V> cast_csr(const Csr &a) {
    CsrT<V> b;
    b.n = a.n;
    b.m = a.m;
    b.rp = a.rp;
    b.ci = a.ci;
    b.v.resize(a.v.size());
    for (size_t k = 0; k < a.v.size(); ++k) b.v[k] = from_d<V>(a.v[k]);
    return b;
}

// y = A x  (PETSc MatMult, utopia/backend/petsc/utopia_petsc_Matrix.cpp:1358): row-ordered sums
template <class T, class V>
void spmv(const CsrT<V> &A, const T *x, T *y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        T s = 0;
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += T(to_d(A.v[k])) * x[A.ci[k]];
        y[i] = s;
    }
}

// r = b - A x  (Eval_Residual, utopia/utopia_core/eval/utopia_Eval_Residual.hpp:19-38)
template <class T, class V>
void residual(const CsrT<V> &A, const T *b, const T *x, T *r) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        T s = 0;
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += T(to_d(A.v[k])) * x[A.ci[k]];
        r[i] = b[i] - s;
    }
}

template <class T>
double dot(int64_t n, const T *a, const T *b) {
    int64_t nb = (n + ORACLE_BLK - 1) / ORACLE_BLK;
    std::vector<double> part(std::max<int64_t>(nb, 1), 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t bi = 0; bi < nb; ++bi) {
        double s = 0;
        int64_t e = std::min(n, (bi + 1) * ORACLE_BLK);
        for (int64_t i = bi * ORACLE_BLK; i < e; ++i) s += double(a[i]) * double(b[i]);
        part[bi] = s;
    }
    double s = 0;
    for (int64_t bi = 0; bi < nb; ++bi) s += part[bi];
    return s;
}
template <class T>
double norm2(int64_t n, const T *a) { return std::sqrt(dot(n, a, a)); }

// CSR transpose (explicit R = transpose(I) of IPRTransfer,
// utopia/solvers/multilevel/transfer/utopia_IPRTransfer.hpp:28-39); columns come out sorted.
Csr transpose(const Csr &A) {
    Csr T;
    T.n = A.m;
    T.m = A.n;
    T.rp.assign(A.m + 1, 0);
    for (int32_t c : A.ci) T.rp[c + 1]++;
    for (int64_t i = 0; i < A.m; ++i) T.rp[i + 1] += T.rp[i];
    T.ci.resize(A.nnz());
    T.v.resize(A.nnz());
    std::vector<int32_t> pos(T.rp.begin(), T.rp.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            int32_t p = pos[A.ci[k]]++;
            T.ci[p] = int32_t(i);
            T.v[p] = A.v[k];
        }
    return T;
}

// C = A B with the full symbolic structure (every structurally produced entry is kept,
// including numerical zeros, as PETSc's MatMatMult/MatPtAP symbolic phase does),
// columns sorted ascending.
Csr spgemm(const Csr &A, const Csr &B) {
    Csr C;
    C.n = A.n;
    C.m = B.m;
    C.rp.assign(A.n + 1, 0);
    std::vector<std::vector<int32_t>> rows_c(A.n);
    std::vector<std::vector<double>> rows_v(A.n);
#pragma omp parallel
    {
        std::vector<int64_t> mark(B.m, -1);
        std::vector<double> acc(B.m, 0.0);
        std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < A.n; ++i) {
            cols.clear();
            for (int32_t ka = A.rp[i]; ka < A.rp[i + 1]; ++ka) {
                int32_t j = A.ci[ka];
                double a = A.v[ka];
                for (int32_t kb = B.rp[j]; kb < B.rp[j + 1]; ++kb) {
                    int32_t c = B.ci[kb];
                    if (mark[c] != i) {
                        mark[c] = i;
                        acc[c] = 0.0;
                        cols.push_back(c);
                    }
                    acc[c] += a * B.v[kb];
                }
            }
            std::sort(cols.begin(), cols.end());
            rows_c[i] = cols;
            rows_v[i].resize(cols.size());
            for (size_t q = 0; q < cols.size(); ++q) rows_v[i][q] = acc[cols[q]];
        }
    }
    for (int64_t i = 0; i < A.n; ++i) C.rp[i + 1] = C.rp[i] + int32_t(rows_c[i].size());
    C.ci.resize(C.rp[A.n]);
    C.v.resize(C.rp[A.n]);
    for (int64_t i = 0; i < A.n; ++i) {
        std::copy(rows_c[i].begin(), rows_c[i].end(), C.ci.begin() + C.rp[i]);
        std::copy(rows_v[i].begin(), rows_v[i].end(), C.v.begin() + C.rp[i]);
    }
    return C;
}

// A_c = P^T A P (utopia::ptap -> MatPtAP, utopia/backend/petsc/eval/utopia_petsc_Eval_Multiply.cpp:12-61)
Csr ptap(const Csr &A, const Csr &P) {
    Csr R = transpose(P);
    Csr AP = spgemm(A, P);
    return spgemm(R, AP);
}

// diag(A) (MatGetDiagonal, utopia/backend/petsc/utopia_petsc_Matrix.cpp:756); 0 where absent
std::vector<double> diag(const Csr &A) {
    std::vector<double> d(A.n, 0.0);
    for (int64_t i = 0; i < A.n; ++i)
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.ci[k] == i) d[i] = A.v[k];
    return d;
}

// e_pseudo_inv (utopia/utopia_core/utopia_ElementWisePseudoInverse.hpp:20-48)
void pseudo_inv(std::vector<double> &d, double tol) {
    for (auto &v : d) v = (std::fabs(v) > tol) ? 1.0 / v : 0.0;
}

// ------------------------------------------------------------------------------------
// Dense Cholesky (coarse-level direct solve; the reference uses PETSc Factorization,
// utopia/backend/petsc/solvers/linear/utopia_petsc_Factorization.hpp)
// ------------------------------------------------------------------------------------
struct Cholesky {
    int64_t n = 0;
    std::vector<double> L;  // row-major lower triangle
    bool ok = false;
    bool factor(const Csr &A) {
        n = A.n;
        L.assign(n * n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) L[i * n + A.ci[k]] = A.v[k];
        for (int64_t j = 0; j < n; ++j) {
            double s = L[j * n + j];
            for (int64_t k = 0; k < j; ++k) s -= L[j * n + k] * L[j * n + k];
            if (!(s > 0.0)) return ok = false;
            double ljj = std::sqrt(s);
            L[j * n + j] = ljj;
#pragma omp parallel for schedule(static)
            for (int64_t i = j + 1; i < n; ++i) {
                double t = L[i * n + j];
                for (int64_t k = 0; k < j; ++k) t -= L[i * n + k] * L[j * n + k];
                L[i * n + j] = t / ljj;
            }
        }
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = i + 1; j < n; ++j) L[i * n + j] = 0.0;
        return ok = true;
    }
    void solve(const double *b, double *x) const {
        std::vector<double> y(n);
        for (int64_t i = 0; i < n; ++i) {
            double s = b[i];
            for (int64_t k = 0; k < i; ++k) s -= L[i * n + k] * y[k];
            y[i] = s / L[i * n + i];
        }
        for (int64_t i = n - 1; i >= 0; --i) {
            double s = y[i];
            for (int64_t k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
            x[i] = s / L[i * n + i];
        }
    }
};

// ------------------------------------------------------------------------------------
// Solver status (utopia/solvers/utopia_SolutionStatus.hpp) and convergence reasons
// (utopia/solvers/utopia_ConvergenceReason.hpp)
// ------------------------------------------------------------------------------------
enum Reason : int {
    CONVERGED_FNORM_ABS = 2,
    CONVERGED_FNORM_RELATIVE = 3,
    CONVERGED_SNORM_RELATIVE = 4,
    DIVERGED_MAX_IT = -5,
    DIVERGED_NAN = -6,
    DIVERGED_INDEFINITE = -8,
};

struct Params {
    double atol = 1e-9, rtol = 1e-9, stol = 1e-11;  // IterativeSolver defaults, utopia_IterativeSolver.hpp:226-229
    int64_t max_it = 1000;
    int64_t norm_freq = 1;
};

}  // namespace

extern "C" {
struct or_status {
    int64_t iterates;
    double gradient_norm;
    double relative_gradient_norm;
    double step_norm;
    int32_t reason;
    int32_t converged;
    int64_t spmv_count;
};
}

namespace {

// IterativeSolver::check_convergence, utopia/solvers/linear/utopia_IterativeSolver.hpp:148-191
bool check_convergence(const Params &p, or_status &st, int64_t it, double g, double r, double s) {
    bool conv = false;
    int reason = 0;
    bool compute = p.norm_freq != 0 && (it % p.norm_freq == 0);
    if (compute) {
        if (g <= p.atol) { reason = CONVERGED_FNORM_ABS; conv = true; }
        if (s <= p.stol) { reason = CONVERGED_SNORM_RELATIVE; conv = true; }
        if (r <= p.rtol) { reason = CONVERGED_FNORM_RELATIVE; conv = true; }
    }
    if (it >= p.max_it) { reason = DIVERGED_MAX_IT; conv = true; }
    if (conv) {
        st.iterates = it;
        st.gradient_norm = g;
        st.relative_gradient_norm = r;
        st.step_norm = s;
        st.reason = reason;
    }
    return conv;
}

// ------------------------------------------------------------------------------------
// Preconditioner interface
// ------------------------------------------------------------------------------------
struct Precond {
    virtual ~Precond() = default;
    virtual void apply(const double *r, double *z) = 0;  // z = M^{-1} r (z zeroed by caller)
};

// InvDiagPreconditioner, utopia/solvers/preconditioners/utopia_TrivialPreconditioners.hpp:20-56
struct InvDiag : Precond {
    std::vector<double> d;
    explicit InvDiag(const Csr &A) {
        d = diag(A);
        pseudo_inv(d, std::numeric_limits<double>::epsilon());
    }
    void apply(const double *r, double *z) override {
        int64_t n = int64_t(d.size());
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) z[i] = d[i] * r[i];
    }
};

// ConjugateGradient::preconditioned_solve, utopia/solvers/smoothers/utopia_ConjugateGradient_impl.hpp:195-294
bool pcg(const Csr &A, const double *b, double *x, Precond &M, const Params &prm, or_status &st) {
    const int64_t n = A.n;
    std::vector<double> r(n), z(n, 0.0), z_new(n, 0.0), p(n), Ap(n), r_new(n);
    int64_t it = 0;
    double alpha, beta, r_norm = 9e9;
    st = or_status{};
    residual(A, b, x, r.data());
    st.spmv_count++;
    M.apply(r.data(), z.data());
    p = z;
    bool stop = false;
    double rz = dot(n, r.data(), z.data());
    while (!stop) {
        spmv(A, p.data(), Ap.data());
        st.spmv_count++;
        alpha = rz / dot(n, p.data(), Ap.data());
        if (std::isinf(alpha) || std::isnan(alpha)) {
            stop = check_convergence(prm, st, it, r_norm, 1, 1);
            if (!stop) st.reason = DIVERGED_NAN;
            break;
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r_new[i] = r[i] - alpha * Ap[i];
        }
        r_norm = norm2(n, r_new.data());
        if (r_norm <= prm.atol) {
            stop = check_convergence(prm, st, it, r_norm, 1, 1);
            break;
        }
        std::fill(z_new.begin(), z_new.end(), 0.0);
        M.apply(r_new.data(), z_new.data());
        double rz_new = dot(n, z_new.data(), r_new.data());
        beta = rz_new / rz;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) p[i] = z_new[i] + beta * p[i];
        std::swap(r, r_new);
        std::swap(z, z_new);
        rz = rz_new;
        stop = check_convergence(prm, st, it, r_norm, 1, 1);
        it++;
    }
    st.converged = r_norm <= prm.atol;
    st.gradient_norm = r_norm;
    return st.converged;
}

// ConjugateGradient::unpreconditioned_solve, utopia_ConjugateGradient_impl.hpp:90-192
bool cg_plain(const Csr &A, const double *b, double *x, const Params &prm, or_status &st) {
    const int64_t n = A.n;
    std::vector<double> r(n), p(n, 0.0), q(n);
    st = or_status{};
    double rho, rho_1 = 1, beta, alpha, r_norm;
    residual(A, b, x, r.data());
    st.spmv_count++;
    r_norm = norm2(n, r.data());
    int64_t it = 1;
    bool converged = false;
    while (!converged) {
        rho = dot(n, r.data(), r.data());
        if (rho == 0.) { converged = true; break; }
        if (it > 1) {
            beta = rho / rho_1;
            for (int64_t i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
        } else {
            p = r;
        }
        spmv(A, p.data(), q.data());
        st.spmv_count++;
        double pq = dot(n, p.data(), q.data());
        if (pq == 0.) { converged = true; break; }
        alpha = rho / pq;
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        rho_1 = rho;
        r_norm = norm2(n, r.data());
        converged = check_convergence(prm, st, it, r_norm, 1, 1);
        it++;
    }
    st.converged = converged;
    st.gradient_norm = r_norm;
    return converged;
}

// ------------------------------------------------------------------------------------
// Multigrid (utopia/solvers/multilevel/utopia_Multigrid.hpp) templated on the working
// scalar T and the level-matrix storage V.  Level 0 is the coarsest level.
// ------------------------------------------------------------------------------------
enum SmootherKind { SM_JACOBI = 0, SM_CHEBYSHEV = 1, SM_POINT_JACOBI = 2 };

struct MgOptions {
    int smoother = SM_CHEBYSHEV;
    int pre = 3, post = 3;  // MultiLevelBase defaults, utopia_MultiLevelBase.hpp:35-42
    double omega = 1.0;     // Jacobi relaxation (1 = the reference's Jacobi)
    double scale_max_eig = 1.2, scale_min_eig = 0.06;  // Chebyshev3level.hpp:183
    double pm_tol = 1e-2;
    int64_t pm_max_it = 30;  // PowerMethod.hpp:150-151
    int fix_semidefinite = 0;
    int masks = 1;
};

template <class T, class V>
struct Mg : Precond {
    int L = 0;
    MgOptions opt;
    std::vector<Csr> A64;        // FP64 level operators (Galerkin products)
    std::vector<CsrT<V>> A;      // storage copies used in the cycle
    std::vector<CsrT<V>> LU;     // PointJacobi off-diagonal operators
    std::vector<CsrT<V>> P, R;   // transfer l: level l <-> level l+1
    std::vector<std::vector<T>> mask, dinv;
    std::vector<double> eig_max, eig_min;
    Cholesky coarse;
    std::vector<std::vector<T>> r, c, cI, rR, help, pp, rc;  // per-level work vectors
    int64_t spmv_count = 0;

    // LinearMultiLevel::galerkin_assembly, utopia_LinearMultiLevel.hpp:201-226
    bool build(const Csr &Afine, const std::vector<Csr> &Pco2fi, const MgOptions &o) {
        opt = o;
        L = int(Pco2fi.size()) + 1;
        std::vector<Csr> lev;
        lev.push_back(Afine);
        for (int i = 1; i < L; ++i) {
            Csr Jh = ptap(lev[i - 1], Pco2fi[L - 1 - i]);
            if (opt.fix_semidefinite) fix_semidefinite(Jh);
            lev.push_back(std::move(Jh));
        }
        std::reverse(lev.begin(), lev.end());
        A64 = lev;
        A.clear();
        for (auto &a : A64) A.push_back(cast_csr<V>(a));
        P.clear();
        R.clear();
        for (int l = 0; l < L - 1; ++l) {
            P.push_back(cast_csr<V>(Pco2fi[l]));
            R.push_back(cast_csr<V>(transpose(Pco2fi[l])));
        }
        make_masks(Pco2fi);
        // Multigrid::update(), utopia_Multigrid.hpp:142-153: smoothers on levels 1..L-1, in order
        dinv.assign(L, {});
        eig_max.assign(L, 0.0);
        eig_min.assign(L, 0.0);
        LU.assign(L, CsrT<V>{});
        GlibcRand rng(1);
        for (int l = 1; l < L; ++l) {
            std::vector<double> d = diag(A64[l]);
            if (opt.smoother == SM_JACOBI) {
                pseudo_inv(d, 0.0);  // Jacobi::update passes tol 0, utopia_Jacobi.hpp:99-110
                dinv[l].resize(d.size());
                for (size_t i = 0; i < d.size(); ++i) dinv[l][i] = T(opt.omega * d[i]);
            } else if (opt.smoother == SM_POINT_JACOBI) {
                // PointJacobi::update, utopia_PointJacobi.hpp:80-101: LU = A - diag(A), d_inv = 1/d (0 -> 1)
                Csr lu = A64[l];
                for (int64_t i = 0; i < lu.n; ++i)
                    for (int32_t k = lu.rp[i]; k < lu.rp[i + 1]; ++k)
                        if (lu.ci[k] == i) lu.v[k] = 0.0;
                LU[l] = cast_csr<V>(lu);
                dinv[l].resize(d.size());
                for (size_t i = 0; i < d.size(); ++i) {
                    double v = 1.0 / d[i];
                    if (v == 0) v = 1;
                    dinv[l][i] = T(v);
                }
            } else {
                power_method(l, rng);
            }
        }
        if (!coarse.factor(A64[0])) return false;
        int64_t maxn = 0;
        r.assign(L, {}); c.assign(L, {}); cI.assign(L, {}); rR.assign(L, {});
        help.assign(L, {}); pp.assign(L, {}); rc.assign(L, {});
        for (int l = 0; l < L; ++l) {
            int64_t n = A64[l].n;
            maxn = std::max(maxn, n);
            r[l].assign(n, 0); c[l].assign(n, 0); cI[l].assign(n, 0); rR[l].assign(n, 0);
            help[l].assign(n, 0); pp[l].assign(n, 0); rc[l].assign(n, 0);
        }
        return true;
    }

    // LinearMultiLevel::fix_semidefinite_operator, utopia_LinearMultiLevel.hpp:89-128
    static void fix_semidefinite(Csr &A) {
        for (int64_t i = 0; i < A.n; ++i)
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
                if (A.ci[k] == i && std::fabs(A.v[k]) < 1e-12) A.v[k] += 1.0;
    }

    // MultiLevelMask::generate_masks, utopia/solvers/multilevel/utopia_MultiLevelMask.hpp:39-115
    void make_masks(const std::vector<Csr> &Pco2fi) {
        mask.assign(L, {});
        const double tol = std::numeric_limits<double>::epsilon() * 1e6;
        std::vector<std::vector<double>> m(L);
        const Csr &Af = A64[L - 1];
        m[L - 1].assign(Af.n, 1.0);
        for (int64_t i = 0; i < Af.n; ++i)
            for (int32_t k = Af.rp[i]; k < Af.rp[i + 1]; ++k)
                if (Af.ci[k] != i && std::fabs(Af.v[k]) > tol) m[L - 1][i] = 0.0;
        for (int l = L - 1; l > 0; --l) {
            Csr Rb = transpose(Pco2fi[l - 1]);
            for (auto &v : Rb.v) v = double(std::fabs(v) > tol);
            m[l - 1].assign(Rb.n, 0.0);
            spmv(Rb, m[l].data(), m[l - 1].data());
            for (auto &v : m[l - 1]) if (v > 1.) v = 1.;
        }
        for (int l = 0; l < L; ++l) {
            mask[l].resize(m[l].size());
            for (size_t i = 0; i < m[l].size(); ++i) mask[l][i] = T(std::fabs(m[l][i] - 1.0));
        }
    }

    // PowerMethod::get_max_eig / compute_max_eig, utopia/solvers/eigensolvers/utopia_PowerMethod.hpp:95-146,
    // then Chebyshev3level::init_eigs, utopia/solvers/smoothers/utopia_Chebyshev3level.hpp:118-121
    void power_method(int l, GlibcRand &rng) {
        const Csr &Al = A64[l];
        int64_t n = Al.n;
        std::vector<double> v(n), w(n);
        for (int64_t i = 0; i < n; ++i) v[i] = (double(rng.next()) / 2147483647.0) + 1;
        double s = 1. / norm2(n, v.data());
        for (auto &e : v) e = s * e;
        int64_t it = 0;
        double lambda = 0, lambda_old = 0;
        bool conv = false;
        while (!conv) {
            spmv(Al, v.data(), w.data());
            lambda = norm2(n, w.data());
            double inv = 1. / lambda;
            for (int64_t i = 0; i < n; ++i) v[i] = inv * w[i];
            it++;
            conv = (std::fabs(lambda_old - lambda) < opt.pm_tol) || it > opt.pm_max_it;
            lambda_old = lambda;
        }
        eig_max[l] = opt.scale_max_eig * lambda;
        eig_min[l] = opt.scale_min_eig * eig_max[l];
    }

    // Jacobi::sweep (utopia_Jacobi.hpp:131-141) with optional relaxation folded into d_inv
    void jacobi(int l, const T *rhs, T *x, int nu) {
        const auto &Al = A[l];
        int64_t n = Al.n;
        T *rr = rc[l].data();
        for (int s = 0; s < nu; ++s) {
            residual(Al, rhs, x, rr);
            spmv_count++;
            for (int64_t i = 0; i < n; ++i) x[i] += dinv[l][i] * rr[i];
        }
    }

    // PointJacobi::sweep, utopia_PointJacobi.hpp:133-144
    void point_jacobi(int l, const T *rhs, T *x, int nu) {
        int64_t n = A[l].n;
        T *rr = rc[l].data();
        for (int s = 0; s < nu; ++s) {
            residual(LU[l], rhs, x, rr);
            spmv_count++;
            for (int64_t i = 0; i < n; ++i) x[i] = dinv[l][i] * rr[i];
        }
    }

    // Chebyshev3level::solve with max_it = sweeps and norm_frequency 0,
    // utopia/solvers/smoothers/utopia_Chebyshev3level.hpp:109-178
    void chebyshev(int l, const T *b, T *x, int nu) {
        const auto &Al = A[l];
        int64_t n = Al.n;
        T *h = help[l].data(), *rr = rc[l].data(), *p = pp[l].data();
        double avg = (eig_max[l] + eig_min[l]) / 2.0;
        double dif = (eig_max[l] - eig_min[l]) / 2.0;
        spmv(Al, x, h);
        spmv_count++;
        for (int64_t i = 0; i < n; ++i) rr[i] = h[i] - b[i];
        double alpha = 0, beta = 0;
        int64_t it = 0;
        while (true) {
            if (it == 0) {
                for (int64_t i = 0; i < n; ++i) p[i] = -1.0 * rr[i];
                alpha = 1.0 / avg;
            } else {
                double da = dif * alpha;
                beta = (it == 1 ? 0.5 : 0.25) * da * da;
                alpha = 1.0 / (avg - (beta / alpha));
                T tb = T(beta);
                for (int64_t i = 0; i < n; ++i) p[i] = -1.0 * rr[i] + tb * p[i];
            }
            T ta = T(alpha);
            for (int64_t i = 0; i < n; ++i) x[i] = x[i] + ta * p[i];
            it++;
            if (it >= nu) return;
            spmv(Al, p, h);
            spmv_count++;
            for (int64_t i = 0; i < n; ++i) rr[i] = rr[i] + ta * h[i];
        }
    }

    void smooth(int l, const T *rhs, T *x, int nu) {
        if (nu <= 0) return;
        if (opt.smoother == SM_JACOBI) jacobi(l, rhs, x, nu);
        else if (opt.smoother == SM_POINT_JACOBI) point_jacobi(l, rhs, x, nu);
        else chebyshev(l, rhs, x, nu);
    }

    void coarse_solve(const T *rhs, T *x) {
        int64_t n = coarse.n;
        std::vector<double> bd(n), xd(n);
        for (int64_t i = 0; i < n; ++i) bd[i] = double(rhs[i]);
        coarse.solve(bd.data(), xd.data());
        for (int64_t i = 0; i < n; ++i) x[i] = T(xd[i]);
    }

    // Multigrid::standard_cycle, utopia_Multigrid.hpp:252-367 (V-cycle, no line search)
    void cycle(int l) {
        auto &rl = r[l];
        auto &cl = c[l];
        std::fill(cl.begin(), cl.end(), T(0));
        if (l == 0) {
            coarse_solve(rl.data(), cl.data());
            return;
        }
        int64_t n = A[l].n;
        smooth(l, rl.data(), cl.data(), opt.pre);
        residual(A[l], rl.data(), cl.data(), rR[l].data());
        spmv_count++;
        spmv(R[l - 1], rR[l].data(), r[l - 1].data());
        if (opt.masks) {
            auto &m = mask[l - 1];
            for (size_t i = 0; i < m.size(); ++i) r[l - 1][i] = m[i] * r[l - 1][i];
        }
        cycle(l - 1);
        spmv(P[l - 1], c[l - 1].data(), cI[l].data());
        for (int64_t i = 0; i < n; ++i) cl[i] += cI[l][i];
        smooth(l, rl.data(), cl.data(), opt.post);
    }

    // one V-cycle from zero initial guess: z = c (Multigrid::apply with max_it 1, x = 0;
    // the extra residual evaluations of utopia_Multigrid.hpp:177,221 do not change z)
    void vcycle(const T *rhs, T *z) {
        auto &rf = r[L - 1];
        std::copy(rhs, rhs + rf.size(), rf.begin());
        cycle(L - 1);
        std::copy(c[L - 1].begin(), c[L - 1].end(), z);
    }

    void apply(const double *rhs, double *z) override {
        int64_t n = A64[L - 1].n;
        if constexpr (std::is_same<T, double>::value) {
            vcycle(rhs, z);
        } else {
            std::vector<T> rt(n), zt(n);
            for (int64_t i = 0; i < n; ++i) rt[i] = T(rhs[i]);
            vcycle(rt.data(), zt.data());
            for (int64_t i = 0; i < n; ++i) z[i] = double(zt[i]);
        }
    }

    // Multigrid::apply as a stand-alone solver, utopia_Multigrid.hpp:162-238
    bool solve(const double *rhs, double *x, const Params &prm, or_status &st) {
        st = or_status{};
        const Csr &Af = A64[L - 1];
        int64_t n = Af.n;
        std::vector<double> res(n), z(n);
        residual(Af, rhs, x, res.data());
        double r_norm = norm2(n, res.data()), r0 = r_norm, rel;
        int64_t it = 1;
        bool conv = false;
        while (!conv) {
            apply(res.data(), z.data());
            for (int64_t i = 0; i < n; ++i) x[i] += z[i];
            residual(Af, rhs, x, res.data());
            r_norm = norm2(n, res.data());
            rel = r_norm / r0;
            conv = check_convergence(prm, st, it, r_norm, rel, 1);
            it++;
        }
        st.converged = st.reason > 0;
        return true;
    }
};

// Flexible CG (Notay's FCG(1)): the outer iteration of the mixed-precision form.
// FP64 residual, dots and scalars; the preconditioner may run in lower precision.
// Build extension: no reference counterpart.  Same stopping rule as
// ConjugateGradient::preconditioned_solve (absolute ||r|| <= atol, or max_it).
bool fcg(const Csr &A, const double *b, double *x, Precond &M, const Params &prm, or_status &st) {
    const int64_t n = A.n;
    std::vector<double> r(n), z(n, 0.0), p(n), q(n);
    st = or_status{};
    residual(A, b, x, r.data());
    st.spmv_count++;
    M.apply(r.data(), z.data());
    p = z;
    // (p, r) by the recurrence (p', r') = (z, r') + beta ((p, r) - alpha (p, q)) (r' = r - alpha q)
    double pr = dot(n, z.data(), r.data());
    int64_t it = 0;
    double r_norm = 9e9;
    bool stop = false;
    while (!stop) {
        spmv(A, p.data(), q.data());
        st.spmv_count++;
        double pq = dot(n, p.data(), q.data());
        double alpha = pr / pq;
        if (std::isinf(alpha) || std::isnan(alpha)) {
            stop = check_convergence(prm, st, it, r_norm, 1, 1);
            if (!stop) st.reason = DIVERGED_NAN;
            break;
        }
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        r_norm = norm2(n, r.data());
        if (r_norm <= prm.atol) {
            stop = check_convergence(prm, st, it, r_norm, 1, 1);
            break;
        }
        std::fill(z.begin(), z.end(), 0.0);
        M.apply(r.data(), z.data());
        double beta = -dot(n, z.data(), q.data()) / pq;
        pr = dot(n, z.data(), r.data()) + beta * (pr - alpha * pq);
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        stop = check_convergence(prm, st, it, r_norm, 1, 1);
        it++;
    }
    st.converged = r_norm <= prm.atol;
    st.gradient_norm = r_norm;
    return st.converged;
}

// BiCGStab, utopia/solvers/smoothers/utopia_BiCGStab_impl.hpp:44-250 (preconditioned :44-155 when M is given,
// unpreconditioned :157-250 otherwise).  Preconditioner applications start from zero.  When the preconditioned
// form stops on ||s|| it returns h = x + alpha y (the reference leaves x one half-step behind there).
bool bicgstab(const Csr &A, const double *b, double *x, Precond *M, const Params &prm, or_status &st) {
    const int64_t n = A.n;
    std::vector<double> r(n), r0(n), p(n, 0.0), v(n, 0.0), h(n), y(n), s(n, 0.0), t(n), z(n), kt(n);
    st = or_status{};
    double rho = 1, rho_old = 1, alpha = 1, omega = 1, beta = 1;
    residual(A, b, x, r.data());
    st.spmv_count++;
    r0 = r;
    int64_t it = 0;
    bool converged = false;
    double r_norm = 1e10;
    auto pc = [&](const std::vector<double> &in, std::vector<double> &out) {
        std::fill(out.begin(), out.end(), 0.0);
        M->apply(in.data(), out.data());
    };
    while (!converged) {
        rho = dot(n, r0.data(), r.data());
        if (!M && rho == 0.) {
            converged = true;
            break;
        }
        beta = (rho / rho_old) * (alpha / omega);
        for (int64_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        const std::vector<double> *q = &p;
        if (M) {
            pc(p, y);
            q = &y;
        }
        spmv(A, q->data(), v.data());
        st.spmv_count++;
        const double r0v = dot(n, r0.data(), v.data());
        if (M && r0v == 0.0) {
            residual(A, b, x, r.data());
            st.spmv_count++;
            r_norm = norm2(n, s.data());
            converged = check_convergence(prm, st, it, r_norm, 1, 1);
            break;
        }
        alpha = rho / r0v;
        for (int64_t i = 0; i < n; ++i) {
            h[i] = x[i] + alpha * (*q)[i];
            s[i] = r[i] - alpha * v[i];
        }
        if (M) {
            r_norm = norm2(n, s.data());
            converged = check_convergence(prm, st, it, r_norm, 1, 1);
            if (converged) {
                std::copy(h.begin(), h.end(), x);
                break;
            }
        }
        const std::vector<double> *zz = &s;
        if (M) {
            pc(s, z);
            zz = &z;
        }
        spmv(A, zz->data(), t.data());
        st.spmv_count++;
        double num, den;
        if (M) {
            pc(t, kt);
            num = dot(n, z.data(), kt.data());
            den = dot(n, kt.data(), kt.data());
        } else {
            num = dot(n, t.data(), s.data());
            den = dot(n, t.data(), t.data());
        }
        omega = num / den;
        if (std::isnan(omega) || (!M && std::isinf(omega))) {
            if (!M) {
                r_norm = norm2(n, s.data());
                converged = check_convergence(prm, st, it, r_norm, 1, 1);
            }
            break;
        }
        for (int64_t i = 0; i < n; ++i) {
            x[i] = h[i] + omega * (*zz)[i];
            r[i] = s[i] - omega * t[i];
        }
        rho_old = rho;
        r_norm = norm2(n, r.data());
        converged = check_convergence(prm, st, it, r_norm, 1, 1);
        it++;
    }
    if (st.reason == 0) {
        st.iterates = it;
        st.gradient_norm = r_norm;
        if (converged) st.reason = CONVERGED_FNORM_ABS;
        else if (std::isnan(omega)) st.reason = DIVERGED_NAN;
    }
    st.converged = st.reason > 0;
    return st.converged;
}

// ------------------------------------------------------------------------------------
// Box-constrained QP
// ------------------------------------------------------------------------------------
// VariableBoundSolverInterface::project, utopia/solvers/nonlinear/constrained/utopia_VariableBoundSolverInterface.hpp:107-155
inline double proj(double l, double u, double x) { return (l >= x) ? l : ((u <= x) ? u : x); }

// MPRGP::get_fi, utopia_MPRGP.hpp:266-287
void get_fi(int64_t n, const double *x, const double *g, const double *lb, const double *ub, double *fi) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) fi[i] = (lb[i] < x[i] && x[i] < ub[i]) ? g[i] : 0.0;
}
// MPRGP::get_beta, utopia_MPRGP.hpp:324-348
void get_beta(int64_t n, const double *x, const double *g, const double *lb, const double *ub, double *be) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double li = lb[i], ui = ub[i], xi = x[i], gi = g[i];
        be[i] = (std::fabs(li - xi) < 1e-14) ? std::min(0.0, gi)
                                             : ((std::fabs(ui - xi) < 1e-14) ? std::max(0.0, gi) : 0.0);
    }
}
// MPRGP::get_alpha_f, utopia_MPRGP.hpp:289-322 (multi_min over the two helper vectors)
double get_alpha_f(int64_t n, const double *x, const double *p, const double *lb, const double *ub) {
    double m = std::numeric_limits<double>::max();
#pragma omp parallel for reduction(min : m) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double h1 = (p[i] > 0) ? ((x[i] - lb[i]) / p[i]) : 1e15;
        double h2 = (p[i] < 0) ? ((x[i] - ub[i]) / p[i]) : 1e15;
        m = std::min(m, std::min(h1, h2));
    }
    return m;
}

// MPRGP::solve (non-Hardik variant, no preconditioner), utopia_MPRGP.hpp:57-262;
// power_method utopia_MPRGP.hpp:351-387
bool mprgp(const Csr &A, const double *rhs, const double *lb, const double *ub, double *x, const Params &prm,
           double eps_eig, int64_t pm_max_it, or_status &st, double *lambda_out) {
    const int64_t n = A.n;
    st = or_status{};
    std::vector<double> fi(n), be(n), gp(n), p(n), y(n), Ap(n), Abeta(n), Ax(n), g(n), h1(n), h2(n);
    // power method
    std::fill(h2.begin(), h2.end(), 1.0);
    double lambda = 0, lambda_old;
    {
        int64_t it = 0;
        bool conv = false;
        while (!conv) {
            h1 = h2;
            spmv(A, h1.data(), h2.data());
            double s = 1.0 / norm2(n, h2.data());
            for (auto &v : h2) v = s * v;
            lambda_old = lambda;
            spmv(A, h2.data(), h1.data());
            lambda = dot(n, h2.data(), h1.data());
            for (int64_t i = 0; i < n; ++i) fi[i] = h2[i] - h1[i];
            double gn = norm2(n, fi.data());
            conv = (gn < eps_eig) || (std::fabs(lambda_old - lambda) < eps_eig) || it > pm_max_it;
            it++;
        }
    }
    if (lambda_out) *lambda_out = lambda;
    const double gamma = 1.0;
    const double alpha_bar = 1.95 / lambda;
    for (int64_t i = 0; i < n; ++i) x[i] = proj(lb[i], ub[i], x[i]);
    spmv(A, x, Ax.data());
    st.spmv_count++;
    for (int64_t i = 0; i < n; ++i) g[i] = Ax[i] - rhs[i];
    get_fi(n, x, g.data(), lb, ub, fi.data());
    get_beta(n, x, g.data(), lb, ub, be.data());
    for (int64_t i = 0; i < n; ++i) { gp[i] = fi[i] + be[i]; p[i] = fi[i]; }
    double beta_beta = dot(n, be.data(), be.data());
    double fi_fi = dot(n, fi.data(), fi.data());
    int64_t it = 0;
    bool converged = false;
    double gnorm = -1, gnorm0 = -1;
    while (!converged) {
        if (beta_beta <= gamma * gamma * fi_fi) {
            spmv(A, p.data(), Ap.data());
            st.spmv_count++;
            double pAp = dot(n, p.data(), Ap.data());
            double gp_dot = dot(n, g.data(), p.data());
            if (pAp <= 0.0) { st.reason = DIVERGED_INDEFINITE; st.iterates = it; return true; }
            double alpha_cg = gp_dot / pAp;
            double alpha_f = get_alpha_f(n, x, p.data(), lb, ub);
            for (int64_t i = 0; i < n; ++i) y[i] = x[i] - alpha_cg * p[i];
            if (alpha_cg <= alpha_f) {
                std::copy(y.begin(), y.end(), x);
                for (int64_t i = 0; i < n; ++i) g[i] = g[i] - alpha_cg * Ap[i];
                get_fi(n, x, g.data(), lb, ub, fi.data());
                double beta_sc = dot(n, fi.data(), Ap.data()) / pAp;
                for (int64_t i = 0; i < n; ++i) p[i] = fi[i] - beta_sc * p[i];
            } else {
                for (int64_t i = 0; i < n; ++i) x[i] = x[i] - alpha_f * p[i];
                for (int64_t i = 0; i < n; ++i) g[i] = g[i] - alpha_f * Ap[i];
                get_fi(n, x, g.data(), lb, ub, fi.data());
                for (int64_t i = 0; i < n; ++i) h1[i] = x[i] - alpha_bar * fi[i];
                for (int64_t i = 0; i < n; ++i) x[i] = proj(lb[i], ub[i], h1[i]);
                spmv(A, x, Ax.data());
                st.spmv_count++;
                for (int64_t i = 0; i < n; ++i) g[i] = Ax[i] - rhs[i];
                get_fi(n, x, g.data(), lb, ub, p.data());
            }
        } else {
            spmv(A, be.data(), Abeta.data());
            st.spmv_count++;
            double g_betta = dot(n, g.data(), be.data());
            double beta_Abeta = dot(n, be.data(), Abeta.data());
            if (beta_Abeta <= 0.0) { st.reason = DIVERGED_INDEFINITE; st.iterates = it; return true; }
            double alpha_cg = g_betta / beta_Abeta;
            for (int64_t i = 0; i < n; ++i) x[i] = x[i] - alpha_cg * be[i];
            for (int64_t i = 0; i < n; ++i) g[i] = g[i] - alpha_cg * Abeta[i];
            get_fi(n, x, g.data(), lb, ub, p.data());
        }
        get_fi(n, x, g.data(), lb, ub, fi.data());
        get_beta(n, x, g.data(), lb, ub, be.data());
        for (int64_t i = 0; i < n; ++i) gp[i] = fi[i] + be[i];
        beta_beta = dot(n, be.data(), be.data());
        fi_fi = dot(n, fi.data(), fi.data());
        gnorm = std::sqrt(dot(n, gp.data(), gp.data()));
        if (it == 0) gnorm0 = gnorm;
        it++;
        converged = check_convergence(prm, st, it, gnorm, gnorm / gnorm0, 1);
    }
    st.converged = st.reason > 0;
    st.gradient_norm = gnorm;
    return converged;
}

// ProjectedGaussSeidel::step, utopia_ProjectedGaussSeidel.hpp:197-318 (no line search).
// colour == nullptr: the reference's lexicographic symmetric sweep.  Otherwise a
// multicolour sweep (build extension): colours 0..nc-1 in turn, then (symmetric) in
// reverse order; within one colour every row reads the correction of the previous
// colour phase, so rows of one colour are independent.
void pgs_step(const Csr &A, const double *b, const double *lb, const double *ub, double *x, const double *dinv,
              int nsweeps, bool symmetric, const int32_t *colour, int ncolours, std::vector<double> &r,
              std::vector<double> &c, std::vector<double> &ubl, std::vector<double> &lbl) {
    const int64_t n = A.n;
    residual(A, b, x, r.data());
    for (int64_t i = 0; i < n; ++i) { ubl[i] = ub[i] - x[i]; lbl[i] = lb[i] - x[i]; }
    std::fill(c.begin(), c.end(), 0.0);
    auto relax = [&](int64_t i) {
        double s = r[i];
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            int32_t j = A.ci[k];
            if (j != i) s -= A.v[k] * c[j];
        }
        c[i] = std::max(std::min(dinv[i] * s, ubl[i]), lbl[i]);
    };
    for (int il = 0; il < nsweeps; ++il) {
        if (!colour) {
            for (int64_t i = 0; i < n; ++i) relax(i);
            if (symmetric)
                for (int64_t i = n - 1; i >= 0; --i) relax(i);
        } else {
            for (int col = 0; col < ncolours; ++col)
                for (int64_t i = 0; i < n; ++i)
                    if (colour[i] == col) relax(i);
            if (symmetric)
                for (int col = ncolours - 1; col >= 0; --col)
                    for (int64_t i = 0; i < n; ++i)
                        if (colour[i] == col) relax(i);
        }
    }
    for (int64_t i = 0; i < n; ++i) x[i] += c[i];
}

// ProjectedGaussSeidel::apply, utopia_ProjectedGaussSeidel.hpp:71-112 (stop on ||x - x_old|| <= stol)
bool pgs(const Csr &A, const double *b, const double *lb, const double *ub, double *x, const Params &prm, int nsweeps,
         bool symmetric, const int32_t *colour, int ncolours, or_status &st) {
    const int64_t n = A.n;
    st = or_status{};
    std::vector<double> d = diag(A), r(n), c(n), ubl(n), lbl(n), xold(x, x + n), dx(n);
    for (auto &v : d) v = 1. / v;
    int64_t iteration = 0;
    bool converged = false;
    while (!converged) {
        pgs_step(A, b, lb, ub, x, d.data(), nsweeps, symmetric, colour, ncolours, r, c, ubl, lbl);
        for (int64_t i = 0; i < n; ++i) dx[i] = x[i] - xold[i];
        double diff = norm2(n, dx.data());
        converged = check_convergence(prm, st, iteration, 1, 1, diff);
        ++iteration;
        if (converged) break;
        std::copy(x, x + n, xold.begin());
    }
    st.converged = st.reason > 0;
    return converged;
}

// Greedy first-fit colouring in index order (build extension; for the 5-point grid
// in lexicographic order it is the red-black colouring (x + y) mod 2).
int greedy_colouring(const Csr &A, int32_t *colour) {
    const int64_t n = A.n;
    int nc = 0;
    std::vector<int64_t> used(64, -1);
    for (int64_t i = 0; i < n; ++i) {
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            int32_t j = A.ci[k];
            if (j < i && colour[j] < 64) used[colour[j]] = i;
        }
        int cc = 0;
        while (cc < 64 && used[cc] == i) ++cc;
        colour[i] = cc;
        nc = std::max(nc, cc + 1);
    }
    return nc;
}

Csr make_csr(int64_t n, int64_t m, const int32_t *rp, const int32_t *ci, const double *v) {
    Csr A;
    A.n = n;
    A.m = m;
    A.rp.assign(rp, rp + n + 1);
    int64_t nnz = rp[n];
    A.ci.assign(ci, ci + nnz);
    A.v.assign(v, v + nnz);
    return A;
}

struct MgHandle {
    int precision = 0;  // 0 fp64, 1 fp32 values+vectors, 2 bf16 values + fp32 vectors
    std::unique_ptr<Mg<double, double>> m64;
    std::unique_ptr<Mg<float, float>> m32;
    std::unique_ptr<Mg<float, bf16>> m16;
    Precond *pc() {
        if (m64) return m64.get();
        if (m32) return m32.get();
        return m16.get();
    }
};

}  // namespace

// ======================================================================================
// C interface (ctypes)
// ======================================================================================
extern "C" {

void or_set_threads(int t) {
#ifdef _OPENMP
    omp_set_num_threads(t > 0 ? t : 1);
#else
    (void)t;
#endif
}
int or_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// glibc-compatible rand() stream (seed 1) for tests of the PowerMethod initial vector
void or_glibc_rand(uint32_t seed, int64_t count, int32_t *out) {
    GlibcRand g(seed);
    for (int64_t i = 0; i < count; ++i) out[i] = g.next();
}

void *or_csr_create(int64_t n, int64_t m, const int32_t *rp, const int32_t *ci, const double *v) {
    return new Csr(make_csr(n, m, rp, ci, v));
}
void or_csr_free(void *h) { delete static_cast<Csr *>(h); }
void or_csr_info(const void *h, int64_t *n, int64_t *m, int64_t *nnz) {
    auto A = static_cast<const Csr *>(h);
    *n = A->n;
    *m = A->m;
    *nnz = A->nnz();
}
void or_csr_get(const void *h, int32_t *rp, int32_t *ci, double *v) {
    auto A = static_cast<const Csr *>(h);
    std::copy(A->rp.begin(), A->rp.end(), rp);
    std::copy(A->ci.begin(), A->ci.end(), ci);
    std::copy(A->v.begin(), A->v.end(), v);
}
void or_spmv(const void *h, const double *x, double *y) { spmv(*static_cast<const Csr *>(h), x, y); }
void or_residual(const void *h, const double *b, const double *x, double *r) {
    residual(*static_cast<const Csr *>(h), b, x, r);
}
double or_dot(int64_t n, const double *a, const double *b) { return dot(n, a, b); }
void *or_transpose(const void *h) { return new Csr(transpose(*static_cast<const Csr *>(h))); }
void *or_spgemm(const void *a, const void *b) {
    return new Csr(spgemm(*static_cast<const Csr *>(a), *static_cast<const Csr *>(b)));
}
void *or_ptap(const void *a, const void *p) {
    return new Csr(ptap(*static_cast<const Csr *>(a), *static_cast<const Csr *>(p)));
}

// precond: 0 none (unpreconditioned_solve), 1 InvDiag, 2 multigrid handle (mg)
int or_cg_solve(const void *hA, const double *b, double *x, int precond, void *mg, double atol, double rtol,
                double stol, int64_t max_it, int flexible, or_status *st) {
    const Csr &A = *static_cast<const Csr *>(hA);
    Params p;
    p.atol = atol;
    p.rtol = rtol;
    p.stol = stol;
    p.max_it = max_it;
    if (precond == 0) return cg_plain(A, b, x, p, *st);
    if (precond == 1) {
        InvDiag M(A);
        return flexible ? fcg(A, b, x, M, p, *st) : pcg(A, b, x, M, p, *st);
    }
    auto *h = static_cast<MgHandle *>(mg);
    return flexible ? fcg(A, b, x, *h->pc(), p, *st) : pcg(A, b, x, *h->pc(), p, *st);
}

// SemismoothNewton, utopia/solvers/nonlinear/constrained/quadratic_programming/utopia_SemismoothNewton_impl.hpp:74-207.
// Inner solves: BiCGStab + InvDiag of the active-row-replaced matrix to linear_rtol * ||residual||.
int or_ssn_solve(const void *hA, const double *b, const double *lb_in, const double *ub_in, double *x, double stol,
                 int64_t max_it, double linear_rtol, or_status *st) {
    const Csr &A = *static_cast<const Csr *>(hA);
    const int64_t n = A.n;
    std::vector<double> lb(n), ub(n), res(n), lam(n, 0.0), active(n, 0.0), c(n);
    for (int64_t i = 0; i < n; ++i) {
        lb[i] = lb_in ? lb_in[i] : -std::numeric_limits<double>::max();
        ub[i] = ub_in ? ub_in[i] : std::numeric_limits<double>::max();
    }
    Params p;
    p.stol = stol;
    p.max_it = max_it;
    *st = or_status{};
    residual(A, b, x, res.data());
    Csr mat = A;
    int64_t it = 0, lin_its = 0;
    bool converged = false;
    while (!converged) {
        int64_t changed = 0;
        for (int64_t i = 0; i < n; ++i) {
            const bool prev = active[i] != 0.0;
            const double d_lb = x[i] + lam[i] - lb[i];
            const double d_ub = x[i] + lam[i] - ub[i];
            const bool alb = d_lb <= 0.0, aub = d_ub >= 0.0;
            const bool act = alb || aub;
            res[i] = alb ? (lb[i] - x[i]) : (aub ? (ub[i] - x[i]) : res[i]);
            active[i] = act ? 1.0 : 0.0;
            changed += (prev != act);
        }
        for (int64_t i = 0; i < n; ++i)
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
                mat.v[k] = active[i] != 0.0 ? (A.ci[k] == i ? 1.0 : 0.0) : A.v[k];
        std::fill(c.begin(), c.end(), 0.0);
        Params lp;
        lp.atol = linear_rtol * norm2(n, res.data());
        lp.max_it = 10000;
        InvDiag M(mat);
        or_status lst{};
        if (!bicgstab(mat, res.data(), c.data(), &M, lp, lst)) return 0;
        lin_its += lst.iterates;
        for (int64_t i = 0; i < n; ++i) x[i] += c[i];
        const double norm_c = norm2(n, c.data());
        ++it;
        if (it > 1 && !changed) {
            converged = true;
            st->iterates = it;
            st->step_norm = norm_c;
            st->reason = CONVERGED_SNORM_RELATIVE;
        } else {
            converged = check_convergence(p, *st, it, 1, 1, norm_c);
        }
        residual(A, b, x, res.data());
        for (int64_t i = 0; i < n; ++i) lam[i] = active[i] * res[i];
    }
    st->converged = st->reason > 0;
    st->spmv_count = lin_its;
    return st->converged;
}

// ShiftedPenaltyQPSolver::apply (utopia/solvers/nonlinear/constrained/penalty/
// utopia_ShiftedPenaltyQPSolver_impl.hpp:87-156) with the ShiftedPenalty term
// (utopia/solvers/nonlinear/constrained/penalty/utopia_ShiftedPenalty.hpp): per iteration
//   g = A x - b; ShiftedPenalty::update (update_shift_aux, :348-463, then
//   p = min(p_max, factor p)); c = gradient (penalty_gradient -p dps, :32-50); H_pen = hessian
//   (active p on the diagonal, :52-75, :181-237); g = -(g + c); H = A + H_pen; c = 0;
//   solve H c = g; x += c; stop on check_convergence(it, 1, 1, ||c||).
// The constraint is the upper bound: update() fills a missing one with the largest double
// (VariableBoundSolverInterface::init_memory, BoxConstraints::fill_empty_bounds), so the
// upper-bound branch of update_shift_aux (:357-409) always runs and a lower bound is inert.
// Selection (Penalty::apply_selection, utopia_Penalty.hpp:51-55) multiplies the constraint-space
// terms; a scaling matrix S maps them (S v); a transformation (T, O) works in the constraint
// space w = O^T (T x), maps directions back by T^T (O v) and the penalty Hessian by
// T^T (O^T D O) T (qp_solve app, utopia/apps/qp_solve/utopia_qp_solve.cpp:68-88).
// T and O are square (n x n).  Inner solves: CG + InvDiag (H is symmetric positive definite) to
// linear_rtol * ||g||.
// shift_io: the shift in constraint space, read (unless zero_shift) and written back.
Csr mat_add(const Csr &A, const Csr &B) {  // MatAXPY(A, 1, B, DIFFERENT_NONZERO_PATTERN)
    Csr C;
    C.n = A.n;
    C.m = A.m;
    C.rp.assign(A.n + 1, 0);
    for (int64_t i = 0; i < A.n; ++i) {
        int32_t a = A.rp[i], b = B.rp[i];
        while (a < A.rp[i + 1] || b < B.rp[i + 1]) {
            const int32_t ca = a < A.rp[i + 1] ? A.ci[a] : INT32_MAX;
            const int32_t cb = b < B.rp[i + 1] ? B.ci[b] : INT32_MAX;
            if (ca == cb) {
                C.ci.push_back(ca);
                C.v.push_back(A.v[a++] + B.v[b++]);
            } else if (ca < cb) {
                C.ci.push_back(ca);
                C.v.push_back(A.v[a++]);
            } else {
                C.ci.push_back(cb);
                C.v.push_back(B.v[b++]);
            }
        }
        C.rp[i + 1] = int32_t(C.ci.size());
    }
    return C;
}

Csr diag_csr(const std::vector<double> &h) {
    Csr D;
    D.n = D.m = int64_t(h.size());
    D.rp.resize(h.size() + 1);
    D.ci.resize(h.size());
    for (size_t i = 0; i < h.size(); ++i) {
        D.rp[i] = int32_t(i);
        D.ci[i] = int32_t(i);
    }
    D.rp[h.size()] = int32_t(h.size());
    D.v = h;
    return D;
}

int or_penalty_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x,
                     const double *selection, const void *hT, const void *hO, const void *hS, double penalty,
                     double penalty_max, double factor, double *shift_io, int zero_shift, double stol,
                     int64_t max_it, double linear_rtol, int64_t linear_max_it, or_status *st) {
    const Csr &A = *static_cast<const Csr *>(hA);
    const int64_t n = A.n;
    const bool trafo = hT && hO;
    const Csr *T = trafo ? static_cast<const Csr *>(hT) : nullptr;
    const Csr *O = trafo ? static_cast<const Csr *>(hO) : nullptr;
    const Csr *S = static_cast<const Csr *>(hS);
    const int64_t m = n;  // T and O are square: the constraint space has the problem's size
    (void)lb;
    std::vector<double> ubfill;
    if (!ub) {
        ubfill.assign(n, std::numeric_limits<double>::max());
        ub = ubfill.data();
    }
    Csr Ot, Tt;
    if (trafo) {
        Ot = transpose(*O);
        Tt = transpose(*T);
    }
    Params p;
    p.stol = stol;
    p.max_it = max_it;
    *st = or_status{};
    double pcur = penalty;  // ShiftedPenalty::reset
    std::vector<double> shift(m, 0.0), active(m), dps(m), w(m), gc(m), h(m), tmp(std::max(n, m)), g(n), c(n);
    if (!zero_shift) std::copy(shift_io, shift_io + m, shift.begin());
    int64_t lin_its = 0;
    bool converged = false;
    for (int64_t it = 1; it <= max_it; ++it) {
        residual(A, b, x, g.data());
        for (int64_t i = 0; i < n; ++i) g[i] = -g[i];  // A x - b
        // constraint-space position
        if (trafo) {
            spmv(*T, x, tmp.data());
            spmv(Ot, tmp.data(), w.data());
        } else {
            std::copy(x, x + n, w.begin());
        }
        for (int64_t i = 0; i < m; ++i) {  // update_shift_aux
            const double di = ub[i] - w[i];
            double si = shift[i];
            double d = di + si;
            const bool a = d <= 0;
            si = double(a) * d;
            d = double(a) * (di + si);
            active[i] = a;
            shift[i] = si;
            dps[i] = d;
        }
        pcur = std::min(penalty_max, factor * pcur);
        for (int64_t i = 0; i < m; ++i) {
            gc[i] = 0.0 - pcur * dps[i];
            h[i] = active[i] * pcur;
            if (selection) {
                gc[i] = selection[i] * gc[i];
                h[i] = selection[i] * h[i];
            }
        }
        if (S) {
            spmv(*S, gc.data(), tmp.data());
            std::copy(tmp.begin(), tmp.begin() + m, gc.begin());
            spmv(*S, h.data(), tmp.data());
            std::copy(tmp.begin(), tmp.begin() + m, h.begin());
        }
        Csr Hpen;
        if (trafo) {
            spmv(*O, gc.data(), tmp.data());
            spmv(Tt, tmp.data(), c.data());
            Hpen = ptap(ptap(diag_csr(h), *O), *T);
        } else {
            std::copy(gc.begin(), gc.end(), c.begin());
            Hpen = diag_csr(h);
        }
        for (int64_t i = 0; i < n; ++i) g[i] = -(g[i] + c[i]);
        const Csr H = mat_add(A, Hpen);
        std::fill(c.begin(), c.end(), 0.0);
        Params lp;
        lp.atol = linear_rtol * norm2(n, g.data());
        lp.max_it = linear_max_it;
        InvDiag M(H);
        or_status lst{};
        pcg(H, g.data(), c.data(), M, lp, lst);
        lin_its += lst.iterates;
        for (int64_t i = 0; i < n; ++i) x[i] += c[i];
        const double norm_c = norm2(n, c.data());
        converged = check_convergence(p, *st, it, 1, 1, norm_c);
        if (converged) break;
    }
    if (shift_io) std::copy(shift.begin(), shift.end(), shift_io);
    st->converged = st->reason > 0;
    st->spmv_count = lin_its;
    return st->converged;
}

// MonotoneMultigrid::update/apply/step (utopia/solvers/multilevel/utopia_MonotoneMultigrid.hpp:135-319):
// pre_smoothing_steps projected Gauss-Seidel steps on the fine level, the active set of
// ActiveSet::determine (utopia/solvers/nonlinear/constrained/utopia_ActiveSet.hpp:47-84:
// x_i <= lb_i + tol or x_i >= ub_i - tol), on a change IPTruncatedTransfer::truncate_interpolation
// (utopia/solvers/multilevel/transfer/utopia_IPTruncatedTransfer.hpp:203-223: the fine transfer
// with the active rows zeroed, structure kept) and galerkin_assembly (:212-227: P_t^T A P_t,
// fix_semidefinite_operator, the linear multigrid rebuilt below it), the coarse correction
// x += P_t MG(P_t^T (b - A x)) with coarse_space_it cycles of the linear multigrid (or the
// direct solve when there is only the fine transfer), then post_smoothing_steps PGS steps.
// Stop test check_convergence(it, ||P(x - g) - x||, 1, ||x - x_old||) for it = 1 .. max_it-1
// (criticality_measure_inf, :348-364; ||g|| when a bound is missing).
// P: interpolations coarse -> fine, the last one the fine-level (truncated) transfer.
// colour/ncolours: the PGS sweep order (nullptr = lexicographic).  active_out: the final
// active set; coarse_out (optional): a copy of the last truncated coarse operator.
int or_mmg_solve(const void *hA, const double *b, const double *lb_in, const double *ub_in, double *x, int nP,
                 const void *const *hP, const int32_t *colour, int ncolours, int pre, int post, int n_local_sweeps,
                 int symmetric, int smoother, double omega, double active_tol, int coarse_space_it, double atol,
                 double rtol, double stol, int64_t max_it, or_status *st, int32_t *active_out, void **coarse_out) {
    const Csr &A = *static_cast<const Csr *>(hA);
    const int64_t n = A.n;
    if (nP < 1) return -1;
    const Csr &I = *static_cast<const Csr *>(hP[nP - 1]);
    std::vector<Csr> rest;
    for (int i = 0; i + 1 < nP; ++i) rest.push_back(*static_cast<const Csr *>(hP[i]));
    const bool both = lb_in && ub_in;
    std::vector<double> lb(n), ub(n);
    for (int64_t i = 0; i < n; ++i) {
        lb[i] = lb_in ? lb_in[i] : -std::numeric_limits<double>::max();
        ub[i] = ub_in ? ub_in[i] : std::numeric_limits<double>::max();
    }
    std::vector<double> dinv = diag(A), r(n), c(n), ubl(n), lbl(n), xold(x, x + n), help(n);
    for (auto &v : dinv) v = 1. / v;
    std::vector<int32_t> active(n, 0);
    Csr It = I;  // truncated transfer (I itself until the first change of the active set)
    Csr AH;
    Cholesky chol;
    std::unique_ptr<Mg<double, double>> mg;
    MgOptions mo;
    mo.smoother = smoother;
    mo.pre = pre;
    mo.post = post;
    mo.omega = omega;
    mo.fix_semidefinite = 1;  // MonotoneMultigrid(): algo_.fix_semidefinite_operators(true)
    mo.masks = 0;             // algo_.must_generate_masks(false)
    auto galerkin = [&]() -> bool {
        AH = ptap(A, It);
        Mg<double, double>::fix_semidefinite(AH);
        if (rest.empty()) return chol.factor(AH);
        mg.reset(new Mg<double, double>);
        return mg->build(AH, rest, mo);
    };
    if (!galerkin()) return -2;
    const int64_t nc = I.m;
    std::vector<double> rc(nc), cc(nc);
    Params p;
    p.atol = atol;
    p.rtol = rtol;
    p.stol = stol;
    p.max_it = max_it;
    *st = or_status{};
    auto smooth = [&](int sweeps) {
        for (int s = 0; s < sweeps; ++s)
            pgs_step(A, b, lb.data(), ub.data(), x, dinv.data(), n_local_sweeps, symmetric != 0, colour, ncolours, r,
                     c, ubl, lbl);
    };
    auto measure = [&]() {  // r = b - A x = -g; ||P(x - g) - x|| or ||g||
        residual(A, b, x, r.data());
        if (!both) return norm2(n, r.data());
        for (int64_t i = 0; i < n; ++i) help[i] = proj(lb[i], ub[i], x[i] + r[i]) - x[i];
        return norm2(n, help.data());
    };
    double g_norm = measure();
    bool converged = false;
    int64_t it = 1;
    for (; it < max_it && !converged; ++it) {
        smooth(pre);
        int64_t changed = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int a = (x[i] <= lb[i] + active_tol || x[i] >= ub[i] - active_tol) ? 1 : 0;
            changed += (a != active[i]);
            active[i] = a;
        }
        if (changed) {
            for (int64_t i = 0; i < n; ++i)
                for (int32_t k = I.rp[i]; k < I.rp[i + 1]; ++k) It.v[k] = active[i] ? 0.0 : I.v[k];
            if (!galerkin()) return -2;
        }
        residual(A, b, x, r.data());
        Csr Rt = transpose(It);
        spmv(Rt, r.data(), rc.data());
        std::fill(cc.begin(), cc.end(), 0.0);
        if (rest.empty()) {
            chol.solve(rc.data(), cc.data());
        } else {
            Params cp;  // algo_.max_it(coarse_space_it); algo_.apply(r_coarse, c_coarse)
            cp.max_it = coarse_space_it;
            or_status cst{};
            mg->solve(rc.data(), cc.data(), cp, cst);
        }
        std::vector<double> corr(n);
        spmv(It, cc.data(), corr.data());
        for (int64_t i = 0; i < n; ++i) x[i] += corr[i];
        smooth(post);
        for (int64_t i = 0; i < n; ++i) help[i] = x[i] - xold[i];
        const double x_diff = norm2(n, help.data());
        g_norm = measure();
        converged = check_convergence(p, *st, it, g_norm, 1, x_diff);
        if (!converged) std::copy(x, x + n, xold.begin());
    }
    if (!converged) {  // the loop ran out at it == max_it without a test that says so
        st->iterates = max_it - 1;
        st->gradient_norm = g_norm;
        st->reason = DIVERGED_MAX_IT;
    }
    st->converged = st->reason > 0;
    if (active_out) std::copy(active.begin(), active.end(), active_out);
    if (coarse_out) *coarse_out = new Csr(AH);
    return st->converged;
}

int or_bicgstab_solve(const void *hA, const double *b, double *x, int precond, void *mg, double atol, int64_t max_it,
                      or_status *st) {
    const Csr &A = *static_cast<const Csr *>(hA);
    Params p;
    p.atol = atol;
    p.max_it = max_it;
    if (precond == 0) return bicgstab(A, b, x, nullptr, p, *st);
    if (precond == 1) {
        InvDiag M(A);
        return bicgstab(A, b, x, &M, p, *st);
    }
    return bicgstab(A, b, x, static_cast<MgHandle *>(mg)->pc(), p, *st);
}

// Multigrid hierarchy: P[] ordered coarse -> fine.  precision: 0 fp64, 1 fp32, 2 bf16 storage.
void *or_mg_create(const void *hA, int nP, const void *const *hP, int precision, int smoother, int pre, int post,
                   double omega, int fix_semidefinite, int masks) {
    const Csr &A = *static_cast<const Csr *>(hA);
    std::vector<Csr> P;
    for (int i = 0; i < nP; ++i) P.push_back(*static_cast<const Csr *>(hP[i]));
    MgOptions o;
    o.smoother = smoother;
    o.pre = pre;
    o.post = post;
    o.omega = omega;
    o.fix_semidefinite = fix_semidefinite;
    o.masks = masks;
    auto h = new MgHandle;
    h->precision = precision;
    bool ok;
    if (precision == 0) { h->m64.reset(new Mg<double, double>); ok = h->m64->build(A, P, o); }
    else if (precision == 1) { h->m32.reset(new Mg<float, float>); ok = h->m32->build(A, P, o); }
    else { h->m16.reset(new Mg<float, bf16>); ok = h->m16->build(A, P, o); }
    if (!ok) { delete h; return nullptr; }
    return h;
}
void or_mg_free(void *h) { delete static_cast<MgHandle *>(h); }
int or_mg_levels(const void *h) {
    auto m = static_cast<const MgHandle *>(h);
    return m->m64 ? m->m64->L : (m->m32 ? m->m32->L : m->m16->L);
}
// FP64 Galerkin operator of level l (0 = coarsest); caller frees
void *or_mg_level_matrix(const void *h, int l) {
    auto m = static_cast<const MgHandle *>(h);
    const auto &v = m->m64 ? m->m64->A64 : (m->m32 ? m->m32->A64 : m->m16->A64);
    return new Csr(v[l]);
}
void or_mg_eigs(const void *h, int l, double *emax, double *emin) {
    auto m = static_cast<const MgHandle *>(h);
    const auto &a = m->m64 ? m->m64->eig_max : (m->m32 ? m->m32->eig_max : m->m16->eig_max);
    const auto &b = m->m64 ? m->m64->eig_min : (m->m32 ? m->m32->eig_min : m->m16->eig_min);
    *emax = a[l];
    *emin = b[l];
}
void or_mg_mask(const void *h, int l, double *out) {
    auto m = static_cast<const MgHandle *>(h);
    if (m->m64) { for (size_t i = 0; i < m->m64->mask[l].size(); ++i) out[i] = m->m64->mask[l][i]; }
    else if (m->m32) { for (size_t i = 0; i < m->m32->mask[l].size(); ++i) out[i] = m->m32->mask[l][i]; }
    else { for (size_t i = 0; i < m->m16->mask[l].size(); ++i) out[i] = m->m16->mask[l][i]; }
}
// z = one V-cycle applied to r (zero initial guess)
void or_mg_vcycle(void *h, const double *r, double *z) { static_cast<MgHandle *>(h)->pc()->apply(r, z); }
int or_mg_solve(void *h, const double *rhs, double *x, double atol, double rtol, int64_t max_it, or_status *st) {
    auto m = static_cast<MgHandle *>(h);
    Params p;
    p.atol = atol;
    p.rtol = rtol;
    p.max_it = max_it;
    if (m->m64) return m->m64->solve(rhs, x, p, *st);
    if (m->m32) return m->m32->solve(rhs, x, p, *st);
    return m->m16->solve(rhs, x, p, *st);
}

int or_mprgp_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x, double atol,
                   double rtol, int64_t max_it, double eps_eig, int64_t pm_max_it, or_status *st, double *lambda) {
    Params p;
    p.atol = atol;
    p.rtol = rtol;
    p.max_it = max_it;
    return mprgp(*static_cast<const Csr *>(hA), b, lb, ub, x, p, eps_eig, pm_max_it, *st, lambda);
}

int or_pgs_solve(const void *hA, const double *b, const double *lb, const double *ub, double *x, double stol,
                 int64_t max_it, int nsweeps, int symmetric, const int32_t *colour, int ncolours, or_status *st) {
    Params p;
    p.stol = stol;
    p.max_it = max_it;
    return pgs(*static_cast<const Csr *>(hA), b, lb, ub, x, p, nsweeps, symmetric != 0, colour, ncolours, *st);
}

int or_colouring(const void *hA, int32_t *colour) { return greedy_colouring(*static_cast<const Csr *>(hA), colour); }

// Agglomerate::create_transfer_matrix (utopia/solvers/multilevel/agglomerate/utopia_Agglomerate.hpp:51-186),
// one process.  Restated from the reference: Dirichlet rows (one stored value) excluded (parent -2) unless
// use_additive_correction (:70-77); a_max_i = max_{j != i} |a_ij| (:88-92); greedy aggregation in row order
// with at most bmax neighbours j, |a_ij| > weight a_max_i, parent_j == -1 (:95-141); leftovers become
// singletons (:143-147); prolongator P(i, parent_i) = (a_max_i != 0) (:162-176).  Returns P and fills parent.
void *or_agglomerate(const void *hA, int64_t bmax, double weight, int use_additive_correction, int32_t *parent_out) {
    const Csr &A = *static_cast<const Csr *>(hA);
    const int64_t n = A.n;
    std::vector<int32_t> parent(n, -1);
    std::vector<double> a_max(n, 0.0);
    int64_t nc = 0;
    if (!use_additive_correction)
        for (int64_t i = 0; i < n; ++i)
            if (A.rp[i + 1] - A.rp[i] == 1) parent[i] = -2;
    for (int64_t i = 0; i < n; ++i)
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.ci[k] != i) a_max[i] = std::max(a_max[i], std::abs(A.v[k]));
    for (int64_t i = 0; i < n; ++i) {
        if (parent[i] != -1) continue;
        parent[i] = int32_t(nc);
        int64_t count = 0;
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            if (weight * a_max[i] < std::abs(A.v[k]) && parent[j] == -1) {
                parent[j] = int32_t(nc);
                ++count;
            }
            if (count >= bmax) break;
        }
        if (count == 0) {
            parent[i] = -1;
            double best = 0;
            int64_t arg = -1;
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
                if (std::abs(A.v[k]) > best) {
                    best = std::abs(A.v[k]);
                    arg = A.ci[k];
                }
            if (arg != -1) parent[i] = parent[arg];
        } else {
            ++nc;
        }
    }
    for (int64_t i = 0; i < n; ++i)
        if (parent[i] == -1) parent[i] = int32_t(nc++);
    auto *P = new Csr();
    P->n = n;
    P->m = nc;
    P->rp.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (parent[i] >= 0) {
            P->ci.push_back(parent[i]);
            P->v.push_back(a_max[i] != 0 ? 1.0 : 0.0);
        }
        P->rp[i + 1] = int32_t(P->ci.size());
    }
    std::copy(parent.begin(), parent.end(), parent_out);
    return P;
}

// Projected-gradient norm || P(x - g) - x ||, g = A x - b (reported for the QP runs)
double or_projected_gradient_norm(const void *hA, const double *b, const double *lb, const double *ub,
                                  const double *x) {
    const Csr &A = *static_cast<const Csr *>(hA);
    std::vector<double> g(A.n), d(A.n);
    spmv(A, x, g.data());
    for (int64_t i = 0; i < A.n; ++i) {
        g[i] -= b[i];
        d[i] = proj(lb[i], ub[i], x[i] - g[i]) - x[i];
    }
    return norm2(A.n, d.data());
}

// Adjoint edge gradient: dL/dtheta_e = -k_e (lam_i - lam_j)(x_i - x_j), k_e = exp(theta_e)
void or_edge_grad(int64_t E, const int32_t *src, const int32_t *dst, const float *theta, const double *lam,
                  const double *x, double *grad) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e) {
        int32_t i = src[e], j = dst[e];
        grad[e] = -std::exp(double(theta[e])) * (lam[i] - lam[j]) * (x[i] - x[j]);
    }
}
// dL/dA_ij = -lam_i x_j on the sparsity pattern
void or_pattern_grad(const void *hA, const double *lam, const double *x, double *gvals) {
    const Csr &A = *static_cast<const Csr *>(hA);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i)
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) gvals[k] = -lam[i] * x[A.ci[k]];
}

}  // extern "C"
