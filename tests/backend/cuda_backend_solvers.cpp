// The reference's own solver templates instantiated over a utopia backend:
//   -DUSE_CUDA_BACKEND: include/utopia_cuda_backend.hpp (CuMatrix / CuVector over the C ABI;
//                       linked against libugpu.so, or against tests/backend/fake_ugpu.cpp)
//   otherwise:          oracle/ref/utopia_ref_backend.hpp (the oracle's CPU backend)
// Solves: ConjugateGradient + InvDiagPreconditioner; Multigrid (Chebyshev3level, Jacobi,
// PointJacobi; dense Cholesky coarse solve) as CG preconditioner and as a stand-alone solver;
// MPRGP and ProjectedGaussSeidel on an obstacle problem.  Built from the reference checkout's
// headers by tests/test_cuda_backend.py.
//
// Usage: cuda_backend_solvers [n]   (n x n 5-point Laplacian, n divisible by 8; default 32)
// Prints per solve: <name> <iterations> <reason> <||x||_2 %.17g> <sum x %.17g>.
// Exits 3 with "no device" on stderr when the CUDA backend cannot create a device context.
#ifdef USE_CUDA_BACKEND
#include "utopia_cuda_backend.hpp"
#else
#include "utopia_ref_backend.hpp"
#endif

#include "utopia_Chebyshev3level.hpp"
#include "utopia_ConjugateGradient.hpp"
#include "utopia_ConjugateGradient_impl.hpp"
#include "utopia_IPRTransfer.hpp"
#include "utopia_Jacobi.hpp"
#include "utopia_MPRGP.hpp"
#include "utopia_Multigrid.hpp"
#include "utopia_PointJacobi.hpp"
#include "utopia_ProjectedGaussSeidel.hpp"
#include "utopia_TrivialPreconditioners.hpp"

#include <cstdio>

using namespace utopia;

#ifdef USE_CUDA_BACKEND
using Mat = CuMatrix;
using Vec = CuVector;
using Coarse = CuCholesky;
static Vec make_vec(const std::vector<double> &h) {
    Vec v;
    v.upload(h);
    return v;
}
static std::vector<double> host(const Vec &v) { return v.download(); }
#else
using Mat = RefMatrix;
using Vec = RefVector;
using Coarse = RefCholesky;
static Vec make_vec(const std::vector<double> &h) {
    Vec v(RefTraits::Layout(SelfCommunicator(), SizeType(h.size()), SizeType(h.size())), 0.0);
    v.data() = h;
    return v;
}
static std::vector<double> host(const Vec &v) { return v.data(); }
#endif

namespace {

// 5-point Laplacian on an n x n interior grid (Dirichlet eliminated)
void laplacian(int n, std::vector<int> &rp, std::vector<int> &ci, std::vector<double> &v) {
    rp.assign(1, 0);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            const int r = j * n + i;
            if (j > 0) ci.push_back(r - n), v.push_back(-1);
            if (i > 0) ci.push_back(r - 1), v.push_back(-1);
            ci.push_back(r), v.push_back(4);
            if (i < n - 1) ci.push_back(r + 1), v.push_back(-1);
            if (j < n - 1) ci.push_back(r + n), v.push_back(-1);
            rp.push_back(int(ci.size()));
        }
}

// bilinear interpolation from (nf/2)^2 to nf^2 (vertex-centred: coarse i <-> fine 2i+1)
void interpolation(int nf, std::vector<int> &rp, std::vector<int> &ci, std::vector<double> &v) {
    const int nc = nf / 2;
    auto w1 = [&](int f, std::vector<std::pair<int, double>> &out) {
        out.clear();
        if (f % 2 == 1) {
            out.push_back({(f - 1) / 2, 1.0});
        } else {
            if (f / 2 - 1 >= 0) out.push_back({f / 2 - 1, 0.5});
            if (f / 2 < nc) out.push_back({f / 2, 0.5});
        }
    };
    std::vector<std::pair<int, double>> wx, wy;
    rp.assign(1, 0);
    for (int j = 0; j < nf; ++j)
        for (int i = 0; i < nf; ++i) {
            w1(i, wx);
            w1(j, wy);
            std::vector<std::pair<int, double>> row;
            for (auto &y : wy)
                for (auto &x : wx) row.push_back({y.first * nc + x.first, y.second * x.second});
            std::sort(row.begin(), row.end());
            for (auto &e : row) ci.push_back(e.first), v.push_back(e.second);
            rp.push_back(int(ci.size()));
        }
}

std::shared_ptr<Mat> make_mat(int m, int n, const std::vector<int> &rp, const std::vector<int> &ci,
                              const std::vector<double> &v) {
    auto A = std::make_shared<Mat>();
    A->from_csr(m, n, rp.data(), ci.data(), v.data());
    return A;
}

void report(const char *name, const SolutionStatus &st, const Vec &x) {
    const auto h = host(x);
    double nrm = 0, sum = 0;
    for (double e : h) nrm += e * e, sum += e;
    std::printf("%s %d %d %.17g %.17g\n", name, st.iterates, st.reason, std::sqrt(nrm), sum);
}

}  // namespace

int main(int argc, char **argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 32;
#ifdef USE_CUDA_BACKEND
    try {
        cuda::context();
    } catch (const std::exception &e) {
        std::fprintf(stderr, "no device: %s\n", e.what());
        return 3;
    }
#endif
    try {
        std::vector<int> rp, ci;
        std::vector<double> v;
        laplacian(n, rp, ci, v);
        auto A = make_mat(n * n, n * n, rp, ci, v);
        std::vector<std::shared_ptr<Mat>> Ps;  // coarse to fine
        for (int nf = n; nf >= n / 4; nf /= 2) {
            std::vector<int> prp, pci;
            std::vector<double> pv;
            interpolation(nf, prp, pci, pv);
            Ps.insert(Ps.begin(), make_mat(nf * nf, (nf / 2) * (nf / 2), prp, pci, pv));
        }
        std::vector<double> hb(size_t(n) * size_t(n));
        for (size_t i = 0; i < hb.size(); ++i) hb[i] = std::sin(0.37 * double(i)) + 0.1;
        const Vec b = make_vec(hb);
        const double atol = 1e-8 * norm2(b);

        {
            ConjugateGradient<Mat, Vec> cg;
            cg.atol(atol);
            cg.max_it(10000);
            cg.set_preconditioner(std::make_shared<InvDiagPreconditioner<Mat, Vec>>());
            Vec x = make_vec(std::vector<double>(hb.size(), 0.0));
            cg.solve(*A, b, x);
            report("cg_invdiag", cg.solution_status(), x);
        }
        for (int sm = 0; sm < 3; ++sm) {
            std::shared_ptr<IterativeSolver<Mat, Vec>> smoother;
            if (sm == 0) smoother = std::make_shared<Chebyshev3level<Mat, Vec>>();
            if (sm == 1) smoother = std::make_shared<Jacobi<Mat, Vec>>();
            if (sm == 2) smoother = std::make_shared<PointJacobi<Mat, Vec>>();
            auto mg = std::make_shared<Multigrid<Mat, Vec>>(smoother, std::make_shared<Coarse>());
            mg->set_transfer_operators(Ps);
            mg->pre_smoothing_steps(3);
            mg->post_smoothing_steps(3);
            mg->max_it(1);
            ConjugateGradient<Mat, Vec> cg;
            cg.atol(atol);
            cg.set_preconditioner(mg);
            Vec x = make_vec(std::vector<double>(hb.size(), 0.0));
            std::srand(1);
            cg.solve(*A, b, x);
            const char *name[3] = {"mg_pcg_chebyshev", "mg_pcg_jacobi", "mg_pcg_point_jacobi"};
            report(name[sm], cg.solution_status(), x);
            if (sm == 0) {  // Multigrid::apply as a stand-alone solver
                mg->max_it(20);
                mg->atol(atol);
                Vec y = make_vec(std::vector<double>(hb.size(), 0.0));
                mg->apply(b, y);
                report("mg_standalone", mg->solution_status(), y);
            }
        }
        {  // obstacle problem: x >= lb
            const double h2 = 1.0 / double((n + 1) * (n + 1));
            std::vector<double> hl(hb.size()), hf(hb.size(), -20.0 * h2);
            for (size_t i = 0; i < hl.size(); ++i) hl[i] = -0.05 + 0.02 * std::cos(0.011 * double(i));
            auto lb = std::make_shared<Vec>(make_vec(hl));
            const Vec f = make_vec(hf);
            MPRGP<Mat, Vec> qp;
            qp.atol(1e-8 * h2);
            qp.max_it(100000);
            qp.set_box_constraints(BoxConstraints<Vec>(lb, nullptr));
            Vec x = make_vec(std::vector<double>(hb.size(), 0.0));
            qp.solve(*A, f, x);
            report("mprgp", qp.solution_status(), x);
            ProjectedGaussSeidel<Mat, Vec> pgs;
            pgs.stol(1e-12);
            pgs.max_it(100000);
            pgs.set_box_constraints(BoxConstraints<Vec>(lb, nullptr));
            Vec y = make_vec(std::vector<double>(hb.size(), 0.0));
            pgs.solve(*A, f, y);
            report("projected_gauss_seidel", pgs.solution_status(), y);
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
