// AlgebraicMultigrid with greedy agglomeration
// (utopia/solvers/multilevel/utopia_AlgebraicMultigrid.hpp:16-177,
//  utopia/solvers/multilevel/agglomerate/utopia_Agglomerate.hpp:51-186).
//
// The reference builds n_levels - 1 piecewise-constant prolongators by aggregating the rows of
// each level's operator in index order, forms every coarser operator by the Galerkin product
// (IPRTransfer::restrict(M) = P^T M P) and runs its Multigrid on that hierarchy.  The
// aggregation is a sequential greedy pass by definition (each row's choice depends on every
// earlier row's), so it runs on the host, in C++, once per level at set-up; the Galerkin
// products, the smoothers and every cycle run on the GPU through the multigrid solver of
// mg.cu, which takes the prolongators as its transfer operators.
#include <algorithm>
#include <cmath>
#include <vector>

#include "abi_util.cuh"
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

// Agglomerate::create_transfer_matrix (utopia_Agglomerate.hpp:51-186) on one process:
//   rows with a single stored value are Dirichlet rows and stay out of every aggregate (parent
//   -2) unless use_additive_correction; a_max_i = max_{j != i} |a_ij|; rows are visited in index
//   order and an unassigned row i opens aggregate c, then takes up to bmax unassigned neighbours
//   j (in column order) with |a_ij| > weight * a_max_i; a row that takes none is undone and joins
//   the aggregate of its largest |a_ij| (diagonal included; that may leave it unassigned or
//   excluded); rows still unassigned at the end become singleton aggregates.
//   The prolongator has P(i, parent_i) = 1 (0 where a_max_i = 0) for parent_i >= 0.
void agglomerate_host(int64_t n, const int32_t *rp, const int32_t *ci, const double *v, int64_t bmax, double weight,
                      bool use_additive_correction, std::vector<int32_t> &parent, std::vector<double> &a_max,
                      int64_t &n_coarse) {
    parent.assign(size_t(n), -1);
    a_max.assign(size_t(n), 0.0);
    n_coarse = 0;
    if (!use_additive_correction) {
        for (int64_t i = 0; i < n; ++i)
            if (rp[i + 1] - rp[i] == 1) parent[size_t(i)] = -2;
    }
    for (int64_t i = 0; i < n; ++i)
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] != i) a_max[size_t(i)] = std::max(a_max[size_t(i)], std::fabs(v[k]));
    for (int64_t i = 0; i < n; ++i) {
        if (parent[size_t(i)] != -1) continue;
        parent[size_t(i)] = int32_t(n_coarse);
        const double ami = a_max[size_t(i)];
        int64_t count = 0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int32_t j = ci[k];
            if (weight * ami < std::fabs(v[k]) && parent[size_t(j)] == -1) {
                parent[size_t(j)] = int32_t(n_coarse);
                count++;
            }
            if (count >= bmax) break;
        }
        if (count == 0) {
            // not a cluster centre: join the aggregate of the strongest entry of the row
            parent[size_t(i)] = -1;
            double max_aij = 0;
            int32_t arg = -1;
            for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
                const double a = std::fabs(v[k]);
                if (a > max_aij) {
                    arg = ci[k];
                    max_aij = a;
                }
            }
            if (arg != -1) parent[size_t(i)] = parent[size_t(arg)];
        } else {
            ++n_coarse;
        }
    }
    for (int64_t i = 0; i < n; ++i)
        if (parent[size_t(i)] == -1) parent[size_t(i)] = int32_t(n_coarse++);
}

namespace {

std::unique_ptr<Mat> prolongator(Context &ctx, int64_t n, int64_t nc, const std::vector<int32_t> &parent,
                                 const std::vector<double> &a_max) {
    std::vector<int32_t> rp(size_t(n) + 1, 0), ci;
    std::vector<double> v;
    ci.reserve(size_t(n));
    v.reserve(size_t(n));
    for (int64_t i = 0; i < n; ++i) {
        if (parent[size_t(i)] >= 0) {
            ci.push_back(parent[size_t(i)]);
            v.push_back(a_max[size_t(i)] != 0 ? 1.0 : 0.0);
        }
        rp[size_t(i) + 1] = int32_t(ci.size());
    }
    auto P = make_csr_device(ctx, n, nc, int64_t(ci.size()), UGPU_F64);
    UGPU_CUDA(cudaMemcpyAsync(P->rowptr.ptr, rp.data(), sizeof(int32_t) * rp.size(), cudaMemcpyHostToDevice,
                              ctx.stream));
    if (!ci.empty()) {
        UGPU_CUDA(cudaMemcpyAsync(P->colidx.ptr, ci.data(), sizeof(int32_t) * ci.size(), cudaMemcpyHostToDevice,
                                  ctx.stream));
        UGPU_CUDA(cudaMemcpyAsync(P->vals.ptr, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice,
                                  ctx.stream));
    }
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));  // host arrays go out of scope
    finalize_matrix(*P);
    return P;
}

void download_csr(const Mat &A, std::vector<int32_t> &rp, std::vector<int32_t> &ci, std::vector<double> &v) {
    Context &c = *A.ctx;
    UGPU_CHECK(A.vdtype == UGPU_F64, UGPU_ERR_ARG, "algebraic multigrid: FP64 operator required");
    rp.resize(size_t(A.nrows) + 1);
    ci.resize(size_t(A.nnz));
    v.resize(size_t(A.nnz));
    UGPU_CUDA(cudaMemcpyAsync(rp.data(), A.rowptr.ptr, sizeof(int32_t) * rp.size(), cudaMemcpyDeviceToHost, c.stream));
    if (A.nnz) {
        UGPU_CUDA(cudaMemcpyAsync(ci.data(), A.colidx.ptr, sizeof(int32_t) * ci.size(), cudaMemcpyDeviceToHost,
                                  c.stream));
        UGPU_CUDA(cudaMemcpyAsync(v.data(), A.vals.ptr, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, c.stream));
    }
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
}

// keys of the aggregation; every other key goes to the multigrid underneath
bool amg_key(const std::string &k) {
    return k == "n_levels" || k == "bmax" || k == "weight" || k == "use_additive_correction" ||
           k == "max_coarse_rows";
}

}  // namespace

class AlgebraicMultigrid final : public Solver {
public:
    explicit AlgebraicMultigrid(Context *c) : Solver(c, UGPU_SOLVER_AMG), mg_(make_multigrid(c)) {
        prm = mg_->prm;                 // the multigrid's parameters, readable through get()
        prm["n_levels"] = 2;            // utopia_AlgebraicMultigrid.hpp:173
        prm["bmax"] = 3;                // utopia_Agglomerate.hpp:43
        prm["weight"] = 1.0 / 3;        // utopia_Agglomerate.hpp:45
        prm["use_additive_correction"] = 0;
        prm["max_coarse_rows"] = 4096;  // n_levels = 0: coarsen until at most this many rows (or a stall)
    }

    void set(const std::string &k, double v) override {
        if (amg_key(k)) {
            Solver::set(k, v);
        } else {
            mg_->set(k, v);  // validates the key
            prm[k] = v;
        }
    }

    // AlgebraicMultigridBuilder::build (utopia_AlgebraicMultigrid.hpp:22-55)
    void update(const Mat *A) override {
        UGPU_CHECK(A && A->nrows == A->ncols, UGPU_ERR_ARG, "algebraic multigrid: square operator required");
        op = A;
        const int64_t want_levels = int64_t(get("n_levels"));
        const int64_t max_coarse = int64_t(get("max_coarse_rows"));
        UGPU_CHECK(want_levels == 0 || want_levels >= 2, UGPU_ERR_ARG, "n_levels must be 0 (automatic) or >= 2");
        transfers_.clear();
        parents_.clear();
        std::unique_ptr<Mat> owned;
        const Mat *cur = A;
        std::vector<int32_t> rp, ci, parent;
        std::vector<double> v, amax;
        for (int64_t l = 0; want_levels == 0 || l < want_levels - 1; ++l) {
            if (want_levels == 0 && l > 0 && cur->nrows <= max_coarse) break;  // at least one coarse level
            download_csr(*cur, rp, ci, v);
            int64_t nc = 0;
            agglomerate_host(cur->nrows, rp.data(), ci.data(), v.data(), int64_t(get("bmax")), get("weight"),
                             get("use_additive_correction") != 0, parent, amax, nc);
            UGPU_CHECK(nc > 0, UGPU_ERR_ARG, "algebraic multigrid: empty coarse level");
            // automatic depth: stop once a level shrinks by less than 4:3 (the Galerkin operators
            // of stalled levels grow dense and would dominate the cycle)
            if (want_levels == 0 && 4 * nc > 3 * cur->nrows) break;
            auto P = prolongator(*ctx, cur->nrows, nc, parent, amax);
            parents_.push_back(parent);
            auto next = ptap(*cur, *P);  // IPRTransfer::restrict(M): P^T M P
            transfers_.push_back(std::move(P));
            owned = std::move(next);
            cur = owned.get();
        }
        UGPU_CHECK(!transfers_.empty(), UGPU_ERR_ARG, "algebraic multigrid: no coarse level");
        // Multigrid takes interpolation operators ordered coarse -> fine
        std::vector<const Mat *> P;
        for (auto it = transfers_.rbegin(); it != transfers_.rend(); ++it) P.push_back(it->get());
        mg_set_transfers(mg_.get(), P);
        mg_->update(A);
    }

    void apply(const Vec &b, Vec &x) override {
        mg_->apply(b, x);
        st = mg_->st;
    }

    int pc_dtype() const override { return mg_->pc_dtype(); }
    void pc_enqueue(const void *r, void *z, const int *done) override { mg_->pc_enqueue(r, z, done); }

    int n_transfers() const { return int(transfers_.size()); }
    int64_t coarse_rows(int l) const { return transfers_.at(size_t(l))->ncols; }
    const std::vector<int32_t> &parent(int l) const { return parents_.at(size_t(l)); }
    const Solver *multigrid() const { return mg_.get(); }

private:
    std::unique_ptr<Solver> mg_;
    std::vector<std::unique_ptr<Mat>> transfers_;  // fine -> coarse, as built
    std::vector<std::vector<int32_t>> parents_;
};

std::unique_ptr<Solver> make_amg(Context *c) { return std::make_unique<AlgebraicMultigrid>(c); }

const Solver *amg_multigrid(const Solver *s) {
    auto *a = dynamic_cast<const AlgebraicMultigrid *>(s);
    return a ? a->multigrid() : s;
}

}  // namespace ugpu

extern "C" {

int ugpu_amg_parent(const ugpu_solver *amg, int level, int32_t *parent, int64_t *n, int64_t *n_coarse) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(amg);
    auto *a = dynamic_cast<const ugpu::AlgebraicMultigrid *>(amg->impl.get());
    UGPU_CHECK(a, UGPU_ERR_ARG, "not an algebraic multigrid solver");
    UGPU_CHECK(level >= 0 && level < a->n_transfers(), UGPU_ERR_ARG, "level out of range");
    const auto &p = a->parent(level);
    if (n) *n = int64_t(p.size());
    if (n_coarse) *n_coarse = a->coarse_rows(level);
    if (parent) std::copy(p.begin(), p.end(), parent);
    UGPU_ABI_END(amg->impl->ctx)
}

}  // extern "C"
