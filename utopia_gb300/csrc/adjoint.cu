// Differentiable solve on a graph with per-edge log-conductances (no reference counterpart).
//
//   A(theta) = sum_e exp(theta_e) (e_i - e_j)(e_i - e_j)^T + diag(boundary conductances)
//   x = A(theta)^{-1} b
//   given dL/dx:  A^T lambda = dL/dx  (A is symmetric: the forward solver and its multigrid
//                 hierarchy are reused unchanged; only x from the forward pass is kept),
//                 dL/db = lambda,
//                 dL/dtheta_e = -exp(theta_e) (lambda_i - lambda_j)(x_i - x_j),
//                 dL/dA_ij = -lambda_i x_j on the sparsity pattern.
//
// The graph keeps, per CSR entry of A, the edge it belongs to (-1 on the diagonal), so the
// assembly is a row-parallel pass with a fixed summation order (deterministic), and the
// gradients are streaming passes over edges or nonzeros (HBM-bound).
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace ugpu {

struct Graph {
    Context *ctx = nullptr;
    int64_t n = 0, E = 0, nnz = 0;
    Buffer src, dst;          // int32[E], src < dst
    Buffer edge_of_pos;       // int32[nnz]: edge of each CSR entry of A, -1 for the diagonal
    Buffer boundary;          // FP64[n]: Dirichlet boundary conductance added to the diagonal
};

namespace {

#define ADJ_LOOP(i, n) \
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

template <class TT>
__global__ void k_graph_assemble(const int32_t *rp, const int32_t *ci, const int32_t *eop, const TT *theta,
                                 const double *bnd, int64_t n, double *vals) {
    ADJ_LOOP(i, n) {
        double d = bnd[i];
        int32_t kd = -1;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int32_t e = eop[k];
            if (e >= 0) {
                const double ke = exp(double(theta[e]));
                vals[k] = -ke;
                d += ke;
            } else if (ci[k] == i) {
                kd = k;
            } else {
                vals[k] = 0.0;
            }
        }
        if (kd >= 0) vals[kd] = d;
    }
}

template <class TT>
__global__ void k_edge_grad(int64_t E, const int32_t *src, const int32_t *dst, const TT *theta, const double *lam,
                            const double *x, TT *grad) {
    ADJ_LOOP(e, E) {
        const int32_t i = src[e], j = dst[e];
        grad[e] = TT(-exp(double(theta[e])) * (lam[i] - lam[j]) * (x[i] - x[j]));
    }
}

__global__ void k_pattern_grad(const int32_t *rp, const int32_t *ci, int64_t n, const double *lam, const double *x,
                               double *g) {
    ADJ_LOOP(i, n) {
        const double li = -lam[i];
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) g[k] = li * x[ci[k]];
    }
}

__global__ void k_check_edges(int64_t E, const int32_t *src, const int32_t *dst, int64_t n, int *bad) {
    ADJ_LOOP(e, E) {
        if (src[e] < 0 || dst[e] < 0 || src[e] >= n || dst[e] >= n || src[e] >= dst[e]) atomicOr(bad, 1);
    }
}

__global__ void k_check_eop(int64_t nnz, const int32_t *eop, int64_t E, int *bad) {
    ADJ_LOOP(k, nnz) {
        if (eop[k] < -1 || eop[k] >= E) atomicOr(bad, 2);
    }
}

}  // namespace

void graph_assemble(Graph &g, const Vec &theta, Mat &A) {
    UGPU_CHECK(theta.n == g.E && (theta.dtype == UGPU_F32 || theta.dtype == UGPU_F64), UGPU_ERR_ARG,
               "graph: theta must be FP32 or FP64 of length E");
    UGPU_CHECK(A.nrows == g.n && A.ncols == g.n && A.nnz == g.nnz && A.vdtype == UGPU_F64, UGPU_ERR_ARG,
               "graph: the operator must be the FP64 n x n pattern the graph was described on");
    Context &c = *g.ctx;
    const int grid = stream_grid(c, g.n);
    if (theta.dtype == UGPU_F32)
        k_graph_assemble<float><<<grid, kBlock, 0, c.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                               g.edge_of_pos.as<int32_t>(), theta.as<float>(),
                                                               g.boundary.as<double>(), g.n, A.vals.as<double>());
    else
        k_graph_assemble<double><<<grid, kBlock, 0, c.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                                g.edge_of_pos.as<int32_t>(), theta.as<double>(),
                                                                g.boundary.as<double>(), g.n, A.vals.as<double>());
    c.launches++;
    UGPU_LAUNCH_CHECK();
    refresh_values(A);  // refresh the sliced-ELL copy of the values
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ugpu

using namespace ugpu;

struct ugpu_graph {
    Graph impl;
};

extern "C" {

int ugpu_graph_create(ugpu_ctx *ctx, int64_t n, int64_t E, const int32_t *src, const int32_t *dst, int64_t nnz,
                      const int32_t *edge_of_pos, const double *boundary, ugpu_graph **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_CHECK(n > 0 && E >= 0 && nnz >= n && nnz < (1ll << 31), UGPU_ERR_ARG, "graph: bad sizes");
    UGPU_CHECK(edge_of_pos && boundary && (E == 0 || (src && dst)), UGPU_ERR_ARG, "graph: null arrays");
    Context &c = ctx->impl;
    auto g = std::make_unique<ugpu_graph>();
    Graph &G = g->impl;
    G.ctx = &c;
    G.n = n;
    G.E = E;
    G.nnz = nnz;
    G.src.alloc(sizeof(int32_t) * std::max<int64_t>(E, 1));
    G.dst.alloc(sizeof(int32_t) * std::max<int64_t>(E, 1));
    G.edge_of_pos.alloc(sizeof(int32_t) * nnz);
    G.boundary.alloc(sizeof(double) * n);
    if (E) {
        UGPU_CUDA(cudaMemcpyAsync(G.src.ptr, src, sizeof(int32_t) * E, cudaMemcpyHostToDevice, c.stream));
        UGPU_CUDA(cudaMemcpyAsync(G.dst.ptr, dst, sizeof(int32_t) * E, cudaMemcpyHostToDevice, c.stream));
    }
    UGPU_CUDA(cudaMemcpyAsync(G.edge_of_pos.ptr, edge_of_pos, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice,
                              c.stream));
    UGPU_CUDA(cudaMemcpyAsync(G.boundary.ptr, boundary, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    Buffer bad;
    bad.alloc(sizeof(int));
    UGPU_CUDA(cudaMemsetAsync(bad.ptr, 0, sizeof(int), c.stream));
    if (E) k_check_edges<<<stream_grid(c, E), kBlock, 0, c.stream>>>(E, G.src.as<int32_t>(), G.dst.as<int32_t>(), n,
                                                                      bad.as<int>());
    k_check_eop<<<stream_grid(c, nnz), kBlock, 0, c.stream>>>(nnz, G.edge_of_pos.as<int32_t>(), E, bad.as<int>());
    c.launches += 2;
    int h = 0;
    UGPU_CUDA(cudaMemcpyAsync(&h, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    UGPU_CHECK(!(h & 1), UGPU_ERR_ARG, "graph: edges must satisfy 0 <= src < dst < n");
    UGPU_CHECK(!(h & 2), UGPU_ERR_ARG, "graph: edge_of_pos entries must lie in [-1, E)");
    *out = g.release();
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_graph_destroy(ugpu_graph *g) {
    UGPU_ABI_BEGIN
    delete g;
    UGPU_ABI_END(nullptr)
}

int ugpu_graph_assemble(ugpu_graph *g, const ugpu_vec *theta, ugpu_mat *A) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(g);
    UGPU_REQUIRE(theta);
    UGPU_REQUIRE(A);
    graph_assemble(g->impl, theta->impl, A->impl);
    UGPU_CUDA(cudaStreamSynchronize(g->impl.ctx->stream));
    UGPU_ABI_END(g ? g->impl.ctx : nullptr)
}

int ugpu_graph_edge_grad(ugpu_graph *g, const ugpu_vec *theta, const ugpu_vec *lam, const ugpu_vec *x,
                         ugpu_vec *grad) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(g);
    UGPU_REQUIRE(theta);
    UGPU_REQUIRE(lam);
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(grad);
    Graph &G = g->impl;
    UGPU_CHECK(theta->impl.n == G.E && grad->impl.n == G.E && theta->impl.dtype == grad->impl.dtype &&
                   (theta->impl.dtype == UGPU_F32 || theta->impl.dtype == UGPU_F64),
               UGPU_ERR_ARG, "edge_grad: theta and grad of length E with the same dtype (FP32 or FP64)");
    UGPU_CHECK(lam->impl.n == G.n && x->impl.n == G.n && lam->impl.dtype == UGPU_F64 && x->impl.dtype == UGPU_F64,
               UGPU_ERR_ARG, "edge_grad: lambda and x are FP64 vectors of length n");
    Context &c = *G.ctx;
    if (G.E) {
        if (theta->impl.dtype == UGPU_F32)
            k_edge_grad<float><<<stream_grid(c, G.E), kBlock, 0, c.stream>>>(
                G.E, G.src.as<int32_t>(), G.dst.as<int32_t>(), theta->impl.as<float>(), lam->impl.as<double>(),
                x->impl.as<double>(), grad->impl.as<float>());
        else
            k_edge_grad<double><<<stream_grid(c, G.E), kBlock, 0, c.stream>>>(
                G.E, G.src.as<int32_t>(), G.dst.as<int32_t>(), theta->impl.as<double>(), lam->impl.as<double>(),
                x->impl.as<double>(), grad->impl.as<double>());
        c.launches++;
        UGPU_LAUNCH_CHECK();
    }
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    UGPU_ABI_END(g ? g->impl.ctx : nullptr)
}

int ugpu_pattern_grad(const ugpu_mat *A, const ugpu_vec *lam, const ugpu_vec *x, ugpu_vec *gvals) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(lam);
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(gvals);
    const Mat &M = A->impl;
    UGPU_CHECK(lam->impl.n == M.nrows && x->impl.n == M.ncols && gvals->impl.n == M.nnz &&
                   lam->impl.dtype == UGPU_F64 && x->impl.dtype == UGPU_F64 && gvals->impl.dtype == UGPU_F64,
               UGPU_ERR_ARG, "pattern_grad: FP64 lambda (nrows), x (ncols), values (nnz)");
    Context &c = *M.ctx;
    if (M.nrows) {
        k_pattern_grad<<<stream_grid(c, M.nrows), kBlock, 0, c.stream>>>(
            M.rowptr.as<int32_t>(), M.colidx.as<int32_t>(), M.nrows, lam->impl.as<double>(), x->impl.as<double>(),
            gvals->impl.as<double>());
        c.launches++;
        UGPU_LAUNCH_CHECK();
    }
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

}  // extern "C"
