// Dense FP64 coarse-level direct solver.
//
// Reference: the coarse solver of utopia::Multigrid (Multigrid::coarse_solve,
// utopia/solvers/multilevel/utopia_Multigrid.hpp:440-444), a PETSc Factorization
// (utopia/backend/petsc/solvers/linear/utopia_petsc_Factorization.hpp).
//
// Set-up: the Galerkin operator of the coarsest level is densified, factored by a
// blocked right-looking Cholesky (A = L L^T), L is inverted blockwise (Y = L^-1) and
// the explicit inverse A^-1 = Y^T Y is formed.  Every coarse solve is then one
// FP64 GEMV with A^-1, an L2-resident matrix for the coarse sizes of the hot path
// (1728^2 and 4096^2 doubles), instead of two latency-bound triangular sweeps.
// GB300's FP64 tensor rate is no higher than its FP64 FMA rate, so the set-up uses
// FP64 FMA tiles.
#include <functional>
#include <cmath>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace ugpu {

namespace {

constexpr int NB = 64;  // Cholesky / inversion block size

template <class V>
__global__ void k_densify(const int32_t *rp, const int32_t *ci, const V *cv, int64_t n, double *D) {
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        for (int64_t c = threadIdx.x; c < n; c += blockDim.x) D[i * n + c] = 0.0;
        __syncthreads();
        for (int32_t k = rp[i] + threadIdx.x; k < rp[i + 1]; k += blockDim.x) D[i * n + ci[k]] = cvt<double>(cv[k]);
        __syncthreads();
    }
}

// unblocked Cholesky of the kb x kb diagonal block at (k0, k0) in shared memory
__global__ void __launch_bounds__(256) k_potrf_diag(double *A, int64_t n, int64_t k0, int kb, int *bad) {
    __shared__ double a[NB][NB + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        int i = e / kb, j = e % kb;
        a[i][j] = A[(k0 + i) * n + k0 + j];
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        __shared__ double d;
        if (threadIdx.x == 0) {
            double v = a[j][j];
            if (!(v > 0.0)) {
                atomicOr(bad, 1);
                v = 1.0;
            }
            d = sqrt(v);
            a[j][j] = d;
        }
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) a[i][j] /= d;
        __syncthreads();
        // trailing update of the lower triangle: a[i][c] -= a[i][j] * a[c][j], j < c <= i
        // (16 x 16 threads over rows and columns)
        const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
        for (int i = j + 1 + ty; i < kb; i += 16) {
            const double aij = a[i][j];
            for (int c = j + 1 + tx; c <= i; c += 16) a[i][c] -= aij * a[c][j];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        int i = e / kb, j = e % kb;
        A[(k0 + i) * n + k0 + j] = (j <= i) ? a[i][j] : 0.0;
    }
}

// inverse of the lower-triangular kb x kb diagonal block of L at (k0, k0), into Li (row-major,
// leading dimension NB): one thread per column solves L_bb x = e_c by forward substitution
__global__ void __launch_bounds__(NB) k_trinv_diag(const double *L, int64_t n, int64_t k0, int kb, double *Li) {
    __shared__ double l[NB][NB + 1];  // the block of L, staged once (coalesced rows)
    const int c = threadIdx.x;
    const double *Lb = L + k0 * n + k0;
    for (int i = 0; i < kb; ++i)
        if (c < kb) l[i][c] = Lb[int64_t(i) * n + c];
    __syncthreads();
    // column c of the inverse, written straight to Li and read back by the same thread
    double *xc = Li + c;
    for (int i = 0; i < NB; ++i) {
        double v = 0.0;
        if (c < kb && i >= c && i < kb) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int q = c; q < i; ++q) s -= l[i][q] * xc[q * NB];
            v = s / l[i][i];
        }
        xc[i * NB] = v;
    }
}

// dst (rows x cols, leading dimension ldd) = src (leading dimension lds)
__global__ void k_copy_block(const double *src, int64_t lds, double *dst, int64_t ldd, int rows, int cols) {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < int64_t(rows) * cols;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = e / cols, j = e % cols;
        dst[i * ldd + j] = src[i * lds + j];
    }
}

// C[M x N] (ldc) += alpha * op(A) op(B); TA/TB: operand stored transposed.
// lower_only: skip tiles strictly above the diagonal (SYRK-style update).
// T x T tiles (64 or 32), 256 threads as 16 x 16, each thread T/16 x T/16 outputs.
template <bool TA, bool TB, int T>
__global__ void __launch_bounds__(256) k_dgemm_t(int M, int N, int K, double alpha, const double *A, int64_t lda,
                                                 const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                                                 bool lower_only) {
    constexpr int TM = T, TN = T, TK = 16, PT = T / 16;
    __shared__ double As[TK][TM + 1];
    __shared__ double Bs[TK][TN + 1];
    const int bm = blockIdx.y * TM, bn = blockIdx.x * TN;
    if (lower_only && bn > bm + TM - 1) return;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[PT][PT] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = threadIdx.x; e < TM * TK; e += 256) {
            int mm = e / TK, kk = e % TK;
            int gm = bm + mm, gk = k0 + kk;
            double v = 0.0;
            if (gm < M && gk < K) v = TA ? A[int64_t(gk) * lda + gm] : A[int64_t(gm) * lda + gk];
            As[kk][mm] = v;
        }
        for (int e = threadIdx.x; e < TN * TK; e += 256) {
            int nn = e / TK, kk = e % TK;
            int gn = bn + nn, gk = k0 + kk;
            double v = 0.0;
            if (gn < N && gk < K) v = TB ? B[int64_t(gn) * ldb + gk] : B[int64_t(gk) * ldb + gn];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            double a[PT], b[PT];
#pragma unroll
            for (int q = 0; q < PT; ++q) {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < PT; ++p)
#pragma unroll
                for (int q = 0; q < PT; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < PT; ++p)
#pragma unroll
        for (int q = 0; q < PT; ++q) {
            int gm = bm + ty + 16 * p, gn = bn + tx + 16 * q;
            if (gm < M && gn < N) {
                double *c = C + int64_t(gm) * ldc + gn;
                *c = (beta == 0.0 ? 0.0 : beta * *c) + alpha * acc[p][q];
            }
        }
}

// the GEMM with the tile that keeps the grid at least two CTAs per SM: 64 x 64 tiles where
// there are that many, else 32 x 32 (a few hundred 64-tiles on 152 SMs leave SMs with one CTA
// beside SMs with two, each pacing its FP64 pipe)
template <bool TA, bool TB>
void dgemm(Context &c, int M, int N, int K, double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
           double beta, double *C, int64_t ldc, bool lower_only) {
    const int64_t tiles64 = int64_t((M + 63) / 64) * ((N + 63) / 64);
    if (tiles64 >= 2 * int64_t(c.sms)) {
        dim3 grid(unsigned((N + 63) / 64), unsigned((M + 63) / 64));
        k_dgemm_t<TA, TB, 64><<<grid, 256, 0, c.stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower_only);
    } else {
        dim3 grid(unsigned((N + 31) / 32), unsigned((M + 31) / 32));
        k_dgemm_t<TA, TB, 32><<<grid, 256, 0, c.stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower_only);
    }
    c.launches++;
}

// A[i][j] = A[j][i] for j > i (the strictly upper triangle from the lower one)
__global__ void k_mirror_lower(double *A, int64_t n) {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n * n; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = e / n, j = e % n;
        if (j > i) A[e] = A[j * n + i];
    }
}

__global__ void k_zero(double *p, int64_t m) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x)
        p[i] = 0.0;
}

// x = Ainv * r, one CTA per row (the coarse matrix has only a few thousand rows, so a warp
// per row would leave each warp a long chain of dependent load rounds); the matrix and the
// vectors share the type T (the FP64 inverse for FP64 vectors, its FP32 copy for FP32).
// Rows are read as 16-byte vectors when n and the pointers allow it.
constexpr int kGemvThreads = 256;
template <class T>
__global__ void __launch_bounds__(kGemvThreads) k_gemv(const T *M, int64_t n, const T *r, T *x, const int *done,
                                                       int vec) {
    if (done && *done) return;
    constexpr int V = 16 / sizeof(T);  // elements per 16-byte vector
    using Vec = typename std::conditional<sizeof(T) == 8, double2, float4>::type;
    __shared__ T part[kGemvThreads / 32];
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const T *row = M + i * n;
        T s = T(0);
        if (vec) {
            const Vec *rv = reinterpret_cast<const Vec *>(row);
            const Vec *xv = reinterpret_cast<const Vec *>(r);
            for (int64_t c = threadIdx.x; c < n / V; c += kGemvThreads) {
                const Vec a = __ldg(rv + c), b = __ldg(xv + c);
                const T *pa = reinterpret_cast<const T *>(&a);
                const T *pb = reinterpret_cast<const T *>(&b);
#pragma unroll
                for (int q = 0; q < V; ++q) s = fma(pa[q], pb[q], s);
            }
        } else {
            for (int64_t c = threadIdx.x; c < n; c += kGemvThreads) s = fma(__ldg(row + c), __ldg(r + c), s);
        }
        s = warp_sum(s);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            T t = threadIdx.x < kGemvThreads / 32 ? part[threadIdx.x] : T(0);
            t = warp_sum(t);
            if (threadIdx.x == 0) x[i] = t;
        }
        __syncthreads();
    }
}

}  // namespace

void DenseCholesky::make_fp32_inverse() {
    UGPU_CHECK(!tri, UGPU_ERR_UNSUPPORTED, "coarse solver: no FP32 inverse above the factored-inverse size");
    Ainv32.alloc(sizeof(float) * std::max<int64_t>(n * n, 1));
    if (n) launch_convert(*ctx, Ainv.ptr, UGPU_F64, Ainv32.ptr, UGPU_F32, n * n);
}

bool DenseCholesky::factor(const Mat &A) {
    UGPU_CHECK(A.nrows == A.ncols, UGPU_ERR_ARG, "coarse solver: square matrix required");
    Context &c = *A.ctx;
    ctx = &c;
    n = A.nrows;
    UGPU_CHECK(n <= 16384, UGPU_ERR_UNSUPPORTED, "coarse solver: dense size limited to 16384");
    L.alloc(sizeof(double) * std::max<int64_t>(n * n, 1));
    Ainv.alloc(sizeof(double) * std::max<int64_t>(n * n, 1));
    Ainv32.release();
    if (n == 0) return true;
    double *Lp = L.as<double>();
    double *Y = Ainv.as<double>();  // holds L^-1 first
    auto dens = [&](auto tag) {
        using V = decltype(tag);
        k_densify<V><<<int(std::min<int64_t>(n, 4096)), 256, 0, c.stream>>>(A.rowptr.as<int32_t>(),
                                                                              A.colidx.as<int32_t>(), A.vals.as<V>(),
                                                                              n, Lp);
    };
    if (A.vdtype == UGPU_F64) dens(double{});
    else if (A.vdtype == UGPU_F32) dens(float{});
    else dens(__nv_bfloat16{});
    c.launches++;
    UGPU_LAUNCH_CHECK();
    Buffer bad;
    bad.alloc(sizeof(int));
    UGPU_CUDA(cudaMemsetAsync(bad.ptr, 0, sizeof(int), c.stream));
    // blocked right-looking Cholesky; the panel below each diagonal block is A21 L11^-T, one
    // GEMM with the block's explicit inverse (kept for the inversion below)
    const int64_t nblk = (n + NB - 1) / NB;
    Buffer Li, T;
    Li.alloc(sizeof(double) * size_t(nblk) * NB * NB);
    T.alloc(sizeof(double) * size_t(std::max<int64_t>(n * NB, 1)));
    double *Lip = Li.as<double>(), *Tp = T.as<double>();
    auto copy_block = [&](const double *src, int64_t lds, double *dst, int64_t ldd, int rows, int cols) {
        const int g = int(std::min<int64_t>((int64_t(rows) * cols + 255) / 256, int64_t(c.sms) * 8));
        k_copy_block<<<std::max(g, 1), 256, 0, c.stream>>>(src, lds, dst, ldd, rows, cols);
        c.launches++;
    };
    for (int64_t k0 = 0; k0 < n; k0 += NB) {
        const int kb = int(std::min<int64_t>(NB, n - k0));
        double *Lb = Lip + (k0 / NB) * NB * NB;
        k_potrf_diag<<<1, 256, 0, c.stream>>>(Lp, n, k0, kb, bad.as<int>());
        k_trinv_diag<<<1, NB, 0, c.stream>>>(Lp, n, k0, kb, Lb);
        c.launches += 2;
        const int64_t rest = n - k0 - kb;
        if (rest > 0) {
            double *A21 = Lp + (k0 + kb) * n + k0;
            copy_block(A21, n, Tp, kb, int(rest), kb);
            dgemm<false, true>(c, int(rest), kb, kb, 1.0, Tp, kb, Lb, NB, 0.0, A21, n, false);
            dgemm<false, true>(c, int(rest), int(rest), kb, -1.0, A21, n, A21, n, 1.0, Lp + (k0 + kb) * n + k0 + kb,
                               n, true);
        }
        UGPU_LAUNCH_CHECK();
    }
    int hbad = 0;
    UGPU_CUDA(cudaMemcpyAsync(&hbad, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    if (hbad) return false;
    // Y = L^-1 by recursive halving: inv([[L11, 0], [L21, L22]]) = [[Y11, 0], [-Y22 L21 Y11, Y22]], halves
    // split at multiples of NB down to the diagonal blocks, whose inverses the factorisation kept.
    // Every product is a GEMM of half the current size (the top two are n/2 x n/2 x n/2), so the
    // grid stays full where a block-row sweep (kb x r0 x r0 products) left most SMs idle.
    k_zero<<<stream_grid(c, n * n), kBlock, 0, c.stream>>>(Y, n * n);
    c.launches++;
    Buffer W;
    W.alloc(sizeof(double) * size_t(std::max<int64_t>((n / 2 + NB) * (n / 2 + NB), 1)));
    double *Wp = W.as<double>();
    std::function<void(int64_t, int64_t)> tri_inv = [&](int64_t r0, int64_t m) {
        if (m <= NB) {  // one diagonal block (r0 is a multiple of NB)
            copy_block(Lip + (r0 / NB) * NB * NB, NB, Y + r0 * n + r0, n, int(m), int(m));
            return;
        }
        const int64_t h = ((m / 2 + NB - 1) / NB) * NB;  // 0 < h < m, a multiple of NB
        tri_inv(r0, h);
        tri_inv(r0 + h, m - h);
        const int64_t m2 = m - h;
        // W = L21 Y11  (m2 x h, leading dimension h)
        dgemm<false, false>(c, int(m2), int(h), int(h), 1.0, Lp + (r0 + h) * n + r0, n, Y + r0 * n + r0, n, 0.0, Wp,
                            h, false);
        // Y21 = -Y22 W
        dgemm<false, false>(c, int(m2), int(h), int(m2), -1.0, Y + (r0 + h) * n + r0 + h, n, Wp, h, 0.0,
                            Y + (r0 + h) * n + r0, n, false);
        UGPU_LAUNCH_CHECK();
    };
    tri_inv(0, n);
    tmp_d.ensure(sizeof(double) * size_t(n));
    tri = n > kDenseTriMin;
    if (tri) {  // Y in the lower triangle, Y^T in the upper one; L keeps the factor
        k_mirror_lower<<<stream_grid(c, n * n), kBlock, 0, c.stream>>>(Y, n);
        c.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaStreamSynchronize(c.stream));
        return true;
    }
    // Ainv = Y^T Y (stored in L's buffer, then swapped): the lower triangle's tiles, then mirrored
    // (the product is symmetric bit for bit: (i, j) and (j, i) sum the same products in one order)
    {
        dgemm<true, false>(c, int(n), int(n), int(n), 1.0, Y, n, Y, n, 0.0, Lp, n, true);
        k_mirror_lower<<<stream_grid(c, n * n), kBlock, 0, c.stream>>>(Lp, n);
        c.launches++;
        UGPU_LAUNCH_CHECK();
    }
    std::swap(L, Ainv);  // Ainv now holds the inverse; L holds L^-1 (kept for diagnostics)
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    return true;
}

// x = Ainv * r with the FP64 inverse, one warp per row: the row streams through 16-byte loads
// spread over the lanes into four independent FP64 partial sums per lane, reduced by shuffles.
// r and x are FP64, or FP32 (the mixed V-cycle: r converted exactly, x rounded once).  A CTA per
// row left most of the grid waiting on its block reductions (1728 rows: 21 us for 3 M FMAs).
template <class VT>
__device__ __forceinline__ double2 gemv_r2(const VT *r, int64_t j) {
    if constexpr (sizeof(VT) == 8) {
        return __ldg(reinterpret_cast<const double2 *>(r) + j);
    } else {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(r) + j);
        return make_double2(f2d_bits(t.x), f2d_bits(t.y));
    }
}
template <class VT>
__global__ void __launch_bounds__(256) k_gemv64_warp(const double *M, int64_t n, const VT *r, VT *x,
                                                     const int *done, int vec) {
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5; i < n; i += nw) {
        const double *row = M + i * n;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        if (vec) {  // n even; row and r aligned for pair loads
            const double2 *rv = reinterpret_cast<const double2 *>(row);
            const int64_t n2 = n >> 1;
            int64_t c = lane;
            for (; c + 32 < n2; c += 64) {
                const double2 a = __ldg(rv + c), b = __ldg(rv + c + 32);
                const double2 ra = gemv_r2(r, c), rb = gemv_r2(r, c + 32);
                s0 = fma(a.x, ra.x, s0);
                s1 = fma(a.y, ra.y, s1);
                s2 = fma(b.x, rb.x, s2);
                s3 = fma(b.y, rb.y, s3);
            }
            if (c < n2) {
                const double2 a = __ldg(rv + c), ra = gemv_r2(r, c);
                s0 = fma(a.x, ra.x, s0);
                s1 = fma(a.y, ra.y, s1);
            }
        } else {
            for (int64_t c = lane; c < n; c += 32) s0 = fma(__ldg(row + c), cvt<double>(__ldg(r + c)), s0);
        }
        const double s = warp_sum((s0 + s1) + (s2 + s3));
        if (lane == 0) x[i] = cvt<VT>(s);
    }
}

// The same product for coarse levels whose right-hand side fits shared memory: r is converted to
// FP64 once per CTA into shared memory, and each row is split over two warps (four rows per CTA),
// so every lane has only a few independent 16-byte row loads and the grid keeps enough of them
// in flight to stream the inverse at HBM rate.
constexpr int kGemvSmemMax = 96 * 1024;  // bytes of r staged per CTA
template <class VT>
__global__ void __launch_bounds__(256) k_gemv64_split(const double *M, int64_t n, const VT *r, VT *x,
                                                      const int *done, int vec) {
    extern __shared__ __align__(16) double sr[];  // r in FP64
    __shared__ double part[8];
    if (done && *done) return;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) sr[j] = cvt<double>(r[j]);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rl = warp >> 1, q = warp & 1;  // row of the four, half of the row
    for (int64_t i0 = 4 * int64_t(blockIdx.x); i0 < n; i0 += 4 * int64_t(gridDim.x)) {
        const int64_t i = i0 + rl;
        double s0 = 0.0, s1 = 0.0;
        if (i < n) {
            const double *row = M + i * n;
            if (vec) {  // n even, rows 16-byte aligned: pairs [q n2 / 4, (q + 1) n2 / 4)
                const int64_t n2 = n >> 1, c0 = q * n2 / 2, c1 = (q + 1) * n2 / 2;
                const double2 *rv = reinterpret_cast<const double2 *>(row);
                const double2 *xv = reinterpret_cast<const double2 *>(sr);
#pragma unroll 4
                for (int64_t c = c0 + lane; c < c1; c += 32) {
                    const double2 a = __ldg(rv + c), b = xv[c];
                    s0 = fma(a.x, b.x, s0);
                    s1 = fma(a.y, b.y, s1);
                }
            } else {
                const int64_t c0 = q * n / 2, c1 = (q + 1) * n / 2;
                for (int64_t c = c0 + lane; c < c1; c += 32) s0 = fma(__ldg(row + c), sr[c], s0);
            }
        }
        const double s = warp_sum(s0 + s1);
        if (lane == 0) part[warp] = s;
        __syncthreads();
        if (threadIdx.x < 4 && i0 + threadIdx.x < n) {
            const double *pp = part + 2 * threadIdx.x;
            x[i0 + threadIdx.x] = cvt<VT>(pp[0] + pp[1]);
        }
        __syncthreads();
    }
}

// One triangle of the tri form: out_i = sum over j <= i (LOWER) or j >= i of M[i][j] in_j, a warp per
// row (row segments are contiguous, the lanes' loads coalesced), four partial sums per lane.
template <class VI, class VO, bool LOWER>
__global__ void __launch_bounds__(256) k_gemv64_tri(const double *M, int64_t n, const VI *in, VO *out,
                                                    const int *done) {
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5; i < n; i += nw) {
        const double *row = M + i * n;
        const int64_t lo = LOWER ? 0 : i, hi = LOWER ? i + 1 : n;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int64_t c = lo + lane;
        for (; c + 96 < hi; c += 128) {
            s0 = fma(__ldg(row + c), cvt<double>(__ldg(in + c)), s0);
            s1 = fma(__ldg(row + c + 32), cvt<double>(__ldg(in + c + 32)), s1);
            s2 = fma(__ldg(row + c + 64), cvt<double>(__ldg(in + c + 64)), s2);
            s3 = fma(__ldg(row + c + 96), cvt<double>(__ldg(in + c + 96)), s3);
        }
        for (; c < hi; c += 32) s0 = fma(__ldg(row + c), cvt<double>(__ldg(in + c)), s0);
        const double s = warp_sum((s0 + s1) + (s2 + s3));
        if (lane == 0) out[i] = cvt<VO>(s);
    }
}

void DenseCholesky::solve(const void *rhs, int rdt, void *x, int xdt, const int *done) {
    Context &c = *ctx;
    if (n == 0) return;
    if (tri) {  // x = Y^T (Y r), the intermediate in FP64
        UGPU_CHECK((rdt == UGPU_F64 || rdt == UGPU_F32) && rdt == xdt, UGPU_ERR_UNSUPPORTED,
                   "coarse solve: FP64 or FP32 vectors");
        const int gw = int(std::min<int64_t>((n + 7) / 8, int64_t(c.sms) * 8));  // a warp per row, 8 per CTA
        double *t = tmp_d.as<double>();
        if (rdt == UGPU_F64) {
            k_gemv64_tri<double, double, true><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n,
                                                                         static_cast<const double *>(rhs), t, done);
            k_gemv64_tri<double, double, false><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n, t,
                                                                          static_cast<double *>(x), done);
        } else {
            k_gemv64_tri<float, double, true><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n,
                                                                        static_cast<const float *>(rhs), t, done);
            k_gemv64_tri<double, float, false><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n, t,
                                                                         static_cast<float *>(x), done);
        }
        c.launches += 2;
        UGPU_LAUNCH_CHECK();
        return;
    }
    int g = int(std::min<int64_t>((n * 32 + 255) / 256, int64_t(c.sms) * 8));
    g = int(std::min<int64_t>(std::max<int64_t>(n, 1), int64_t(c.sms) * 8));
    auto al = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    const int gw = int(std::min<int64_t>((n + 7) / 8, int64_t(c.sms) * 8));  // a warp per row, 8 per CTA
    const bool split = (rdt == xdt) && (rdt == UGPU_F64 || (rdt == UGPU_F32 && !Ainv32.ptr)) &&
                       size_t(n) * sizeof(double) <= size_t(kGemvSmemMax);
    if (split) {
        const int gs = int(std::min<int64_t>((n + 3) / 4, int64_t(c.sms) * 8));  // four rows per CTA
        const size_t smem = size_t(n) * sizeof(double);
        const int vec = (n % 2 == 0) && al(Ainv.ptr);
        if (rdt == UGPU_F64) {
            static bool attr = false;
            if (!attr) {
                UGPU_CUDA(cudaFuncSetAttribute(k_gemv64_split<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kGemvSmemMax));
                attr = true;
            }
            k_gemv64_split<double><<<gs, 256, smem, c.stream>>>(Ainv.as<double>(), n,
                                                                static_cast<const double *>(rhs),
                                                                static_cast<double *>(x), done, vec);
        } else {
            static bool attr = false;
            if (!attr) {
                UGPU_CUDA(cudaFuncSetAttribute(k_gemv64_split<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kGemvSmemMax));
                attr = true;
            }
            k_gemv64_split<float><<<gs, 256, smem, c.stream>>>(Ainv.as<double>(), n, static_cast<const float *>(rhs),
                                                               static_cast<float *>(x), done, vec);
        }
        c.launches++;
        UGPU_LAUNCH_CHECK();
        return;
    }
    if (rdt == UGPU_F64 && xdt == UGPU_F64) {
        const int vec = (n % 2 == 0) && al(Ainv.ptr) && al(rhs);
        k_gemv64_warp<double><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n, static_cast<const double *>(rhs),
                                                         static_cast<double *>(x), done, vec);
    } else if (rdt == UGPU_F32 && xdt == UGPU_F32 && Ainv32.ptr) {
        // FP32 inverse (only when make_fp32_inverse was called)
        const int vec = (n % 4 == 0) && al(Ainv32.ptr) && al(rhs);
        k_gemv<float><<<g, kGemvThreads, 0, c.stream>>>(Ainv32.as<float>(), n, static_cast<const float *>(rhs),
                                                         static_cast<float *>(x), done, vec);
    } else if (rdt == UGPU_F32 && xdt == UGPU_F32) {
        // FP64 solve for FP32 vectors
        const int vec = (n % 2 == 0) && al(Ainv.ptr) && (reinterpret_cast<uintptr_t>(rhs) & 7u) == 0;
        k_gemv64_warp<float><<<gw, 256, 0, c.stream>>>(Ainv.as<double>(), n, static_cast<const float *>(rhs),
                                                        static_cast<float *>(x), done, vec);
    } else
        throw Error(UGPU_ERR_UNSUPPORTED, "coarse solve: FP64 or FP32 vectors");
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

}  // namespace ugpu
