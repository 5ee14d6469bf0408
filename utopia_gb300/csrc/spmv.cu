// CSR matrices, the sliced-ELL layout, and the SpMV-family kernels with fused epilogues.
//
// Reference call sites replaced: PetscMatrix::multiply -> MatMult
// (utopia/backend/petsc/utopia_petsc_Matrix.cpp:1358), MatMultAdd (:1400-1404),
// Eval_Residual (utopia/utopia_core/eval/utopia_Eval_Residual.hpp:19-38), the Jacobi
// sweep (utopia/solvers/smoothers/utopia_Jacobi.hpp:131-141), MatGetDiagonal (:756).
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace ugpu {

namespace {

// ------------------------------------------------------------------------------------
// CSR validation (kernels never index outside the arrays they were given)
// ------------------------------------------------------------------------------------
__global__ void k_check_rowptr(const int32_t *rp, int64_t n, int64_t nnz, int *bad) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        int32_t a = rp[i], b = rp[i + 1];
        if (a < 0 || b < a || b > nnz) atomicOr(bad, 1);
    }
}

__global__ void k_check_cols(const int32_t *rp, const int32_t *ci, int64_t n, int64_t ncols, int *bad) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        int32_t prev = -1;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
            int32_t c = ci[k];
            if (c < 0 || c >= ncols) atomicOr(bad, 2);
            if (c <= prev) atomicOr(bad, 4);
            prev = c;
        }
    }
}

__global__ void k_row_lengths_max(const int32_t *rp, int64_t n, unsigned int *mx) {
    unsigned int m = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        m = max(m, unsigned(rp[i + 1] - rp[i]));
    atomicMax(mx, m);
}

template <class V>
__global__ void k_diag(const int32_t *rp, const int32_t *ci, const V *v, int64_t n, double *d) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double di = 0.0;
        for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i) di = cvt<double>(v[k]);
        d[i] = di;
    }
}

// ------------------------------------------------------------------------------------
// sliced-ELL construction
// ------------------------------------------------------------------------------------
constexpr int kAnalyzeThreads = 128;

// per slice: width and kind.  Diagonal slices collect the sorted distinct offsets
// (col - row) by repeated min-extraction over the slice's entries.
__global__ void __launch_bounds__(kAnalyzeThreads) k_sell_analyze(const int32_t *rp, const int32_t *ci, int64_t n,
                                                                   int S, int64_t nslices, int sval,
                                                                   int32_t *width, int32_t *offs_tmp) {
    __shared__ int s_maxrow;
    __shared__ long long s_min;
    for (int64_t s = blockIdx.x; s < nslices; s += gridDim.x) {
        int64_t r0 = s * S, r1 = min(n, r0 + S);
        if (threadIdx.x == 0) s_maxrow = 0;
        __syncthreads();
        int mr = 0;
        for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) mr = max(mr, rp[r + 1] - rp[r]);
        atomicMax(&s_maxrow, mr);
        __syncthreads();
        int maxrow = s_maxrow;
        __syncthreads();
        int nd = 0;
        bool diag_ok = maxrow <= kMaxDiagSlots;
        long long prev = LLONG_MIN;
        while (diag_ok) {
            if (threadIdx.x == 0) s_min = LLONG_MAX;
            __syncthreads();
            long long m = LLONG_MAX;
            for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
                for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
                    long long off = (long long)ci[k] - r;
                    if (off > prev && off < m) m = off;
                }
            atomicMin(&s_min, m);
            __syncthreads();
            long long mm = s_min;
            __syncthreads();
            if (mm == LLONG_MAX) break;
            if (nd >= kMaxDiagSlots || mm > INT_MAX || mm < INT_MIN) {
                diag_ok = false;
                break;
            }
            if (threadIdx.x == 0) offs_tmp[s * kMaxDiagSlots + nd] = int32_t(mm);
            nd++;
            prev = mm;
        }
        // bytes: diagonal = nd*S*sval (+4*nd), explicit = maxrow*S*(sval+4)
        if (diag_ok && (long long)nd * S * sval + 4ll * nd <= (long long)maxrow * S * (sval + 4)) {
            if (threadIdx.x == 0) width[s] = nd;
        } else {
            if (threadIdx.x == 0) width[s] = -maxrow;
        }
        __syncthreads();
    }
}

template <class V>
__global__ void __launch_bounds__(kAnalyzeThreads) k_sell_fill(const int32_t *rp, const int32_t *ci, const V *cv,
                                                                int64_t n, int64_t ncols, int S, int64_t nslices,
                                                                const int32_t *width, const int64_t *sptr,
                                                                const int64_t *aux, const int32_t *offs_tmp,
                                                                int32_t *offs, int32_t *cols, V *vals) {
    __shared__ int32_t s_off[kMaxDiagSlots];
    for (int64_t s = blockIdx.x; s < nslices; s += gridDim.x) {
        int w = width[s];
        int64_t base = sptr[s];
        int64_t r0 = s * S;
        if (w >= 0) {
            for (int k = threadIdx.x; k < w; k += blockDim.x) {
                s_off[k] = offs_tmp[s * kMaxDiagSlots + k];
                offs[aux[s] + k] = s_off[k];
            }
            __syncthreads();
            for (int64_t e = threadIdx.x; e < int64_t(w) * S; e += blockDim.x) vals[base + e] = cvt<V>(0.0);
            __syncthreads();
            for (int rl = threadIdx.x; rl < S; rl += blockDim.x) {
                int64_t r = r0 + rl;
                if (r >= n) continue;
                int slot = 0;
                for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
                    int32_t off = int32_t((long long)ci[k] - r);
                    while (slot < w && s_off[slot] < off) ++slot;
                    if (slot < w && s_off[slot] == off) vals[base + int64_t(slot) * S + rl] = cv[k];
                }
            }
            __syncthreads();
        } else {
            int wd = -w;
            int64_t cb = aux[s];
            for (int rl = threadIdx.x; rl < S; rl += blockDim.x) {
                int64_t r = r0 + rl;
                int32_t len = (r < n) ? rp[r + 1] - rp[r] : 0;
                int32_t start = (r < n) ? rp[r] : 0;
                int32_t padcol = (len > 0) ? ci[start] : 0;
                if (padcol >= ncols) padcol = 0;
                for (int k = 0; k < wd; ++k) {
                    bool real = k < len;
                    vals[base + int64_t(k) * S + rl] = real ? cv[start + k] : cvt<V>(0.0);
                    cols[cb + int64_t(k) * S + rl] = real ? ci[start + k] : padcol;
                }
            }
        }
    }
}

// ------------------------------------------------------------------------------------
// SpMV kernels
// ------------------------------------------------------------------------------------
struct SliceHdr {
    int64_t base;  // value offset of the slice (elements)
    int w;         // width; negative: explicit-column slice
    int aux;       // diagonal slices: index into offs; explicit slices: index into cols
};

struct SellView {
    const int4 *hdr;
    const int64_t *sptr;
    const int32_t *width;
    const int64_t *aux;
    const int32_t *offs;
    const int32_t *cols;
    const void *vals;
    int64_t nslices, nrows, ncols;
};

template <class V, int R>
struct VecLoad;
template <>
struct VecLoad<double, 2> {
    __device__ __forceinline__ static void load(const double *p, double (&v)[2]) {
        double2 t = __ldcs(reinterpret_cast<const double2 *>(p));
        v[0] = t.x;
        v[1] = t.y;
    }
};
template <>
struct VecLoad<float, 4> {
    __device__ __forceinline__ static void load(const float *p, float (&v)[4]) {
        float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
};
template <>
struct VecLoad<__nv_bfloat16, 4> {
    __device__ __forceinline__ static void load(const __nv_bfloat16 *p, float (&v)[4]) {
        uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162 *>(&t.x);
        __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162 *>(&t.y);
        float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        v[0] = fa.x; v[1] = fa.y; v[2] = fb.x; v[3] = fb.y;
    }
};

template <int R>
__device__ __forceinline__ void load_cols(const int32_t *p, int32_t (&c)[R]) {
    if constexpr (R == 2) {
        int2 t = __ldcs(reinterpret_cast<const int2 *>(p));
        c[0] = t.x; c[1] = t.y;
    } else {
        int4 t = __ldcs(reinterpret_cast<const int4 *>(p));
        c[0] = t.x; c[1] = t.y; c[2] = t.z; c[3] = t.w;
    }
}

template <class T>
struct EpiParams {
    const T *x;      // input vector (or the "u" of xin = u + beta*w)
    const T *wvec;   // fused direction: previous p
    T *pout;         // fused direction: new p written for own rows
    const double *beta_ptr;
    const T *v;      // epilogue vector
    const T *w;      // per-row weights (Jacobi)
    T *y;
    T *vout;         // Chebyshev residual (in/out)
    T *x2;           // Chebyshev iterate (in/out)
    T s0, s1, s2, s3;
    int x2_zero;
    const T *dv;     // second dot operand
    double *dot_partials;
    double *dot_out;
    unsigned int *dot_counter;
    const int *done;
    const int *gate;
};

// the product's input vector: x (XM 0), x + beta*p (XM 1), or w .* v formed on the fly
// (XM 2: the first Jacobi iterate from zero, x1 = w .* rhs)
template <class T, int XM>
__device__ __forceinline__ T xin_at(const EpiParams<T> &e, T beta, int64_t j) {
    if constexpr (XM == 1) {
        return __ldg(e.x + j) + beta * __ldg(e.wvec + j);
    } else if constexpr (XM == 2) {
        return __ldg(e.w + j) * __ldg(e.v + j);
    } else {
        return __ldg(e.x + j);
    }
}

// row epilogue; returns the value stored to y[row]
template <class T, int EPI>
__device__ __forceinline__ T epilogue(const EpiParams<T> &e, int64_t row, T acc, T xrow) {
    if constexpr (EPI == EPI_STORE) return acc;
    if constexpr (EPI == EPI_ADD) return acc + e.v[row];
    if constexpr (EPI == EPI_RESIDUAL) return e.v[row] - acc;
    if constexpr (EPI == EPI_SUB) return acc - e.v[row];
    if constexpr (EPI == EPI_JACOBI) return xrow + e.w[row] * (e.v[row] - acc);
    if constexpr (EPI == EPI_SCALE) return e.w[row] * acc;
    if constexpr (EPI == EPI_PJACOBI) return e.w[row] * (e.v[row] - acc);
    if constexpr (EPI == EPI_CHEB) {
        // r = r + alpha_prev * (A p); p_new = -1 * r + beta * p; x = x + alpha * p_new
        T r = e.vout[row] + e.s0 * acc;
        e.vout[row] = r;
        T pn = T(-1) * r + e.s1 * xrow;
        T xv = e.x2_zero ? T(0) : e.x2[row];
        if (e.s3 != T(0)) xv = xv + e.s3 * xrow;  // deferred x += alpha_0 p_0 of the first step
        e.x2[row] = xv + e.s2 * pn;
        return pn;
    }
    if constexpr (EPI == EPI_CHEB0) {
        // r = A x - b; p = -1 * r  (x += alpha_0 p_0 is deferred to the next step: x is
        // the gathered input of this product)
        T r = acc - e.v[row];
        e.vout[row] = r;
        T pn = T(-1) * r;
        return pn;
    }
    return acc;
}

constexpr int kSpmvWarps = 8;

// tuning knobs of the sliced-ELL kernel: slot-loop unroll depth and the minimum CTAs
// per SM promised to the register allocator (0: no promise)
#ifndef UGPU_SELL_UNROLL
#define UGPU_SELL_UNROLL 4
#endif
#ifndef UGPU_SELL_MINB
#define UGPU_SELL_MINB 4
#endif
#define UGPU_XSTR(x) UGPU_STR(x)
#define UGPU_STR(x) #x
#define UGPU_PRAGMA_UNROLL(n) _Pragma(UGPU_XSTR(unroll n))
#if UGPU_SELL_MINB > 0
#define UGPU_SELL_BOUNDS __launch_bounds__(kSpmvWarps * 32, UGPU_SELL_MINB)
#else
#define UGPU_SELL_BOUNDS __launch_bounds__(kSpmvWarps * 32)
#endif

// One warp per slice (grid-stride); R rows per lane; slot-major vector loads.
template <class V, class T, int R, int EPI, int XM, bool DOT>
__global__ void UGPU_SELL_BOUNDS k_sell_spmv(SellView m, EpiParams<T> e) {
    if ((e.done && *e.done) || (e.gate && !*e.gate)) return;
    constexpr int S = 32 * R;
    using LV = typename std::conditional<std::is_same<V, __nv_bfloat16>::value, float, V>::type;
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const V *vals = static_cast<const V *>(m.vals);
    T beta = T(0);
    if constexpr (XM == 1) beta = T(*e.beta_ptr);
    double dacc = 0.0, dacc2 = 0.0;
    // Slices are interleaved over warps (neighbouring warps stream neighbouring slices, which
    // keeps DRAM pages and the x-gathers local).  Each slice's header is one 16-byte load;
    // headers are fetched two slices ahead and diagonal offsets one slice ahead, so a slice
    // never waits on a chain of dependent loads.
    const int64_t ns = m.nslices;
    auto load_hdr = [&](int64_t s) -> SliceHdr {
        SliceHdr h{0, 0, 0};
        if (s < ns) {
            const int4 q = __ldg(reinterpret_cast<const int4 *>(m.hdr) + s);
            h.base = (int64_t(uint32_t(q.y)) << 32) | uint32_t(q.x);
            h.w = q.z;
            h.aux = q.w;
        }
        return h;
    };
    auto load_offs = [&](const SliceHdr &h, int64_t s, int32_t &lo, int32_t &hi) {
        const bool diag = s < ns && h.w >= 0;
        lo = (diag && lane < h.w) ? __ldg(m.offs + h.aux + lane) : 0;
        hi = (diag && lane + 32 < h.w) ? __ldg(m.offs + h.aux + 32 + lane) : 0;
    };
    SliceHdr h_cur = load_hdr(warp0), h_nxt = load_hdr(warp0 + nwarps);
    int32_t o_lo, o_hi;
    load_offs(h_cur, warp0, o_lo, o_hi);
    for (int64_t s = warp0; s < ns; s += nwarps) {
        int32_t n_lo, n_hi;
        load_offs(h_nxt, s + nwarps, n_lo, n_hi);
        const SliceHdr h_nn = load_hdr(s + 2 * nwarps);
        const int w = h_cur.w;
        const int64_t base = h_cur.base;
        const int64_t aux = h_cur.aux;
        const int32_t off_lo = o_lo, off_hi = o_hi;
        h_cur = h_nxt;
        h_nxt = h_nn;
        o_lo = n_lo;
        o_hi = n_hi;
        const int64_t row0 = s * S + int64_t(lane) * R;
        T acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = T(0);
        if (w >= 0) {
            // the slice's offsets were read once (coalesced) and are broadcast by shuffle, so
            // the gathers of a slot depend on no load but the value stream's
            const int r0i = int(row0);  // nrows, ncols < 2^31
            const int cmax = int(m.ncols) - 1;
            UGPU_PRAGMA_UNROLL(UGPU_SELL_UNROLL)
            for (int k = 0; k < w; ++k) {
                const int32_t off = __shfl_sync(0xffffffffu, k < 32 ? off_lo : off_hi, k & 31);
                LV v[R];
                VecLoad<V, R>::load(vals + base + int64_t(k) * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    int c = r0i + r + off;
                    c = c < 0 ? 0 : (c > cmax ? cmax : c);
                    acc[r] = fma(T(v[r]), xin_at<T, XM>(e, beta, c), acc[r]);
                }
            }
        } else {
            const int wd = -w;
            const int32_t *cols = m.cols + aux;
#pragma unroll 2
            for (int k = 0; k < wd; ++k) {
                LV v[R];
                int32_t c[R];
                VecLoad<V, R>::load(vals + base + int64_t(k) * S + lane * R, v);
                load_cols<R>(cols + int64_t(k) * S + lane * R, c);
#pragma unroll
                for (int r = 0; r < R; ++r) acc[r] = fma(T(v[r]), xin_at<T, XM>(e, beta, c[r]), acc[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int64_t row = row0 + r;
            if (row < m.nrows) {
                T xr = T(0);
                if constexpr (XM != 0 || EPI == EPI_JACOBI || EPI == EPI_CHEB || DOT) xr = xin_at<T, XM>(e, beta, row);
                if constexpr (XM == 1) e.pout[row] = xr;
                T out = epilogue<T, EPI>(e, row, acc[r], xr);
                e.y[row] = out;
                if constexpr (DOT) {
                    dacc = fma(double(xr), double(out), dacc);
                    if (e.dv) dacc2 = fma(double(xr), double(e.dv[row]), dacc2);
                }
            }
        }
    }
    if constexpr (DOT) {
        const int nd = e.dv ? 2 : 1;
        double a[2] = {dacc, dacc2};
        block_reduce_store<2>(a, nd, e.dot_partials, gridDim.x, blockIdx.x);
        finish_last_block(nd, e.dot_partials, gridDim.x, e.dot_out, e.dot_counter);
    }
}

// CSR baseline: G lanes per row, lane-strided accumulation, shuffle reduction.
// The loop is warp-uniform (each warp covers 32/G rows per step) so the shuffles
// always see the full warp.
template <class V, class T, int G, int EPI, int XM, bool DOT>
__global__ void __launch_bounds__(256) k_csr_spmv(const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                                                  const V *__restrict__ cv, int64_t nrows, EpiParams<T> e) {
    if ((e.done && *e.done) || (e.gate && !*e.gate)) return;
    constexpr int RPW = 32 / G;  // rows per warp step
    const int lane = threadIdx.x & 31;
    const int sub = lane % G;
    const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    T beta = T(0);
    if constexpr (XM == 1) beta = T(*e.beta_ptr);
    double dacc = 0.0, dacc2 = 0.0;
    for (int64_t wb = warp0 * RPW; wb < nrows; wb += nwarps * RPW) {
        const int64_t row = wb + lane / G;
        T acc = T(0);
        if (row < nrows) {
            const int32_t k1 = __ldg(rp + row + 1);
            for (int32_t k = __ldg(rp + row) + sub; k < k1; k += G)
                acc = fma(cvt<T>(__ldcs(cv + k)), xin_at<T, XM>(e, beta, __ldcs(ci + k)), acc);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (row < nrows && sub == 0) {
            T xr = T(0);
            if constexpr (XM != 0 || EPI == EPI_JACOBI || EPI == EPI_CHEB || DOT) xr = xin_at<T, XM>(e, beta, row);
            if constexpr (XM == 1) e.pout[row] = xr;
            T out = epilogue<T, EPI>(e, row, acc, xr);
            e.y[row] = out;
            if constexpr (DOT) {
                dacc = fma(double(xr), double(out), dacc);
                if (e.dv) dacc2 = fma(double(xr), double(e.dv[row]), dacc2);
            }
        }
    }
    if constexpr (DOT) {
        const int nd = e.dv ? 2 : 1;
        double a[2] = {dacc, dacc2};
        block_reduce_store<2>(a, nd, e.dot_partials, gridDim.x, blockIdx.x);
        finish_last_block(nd, e.dot_partials, gridDim.x, e.dot_out, e.dot_counter);
    }
}

template <class T>
EpiParams<T> make_epi(const SpmvArgs &a) {
    EpiParams<T> e{};
    e.x = static_cast<const T *>(a.x);
    e.wvec = static_cast<const T *>(a.p);
    e.pout = static_cast<T *>(a.pout);
    e.beta_ptr = a.beta_ptr;
    e.v = static_cast<const T *>(a.v);
    e.w = static_cast<const T *>(a.w);
    e.y = static_cast<T *>(a.y);
    e.vout = static_cast<T *>(a.vout);
    e.x2 = static_cast<T *>(a.x2);
    e.s0 = T(a.s0);
    e.s1 = T(a.s1);
    e.s2 = T(a.s2);
    e.s3 = T(a.s3);
    e.x2_zero = a.x2_zero;
    e.dv = static_cast<const T *>(a.dv);
    e.dot_partials = a.dot_partials;
    e.dot_out = a.dot_out;
    e.dot_counter = a.dot_counter;
    e.done = a.done;
    e.gate = a.gate;
    return e;
}

int spmv_grid(const Context &ctx, int64_t units_per_cta_work, int64_t total) {
    int64_t g = (total + units_per_cta_work - 1) / units_per_cta_work;
    int64_t cap = int64_t(ctx.sms) * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return int(g);
}

template <class V, class T, int R, int EPI, int XM, bool DOT>
void sell_launch(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const Sell &s = *A.sell;
    SellView m{s.hdr.as<int4>(), s.slice_ptr.as<int64_t>(), s.slice_w.as<int32_t>(), s.slice_aux.as<int64_t>(),
               s.offs.as<int32_t>(),
               s.cols.as<int32_t>(), s.vals.ptr, s.nslices, A.nrows, A.ncols};
    // one wave of resident CTAs (grid-stride over slices)
    static int per_sm = 0;
    if (per_sm == 0) {
        UGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sell_spmv<V, T, R, EPI, XM, DOT>,
                                                                kSpmvWarps * 32, 0));
        if (per_sm < 1) per_sm = 1;
    }
    int64_t want = (s.nslices + kSpmvWarps - 1) / kSpmvWarps;
    int g = int(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(ctx.sms) * per_sm)));
    if constexpr (DOT) g = std::min(g, kSpmvDotGrid);
    k_sell_spmv<V, T, R, EPI, XM, DOT><<<g, kSpmvWarps * 32, 0, ctx.stream>>>(m, make_epi<T>(a));
}

template <class V, class T, int EPI, int XM, bool DOT>
void csr_launch(Context &ctx, const Mat &A, const SpmvArgs &a) {
    double avg = A.nrows ? double(A.nnz) / double(A.nrows) : 0;
    const int32_t *rp = A.rowptr.as<int32_t>();
    const int32_t *ci = A.colidx.as<int32_t>();
    const V *cv = A.vals.as<V>();
    auto e = make_epi<T>(a);
    auto go = [&](auto Gc) {
        constexpr int G = decltype(Gc)::value;
        int g = spmv_grid(ctx, 256 / G, A.nrows);
        if constexpr (DOT) g = std::min(g, kSpmvDotGrid);
        k_csr_spmv<V, T, G, EPI, XM, DOT><<<g, 256, 0, ctx.stream>>>(rp, ci, cv, A.nrows, e);
    };
    if (avg <= 2) go(std::integral_constant<int, 1>{});
    else if (avg <= 6) go(std::integral_constant<int, 4>{});
    else if (avg <= 16) go(std::integral_constant<int, 8>{});
    else go(std::integral_constant<int, 32>{});
}

template <class V, class T, int EPI, int XM, bool DOT>
void dispatch_fmt(Context &ctx, const Mat &A, const SpmvArgs &a) {
    if (a.use_csr || A.format == UGPU_FORMAT_CSR || !A.sell) {
        csr_launch<V, T, EPI, XM, DOT>(ctx, A, a);
    } else {
        constexpr int R = std::is_same<V, double>::value ? 2 : 4;
        UGPU_CHECK(A.sell->R == R, UGPU_ERR_INTERNAL, "sliced-ELL rows-per-thread mismatch");
        sell_launch<V, T, R, EPI, XM, DOT>(ctx, A, a);
    }
}

template <class V, class T>
void dispatch_epi(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const int xm = a.p ? 1 : a.xmode;
    const bool dot = a.dot_partials != nullptr;
    UGPU_CHECK(xm >= 0 && xm <= 2, UGPU_ERR_INTERNAL, "unknown SpMV input mode");
#define UGPU_EPI_CASE(E)                                                                   \
    case E:                                                                                \
        UGPU_CHECK(xm == 0 && !dot, UGPU_ERR_INTERNAL, "fused forms need EPI_STORE/EPI_JACOBI"); \
        dispatch_fmt<V, T, E, 0, false>(ctx, A, a);                                        \
        break;
    switch (a.epilogue) {
        case EPI_STORE:
            UGPU_CHECK(xm != 2, UGPU_ERR_INTERNAL, "scaled input needs a Jacobi epilogue");
            if (xm == 1 && dot) dispatch_fmt<V, T, EPI_STORE, 1, true>(ctx, A, a);
            else if (xm == 1) dispatch_fmt<V, T, EPI_STORE, 1, false>(ctx, A, a);
            else if (dot) dispatch_fmt<V, T, EPI_STORE, 0, true>(ctx, A, a);
            else dispatch_fmt<V, T, EPI_STORE, 0, false>(ctx, A, a);
            break;
        case EPI_JACOBI:
            UGPU_CHECK(xm != 1 && !dot, UGPU_ERR_INTERNAL, "Jacobi sweep: plain or scaled input");
            if (xm == 2) dispatch_fmt<V, T, EPI_JACOBI, 2, false>(ctx, A, a);
            else dispatch_fmt<V, T, EPI_JACOBI, 0, false>(ctx, A, a);
            break;
        case EPI_PJACOBI:
            UGPU_CHECK(xm != 1 && !dot, UGPU_ERR_INTERNAL, "PointJacobi sweep: plain or scaled input");
            if (xm == 2) dispatch_fmt<V, T, EPI_PJACOBI, 2, false>(ctx, A, a);
            else dispatch_fmt<V, T, EPI_PJACOBI, 0, false>(ctx, A, a);
            break;
        UGPU_EPI_CASE(EPI_ADD)
        UGPU_EPI_CASE(EPI_RESIDUAL)
        UGPU_EPI_CASE(EPI_SUB)
        UGPU_EPI_CASE(EPI_SCALE)
        UGPU_EPI_CASE(EPI_CHEB)
        UGPU_EPI_CASE(EPI_CHEB0)
        default: throw Error(UGPU_ERR_ARG, "unknown SpMV epilogue");
    }
#undef UGPU_EPI_CASE
}

}  // namespace

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
void build_sell(Mat &A) {
    Context &ctx = *A.ctx;
    auto s = std::make_unique<Sell>();
    const int sval = int(dtype_size(A.vdtype));
    s->R = (A.vdtype == UGPU_F64) ? 2 : 4;
    s->S = 32 * s->R;
    const int S = s->S;
    s->nslices = (A.nrows + S - 1) / S;
    const int64_t ns = s->nslices;
    Buffer width, offs_tmp;
    width.alloc(sizeof(int32_t) * std::max<int64_t>(ns, 1));
    offs_tmp.alloc(sizeof(int32_t) * std::max<int64_t>(ns, 1) * kMaxDiagSlots);
    const int gA = int(std::min<int64_t>(std::max<int64_t>(ns, 1), int64_t(ctx.sms) * 16));
    if (ns > 0) {
        k_sell_analyze<<<gA, kAnalyzeThreads, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                               A.nrows, S, ns, sval, width.as<int32_t>(),
                                                               offs_tmp.as<int32_t>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    std::vector<int32_t> hw(ns);
    if (ns) UGPU_CUDA(cudaMemcpyAsync(hw.data(), width.ptr, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    std::vector<int64_t> sptr(ns + 1, 0), aux(ns, 0);
    int64_t noffs = 0, ncol = 0, ndiag = 0;
    int maxw = 0;
    for (int64_t i = 0; i < ns; ++i) {
        int w = hw[i];
        int wd = w >= 0 ? w : -w;
        maxw = std::max(maxw, wd);
        sptr[i + 1] = sptr[i] + int64_t(wd) * S;
        if (w >= 0) {
            aux[i] = noffs;
            noffs += w;
            ndiag++;
        } else {
            aux[i] = ncol;
            ncol += int64_t(wd) * S;
        }
    }
    s->nstored = sptr[ns];
    s->ndiag_slices = ndiag;
    s->max_width = maxw;
    s->noffs = noffs;
    s->ncols_explicit = ncol;
    s->slice_ptr.alloc(sizeof(int64_t) * (ns + 1));
    s->slice_w.alloc(sizeof(int32_t) * std::max<int64_t>(ns, 1));
    s->slice_aux.alloc(sizeof(int64_t) * std::max<int64_t>(ns, 1));
    s->offs.alloc(sizeof(int32_t) * std::max<int64_t>(noffs, 1));
    s->cols.alloc(sizeof(int32_t) * std::max<int64_t>(ncol, 4));
    s->vals.alloc(size_t(sval) * std::max<int64_t>(s->nstored, 8));
    UGPU_CHECK(noffs < (1ll << 31) && ncol < (1ll << 31), UGPU_ERR_UNSUPPORTED, "sliced ELL: index space above 2^31");
    std::vector<int4> hh(std::max<int64_t>(ns, 1));
    for (int64_t i = 0; i < ns; ++i)
        hh[i] = make_int4(int(uint32_t(uint64_t(sptr[i]) & 0xffffffffu)), int(uint32_t(uint64_t(sptr[i]) >> 32)),
                          hw[i], int(aux[i]));
    s->hdr.alloc(sizeof(int4) * std::max<int64_t>(ns, 1));
    if (ns) UGPU_CUDA(cudaMemcpyAsync(s->hdr.ptr, hh.data(), sizeof(int4) * ns, cudaMemcpyHostToDevice, ctx.stream));
    UGPU_CUDA(cudaMemcpyAsync(s->slice_ptr.ptr, sptr.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice,
                              ctx.stream));
    if (ns) {
        UGPU_CUDA(cudaMemcpyAsync(s->slice_w.ptr, hw.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, ctx.stream));
        UGPU_CUDA(cudaMemcpyAsync(s->slice_aux.ptr, aux.data(), sizeof(int64_t) * ns, cudaMemcpyHostToDevice,
                                  ctx.stream));
        auto fill = [&](auto tag) {
            using V = decltype(tag);
            k_sell_fill<V><<<gA, kAnalyzeThreads, 0, ctx.stream>>>(
                A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(), A.vals.as<V>(), A.nrows, A.ncols, S, ns,
                s->slice_w.as<int32_t>(), s->slice_ptr.as<int64_t>(), s->slice_aux.as<int64_t>(),
                offs_tmp.as<int32_t>(), s->offs.as<int32_t>(), s->cols.as<int32_t>(), s->vals.as<V>());
        };
        if (A.vdtype == UGPU_F64) fill(double{});
        else if (A.vdtype == UGPU_F32) fill(float{});
        else fill(__nv_bfloat16{});
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));  // host vectors above must outlive the copies
    A.sell = std::move(s);
}

void ensure_diag(Mat &A) {
    if (A.has_diag) return;
    Context &ctx = *A.ctx;
    A.diag.alloc(sizeof(double) * std::max<int64_t>(A.nrows, 1));
    if (A.nrows) {
        int g = stream_grid(ctx, A.nrows);
        if (A.vdtype == UGPU_F64)
            k_diag<double><<<g, kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                         A.vals.as<double>(), A.nrows, A.diag.as<double>());
        else if (A.vdtype == UGPU_F32)
            k_diag<float><<<g, kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                        A.vals.as<float>(), A.nrows, A.diag.as<double>());
        else
            k_diag<__nv_bfloat16><<<g, kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(),
                                                                A.vals.as<__nv_bfloat16>(), A.nrows,
                                                                A.diag.as<double>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    A.has_diag = true;
}

void validate_csr(Mat &A) {
    Context &ctx = *A.ctx;
    Buffer flag;
    flag.alloc(sizeof(int));
    UGPU_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), ctx.stream));
    int32_t ends[2] = {0, 0};
    UGPU_CUDA(cudaMemcpyAsync(&ends[0], A.rowptr.as<int32_t>(), sizeof(int32_t), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaMemcpyAsync(&ends[1], A.rowptr.as<int32_t>() + A.nrows, sizeof(int32_t), cudaMemcpyDeviceToHost,
                              ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    UGPU_CHECK(ends[0] == 0 && int64_t(ends[1]) == A.nnz, UGPU_ERR_ARG, "CSR: rowptr[0] != 0 or rowptr[n] != nnz");
    int h = 0;
    if (A.nrows) {
        k_check_rowptr<<<stream_grid(ctx, A.nrows), kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.nrows, A.nnz,
                                                                            flag.as<int>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
        UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
        UGPU_CHECK(h == 0, UGPU_ERR_ARG, "CSR: rowptr is not non-decreasing within [0, nnz]");
        k_check_cols<<<stream_grid(ctx, A.nrows), kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(),
                                                                          A.colidx.as<int32_t>(), A.nrows, A.ncols,
                                                                          flag.as<int>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
        UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
        UGPU_CHECK(!(h & 2), UGPU_ERR_ARG, "CSR: column index out of range");
        UGPU_CHECK(!(h & 4), UGPU_ERR_ARG, "CSR: column indices must be strictly ascending within each row");
    }
}

void finalize_matrix(Mat &A) {
    Context &ctx = *A.ctx;
    if (A.nrows) {
        Buffer mx;
        mx.alloc(sizeof(unsigned int));
        UGPU_CUDA(cudaMemsetAsync(mx.ptr, 0, sizeof(unsigned int), ctx.stream));
        k_row_lengths_max<<<stream_grid(ctx, A.nrows), kBlock, 0, ctx.stream>>>(A.rowptr.as<int32_t>(), A.nrows,
                                                                               mx.as<unsigned int>());
        ctx.launches++;
        unsigned int h = 0;
        UGPU_CUDA(cudaMemcpyAsync(&h, mx.ptr, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx.stream));
        UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
        A.max_row = h;
    }
    // very long rows are better served by the warp-per-row CSR kernel; matrices without
    // entries or columns never touch x and stay in CSR
    if (A.max_row <= 4 * kMaxDiagSlots && A.nnz > 0 && A.ncols > 0) {
        build_sell(A);
        A.format = UGPU_FORMAT_SELL;
    } else {
        A.format = UGPU_FORMAT_CSR;
    }
}

std::unique_ptr<Mat> make_csr_device(Context &ctx, int64_t nrows, int64_t ncols, int64_t nnz, int vdtype) {
    auto A = std::make_unique<Mat>();
    A->ctx = &ctx;
    A->nrows = nrows;
    A->ncols = ncols;
    A->nnz = nnz;
    A->vdtype = vdtype;
    A->rowptr.alloc(sizeof(int32_t) * (nrows + 1));
    A->colidx.alloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1));
    A->vals.alloc(dtype_size(vdtype) * std::max<int64_t>(nnz, 1));
    return A;
}

std::unique_ptr<Mat> cast_matrix(const Mat &A, int vdtype) {
    Context &ctx = *A.ctx;
    auto B = make_csr_device(ctx, A.nrows, A.ncols, A.nnz, vdtype);
    UGPU_CUDA(cudaMemcpyAsync(B->rowptr.ptr, A.rowptr.ptr, sizeof(int32_t) * (A.nrows + 1), cudaMemcpyDeviceToDevice,
                              ctx.stream));
    if (A.nnz) {
        UGPU_CUDA(cudaMemcpyAsync(B->colidx.ptr, A.colidx.ptr, sizeof(int32_t) * A.nnz, cudaMemcpyDeviceToDevice,
                                  ctx.stream));
        launch_convert(ctx, A.vals.ptr, A.vdtype, B->vals.ptr, vdtype, A.nnz);
    }
    B->max_row = A.max_row;
    finalize_matrix(*B);
    return B;
}

void launch_spmv(Context &ctx, const Mat &A, const SpmvArgs &a) {
    if (A.nrows == 0) return;
    if (a.vec_dtype == UGPU_F64) {
        UGPU_CHECK(A.vdtype == UGPU_F64, UGPU_ERR_UNSUPPORTED, "FP64 vectors need an FP64 matrix");
        dispatch_epi<double, double>(ctx, A, a);
    } else if (a.vec_dtype == UGPU_F32) {
        if (A.vdtype == UGPU_F32) dispatch_epi<float, float>(ctx, A, a);
        else if (A.vdtype == UGPU_BF16) dispatch_epi<__nv_bfloat16, float>(ctx, A, a);
        else throw Error(UGPU_ERR_UNSUPPORTED, "FP32 vectors need an FP32 or BF16 matrix");
    } else {
        throw Error(UGPU_ERR_UNSUPPORTED, "SpMV vectors must be FP64 or FP32");
    }
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

}  // namespace ugpu

using namespace ugpu;

namespace {
void check_spmv_vec(const Mat &A, const Vec *x, int64_t n, const char *what) {
    UGPU_CHECK(x != nullptr, UGPU_ERR_ARG, std::string("null vector: ") + what);
    UGPU_CHECK(x->n == n, UGPU_ERR_ARG, std::string("size mismatch: ") + what);
}
}  // namespace

extern "C" {

int ugpu_csr_create(ugpu_ctx *ctx, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t *rowptr,
                    const int32_t *colidx, const double *values, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(rowptr);
    UGPU_CHECK(nrows >= 0 && ncols >= 0 && nnz >= 0 && nnz < (1ll << 31), UGPU_ERR_ARG, "CSR: bad sizes");
    UGPU_CHECK(nnz == 0 || (colidx && values), UGPU_ERR_ARG, "CSR: null arrays");
    auto &c = ctx->impl;
    auto A = make_csr_device(c, nrows, ncols, nnz, UGPU_F64);
    UGPU_CUDA(cudaMemcpyAsync(A->rowptr.ptr, rowptr, sizeof(int32_t) * (nrows + 1), cudaMemcpyHostToDevice, c.stream));
    if (nnz) {
        UGPU_CUDA(cudaMemcpyAsync(A->colidx.ptr, colidx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, c.stream));
        UGPU_CUDA(cudaMemcpyAsync(A->vals.ptr, values, sizeof(double) * nnz, cudaMemcpyHostToDevice, c.stream));
    }
    validate_csr(*A);
    finalize_matrix(*A);
    auto h = new ugpu_mat;
    h->impl = std::move(*A);
    *out = h;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_csr_create_device(ugpu_ctx *ctx, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t *rowptr,
                           const int32_t *colidx, const double *values, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_REQUIRE(rowptr);
    UGPU_CHECK(nrows >= 0 && ncols >= 0 && nnz >= 0 && nnz < (1ll << 31), UGPU_ERR_ARG, "CSR: bad sizes");
    UGPU_CHECK(nnz == 0 || (colidx && values), UGPU_ERR_ARG, "CSR: null arrays");
    auto &c = ctx->impl;
    auto A = make_csr_device(c, nrows, ncols, nnz, UGPU_F64);
    UGPU_CUDA(cudaMemcpyAsync(A->rowptr.ptr, rowptr, sizeof(int32_t) * (nrows + 1), cudaMemcpyDeviceToDevice,
                              c.stream));
    if (nnz) {
        UGPU_CUDA(cudaMemcpyAsync(A->colidx.ptr, colidx, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, c.stream));
        UGPU_CUDA(cudaMemcpyAsync(A->vals.ptr, values, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, c.stream));
    }
    validate_csr(*A);
    finalize_matrix(*A);
    auto h = new ugpu_mat;
    h->impl = std::move(*A);
    *out = h;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_mat_destroy(ugpu_mat *A) {
    UGPU_ABI_BEGIN
    delete A;
    UGPU_ABI_END(nullptr)
}

int ugpu_mat_info(const ugpu_mat *A, int64_t *nrows, int64_t *ncols, int64_t *nnz, int *value_dtype) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    if (nrows) *nrows = A->impl.nrows;
    if (ncols) *ncols = A->impl.ncols;
    if (nnz) *nnz = A->impl.nnz;
    if (value_dtype) *value_dtype = A->impl.vdtype;
    UGPU_ABI_END(nullptr)
}

int ugpu_csr_download(const ugpu_mat *A, int32_t *rowptr, int32_t *colidx, double *values) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = A->impl;
    auto &c = *M.ctx;
    if (rowptr)
        UGPU_CUDA(cudaMemcpyAsync(rowptr, M.rowptr.ptr, sizeof(int32_t) * (M.nrows + 1), cudaMemcpyDeviceToHost,
                                  c.stream));
    if (colidx && M.nnz)
        UGPU_CUDA(cudaMemcpyAsync(colidx, M.colidx.ptr, sizeof(int32_t) * M.nnz, cudaMemcpyDeviceToHost, c.stream));
    if (values && M.nnz) {
        if (M.vdtype == UGPU_F64) {
            UGPU_CUDA(cudaMemcpyAsync(values, M.vals.ptr, sizeof(double) * M.nnz, cudaMemcpyDeviceToHost, c.stream));
        } else {
            Buffer tmp;
            tmp.alloc(sizeof(double) * M.nnz);
            launch_convert(c, M.vals.ptr, M.vdtype, tmp.ptr, UGPU_F64, M.nnz);
            UGPU_CUDA(cudaMemcpyAsync(values, tmp.ptr, sizeof(double) * M.nnz, cudaMemcpyDeviceToHost, c.stream));
            UGPU_CUDA(cudaStreamSynchronize(c.stream));
        }
    }
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_mat_update_values(ugpu_mat *A, const double *values) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = A->impl;
    auto &c = *M.ctx;
    UGPU_CHECK(M.nnz == 0 || values, UGPU_ERR_ARG, "null values");
    if (M.nnz) {
        Buffer tmp;
        tmp.alloc(sizeof(double) * M.nnz);
        UGPU_CUDA(cudaMemcpyAsync(tmp.ptr, values, sizeof(double) * M.nnz, cudaMemcpyHostToDevice, c.stream));
        launch_convert(c, tmp.ptr, UGPU_F64, M.vals.ptr, M.vdtype, M.nnz);
        UGPU_CUDA(cudaStreamSynchronize(c.stream));
    }
    M.has_diag = false;
    finalize_matrix(M);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_mat_cast(const ugpu_mat *A, int value_dtype, ugpu_mat **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(out);
    dtype_size(value_dtype);
    auto B = cast_matrix(A->impl, value_dtype);
    auto h = new ugpu_mat;
    h->impl = std::move(*B);
    *out = h;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_mat_set_format(ugpu_mat *A, int format) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_CHECK(format == UGPU_FORMAT_CSR || format == UGPU_FORMAT_SELL, UGPU_ERR_ARG, "unknown format");
    if (format == UGPU_FORMAT_SELL && (A->impl.nnz == 0 || A->impl.ncols == 0)) format = UGPU_FORMAT_CSR;
    if (format == UGPU_FORMAT_SELL && !A->impl.sell) build_sell(A->impl);
    A->impl.format = format;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_mat_sell_info(const ugpu_mat *A, int64_t *nslices, int64_t *nstored, int64_t *ndiag_slices,
                       int *rows_per_slice) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_CHECK(A->impl.sell != nullptr, UGPU_ERR_STATE, "matrix has no sliced-ELL layout");
    auto &s = *A->impl.sell;
    if (nslices) *nslices = s.nslices;
    if (nstored) *nstored = s.nstored;
    if (ndiag_slices) *ndiag_slices = s.ndiag_slices;
    if (rows_per_slice) *rows_per_slice = s.S;
    UGPU_ABI_END(nullptr)
}

int ugpu_diag(const ugpu_mat *A, ugpu_vec *d) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(d);
    auto &M = const_cast<Mat &>(A->impl);
    UGPU_CHECK(d->impl.n == M.nrows, UGPU_ERR_ARG, "diag: size mismatch");
    ensure_diag(M);
    launch_convert(*M.ctx, M.diag.ptr, UGPU_F64, d->impl.buf.ptr, d->impl.dtype, M.nrows);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_spmv(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = A->impl;
    check_spmv_vec(M, x ? &x->impl : nullptr, M.ncols, "x");
    check_spmv_vec(M, y ? &y->impl : nullptr, M.nrows, "y");
    UGPU_CHECK(x->impl.dtype == y->impl.dtype, UGPU_ERR_ARG, "x and y dtypes differ");
    UGPU_CHECK(x->impl.buf.ptr != y->impl.buf.ptr, UGPU_ERR_ARG, "y must not alias x");
    SpmvArgs a;
    a.x = x->impl.buf.ptr;
    a.y = y->impl.buf.ptr;
    a.vec_dtype = x->impl.dtype;
    a.epilogue = EPI_STORE;
    launch_spmv(*M.ctx, M, a);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_spmv_add(const ugpu_mat *A, const ugpu_vec *x, const ugpu_vec *v, ugpu_vec *y) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = A->impl;
    check_spmv_vec(M, x ? &x->impl : nullptr, M.ncols, "x");
    check_spmv_vec(M, v ? &v->impl : nullptr, M.nrows, "v");
    check_spmv_vec(M, y ? &y->impl : nullptr, M.nrows, "y");
    UGPU_CHECK(x->impl.dtype == y->impl.dtype && v->impl.dtype == y->impl.dtype, UGPU_ERR_ARG, "dtypes differ");
    UGPU_CHECK(x->impl.buf.ptr != y->impl.buf.ptr, UGPU_ERR_ARG, "y must not alias x");
    SpmvArgs a;
    a.x = x->impl.buf.ptr;
    a.v = v->impl.buf.ptr;
    a.y = y->impl.buf.ptr;
    a.vec_dtype = x->impl.dtype;
    a.epilogue = EPI_ADD;
    launch_spmv(*M.ctx, M, a);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_residual(const ugpu_mat *A, const ugpu_vec *b, const ugpu_vec *x, ugpu_vec *r) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = A->impl;
    check_spmv_vec(M, x ? &x->impl : nullptr, M.ncols, "x");
    check_spmv_vec(M, b ? &b->impl : nullptr, M.nrows, "b");
    check_spmv_vec(M, r ? &r->impl : nullptr, M.nrows, "r");
    UGPU_CHECK(x->impl.dtype == r->impl.dtype && b->impl.dtype == r->impl.dtype, UGPU_ERR_ARG, "dtypes differ");
    UGPU_CHECK(x->impl.buf.ptr != r->impl.buf.ptr, UGPU_ERR_ARG, "r must not alias x");
    SpmvArgs a;
    a.x = x->impl.buf.ptr;
    a.v = b->impl.buf.ptr;
    a.y = r->impl.buf.ptr;
    a.vec_dtype = x->impl.dtype;
    a.epilogue = EPI_RESIDUAL;
    launch_spmv(*M.ctx, M, a);
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

int ugpu_jacobi_sweep(const ugpu_mat *A, const ugpu_vec *b, const ugpu_vec *x, double omega, ugpu_vec *x_out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    auto &M = const_cast<Mat &>(A->impl);
    UGPU_CHECK(M.nrows == M.ncols, UGPU_ERR_ARG, "Jacobi needs a square matrix");
    check_spmv_vec(M, x ? &x->impl : nullptr, M.ncols, "x");
    check_spmv_vec(M, b ? &b->impl : nullptr, M.nrows, "b");
    check_spmv_vec(M, x_out ? &x_out->impl : nullptr, M.nrows, "x_out");
    UGPU_CHECK(x->impl.buf.ptr != x_out->impl.buf.ptr, UGPU_ERR_ARG, "x_out must not alias x");
    UGPU_CHECK(x->impl.dtype == x_out->impl.dtype && b->impl.dtype == x->impl.dtype, UGPU_ERR_ARG, "dtypes differ");
    auto &c = *M.ctx;
    ensure_diag(M);
    // weights w = omega * pseudo_inverse(diag) (tol 0, as Jacobi::update)
    Buffer w64, w;
    w64.alloc(sizeof(double) * std::max<int64_t>(M.nrows, 1));
    Vec din, dout;
    din.ctx = dout.ctx = &c;
    din.n = dout.n = M.nrows;
    din.dtype = dout.dtype = UGPU_F64;
    din.buf.borrow(M.diag.ptr, M.diag.bytes);
    dout.buf.borrow(w64.ptr, w64.bytes);
    launch_pseudo_inverse(c, din, dout, 0.0);
    Vec wv;
    wv.ctx = &c;
    wv.n = M.nrows;
    wv.dtype = UGPU_F64;
    wv.buf.borrow(w64.ptr, w64.bytes);
    launch_axpby(c, M.nrows, omega, dout, 0.0, wv);
    const void *wp = w64.ptr;
    if (x->impl.dtype != UGPU_F64) {
        w.alloc(sizeof(float) * std::max<int64_t>(M.nrows, 1));
        launch_convert(c, w64.ptr, UGPU_F64, w.ptr, UGPU_F32, M.nrows);
        wp = w.ptr;
    }
    SpmvArgs a;
    a.x = x->impl.buf.ptr;
    a.v = b->impl.buf.ptr;
    a.w = wp;
    a.y = x_out->impl.buf.ptr;
    a.vec_dtype = x->impl.dtype;
    a.epilogue = EPI_JACOBI;
    launch_spmv(c, M, a);
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

}  // extern "C"
