// CSR matrices, the sliced-ELL layout, and the SpMV-family kernels with fused epilogues.
//
// Reference call sites replaced: PetscMatrix::multiply -> MatMult
// (utopia/backend/petsc/utopia_petsc_Matrix.cpp:1358), MatMultAdd (:1400-1404),
// Eval_Residual (utopia/utopia_core/eval/utopia_Eval_Residual.hpp:19-38), the Jacobi
// sweep (utopia/solvers/smoothers/utopia_Jacobi.hpp:131-141), MatGetDiagonal (:756).
#include <map>
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

// Slice kinds, as encoded in the width word of a slice header:
//   diagonal  0 <= w < kAnchoredTag   entries keyed by col - row (one int32 key per slot)
//   anchored  w - kAnchoredTag        entries keyed by col - anchor(row), anchor = the row's
//                                     first column (one key per slot + one anchor per row)
//   explicit  -w                      one column index per stored entry
// Anchored keying fits transfer operators: every row of an interpolation (or of its
// transpose) has the same shape relative to its first column, so a slice needs as many
// slots as that shape has entries.
constexpr int kAnchoredTag = 1 << 16;

// Sorted distinct keys of a slice; returns the count, or -1 if more than kMaxDiagSlots (or a key
// outside int32).  ANCH: key = col - first column, else col - row.  The keys go into a shared-memory
// hash set (256 slots: inserts stop counting past kMaxDiagSlots, and at most one insert per thread
// is in flight beyond that, so the set never fills), then each distinct key is placed by its rank.
// One pass over the slice's entries, where extracting the minimum key by key took one pass per key.
constexpr int kKeySlots = 256;
static_assert(kKeySlots >= kMaxDiagSlots + kAnalyzeThreads, "key set too small");
template <bool ANCH>
__device__ int slice_keys(const int32_t *rp, const int32_t *ci, int64_t r0, int64_t r1, int32_t *out) {
    __shared__ long long s_tab[kKeySlots];
    __shared__ long long s_key[kMaxDiagSlots];
    __shared__ int s_cnt, s_bad;
    const long long kEmpty = LLONG_MAX;
    for (int i = threadIdx.x; i < kKeySlots; i += blockDim.x) s_tab[i] = kEmpty;
    if (threadIdx.x == 0) {
        s_cnt = 0;
        s_bad = 0;
    }
    __syncthreads();
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int32_t k0 = rp[r], k1 = rp[r + 1];
        const long long base = ANCH ? (k1 > k0 ? (long long)ci[k0] : 0ll) : r;
        for (int32_t k = k0; k < k1; ++k) {
            if (*reinterpret_cast<volatile int *>(&s_bad) || *reinterpret_cast<volatile int *>(&s_cnt) > kMaxDiagSlots)
                break;
            const long long off = (long long)ci[k] - base;
            if (off > INT_MAX || off < INT_MIN) {
                s_bad = 1;
                break;
            }
            unsigned h = (unsigned(off) * 2654435761u) >> 24;  // 8-bit slot index
            bool placed = false;
            for (int probe = 0; probe < kKeySlots && !placed; ++probe) {
                const long long prev = (long long)atomicCAS(reinterpret_cast<unsigned long long *>(&s_tab[h]),
                                                            (unsigned long long)kEmpty, (unsigned long long)off);
                if (prev == kEmpty) {  // a new key
                    if (atomicAdd(&s_cnt, 1) >= kMaxDiagSlots) s_bad = 1;
                    placed = true;
                } else if (prev == off) {
                    placed = true;
                } else {
                    h = (h + 1) & (kKeySlots - 1);
                }
            }
            if (!placed) s_bad = 1;  // a full set (excluded by its size; the loop stays bounded)
        }
    }
    __syncthreads();
    const int bad = s_bad;
    const int nd = s_cnt;
    __syncthreads();
    if (bad) return -1;
    // compact, then place each key by its rank (keys are distinct)
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < kKeySlots; i += blockDim.x)
        if (s_tab[i] != kEmpty) s_key[atomicAdd(&s_cnt, 1)] = s_tab[i];
    __syncthreads();
    for (int t = threadIdx.x; t < nd; t += blockDim.x) {
        const long long k = s_key[t];
        int rank = 0;
        for (int u = 0; u < nd; ++u) rank += s_key[u] < k ? 1 : 0;
        out[rank] = int32_t(k);
    }
    __syncthreads();
    return nd;
}

// per slice: kind and width (the cheapest of the three layouts in bytes)
__global__ void __launch_bounds__(kAnalyzeThreads) k_sell_analyze(const int32_t *rp, const int32_t *ci, int64_t n,
                                                                   int S, int64_t nslices, int sval,
                                                                   int32_t *width, int32_t *offs_tmp) {
    __shared__ int s_maxrow;
    for (int64_t s = blockIdx.x; s < nslices; s += gridDim.x) {
        int64_t r0 = s * S, r1 = min(n, r0 + S);
        if (threadIdx.x == 0) s_maxrow = 0;
        __syncthreads();
        int mr = 0;
        for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) mr = max(mr, rp[r + 1] - rp[r]);
        atomicMax(&s_maxrow, mr);
        __syncthreads();
        const int maxrow = s_maxrow;
        __syncthreads();
        // bytes: diagonal nd*S*sval + 4nd; anchored na*S*sval + 4na + 4S + 8; explicit maxrow*S*(sval+4)
        const long long expl = (long long)maxrow * S * (sval + 4);
        int32_t *keys = offs_tmp + s * kMaxDiagSlots;
        const int nd = maxrow <= kMaxDiagSlots ? slice_keys<false>(rp, ci, r0, r1, keys) : -1;
        int kind_w = -maxrow;
        if (nd >= 0 && (long long)nd * S * sval + 4ll * nd <= expl) {
            kind_w = nd;
        } else if (maxrow <= kMaxDiagSlots) {
            const int na = slice_keys<true>(rp, ci, r0, r1, keys);
            if (na >= 0 && (long long)na * S * sval + 4ll * na + 4ll * S + 8 < expl) kind_w = kAnchoredTag + na;
        }
        if (threadIdx.x == 0) width[s] = kind_w;
        __syncthreads();
    }
}

// Position of row rl of a slice inside one slot of S = 32 R entries: rl itself, or in the
// lane-interleaved layout (lane l owns rows l + 32 r) l R + r for rl = 32 r + l.
__host__ __device__ __forceinline__ int sell_pos(int rl, int S, bool interleaved) {
    return interleaved ? (rl & 31) * (S >> 5) + (rl >> 5) : rl;
}

template <class V>
__global__ void __launch_bounds__(kAnalyzeThreads) k_sell_fill(const int32_t *rp, const int32_t *ci, const V *cv,
                                                                int64_t n, int64_t ncols, int S, int64_t nslices,
                                                                const int32_t *width, const int64_t *sptr,
                                                                const int64_t *aux, const int32_t *offs_tmp,
                                                                int32_t *offs, int32_t *cols, V *vals, bool il) {
    __shared__ int32_t s_off[kMaxDiagSlots];
    __shared__ int s_amin, s_amax;
    for (int64_t s = blockIdx.x; s < nslices; s += gridDim.x) {
        int w = width[s];
        int64_t base = sptr[s];
        int64_t r0 = s * S;
        if (w >= 0 && w < kAnchoredTag) {
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
                    if (slot < w && s_off[slot] == off) vals[base + int64_t(slot) * S + sell_pos(rl, S, il)] = cv[k];
                }
            }
            __syncthreads();
        } else if (w >= kAnchoredTag) {
            // anchors at cols[cb, cb + S) in slot-position order, keys at cols[cb + S, cb + S + wa),
            // then the slice's smallest and largest anchor (the x range its gathers can touch)
            const int wa = w - kAnchoredTag;
            const int64_t cb = aux[s];
            for (int k = threadIdx.x; k < wa; k += blockDim.x) {
                s_off[k] = offs_tmp[s * kMaxDiagSlots + k];
                cols[cb + S + k] = s_off[k];
            }
            if (threadIdx.x == 0) {
                s_amin = INT_MAX;
                s_amax = INT_MIN;
            }
            __syncthreads();
            for (int rl = threadIdx.x; rl < S; rl += blockDim.x) {
                const int64_t r = r0 + rl;
                if (r < n && rp[r + 1] > rp[r]) {
                    atomicMin(&s_amin, ci[rp[r]]);
                    atomicMax(&s_amax, ci[rp[r]]);
                }
            }
            for (int64_t e = threadIdx.x; e < int64_t(wa) * S; e += blockDim.x) vals[base + e] = cvt<V>(0.0);
            __syncthreads();
            const int amin = s_amin == INT_MAX ? 0 : s_amin;
            const int amax = s_amin == INT_MAX ? 0 : s_amax;
            if (threadIdx.x == 0) {
                cols[cb + S + wa] = amin;
                cols[cb + S + wa + 1] = amax;
            }
            for (int rl = threadIdx.x; rl < S; rl += blockDim.x) {
                const int64_t r = r0 + rl;
                const bool has = r < n && rp[r + 1] > rp[r];
                const int32_t a = has ? ci[rp[r]] : amin;  // empty and padding rows: any anchor in range
                const int p = sell_pos(rl, S, il);
                cols[cb + p] = a;
                if (!has) continue;
                int slot = 0;
                for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
                    const int32_t key = ci[k] - a;
                    while (slot < wa && s_off[slot] < key) ++slot;
                    if (slot < wa && s_off[slot] == key) vals[base + int64_t(slot) * S + p] = cv[k];
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
                const int p = sell_pos(rl, S, il);
                for (int k = 0; k < wd; ++k) {
                    bool real = k < len;
                    vals[base + int64_t(k) * S + p] = real ? cv[start + k] : cvt<V>(0.0);
                    cols[cb + int64_t(k) * S + p] = real ? ci[start + k] : padcol;
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
    int il;  // lane-interleaved rows
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
    // box-constrained QP input (XM 3): xin = qmode ? x : xalt, and with qmode the step bound (the
    // minimum over rows of qp_alpha_f_key) folded into *qmin with atomicMin
    const int *qmode;
    const T *xalt;
    const T *qx, *qlb, *qub;
    unsigned long long *qmin;
    // final dots of y with FP64 vectors (SpmvArgs::fa, fb)
    const double *fa, *fb;
    double *fpart, *fout;
    unsigned int *fcnt;
    // sw_out = sw .* y (SpmvArgs::sw_out)
    T *sw_out;
    const T *sw;
    int vec_ok;      // every vector pointer above is 16-byte aligned
};

// y_row's share of the final dots
template <class T>
__device__ __forceinline__ void final_dots_row(const EpiParams<T> &e, int64_t row, T y, double &f0, double &f1) {
    const double yd = cvt<double>(y);
    f0 = fma(yd, __ldg(e.fa + row), f0);
    if (e.fb) f1 = fma(yd, __ldg(e.fb + row), f1);
}
// the CTA's final-dot partials, finished by the last CTA (every thread of the CTA calls it)
template <class T>
__device__ __forceinline__ void final_dots_finish(const EpiParams<T> &e, double f0, double f1) {
    const int nd = e.fb ? 2 : 1;
    double a[2] = {f0, f1};
    block_reduce_store<2>(a, nd, e.fpart, gridDim.x, blockIdx.x);
    finish_last_block(nd, e.fpart, gridDim.x, e.fout, e.fcnt);
}

// the MPRGP step bound of one row as an order key (utopia_MPRGP.hpp:289-316, get_alpha_f:
// min((p > 0) ? (x - l) / p : 1e15, (p < 0) ? (x - u) / p : 1e15)), one division, the
// comparisons on the integer pipes
__device__ __forceinline__ unsigned long long qp_alpha_f_key(double x, double p, double l, double u) {
    const long long pk = dkey(p);
    if (pk == 0) return qp_key(1e15);
    const double h = (x - (pk > 0 ? l : u)) / p;
    const unsigned long long hk = qp_key(h), big = qp_key(1e15);
    return hk < big ? hk : big;
}
// A bracket [lo, hi] of qp_alpha_f_key's h = (x - l) / p (p > 0) or (x - u) / p (p < 0) from
// single-precision arithmetic alone, as order keys: the key of the double-precision h lies
// inside.  x, the bound b and p are truncated to binary32 (relative error < 2^-23 each); the
// difference x - b is used only where it does not cancel (|x| + |b| <= 8 |x - b|, so it is within
// 2^-20), and the quotient by the fast reciprocal (2 ulp) stays within 2^-19; the bracket widens it
// by 2^-16.  Rows with p = 0, and rows whose bound is at infinity on the side p moves towards
// (|b| >= 2^61, |p| < 2^10: h > 2^50 > 1e15), bound at the cap 1e15 and get no bracket
// (lo = hi = ~0); rows outside these cases (operands outside 2^-60 .. 2^60, cancellation) get
// lo = 0, hi = ~0: they are always evaluated exactly.
__device__ __forceinline__ void qp_alpha_f_bracket(double x, double p, double l, double u, unsigned long long &lo,
                                                   unsigned long long &hi) {
    const long long pk = dkey(p);
    if (pk == 0) {
        lo = hi = ~0ull;
        return;
    }
    const double b = pk > 0 ? l : u;
    const uint64_t bx = (uint64_t)__double_as_longlong(x), bb = (uint64_t)__double_as_longlong(b),
                   bp = (uint64_t)__double_as_longlong(p);
    const uint32_t ex = uint32_t(bx >> 52) & 0x7ffu, eb = uint32_t(bb >> 52) & 0x7ffu,
                   ep = uint32_t(bp >> 52) & 0x7ffu;
    lo = 0ull;  // by default: evaluated exactly
    hi = ~0ull;
    const bool x_ok = ex - 963u <= 120u || (bx << 1) == 0;  // 2^-60 <= |x| < 2^61, or zero
    const bool b_ok = eb - 963u <= 120u || (bb << 1) == 0;
    if (ep - 963u > 120u || !x_ok) return;
    if (!b_ok) {
        // b beyond 2^61 on the far side (b < 0 for p > 0, b > 0 for p < 0): h > 2^60 / 2^10
        const bool far = (pk > 0) == ((bb >> 63) != 0);
        if (eb >= 1084u && eb != 2047u && ep < 1033u && far) lo = hi = ~0ull;
        return;
    }
    auto trunc32 = [](uint64_t v, uint32_t e) {
        if ((v << 1) == 0) return __uint_as_float(uint32_t(v >> 32) & 0x80000000u);
        return __uint_as_float((uint32_t(v >> 32) & 0x80000000u) | ((e - 896u) << 23) |
                               uint32_t((v & 0xfffffffffffffull) >> 29));
    };
    const float xf = trunc32(bx, ex), bf = trunc32(bb, eb);
    const float af = xf - bf;
    if (!(fabsf(xf) + fabsf(bf) <= 8.0f * fabsf(af))) return;  // x - b cancels: evaluated exactly
    const float q = __fdividef(af, trunc32(bp, ep));
    const float q1 = q * (1.0f - 0x1p-16f), q2 = q * (1.0f + 0x1p-16f);
    lo = qp_key(f2d_bits(fminf(q1, q2)));
    hi = qp_key(f2d_bits(fmaxf(q1, q2)));
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
// The exact step bounds of a lane's R rows that can still be the minimum (whole warp, converged):
// rows whose bracket starts above the least of the warp's bracket ends, of this thread's minimum
// so far and of the grid's running minimum *gmin cannot be the minimum and skip the division.
// Every value the bound takes is the key of an exactly evaluated row (or 1e15, the cap every
// row's bound has), so the minimum is the one all rows' exact keys give.  Improvements go to
// *gmin at once, so that later slices filter against them.
template <int R, class T>
__device__ __forceinline__ void qp_alpha_f_select(const EpiParams<T> &e, const int64_t (&row)[R],
                                                  const double (&p)[R], const unsigned long long (&lo)[R],
                                                  unsigned long long hmin, unsigned long long *gmin,
                                                  unsigned long long &qmn) {
    hmin = warp_min_u64(hmin);
    const unsigned long long g = *reinterpret_cast<volatile const unsigned long long *>(gmin);
    unsigned long long b = hmin < qmn ? hmin : qmn;
    b = g < b ? g : b;
    unsigned long long found = ~0ull;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (lo[r] <= b) {  // a candidate: its operands again from the caches (few rows per warp)
            const int64_t i = row[r];
            const unsigned long long k = qp_alpha_f_key(double(e.qx[i]), p[r], double(e.qlb[i]), double(e.qub[i]));
            found = k < found ? k : found;
        }
    }
    qmn = found < qmn ? found : qmn;
    found = warp_min_u64(found);
    if ((threadIdx.x & 31) == 0 && found < g) atomicMin(gmin, found);
}

// CTA minimum of the keys, folded into *out with one atomicMin (every thread of the CTA calls it)
__device__ __forceinline__ void block_atomic_min_u64(unsigned long long v, unsigned long long *out) {
    __shared__ unsigned long long sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_min_u64(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        unsigned long long t = lane < nw ? sh[lane] : ~0ull;
        t = warp_min_u64(t);
        if (lane == 0) atomicMin(out, t);
    }
}

// R consecutive entries of a vector as 16-byte loads / stores (R * sizeof(T) is 16 or 32;
// the caller guarantees 16-byte alignment)
template <class T, int R>
__device__ __forceinline__ void ld16(const T *p, T (&a)[R]) {
    static_assert((sizeof(T) * R) % 16 == 0, "16-byte rows");
#pragma unroll
    for (int i = 0; i < int(sizeof(T) * R / 16); ++i) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p) + i);
        memcpy(reinterpret_cast<char *>(a) + 16 * i, &t, 16);
    }
}
template <class T, int R>
__device__ __forceinline__ void st16(T *p, const T (&a)[R]) {
#pragma unroll
    for (int i = 0; i < int(sizeof(T) * R / 16); ++i) {
        float4 t;
        memcpy(&t, reinterpret_cast<const char *>(a) + 16 * i, 16);
        reinterpret_cast<float4 *>(p)[i] = t;
    }
}

// the product's input vector: x (XM 0), x + beta*p (XM 1), or w .* v formed on the fly
// (XM 2: the first Jacobi iterate from zero, x1 = w .* rhs)
template <class T, int XM>
__device__ __forceinline__ T xin_at(const EpiParams<T> &e, T beta, int64_t j, bool qpc = false) {
    if constexpr (XM == 1) {
        return __ldg(e.x + j) + beta * __ldg(e.wvec + j);
    } else if constexpr (XM == 3) {
        return qpc ? __ldg(e.x + j) : __ldg(e.xalt + j);
    } else if constexpr (XM == 2) {
        return __ldg(e.w + j) * __ldg(e.v + j);
    } else {
        return __ldg(e.x + j);
    }
}

// which per-row vectors an epilogue reads (besides the product input x)
template <int EPI>
constexpr bool epi_reads_v() {
    return EPI == EPI_ADD || EPI == EPI_RESIDUAL || EPI == EPI_SUB || EPI == EPI_JACOBI || EPI == EPI_PJACOBI;
}
template <int EPI>
constexpr bool epi_reads_w() {
    return EPI == EPI_JACOBI || EPI == EPI_SCALE || EPI == EPI_PJACOBI || EPI == EPI_SCALE_SW;
}
// epilogues that also write sw_out = sw .* y (compiled only into those instantiations)
template <int EPI>
constexpr bool epi_writes_sw() {
    return EPI == EPI_STORE_SW || EPI == EPI_SCALE_SW;
}
template <int EPI, int XM, bool DOT>
constexpr bool epi_reads_x() {
    return XM != 0 || EPI == EPI_JACOBI || EPI == EPI_CHEB || DOT;
}

// the stateless epilogues, from the row's product acc, input x, vector v and weight w
template <class T, int EPI>
__device__ __forceinline__ T epi_row(T acc, T xrow, T vrow, T wrow) {
    if constexpr (EPI == EPI_ADD) return acc + vrow;
    if constexpr (EPI == EPI_RESIDUAL) return vrow - acc;
    if constexpr (EPI == EPI_SUB) return acc - vrow;
    if constexpr (EPI == EPI_JACOBI) return xrow + wrow * (vrow - acc);
    if constexpr (EPI == EPI_SCALE || EPI == EPI_SCALE_SW) return wrow * acc;
    if constexpr (EPI == EPI_PJACOBI) return wrow * (vrow - acc);
    return acc;
}

// row epilogue; returns the value stored to y[row]
template <class T, int EPI>
__device__ __forceinline__ T epilogue(const EpiParams<T> &e, int64_t row, T acc, T xrow) {
    if constexpr (EPI != EPI_CHEB && EPI != EPI_CHEB0) {
        T vrow = T(0), wrow = T(0);
        if constexpr (epi_reads_v<EPI>()) vrow = e.v[row];
        if constexpr (epi_reads_w<EPI>()) wrow = e.w[row];
        return epi_row<T, EPI>(acc, xrow, vrow, wrow);
    }
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
constexpr int kStagedMaxWidth = 32;  // widest diagonal slice the staged kernel takes

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
    bool qpc = false;
    if constexpr (XM == 3) qpc = *e.qmode != 0;
    double dacc = 0.0, dacc2 = 0.0, f0 = 0.0, f1 = 0.0;
    // QP step bound: every row's bound is at most 1e15 (n >= 1), so the minimum starts there
    unsigned long long qmn = XM == 3 ? qp_key(1e15) : ~0ull;
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
        const bool keyed = s < ns && h.w >= 0;  // diagonal or anchored
        const bool anch = h.w >= kAnchoredTag;
        const int wk = anch ? h.w - kAnchoredTag : h.w;
        const int32_t *kp = anch ? m.cols + h.aux + S : m.offs + h.aux;
        lo = (keyed && lane < wk) ? __ldg(kp + lane) : 0;
        hi = (keyed && lane + 32 < wk) ? __ldg(kp + 32 + lane) : 0;
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
        // a lane's rows: row0 + r * rs (consecutive, or 32 apart in the interleaved layout)
        const int rs = m.il ? 32 : 1;
        const int64_t row0 = s * S + (m.il ? int64_t(lane) : int64_t(lane) * R);
        T acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = T(0);
        if (w >= 0 && w < kAnchoredTag) {
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
                    int c = r0i + r * rs + off;
                    c = c < 0 ? 0 : (c > cmax ? cmax : c);
                    acc[r] = fma(T(v[r]), xin_at<T, XM>(e, beta, c, qpc), acc[r]);
                }
            }
        } else if (w >= kAnchoredTag) {
            // anchored: row r gathers at gb[r] + key, gb = the row's first column (stored at
            // the row's slot position lane R + r); keys broadcast by shuffle as above
            const int wk = w - kAnchoredTag;
            const int cmax = int(m.ncols) - 1;
            int gb[R];
            load_cols<R>(m.cols + aux + lane * R, gb);
            UGPU_PRAGMA_UNROLL(UGPU_SELL_UNROLL)
            for (int k = 0; k < wk; ++k) {
                const int32_t off = __shfl_sync(0xffffffffu, k < 32 ? off_lo : off_hi, k & 31);
                LV v[R];
                VecLoad<V, R>::load(vals + base + int64_t(k) * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    int c = gb[r] + off;
                    c = c < 0 ? 0 : (c > cmax ? cmax : c);
                    acc[r] = fma(T(v[r]), xin_at<T, XM>(e, beta, c, qpc), acc[r]);
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
                for (int r = 0; r < R; ++r) acc[r] = fma(T(v[r]), xin_at<T, XM>(e, beta, c[r], qpc), acc[r]);
            }
        }
        constexpr bool kVecEpi = EPI != EPI_CHEB && EPI != EPI_CHEB0;
        // QP step bound: the lane's rows, their p and their brackets (XM == 3)
        double qp_[R];
        int64_t qrow_[R];
        unsigned long long qlo_[R], qhmin = ~0ull;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            qlo_[r] = ~0ull;
            qp_[r] = 0.0;
            qrow_[r] = 0;
        }
        if (kVecEpi && e.vec_ok && !m.il && row0 + R <= m.nrows) {
            // a lane's R rows are consecutive: its epilogue vectors are 16-byte loads
            T xr[R], vr[R], wr[R], out[R];
            if constexpr (epi_reads_x<EPI, XM, DOT>()) {
                if constexpr (XM == 1) {
                    T a[R], b[R];
                    ld16<T, R>(e.x + row0, a);
                    ld16<T, R>(e.wvec + row0, b);
#pragma unroll
                    for (int r = 0; r < R; ++r) xr[r] = a[r] + beta * b[r];
                    st16<T, R>(e.pout + row0, xr);
                } else if constexpr (XM == 2) {
                    T a[R], b[R];
                    ld16<T, R>(e.w + row0, a);
                    ld16<T, R>(e.v + row0, b);
#pragma unroll
                    for (int r = 0; r < R; ++r) xr[r] = a[r] * b[r];
                } else if constexpr (XM == 3) {
                    if (qpc) {
                        T xx[R], l[R], u[R];
                        ld16<T, R>(e.x + row0, xr);
                        ld16<T, R>(e.qx + row0, xx);
                        ld16<T, R>(e.qlb + row0, l);
                        ld16<T, R>(e.qub + row0, u);
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            qrow_[r] = row0 + r;
                            qp_[r] = double(xr[r]);
                            unsigned long long hi;
                            qp_alpha_f_bracket(double(xx[r]), qp_[r], double(l[r]), double(u[r]), qlo_[r], hi);
                            qhmin = hi < qhmin ? hi : qhmin;
                        }
                    } else {
                        ld16<T, R>(e.xalt + row0, xr);
                    }
                } else {
                    ld16<T, R>(e.x + row0, xr);
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) xr[r] = T(0);
            }
            if constexpr (epi_reads_v<EPI>()) ld16<T, R>(e.v + row0, vr);
            if constexpr (epi_reads_w<EPI>()) ld16<T, R>(e.w + row0, wr);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                out[r] = epi_row<T, EPI>(acc[r], xr[r], epi_reads_v<EPI>() ? vr[r] : T(0),
                                         epi_reads_w<EPI>() ? wr[r] : T(0));
            }
            st16<T, R>(e.y + row0, out);
            if constexpr (epi_writes_sw<EPI>()) {
                T sw[R];
                ld16<T, R>(e.sw + row0, sw);
#pragma unroll
                for (int r = 0; r < R; ++r) sw[r] = sw[r] * out[r];
                st16<T, R>(e.sw_out + row0, sw);
            }
            if (e.fa) {
#pragma unroll
                for (int r = 0; r < R; ++r) final_dots_row<T>(e, row0 + r, out[r], f0, f1);
            }
            if constexpr (DOT) {
                T dr[R];
                if (e.dv) ld16<T, R>(e.dv + row0, dr);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    dacc = fma(double(xr[r]), double(out[r]), dacc);
                    if (e.dv) dacc2 = fma(double(xr[r]), double(dr[r]), dacc2);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int64_t row = row0 + int64_t(r) * rs;
                if (row < m.nrows) {
                    T xr = T(0);
                    if constexpr (epi_reads_x<EPI, XM, DOT>()) xr = xin_at<T, XM>(e, beta, row, qpc);
                    if constexpr (XM == 1) e.pout[row] = xr;
                    if constexpr (XM == 3) {
                        if (qpc) {
                            qrow_[r] = row;
                            qp_[r] = double(xr);
                            unsigned long long hi;
                            qp_alpha_f_bracket(double(e.qx[row]), qp_[r], double(e.qlb[row]), double(e.qub[row]),
                                               qlo_[r], hi);
                            qhmin = hi < qhmin ? hi : qhmin;
                        }
                    }
                    T out = epilogue<T, EPI>(e, row, acc[r], xr);
                    e.y[row] = out;
                    if constexpr (epi_writes_sw<EPI>()) e.sw_out[row] = e.sw[row] * out;
                    if (e.fa) final_dots_row<T>(e, row, out, f0, f1);
                    if constexpr (DOT) {
                        dacc = fma(double(xr), double(out), dacc);
                        if (e.dv) dacc2 = fma(double(xr), double(e.dv[row]), dacc2);
                    }
                }
            }
        }
        if constexpr (XM == 3) {
            if (qpc) qp_alpha_f_select<R, T>(e, qrow_, qp_, qlo_, qhmin, e.qmin, qmn);
        }
    }
    if (e.fa) final_dots_finish<T>(e, f0, f1);
    if constexpr (XM == 3) {
        if (qpc) block_atomic_min_u64(qmn, e.qmin);
    }
    if constexpr (DOT) {
        const int nd = e.dv ? 2 : 1;
        double a[2] = {dacc, dacc2};
        block_reduce_store<2>(a, nd, e.dot_partials, gridDim.x, blockIdx.x);
        finish_last_block(nd, e.dot_partials, gridDim.x, e.dot_out, e.dot_counter);
    }
}

// ------------------------------------------------------------------------------------
// Shared-memory staged sliced-ELL product (FP32 vectors; FP32 or BF16 values; every slice
// diagonal, lane-interleaved rows).
//
// The register kernel above keeps a few loads per lane in flight and waits on DRAM latency
// at every slot and at the epilogue.  Here each warp owns a ring of NST stages in shared
// memory and keeps NST slices in flight with bulk asynchronous copies (cp.async.bulk,
// completion counted in bytes on one mbarrier per stage):
//   * the slice's value stream (w slots x S rows, contiguous),
//   * the x windows it gathers from: slot k reads x[row + off_k] for the slice's S rows,
//     a contiguous window; offsets closer than kStagedGap share one window,
//   * the slice's rows of the epilogue vectors (v, w, and x for the Jacobi form).
// Every x gather and epilogue read then hits shared memory, and with the interleaved row
// layout a warp's reads for one r are 32 consecutive floats (conflict-free).  Row sums run
// over the slots in the same order as the register kernel, so both give identical bits.
// ------------------------------------------------------------------------------------
constexpr int kStagedWarps = 4;      // warps per CTA
constexpr int kStagedMaxStages = 4;
constexpr int kStagedGap = 16;       // offsets at most this far apart share one x window
constexpr int kStagedXBudget = 2048; // most x-window floats per slice that are staged
constexpr int kStagedMinWarps = 8;   // fewest resident warps per SM the staged kernel runs with
constexpr bool kStagedGlobalX = false;  // run operators with wider windows here (x through the caches)
constexpr int kStagedDesc = 68;      // ints per stage descriptor: w, flags, off[32], xb[32], x-row offset, pad
constexpr long long kStagedSpinCycles = 2000000000ll;  // ~1 s at 2 GHz: give up a wait after this
// Window templates.  An interior diagonal slice (no gather of its rows leaves [0, ncols)) stages
// x windows whose layout relative to its first row depends on its offset list alone, so slices
// with the same offsets share one template, built with the layout: int4[0] = {w, windows, floats
// staged, window offset of the slot with offset 0 (or INT_MIN)}; int4[1..9) = the slots' window
// offsets (32 ints); int4[9 + g] = {first float of window g relative to the slice's first row,
// floats, offset in the stage's window region, 0}.  The issue step then reads its copies and
// descriptors instead of grouping the offsets itself.
constexpr int kTmplInt4 = 9 + kStagedMaxWidth;

struct StagedCfg {
    long long spin;        // cycles a wait for a stage's copies may take before the kernel gives up
    int withhold;          // test only: warp 0 of CTA 0 issues no copy for its first slice (the
                           // expected bytes never arrive, so that wait runs out)
    int nst;               // stages per warp
    uint32_t warp_bytes;   // shared bytes per warp (barriers + descriptors + stages)
    uint32_t hdr_bytes;    // barriers + descriptors
    uint32_t stage_bytes;
    uint32_t o_x, o_x2, o_xr, o_v, o_w, o_a;  // byte offsets inside a stage (o_a: anchors)
    int xcap;              // floats of one window region
    int xglobal;           // x is gathered from global memory (windows too wide to stage)
    uint32_t red_off;      // byte offset of the final dots' reduction scratch (after the warps' rings)
    const int *tmpl_id;    // per slice: its window template, or -1 (see StagedTemplate)
    const int4 *tmpl;      // kTmplInt4 int4 per template
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for a stage's copies; false if they did not land within `spin` cycles
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long long spin) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > spin) return false;
    }
    return true;
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Floats of x that the staged kernel copies for slice s (offsets off[0..w) ascending): one
// window per group of offsets at most kStagedGap apart, each covering the group's clamped
// gathers rounded out to 16 bytes.  Same arithmetic as the kernel's issue step.
__device__ __forceinline__ int staged_window_floats(const int32_t *off, int w, int gmin, int gmax, int cmax) {
    int total = 0;
    for (int a = 0; a < w;) {
        int b = a;
        while (b + 1 < w && off[b + 1] - off[b] <= kStagedGap) ++b;
        const int lo = min(max(gmin + off[a], 0), cmax);
        const int hi = min(max(gmax + off[b], 0), cmax);
        total += ((hi + 4) & ~3) - (lo & ~3);
        a = b + 1;
    }
    return total;
}

__global__ void k_sell_window_max(const int4 *hdr, const int32_t *offs, const int32_t *cols, int64_t ns, int S,
                                  int64_t ncols, int *out) {
    int best = 0;
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < ns; s += int64_t(gridDim.x) * blockDim.x) {
        const int4 q = hdr[s];
        const int r0 = int(s * S);
        if (q.z >= kAnchoredTag) {
            const int w = q.z - kAnchoredTag;
            const int32_t *kp = cols + q.w + S;
            if (w > 0) best = max(best, staged_window_floats(kp, w, kp[w], kp[w + 1], int(ncols) - 1));
        } else if (q.z > 0) {
            best = max(best, staged_window_floats(offs + q.w, q.z, r0, r0 + S - 1, int(ncols) - 1));
        }
    }
    best = max(best, __reduce_max_sync(0xffffffffu, best));
    if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

template <class V>
__device__ __forceinline__ void smem_vals4(const V *p, float (&v)[4]);
template <>
__device__ __forceinline__ void smem_vals4<float>(const float *p, float (&v)[4]) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
template <>
__device__ __forceinline__ void smem_vals4<__nv_bfloat16>(const __nv_bfloat16 *p, float (&v)[4]) {
    const uint2 t = *reinterpret_cast<const uint2 *>(p);
    const float2 fa = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&t.x));
    const float2 fb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&t.y));
    v[0] = fa.x; v[1] = fa.y; v[2] = fb.x; v[3] = fb.y;
}

// a lane's four anchors in a staged slice: rows l + 32 r sit at slot positions 4 l + r
__device__ __forceinline__ void stage_anchors(const int *sa, int lane, int (&a)[4]) {
    const int4 q = *reinterpret_cast<const int4 *>(sa + 4 * lane);
    a[0] = q.x; a[1] = q.y; a[2] = q.z; a[3] = q.w;
}

template <int EPI, int XM>
struct StagedNeeds {
    static constexpr bool xr = XM == 0 && EPI == EPI_JACOBI;                // x rows (Jacobi form)
    static constexpr bool v = epi_reads_v<EPI>() || XM == 2;
    static constexpr bool w = epi_reads_w<EPI>() || XM == 2;
};

// ANCH: the operator has anchored slices (transfers); false compiles the diagonal-only kernel
template <class V, int EPI, int XM, bool ANCH>
__global__ void __launch_bounds__(kStagedWarps * 32) k_sell_staged(SellView m, EpiParams<float> e, StagedCfg cfg,
                                                                   int *kflag) {
    if ((e.done && *e.done) || (e.gate && !*e.gate)) return;
    constexpr int R = 4, S = 32 * R;
    using Nd = StagedNeeds<EPI, XM>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int nst = cfg.nst;
    unsigned char *wbase = smem + size_t(wib) * cfg.warp_bytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(wbase);
    int *desc = reinterpret_cast<int *>(wbase + 8 * kStagedMaxStages);
    unsigned char *stage0 = wbase + cfg.hdr_bytes;
    const V *vals = static_cast<const V *>(m.vals);
    const int64_t ns = m.nslices;
    const int64_t warp0 = int64_t(blockIdx.x) * kStagedWarps + wib;
    const int64_t nwarps = int64_t(gridDim.x) * kStagedWarps;
    const int cmax = int(m.ncols) - 1;
    const unsigned full = 0xffffffffu;
    double f0 = 0.0, f1 = 0.0;  // final dots (e.fa) over this thread's rows

    if (lane == 0) {
        for (int i = 0; i < nst; ++i) mbar_init(&bar[i], 1);
        mbar_fence_init();
    }
    __syncwarp();

    // per-slice metadata a lane needs to issue its copies: header and its slot's offset.
    // Headers are loaded one slice before the offsets they point to, so neither load waits
    // on the other inside an iteration.
    struct Meta {
        int64_t base;
        int w;      // slots
        int off;    // this lane's key
        int aux;
        int anch;   // anchored slice
        int amin, amax;
        int tid;    // window template (interior diagonal slices), or -1
    };
    struct Hdr {
        int4 q;
        int tid;
    };
    auto load_hdr = [&](int64_t s) -> Hdr {
        if (s >= ns) return Hdr{make_int4(0, 0, 0, 0), -1};
        return Hdr{__ldg(reinterpret_cast<const int4 *>(m.hdr) + s), cfg.tmpl_id ? __ldg(cfg.tmpl_id + s) : -1};
    };
    auto meta_of = [&](const Hdr &hq) -> Meta {
        const int4 q = hq.q;
        const int anch = ANCH && q.z >= kAnchoredTag;
        Meta mt{(int64_t(uint32_t(q.y)) << 32) | uint32_t(q.x), anch ? q.z - kAnchoredTag : q.z, 0, q.w, anch, 0, 0,
                hq.tid};
        if (mt.tid >= 0) return mt;  // the template holds the slice's copies and descriptors
        const int32_t *kp = anch ? m.cols + q.w + S : m.offs + q.w;
        if (lane < mt.w) mt.off = __ldg(kp + lane);
        if (anch) {
            mt.amin = __ldg(kp + mt.w);
            mt.amax = __ldg(kp + mt.w + 1);
        }
        return mt;
    };

    // issue the copies of slice s into stage st (whole warp, converged)
    auto issue = [&](int64_t s, int st, const Meta &mt) {
        unsigned char *sg = stage0 + size_t(st) * cfg.stage_bytes;
        int *d = desc + st * kStagedDesc;
        const int w = mt.w;
        const int r0 = int(s * S);
        const int rows = int(min(int64_t(S), m.nrows - int64_t(r0)));
        if (mt.tid >= 0) {
            // interior diagonal slice with a window template (windows staged, never x from global)
            const int4 *T = cfg.tmpl + size_t(mt.tid) * kTmplInt4;
            const int4 t0 = __ldg(T);  // {w, windows, floats, x-row offset}
            const bool xr_win = Nd::xr && t0.w != INT_MIN;
            if (lane < w) d[34 + lane] = __ldg(reinterpret_cast<const int *>(T + 1) + lane);
            if (lane == 0) {
                d[0] = w;
                d[1] = 1 | (xr_win ? 4 : 0);
                d[66] = t0.w;
            }
            const uint32_t vbytes = uint32_t(w) * S * uint32_t(sizeof(V));
            const uint32_t rbytes = uint32_t(rows) * 4u;
            uint32_t total = vbytes + uint32_t(t0.z) * 4u * (XM == 2 ? 2u : 1u);
            if (Nd::xr && !xr_win) total += rbytes;
            if (Nd::v) total += rbytes;
            if (Nd::w) total += rbytes;
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive_expect_tx(&bar[st], total);
            __syncwarp();
            if (cfg.withhold && blockIdx.x == 0 && wib == 0 && s == warp0) return;
            if (lane == 0 && vbytes) bulk_g2s(sg, vals + mt.base, vbytes, &bar[st]);
            if (lane < t0.y) {
                const int4 wd = __ldg(T + 9 + lane);  // {first float - r0, floats, window offset}
                if constexpr (XM == 2) {
                    bulk_g2s(sg + cfg.o_x + 4u * wd.z, e.w + r0 + wd.x, 4u * wd.y, &bar[st]);
                    bulk_g2s(sg + cfg.o_x2 + 4u * wd.z, e.v + r0 + wd.x, 4u * wd.y, &bar[st]);
                } else {
                    bulk_g2s(sg + cfg.o_x + 4u * wd.z, e.x + r0 + wd.x, 4u * wd.y, &bar[st]);
                }
            }
            if (Nd::xr && !xr_win && lane == 1) bulk_g2s(sg + cfg.o_xr, e.x + r0, rbytes, &bar[st]);
            if (Nd::v && lane == 2) bulk_g2s(sg + cfg.o_v, e.v + r0, rbytes, &bar[st]);
            if (Nd::w && lane == 3) bulk_g2s(sg + cfg.o_w, e.w + r0, rbytes, &bar[st]);
            return;
        }
        const int offk = mt.off;
        const int prev = __shfl_up_sync(full, offk, 1);
        const bool start = !cfg.xglobal && lane < w && (lane == 0 || offk - prev > kStagedGap);
        const unsigned gmask = __ballot_sync(full, start);
        // my group's last slot: one before the next group start, or w - 1
        const unsigned after = lane == 31 ? 0u : (gmask & ~((2u << lane) - 1u));
        const int last = after ? (__ffs(after) - 2) : (w - 1);
        const int offl = __shfl_sync(full, offk, last & 31);
        // gathers of row i at slot k: gbase(i) + key_k, gbase = the row (diagonal slice) or its
        // anchor (anchored slice), gbase in [gmin, gmax]
        const int gmin = mt.anch ? mt.amin : r0;
        const int gmax = mt.anch ? mt.amax : r0 + S - 1;
        int len = 0, lo_r = 0;
        if (start) {
            // clamped columns of the group's gathers lie in [lo, hi]; the window covers it
            // rounded out to 16 bytes (ncols is a multiple of 4, so it stays inside x)
            const int lo = min(max(gmin + offk, 0), cmax);
            const int hi = min(max(gmax + offl, 0), cmax);
            lo_r = lo & ~3;
            len = ((hi + 4) & ~3) - lo_r;
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += t;
        }
        const int woff = incl - len;  // float offset of my window in the stage's window region
        const int xtot = __shfl_sync(full, incl, 31);
        const unsigned upto = lane == 31 ? gmask : (gmask & ((2u << lane) - 1u));
        const int first = upto ? 31 - __clz(upto) : 0;
        const int xb = __shfl_sync(full, woff - lo_r, first);
        // the stage is free: every lane's reads of its previous slice are done
        // interior slice: no gather of any row leaves [0, ncols), so slot k's read for row i
        // sits at gbase(i) + (key_k + xb_k) without clamping (diagonal: (r0 + key_k + xb_k)
        // + l + 32 r for lane l, row 32 r + l)
        const int off_lo = __shfl_sync(full, offk, 0);
        const int off_hi = __shfl_sync(full, offk, (w - 1) & 31);
        const bool interior = w > 0 && gmin + off_lo >= 0 && gmax + off_hi <= cmax;
        if (lane < w) {
            d[2 + lane] = offk;
            d[34 + lane] = interior ? (mt.anch ? 0 : r0) + offk + xb : xb;
        }
        if (lane == 0) {
            d[0] = w;
            d[1] = (interior ? 1 : 0) | (mt.anch ? 2 : 0);
        }
        const uint32_t vbytes = uint32_t(w) * S * uint32_t(sizeof(V));
        const uint32_t rbytes = uint32_t(rows) * 4u;
        uint32_t total = vbytes + uint32_t(xtot) * 4u * (XM == 2 ? 2u : 1u);
        if (Nd::xr) total += rbytes;
        if (Nd::v) total += rbytes;
        if (Nd::w) total += rbytes;
        if (ANCH && mt.anch) total += S * 4u;
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive_expect_tx(&bar[st], total);
        __syncwarp();
        // test only: the first slice of warp 0 in CTA 0 gets no copy at all (nothing of that
        // stage is in flight; its wait runs out)
        if (cfg.withhold && blockIdx.x == 0 && wib == 0 && s == warp0) return;
        if (lane == 0 && vbytes) bulk_g2s(sg, vals + mt.base, vbytes, &bar[st]);
        if (start) {
            if constexpr (XM == 2) {
                bulk_g2s(sg + cfg.o_x + 4u * woff, e.w + lo_r, 4u * len, &bar[st]);
                bulk_g2s(sg + cfg.o_x2 + 4u * woff, e.v + lo_r, 4u * len, &bar[st]);
            } else {
                bulk_g2s(sg + cfg.o_x + 4u * woff, e.x + lo_r, 4u * len, &bar[st]);
            }
        }
        if (Nd::xr && lane == 1) bulk_g2s(sg + cfg.o_xr, e.x + r0, rbytes, &bar[st]);
        if (Nd::v && lane == 2) bulk_g2s(sg + cfg.o_v, e.v + r0, rbytes, &bar[st]);
        if (Nd::w && lane == 3) bulk_g2s(sg + cfg.o_w, e.w + r0, rbytes, &bar[st]);
        if (ANCH && mt.anch && lane == 4) bulk_g2s(sg + cfg.o_a, m.cols + mt.aux, S * 4u, &bar[st]);
    };

    // the product and epilogue of slice s from stage st
    auto compute = [&](int64_t s, int st) {
        const unsigned char *sg = stage0 + size_t(st) * cfg.stage_bytes;
        const int *d = desc + st * kStagedDesc;
        const int w = d[0];
        const int r0 = int(s * S);
        const V *sv = reinterpret_cast<const V *>(sg);
        const float *sx = reinterpret_cast<const float *>(sg + cfg.o_x);
        const float *sx2 = reinterpret_cast<const float *>(sg + cfg.o_x2);
        float acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = 0.f;
        const int flags = ANCH ? (d[1] & 3) : (d[1] & 1);
        const bool xr_win = Nd::xr && (d[1] & 4);  // the row's own x from the window (template slices)
        const int xr_off = d[66];
        const int *sa = reinterpret_cast<const int *>(sg + cfg.o_a);
        if (ANCH && cfg.xglobal) {
            // values (and anchors) staged, x gathered through L1 / L2
            int gb[R];
            if (flags & 2) {
                stage_anchors(sa, lane, gb);
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) gb[r] = r0 + lane + 32 * r;
            }
            const bool inner = flags & 1;
#pragma unroll 4
            for (int k = 0; k < w; ++k) {
                const int off = d[2 + k];
                float v[R];
                smem_vals4<V>(sv + k * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    int c = gb[r] + off;
                    if (!inner) c = min(max(c, 0), cmax);
                    float xv;
                    if constexpr (XM == 2) xv = __ldg(e.w + c) * __ldg(e.v + c);
                    else xv = __ldg(e.x + c);
                    acc[r] = fmaf(v[r], xv, acc[r]);
                }
            }
        } else if (ANCH && flags == 3) {
            // anchored, interior
            int a[R];
            stage_anchors(sa, lane, a);
#pragma unroll 4
            for (int k = 0; k < w; ++k) {
                const int dk = d[34 + k];
                float v[R];
                smem_vals4<V>(sv + k * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int c = a[r] + dk;
                    float xv;
                    if constexpr (XM == 2) xv = sx[c] * sx2[c];
                    else xv = sx[c];
                    acc[r] = fmaf(v[r], xv, acc[r]);
                }
            }
        } else if (flags == 1) {
            // diagonal, interior
            const float *xl = sx + lane;
#pragma unroll 4
            for (int k = 0; k < w; ++k) {
                const float *xp = xl + d[34 + k];
                float v[R];
                smem_vals4<V>(sv + k * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    float xv;
                    if constexpr (XM == 2) xv = xp[32 * r] * xp[32 * r + (sx2 - sx)];
                    else xv = xp[32 * r];
                    acc[r] = fmaf(v[r], xv, acc[r]);
                }
            }
        } else {
            // boundary slice: clamp every gather
            int gb[R];
            if (ANCH && (flags & 2)) {
                stage_anchors(sa, lane, gb);
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) gb[r] = r0 + lane + 32 * r;
            }
#pragma unroll 4
            for (int k = 0; k < w; ++k) {
                const int off = d[2 + k];
                const int xb = d[34 + k];
                float v[R];
                smem_vals4<V>(sv + k * S + lane * R, v);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int c = min(max(gb[r] + off, 0), cmax) + xb;
                    float xv;
                    if constexpr (XM == 2) xv = sx[c] * sx2[c];
                    else xv = sx[c];
                    acc[r] = fmaf(v[r], xv, acc[r]);
                }
            }
        }
        const float *sxr = reinterpret_cast<const float *>(sg + cfg.o_xr);
        const float *svv = reinterpret_cast<const float *>(sg + cfg.o_v);
        const float *sww = reinterpret_cast<const float *>(sg + cfg.o_w);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int rl = lane + 32 * r;
            const int64_t row = int64_t(r0) + rl;
            if (row < m.nrows) {
                float vr = 0.f, wr = 0.f, xr = 0.f;
                if constexpr (Nd::v) vr = svv[rl];
                if constexpr (Nd::w) wr = sww[rl];
                if constexpr (XM == 2) xr = wr * vr;
                else if constexpr (Nd::xr) xr = xr_win ? sx[rl + xr_off] : sxr[rl];
                const float out = epi_row<float, EPI>(acc[r], xr, vr, wr);
                e.y[row] = out;
                if (e.fa) final_dots_row<float>(e, row, out, f0, f1);
            }
        }
    };

    // prologue: fill the ring
    for (int i = 0; i < nst; ++i) {
        const int64_t s = warp0 + int64_t(i) * nwarps;
        if (s < ns) issue(s, i, meta_of(load_hdr(s)));
    }
    Hdr hq = load_hdr(warp0 + int64_t(nst) * nwarps);
    int it = 0, st = 0;
    uint32_t phase = 0;  // parity of the stage's current use: flips each pass around the ring
    bool ok = true;
    for (int64_t s = warp0; s < ns; s += nwarps, ++it) {
        const int64_t s_next = s + int64_t(nst) * nwarps;
        const Meta mt = meta_of(hq);  // in flight while this slice is computed
        hq = load_hdr(s_next + nwarps);
        if (!mbar_wait_bounded(&bar[st], phase, cfg.spin)) {
            ok = false;
            break;
        }
        compute(s, st);
        __syncwarp();
        if (s_next < ns) issue(s_next, st, mt);
        if (++st == nst) {
            st = 0;
            phase ^= 1u;
        }
    }
    if (!ok) {
        // record the failure and let the copies still in flight land before the CTA exits
        if (lane == 0) atomicExch(kflag, 1);
        for (int j = 0; j < nst; ++j) {
            const int64_t s = warp0 + int64_t(it + j) * nwarps;
            if (s < ns) mbar_wait_bounded(&bar[(it + j) % nst], uint32_t((it + j) / nst) & 1u, cfg.spin);
        }
    }
    if (e.fa)
        block_reduce_finish_in(f0, f1, e.fb ? 2 : 1, e.fpart, gridDim.x, e.fout, e.fcnt,
                               reinterpret_cast<double *>(smem + cfg.red_off));
}


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
    bool qpc = false;
    if constexpr (XM == 3) qpc = *e.qmode != 0;
    double dacc = 0.0, dacc2 = 0.0, f0 = 0.0, f1 = 0.0;
    unsigned long long qmn = ~0ull;
    for (int64_t wb = warp0 * RPW; wb < nrows; wb += nwarps * RPW) {
        const int64_t row = wb + lane / G;
        T acc = T(0);
        if (row < nrows) {
            const int32_t k1 = __ldg(rp + row + 1);
            for (int32_t k = __ldg(rp + row) + sub; k < k1; k += G)
                acc = fma(cvt<T>(__ldcs(cv + k)), xin_at<T, XM>(e, beta, __ldcs(ci + k), qpc), acc);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (row < nrows && sub == 0) {
            T xr = T(0);
            if constexpr (epi_reads_x<EPI, XM, DOT>()) xr = xin_at<T, XM>(e, beta, row, qpc);
            if constexpr (XM == 1) e.pout[row] = xr;
            if constexpr (XM == 3) {
                if (qpc) {
                    const unsigned long long k = qp_alpha_f_key(double(e.qx[row]), double(xr), double(e.qlb[row]),
                                                                double(e.qub[row]));
                    qmn = k < qmn ? k : qmn;
                }
            }
            T out = epilogue<T, EPI>(e, row, acc, xr);
            e.y[row] = out;
            if constexpr (epi_writes_sw<EPI>()) e.sw_out[row] = e.sw[row] * out;
            if (e.fa) final_dots_row<T>(e, row, out, f0, f1);
            if constexpr (DOT) {
                dacc = fma(double(xr), double(out), dacc);
                if (e.dv) dacc2 = fma(double(xr), double(e.dv[row]), dacc2);
            }
        }
    }
    if (e.fa) final_dots_finish<T>(e, f0, f1);
    if constexpr (XM == 3) {
        if (qpc) block_atomic_min_u64(qmn, e.qmin);
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
    e.qmode = a.qmode;
    e.xalt = static_cast<const T *>(a.xalt);
    e.qx = static_cast<const T *>(a.qx);
    e.qlb = static_cast<const T *>(a.qlb);
    e.qub = static_cast<const T *>(a.qub);
    e.qmin = a.qmin;
    e.sw_out = static_cast<T *>(a.sw_out);
    e.sw = static_cast<const T *>(a.sw);
    e.fa = a.fa;
    e.fb = a.fb;
    e.fpart = a.fpart;
    e.fout = a.fout;
    e.fcnt = a.fcnt;
    auto al = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    e.vec_ok = al(a.x) && al(a.p) && al(a.pout) && al(a.v) && al(a.w) && al(a.y) && al(a.dv) && al(a.xalt) &&
               al(a.qx) && al(a.qlb) && al(a.qub) && al(a.sw_out) && al(a.sw);
    return e;
}

int spmv_grid(const Context &ctx, int64_t units_per_cta_work, int64_t total) {
    int64_t g = (total + units_per_cta_work - 1) / units_per_cta_work;
    // up to four waves of resident CTAs: a warp's rows are a serial chain of dependent loads,
    // so few rows per warp keep more of them in flight
    int64_t cap = int64_t(ctx.sms) * 32;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return int(g);
}

template <class V, class T, int R, int EPI, int XM, bool DOT>
void sell_launch(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const Sell &s = *A.sell;
    SellView m{s.hdr.as<int4>(), s.slice_ptr.as<int64_t>(), s.slice_w.as<int32_t>(), s.slice_aux.as<int64_t>(),
               s.offs.as<int32_t>(),
               s.cols.as<int32_t>(), s.vals.ptr, s.nslices, A.nrows, A.ncols, s.interleaved ? 1 : 0};
    // one wave of resident CTAs (grid-stride over slices)
    static int per_sm = 0;
    if (per_sm == 0) {
        UGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sell_spmv<V, T, R, EPI, XM, DOT>,
                                                                kSpmvWarps * 32, 0));
        if (per_sm < 1) per_sm = 1;
    }
    int64_t want = (s.nslices + kSpmvWarps - 1) / kSpmvWarps;
    int g = int(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(ctx.sms) * per_sm)));
    if (DOT || a.fa) g = std::min(g, kSpmvDotGrid);
    k_sell_spmv<V, T, R, EPI, XM, DOT><<<g, kSpmvWarps * 32, 0, ctx.stream>>>(m, make_epi<T>(a));
}

#ifndef UGPU_SELL_STAGED
#define UGPU_SELL_STAGED 1
#endif

inline uint32_t round128(uint32_t b) { return (b + 127u) & ~127u; }

template <class V, int EPI, int XM, bool ANCH>
bool staged_launch_t(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const Sell &s = *A.sell;
    const EpiParams<float> e = make_epi<float>(a);
    if (!e.vec_ok) return false;
    using Nd = StagedNeeds<EPI, XM>;
    constexpr int S = 128;
    StagedCfg c{};
    const int wcap = std::max(1, s.max_width);
    // x windows wider than the budget (restrictions: anchors two fine points apart under nine
    // key groups) are not staged.  Gathering their x through the caches from this kernel
    // (xglobal) was measured slower than the register kernel, whose 64 warps per SM hide the
    // gather latency better, so such operators go there.
    c.xglobal = s.xwin_max > kStagedXBudget ? 1 : 0;
    if (c.xglobal && !kStagedGlobalX) return false;
    const bool tm = s.ntmpl > 0 && !c.xglobal;
    c.tmpl_id = tm ? s.tmpl_id.as<int>() : nullptr;
    c.tmpl = tm ? s.tmpl.as<int4>() : nullptr;
    c.xcap = c.xglobal ? 0 : std::max(4, s.xwin_max);
    const uint32_t vals_b = round128(uint32_t(wcap) * S * uint32_t(sizeof(V)));
    const uint32_t x_b = round128(uint32_t(c.xcap) * 4u);
    uint32_t o = vals_b;
    c.o_x = o;
    o += x_b;
    c.o_x2 = o;
    if (XM == 2) o += x_b;
    c.o_xr = o;
    if (Nd::xr) o += S * 4;
    c.o_v = o;
    if (Nd::v) o += S * 4;
    c.o_w = o;
    if (Nd::w) o += S * 4;
    c.o_a = o;
    if (s.nanch_slices) o += S * 4;
    c.stage_bytes = round128(o);
    c.hdr_bytes = round128(8u * kStagedMaxStages + 4u * kStagedDesc * kStagedMaxStages);
    auto kern = k_sell_staged<V, EPI, XM, ANCH>;
    static bool attr = false;
    if (!attr) {
        UGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr = true;
    }
    // Ring depth: the per-slice work is latency-bound instruction issue, so first as many
    // resident warps as possible up to 16 per SM, then as many bytes in flight as possible
    // (about 64 KB per SM covers the HBM latency-bandwidth product).
    int best_nst = 0, best_per_sm = 0;
    long long best_score = 0;
    // the final dots' reduction scratch, after the warps' rings (folded dots only)
    const uint32_t red_bytes = a.fa ? uint32_t(round128(sizeof(double) * kRedScratchDoubles)) : 0u;
    for (int nst = kStagedMaxStages; nst >= 2; --nst) {
        const uint32_t cta = kStagedWarps * (c.hdr_bytes + uint32_t(nst) * c.stage_bytes) + red_bytes;
        if (cta > 227u * 1024u) continue;
        int per_sm = 0;
        UGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kStagedWarps * 32, cta));
        const long long warps = per_sm * kStagedWarps;
        const long long inflight = warps * (nst - 1) * c.stage_bytes;
        const long long score = std::min(warps, 16ll) * 1000000ll + std::min(inflight, 65536ll) * 8 + warps;
        if (per_sm > 0 && score > best_score) {
            best_score = score;
            best_nst = nst;
            best_per_sm = per_sm;
        }
    }
    // a large operator with too few resident warps to hide the per-slice latency chain: the
    // register kernel (up to 64 warps per SM) does better; small operators keep the deep
    // prefetch of the ring
    if (best_nst == 0) return false;
    if (best_per_sm * kStagedWarps < kStagedMinWarps && s.nslices >= 16 * int64_t(ctx.sms)) return false;
    c.nst = best_nst;
    c.spin = ctx.staged_test_spin > 0 ? ctx.staged_test_spin : kStagedSpinCycles;
    c.withhold = ctx.staged_test_spin > 0 ? 1 : 0;
    c.warp_bytes = c.hdr_bytes + uint32_t(best_nst) * c.stage_bytes;
    c.red_off = kStagedWarps * c.warp_bytes;
    const uint32_t cta = c.red_off + red_bytes;
    SellView m{s.hdr.as<int4>(), s.slice_ptr.as<int64_t>(), s.slice_w.as<int32_t>(), s.slice_aux.as<int64_t>(),
               s.offs.as<int32_t>(), s.cols.as<int32_t>(), s.vals.ptr, s.nslices, A.nrows, A.ncols, 1};
    const int64_t want = (s.nslices + kStagedWarps - 1) / kStagedWarps;
    int g = int(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(ctx.sms) * best_per_sm)));
    if (a.fa) g = std::min(g, kSpmvDotGrid);
    kern<<<g, kStagedWarps * 32, cta, ctx.stream>>>(m, e, c, ctx.d_kflags());
    return true;
}

// Launches the staged kernel when the matrix and vectors allow it; false otherwise.  Operators
// with anchored slices (interpolations) take the anchored variant, built for the product and
// the prolongation's add form only.
template <class V, int EPI, int XM>
bool staged_launch(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const Sell &s = *A.sell;
    if (!UGPU_SELL_STAGED || !s.interleaved || s.max_width > kStagedMaxWidth || s.nslices == 0) return false;
    if (s.nanch_slices == 0) return staged_launch_t<V, EPI, XM, false>(ctx, A, a);
    if constexpr ((EPI == EPI_ADD || EPI == EPI_STORE) && XM == 0) return staged_launch_t<V, EPI, XM, true>(ctx, A, a);
    return false;
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
        if (DOT || a.fa) g = std::min(g, kSpmvDotGrid);
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
        if constexpr (std::is_same<T, float>::value && !std::is_same<V, double>::value && !DOT &&
                      (XM == 0 || XM == 2) && EPI != EPI_CHEB && EPI != EPI_CHEB0 && !epi_writes_sw<EPI>()) {
            if (staged_launch<V, EPI, XM>(ctx, A, a)) return;
        }
        // transfer-like operators (not all slices diagonal) with fewer than two slices per SM: in
        // the register kernel one lane per row would serialize each long row's gathers over too
        // few warps, so the CSR kernel (several lanes per row) runs them
        const bool few = A.sell->ndiag_slices < A.sell->nslices && A.sell->nslices < int64_t(ctx.sms) * 2;
        if (few) csr_launch<V, T, EPI, XM, DOT>(ctx, A, a);
        else sell_launch<V, T, R, EPI, XM, DOT>(ctx, A, a);
    }
}

template <class V, class T>
void dispatch_epi(Context &ctx, const Mat &A, const SpmvArgs &a) {
    const int xm = a.xmode == 3 ? 3 : (a.p ? 1 : a.xmode);  // 3: the QP input select
    const bool dot = a.dot_partials != nullptr;
    UGPU_CHECK(xm >= 0 && xm <= 3, UGPU_ERR_INTERNAL, "unknown SpMV input mode");
    if (xm == 3) {
        // box-constrained QP input: FP64 only, product stored, two dots
        UGPU_CHECK(a.epilogue == EPI_STORE && dot && a.qmode && a.qmin && a.xalt && a.qx && a.qlb && a.qub,
                   UGPU_ERR_INTERNAL, "QP input mode: EPI_STORE with dots and the QP operands");
        if constexpr (std::is_same<T, double>::value) {
            dispatch_fmt<V, T, EPI_STORE, 3, true>(ctx, A, a);
            return;
        }
        throw Error(UGPU_ERR_INTERNAL, "QP input mode needs FP64 vectors");
    }
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
        case EPI_STORE_SW:
        case EPI_SCALE_SW:
            UGPU_CHECK(xm == 0 && !dot && a.sw_out && a.sw, UGPU_ERR_INTERNAL, "sw epilogues: plain input, sw and sw_out");
            if (a.epilogue == EPI_STORE_SW) dispatch_fmt<V, T, EPI_STORE_SW, 0, false>(ctx, A, a);
            else dispatch_fmt<V, T, EPI_SCALE_SW, 0, false>(ctx, A, a);
            break;
        default: throw Error(UGPU_ERR_ARG, "unknown SpMV epilogue");
    }
#undef UGPU_EPI_CASE
}

}  // namespace

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------

// The staged kernel's window templates of an interleaved layout: every interior diagonal slice
// gets the template of its offset list (the same grouping into windows as the kernel's own issue
// step: offsets at most kStagedGap apart share a window, rounded out to 16 bytes).
void build_staged_templates(Mat &A, Sell &s, const std::vector<int32_t> &hw, const std::vector<int64_t> &aux) {
    Context &ctx = *A.ctx;
    const int64_t ns = s.nslices;
    const int S = s.S;
    std::vector<int32_t> ho(std::max<int64_t>(s.noffs, 1));
    if (s.noffs)
        UGPU_CUDA(cudaMemcpyAsync(ho.data(), s.offs.ptr, sizeof(int32_t) * s.noffs, cudaMemcpyDeviceToHost,
                                  ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    std::map<std::vector<int32_t>, int> index;
    std::vector<int4> blocks;
    std::vector<int32_t> tid(ns, -1);
    const int64_t cmax = A.ncols - 1;
    for (int64_t i = 0; i < ns; ++i) {
        const int w = hw[i];
        if (w <= 0 || w >= kAnchoredTag || w > kStagedMaxWidth) continue;
        const int32_t *o = ho.data() + aux[i];
        const int64_t r0 = i * S;
        if (r0 + o[0] < 0 || r0 + S - 1 + o[w - 1] > cmax) continue;  // a boundary slice: clamped gathers
        std::vector<int32_t> key(o, o + w);
        auto it = index.find(key);
        if (it == index.end()) {
            const int t = int(index.size());
            it = index.emplace(std::move(key), t).first;
            std::vector<int4> b(kTmplInt4, make_int4(0, 0, 0, 0));
            int *d34 = reinterpret_cast<int *>(&b[1]);
            int nwin = 0, woff = 0, xr = INT_MIN;
            for (int a = 0; a < w;) {
                int e = a;
                while (e + 1 < w && o[e + 1] - o[e] <= kStagedGap) ++e;
                const int lo_r = o[a] & ~3;               // relative to the slice's first row (a multiple of 4)
                const int len = ((S - 1 + o[e] + 4) & ~3) - lo_r;
                b[9 + nwin] = make_int4(lo_r, len, woff, 0);
                for (int k = a; k <= e; ++k) {
                    d34[k] = o[k] + woff - lo_r;
                    if (o[k] == 0) xr = d34[k];
                }
                woff += len;
                ++nwin;
                a = e + 1;
            }
            b[0] = make_int4(w, nwin, woff, xr);
            blocks.insert(blocks.end(), b.begin(), b.end());
        }
        tid[i] = it->second;
    }
    s.ntmpl = int(index.size());
    if (s.ntmpl == 0) return;
    s.tmpl.alloc(sizeof(int4) * blocks.size());
    s.tmpl_id.alloc(sizeof(int32_t) * ns);
    UGPU_CUDA(cudaMemcpyAsync(s.tmpl.ptr, blocks.data(), sizeof(int4) * blocks.size(), cudaMemcpyHostToDevice,
                              ctx.stream));
    UGPU_CUDA(cudaMemcpyAsync(s.tmpl_id.ptr, tid.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));  // the host vectors must outlive the copies
}

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
    int64_t noffs = 0, ncol = 0, ndiag = 0, nanch = 0;
    int maxw = 0;
    for (int64_t i = 0; i < ns; ++i) {
        const int w = hw[i];
        const bool anch = w >= kAnchoredTag;
        const int wd = anch ? w - kAnchoredTag : (w >= 0 ? w : -w);
        maxw = std::max(maxw, wd);
        sptr[i + 1] = sptr[i] + int64_t(wd) * S;
        if (anch) {
            aux[i] = ncol;  // anchors, keys, smallest and largest anchor; 16-byte aligned
            ncol += (int64_t(S) + wd + 2 + 3) & ~int64_t(3);
            nanch++;
        } else if (w >= 0) {
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
    s->nanch_slices = nanch;
    s->interleaved = A.vdtype != UGPU_F64 && ndiag + nanch == ns && maxw <= kStagedMaxWidth && A.nrows % 4 == 0 &&
                     A.ncols % 4 == 0;
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
                offs_tmp.as<int32_t>(), s->offs.as<int32_t>(), s->cols.as<int32_t>(), s->vals.as<V>(),
                s->interleaved);
        };
        if (A.vdtype == UGPU_F64) fill(double{});
        else if (A.vdtype == UGPU_F32) fill(float{});
        else fill(__nv_bfloat16{});
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    Buffer wmax;
    int h_wmax = 0;
    if (ns && s->interleaved) {
        wmax.alloc(sizeof(int));
        UGPU_CUDA(cudaMemsetAsync(wmax.ptr, 0, sizeof(int), ctx.stream));
        k_sell_window_max<<<gA, kAnalyzeThreads, 0, ctx.stream>>>(s->hdr.as<int4>(), s->offs.as<int32_t>(),
                                                                  s->cols.as<int32_t>(), ns, S, A.ncols,
                                                                  wmax.as<int>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaMemcpyAsync(&h_wmax, wmax.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    }
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));  // host vectors above must outlive the copies
    s->xwin_max = h_wmax;
    if (ns && s->interleaved && h_wmax <= kStagedXBudget) build_staged_templates(A, *s, hw, aux);
    s->keys = std::move(offs_tmp);  // kept: a later values-only refresh re-runs the fill alone
    A.sell = std::move(s);
}

// The values of A changed, its structure did not: the sliced-ELL values are filled again from
// the CSR values with the slice keys of the analysis (a matrix without the layout is finalised)
void refresh_values(Mat &A) {
    A.has_diag = false;
    Sell *s = A.sell.get();
    if (!s || !s->keys.ptr || A.nnz == 0) {
        finalize_matrix(A);
        return;
    }
    Context &ctx = *A.ctx;
    const int64_t ns = s->nslices;
    if (ns == 0) return;
    const int gA = int(std::min<int64_t>(ns, int64_t(ctx.sms) * 16));
    auto fill = [&](auto tag) {
        using V = decltype(tag);
        k_sell_fill<V><<<gA, kAnalyzeThreads, 0, ctx.stream>>>(
            A.rowptr.as<int32_t>(), A.colidx.as<int32_t>(), A.vals.as<V>(), A.nrows, A.ncols, s->S, ns,
            s->slice_w.as<int32_t>(), s->slice_ptr.as<int64_t>(), s->slice_aux.as<int64_t>(), s->keys.as<int32_t>(),
            s->offs.as<int32_t>(), s->cols.as<int32_t>(), s->vals.as<V>(), s->interleaved);
    };
    if (A.vdtype == UGPU_F64) fill(double{});
    else if (A.vdtype == UGPU_F32) fill(float{});
    else fill(__nv_bfloat16{});
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
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

int ugpu_test_staged_wait_timeout(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y, int64_t spin_cycles,
                                  int *launched) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(y);
    UGPU_REQUIRE(launched);
    UGPU_CHECK(spin_cycles > 0 && spin_cycles <= 100000000ll, UGPU_ERR_ARG,
               "test wait limit: 1 .. 1e8 cycles");
    Context &ctx = *A->impl.ctx;
    UGPU_CHECK(x->impl.dtype == UGPU_F32 && y->impl.dtype == UGPU_F32 && A->impl.vdtype != UGPU_F64, UGPU_ERR_ARG,
               "the staged kernel takes FP32 / BF16 operators with FP32 vectors");
    check_spmv_vec(A->impl, &x->impl, A->impl.ncols, "x");
    check_spmv_vec(A->impl, &y->impl, A->impl.nrows, "y");
    SpmvArgs a;
    a.x = x->impl.data();
    a.y = y->impl.data();
    a.vec_dtype = UGPU_F32;
    struct Reset {
        Context &c;
        ~Reset() { c.staged_test_spin = 0; }
    } reset{ctx};
    ctx.staged_test_spin = spin_cycles;
    bool staged = false;
    if (A->impl.sell && A->impl.format == UGPU_FORMAT_SELL) {
        if (A->impl.vdtype == UGPU_F32) staged = staged_launch<float, EPI_STORE, 0>(ctx, A->impl, a);
        else staged = staged_launch<__nv_bfloat16, EPI_STORE, 0>(ctx, A->impl, a);
    }
    UGPU_LAUNCH_CHECK();
    *launched = staged ? 1 : 0;
    UGPU_ABI_END(A ? A->impl.ctx : nullptr)
}

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
    refresh_values(M);
    UGPU_CUDA(cudaStreamSynchronize(c.stream));
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

int ugpu_mat_sell_layout(const ugpu_mat *A, int *interleaved, int64_t *anchored_slices) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_CHECK(A->impl.sell != nullptr, UGPU_ERR_STATE, "matrix has no sliced-ELL layout");
    if (interleaved) *interleaved = A->impl.sell->interleaved ? 1 : 0;
    if (anchored_slices) *anchored_slices = A->impl.sell->nanch_slices;
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

int ugpu_spmv_dot(const ugpu_mat *A, const ugpu_vec *x, ugpu_vec *y, ugpu_vec *dot) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(A);
    UGPU_REQUIRE(dot);
    auto &M = A->impl;
    check_spmv_vec(M, x ? &x->impl : nullptr, M.ncols, "x");
    check_spmv_vec(M, y ? &y->impl : nullptr, M.nrows, "y");
    UGPU_CHECK(M.nrows == M.ncols, UGPU_ERR_ARG, "spmv_dot: square operator");
    UGPU_CHECK(x->impl.dtype == y->impl.dtype, UGPU_ERR_ARG, "x and y dtypes differ");
    UGPU_CHECK(x->impl.buf.ptr != y->impl.buf.ptr, UGPU_ERR_ARG, "y must not alias x");
    UGPU_CHECK(dot->impl.dtype == UGPU_F64 && dot->impl.n >= 1, UGPU_ERR_ARG, "spmv_dot: an FP64 dot vector");
    UGPU_CHECK(dot->impl.buf.ptr != x->impl.buf.ptr && dot->impl.buf.ptr != y->impl.buf.ptr, UGPU_ERR_ARG,
               "spmv_dot: the dot vector must not alias x or y");
    Context &ctx = *M.ctx;
    if (M.nrows == 0) {
        UGPU_CUDA(cudaMemsetAsync(dot->impl.buf.ptr, 0, sizeof(double), ctx.stream));
    } else {
        SpmvArgs a;
        a.x = x->impl.buf.ptr;
        a.y = y->impl.buf.ptr;
        a.vec_dtype = x->impl.dtype;
        a.epilogue = EPI_STORE;
        a.dot_partials = ctx.d_partials();
        a.dot_out = dot->impl.as<double>();
        a.dot_counter = ctx.d_counters() + 8;
        launch_spmv(ctx, M, a);
    }
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
