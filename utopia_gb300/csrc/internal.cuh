// Internal declarations of the GB300 sparse-solver backend (libugpu).
//
// Host C++ objects (context, vectors, matrices, solvers) and the device kernels
// they launch.  Everything public goes through the C ABI in include/ugpu.h.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ugpu.h"

namespace ugpu {

// ------------------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define UGPU_CUDA(call)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            throw ::ugpu::Error(UGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define UGPU_CHECK(cond, code, msg)                     \
    do {                                                \
        if (!(cond)) throw ::ugpu::Error((code), (msg)); \
    } while (0)

#define UGPU_LAUNCH_CHECK() UGPU_CUDA(cudaGetLastError())

constexpr int kSMs = 152;          // GB300: 2 dies x 76 SMs (checked against the device at start-up)
constexpr int kBlock = 256;        // default CTA size of the streaming kernels
constexpr int kRedBlocks = 4 * kSMs;  // fixed grid of the deterministic reductions (608 CTAs)
constexpr int kMaxDots = 8;        // dots computed in one fused pass
constexpr int kSpmvDotGrid = 1024; // grid cap of SpMV kernels that also reduce a dot

// ------------------------------------------------------------------------------------
// device buffer (owned or borrowed)
// ------------------------------------------------------------------------------------
struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    bool owned = false;
    Buffer() = default;
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;
    Buffer(Buffer &&o) noexcept { steal(o); }
    Buffer &operator=(Buffer &&o) noexcept {
        if (this != &o) {
            release();
            steal(o);
        }
        return *this;
    }
    ~Buffer() { release(); }
    void steal(Buffer &o) {
        ptr = o.ptr;
        bytes = o.bytes;
        owned = o.owned;
        o.ptr = nullptr;
        o.bytes = 0;
        o.owned = false;
    }
    void alloc(size_t b) {
        release();
        if (b == 0) b = 16;
        UGPU_CUDA(cudaMalloc(&ptr, b));
        bytes = b;
        owned = true;
    }
    // keep an owned allocation of at least b bytes (alloc only when it is too small)
    void ensure(size_t b) {
        if (owned && ptr && bytes >= std::max<size_t>(b, 16)) return;
        alloc(b);
    }
    void borrow(void *p, size_t b) {
        release();
        ptr = p;
        bytes = b;
        owned = false;
    }
    void release() {
        if (owned && ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        owned = false;
    }
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

// ------------------------------------------------------------------------------------
// Context: device, stream, reduction scratch, timing
// ------------------------------------------------------------------------------------
struct Context {
    int device = 0;
    int sms = kSMs;
    cudaStream_t stream = nullptr;
    std::string last_error;
    // deterministic two-stage reductions: per-CTA partials, then one CTA sums them in order
    Buffer partials;   // kMaxDots * kRedBlocks doubles
    Buffer scalars;    // generic device scalars (results of reductions), 256 doubles
    Buffer counters;   // last-CTA tickets of the reductions
    Buffer kflags;     // int[4] device error flags; [0]: a staged SpMV gave up waiting for its copies
    long long staged_test_spin = 0;  // > 0 only inside ugpu_test_staged_wait_timeout
    double *host_scalars = nullptr;  // pinned mirror
    int64_t launches = 0;            // kernels launched through this context (instrumentation)
    Context(int dev);
    ~Context();
    double *d_partials() const { return partials.as<double>(); }
    double *d_scalars() const { return scalars.as<double>(); }
    unsigned int *d_counters() const { return counters.as<unsigned int>(); }
    int *d_kflags() const { return kflags.as<int>(); }
    void check_kernel_flags();  // throws (and clears) if a kernel recorded an error
};

// ------------------------------------------------------------------------------------
// Vectors
// ------------------------------------------------------------------------------------
inline size_t dtype_size(int dt) {
    switch (dt) {
        case UGPU_F64: return 8;
        case UGPU_F32: return 4;
        case UGPU_BF16: return 2;
        default: throw Error(UGPU_ERR_ARG, "unknown dtype");
    }
}

struct Vec {
    Context *ctx = nullptr;
    int64_t n = 0;
    int dtype = UGPU_F64;
    Buffer buf;
    void *data() const { return buf.ptr; }
    template <class T>
    T *as() const { return buf.as<T>(); }
};

// ------------------------------------------------------------------------------------
// Matrices.  CSR (int32 indices) is the interchange format; every matrix also gets
// a sliced-ELL layout used by the SpMV-family kernels:
//   * slices of S = 32*R consecutive rows (R rows per thread, R*sizeof(value) = 16 B
//     for FP64/FP32 and 8 B for BF16 so each thread issues vector loads),
//   * slot-major storage inside a slice: val[base + k*S + row_in_slice],
//   * a slice is "diagonal" when the entries of every row can be keyed by the offset
//     col - row and the slice has at most kMaxDiagSlots distinct offsets: then only
//     one int32 offset per slot is stored instead of S column indices (stencil and
//     Galerkin operators), otherwise columns are stored explicitly (transfers).
//   Within a row, slots follow ascending column order, so the per-row summation
//   order equals the CSR order.  Padding slots hold value 0 and an in-range column.
// ------------------------------------------------------------------------------------
constexpr int kMaxDiagSlots = 64;

struct Sell {
    int R = 2;          // rows per thread
    int S = 64;         // rows per slice (32*R)
    int64_t nslices = 0;
    int64_t nstored = 0;   // stored value slots (incl. padding)
    int64_t ndiag_slices = 0;
    int64_t nanch_slices = 0;  // slices keyed by col - (first column of the row)
    int max_width = 0;
    Buffer hdr;         // int4[nslices] packed {value offset lo, hi, width word, aux} read by the kernels
    Buffer slice_ptr;   // int64[nslices+1] value offset of slice (elements)
    Buffer slice_w;     // int32[nslices]   width word: w (diagonal), kAnchoredTag + w (anchored), -w (explicit)
    Buffer slice_aux;   // int64[nslices]   diagonal slices: index into offs; anchored / explicit: index into cols
    Buffer offs;        // int32 per diagonal slot
    Buffer cols;        // int32 per explicit slot entry
    Buffer vals;        // value storage (dtype of the matrix)
    int64_t ncols_explicit = 0;
    int64_t noffs = 0;
    // lane-interleaved rows: lane l owns rows l + 32 r of a slice and row 32 r + l is stored
    // at slot position l R + r (FP32 / BF16 matrices whose slices are all diagonal, read by
    // the shared-memory staged kernel); otherwise lane l owns rows l R + r at position l R + r
    bool interleaved = false;
    int xwin_max = 0;   // interleaved: most x-window floats one slice stages (staged kernel's grouping)
    Buffer tmpl_id;     // interleaved: int32[nslices] window template of an interior diagonal slice, or -1
    Buffer tmpl;        // the templates (layout in spmv.cu)
    int ntmpl = 0;
    Buffer keys;        // int32[nslices * kMaxDiagSlots] slice keys of the analysis (values-only refresh)
};

struct PtapPlan;

struct Mat {
    Context *ctx = nullptr;
    int64_t nrows = 0, ncols = 0, nnz = 0;
    int vdtype = UGPU_F64;  // value dtype
    Buffer rowptr;          // int32[nrows+1]
    Buffer colidx;          // int32[nnz]
    Buffer vals;            // vdtype[nnz]
    Buffer diag;            // FP64 diagonal (lazily built)
    bool has_diag = false;
    std::unique_ptr<Sell> sell;
    int format = UGPU_FORMAT_SELL;  // which layout the SpMV family uses
    int64_t max_row = 0;
    std::shared_ptr<PtapPlan> ptap_plan;  // set when the matrix is a Galerkin product with a kept structure
};

// sliced-ELL construction (device side), validation and set-up, spmv.cu
void build_sell(Mat &A);
void ensure_diag(Mat &A);
void validate_csr(Mat &A);
void finalize_matrix(Mat &A);
void refresh_values(Mat &A);  // values changed, structure unchanged: refill the SpMV layout
// exclusive scan of n int64 into out[0..n] (out holds n + 1 entries; out[n] = the total, returned)
int64_t device_exclusive_scan(Context &ctx, const int64_t *in, int64_t *out, int64_t n);

// ------------------------------------------------------------------------------------
// Kernels: BLAS1 and reductions (blas1.cu)
// ------------------------------------------------------------------------------------
// fused multi-dot: out_slot[k] = sum_i a_k[i]*b_k[i] for k < nd, accumulated in FP64,
// deterministic (fixed grid, fixed in-CTA order, partials summed in CTA order)
struct DotArgs {
    const void *a[kMaxDots];
    const void *b[kMaxDots];
    int dtype_a[kMaxDots];
    int dtype_b[kMaxDots];
    int nd;
};
void launch_dots(Context &ctx, int64_t n, const DotArgs &args, double *d_out);
void launch_dots_into(Context &ctx, int64_t n, const DotArgs &args, double *d_out, double *partials,
                      unsigned int *counter);
void host_dots(Context &ctx, int64_t n, const DotArgs &args, double *out);
int reduce_grid(int64_t n);
int stream_grid(const Context &ctx, int64_t n);
void launch_min2(Context &ctx, int64_t n, const double *a, const double *b, double *d_out, double *partials,
                 unsigned int *counter);
void launch_project(Context &ctx, int64_t n, const double *lb, const double *ub, double *x);
void launch_set(Context &ctx, Vec &v, double value);
void launch_convert(Context &ctx, const void *src, int sdt, void *dst, int ddt, int64_t n);
void launch_axpby(Context &ctx, int64_t n, double alpha, const Vec &x, double beta, Vec &y);
void launch_pointwise(Context &ctx, int op, const Vec &a, const Vec &b, Vec &out);
void launch_pseudo_inverse(Context &ctx, const Vec &in, Vec &out, double tol);
double launch_min_reduce(Context &ctx, int64_t n, const double *a, const double *b);

// ------------------------------------------------------------------------------------
// SpMV family (spmv.cu).  The input vector x may be formed on the fly as
// xin_j = x_j + beta * p_j (CG direction update fused into the product).
// ------------------------------------------------------------------------------------
enum SpmvEpilogue : int {
    EPI_STORE = 0,      // y = A x
    EPI_ADD = 1,        // y = A x + v
    EPI_RESIDUAL = 2,   // y = v - A x
    EPI_JACOBI = 3,     // y = x + w (v - A x)       (w: per-row weights, e.g. omega/diag)
    EPI_SUB = 4,        // y = A x - v
    EPI_SCALE = 5,      // y = w .* (A x)                     (restriction with a mask)
    EPI_PJACOBI = 6,    // y = w .* (v - A x)                 (PointJacobi sweep with LU = A - D)
    EPI_CHEB = 7,       // Chebyshev3level step: vout += s0*(A x); y = -vout + s1*x; x2 += s3*x; x2 += s2*y
    EPI_CHEB0 = 8,      // Chebyshev3level start: vout = A x - v; y = -vout
    EPI_STORE_SW = 9,   // y = A x;       sw_out = sw .* y    (restriction writing the next level's w .* b)
    EPI_SCALE_SW = 10,  // y = w .* (A x); sw_out = sw .* y   (the same with a mask)
};

struct SpmvArgs {
    const void *x = nullptr;    // input vector
    const void *v = nullptr;    // epilogue vector (v / rhs)
    const void *w = nullptr;    // per-row weights (Jacobi)
    void *y = nullptr;          // output
    void *vout = nullptr;       // in/out vector of the Chebyshev epilogues (residual)
    void *x2 = nullptr;         // in/out iterate of the Chebyshev epilogues
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int x2_zero = 0;            // Chebyshev: the iterate x2 starts at zero (not read)
    int xmode = 0;              // input vector: 0 x; 1 x + beta*p (p, pout, beta_ptr); 2 w .* v (no x)
    // fused CG direction: xin = x + beta_scale * (*beta_ptr) * p, written back to pout
    const void *p = nullptr;
    void *pout = nullptr;
    const double *beta_ptr = nullptr;
    int epilogue = EPI_STORE;
    int vec_dtype = UGPU_F64;   // dtype of x, v, w, y, p
    const void *dv = nullptr;        // if set (with dot_partials): second dot sum_i xin_i * dv_i
    double *dot_partials = nullptr;  // if set: per-CTA partial of sum_i xin_i * (A xin)_i
    double *dot_out = nullptr;       // final dot (written by the last CTA)
    unsigned int *dot_counter = nullptr;
    const int *done = nullptr;       // if set and *done != 0: the kernel does nothing
    const int *gate = nullptr;       // if set and *gate == 0: the kernel does nothing
    // xmode 3 (box-constrained QP, FP64): input xin = *qmode ? x : xalt; with *qmode the step bound
    // min over rows of (qx - qlb) / xin (xin > 0), (qx - qub) / xin (xin < 0), 1e15 is atomically
    // min-combined into *qmin as an order-preserving key (qp_key)
    const int *qmode = nullptr;
    const void *xalt = nullptr;
    const void *qx = nullptr, *qlb = nullptr, *qub = nullptr;
    unsigned long long *qmin = nullptr;
    // final dots of the product's output y with FP64 vectors: fout[0] = (y, fa), fout[1] = (y, fb)
    // (fb may be null), fixed-order two-stage reduction finished by the last CTA (fpart: per-CTA
    // partials, fcnt: its ticket); set only on Jacobi / PointJacobi sweeps (a preconditioner's
    // last kernel computing its outer Krylov iteration's dots)
    const double *fa = nullptr, *fb = nullptr;
    double *fpart = nullptr, *fout = nullptr;
    unsigned int *fcnt = nullptr;
    // EPI_STORE_SW / EPI_SCALE_SW: sw_out[row] = sw[row] * y[row] (the next level's first Jacobi
    // iterate w .* b, written by the restriction that forms b)
    void *sw_out = nullptr;
    const void *sw = nullptr;
    bool use_csr = false;
};
void launch_spmv(Context &ctx, const Mat &A, const SpmvArgs &a);

// ------------------------------------------------------------------------------------
// SpGEMM / transpose (spgemm.cu), dense coarse solve (dense.cu)
// ------------------------------------------------------------------------------------
// what a numeric-only SpGEMM of the same structure needs: per-row product bounds, the rows
// beyond the warp tiers
struct SpgemmPlan {
    Buffer ub, big, over;  // row bounds, rows beyond the warp tiers, the mid tier's overflow rows
    int h_nbig = 0, h_nover = 0;
    unsigned long long max_ub = 0;
};
// finalize = false: CSR arrays only (no SpMV layout), for intermediates that only feed products
std::unique_ptr<Mat> transpose(const Mat &A, bool finalize = true);
std::unique_ptr<Mat> spgemm(const Mat &A, const Mat &B, bool finalize = true, SpgemmPlan *plan = nullptr);
void spgemm_numeric(const Mat &A, const Mat &B, Mat &C, const SpgemmPlan &plan);
// Galerkin product P^T A P whose structure is kept for numeric-only recomputation
struct PtapPlan;
std::unique_ptr<Mat> ptap_with_plan(const Mat &A, const Mat &P, std::shared_ptr<PtapPlan> &plan);
// recompute Ac = P^T A P in place; false (nothing done) if A or P no longer have the plan's structure
bool ptap_numeric(const Mat &A, const Mat &P, Mat &Ac, PtapPlan &plan, bool finalize = true);
unsigned long long structure_digest(const Mat &A);
// T = P^T and the entry permutation (T.vals[k] = P.vals[perm[k]]) that refreshes T's values
std::unique_ptr<Mat> transpose_with_perm(const Mat &P, Buffer &perm, bool finalize = true);
void gather_values(Context &ctx, int64_t n, const double *src, const int64_t *perm, double *dst);
std::unique_ptr<Mat> ptap(const Mat &A, const Mat &P);
std::unique_ptr<Mat> cast_matrix(const Mat &A, int vdtype);
std::unique_ptr<Mat> make_csr_device(Context &ctx, int64_t nrows, int64_t ncols, int64_t nnz, int vdtype);

constexpr int64_t kDenseTriMin = 4096;  // coarse sizes above which the inverse stays factored (tri)
struct DenseCholesky {
    Context *ctx = nullptr;
    int64_t n = 0;
    Buffer L;      // n*n FP64, row-major, lower triangle
    Buffer Ainv;   // n*n FP64 explicit inverse (L^-T L^-1), applied as one GEMV per coarse solve; for n
                   // above kDenseTriMin instead Y = L^-1 in the lower triangle and Y^T in the upper one
                   // (tri), applied as two triangular GEMVs: the same FMAs per solve without the n^3
                   // product Y^T Y at set-up
    bool tri = false;
    Buffer Ainv32; // its FP32 copy for FP32 vectors (make_fp32_inverse; dropped by factor())
    Buffer tmp_d;  // FP64 rhs/solution staging
    bool factor(const Mat &A);           // returns false if not SPD
    void make_fp32_inverse();            // FP32 copy of the inverse (coarse solves with FP32 vectors)
    void solve(const void *rhs, int rdt, void *x, int xdt, const int *done = nullptr);
};

// ------------------------------------------------------------------------------------
// small helpers
// ------------------------------------------------------------------------------------
inline int grid_for(int64_t n, int block = kBlock, int per_thread = 1) {
    int64_t g = (n + int64_t(block) * per_thread - 1) / (int64_t(block) * per_thread);
    if (g < 1) g = 1;
    if (g > (1ll << 30)) g = 1 << 30;
    return int(g);
}

}  // namespace ugpu

// opaque ABI handle types are the internal objects
struct ugpu_ctx { ugpu::Context impl; explicit ugpu_ctx(int d) : impl(d) {} };
struct ugpu_vec { ugpu::Vec impl; };
struct ugpu_mat { ugpu::Mat impl; };
