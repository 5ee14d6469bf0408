// Context, vectors, BLAS-1 kernels and deterministic reductions.
#include <cmath>
#include <cstring>

#include "abi_util.cuh"
#include "device_util.cuh"

namespace ugpu {

thread_local std::string g_last_error;

Context::Context(int dev) : device(dev) {
    int count = 0;
    UGPU_CUDA(cudaGetDeviceCount(&count));
    UGPU_CHECK(dev >= 0 && dev < count, UGPU_ERR_ARG, "device index out of range");
    UGPU_CUDA(cudaSetDevice(dev));
    cudaDeviceProp prop;
    UGPU_CUDA(cudaGetDeviceProperties(&prop, dev));
    sms = prop.multiProcessorCount;
    UGPU_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    partials.alloc(sizeof(double) * kMaxDots * kRedBlocks);
    scalars.alloc(sizeof(double) * 256);
    counters.alloc(sizeof(unsigned int) * 64);
    UGPU_CUDA(cudaMemset(counters.ptr, 0, counters.bytes));
    UGPU_CUDA(cudaMemset(scalars.ptr, 0, scalars.bytes));
    kflags.alloc(sizeof(int) * 4);
    UGPU_CUDA(cudaMemset(kflags.ptr, 0, kflags.bytes));
    UGPU_CUDA(cudaMallocHost(&host_scalars, sizeof(double) * 256));
}

void Context::check_kernel_flags() {
    int h[4] = {0, 0, 0, 0};
    UGPU_CUDA(cudaMemcpyAsync(h, kflags.ptr, sizeof(h), cudaMemcpyDeviceToHost, stream));
    UGPU_CUDA(cudaStreamSynchronize(stream));
    if (h[0]) {
        UGPU_CUDA(cudaMemsetAsync(kflags.ptr, 0, kflags.bytes, stream));
        throw Error(UGPU_ERR_CUDA, "a staged SpMV kernel timed out waiting for its shared-memory copies; "
                                   "its output is invalid");
    }
}

Context::~Context() {
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    if (host_scalars) cudaFreeHost(host_scalars);
}

// ------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------
namespace {

template <class T>
__global__ void k_set(T *v, int64_t n, T val) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = val;
}

template <class S, class D>
__global__ void k_convert(const S *s, D *d, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        d[i] = cvt<D>(s[i]);
}

template <class T>
__global__ void k_axpby(int64_t n, T alpha, const T *__restrict__ x, T beta, T *__restrict__ y) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        T xi = x[i];
        y[i] = (beta == T(0)) ? alpha * xi : alpha * xi + beta * y[i];
    }
}

template <class T>
__global__ void k_pointwise(int op, int64_t n, const T *a, const T *b, T *out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        T x = a[i], y = b[i], r;
        switch (op) {
            case UGPU_EMUL: r = x * y; break;
            case UGPU_EDIV: r = x / y; break;
            case UGPU_EMIN: r = x < y ? x : y; break;
            default: r = x > y ? x : y; break;
        }
        out[i] = r;
    }
}

template <class T>
__global__ void k_pseudo_inverse(int64_t n, const T *in, T *out, T tol) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        T v = in[i];
        out[i] = (fabs(v) > tol) ? T(1) / v : T(0);
    }
}

// project(lb, ub, x): x = (l >= x) ? l : ((u <= x) ? u : x)
__global__ void k_project(int64_t n, const double *lb, const double *ub, double *x) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double l = lb ? lb[i] : -DBL_MAX_D, u = ub ? ub[i] : DBL_MAX_D, xi = x[i];
        x[i] = (l >= xi) ? l : ((u <= xi) ? u : xi);
    }
}

__device__ __forceinline__ double load_any(const void *p, int dt, int64_t i) {
    switch (dt) {
        case UGPU_F64: return static_cast<const double *>(p)[i];
        case UGPU_F32: return f2d_bits(static_cast<const float *>(p)[i]);
        default: return f2d_bits(__bfloat162float(static_cast<const __nv_bfloat16 *>(p)[i]));
    }
}

// Fused multi-dot with a deterministic two-stage reduction: every CTA reduces a fixed
// strided subset in a fixed order; the last CTA to finish sums the CTA partials in
// CTA order and writes out[k].  MODE 0: all operands FP64, 1: all FP32, 2: mixed.
template <int MODE>
__global__ void __launch_bounds__(kBlock) k_dots(int64_t n, DotArgs args, double *partials, double *out,
                                                unsigned int *counter) {
    const int nd = args.nd;
    double acc[kMaxDots];
#pragma unroll
    for (int k = 0; k < kMaxDots; ++k) acc[k] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += stride) {
#pragma unroll
        for (int k = 0; k < kMaxDots; ++k) {
            if (k < nd) {
                double a, b;
                if (MODE == 0) {
                    a = static_cast<const double *>(args.a[k])[i];
                    b = static_cast<const double *>(args.b[k])[i];
                } else if (MODE == 1) {
                    a = double(static_cast<const float *>(args.a[k])[i]);
                    b = double(static_cast<const float *>(args.b[k])[i]);
                } else {
                    a = load_any(args.a[k], args.dtype_a[k], i);
                    b = load_any(args.b[k], args.dtype_b[k], i);
                }
                acc[k] = fma(a, b, acc[k]);
            }
        }
    }
    block_reduce_store<kMaxDots>(acc, nd, partials, gridDim.x, blockIdx.x);
    finish_last_block(nd, partials, gridDim.x, out, counter);
}

__global__ void k_min2(int64_t n, const double *a, const double *b, double *partials, double *out,
                       unsigned int *counter) {
    double m = DBL_MAX_D;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double x = a[i], y = b[i];
        m = fmin(m, fmin(x, y));
    }
    m = block_reduce_min(m);
    if (threadIdx.x == 0) partials[blockIdx.x] = m;
    __threadfence();
    __shared__ bool last;
    if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (last) {
        double v = DBL_MAX_D;
        for (int j = threadIdx.x; j < gridDim.x; j += blockDim.x) v = fmin(v, __ldcg(partials + j));
        v = block_reduce_min(v);
        if (threadIdx.x == 0) {
            *out = v;
            *counter = 0;
        }
    }
}

// Reducible / Normed reductions: sums in a fixed two-stage order, min/max as a min of
// (optionally negated, absolute) values
__global__ void k_vec_reduce(int op, int64_t n, const double *v, double *partials, double *out,
                             unsigned int *counter) {
    const bool is_sum = (op == UGPU_RED_SUM || op == UGPU_RED_ASUM);
    double acc = is_sum ? 0.0 : DBL_MAX_D;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double x = v[i];
        switch (op) {
            case UGPU_RED_SUM: acc += x; break;
            case UGPU_RED_ASUM: acc += fabs(x); break;
            case UGPU_RED_MIN: acc = fmin(acc, x); break;
            case UGPU_RED_MAX: acc = fmin(acc, -x); break;
            default: acc = fmin(acc, -fabs(x)); break;
        }
    }
    if (is_sum) {
        double a[1] = {acc};
        block_reduce_store<1>(a, 1, partials, gridDim.x, blockIdx.x);
        double s[1];
        if (finish_last_block(1, partials, gridDim.x, s, counter) && threadIdx.x == 0) *out = s[0];
        return;
    }
    acc = block_reduce_min(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    __threadfence();
    __shared__ bool last;
    if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (last) {
        double m = DBL_MAX_D;
        for (int j = threadIdx.x; j < gridDim.x; j += blockDim.x) m = fmin(m, __ldcg(partials + j));
        m = block_reduce_min(m);
        if (threadIdx.x == 0) {
            *out = (op == UGPU_RED_MIN) ? m : -m;
            *counter = 0;
        }
    }
}

__global__ void k_vec_transform(int op, int64_t n, double param, double *v) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double x = v[i];
        double r;
        switch (op) {
            case UGPU_TR_SQRT: r = sqrt(x); break;
            case UGPU_TR_POW2: r = x * x; break;
            case UGPU_TR_LOG: r = log(x); break;
            case UGPU_TR_EXP: r = exp(x); break;
            case UGPU_TR_COS: r = cos(x); break;
            case UGPU_TR_SIN: r = sin(x); break;
            case UGPU_TR_ABS: r = fabs(x); break;
            case UGPU_TR_MINUS: r = -x; break;
            case UGPU_TR_POW: r = pow(x, param); break;
            case UGPU_TR_RECIPROCAL: r = param / x; break;
            case UGPU_TR_SHIFT: r = x + param; break;
            default: r = x * param; break;
        }
        v[i] = r;
    }
}

}  // namespace

int reduce_grid(int64_t n) {
    int64_t g = (n + int64_t(kBlock) * 4 - 1) / (int64_t(kBlock) * 4);
    if (g < 1) g = 1;
    if (g > kRedBlocks) g = kRedBlocks;
    return int(g);
}

int stream_grid(const Context &ctx, int64_t n) {
    int64_t g = (n + kBlock - 1) / kBlock;
    int64_t cap = int64_t(ctx.sms) * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return int(g);
}

void launch_dots_into(Context &ctx, int64_t n, const DotArgs &args, double *d_out, double *partials,
                      unsigned int *counter) {
    UGPU_CHECK(args.nd >= 1 && args.nd <= kMaxDots, UGPU_ERR_ARG, "1..8 dots per pass");
    bool all64 = true, all32 = true;
    for (int k = 0; k < args.nd; ++k) {
        all64 &= args.dtype_a[k] == UGPU_F64 && args.dtype_b[k] == UGPU_F64;
        all32 &= args.dtype_a[k] == UGPU_F32 && args.dtype_b[k] == UGPU_F32;
    }
    int g = reduce_grid(n);
    if (all64)
        k_dots<0><<<g, kBlock, 0, ctx.stream>>>(n, args, partials, d_out, counter);
    else if (all32)
        k_dots<1><<<g, kBlock, 0, ctx.stream>>>(n, args, partials, d_out, counter);
    else
        k_dots<2><<<g, kBlock, 0, ctx.stream>>>(n, args, partials, d_out, counter);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

void launch_dots(Context &ctx, int64_t n, const DotArgs &args, double *d_out) {
    launch_dots_into(ctx, n, args, d_out, ctx.d_partials(), ctx.d_counters());
}

void launch_set(Context &ctx, Vec &v, double value) {
    int g = stream_grid(ctx, v.n);
    switch (v.dtype) {
        case UGPU_F64: k_set<double><<<g, kBlock, 0, ctx.stream>>>(v.as<double>(), v.n, value); break;
        case UGPU_F32: k_set<float><<<g, kBlock, 0, ctx.stream>>>(v.as<float>(), v.n, float(value)); break;
        default:
            k_set<__nv_bfloat16><<<g, kBlock, 0, ctx.stream>>>(v.as<__nv_bfloat16>(), v.n,
                                                                __float2bfloat16(float(value)));
    }
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

template <class S>
static void convert_from(Context &ctx, const S *s, void *dst, int ddt, int64_t n, int g) {
    switch (ddt) {
        case UGPU_F64: k_convert<S, double><<<g, kBlock, 0, ctx.stream>>>(s, static_cast<double *>(dst), n); break;
        case UGPU_F32: k_convert<S, float><<<g, kBlock, 0, ctx.stream>>>(s, static_cast<float *>(dst), n); break;
        default:
            k_convert<S, __nv_bfloat16><<<g, kBlock, 0, ctx.stream>>>(s, static_cast<__nv_bfloat16 *>(dst), n);
    }
}

void launch_convert(Context &ctx, const void *src, int sdt, void *dst, int ddt, int64_t n) {
    if (n == 0) return;
    if (sdt == ddt) {
        UGPU_CUDA(cudaMemcpyAsync(dst, src, n * dtype_size(sdt), cudaMemcpyDeviceToDevice, ctx.stream));
        return;
    }
    int g = stream_grid(ctx, n);
    switch (sdt) {
        case UGPU_F64: convert_from(ctx, static_cast<const double *>(src), dst, ddt, n, g); break;
        case UGPU_F32: convert_from(ctx, static_cast<const float *>(src), dst, ddt, n, g); break;
        default: convert_from(ctx, static_cast<const __nv_bfloat16 *>(src), dst, ddt, n, g);
    }
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

void launch_axpby(Context &ctx, int64_t n, double alpha, const Vec &x, double beta, Vec &y) {
    UGPU_CHECK(x.dtype == y.dtype && x.n == y.n, UGPU_ERR_ARG, "axpby: size/dtype mismatch");
    if (n == 0) return;
    int g = stream_grid(ctx, n);
    if (x.dtype == UGPU_F64)
        k_axpby<double><<<g, kBlock, 0, ctx.stream>>>(n, alpha, x.as<double>(), beta, y.as<double>());
    else if (x.dtype == UGPU_F32)
        k_axpby<float><<<g, kBlock, 0, ctx.stream>>>(n, float(alpha), x.as<float>(), float(beta), y.as<float>());
    else
        throw Error(UGPU_ERR_UNSUPPORTED, "axpby: bf16 vectors are storage only");
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

void launch_pointwise(Context &ctx, int op, const Vec &a, const Vec &b, Vec &out) {
    UGPU_CHECK(a.dtype == b.dtype && a.dtype == out.dtype && a.n == b.n && a.n == out.n, UGPU_ERR_ARG,
               "pointwise: size/dtype mismatch");
    UGPU_CHECK(op >= 0 && op <= 3, UGPU_ERR_ARG, "pointwise: unknown op");
    if (a.n == 0) return;
    int g = stream_grid(ctx, a.n);
    if (a.dtype == UGPU_F64)
        k_pointwise<double><<<g, kBlock, 0, ctx.stream>>>(op, a.n, a.as<double>(), b.as<double>(), out.as<double>());
    else if (a.dtype == UGPU_F32)
        k_pointwise<float><<<g, kBlock, 0, ctx.stream>>>(op, a.n, a.as<float>(), b.as<float>(), out.as<float>());
    else
        throw Error(UGPU_ERR_UNSUPPORTED, "pointwise: bf16 vectors are storage only");
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

void launch_pseudo_inverse(Context &ctx, const Vec &in, Vec &out, double tol) {
    UGPU_CHECK(in.dtype == out.dtype && in.n == out.n, UGPU_ERR_ARG, "pseudo_inverse: size/dtype mismatch");
    if (in.n == 0) return;
    int g = stream_grid(ctx, in.n);
    if (in.dtype == UGPU_F64)
        k_pseudo_inverse<double><<<g, kBlock, 0, ctx.stream>>>(in.n, in.as<double>(), out.as<double>(), tol);
    else if (in.dtype == UGPU_F32)
        k_pseudo_inverse<float><<<g, kBlock, 0, ctx.stream>>>(in.n, in.as<float>(), out.as<float>(), float(tol));
    else
        throw Error(UGPU_ERR_UNSUPPORTED, "pseudo_inverse: bf16 vectors are storage only");
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

void launch_min2(Context &ctx, int64_t n, const double *a, const double *b, double *d_out, double *partials,
                 unsigned int *counter) {
    int g = reduce_grid(n);
    k_min2<<<g, kBlock, 0, ctx.stream>>>(n, a, b, partials, d_out, counter);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

double launch_min_reduce(Context &ctx, int64_t n, const double *a, const double *b) {
    if (n == 0) return DBL_MAX_D;
    launch_min2(ctx, n, a, b, ctx.d_scalars(), ctx.d_partials(), ctx.d_counters());
    UGPU_CUDA(cudaMemcpyAsync(ctx.host_scalars, ctx.d_scalars(), sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    return ctx.host_scalars[0];
}

void launch_project(Context &ctx, int64_t n, const double *lb, const double *ub, double *x) {
    if (n == 0) return;
    k_project<<<stream_grid(ctx, n), kBlock, 0, ctx.stream>>>(n, lb, ub, x);
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
}

// synchronous host-returning dots
void host_dots(Context &ctx, int64_t n, const DotArgs &args, double *out) {
    if (n == 0) {
        for (int k = 0; k < args.nd; ++k) out[k] = 0.0;
        return;
    }
    launch_dots(ctx, n, args, ctx.d_scalars());
    UGPU_CUDA(cudaMemcpyAsync(ctx.host_scalars, ctx.d_scalars(), sizeof(double) * args.nd, cudaMemcpyDeviceToHost,
                              ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    for (int k = 0; k < args.nd; ++k) out[k] = ctx.host_scalars[k];
}

}  // namespace ugpu

using namespace ugpu;

// ======================================================================================
// C ABI
// ======================================================================================
extern "C" {

int ugpu_create(int device, ugpu_ctx **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(out);
    *out = new ugpu_ctx(device);
    UGPU_ABI_END(nullptr)
}

int ugpu_destroy(ugpu_ctx *ctx) {
    UGPU_ABI_BEGIN
    delete ctx;
    UGPU_ABI_END(nullptr)
}

const char *ugpu_last_error(const ugpu_ctx *ctx) {
    if (ctx) return ctx->impl.last_error.c_str();
    return g_last_error.c_str();
}

int ugpu_synchronize(ugpu_ctx *ctx) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    ctx->impl.check_kernel_flags();
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_launch_count(const ugpu_ctx *ctx, int64_t *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    *out = ctx->impl.launches;
    UGPU_ABI_END(nullptr)
}

int ugpu_stream(const ugpu_ctx *ctx, void **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    *out = (void *)ctx->impl.stream;
    UGPU_ABI_END(nullptr)
}

int ugpu_vec_create(ugpu_ctx *ctx, int64_t n, int dtype, ugpu_vec **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_CHECK(n >= 0, UGPU_ERR_ARG, "negative size");
    auto v = std::make_unique<ugpu_vec>();
    v->impl.ctx = &ctx->impl;
    v->impl.n = n;
    v->impl.dtype = dtype;
    v->impl.buf.alloc(size_t(n) * dtype_size(dtype));
    UGPU_CUDA(cudaMemsetAsync(v->impl.buf.ptr, 0, v->impl.buf.bytes, ctx->impl.stream));
    *out = v.release();
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_vec_wrap_device(ugpu_ctx *ctx, void *device_ptr, int64_t n, int dtype, ugpu_vec **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(out);
    UGPU_CHECK(n == 0 || device_ptr, UGPU_ERR_ARG, "null device pointer");
    UGPU_CHECK(dtype >= UGPU_F64 && dtype <= UGPU_BF16, UGPU_ERR_ARG, "unknown dtype");
    UGPU_CHECK(n >= 0, UGPU_ERR_ARG, "negative length");
    auto v = std::make_unique<ugpu_vec>();
    v->impl.ctx = &ctx->impl;
    v->impl.n = n;
    v->impl.dtype = dtype;
    v->impl.buf.borrow(device_ptr, size_t(n) * dtype_size(dtype));
    *out = v.release();
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}

int ugpu_vec_destroy(ugpu_vec *v) {
    UGPU_ABI_BEGIN
    delete v;
    UGPU_ABI_END(nullptr)
}

int ugpu_vec_size(const ugpu_vec *v, int64_t *n, int *dtype) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    if (n) *n = v->impl.n;
    if (dtype) *dtype = v->impl.dtype;
    UGPU_ABI_END(nullptr)
}

int ugpu_vec_device_ptr(const ugpu_vec *v, void **out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    UGPU_REQUIRE(out);
    *out = v->impl.buf.ptr;
    UGPU_ABI_END(nullptr)
}

int ugpu_vec_upload(ugpu_vec *v, const void *host) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    UGPU_CHECK(host || v->impl.n == 0, UGPU_ERR_ARG, "null host pointer");
    auto &c = *v->impl.ctx;
    if (v->impl.n) {
        UGPU_CUDA(cudaMemcpyAsync(v->impl.buf.ptr, host, v->impl.n * dtype_size(v->impl.dtype),
                                  cudaMemcpyHostToDevice, c.stream));
        UGPU_CUDA(cudaStreamSynchronize(c.stream));
    }
    UGPU_ABI_END(v ? v->impl.ctx : nullptr)
}

int ugpu_vec_download(const ugpu_vec *v, void *host) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    UGPU_CHECK(host || v->impl.n == 0, UGPU_ERR_ARG, "null host pointer");
    auto &c = *v->impl.ctx;
    if (v->impl.n) {
        UGPU_CUDA(cudaMemcpyAsync(host, v->impl.buf.ptr, v->impl.n * dtype_size(v->impl.dtype),
                                  cudaMemcpyDeviceToHost, c.stream));
    }
    c.check_kernel_flags();
    UGPU_ABI_END(v ? v->impl.ctx : nullptr)
}

int ugpu_vec_set(ugpu_vec *v, double value) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    if (v->impl.n) launch_set(*v->impl.ctx, v->impl, value);
    UGPU_ABI_END(v ? v->impl.ctx : nullptr)
}

int ugpu_vec_copy(const ugpu_vec *x, ugpu_vec *y) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(y);
    UGPU_CHECK(x->impl.n == y->impl.n, UGPU_ERR_ARG, "copy: size mismatch");
    launch_convert(*x->impl.ctx, x->impl.buf.ptr, x->impl.dtype, y->impl.buf.ptr, y->impl.dtype, x->impl.n);
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}

int ugpu_axpby(double alpha, const ugpu_vec *x, double beta, ugpu_vec *y) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_REQUIRE(y);
    launch_axpby(*x->impl.ctx, x->impl.n, alpha, x->impl, beta, y->impl);
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}

int ugpu_dots(int k, const ugpu_vec *const *a, const ugpu_vec *const *b, double *out) {
    UGPU_ABI_BEGIN
    UGPU_CHECK(k >= 1 && k <= kMaxDots, UGPU_ERR_ARG, "dots: 1..8 pairs");
    UGPU_REQUIRE(a);
    UGPU_REQUIRE(b);
    UGPU_REQUIRE(out);
    DotArgs args{};
    args.nd = k;
    int64_t n = a[0]->impl.n;
    for (int i = 0; i < k; ++i) {
        UGPU_CHECK(a[i] && b[i], UGPU_ERR_ARG, "dots: null vector");
        UGPU_CHECK(a[i]->impl.n == n && b[i]->impl.n == n, UGPU_ERR_ARG, "dots: size mismatch");
        args.a[i] = a[i]->impl.buf.ptr;
        args.b[i] = b[i]->impl.buf.ptr;
        args.dtype_a[i] = a[i]->impl.dtype;
        args.dtype_b[i] = b[i]->impl.dtype;
    }
    host_dots(*a[0]->impl.ctx, n, args, out);
    UGPU_ABI_END((a && a[0]) ? a[0]->impl.ctx : nullptr)
}

int ugpu_dot(const ugpu_vec *a, const ugpu_vec *b, double *out) {
    const ugpu_vec *aa[1] = {a};
    const ugpu_vec *bb[1] = {b};
    return ugpu_dots(1, aa, bb, out);
}

int ugpu_norm2(const ugpu_vec *a, double *out) {
    int rc = ugpu_dot(a, a, out);
    if (rc == UGPU_OK) *out = std::sqrt(*out);
    return rc;
}

int ugpu_pointwise(int op, const ugpu_vec *a, const ugpu_vec *b, ugpu_vec *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(a);
    UGPU_REQUIRE(b);
    UGPU_REQUIRE(out);
    launch_pointwise(*a->impl.ctx, op, a->impl, b->impl, out->impl);
    UGPU_ABI_END(a ? a->impl.ctx : nullptr)
}

int ugpu_pseudo_inverse(const ugpu_vec *in, ugpu_vec *out, double tol) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(in);
    UGPU_REQUIRE(out);
    launch_pseudo_inverse(*in->impl.ctx, in->impl, out->impl, tol);
    UGPU_ABI_END(in ? in->impl.ctx : nullptr)
}

int ugpu_multi_min(const ugpu_vec *a, const ugpu_vec *b, double *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(a);
    UGPU_REQUIRE(b);
    UGPU_REQUIRE(out);
    UGPU_CHECK(a->impl.dtype == UGPU_F64 && b->impl.dtype == UGPU_F64 && a->impl.n == b->impl.n, UGPU_ERR_ARG,
               "multi_min: FP64 vectors of equal size");
    *out = launch_min_reduce(*a->impl.ctx, a->impl.n, a->impl.as<double>(), b->impl.as<double>());
    UGPU_ABI_END(a ? a->impl.ctx : nullptr)
}

int ugpu_vec_reduce(const ugpu_vec *v, int op, double *out) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    UGPU_REQUIRE(out);
    UGPU_CHECK(v->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "vec_reduce: FP64 vector");
    UGPU_CHECK(op >= UGPU_RED_SUM && op <= UGPU_RED_AMAX, UGPU_ERR_ARG, "vec_reduce: unknown op");
    Context &ctx = *v->impl.ctx;
    const int64_t n = v->impl.n;
    if (n == 0) {
        *out = 0.0;
        return UGPU_OK;
    }
    k_vec_reduce<<<reduce_grid(n), kBlock, 0, ctx.stream>>>(op, n, v->impl.as<double>(), ctx.d_partials(),
                                                            ctx.d_scalars(), ctx.d_counters());
    ctx.launches++;
    UGPU_LAUNCH_CHECK();
    UGPU_CUDA(cudaMemcpyAsync(ctx.host_scalars, ctx.d_scalars(), sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    *out = ctx.host_scalars[0];
    UGPU_ABI_END(v ? v->impl.ctx : nullptr)
}

int ugpu_vec_transform(ugpu_vec *v, int op, double param) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(v);
    UGPU_CHECK(v->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "vec_transform: FP64 vector");
    UGPU_CHECK(op >= UGPU_TR_SQRT && op <= UGPU_TR_SCALE, UGPU_ERR_ARG, "vec_transform: unknown op");
    Context &ctx = *v->impl.ctx;
    const int64_t n = v->impl.n;
    if (n) {
        k_vec_transform<<<stream_grid(ctx, n), kBlock, 0, ctx.stream>>>(op, n, param, v->impl.as<double>());
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    }
    UGPU_ABI_END(v ? v->impl.ctx : nullptr)
}

int ugpu_project(const ugpu_vec *lb, const ugpu_vec *ub, ugpu_vec *x) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(x);
    UGPU_CHECK(x->impl.dtype == UGPU_F64, UGPU_ERR_ARG, "project: FP64 vectors");
    UGPU_CHECK(!lb || (lb->impl.n == x->impl.n && lb->impl.dtype == UGPU_F64), UGPU_ERR_ARG, "project: lb");
    UGPU_CHECK(!ub || (ub->impl.n == x->impl.n && ub->impl.dtype == UGPU_F64), UGPU_ERR_ARG, "project: ub");
    launch_project(*x->impl.ctx, x->impl.n, lb ? lb->impl.as<double>() : nullptr,
                   ub ? ub->impl.as<double>() : nullptr, x->impl.as<double>());
    UGPU_ABI_END(x ? x->impl.ctx : nullptr)
}

}  // extern "C"

// ======================================================================================
// Allocation-free fused dots
//
// Some callers of this library cannot allocate device memory: host codes that have
// handed all device memory to their own allocator or memory space up front (a PETSc /
// Kokkos / PyTorch memory pool that must see no cudaMalloc or cudaFree from a library),
// and hot loops that cannot afford the device-wide synchronisation cudaFree implies.
// ugpu_dots_noalloc computes the same deterministic fused dots as ugpu_dots without a
// context and without allocating: its scratch (the per-CTA partials and the last-CTA
// ticket) is a file-scope device array of fixed size, reserved in every GPU that loads
// the library until the process exits.
// ======================================================================================
namespace {

constexpr int kNoAllocMaxPairs = kMaxDots;               // at most 8 dot pairs per call
constexpr int kNoAllocPartials = kMaxDots * kRedBlocks;  // 4864 doubles of CTA partials

// [0, kNoAllocPartials): CTA partials; the next 32 doubles hold the last-CTA ticket
// (38.9 KB in total)
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocPartials + 32];

// Device address of the scratch array in the current context.  The array's name is a
// host-side stand-in in host code, so the address comes from cudaGetSymbolAddress.  It is
// looked up on every call (cheap once the module is loaded), so a reset device or another
// context on the same device never sees a stale address.  The first call in a context
// loads the module's device globals, so it should come before any stream capture.
double *noalloc_scratch() {
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        throw Error(UGPU_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    return p;
}

}  // namespace

extern "C" int ugpu_dots_noalloc(int k, const void *const *a, const void *const *b, const int *dtype_a,
                                 const int *dtype_b, int64_t n, double *d_out, void *stream) {
    UGPU_ABI_BEGIN
    UGPU_CHECK(k >= 1, UGPU_ERR_ARG, "dots_noalloc: at least one pair");
    UGPU_CHECK(k <= kNoAllocMaxPairs, UGPU_ERR_ARG,
               "dots_noalloc: more than 8 pairs exceed the fixed scratch (8 x 608 CTA partials); split the call");
    UGPU_CHECK(n >= 0, UGPU_ERR_ARG, "dots_noalloc: negative length");
    UGPU_CHECK(a && b && dtype_a && dtype_b && d_out, UGPU_ERR_ARG, "dots_noalloc: null argument");
    DotArgs args{};
    args.nd = k;
    for (int i = 0; i < k; ++i) {
        UGPU_CHECK(n == 0 || (a[i] && b[i]), UGPU_ERR_ARG, "dots_noalloc: null vector");
        UGPU_CHECK(dtype_a[i] >= UGPU_F64 && dtype_a[i] <= UGPU_BF16 && dtype_b[i] >= UGPU_F64 &&
                       dtype_b[i] <= UGPU_BF16,
                   UGPU_ERR_ARG, "dots_noalloc: unknown dtype");
        args.a[i] = a[i];
        args.b[i] = b[i];
        args.dtype_a[i] = dtype_a[i];
        args.dtype_b[i] = dtype_b[i];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        UGPU_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * k, s));
        return UGPU_OK;
    }
    double *partials = noalloc_scratch();
    // The ticket starts at zero (the array is zero-initialised when the module loads) and
    // the last CTA of every k_dots launch puts it back to zero, so no per-call clear.
    unsigned int *ticket = reinterpret_cast<unsigned int *>(partials + kNoAllocPartials);
    bool all64 = true, all32 = true;
    for (int i = 0; i < k; ++i) {
        all64 &= args.dtype_a[i] == UGPU_F64 && args.dtype_b[i] == UGPU_F64;
        all32 &= args.dtype_a[i] == UGPU_F32 && args.dtype_b[i] == UGPU_F32;
    }
    const int g = reduce_grid(n);  // at most kRedBlocks CTAs: the partials fit the scratch
    if (all64)
        k_dots<0><<<g, kBlock, 0, s>>>(n, args, partials, d_out, ticket);
    else if (all32)
        k_dots<1><<<g, kBlock, 0, s>>>(n, args, partials, d_out, ticket);
    else
        k_dots<2><<<g, kBlock, 0, s>>>(n, args, partials, d_out, ticket);
    UGPU_CUDA(cudaGetLastError());
    UGPU_ABI_END(nullptr)
}
