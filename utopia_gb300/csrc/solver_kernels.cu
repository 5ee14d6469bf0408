// Elementwise kernels of the solver loops.  Each takes a device stop flag: when the
// outer iteration has already stopped (*done != 0) the kernel returns at once, so a
// captured batch of iterations can run past the converged one without changing it.
#include "device_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {

#define UGPU_GRID_LOOP(i, n) \
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

template <class T>
__global__ void k_scale_into(int64_t n, const T *w, const T *r, T *out, const int *done) {
    if (done && *done) return;
    UGPU_GRID_LOOP(i, n) out[i] = w[i] * r[i];
}

// rr = -1 * r ; p = -1 * rr   (Chebyshev3level start from a zero iterate: r = A*0 - b)
template <class T>
__global__ void k_neg_copy(int64_t n, const T *r, T *rr, T *p, const int *done) {
    if (done && *done) return;
    UGPU_GRID_LOOP(i, n) {
        T v = T(-1) * r[i];
        rr[i] = v;
        p[i] = T(-1) * v;
    }
}

template <class T>
__global__ void k_axpy(int64_t n, T a, const T *x, T *y, const int *done) {
    if (done && *done) return;
    UGPU_GRID_LOOP(i, n) y[i] = y[i] + a * x[i];
}

template <class T>
__global__ void k_setv(int64_t n, T v, T *y, const int *done) {
    if (done && *done) return;
    UGPU_GRID_LOOP(i, n) y[i] = v;
}

template <class S, class D>
__global__ void k_conv(int64_t n, const S *s, D *d, const int *done) {
    if (done && *done) return;
    UGPU_GRID_LOOP(i, n) d[i] = cvt<D>(s[i]);
}

int grid_of(const Context &c, int64_t n) { return stream_grid(c, n); }

}  // namespace

void enq_scale_into(Context &c, int dt, int64_t n, const void *w, const void *r, void *out, const int *done) {
    if (!n) return;
    if (dt == UGPU_F64)
        k_scale_into<double><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, (const double *)w, (const double *)r,
                                                                     (double *)out, done);
    else
        k_scale_into<float><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, (const float *)w, (const float *)r,
                                                                    (float *)out, done);
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

void enq_neg_copy(Context &c, int dt, int64_t n, const void *r, void *rr, void *p, const int *done) {
    if (!n) return;
    if (dt == UGPU_F64)
        k_neg_copy<double><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, (const double *)r, (double *)rr, (double *)p,
                                                                   done);
    else
        k_neg_copy<float><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, (const float *)r, (float *)rr, (float *)p, done);
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

void enq_axpy(Context &c, int dt, int64_t n, double alpha, const void *x, void *y, const int *done) {
    if (!n) return;
    if (dt == UGPU_F64)
        k_axpy<double><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, alpha, (const double *)x, (double *)y, done);
    else
        k_axpy<float><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, float(alpha), (const float *)x, (float *)y, done);
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

void enq_set(Context &c, int dt, int64_t n, double v, void *y, const int *done) {
    if (!n) return;
    if (dt == UGPU_F64)
        k_setv<double><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, v, (double *)y, done);
    else
        k_setv<float><<<grid_of(c, n), kBlock, 0, c.stream>>>(n, float(v), (float *)y, done);
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

void enq_convert(Context &c, int sdt, const void *src, int ddt, void *dst, int64_t n, const int *done) {
    if (!n) return;
    int g = grid_of(c, n);
    if (sdt == UGPU_F64 && ddt == UGPU_F32)
        k_conv<double, float><<<g, kBlock, 0, c.stream>>>(n, (const double *)src, (float *)dst, done);
    else if (sdt == UGPU_F32 && ddt == UGPU_F64)
        k_conv<float, double><<<g, kBlock, 0, c.stream>>>(n, (const float *)src, (double *)dst, done);
    else if (sdt == ddt && sdt == UGPU_F64)
        k_conv<double, double><<<g, kBlock, 0, c.stream>>>(n, (const double *)src, (double *)dst, done);
    else if (sdt == ddt && sdt == UGPU_F32)
        k_conv<float, float><<<g, kBlock, 0, c.stream>>>(n, (const float *)src, (float *)dst, done);
    else
        throw Error(UGPU_ERR_UNSUPPORTED, "convert: FP64/FP32 only");
    c.launches++;
    UGPU_LAUNCH_CHECK();
}

void enq_copy(Context &c, int dt, int64_t n, const void *src, void *dst, const int *done) {
    enq_convert(c, dt, src, dt, dst, n, done);
}

}  // namespace ugpu
