// FP64 throughput of this GPU, measured: the denominator of the FP64-pipe fractions that the
// benchmark reports beside the HBM fractions.  GB300 keeps a small FP64 rate (about two fused
// multiply-adds per clock per SM), and the solver kernels on FP64 vectors run into it before
// they run into HBM, so the pipe's measured rate is what their FP64 work is compared with.
//
//   kind 0: DFMA -- independent FMA chains on every thread of a full grid
//   kind 1: DMMA -- mma.sync m8n8k4 FP64 (the FP64 tensor path), independent accumulators
//
// Both are pure register arithmetic with fixed trip counts; the result is kept live by a
// store that the host makes unreachable (sentinel).
#include "abi_util.cuh"

namespace ugpu {
namespace {

constexpr int kCalBlock = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kCalBlock) k_dfma_rate(int iters, double b, double c, double sentinel,
                                                         double *out) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = 1.0 + 1e-9 * threadIdx.x + 1e-3 * k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == sentinel) out[0] = s;
}

__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(kCalBlock) k_dmma_rate(int iters, double av, double bv, double sentinel,
                                                         double *out) {
    double d[4][2];
#pragma unroll
    for (int k = 0; k < 4; ++k) d[k][0] = d[k][1] = 1e-3 * k;
    const double a = av * (1.0 + 1e-6 * (threadIdx.x & 31)), b = bv;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) dmma_8x8x4(d[k][0], d[k][1], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) s += d[k][0] + d[k][1];
    if (s == sentinel) out[0] = s;
}

}  // namespace
}  // namespace ugpu

using namespace ugpu;

extern "C" int ugpu_fp64_rate(ugpu_ctx *ctx, int kind, double *flops_per_s) {
    UGPU_ABI_BEGIN
    UGPU_REQUIRE(ctx);
    UGPU_REQUIRE(flops_per_s);
    UGPU_CHECK(kind == 0 || kind == 1, UGPU_ERR_ARG, "fp64_rate: kind 0 (DFMA) or 1 (DMMA)");
    Context &c = ctx->impl;
    Buffer out;
    out.alloc(sizeof(double));
    const int grid = c.sms * 8;
    // about 10 ms per launch at the expected rates
    const int iters = kind == 0 ? 4096 : 1024;
    const double flops = kind == 0 ? 2.0 * kChains * double(iters) * grid * kCalBlock
                                   : 512.0 * 4.0 * double(iters) * grid * (kCalBlock / 32);
    cudaEvent_t e0, e1;
    UGPU_CUDA(cudaEventCreate(&e0));
    UGPU_CUDA(cudaEventCreate(&e1));
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        UGPU_CUDA(cudaEventRecord(e0, c.stream));
        if (kind == 0)
            k_dfma_rate<<<grid, kCalBlock, 0, c.stream>>>(iters, 0.9999999, 1e-7, -1.0, out.as<double>());
        else
            k_dmma_rate<<<grid, kCalBlock, 0, c.stream>>>(iters, 1e-3, 1e-3, -1.0, out.as<double>());
        c.launches++;
        UGPU_LAUNCH_CHECK();
        UGPU_CUDA(cudaEventRecord(e1, c.stream));
        UGPU_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        UGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms > 0.f) best = std::max(best, flops / (double(ms) * 1e-3));  // rep 0 warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *flops_per_s = best;
    UGPU_ABI_END(ctx ? &ctx->impl : nullptr)
}
