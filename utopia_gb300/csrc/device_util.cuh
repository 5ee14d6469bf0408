// Device-side helpers: conversions, warp/CTA reductions, last-CTA finalisation.
#pragma once
#include <cuda_bf16.h>

#include "internal.cuh"

namespace ugpu {

#define DBL_MAX_D 1.7976931348623157e308

template <class D>
__device__ __forceinline__ D cvt(double v);
template <class D>
__device__ __forceinline__ D cvt(float v);
template <class D>
__device__ __forceinline__ D cvt(__nv_bfloat16 v);

template <>
__device__ __forceinline__ double cvt<double>(double v) { return v; }
template <>
__device__ __forceinline__ float cvt<float>(double v) { return float(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(double v) { return __float2bfloat16(float(v)); }
template <>
__device__ __forceinline__ double cvt<double>(float v) { return double(v); }
template <>
__device__ __forceinline__ float cvt<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(float v) { return __float2bfloat16(v); }
template <>
__device__ __forceinline__ double cvt<double>(__nv_bfloat16 v) { return double(__bfloat162float(v)); }
template <>
__device__ __forceinline__ float cvt<float>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(__nv_bfloat16 v) { return v; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// CTA-wide sum (any blockDim multiple of 32, <= 1024); result valid in every thread
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = (lane < nw) ? sh[lane] : 0.0;
    t = warp_sum(t);
    return t;
}

__device__ __forceinline__ double block_reduce_min(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = (lane < nw) ? sh[lane] : DBL_MAX_D;
    return warp_min(t);
}

// Reduce NK per-thread accumulators over the CTA and store partials[k*G + blk] for k < nd.
template <int NK>
__device__ __forceinline__ void block_reduce_store(const double (&acc)[NK], int nd, double *partials, int G,
                                                   int blk) {
    __shared__ double sh[NK][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        if (k < nd) {
            double v = warp_sum(acc[k]);
            if (lane == 0) sh[k][w] = v;
        }
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < NK; ++k) {
            if (k < nd) {
                double v = (lane < nw) ? sh[k][lane] : 0.0;
                v = warp_sum(v);
                if (lane == 0) partials[size_t(k) * G + blk] = v;
            }
        }
    }
}

// Last-CTA-done: the final CTA sums the G partials of each of the nd slots in a fixed
// order and writes out[k]; it also rearms the counter.  Returns true in that CTA.
__device__ __forceinline__ bool finish_last_block(int nd, const double *partials, int G, double *out,
                                                  unsigned int *counter) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last = (atomicAdd(counter, 1u) == unsigned(G) - 1u);
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    for (int k = 0; k < nd; ++k) {
        double s = 0.0;
        for (int j = threadIdx.x; j < G; j += blockDim.x) s += __ldcg(partials + size_t(k) * G + j);
        s = block_sum(s);
        if (threadIdx.x == 0) out[k] = s;
    }
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

}  // namespace ugpu
