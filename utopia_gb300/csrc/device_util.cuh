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
// Exact IEEE-754 binary32 -> binary64 and round-to-nearest-even binary64 -> binary32 by bit
// manipulation on the integer pipes, every class of input included (zeros, subnormals,
// infinities, NaNs with their payload, quietened).  On GB300 the FP64 pipe (about two operations
// per clock per SM) also executes the hardware conversions and bounds the FP64 vector kernels of
// the mixed solver; a hardware fallback for the rare classes would still be issued for every
// element once the compiler turns the branch into predicated code, so there is none.
__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint32_t m = u & 0x7fffffu;
    uint32_t de;   // the binary64 exponent field
    uint64_t dm;   // the binary64 fraction field
    if (e - 1u < 254u) {  // normal: rebias the exponent (1023 - 127), widen the fraction
        de = e + 896u;
        dm = uint64_t(m) << 29;
    } else if (e == 0xffu) {  // infinity, or NaN (payload kept, quiet bit set)
        de = 0x7ffu;
        dm = (uint64_t(m) << 29) | (m ? (1ull << 51) : 0ull);
    } else if (m == 0u) {  // signed zero
        de = 0u;
        dm = 0ull;
    } else {  // subnormal m 2^-149 = 2^(p-149) (1 + ...), p the leading one's position
        const uint32_t p = 31u - uint32_t(__clz(m));
        de = p + 874u;
        dm = (uint64_t(m) << (52u - p)) & 0xfffffffffffffull;
    }
    return __longlong_as_double((long long)((uint64_t(u & 0x80000000u) << 32) | (uint64_t(de) << 52) | dm));
}
__device__ __forceinline__ float d2f_bits(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t e = uint32_t(b >> 52) & 0x7ffu;
    const uint64_t m = b & 0xfffffffffffffull;
    uint32_t r;
    if (e - 897u < 254u) {  // the result's exponent is a normal float exponent (1..254)
        r = ((e - 896u) << 23) | uint32_t(m >> 29);  // truncated exponent and fraction
        const uint64_t rem = m & 0x1fffffffull;      // the 29 dropped bits
        const uint64_t half = 0x10000000ull;
        r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;  // a carry may raise the exponent (to inf)
    } else if (e == 0x7ffu) {  // infinity, or NaN (the payload's top bits, quiet bit set)
        r = 0x7f800000u | (m ? (0x400000u | uint32_t(m >> 29)) : 0u);
    } else if (e >= 1151u) {  // |d| >= 2^128: overflow
        r = 0x7f800000u;
    } else {  // a float subnormal or zero: k = round(M 2^(e - 926)), M the 53-bit significand
        const uint64_t M = m | (e ? (1ull << 52) : 0ull);
        const uint32_t sh = e ? 926u - e : 925u;  // at least 30
        if (sh >= 64u) {
            r = 0u;
        } else {
            const uint64_t k = M >> sh;
            const uint64_t rem = M & ((1ull << sh) - 1ull);
            const uint64_t half = 1ull << (sh - 1u);
            r = uint32_t(k) + ((rem > half || (rem == half && (k & 1ull))) ? 1u : 0u);
        }
    }
    return __uint_as_float((uint32_t(b >> 32) & 0x80000000u) | r);
}

template <>
__device__ __forceinline__ float cvt<float>(double v) { return d2f_bits(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(double v) { return __float2bfloat16(float(v)); }
template <>
__device__ __forceinline__ double cvt<double>(float v) { return f2d_bits(v); }
template <>
__device__ __forceinline__ float cvt<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(float v) { return __float2bfloat16(v); }
template <>
__device__ __forceinline__ double cvt<double>(__nv_bfloat16 v) { return f2d_bits(__bfloat162float(v)); }
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

// The two-stage reduction of block_reduce_store + finish_last_block over a caller-provided
// shared scratch of kRedScratchDoubles doubles (for kernels whose shared memory is all sized at
// launch): the CTA's nd <= 2 sums go to partials[k*G + blk]; the last CTA to finish sums the G
// partials of each slot in a fixed order into out[k] and rearms the counter.
constexpr int kRedScratchDoubles = 2 * 32 + 32 + 2;
__device__ __forceinline__ void block_reduce_finish_in(double a0, double a1, int nd, double *partials, int G,
                                                       double *out, unsigned int *counter, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    double *wsum = sh;            // [2][32]
    double *tsum = sh + 64;       // [32]
    int *last = reinterpret_cast<int *>(sh + 96);
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    if (lane == 0) {
        wsum[w] = a0;
        wsum[32 + w] = a1;
    }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < nd; ++k) {
            double v = (lane < nw) ? wsum[32 * k + lane] : 0.0;
            v = warp_sum(v);
            if (lane == 0) partials[size_t(k) * G + blockIdx.x] = v;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) *last = (atomicAdd(counter, 1u) == unsigned(G) - 1u) ? 1 : 0;
    __syncthreads();
    if (!*last) return;
    __threadfence();
    for (int k = 0; k < nd; ++k) {
        double s = 0.0;
        for (int j = threadIdx.x; j < G; j += blockDim.x) s += __ldcg(partials + size_t(k) * G + j);
        s = warp_sum(s);
        __syncthreads();
        if (lane == 0) tsum[w] = s;
        __syncthreads();
        double t = (lane < nw) ? tsum[lane] : 0.0;
        t = warp_sum(t);
        if (threadIdx.x == 0) out[k] = t;
    }
    if (threadIdx.x == 0) *counter = 0u;
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

constexpr int pow2_at_least(int k) { return k <= 1 ? 1 : 2 * pow2_at_least((k + 1) / 2); }

// Warp sums of P per-lane values (P a power of two, at most 32) with P - 1 + 5 - log2(P) FP64 adds
// per lane instead of 5 P: each of the first log2(P) butterfly steps also splits the values
// between the lane halves (a lane keeps half of what it holds and adds its partner's share of that
// half), the remaining steps add one value.  The sum of value k ends in the lanes
// [k 32/P, (k + 1) 32/P).  On GB300 FP64 adds are scarce (about two per clock per SM), and the
// reductions of kernels with few rows per thread otherwise spend a large part of them here.
template <int P>
__device__ __forceinline__ double warp_sum_split(const double (&a)[P]) {
    double v[P];
#pragma unroll
    for (int k = 0; k < P; ++k) v[k] = a[k];
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int m = P, o = 16; m > 1; m >>= 1, o >>= 1) {
        const bool upper = (lane & o) != 0;
        const int h = m / 2;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const double send = upper ? v[j] : v[h + j];
            const double keep = upper ? v[h + j] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    double s = v[0];
#pragma unroll
    for (int o = 16 / P; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Reduce NK per-thread accumulators over the CTA and store partials[k*G + blk] for k < nd.
template <int NK>
__device__ __forceinline__ void block_reduce_store(const double (&acc)[NK], int nd, double *partials, int G,
                                                   int blk) {
    constexpr int P = pow2_at_least(NK);
    __shared__ double sh[P][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    constexpr int log2P = P >= 32 ? 5 : P >= 16 ? 4 : P >= 8 ? 3 : P >= 4 ? 2 : P >= 2 ? 1 : 0;
    if (5 * nd > P - 1 + 5 - log2P) {  // the split butterfly adds less than nd separate sums
        double a[P];
#pragma unroll
        for (int k = 0; k < P; ++k) a[k] = (k < NK) ? acc[k] : 0.0;
        const double s = warp_sum_split<P>(a);
        constexpr int L = 32 / P;  // lanes per value
        if ((lane & (L - 1)) == 0) sh[lane / L][w] = s;
    } else {
#pragma unroll
        for (int k = 0; k < NK; ++k) {
            if (k < nd) {
                const double v = warp_sum(acc[k]);
                if (lane == 0) sh[k][w] = v;
            }
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

// ---- exact comparisons of doubles with integer operations ---------------------------
// GB300 retires about two FP64 operations per clock per SM, so comparisons, minima and
// selects of the box-constrained solvers run on the integer pipes instead: a double's bit
// pattern, read as a signed-magnitude integer, orders like the double itself.  Operands are not
// NaN (bounds, iterates); -0 and +0 compare equal, as in IEEE arithmetic.
// The bit pattern of |d|: the sign is cleared by an integer AND in inline assembly.  Written as
// C++ (`bits & 0x7fff...`), the compiler recognises the mask as fabs and issues an FP64
// instruction for it (measured: one DADD per use), which is what these helpers exist to avoid.
__device__ __forceinline__ long long dmag(double d) {
    long long r;
    asm("and.b64 %0, %1, 0x7FFFFFFFFFFFFFFF;" : "=l"(r) : "l"(__double_as_longlong(d)));
    return r;
}
// signed key: a < b <=> dkey(a) < dkey(b) (-0 and +0 share the key 0)
__device__ __forceinline__ long long dkey(double d) {
    const long long u = __double_as_longlong(d);
    return u < 0 ? -dmag(d) : u;
}
__device__ __forceinline__ bool dlt(double a, double b) { return dkey(a) < dkey(b); }
// |d| < t for t > 0 (false for NaN, as the FP comparison)
__device__ __forceinline__ bool dabs_lt(double d, double t) { return dmag(d) < __double_as_longlong(t); }
// std::min(0.0, g) = (g < 0) ? g : 0.0 and std::max(0.0, g) = (0 < g) ? g : 0.0
__device__ __forceinline__ double dmin0(double g) {
    const long long u = __double_as_longlong(g), m = dmag(g);
    return (u < 0 && m != 0 && m <= 0x7ff0000000000000ll) ? g : 0.0;
}
__device__ __forceinline__ double dmax0(double g) {
    const long long u = __double_as_longlong(g);
    return (u > 0 && u <= 0x7ff0000000000000ll) ? g : 0.0;
}
// order-preserving unsigned 64-bit keys of doubles (x < y <=> key(x) < key(y); -0 and +0 share
// a key), so a minimum over doubles can be combined with atomicMin on the keys
__device__ __forceinline__ unsigned long long qp_key(double d) {
    return static_cast<unsigned long long>(dkey(d)) ^ 0x8000000000000000ull;
}
__device__ __forceinline__ double qp_unkey(unsigned long long k) {
    const long long s = static_cast<long long>(k ^ 0x8000000000000000ull);
    return __longlong_as_double(s < 0 ? ((-s) | static_cast<long long>(0x8000000000000000ull)) : s);
}

}  // namespace ugpu
