// pd_device.cuh -- device helpers shared by the PD kernels (sm_103a).
//
// GB300 executes FP64 at about 1/64 of its FP32 rate, so per-element FP64
// arithmetic is kept out of every loop that runs per bond or per CG element.
// Dot products accumulate in "double-float" form (an unevaluated sum of two
// FP32 words, ~48-bit significand; exact products via FMA, Knuth two-sum
// additions) inside a block, and only the per-block totals are FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pd_kernels.h"

namespace pdgb {

enum : int { ACT_ACTIVE = 0, ACT_SEMI = 1, ACT_INACTIVE = 2, ACT_INVISIBLE = 3,
             ACT_CLAMPED = 4, ACT_PRESCRIBED = 5 };

__device__ __forceinline__ bool is_dirichlet(int a)
{
    return a == ACT_INVISIBLE || a == ACT_CLAMPED || a == ACT_PRESCRIBED;
}

// ---- double-float accumulation ------------------------------------------------
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_zero() { return DF{0.f, 0.f}; }

// hi+lo += a*b, with the product formed exactly (p + pe == a*b).
__device__ __forceinline__ void df_fma(DF& acc, float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float s = __fadd_rn(acc.hi, p);
    const float bb = __fsub_rn(s, acc.hi);
    const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    const float lo = __fadd_rn(__fadd_rn(acc.lo, pe), err);
    acc.hi = __fadd_rn(s, lo);
    acc.lo = __fsub_rn(lo, __fsub_rn(acc.hi, s));
}

__device__ __forceinline__ void df_add(DF& acc, DF o)
{
    const float s = __fadd_rn(acc.hi, o.hi);
    const float bb = __fsub_rn(s, acc.hi);
    const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(o.hi, bb));
    const float lo = __fadd_rn(__fadd_rn(acc.lo, o.lo), err);
    acc.hi = __fadd_rn(s, lo);
    acc.lo = __fsub_rn(lo, __fsub_rn(acc.hi, s));
}

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }

// Overloads so templated kernels accumulate FP32 data in double-float and FP64
// data directly in FP64.
struct DotAcc32 {
    DF v;
    __device__ __forceinline__ DotAcc32() : v(df_zero()) {}
    __device__ __forceinline__ void fma(float a, float b) { df_fma(v, a, b); }
    __device__ __forceinline__ double value() const { return df_to_double(v); }
};
struct DotAcc64 {
    double v;
    __device__ __forceinline__ DotAcc64() : v(0.0) {}
    __device__ __forceinline__ void fma(double a, double b) { v = __fma_rn(a, b, v); }
    __device__ __forceinline__ double value() const { return v; }
};
template <typename Real> struct DotAccFor;
template <> struct DotAccFor<float> { using type = DotAcc32; };
template <> struct DotAccFor<double> { using type = DotAcc64; };

// ---- vector types ------------------------------------------------------------
template <typename Real> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = dbl4; };

template <typename V> __device__ __forceinline__ V make_v4(double x, double y, double z);
template <> __device__ __forceinline__ float4 make_v4<float4>(double x, double y, double z)
{
    return make_float4((float)x, (float)y, (float)z, 0.f);
}
template <> __device__ __forceinline__ dbl4 make_v4<dbl4>(double x, double y, double z)
{
    return make_dbl4(x, y, z, 0.0);
}

// ---- group (sub-warp) reductions over G aligned lanes -------------------------
template <int G>
__device__ __forceinline__ unsigned group_mask()
{
    if constexpr (G >= 32) {
        return 0xffffffffu;
    } else {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned base = lane & ~(unsigned)(G - 1);
        return ((1u << G) - 1u) << base;
    }
}

template <int G, typename T>
__device__ __forceinline__ T group_sum(T v, unsigned mask)
{
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, G);
    return v;
}

template <int G>
__device__ __forceinline__ float group_minf(float v, unsigned mask)
{
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) v = fminf(v, __shfl_xor_sync(mask, v, off, G));
    return v;
}

template <int G>
__device__ __forceinline__ double group_min(double v, unsigned mask)
{
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(mask, v, off, G);
        v = o < v ? o : v;
    }
    return v;
}

// ---- block reduction with a last-block finisher -------------------------------
// Warp-level sums stay in the accumulator's own form (double-float for FP32
// data), so FP64 arithmetic happens once per warp, not once per element.
__device__ __forceinline__ double warp_total(DotAcc32 a)
{
    DF v = a.v;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        DF o;
        o.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
        o.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
        df_add(v, o);
    }
    return df_to_double(v);
}
__device__ __forceinline__ double warp_total(DotAcc64 a)
{
    double v = a.v;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Every block contributes one FP64 partial; the last block to arrive sums the
// partials in index order (deterministic for a fixed grid) and runs `fin`
// on thread 0.  Must be reached by every thread of the block.
template <typename Acc, typename Fin>
__device__ __forceinline__ void block_reduce_finish(Acc acc, ReduceSlot slot, Fin fin)
{
    __shared__ double warp_sums[kBlock / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();   // a previous reduction of this block may still read warp_sums
    const double w = warp_total(acc);
    if (lane == 0) warp_sums[warp] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += warp_sums[i];
        slot.partials[blockIdx.x] = t;
        __threadfence();
        const unsigned prev = atomicAdd(slot.counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
        t += ((volatile double*)slot.partials)[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    __syncthreads();
    if (lane == 0) warp_sums[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) total += warp_sums[i];
        *slot.counter = 0u;
        fin(total);
    }
}

// Two sums at once (block partials of the second in partials_b), the same
// fixed order as block_reduce_finish; fin(total_a, total_b) runs once.
template <typename Acc, typename Fin>
__device__ __forceinline__ void block_reduce_finish2(Acc a, Acc b, ReduceSlot slot, double* partials_b, Fin fin)
{
    __shared__ double sums_a[kBlock / 32], sums_b[kBlock / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    const double wa = warp_total(a), wb = warp_total(b);
    if (lane == 0) {
        sums_a[warp] = wa;
        sums_b[warp] = wb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            ta += sums_a[i];
            tb += sums_b[i];
        }
        slot.partials[blockIdx.x] = ta;
        partials_b[blockIdx.x] = tb;
        __threadfence();
        const unsigned prev = atomicAdd(slot.counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double ta = 0.0, tb = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        ta += ((volatile double*)slot.partials)[i];
        tb += ((volatile double*)partials_b)[i];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ta += __shfl_xor_sync(0xffffffffu, ta, off);
        tb += __shfl_xor_sync(0xffffffffu, tb, off);
    }
    __syncthreads();
    if (lane == 0) {
        sums_a[warp] = ta;
        sums_b[warp] = tb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double total_a = 0.0, total_b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            total_a += sums_a[i];
            total_b += sums_b[i];
        }
        *slot.counter = 0u;
        fin(total_a, total_b);
    }
}

}  // namespace pdgb
