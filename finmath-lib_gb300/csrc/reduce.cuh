// reduce.cuh -- deterministic compensated (double-double) reductions.
//
// The reference averages with Kahan summation in path order
// (montecarlo/RandomVariableFromDoubleArray.java:287-308).  On the GPU every partial
// sum is an unevaluated pair hi + lo built from error-free TwoSum steps, combined in a
// fixed tree (lane order, warp order, block order), so results are reproducible run to
// run and agree with the sequential Kahan sum to within one rounding.  TwoSum has no
// products, so FMA contraction cannot change it.
#pragma once

#include "dfloat.cuh"

namespace lmm {

struct dd {
    double hi, lo;
};

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ dd dd_add(dd x, dd y)
{
    double s, e;
    two_sum(x.hi, y.hi, s, e);
    e = e + (x.lo + y.lo);
    const double hi = s + e;
    return dd{hi, e - (hi - s)};
}

__device__ __forceinline__ dd dd_add_d(dd x, double y)
{
    double s, e;
    two_sum(x.hi, y, s, e);
    e = e + x.lo;
    const double hi = s + e;
    return dd{hi, e - (hi - s)};
}

__device__ __forceinline__ dd warp_dd_sum(dd v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dd o;
        o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
        o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
        v = dd_add(v, o);
    }
    return v;
}

// Block-wide sum; the full result is valid in thread 0.  All threads must call it.
__device__ __forceinline__ dd block_dd_sum(dd v)
{
    __shared__ dd warp_part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    v = warp_dd_sum(v);
    if (lane == 0) warp_part[warp] = v;
    __syncthreads();
    if (warp == 0) {
        dd w = (lane < nwarps) ? warp_part[lane] : dd{0.0, 0.0};
        w = warp_dd_sum(w);
        if (lane == 0) v = w;
    }
    __syncthreads();
    return v;
}

// Block-wide sum of one double per thread written as (hi, lo) to out[0..1] by thread 0.
__device__ __forceinline__ void block_dd_partial(double x, double* out)
{
    const dd s = block_dd_sum(dd{x, 0.0});
    if (threadIdx.x == 0) {
        out[0] = s.hi;
        out[1] = s.lo;
    }
}

// Warp sums of eight doubles per lane as a transposed reduction: three exchange levels each
// halve the values a lane holds (lanes with the level's bit set keep the upper half, the
// others the lower half, and add what the partner sends), then two plain levels -- 9 FP64
// additions per warp for the eight sums instead of 40.  Returns, in the lanes with
// (lane & 3) == 0, the sum of value index (lane >> 2) & 7; all lanes must call it.
__device__ __forceinline__ double warp_sum8_transposed(double (&v)[8], int lane)
{
    const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double keep = u16 ? v[q + 4] : v[q], send = u16 ? v[q] : v[q + 4];
        v[q] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const double keep = u8 ? v[q + 2] : v[q], send = u8 ? v[q] : v[q + 2];
        v[q] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    {
        const double keep = u4 ? v[1] : v[0], send = u4 ? v[0] : v[1];
        v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    return v[0];
}

// Block sums of NV doubles per thread, for the mixed-precision form: plain FP64 within each
// warp (lane order), compensated across the warps (warp order).  Thread i < NV writes the
// (hi, lo) pair of sum i to out + 2 (i * stride).  All threads must call it.
template <int NV>
__device__ __forceinline__ void block_sums_warp_plain(const double (&v)[NV], double* out, int stride)
{
    __shared__ double ws[32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        double x = v[i];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if (lane == 0) ws[warp][i] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        dd acc{0.0, 0.0};
        for (int w = 0; w < nwarps; w++) acc = dd_add_d(acc, ws[w][threadIdx.x]);
        out[2 * (size_t)threadIdx.x * stride] = acc.hi;
        out[2 * (size_t)threadIdx.x * stride + 1] = acc.lo;
    }
}

}  // namespace lmm
