// fp64math.cuh -- FP64 exponential of a small argument and FP64 reciprocal with few FP64
// instructions, for the FP64 path kernel, which the GPU's narrow FP64 pipe bounds.
//
// exp_small: the table-driven method of P. T. P. Tang ("Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989) on
// |d| <= 1: d = k/256 + r with k = rint(256 d) and |r| <= 1/512, exp(d) = exp(k/256) p(r)
// with p the degree-5 Taylor polynomial of exp (truncation below 2^-64) and exp(k/256)
// from a 513-entry table (4 KB, cached in L1) computed on the host in extended precision
// and rounded to FP64.  Nine FP64 instructions, within a few ulp; larger arguments,
// infinities and NaN take CUDA's exp.
//
// rcp_newton: the FP32 reciprocal of s (converted in integer operations) refined by two
// Newton-Raphson steps r <- r + r (1 - s r) in FP64 (relative error 2^-23 -> 2^-46 -> one
// ulp), four FP64 instructions; for s > 0 in the normal FP32 range.
#pragma once

#include "dfloat.cuh"
#include "lmm_internal.h"

namespace lmm {

__device__ __forceinline__ double exp_small(double d, const double* __restrict__ tab)
{
    const long long ab = __double_as_longlong(d) & 0x7fffffffffffffffLL;
    if (ab > 0x3ff0000000000000LL) return exp(d);  // |d| > 1, infinities and NaN
    const double t = fma(d, (double)kExpTableHalf, 0x1.8p52);  // 1.5 2^52 + rint(256 d): the low word is rint(256 d)
    const int k = __double2loint(t);
    const double r = fma(t - 0x1.8p52, -1.0 / kExpTableHalf, d);  // d - k/256 (exact by Sterbenz's lemma)
    double p = 1.0 / 120.0;
    p = fma(p, r, 1.0 / 24.0);
    p = fma(p, r, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    return __ldg(tab + kExpTableHalf + k) * p;
}

__device__ __forceinline__ double rcp_newton(double s)
{
    double r = f32_to_f64_int(__frcp_rn(f64_to_f32_int(s)));
    double e = fma(-s, r, 1.0);
    r = fma(r, e, r);
    e = fma(-s, r, 1.0);
    return fma(r, e, r);
}

}  // namespace lmm
