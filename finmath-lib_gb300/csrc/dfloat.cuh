// dfloat.cuh -- FP32 sums and dot products carried in twice the working precision.
//
// Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005:
// Sum2 and Dot2 keep the running FP32 sum p and, in s, the FP32 sum of the exact rounding
// errors of every addition (Knuth's TwoSum) and every product (TwoProduct by one fused
// multiply-add).  p + s is as accurate as the sum evaluated in twice the precision and
// rounded, i.e. about 2^-48 relative per accumulated term instead of FP32's 2^-24.
// Products that feed an error-free sum use __fmul_rn, which the compiler never contracts
// into a fused multiply-add (a contraction would break the exactness these steps rely on
// in translation units built with FMA contraction on).
//
// The mixed-precision form uses these where a value needs more than FP32 accuracy but FP64
// would cost the GB300's narrow FP64 pipe (a Dot2 term is nine FP32 operations): the
// conditional expectation X beta of the backward induction and the adjoint seeds' per-date
// cash-flow sums.  The regression's Gram and X^T y sums stay FP64.  The operations
// below must not be reassociated; nvcc does not reassociate FP32 arithmetic, and the one
// product that has to be fused is an explicit fmaf.
#pragma once

namespace lmm {

struct Sum2 {
    float p;  // running sum
    float s;  // sum of the rounding errors of p
};

// x + y = a + b exactly, x = fl(a + b) (TwoSum, no ordering condition on a and b)
__device__ __forceinline__ void two_sum(float a, float b, float& x, float& y)
{
    const float s = a + b;
    const float z = s - a;
    y = (a - (s - z)) + (b - z);
    x = s;
}

// acc += x
__device__ __forceinline__ void sum2_add(Sum2& acc, float x)
{
    float p, q;
    two_sum(acc.p, x, p, q);
    acc.p = p;
    acc.s += q;
}

// acc += x * y, the product's rounding error included
__device__ __forceinline__ void dot2_add(Sum2& acc, float x, float y)
{
    const float h = __fmul_rn(x, y);
    const float r = fmaf(x, y, -h);
    float p, q;
    two_sum(acc.p, h, p, q);
    acc.p = p;
    acc.s += q + r;
}

__device__ __forceinline__ double sum2_value(const Sum2& acc) { return (double)acc.p + (double)acc.s; }

// a + b of two partial sums (the error of the leading parts kept exactly)
__device__ __forceinline__ Sum2 sum2_merge(const Sum2& a, const Sum2& b)
{
    float p, q;
    two_sum(a.p, b.p, p, q);
    return Sum2{p, (a.s + b.s) + q};
}

// a double split into two floats with hi + lo = v to about 2^-48 relative
__device__ __forceinline__ void split_double(double v, float& hi, float& lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// IEEE 754 binary64 -> binary32, round to nearest even, in integer operations: on this GPU a
// hardware conversion from FP64 issues to the narrow FP64 pipe.  Results outside the normal
// float range (zero, subnormal, overflow, infinity, NaN) take the hardware conversion.
__device__ __forceinline__ float f64_to_f32_int(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) return (float)x;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // the leading 23 fraction bits
    const unsigned rest = lo & 0x1fffffffu;                   // the 29 bits rounded away
    unsigned bits = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
    if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) bits += 1u;  // a carry moves into the exponent
    return __uint_as_float(bits);
}

// binary32 -> binary64 (exact) in integer operations; zero, subnormal, infinity and NaN
// take the hardware conversion
__device__ __forceinline__ double f32_to_f64_int(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 255u) {
        if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
        return (double)f;
    }
    const unsigned hi = (b & 0x80000000u) | ((e - 127u + 1023u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}

// ---------------------------------------------------------------- double-float sums for the FP64 path kernel
// A value carried as an unevaluated pair p + s of floats (p the running FP32 value, s the
// FP32 sum of the exact errors): Dot2 accumulation, about 2^-48 relative per accumulated term.

// p + s += (ah + al) (bh + bl), the al bl term dropped; the product's rounding error is exact
// (one fused multiply-add) and the two cross terms ride in the same error accumulator
__device__ __forceinline__ void df_dot_acc(float& p, float& s, float ah, float al, float bh, float bl)
{
    const float h = __fmul_rn(ah, bh);
    float r = fmaf(ah, bh, -h);
    r = fmaf(ah, bl, r);
    r = fmaf(al, bh, r);
    float x, q;
    two_sum(p, h, x, q);
    p = x;
    s = s + (q + r);
}

// df_dot_acc for two lanes at once on the paired FP32 pipe (the same operations, lane by
// lane): bn = -bh; subtractions as fused multiply-adds with -1, which round once like the
// subtraction itself, so every lane's result equals df_dot_acc's bit for bit
__device__ __forceinline__ void df_dot_acc2(float2& p, float2& s, float2 ah, float2 al, float2 bh, float2 bl, float2 bn)
{
    const float2 M1 = make_float2(-1.0f, -1.0f);
    const float2 hn = __fmul2_rn(ah, bn);   // -h, h = ah bh rounded
    float2 r = __ffma2_rn(ah, bh, hn);      // ah bh - h, exactly
    r = __ffma2_rn(ah, bl, r);
    r = __ffma2_rn(al, bh, r);
    const float2 x = __ffma2_rn(hn, M1, p); // p + h
    const float2 z = __ffma2_rn(p, M1, x);  // x - p
    const float2 t = __ffma2_rn(z, M1, x);  // x - z
    const float2 u = __ffma2_rn(t, M1, p);  // p - (x - z)
    const float2 v = __fadd2_rn(hn, z);     // z - h
    const float2 q = __ffma2_rn(v, M1, u);  // (p - (x - z)) + (h - z): TwoSum's error
    p = x;
    s = __fadd2_rn(s, __fadd2_rn(q, r));
}

// binary64 -> binary32 for values whose magnitude lies in FP32's normal range or below it
// (the forward rates, increments and their remainders): round to nearest even in integer
// operations only -- magnitudes below FP32's normal range become a signed zero, and nothing
// falls back to the hardware conversion, whose FP64-pipe instruction a compiler would
// otherwise execute predicated on every call.  Not for magnitudes of 2^128 and above.
__device__ __forceinline__ float f64_to_f32_small(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned bits = (hi & 0x80000000u) | ((unsigned)(e > 0 ? e : 0) << 23) | m;
    if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) bits += 1u;
    return __uint_as_float(e > 0 ? bits : (hi & 0x80000000u));
}

// a double as hi + lo floats (hi = x rounded to FP32 in integer operations, lo = the rounded
// remainder: one FP64 subtraction, which is exact), about 2^-48 relative; |x| < 2^128
__device__ __forceinline__ void df_split(double x, float& hi, float& lo)
{
    hi = f64_to_f32_small(x);
    lo = f64_to_f32_small(x - f32_to_f64_int(hi));
}

__device__ __forceinline__ double df_to_double(float hi, float lo) { return f32_to_f64_int(hi) + f32_to_f64_int(lo); }

// binary32 -> binary64 in integer operations for normal floats and zero (subnormals become
// zero; no infinity or NaN may reach it): no branch to the hardware conversion
__device__ __forceinline__ double f32_to_f64_nz(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned hi = (b & 0x80000000u) | (e ? (((e + (1023u - 127u)) << 20) | ((b & 0x7fffffu) >> 3)) : 0u);
    return __hiloint2double((int)hi, e ? (int)(b << 29) : 0);
}

// a double as hi + lo floats without an FP64 instruction: hi = x rounded to FP32 (as
// f64_to_f32_small), lo = x - hi rounded to FP32, where x - hi is the signed integer D of
// the 29 fraction bits rounded away (|D| <= 2^28) times x's last place 2^(e - 1075).  For
// |x| in FP32's normal range; lo becomes zero where x's last place is below 2^-126.
__device__ __forceinline__ void df_split_int(double x, float& hi, float& lo)
{
    const unsigned xh = (unsigned)__double2hiint(x), xl = (unsigned)__double2loint(x);
    const int ex = (int)((xh >> 20) & 0x7ffu);
    const int e = ex - 1023 + 127;
    const unsigned m = ((xh & 0xfffffu) << 3) | (xl >> 29);
    const unsigned rest = xl & 0x1fffffffu;
    const bool up = rest > 0x10000000u || (rest == 0x10000000u && (m & 1u));
    unsigned bits = (xh & 0x80000000u) | ((unsigned)(e > 0 ? e : 0) << 23) | m;
    if (up) bits += 1u;
    hi = __uint_as_float(e > 0 ? bits : (xh & 0x80000000u));
    const int D = up ? (int)rest - (1 << 29) : (int)rest;           // |x| - |hi| in last places
    const int se = ex - 1075 + 127;                                  // biased FP32 exponent of the last place
    const float ulp = __uint_as_float(se > 0 ? (unsigned)se << 23 : 0u);
    const float l = __int2float_rn(D) * ulp;                        // exact scaling by a power of two
    lo = (xh & 0x80000000u) ? -l : l;
}

}  // namespace lmm
