// exact_sum.cuh -- order-independent sums of double-double partials in integer arithmetic.
//
// The regression's cross-block sums (X^T y over the blocks of a backward-induction step) are
// taken by one block after all others have finished, so their cost is serial.  As
// double-double additions they cost about eleven FP64 instructions a value, which on a GPU
// whose FP64 rate is 1/64 of its FP32 rate kept one SM busy for ~20 us per exercise date.
// Here every value is placed instead, as a signed integer multiple of 2^(E - 1193) (E the
// largest exponent field among the values), into a 192-bit two's complement accumulator on
// the integer pipes; the lanes' accumulators are added by a shuffle tree.  The result is the
// exact sum of the inputs (parts of values more than 2^170 below the largest are dropped),
// independent of the order of the values, returned as hi + lo.
#pragma once

#include <cstdint>
#include <cstring>

#include "reduce.cuh"

namespace lmm {

// Six 32-bit limbs, least significant first, two's complement.  A double whose exponent
// field is E has its leading bit at bit 170, so up to 2^19 values stay below the sign bit.
struct Fixed192 {
    uint32_t w[6];
};

constexpr int kFixedLead = 170;  // bit of a leading 2^(E - 1023)

__host__ __device__ __forceinline__ uint64_t f64_bits(double v)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}

__host__ __device__ __forceinline__ int clz32(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return __clz((int)x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// bits [32, 64) of the 64-bit (hi:lo) shifted left by r < 32
__host__ __device__ __forceinline__ uint32_t shl_upper32(uint32_t lo, uint32_t hi, unsigned r)
{
    return r ? (hi << r) | (lo >> (32u - r)) : hi;
}

// a += x + carry (mod 2^192)
__host__ __device__ __forceinline__ void fixed_add(Fixed192& a, const uint32_t (&x)[6], uint32_t carry)
{
    uint64_t c = carry;
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const uint64_t t = (uint64_t)a.w[i] + x[i] + c;
        a.w[i] = (uint32_t)t;
        c = t >> 32;
    }
}

// exponent field of v (0x7ff: infinite or NaN)
__host__ __device__ __forceinline__ unsigned f64_exponent_field(double v) { return (unsigned)(f64_bits(v) >> 52) & 0x7ffu; }

// a += v for a finite v whose exponent field is at most emax (emax >= 1)
__host__ __device__ __forceinline__ void fixed_add_double(Fixed192& a, double v, unsigned emax)
{
    const uint64_t b = f64_bits(v);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    uint64_t M = b & 0xfffffffffffffull;  // v = M 2^(max(e,1) - 1075)
    if (e) M |= 1ull << 52;
    int s = (int)(e ? e : 1u) - (int)emax + (kFixedLead - 52);
    if (s < 0) {
        M = s > -53 ? M >> -s : 0ull;  // below the unit: dropped
        s = 0;
    }
    if (M == 0) return;
    const uint32_t lo = (uint32_t)M, hi = (uint32_t)(M >> 32);
    const unsigned r = (unsigned)s & 31u, l0 = (unsigned)s >> 5;  // l0 <= 3
    const uint32_t c0 = lo << r, c1 = shl_upper32(lo, hi, r), c2 = shl_upper32(hi, 0u, r);
    const uint32_t m = (b >> 63) ? 0xffffffffu : 0u;  // negative: add the complement plus one
    uint32_t x[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const unsigned u = (unsigned)i;
        const uint32_t c = u == l0 ? c0 : u == l0 + 1 ? c1 : u == l0 + 2 ? c2 : 0u;
        x[i] = c ^ m;
    }
    fixed_add(a, x, m & 1u);
}

__host__ __device__ __forceinline__ uint32_t fixed_limb(const Fixed192& a, int i)
{
    uint32_t r = 0u;
#pragma unroll
    for (int k = 0; k < 6; k++) r = k == i ? a.w[k] : r;
    return r;
}

// bits [pos, pos + 64) of a (zeros outside [0, 192))
__host__ __device__ __forceinline__ uint64_t fixed_bits64(const Fixed192& a, int pos)
{
    const int li = pos >= 0 ? pos / 32 : -((31 - pos) / 32);  // floor(pos / 32)
    const unsigned r = (unsigned)(pos - 32 * li);
    const uint32_t l0 = fixed_limb(a, li), l1 = fixed_limb(a, li + 1), l2 = fixed_limb(a, li + 2);
    const uint32_t o0 = r ? (l0 >> r) | (l1 << (32u - r)) : l0;
    const uint32_t o1 = r ? (l1 >> r) | (l2 << (32u - r)) : l1;
    return ((uint64_t)o1 << 32) | o0;
}

// a 2^(emax - 1193) as hi + lo, hi within half an ulp of the sum (rounded to nearest except
// when the top 64 bits sit exactly on a rounding tie), lo the rest to about 2^-116 of hi
__host__ __device__ inline dd fixed_to_dd(Fixed192 a, unsigned emax)
{
    const bool neg = (a.w[5] >> 31) != 0u;
    if (neg) {
        uint64_t c = 1;
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const uint64_t t = (uint64_t)(uint32_t)~a.w[i] + c;
            a.w[i] = (uint32_t)t;
            c = t >> 32;
        }
    }
    int top = -1;
#pragma unroll
    for (int i = 0; i < 6; i++)
        if (a.w[i]) top = i;
    if (top < 0) return dd{0.0, 0.0};
    const uint32_t wt = fixed_limb(a, top);
    const int lb = 32 * top + 31 - clz32(wt);  // leading bit
    const uint64_t T = fixed_bits64(a, lb - 63), R = fixed_bits64(a, lb - 127);
    const double hu = (double)T;  // rounded to nearest
    const uint64_t H = hu >= 18446744073709551616.0 ? 0ull : (uint64_t)hu;
    const double lu = (double)(int64_t)(T - H) + (double)R * 0x1p-64;
    const int x = lb - 63 + (int)emax - 1075 - (kFixedLead - 52);
    dd out{ldexp(hu, x), ldexp(lu, x)};
    if (neg) {
        out.hi = -out.hi;
        out.lo = -out.lo;
    }
    return out;
}

#ifdef __CUDACC__
// Sum over k < count of the pairs v[k * stride] + v[k * stride + 1] by the calling warp (all
// 32 lanes call it); the result is the same in every lane.  Inputs with an infinite or NaN
// part give the plain double-double sum, which carries them through.
__device__ inline dd warp_exact_pair_sum(const double* v, int count, int stride)
{
    const int lane = threadIdx.x & 31;
    unsigned emax = 0u;
    int bad = 0;
    for (int k = lane; k < count; k += 32) {
        const unsigned e0 = f64_exponent_field(v[(size_t)k * stride]), e1 = f64_exponent_field(v[(size_t)k * stride + 1]);
        bad |= (e0 == 0x7ffu) | (e1 == 0x7ffu);
        emax = max(emax, max(e0, e1));
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    if (__any_sync(0xffffffffu, bad)) {
        dd acc{0.0, 0.0};
        for (int k = lane; k < count; k += 32) acc = dd_add(acc, dd{v[(size_t)k * stride], v[(size_t)k * stride + 1]});
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            dd o;
            o.hi = __shfl_xor_sync(0xffffffffu, acc.hi, off);
            o.lo = __shfl_xor_sync(0xffffffffu, acc.lo, off);
            acc = dd_add(acc, o);
        }
        return acc;
    }
    if (emax == 0u) emax = 1u;  // zeros and subnormals only
    Fixed192 a{};
    for (int k = lane; k < count; k += 32) {
        fixed_add_double(a, v[(size_t)k * stride], emax);
        fixed_add_double(a, v[(size_t)k * stride + 1], emax);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        uint32_t x[6];
#pragma unroll
        for (int i = 0; i < 6; i++) x[i] = __shfl_xor_sync(0xffffffffu, a.w[i], off);
        fixed_add(a, x, 0u);
    }
    return fixed_to_dd(a, emax);
}
#endif

}  // namespace lmm
