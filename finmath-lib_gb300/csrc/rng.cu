// rng.cu -- K1: partitioned MT19937 + Wichura inverse normal (Brownian increments).
//
// Reference: BrownianMotionFromMersenneRandomNumbers.doGenerateBrownianMotion
// (montecarlo/BrownianMotionFromMersenneRandomNumbers.java:141-191) draws, from one
// MersenneTwister stream, u = nextDouble() for path -> time -> factor and stores
// dW[t][f][p] = NormalDistribution.inverseCumulativeDistribution(u) * sqrt(dt_t).
//
// GB300 design: the stream of V values (2 words each) is cut into one contiguous chunk
// per resident generator CTA.  mt_jump_kernel moves the seeded state to each chunk start
// with GF(2) jump polynomials (one per nonzero base-8 digit of the chunk index, at most
// three for 512 chunks; each jump is an XOR of windows of the raw word sequence held in
// shared memory) and writes the start states to HBM.  mt_generate_kernel (three CTAs per
// SM) then regenerates 624 words at a time in three dependency phases (227/227/170 words)
// over a double-buffered state and converts word pairs to values.  Uniforms are
// bit-identical to the single stream.  The increments leave through a shared-memory tile
// (increments_loop) so that each [t][f] row is written in 64-byte segments although the
// stream runs path-major.
//
// This translation unit is compiled with -fmad=false (the error-free transforms below rely
// on every add and multiply rounding separately).  The FP64 inverse normal evaluates the
// reference's rational functions in double-float arithmetic on the FP32 pipe (within 5e-14
// relative of the reference's normals; the uniforms stay bit-exact).
#include "fp64math.cuh"
#include "lmm_internal.h"

#include <cmath>
#include <cstring>

namespace lmm {
namespace {

constexpr int kRngThreads = 320;   // the chunk-jump kernel
// The generator: ten draw warps (one draw per thread of a 312-draw round) and two tail warps,
// which evaluate the tail draws of the rounds before while the draw warps evaluate the
// central draws of the current one.
constexpr int kDrawThreads = 320;
constexpr int kTailWarpThreads = 64;
constexpr int kGenThreads = kDrawThreads + kTailWarpThreads;
constexpr int kTailQueue = 512;    // ring buffer of pending tail draws (a power of two)

struct RngParams {
    int64_t central_max;      // |m - 2^51| <= central_max  <=>  |u - 0.5| <= 0.425 for u = m 2^-52
    uint32_t magic_tf;        // floor((2^32-1)/TF): division by the values per path
    uint32_t magic_f;         // floor((2^32-1)/F)
    const uint32_t* seeded;   // [624]
    const uint16_t* jump_bits;  // set-bit positions of the jump polynomials (see RngPlan)
    int bit_off[kMaxJumps], bit_cnt[kMaxJumps];  // list j * 7 + d - 1: digit j has the value d
    int ndigits;
    int64_t num_values;
    int64_t chunk_values;
    int values_per_path;
    int num_paths;
    int num_factors;
    int mode;
    int tile_k;               // paths per increments tile (a power of two <= 32)
    const double* sqrt_dt;    // mode 1
    const float* sqrt_dt32;   // mode 2
    void* out;
};

// x / d and x % d for a block-uniform divisor d < 2^31 and x < 2^31, with M = floor((2^32-1)/d):
// __umulhi(x, M) is the quotient or one less.
__device__ __forceinline__ void divmod_u32(uint32_t x, uint32_t d, uint32_t M, uint32_t& q, uint32_t& r)
{
    q = __umulhi(x, M);
    r = x - q * d;
    if (r >= d) {
        q++;
        r -= d;
    }
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y)
{
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

// x[n] = x[n-227] ^ twist(upper(x[n-624]) | lower(x[n-623]))
__device__ __forceinline__ uint32_t mt_next(uint32_t x_m, uint32_t x_0, uint32_t x_1)
{
    const uint32_t y = (x_0 & 0x80000000u) | (x_1 & 0x7fffffffu);
    return x_m ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// NormalDistribution.inverseCumulativeNormalDistributionWichura (functions/NormalDistribution.java:67-162),
// AS241 (Wichura 1988): the reference's coefficients and branches.  The central branch
// (|p - 0.5| <= 0.425, ~85 % of draws) and the tails are separate functions so that the
// generator runs each on a compacted set of lanes.
//
// The FP64 form evaluates the rational functions in double-float arithmetic on the FP32
// pipe (on this GPU FP64 issues at 1/64 of the FP32 rate, and the FP64 Horner steps were
// most of the generator's time): the argument r is formed in FP64 and split into a pair
// of floats hi + lo, each Horner step v <- v r + c runs on float pairs (the product's
// rounding error by fused multiply-adds, the sum by TwoSum, a renormalisation), and the
// quotient is the rounded FP32 quotient plus the residual's quotient.  Every term of the
// polynomials is positive on its branch (no cancellation), so the pair carries about
// 2^-47 relative per step: the normals stay within 5e-14 relative of the reference's FP64
// evaluation, four FP64 instructions per central draw instead of 24.  The tails take
// their logarithm and square root on float pairs as well (restated from the mathematics
// below; CUDA's FP64 log and sqrt were most of the tail's FP64 instructions).

// a coefficient c as hi + lo floats: hi = c rounded to FP32, lo = the rounded remainder
struct DfCoef {
    float h, l;
};
__host__ __device__ constexpr DfCoef dfc(double c) { return DfCoef{(float)c, (float)(c - (double)(float)c)}; }

// Numerator (lane x) and denominator (lane y) polynomials c[0] r^7 + ... + c[7] for
// r = rh + rl, by Horner steps on float pairs, both at once on the paired FP32 pipe: each
// step forms -p = -(v_h r_h) and the product's exact error v_h r_h - p by fused multiply-
// adds (plus the cross terms v_h r_l, v_l r_h), adds the coefficient by TwoSum
// (subtractions as fused multiply-adds with -1, which round once like a subtraction) and
// renormalises the pair.
__device__ __forceinline__ void df_horner8x2(float rh, float rl, const DfCoef (&a)[8], const DfCoef (&b)[8],
                                             float2& vh, float2& vl)
{
    const float2 R = make_float2(rh, rh), Rn = make_float2(-rh, -rh), Rl = make_float2(rl, rl);
    const float2 M1 = make_float2(-1.0f, -1.0f);
    vh = make_float2(a[0].h, b[0].h);
    vl = make_float2(a[0].l, b[0].l);
#pragma unroll
    for (int i = 1; i < 8; i++) {
        const float2 C = make_float2(a[i].h, b[i].h), CL = make_float2(a[i].l, b[i].l);
        const float2 pn = __fmul2_rn(vh, Rn);      // -p, p = v_h r_h rounded
        float2 e = __ffma2_rn(vh, R, pn);          // v_h r_h - p, exactly
        e = __ffma2_rn(vh, Rl, e);
        e = __ffma2_rn(vl, R, e);
        const float2 s = __ffma2_rn(pn, M1, C);    // C + p
        const float2 z = __ffma2_rn(C, M1, s);     // s - C
        const float2 u = __ffma2_rn(z, M1, s);     // s - z
        const float2 v = __ffma2_rn(u, M1, C);     // C - u
        const float2 w = __fadd2_rn(pn, z);        // -(p - z)
        const float2 err = __ffma2_rn(w, M1, v);   // (C - (s - z)) + (p - z): the TwoSum error
        const float2 t = __fadd2_rn(__fadd2_rn(e, CL), err);
        vh = __fadd2_rn(s, t);
        vl = __ffma2_rn(__ffma2_rn(s, M1, vh), M1, t);  // t - (vh - s)
    }
}

// a double as hi + lo floats (hi rounded in integer operations, lo the rounded remainder of
// one exact FP64 subtraction)
__device__ __forceinline__ void df_split_nz(double x, float& hi, float& lo)
{
    hi = f64_to_f32_small(x);
    lo = f64_to_f32_small(x - f32_to_f64_nz(hi));
}

// (nh + nl) / (dh + dl) for positive pairs: the rounded FP32 quotient yh plus the quotient
// of the residual nh + nl - yh (dh + dl), formed exactly up to its last rounding
__device__ __forceinline__ double df_quotient(float nh, float nl, float dh, float dl)
{
    const float yh = __fdiv_rn(nh, dh);
    const float p = __fmul_rn(yh, dh);
    const float e = fmaf(yh, dh, -p);
    float res = (nh - p) - e;  // nh - p is exact: p lies within a few ulp of nh
    res = res + nl;
    res = fmaf(-yh, dl, res);
    const float yl = __fmul_rn(res, __frcp_rn(dh));
    return f32_to_f64_nz(yh) + f32_to_f64_nz(yl);
}

// The central branch for q = dq 2^-52 (|q| <= 0.425): q converted in integer operations,
// r = 0.180625 - q^2 by one FP64 fused multiply-add, the two degree-7 polynomials and their
// quotient on float pairs, and q times the quotient in FP64.
__device__ __forceinline__ double icdf_central(int64_t dq)
{
    constexpr DfCoef a[8] = {dfc(2.5090809287301226727e+03), dfc(3.3430575583588128105e+04),
                             dfc(6.7265770927008700853e+04), dfc(4.5921953931549871457e+04),
                             dfc(1.3731693765509461125e+04), dfc(1.9715909503065514427e+03),
                             dfc(1.3314166789178437745e+02), dfc(3.3871328727963666080e+00)};
    constexpr DfCoef b[8] = {dfc(5.2264952788528545610e+03), dfc(2.8729085735721942674e+04),
                             dfc(3.9307895800092710610e+04), dfc(2.1213794301586595867e+04),
                             dfc(5.3941960214247511077e+03), dfc(6.8718700749205790830e+02),
                             dfc(4.2313330701600911252e+01), dfc(1.0)};
    double q = 0.0;
    if (dq != 0) {
        // |dq| < 2^51: exact as a double; exponent from the leading bit, scaled by 2^-52
        const unsigned long long m = (unsigned long long)(dq < 0 ? -dq : dq);
        const int lead = 63 - __clzll((long long)m);  // m in [2^lead, 2^(lead+1))
        const unsigned long long frac = (m << (52 - lead)) & 0xfffffffffffffull;
        const unsigned long long bits = (dq < 0 ? 0x8000000000000000ull : 0ull) |
                                        ((unsigned long long)(1023 + lead - 52) << 52) | frac;
        q = __longlong_as_double((long long)bits);
    }
    const double r = fma(-q, q, 0.180625);  // > 0 on the branch
    float rh, rl;
    float2 vh, vl;
    df_split_nz(r, rh, rl);
    df_horner8x2(rh, rl, a, b, vh, vl);
    return q * df_quotient(vh.x, vl.x, vh.y, vl.y);
}

// ---- float-pair arithmetic of the tail branch
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e)
{
    s = a + b;  // |a| >= |b|
    e = b - (s - a);
}

__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& sh, float& sl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    df_fast_two_sum(s, (al + bl) + e, sh, sl);
}

// The logarithm's table: for j = 0..127, r_j = 1/c_j rounded to FP32 with c_j = 1 + (j + 1/2)/128,
// and -log(r_j) as a float pair (FP64 log, split), built by each generator block in shared
// memory (FP64 form only).
struct LogTable {
    float r[128], lh[128], ll[128];
};

__device__ __forceinline__ void build_log_table(LogTable& t, int tid)
{
    if (tid < 128) {
        const float r = (float)(1.0 / (1.0 + ((double)tid + 0.5) / 128.0));
        const double lg = -log((double)r);
        t.r[tid] = r;
        t.lh[tid] = (float)lg;
        t.ll[tid] = (float)(lg - (double)t.lh[tid]);
    }
}

// sqrt(-log t) for t = M 2^-52, 1 <= M < 2^50, as a float pair (about 2^-46 relative), from
// the mathematics of the logarithm (Tang's table-driven reduction): t = x 2^k with x in [1, 2)
// read exactly from the integer; with j the leading seven fraction bits of x,
// y = x r_j - 1 (|y| <= 1/256, x r_j formed exactly), log x = -log(r_j) + log(1 + y) and
// log(1 + y) = y - y^2/2 + y^3 (1/3 - y/4 + y^2/5) (the truncated terms are below 2^-50; the
// cubic part in FP32, since it enters below 2^-24); log t = k log 2 + log x; the square
// root as the rounded FP32 root plus the residual's correction.
__device__ __forceinline__ void df_sqrt_neg_log(int64_t M, const LogTable& tab, float& rh, float& rl)
{
    constexpr DfCoef ln2 = dfc(0.693147180559945309417232121458176568);
    const unsigned long long um = (unsigned long long)M;
    const int lead = 63 - __clzll((long long)um);        // M in [2^lead, 2^(lead+1))
    const unsigned long long norm = um << (63 - lead);  // the leading one at bit 63
    const unsigned top = (unsigned)(norm >> 40);         // 24 bits: x's leading bits
    const float xh = __uint2float_rn(top) * 0x1.0p-23f;  // exact, in [1, 2)
    const unsigned rest = (unsigned)((norm >> 16) & 0xffffffull), rest2 = (unsigned)(norm & 0xffffull);
    const float xl = __fmaf_rn(__uint2float_rn(rest2), 0x1.0p-63f, __uint2float_rn(rest) * 0x1.0p-47f);
    const int j = (int)((top >> 16) & 127u);
    const float r = tab.r[j];
    // y = x r - 1: xh r as the exact pair (p, pe), p - 1 exact (p within 1/256 of 1)
    const float p = __fmul_rn(xh, r);
    const float pe = fmaf(xh, r, -p);
    float s, e;
    two_sum(p - 1.0f, pe, s, e);
    float yh, yl;
    df_fast_two_sum(s, fmaf(xl, r, e), yh, yl);
    // y^2 / 2 as a pair, the cubic part in FP32
    const float h2 = __fmul_rn(yh, yh);
    float e2 = fmaf(yh, yh, -h2);
    e2 = fmaf(yh + yh, yl, e2);
    const float B = fmaf(fmaf(yh, 0.2f, -0.25f), yh, 1.0f / 3.0f);
    const float y3B = __fmul_rn(__fmul_rn(__fmul_rn(yh, yh), yh), B);
    float ah, al;
    df_add(yh, yl, -0.5f * h2, -0.5f * e2, ah, al);
    df_add(ah, al, y3B, 0.0f, ah, al);
    df_add(ah, al, tab.lh[j], tab.ll[j], ah, al);  // log x
    const float K = (float)(lead - 52);
    const float pk = __fmul_rn(K, ln2.h);
    float ek = fmaf(K, ln2.h, -pk);
    ek = fmaf(K, ln2.l, ek);
    float Lh, Ll;
    df_add(pk, ek, ah, al, Lh, Ll);  // log t < -2.59
    const float nh = -Lh, nl = -Ll;
    const float q = __fsqrt_rn(nh);
    const float res = fmaf(-q, q, nh) + nl;
    df_fast_two_sum(q, __fmul_rn(res, __frcp_rn(q + q)), rh, rl);
}

// The tail branch (|p - 1/2| > 0.425, the draws the central test rejected) of the same
// transform for the tail probability t = M 2^-52 = min(u, 1 - u) > 0, without its sign:
// r = sqrt(-log t), then the rational functions of r - 1.6 (r <= 5) or r - 5 and their
// quotient, all on float pairs (the shifted argument is >= 0 and every coefficient positive).
__device__ double icdf_tail(int64_t M, const LogTable& tab)
{
    constexpr DfCoef c[8] = {dfc(7.74545014278341407640e-04), dfc(2.27238449892691845833e-02),
                             dfc(2.41780725177450611770e-01), dfc(1.27045825245236838258e+00),
                             dfc(3.64784832476320460504e+00), dfc(5.76949722146069140550e+00),
                             dfc(4.63033784615654529590e+00), dfc(1.42343711074968357734e+00)};
    constexpr DfCoef d[8] = {dfc(1.05075007164441684324e-09), dfc(5.47593808499534494600e-04),
                             dfc(1.51986665636164571966e-02), dfc(1.48103976427480074590e-01),
                             dfc(6.89767334985100004550e-01), dfc(1.67638483018380384940e+00),
                             dfc(2.05319162663775882187e+00), dfc(1.0)};
    constexpr DfCoef e[8] = {dfc(2.01033439929228813265e-07), dfc(2.71155556874348757815e-05),
                             dfc(1.24266094738807843860e-03), dfc(2.65321895265761230930e-02),
                             dfc(2.96560571828504891230e-01), dfc(1.78482653991729133580e+00),
                             dfc(5.46378491116411436990e+00), dfc(6.65790464350110377720e+00)};
    constexpr DfCoef f[8] = {dfc(2.04426310338993978564e-15), dfc(1.42151175831644588870e-07),
                             dfc(1.84631831751005468180e-05), dfc(7.86869131145613259100e-04),
                             dfc(1.48753612908506148525e-02), dfc(1.36929880922735805310e-01),
                             dfc(5.99832206555887937690e-01), dfc(1.0)};
    constexpr DfCoef c16 = dfc(1.6);
    float rh, rl, xh, xl;
    df_sqrt_neg_log(M, tab, rh, rl);
    float2 vh, vl;
    if (rh < 5.0f || (rh == 5.0f && rl <= 0.0f)) {
        df_add(rh, rl, -c16.h, -c16.l, xh, xl);
        df_horner8x2(xh, xl, c, d, vh, vl);
    } else {
        df_add(rh, rl, -5.0f, 0.0f, xh, xl);
        df_horner8x2(xh, xl, e, f, vh, vl);
    }
    return df_quotient(vh.x, vl.x, vh.y, vl.y);
}

// FP32 evaluation of the same rational approximations (mixed-precision form).  The draw
// u = (hi 2^26 + lo) 2^-52 is handled in 32-bit pieces: q = u - 1/2 = (dh 2^26 + lo) 2^-52
// with dh = hi - 2^25, and a tail probability min(u, 1-u) from the same pieces.
__device__ __forceinline__ float horner8f(float r, const float (&c)[8])
{
    // c[0] r^7 + ... + c[7], with fused multiply-adds (this file is built without contraction)
    float v = c[0];
#pragma unroll
    for (int i = 1; i < 8; i++) v = fmaf(v, r, c[i]);
    return v;
}

__device__ __forceinline__ float icdf_central_f32(float q)
{
    constexpr float a[8] = {2.5090809287301226727e+03f, 3.3430575583588128105e+04f, 6.7265770927008700853e+04f,
                            4.5921953931549871457e+04f, 1.3731693765509461125e+04f, 1.9715909503065514427e+03f,
                            1.3314166789178437745e+02f, 3.3871328727963666080e+00f};
    constexpr float b[8] = {5.2264952788528545610e+03f, 2.8729085735721942674e+04f, 3.9307895800092710610e+04f,
                            2.1213794301586595867e+04f, 5.3941960214247511077e+03f, 6.8718700749205790830e+02f,
                            4.2313330701600911252e+01f, 1.0f};
    const float r = fmaf(-q, q, 0.180625f);
    return __fdividef(q * horner8f(r, a), horner8f(r, b));
}

// tail branch for the tail probability t = min(u, 1-u) > 0; the sign is the caller's
__device__ __forceinline__ float icdf_tail_f32(float t)
{
    constexpr float c[8] = {7.74545014278341407640e-04f, 2.27238449892691845833e-02f, 2.41780725177450611770e-01f,
                            1.27045825245236838258e+00f, 3.64784832476320460504e+00f, 5.76949722146069140550e+00f,
                            4.63033784615654529590e+00f, 1.42343711074968357734e+00f};
    constexpr float d[8] = {1.05075007164441684324e-09f, 5.47593808499534494600e-04f, 1.51986665636164571966e-02f,
                            1.48103976427480074590e-01f, 6.89767334985100004550e-01f, 1.67638483018380384940e+00f,
                            2.05319162663775882187e+00f, 1.0f};
    constexpr float e[8] = {2.01033439929228813265e-07f, 2.71155556874348757815e-05f, 1.24266094738807843860e-03f,
                            2.65321895265761230930e-02f, 2.96560571828504891230e-01f, 1.78482653991729133580e+00f,
                            5.46378491116411436990e+00f, 6.65790464350110377720e+00f};
    constexpr float f[8] = {2.04426310338993978564e-15f, 1.42151175831644588870e-07f, 1.84631831751005468180e-05f,
                            7.86869131145613259100e-04f, 1.48753612908506148525e-02f, 1.36929880922735805310e-01f,
                            5.99832206555887937690e-01f, 1.0f};
    float r = sqrtf(-__logf(t));
    if (r <= 5.0f) {
        r -= 1.6f;
        return __fdividef(horner8f(r, c), horner8f(r, d));
    }
    r -= 5.0f;
    return __fdividef(horner8f(r, e), horner8f(r, f));
}

constexpr int kStateWords = 2 * kMtN;  // the two state buffers at the start of shared memory

// nxt = one regeneration of the 624-word state cur (three dependent phases of <= 227 words)
__device__ __forceinline__ void mt_regenerate(const uint32_t* cur, uint32_t* nxt, int tid)
{
    if (tid < 227) nxt[tid] = mt_next(cur[tid + kMtM], cur[tid], cur[tid + 1]);
    __syncthreads();
    if (tid < 227) {
        const int k = 227 + tid;
        nxt[k] = mt_next(nxt[k - 227], cur[k], cur[k + 1]);
    }
    __syncthreads();
    if (tid < 170) {
        const int k = 454 + tid;
        nxt[k] = mt_next(nxt[k - 227], cur[k], (k == kMtN - 1) ? nxt[0] : cur[k + 1]);
    }
    __syncthreads();
}

// Brownian increments dW[t*F+k][p] of the chunk [v0, v1) of the stream.  The stream runs
// path-major (path p's T*F draws are consecutive) while the output rows are [t*F+k][P]:
// the draws go to a shared-memory tile of K consecutive paths x T*F values, and each full
// tile leaves as row segments of K consecutive paths (K x element size = 128 bytes when the
// tile fits).  Column k of row r of the tile sits at k ^ (r mod K), so that both the
// column-wise fill and the row-wise drain are free of bank conflicts.
// Drain the tile of paths [pt, pt+K) to the increment rows.  An interior tile (all its
// draws inside the chunk) needs no per-element test.
template <typename OutT>
__device__ __forceinline__ void drain_tile(const OutT* tile, OutT* out, int TF, int K, int P, int64_t pt, int64_t ps,
                                           int ts, int64_t pe, int te, int r0, int rstep, int dk)
{
    const int64_t path = pt + dk;
    const bool interior = (pt > ps || ts == 0) && pt + K - 1 < pe;
    if (interior) {
        OutT* o = out + (size_t)r0 * P + path;
        const size_t ostep = (size_t)rstep * P;
        for (int r = r0; r < TF; r += rstep, o += ostep) *o = tile[r * K + (dk ^ (r & (K - 1)))];
    } else {
        for (int r = r0; r < TF; r += rstep)
            if (path < P && (path > ps || r >= ts) && (path < pe || (path == pe && r < te)))
                out[(size_t)r * P + path] = tile[r * K + (dk ^ (r & (K - 1)))];
    }
}

// The pending tail draws: a ring buffer of (draw word, position) entries; an evaluated
// entry holds its increment's bits in place of the draw.
struct TailQueue {
    unsigned long long w[kTailQueue];
    int2 pos[kTailQueue];  // (path relative to the chunk's first path, step * F + factor); path -1: placed
    int head;              // oldest entry not yet placed
    int snap;              // entries appended before the current round
    int tail;              // next free entry (atomic)
};

// One tail draw's increment (the draw word as the central test queued it), as the bits of the
// element type
template <typename OutT>
__device__ __forceinline__ unsigned long long tail_increment(const RngParams& prm, const LogTable& tab,
                                                             unsigned long long w, int row)
{
    uint32_t t, k;
    divmod_u32((uint32_t)row, (uint32_t)prm.num_factors, prm.magic_f, t, k);
    if constexpr (sizeof(OutT) == 8) {
        // the tail probability min(u, 1 - u) = M 2^-52 exactly; u = 0 gives 0 as in the reference
        const int64_t m = (int64_t)w;
        const bool lower = m < ((int64_t)1 << 51);
        const int64_t M = lower ? m : ((int64_t)1 << 52) - m;
        double val = 0.0;
        if (M > 0) {
            const double v = icdf_tail(M, tab);
            val = (lower ? -v : v) * __ldg(prm.sqrt_dt + t);
        }
        return (unsigned long long)__double_as_longlong(val);
    } else {
        const uint32_t hi = (uint32_t)(w >> 32), lo = (uint32_t)w;
        const bool lower = hi < (1u << 25);
        // min(u, 1-u): u itself below 1/2; 1-u = ((2^26-1-hi) 2^26 + (2^26-lo)) 2^-52 above
        const float tp = lower ? fmaf((float)lo, 0x1.0p-52f, (float)hi * 0x1.0p-26f)
                               : fmaf((float)((1u << 26) - lo), 0x1.0p-52f, (float)((1u << 26) - 1u - hi) * 0x1.0p-26f);
        float v = tp > 0.0f ? icdf_tail_f32(tp) : 0.0f;
        if (lower) v = -v;
        return (unsigned long long)__float_as_uint(v * __ldg(prm.sqrt_dt32 + t));
    }
}

template <typename OutT>
__device__ __forceinline__ OutT from_bits(unsigned long long b)
{
    if constexpr (sizeof(OutT) == 8) return __longlong_as_double((long long)b);
    else return __uint_as_float((unsigned)b);
}

// Brownian increments dW[t*F+k][p] of the chunk [v0, v1) of the stream.  The stream runs
// path-major (path p's T*F draws are consecutive) while the output rows are [t*F+k][P]:
// the draws go to a shared-memory tile of K consecutive paths x T*F values, and each full
// tile leaves as row segments of K consecutive paths (K x element size = 128 bytes when the
// tile fits).  Column k of row r of the tile sits at k ^ (r mod K), so that both the
// column-wise fill and the row-wise drain are free of bank conflicts.  Draw thread i owns
// draw i of every round; its position (path, step, factor) advances by the round's 312 draws
// without divisions.  A draw in the central region is evaluated at once; a tail draw (about
// 15 %) joins the queue, whose entries the two tail warps evaluate during the next round
// (up to 64 a round), so that the slow tail branch runs beside the central draws instead of
// after them.  Entries still pending when a tile is about to drain (and at the chunk's end,
// or when the queue fills) are evaluated by every thread in the round's second interval.
template <typename OutT>
__device__ __forceinline__ void increments_loop(const RngParams& prm, uint32_t* x, int tid, int64_t v0, int64_t v1,
                                                TailQueue& q, const LogTable& tab)
{
    constexpr bool kExact = sizeof(OutT) == 8;  // FP64 increments (the parity form)
    // The FP64 tail branch costs more than a round's central draws, so the tail warps take it
    // off the critical path; the FP32 one is cheap enough that the extra queue traffic would
    // cost more than it saves: the FP32 form evaluates every round's tails in its second
    // interval, by all threads.
    constexpr bool kTailWarps = kExact;
    constexpr int kRound = kMtN / 2;
    constexpr int kMask = kTailQueue - 1;
    const int TF = prm.values_per_path, F = prm.num_factors, P = prm.num_paths, K = prm.tile_k;
    const int T = TF / F;
    OutT* tile = reinterpret_cast<OutT*>(x + kStateWords);
    OutT* out = static_cast<OutT*>(prm.out);
    const int64_t ps = v0 / TF, pe = v1 / TF;
    const int ts = (int)(v0 - ps * TF), te = (int)(v1 - pe * TF);  // chunk = [(ps, ts), (pe, te))
    // positions relative to the chunk's first path ps
    int rpo = 0, rtf = ts;  // the round's first draw
    int spo, st, sk;        // this thread's draw: path, time step, factor
    {
        uint32_t q0, r, t, k;
        divmod_u32((uint32_t)(ts + tid), (uint32_t)TF, prm.magic_tf, q0, r);
        divmod_u32(r, (uint32_t)F, prm.magic_f, t, k);
        spo = (int)q0;
        st = (int)t;
        sk = (int)k;
    }
    const int a_tf = kRound % TF, a_po = kRound / TF, a_t = a_tf / F, a_k = a_tf % F;
    int pt = 0;  // first path of the tile, relative to ps
    const int lane = tid & 31, warp = tid >> 5;
    const int rpp = 32 / K;  // tile rows drained per warp pass
    const int nthreads = blockDim.x;  // the FP32 form runs without the tail warps
    const int dk = lane % K, r0 = warp * rpp + lane / K, rstep = (nthreads / 32) * rpp;
    const int rounds = (int)((v1 - v0 + kRound - 1) / kRound);
    if (tid == 0) {
        q.head = 0;
        q.snap = 0;
        q.tail = 0;
    }
    // Software pipeline: the words of round rd sit in `cur`; while the block turns them into
    // increments it also twists them into round rd+1's words in `nxt` (the three phases of
    // the twist share the three barrier intervals of the round's draws, pending tails and
    // placement).
    uint32_t* cur = x + kMtN;
    uint32_t* nxt = x;
    mt_regenerate(x, cur, tid);  // round 0 from the jumped state (its barriers also publish the queue)
    for (int rd = 0; rd < rounds; rd++) {
        const bool more = rd + 1 < rounds;
        const int nv = min(kRound, (int)(v1 - v0 - (int64_t)rd * kRound));
        uint32_t dl, rl;
        divmod_u32((uint32_t)(rtf + nv - 1), (uint32_t)TF, prm.magic_tf, dl, rl);
        const int plast = rpo + (int)dl;  // path of the round's last draw
        const int head = q.head, snap = q.snap;
        const int take = kTailWarps ? min(snap - head, kTailWarpThreads) : 0;  // the tail warps' share
        // ---- interval 1: twist phase 1 of round rd+1; central draws of round rd; the tail
        // warps evaluate pending entries [head, head + take)
        if (more && tid < 227) nxt[tid] = mt_next(cur[tid + kMtM], cur[tid], cur[tid + 1]);
        OutT hv0 = OutT(0);
        int hp0 = -1, hf0 = 0;  // held draw: path (relative to ps; -1: none), row
        if (tid < nv) {
            const uint2 ww = *reinterpret_cast<const uint2*>(cur + 2 * tid);
            const uint32_t w1 = mt_temper(ww.x), w2 = mt_temper(ww.y);
            bool central;
            unsigned long long qw;
            if constexpr (kExact) {
                // |u - 1/2| <= 0.425 tested exactly on the 52-bit grid, u = m 2^-52
                const int64_t m = (int64_t)(((uint64_t)(w1 >> 6) << 26) | (uint64_t)(w2 >> 6));
                const int64_t dq = m - ((int64_t)1 << 51);
                central = (dq < 0 ? -dq : dq) <= prm.central_max;
                if (central) hv0 = icdf_central(dq) * __ldg(prm.sqrt_dt + st);
                qw = (unsigned long long)m;
            } else {
                const uint32_t hi = w1 >> 6, lo = w2 >> 6;  // u = (hi 2^26 + lo) 2^-52
                const float qv = fmaf((float)lo, 0x1.0p-52f, (float)((int)hi - (1 << 25)) * 0x1.0p-26f);
                central = fabsf(qv) <= 0.425f;
                if (central) hv0 = icdf_central_f32(qv) * __ldg(prm.sqrt_dt32 + st);
                qw = ((unsigned long long)hi << 32) | lo;
            }
            if (central) {
                hp0 = spo;
                hf0 = st * F + sk;
            } else {
                const int e = atomicAdd(&q.tail, 1) & kMask;
                q.w[e] = qw;
                q.pos[e] = make_int2(spo, st * F + sk);
            }
        } else if (tid >= kDrawThreads) {
            const int i = tid - kDrawThreads;
            if (i < take) {
                const int e = (head + i) & kMask;
                q.w[e] = tail_increment<OutT>(prm, tab, q.w[e], q.pos[e].y);
            }
        }
        __syncthreads();
        // ---- interval 2: twist phase 2; before a drain (and at the end, or when the queue is
        // nearly full) every thread evaluates the remaining pending entries
        if (more && tid < 227) {
            const int k = 227 + tid;
            nxt[k] = mt_next(nxt[k - 227], cur[k], cur[k + 1]);
        }
        const int qend = q.tail;
        const bool flush = !kTailWarps || !more || plast >= pt + K ||
                           qend - (head + take) > kTailQueue - kRound - kTailWarpThreads;
        const int done = flush ? qend : head + take;  // entries [head, done) are evaluated after this interval
        OutT hv1 = OutT(0);
        int hp1 = -1, hf1 = 0;  // FP32: the round's tail draw held by this thread
        if constexpr (kTailWarps) {
            if (flush)
                for (int e = head + take + tid; e < qend; e += nthreads)
                    q.w[e & kMask] = tail_increment<OutT>(prm, tab, q.w[e & kMask], q.pos[e & kMask].y);
        } else if (tid < qend - head) {  // at most one round's tails, one per thread
            const int e = (head + tid) & kMask;
            hv1 = from_bits<OutT>(tail_increment<OutT>(prm, tab, q.w[e], q.pos[e].y));
            hp1 = q.pos[e].x;
            hf1 = q.pos[e].y;
        }
        __syncthreads();
        // ---- interval 3: twist phase 3; place the held draws and the evaluated entries,
        // draining the tile when needed
        if (more && tid < 170) {
            const int k = 454 + tid;
            nxt[k] = mt_next(nxt[k - 227], cur[k], (k == kMtN - 1) ? nxt[0] : cur[k + 1]);
        }
        while (true) {
            if (hp0 >= 0 && hp0 < pt + K) {
                tile[hf0 * K + ((hp0 - pt) ^ (hf0 & (K - 1)))] = hv0;
                hp0 = -1;
            }
            if constexpr (kTailWarps) {
                for (int e = head + tid; e < done; e += nthreads) {
                    const int2 ps2 = q.pos[e & kMask];
                    if (ps2.x >= 0 && ps2.x < pt + K) {
                        tile[ps2.y * K + ((ps2.x - pt) ^ (ps2.y & (K - 1)))] = from_bits<OutT>(q.w[e & kMask]);
                        q.pos[e & kMask].x = -1;
                    }
                }
            } else if (hp1 >= 0 && hp1 < pt + K) {
                tile[hf1 * K + ((hp1 - pt) ^ (hf1 & (K - 1)))] = hv1;
                hp1 = -1;
            }
            if (plast < pt + K) break;
            __syncthreads();
            drain_tile<OutT>(tile, out, TF, K, P, ps + pt, ps, ts, pe, te, r0, rstep, dk);
            __syncthreads();
            pt += K;
        }
        if (tid == 0) {
            q.head = done;
            q.snap = q.tail;  // every append of this round happened before the barriers above
        }
        __syncthreads();  // round rd+1's words complete; `cur` is free for round rd+2
        // advance the round's and this thread's positions by 312 draws
        rtf += a_tf;
        rpo += a_po;
        if (rtf >= TF) {
            rtf -= TF;
            rpo++;
        }
        sk += a_k;
        st += a_t;
        spo += a_po;
        if (sk >= F) {
            sk -= F;
            st++;
        }
        if (st >= T) {
            st -= T;
            spo++;
        }
        uint32_t* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    __syncthreads();
    drain_tile<OutT>(tile, out, TF, K, P, ps + pt, ps, ts, pe, te, r0, rstep, dk);
}

// Chunk start states: the seeded state moved to word offset 2 v0 = c * stride by one GF(2)
// jump per nonzero base-8 digit of the chunk index c, written to states[c][624].  Its own
// kernel: the jump window (kJumpWindow words of shared memory) would otherwise cap the
// generator at two blocks per SM.
// Block b starts from src[b >> src_shift] (the seeded state when src is null) and applies the
// digits j_lo..j_hi-1 of the chunk index c = b << idx_shift, writing dst[b].  One launch
// with all digits moves every chunk by up to three jumps; two levels (the groups of eight
// chunks by their upper digits, then each chunk from its group by its lowest digit) take at
// most two jumps per group and one per chunk.
__global__ void __launch_bounds__(kRngThreads) mt_jump_kernel(const RngParams prm, const uint32_t* src, int src_shift,
                                                              int idx_shift, int j_lo, int j_hi, uint32_t* dst)
{
    extern __shared__ __align__(16) uint32_t x[];  // the jump window
    const int tid = threadIdx.x;
    const int64_t b = blockIdx.x;
    const int64_t c = b << idx_shift;
    if (c * prm.chunk_values >= prm.num_values) return;
    const uint32_t* s0 = src ? src + (size_t)(b >> src_shift) * kMtN : prm.seeded;
    for (int i = tid; i < kMtN; i += kRngThreads) x[i] = s0[i];
    __syncthreads();

    // jump to word offset 2*v0 = c * stride: apply x^(d 8^j stride) for every nonzero
    // base-8 digit d of c (position j) in [j_lo, j_hi)
    for (int j = j_lo; j < j_hi; j++) {
        const int d = (int)((c >> (kJumpDigitBits * j)) & (kJumpBase - 1));
        if (d == 0) continue;
        const int list = j * (kJumpBase - 1) + d - 1;
        for (int base = kMtN; base < kJumpWindow; base += 227) {
            const int n = base + tid;
            if (tid < 227 && n < kJumpWindow) x[n] = mt_next(x[n - 227], x[n - kMtN], x[n - kMtN + 1]);
            __syncthreads();
        }
        // the new state word n is the XOR over the set bits i of the polynomial of x[i + n]
        const uint16_t* bits = prm.jump_bits + prm.bit_off[list];
        const int cnt = prm.bit_cnt[list];
        const bool two = tid + kRngThreads < kMtN;
        const uint32_t* x0 = x + tid;
        const uint32_t* x1 = x + (two ? tid + kRngThreads : tid);
        uint32_t acc0 = 0, acc1 = 0;
        int k = 0;
        for (; k + 8 <= cnt; k += 8) {
            const uint4 w = __ldg(reinterpret_cast<const uint4*>(bits + k));  // eight 16-bit positions
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const uint32_t i0 = ww[h] & 0xffffu, i1 = ww[h] >> 16;
                acc0 ^= x0[i0] ^ x0[i1];
                acc1 ^= x1[i0] ^ x1[i1];
            }
        }
        for (; k < cnt; k++) {
            const uint32_t i = __ldg(bits + k);
            acc0 ^= x0[i];
            acc1 ^= x1[i];
        }
        __syncthreads();
        x[tid] = acc0;
        if (two) x[tid + kRngThreads] = acc1;
        __syncthreads();
    }

    for (int i = tid; i < kMtN; i += kRngThreads) dst[b * kMtN + i] = x[i];
}

__global__ void __launch_bounds__(kGenThreads, 3) mt_generate_kernel(const RngParams prm, const uint32_t* states)
{
    // shared memory: the two state buffers (kStateWords words) followed by the increments tile
    extern __shared__ __align__(16) uint32_t x[];
    __shared__ TailQueue tails;
    __shared__ LogTable logtab;
    const int tid = threadIdx.x;
    const int64_t c = blockIdx.x;
    const int64_t v0 = c * prm.chunk_values;
    if (v0 >= prm.num_values) return;
    const int64_t v1 = min(v0 + prm.chunk_values, prm.num_values);

    for (int i = tid; i < kMtN; i += (int)blockDim.x) x[i] = states[c * kMtN + i];  // the chunk's start state
    if (prm.mode == 1) build_log_table(logtab, tid);
    __syncthreads();

    if (prm.mode == 1) {
        increments_loop<double>(prm, x, tid, v0, v1, tails, logtab);
    } else if (prm.mode == 2) {
        increments_loop<float>(prm, x, tid, v0, v1, tails, logtab);
    } else {
        // uniforms in stream order (contiguous stores)
        uint32_t* cur = x;
        uint32_t* nxt = x + kMtN;
        for (int64_t v = v0; v < v1; v += kMtN / 2) {
            mt_regenerate(cur, nxt, tid);
            if (tid < kMtN / 2 && v + tid < v1) {
                const uint32_t w1 = mt_temper(nxt[2 * tid]);
                const uint32_t w2 = mt_temper(nxt[2 * tid + 1]);
                const int64_t m = (int64_t)(((uint64_t)(w1 >> 6) << 26) | (uint64_t)(w2 >> 6));  // u = m 2^-52
                static_cast<double*>(prm.out)[v + tid] = (double)m * 0x1.0p-52;
            }
            uint32_t* tmp = cur;
            cur = nxt;
            nxt = tmp;
        }
    }
}

}  // namespace

int plan_mt_generate(int64_t num_values, int values_per_path, int elem_bytes, RngPlan* plan)
{
    int dev = 0, sms = 0, per_sm = 0;
    LMM_CUDA(cudaGetDevice(&dev));
    LMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // the increments tile: K paths x values_per_path, K x element = 128 bytes when it fits
    int kbytes = 128;
    const size_t budget = 64 * 1024;  // three generator CTAs per SM beside the static tail queue and log table (10 KB)
    if (values_per_path > 1) {
        while (kbytes > elem_bytes && (size_t)values_per_path * kbytes + kStateWords * 4 > budget) kbytes /= 2;
        if ((size_t)values_per_path * kbytes + kStateWords * 4 > budget)
            return fail(LMM_ERR_INVALID, "too many increments per path for the generator tile");
    }
    plan->tile_k = values_per_path > 1 ? kbytes / elem_bytes : 1;
    const size_t tile_bytes = (size_t)values_per_path * plan->tile_k * elem_bytes;  // a one-path tile when 1 value per path
    plan->smem_bytes = (int)((size_t)kStateWords * 4 + tile_bytes);
    LMM_CUDA(cudaFuncSetAttribute(mt_generate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024));
    LMM_CUDA(cudaFuncSetAttribute(mt_jump_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kJumpWindow * 4));
    LMM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mt_generate_kernel, elem_bytes == 8 ? kGenThreads : kDrawThreads,
                                                           plan->smem_bytes));
    const int resident = sms * (per_sm > 0 ? per_sm : 1);
    // one chunk per resident CTA, at least 4096 values per chunk
    int64_t chunks = resident;
    int64_t chunk_values = (num_values + chunks - 1) / chunks;
    if (chunk_values < 4096) chunk_values = 4096;
    chunks = (num_values + chunk_values - 1) / chunk_values;
    int ndigits = 0;
    while (ndigits < 21 && ((int64_t)1 << (kJumpDigitBits * ndigits)) < chunks) ndigits++;
    plan->chunks = chunks;
    plan->chunk_values = chunk_values;
    plan->ndigits = ndigits;
    plan->polys.clear();
    const int nlists = ndigits * (kJumpBase - 1);
    if (nlists > kMaxJumps) return fail(LMM_ERR_INVALID, "too many generator chunks");
    if (ndigits > 0) {
        const std::vector<uint64_t>& v = mt_jump_digit_polynomials(2ull * (uint64_t)chunk_values, ndigits);
        std::vector<uint16_t> list;
        for (int j = 0; j < nlists; j++) {
            while (list.size() % 8) list.push_back(0);  // each list starts 16-byte aligned
            plan->bit_off[j] = (int)list.size();
            for (int q = 0; q < kPolyWords; q++)
                for (int b = 0; b < 64; b++)
                    if ((v[(size_t)j * kPolyWords + q] >> b) & 1ull) list.push_back((uint16_t)(q * 64 + b));
            plan->bit_cnt[j] = (int)list.size() - plan->bit_off[j];
        }
        while (list.size() % 8) list.push_back(0);
        plan->polys.resize(list.size() / 4);
        std::memcpy(plan->polys.data(), list.data(), list.size() * sizeof(uint16_t));
    }
    return LMM_OK;
}

int launch_mt_generate(const RngLaunch& a, cudaStream_t s, int* num_launches)
{
    if (a.num_values <= 0) return LMM_OK;
    RngParams prm;
    prm.seeded = a.d_seeded;
    prm.jump_bits = reinterpret_cast<const uint16_t*>(a.d_jumps);
    prm.ndigits = a.plan->ndigits;
    if (prm.ndigits * (kJumpBase - 1) > kMaxJumps || ((int64_t)1 << (kJumpDigitBits * prm.ndigits)) < a.plan->chunks)
        return fail(LMM_ERR_INVALID, "generator plan does not cover its chunks");
    for (int j = 0; j < prm.ndigits * (kJumpBase - 1); j++) {
        prm.bit_off[j] = a.plan->bit_off[j];
        prm.bit_cnt[j] = a.plan->bit_cnt[j];
    }
    prm.num_values = a.num_values;
    prm.chunk_values = a.plan->chunk_values;
    prm.values_per_path = a.values_per_path;
    prm.num_paths = a.num_paths;
    prm.num_factors = a.num_factors;
    prm.mode = a.mode;
    prm.sqrt_dt = a.d_sqrt_dt;
    prm.sqrt_dt32 = a.d_sqrt_dt32;
    prm.out = a.d_out;
    prm.central_max = (int64_t)std::floor(0.425 * 4503599627370496.0);  // exact: 0.425 scaled by 2^52
    prm.magic_tf = a.values_per_path > 0 ? 0xFFFFFFFFu / (uint32_t)a.values_per_path : 0u;
    prm.magic_f = a.num_factors > 0 ? 0xFFFFFFFFu / (uint32_t)a.num_factors : 0u;
    if (a.mode == 2 && !a.d_sqrt_dt32) return fail(LMM_ERR_INVALID, "FP32 increments need the FP32 step table");
    if (a.mode != 0 && (a.values_per_path <= 0 || a.num_factors <= 0 || a.values_per_path >= (1 << 30)))
        return fail(LMM_ERR_INVALID, "Brownian increments need 1 <= factors and values per path < 2^30");
    prm.tile_k = a.plan->tile_k;
    if (a.mode != 0) {
        const size_t elem = a.mode == 1 ? sizeof(double) : sizeof(float);
        const int K = a.plan->tile_k;
        if (K < 1 || K > 32 || (K & (K - 1)) ||
            (size_t)a.plan->smem_bytes < kStateWords * sizeof(uint32_t) + (size_t)a.values_per_path * K * elem)
            return fail(LMM_ERR_INVALID, "generator plan does not match the increments layout");
    }
    const bool two_level = prm.ndigits > 1;
    {
        KernelTimer kt(K_MT_JUMP_GENERATE, s, two_level ? 3 : 2);
        const int64_t groups = (a.plan->chunks + kJumpBase - 1) >> kJumpDigitBits;
        uint32_t* states = nullptr;  // [chunks][624] chunk start states, then [groups][624] group states
        const int arc = device_alloc(reinterpret_cast<void**>(&states),
                                     sizeof(uint32_t) * kMtN * (size_t)(a.plan->chunks + (two_level ? groups : 0)), s,
                                     "cudaMallocAsync (generator chunk states)");
        if (arc) return arc;
        if (two_level) {
            uint32_t* gstates = states + (size_t)a.plan->chunks * kMtN;
            mt_jump_kernel<<<(unsigned)groups, kRngThreads, (size_t)kJumpWindow * 4, s>>>(prm, nullptr, 0, kJumpDigitBits, 1,
                                                                                          prm.ndigits, gstates);
            mt_jump_kernel<<<(unsigned)a.plan->chunks, kRngThreads, (size_t)kJumpWindow * 4, s>>>(prm, gstates, kJumpDigitBits,
                                                                                                   0, 0, 1, states);
        } else {
            mt_jump_kernel<<<(unsigned)a.plan->chunks, kRngThreads, (size_t)kJumpWindow * 4, s>>>(prm, nullptr, 0, 0, 0,
                                                                                                   prm.ndigits, states);
        }
        // the FP64 form with its two tail warps, the FP32 form and the uniforms with the draw warps
        const int threads = prm.mode == 1 ? kGenThreads : kDrawThreads;
        mt_generate_kernel<<<(unsigned)a.plan->chunks, threads, (size_t)a.plan->smem_bytes, s>>>(prm, states);
        const cudaError_t e = cudaGetLastError();
        cudaFreeAsync(states, s);
        if (e != cudaSuccess) return cuda_fail(e, "generator launch");
        LMM_CUDA(cudaGetLastError());
    }
    if (num_launches) (*num_launches) += two_level ? 3 : 2;
    return LMM_OK;
}

}  // namespace lmm
