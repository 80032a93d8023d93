// rng.cu -- K1: partitioned MT19937 + Wichura inverse normal (Brownian increments).
//
// Reference: BrownianMotionFromMersenneRandomNumbers.doGenerateBrownianMotion
// (montecarlo/BrownianMotionFromMersenneRandomNumbers.java:141-191) draws, from one
// MersenneTwister stream, u = nextDouble() for path -> time -> factor and stores
// dW[t][f][p] = NormalDistribution.inverseCumulativeDistribution(u) * sqrt(dt_t).
//
// GB300 design: the stream of V values (2 words each) is cut into one contiguous chunk
// per CTA.  A CTA first moves the seeded state to its chunk start with GF(2) jump
// polynomials (one per set bit of its chunk index; each jump is an XOR of windows of
// the raw word sequence held in shared memory), then regenerates 624 words at a time
// in three dependency phases (227/227/170 words) over a double-buffered state, and
// converts word pairs to values.  Uniforms are bit-identical to the single stream.
//
// This translation unit is compiled with -fmad=false: the FP64 inverse normal must
// round exactly like the reference's unfused Java arithmetic.
#include "lmm_internal.h"

#include <cmath>

namespace lmm {
namespace {

constexpr int kRngThreads = 320;

struct RngParams {
    int64_t central_max;      // |m - 2^51| <= central_max  <=>  |u - 0.5| <= 0.425 for u = m 2^-52
    uint32_t magic_tf;        // floor((2^32-1)/TF): division by the values per path
    uint32_t magic_f;         // floor((2^32-1)/F)
    const uint32_t* seeded;   // [624]
    const uint64_t* jumps;    // [njumps][312]
    int njumps;
    int64_t num_values;
    int64_t chunk_values;
    int values_per_path;
    int num_paths;
    int num_factors;
    int mode;
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
// AS241 (Wichura 1988) with the reference's evaluation order.  The central branch
// (|p - 0.5| <= 0.425, ~85 % of draws) and the tails are separate functions so that the
// generator can run each on a compacted set of lanes.
__device__ __forceinline__ double icdf_central(double q)
{
    const double r = 0.180625 - q * q;
    const double num = (((((((2.5090809287301226727e+03 * r + 3.3430575583588128105e+04) * r +
                             6.7265770927008700853e+04) * r + 4.5921953931549871457e+04) * r +
                           1.3731693765509461125e+04) * r + 1.9715909503065514427e+03) * r +
                         1.3314166789178437745e+02) * r + 3.3871328727963666080e+00);
    const double den = (((((((5.2264952788528545610e+03 * r + 2.8729085735721942674e+04) * r +
                             3.9307895800092710610e+04) * r + 2.1213794301586595867e+04) * r +
                           5.3941960214247511077e+03) * r + 6.8718700749205790830e+02) * r +
                         4.2313330701600911252e+01) * r + 1.0);
    return q * num / den;
}

__device__ double icdf_wichura(double p)
{
    const double q = p - 0.5;
    if (fabs(q) <= 0.425) {
        const double r = 0.180625 - q * q;
        const double num = (((((((2.5090809287301226727e+03 * r + 3.3430575583588128105e+04) * r +
                                 6.7265770927008700853e+04) * r + 4.5921953931549871457e+04) * r +
                               1.3731693765509461125e+04) * r + 1.9715909503065514427e+03) * r +
                             1.3314166789178437745e+02) * r + 3.3871328727963666080e+00);
        const double den = (((((((5.2264952788528545610e+03 * r + 2.8729085735721942674e+04) * r +
                                 3.9307895800092710610e+04) * r + 2.1213794301586595867e+04) * r +
                               5.3941960214247511077e+03) * r + 6.8718700749205790830e+02) * r +
                             4.2313330701600911252e+01) * r + 1.0);
        return q * num / den;
    }
    double r = (q < 0.0) ? p : 1.0 - p;
    if (r <= 0.0) return 0.0;
    r = sqrt(-log(r));
    double v;
    if (r <= 5.0) {
        r -= 1.6;
        v = (((((((7.74545014278341407640e-04 * r + 2.27238449892691845833e-02) * r +
                  2.41780725177450611770e-01) * r + 1.27045825245236838258e+00) * r +
                3.64784832476320460504e+00) * r + 5.76949722146069140550e+00) * r +
              4.63033784615654529590e+00) * r + 1.42343711074968357734e+00) /
            (((((((1.05075007164441684324e-09 * r + 5.47593808499534494600e-04) * r +
                  1.51986665636164571966e-02) * r + 1.48103976427480074590e-01) * r +
                6.89767334985100004550e-01) * r + 1.67638483018380384940e+00) * r +
              2.05319162663775882187e+00) * r + 1.0);
    } else {
        r -= 5.0;
        v = (((((((2.01033439929228813265e-07 * r + 2.71155556874348757815e-05) * r +
                  1.24266094738807843860e-03) * r + 2.65321895265761230930e-02) * r +
                2.96560571828504891230e-01) * r + 1.78482653991729133580e+00) * r +
              5.46378491116411436990e+00) * r + 6.65790464350110377720e+00) /
            (((((((2.04426310338993978564e-15 * r + 1.42151175831644588870e-07) * r +
                  1.84631831751005468180e-05) * r + 7.86869131145613259100e-04) * r +
                1.48753612908506148525e-02) * r + 1.36929880922735805310e-01) * r +
              5.99832206555887937690e-01) * r + 1.0);
    }
    return (q < 0.0) ? -v : v;
}

// FP32 evaluation of the same rational approximations (mixed-precision form).  The draw
// u = (hi 2^26 + lo) 2^-52 is handled in 32-bit pieces: q = u - 1/2 = (dh 2^26 + lo) 2^-52
// with dh = hi - 2^25, and a tail probability min(u, 1-u) from the same pieces.
__device__ __forceinline__ float icdf_central_f32(float q)
{
    const float r = 0.180625f - q * q;
    const float num = (((((((2.5090809287301226727e+03f * r + 3.3430575583588128105e+04f) * r +
                            6.7265770927008700853e+04f) * r + 4.5921953931549871457e+04f) * r +
                          1.3731693765509461125e+04f) * r + 1.9715909503065514427e+03f) * r +
                        1.3314166789178437745e+02f) * r + 3.3871328727963666080e+00f);
    const float den = (((((((5.2264952788528545610e+03f * r + 2.8729085735721942674e+04f) * r +
                            3.9307895800092710610e+04f) * r + 2.1213794301586595867e+04f) * r +
                          5.3941960214247511077e+03f) * r + 6.8718700749205790830e+02f) * r +
                        4.2313330701600911252e+01f) * r + 1.0f);
    return __fdividef(q * num, den);
}

// tail branch for the tail probability t = min(u, 1-u) > 0; the sign is the caller's
__device__ __forceinline__ float icdf_tail_f32(float t)
{
    float r = sqrtf(-__logf(t));
    if (r <= 5.0f) {
        r -= 1.6f;
        return __fdividef((((((((7.74545014278341407640e-04f * r + 2.27238449892691845833e-02f) * r +
                                2.41780725177450611770e-01f) * r + 1.27045825245236838258e+00f) * r +
                              3.64784832476320460504e+00f) * r + 5.76949722146069140550e+00f) * r +
                            4.63033784615654529590e+00f) * r + 1.42343711074968357734e+00f),
                          (((((((1.05075007164441684324e-09f * r + 5.47593808499534494600e-04f) * r +
                                1.51986665636164571966e-02f) * r + 1.48103976427480074590e-01f) * r +
                              6.89767334985100004550e-01f) * r + 1.67638483018380384940e+00f) * r +
                            2.05319162663775882187e+00f) * r + 1.0f));
    }
    r -= 5.0f;
    return __fdividef((((((((2.01033439929228813265e-07f * r + 2.71155556874348757815e-05f) * r +
                            1.24266094738807843860e-03f) * r + 2.65321895265761230930e-02f) * r +
                          2.96560571828504891230e-01f) * r + 1.78482653991729133580e+00f) * r +
                        5.46378491116411436990e+00f) * r + 6.65790464350110377720e+00f),
                      (((((((2.04426310338993978564e-15f * r + 1.42151175831644588870e-07f) * r +
                            1.84631831751005468180e-05f) * r + 7.86869131145613259100e-04f) * r +
                          1.48753612908506148525e-02f) * r + 1.36929880922735805310e-01f) * r +
                        5.99832206555887937690e-01f) * r + 1.0f));
}

__global__ void __launch_bounds__(kRngThreads, 2) mt_generate_kernel(const RngParams prm)
{
    extern __shared__ uint32_t x[];  // kJumpWindow words: jump window, then 2 x 624 state buffers
    const int tid = threadIdx.x;
    const int64_t c = blockIdx.x;
    const int64_t v0 = c * prm.chunk_values;
    if (v0 >= prm.num_values) return;
    const int64_t v1 = min(v0 + prm.chunk_values, prm.num_values);

    for (int i = tid; i < kMtN; i += kRngThreads) x[i] = prm.seeded[i];
    __syncthreads();

    // ---- jump to word offset 2*v0 = c * stride: apply x^(2^j stride) for every set bit j of c
    for (int j = 0; j < prm.njumps; j++) {
        if (!((c >> j) & 1)) continue;
        for (int base = kMtN; base < kJumpWindow; base += 227) {
            const int n = base + tid;
            if (tid < 227 && n < kJumpWindow) x[n] = mt_next(x[n - 227], x[n - kMtN], x[n - kMtN + 1]);
            __syncthreads();
        }
        const uint64_t* g = prm.jumps + (size_t)j * kPolyWords;
        uint32_t acc0 = 0, acc1 = 0;
        const bool two = tid + kRngThreads < kMtN;
        for (int q = 0; q < kPolyWords; q++) {
            uint64_t bits = __ldg(g + q);
            while (bits) {
                const int b = __ffsll((long long)bits) - 1;
                bits &= bits - 1;
                const int i = q * 64 + b;
                acc0 ^= x[i + tid];
                if (two) acc1 ^= x[i + tid + kRngThreads];
            }
        }
        __syncthreads();
        x[tid] = acc0;
        if (two) x[tid + kRngThreads] = acc1;
        __syncthreads();
    }

    // ---- generate: 624 words -> 312 values per round
    uint32_t* cur = x;
    uint32_t* nxt = x + kMtN;
    // tail draws of a round, processed by consecutive lanes after the central ones
    __shared__ unsigned long long tail_w[kMtN / 2];
    __shared__ short tail_i[kMtN / 2];
    __shared__ int tail_n;
    const int TF = prm.values_per_path;
    const int F = prm.num_factors;
    const int P = prm.num_paths;
    const bool normals = prm.mode != 0;      // uniforms (mode 0) carry no path position
    int64_t path0 = normals ? v0 / TF : 0;   // path of the chunk's first value
    int tf0 = (int)(v0 - path0 * TF);        // its position within the path
    for (int64_t v = v0; v < v1; v += kMtN / 2) {
        if (tid < 227) nxt[tid] = mt_next(cur[tid + kMtM], cur[tid], cur[tid + 1]);
        __syncthreads();
        if (tid < 227) {
            const int k = 227 + tid;
            nxt[k] = mt_next(nxt[k - 227], cur[k], cur[k + 1]);
        }
        if (tid == 0) tail_n = 0;  // every lane finished the previous round's tails before the barrier above
        __syncthreads();
        if (tid < 170) {
            const int k = 454 + tid;
            nxt[k] = mt_next(nxt[k - 227], cur[k], (k == kMtN - 1) ? nxt[0] : cur[k + 1]);
        }
        __syncthreads();
        if (prm.mode == 2) {
            // FP32 increments: 32-bit integer and FP32 arithmetic only
            if (tid < kMtN / 2 && v + tid < v1) {
                const uint32_t hi = mt_temper(nxt[2 * tid]) >> 6;   // u = (hi 2^26 + lo) 2^-52
                const uint32_t lo = mt_temper(nxt[2 * tid + 1]) >> 6;
                const int dh = (int)hi - (1 << 25);
                const float q = fmaf((float)lo, 0x1.0p-52f, (float)dh * 0x1.0p-26f);
                if (fabsf(q) <= 0.425f) {
                    uint32_t po, tf, t, kf;
                    divmod_u32((uint32_t)(tf0 + tid), (uint32_t)TF, prm.magic_tf, po, tf);
                    divmod_u32(tf, (uint32_t)F, prm.magic_f, t, kf);
                    static_cast<float*>(prm.out)[(size_t)tf * (size_t)P + (size_t)(path0 + po)] =
                        icdf_central_f32(q) * __ldg(prm.sqrt_dt32 + t);
                } else {
                    const int slot = atomicAdd(&tail_n, 1);
                    tail_w[slot] = ((unsigned long long)hi << 32) | lo;
                    tail_i[slot] = (short)tid;
                }
            }
            __syncthreads();
            const int n_tail = tail_n;
            for (int k = tid; k < n_tail; k += kRngThreads) {
                const unsigned long long w = tail_w[k];
                const uint32_t hi = (uint32_t)(w >> 32), lo = (uint32_t)w;
                const bool lower = hi < (1u << 25);
                // min(u, 1-u): u itself below 1/2; 1-u = ((2^26-1-hi) 2^26 + (2^26-lo)) 2^-52 above
                const float tp = lower ? fmaf((float)lo, 0x1.0p-52f, (float)hi * 0x1.0p-26f)
                                       : fmaf((float)((1u << 26) - lo), 0x1.0p-52f, (float)((1u << 26) - 1u - hi) * 0x1.0p-26f);
                float x = tp > 0.0f ? icdf_tail_f32(tp) : 0.0f;
                if (lower) x = -x;
                uint32_t po, tf, t, kf;
                divmod_u32((uint32_t)(tf0 + tail_i[k]), (uint32_t)TF, prm.magic_tf, po, tf);
                divmod_u32(tf, (uint32_t)F, prm.magic_f, t, kf);
                static_cast<float*>(prm.out)[(size_t)tf * (size_t)P + (size_t)(path0 + po)] = x * __ldg(prm.sqrt_dt32 + t);
            }
        } else {
            if (tid < kMtN / 2) {
                const int64_t vv = v + tid;
                if (vv < v1) {
                    const uint32_t w1 = mt_temper(nxt[2 * tid]);
                    const uint32_t w2 = mt_temper(nxt[2 * tid + 1]);
                    const int64_t m = (int64_t)(((uint64_t)(w1 >> 6) << 26) | (uint64_t)(w2 >> 6));  // u = m 2^-52
                    if (prm.mode == 0) {
                        static_cast<double*>(prm.out)[vv] = (double)m * 0x1.0p-52;
                    } else {
                        // exact FP64 increments: |u - 1/2| <= 0.425 tested on the integer grid
                        const int64_t dq = m - ((int64_t)1 << 51);
                        if ((dq < 0 ? -dq : dq) <= prm.central_max) {
                            uint32_t po, tf, t, kf;
                            divmod_u32((uint32_t)(tf0 + tid), (uint32_t)TF, prm.magic_tf, po, tf);
                            divmod_u32(tf, (uint32_t)F, prm.magic_f, t, kf);
                            const size_t o = (size_t)tf * (size_t)P + (size_t)(path0 + po);
                            static_cast<double*>(prm.out)[o] = icdf_central((double)dq * 0x1.0p-52) * __ldg(prm.sqrt_dt + t);
                        } else {
                            const int slot = atomicAdd(&tail_n, 1);
                            tail_w[slot] = (unsigned long long)m;
                            tail_i[slot] = (short)tid;
                        }
                    }
                }
            }
            if (prm.mode == 1) {
                __syncthreads();
                const int n_tail = tail_n;
                for (int k = tid; k < n_tail; k += kRngThreads) {
                    const int64_t m = (int64_t)tail_w[k];
                    uint32_t po, tf, t, kf;
                    divmod_u32((uint32_t)(tf0 + tail_i[k]), (uint32_t)TF, prm.magic_tf, po, tf);
                    divmod_u32(tf, (uint32_t)F, prm.magic_f, t, kf);
                    const size_t o = (size_t)tf * (size_t)P + (size_t)(path0 + po);
                    static_cast<double*>(prm.out)[o] = icdf_wichura((double)m * 0x1.0p-52) * __ldg(prm.sqrt_dt + t);
                }
            }
        }
        // advance the (path, value-in-path) position by the 312 values of this round
        tf0 += kMtN / 2;
        if (normals && tf0 >= TF) {
            const int64_t adv = tf0 / TF;
            path0 += adv;
            tf0 -= (int)(adv * TF);
        }
        uint32_t* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

}  // namespace

int plan_mt_generate(int64_t num_values, RngPlan* plan)
{
    static int resident = 0;
    if (!resident) {
        int dev = 0, sms = 0, per_sm = 0;
        LMM_CUDA(cudaGetDevice(&dev));
        LMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        LMM_CUDA(cudaFuncSetAttribute(mt_generate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kJumpWindow * (int)sizeof(uint32_t)));
        LMM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mt_generate_kernel, kRngThreads,
                                                               kJumpWindow * sizeof(uint32_t)));
        resident = sms * (per_sm > 0 ? per_sm : 1);
    }
    // one chunk per resident CTA, at least 4096 values per chunk
    int64_t chunks = resident;
    int64_t chunk_values = (num_values + chunks - 1) / chunks;
    if (chunk_values < 4096) chunk_values = 4096;
    chunks = (num_values + chunk_values - 1) / chunk_values;
    int njumps = 0;
    while (((int64_t)1 << njumps) < chunks) njumps++;
    plan->chunks = chunks;
    plan->chunk_values = chunk_values;
    plan->njumps = njumps;
    plan->polys.clear();
    if (njumps > 0) {
        const std::vector<uint64_t>& v = mt_jump_polynomials(2ull * (uint64_t)chunk_values, njumps);
        plan->polys.assign(v.begin(), v.begin() + (size_t)njumps * kPolyWords);
    }
    return LMM_OK;
}

int launch_mt_generate(const RngLaunch& a, cudaStream_t s, int* num_launches)
{
    if (a.num_values <= 0) return LMM_OK;
    RngParams prm;
    prm.seeded = a.d_seeded;
    prm.jumps = a.d_jumps;
    prm.njumps = a.plan->njumps;
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
    {
        KernelTimer kt(K_MT_JUMP_GENERATE, s);
        mt_generate_kernel<<<(unsigned)a.plan->chunks, kRngThreads, kJumpWindow * sizeof(uint32_t), s>>>(prm);
        LMM_CUDA(cudaGetLastError());
    }
    if (num_launches) (*num_launches)++;
    return LMM_OK;
}

}  // namespace lmm
