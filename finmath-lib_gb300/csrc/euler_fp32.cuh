// euler_fp32.cuh -- the mixed-precision form's Euler-log component step, shared by the FP32
// path kernel (paths_fp32.cu) and the adjoint's replay of the steps between checkpoints
// (adjoint.cu), so that a replayed forward rate is bit for bit the one the path kernel stored.
//
// EulerSchemeFromProcessModel.java:235-255 in its EULER_FUNCTIONAL form with the spot drift
// of LIBORMarketModelFromCovarianceModel.java:1125-1191, carried on the forward rate itself:
// L' = min(L exp(d), cap), d = sum_k G_k lambda_jk - dt variance_j / 2, with the drift's
// running sums G_k = dW_k + dt S_k, S_k = sum_{l<=j} os_l lambda_lk, in base-2 units (G and
// dt carry log2 e, so exp(d) = exp2(d')).
#pragma once

namespace lmm {
namespace euler32 {

constexpr float kLog2e = 1.4426950408889634f;

// row pitch of a step's component rows: FMAX loadings (zero padded), the drift term
// (variance * -0.5 * dt, times log2 e) and 1/delta, rounded up to whole float4 vectors
__host__ __device__ constexpr int row_pitch(int fmax) { return (fmax + 2 + 3) / 4 * 4; }

// The SFU's approximate reciprocal and base-2 exponential with flush-to-zero, one MUFU
// instruction each: the arguments here (L + 1/delta in (0, 1e5 + 2], and the step
// increment times log2 e) are normal numbers far from the range edges that __fdividef and
// __expf guard with extra compares, selects and scalings.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float exp2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// dt of step i in base-2 units
__device__ __forceinline__ float step_dt(const float* dt32, int i) { return __ldg(dt32 + i) * kLog2e; }

// the step's running sums at the start of the component loop: the increments of factors
// (2m, 2m+1) in base-2 units (zero for absent factors)
__device__ __forceinline__ float2 start_sum(float dw0, float dw1) { return __fmul2_rn(make_float2(dw0, dw1), make_float2(kLog2e, kLog2e)); }

// One component-step: Lj the component's rate, lr its row, dt the step's dt in base-2 units,
// G the running sums (updated with this component's os dt lambda).  The sums over factors run
// on paired FMAs, the dot product in two accumulators (even and odd factor pairs).
template <int FMAX, bool CAPPED>
__device__ __forceinline__ float component_step(float Lj, const float (&lr)[row_pitch(FMAX)], float dt,
                                                float2 (&G2)[(FMAX + 1) / 2], float cap)
{
    constexpr int FH = (FMAX + 1) / 2;
    const float osdt = (Lj * dt) * rcp_approx(Lj + lr[FMAX + 1]);
    const float2 os2 = make_float2(osdt, osdt);
    float2 da, db = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int m = 0; m < FH; m++) {
        // factors 2m and 2m+1 (the rows are zero padded beyond F; for an odd FMAX the last
        // pair's second entry is the drift term, multiplied by G = 0)
        const float2 l2 = make_float2(lr[2 * m], 2 * m + 1 < FMAX ? lr[2 * m + 1] : 0.0f);
        G2[m] = __ffma2_rn(os2, l2, G2[m]);
        if (m == 0) da = __fmul2_rn(G2[m], l2);
        else if (m == 1) db = __fmul2_rn(G2[m], l2);
        else if (m & 1) db = __ffma2_rn(G2[m], l2, db);
        else da = __ffma2_rn(G2[m], l2, da);
    }
    const float2 s2 = __fadd2_rn(da, db);
    float v = Lj * exp2_approx((s2.x + s2.y) + lr[FMAX]);
    if (CAPPED) v = fminf(v, cap);
    return v;
}

}  // namespace euler32
}  // namespace lmm
