// paths_fp64.cuh -- K2 (plain FP64 form): fused Euler-log path kernel.
//
// Reference: EulerSchemeFromProcessModel.doPrecalculateProcess
// (montecarlo/process/EulerSchemeFromProcessModel.java:170-326) with the drift of
// LIBORMarketModelFromCovarianceModel.getDrift (…/models/LIBORMarketModelFromCovarianceModel.java:1125-1191),
// the state-space transforms (:1200-1223) and the spot numeraire (:1017-1074).
//
// One thread owns one path.  Its forward vector lives in registers across all T
// steps; the spot-measure drift is the running sum S_k += L_j/(L_j + 1/delta_j) * lambda_jk
// over alive components j, so a step costs O(N*F) instead of O(N^2*F).  Only the time
// indices that products observe are written, as [slot][component][path] rows (coalesced
// across the warp).  The spot numeraire N(T_l) = prod (1 + L_i(T_i) delta_i) is formed
// at the end from the frozen fixings, and each block writes compensated partial sums
// of 1/N(T_l) for the numeraire adjustment.
//
// Compiled with -fmad=false.  On this GPU an FP64 instruction costs as much pipe time as
// 64 FP32 ones, so the fast kernel keeps in FP64 only what needs FP64's range and
// accuracy -- the forward rates, the exponential of the step and the numeraire -- and moves
// the rest to the FP32 pipe in double-float arithmetic (pairs of floats, about 2^-48
// relative, dfloat.cuh):
//  * the drift's running sums S_k carry dt and the increments dW_k along (G_k = dW_k +
//    dt S_k), as double-float pairs, so that a component costs 2F double-float multiply-adds
//    (Dot2 steps: 12 FP32 instructions each, two factors at once on paired FP32
//    instructions) and no FP64 multiply-add;
//  * L / (L + 1/delta) is the FP32 reciprocal refined by one double-float Newton step;
//  * the Euler-log step exp(log L + d) (EULER_FUNCTIONAL) is evaluated as L exp(d), and the
//    EULER step exp(Y + d) as exp(Y) exp(d) with exp(Y) carried instead of Y, where exp(d)
//    is the table method of exp_small (fp64math.cuh) with its argument reduction and the
//    polynomial of the reduced argument on float pairs (about 2^-48 relative): three FP64
//    instructions per component-step in all (L times the table entry, times the pair);
//  * L and the increments are split into float pairs in integer operations.
// The increment d has an absolute error of a few 1e-16 and exp(r) about 2^-48 relative per
// step, so the states agree with the reference's order to about 1e-13 relative, inside the
// 1e-12 parity bound.  The general
// kernel keeps the reference's literal order throughout (CUDA's exp/log, correctly rounded
// division, unfused).
#pragma once

#include "dfloat.cuh"
#include <cmath>

#include "fp64math.cuh"
#include "lmm_internal.h"
#include "reduce.cuh"
#include "unroll_range.cuh"

namespace lmm {
namespace {

constexpr int kPathThreads = 128;

// a component index known only at run time, for the rolled component loop
struct RuntimeIndex {
    int value;
};

// v capped at the bit pattern capbits of a positive cap: for v >= 0 (exp's range) the IEEE
// order is the integer order of the bit patterns, so the comparison needs no FP64
// instruction (the GPU's FP64 pipe bounds this kernel); NaN stays NaN (Math.min semantics)
__device__ __forceinline__ double cap_positive(double v, long long capbits)
{
    const long long b = __double_as_longlong(v);
    return (b > capbits && b <= 0x7ff0000000000000LL) ? __longlong_as_double(capbits) : v;
}

// the SFU's approximate reciprocal (flush-to-zero; the argument here is L + 1/delta > 0)
__device__ __forceinline__ float rcp_approx_f32(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The forward vector of a path: in registers, or (SMEM) in the thread's own column of a
// shared-memory array [NMAX][threads], which frees NMAX * 2 registers a thread so that more
// warps share an SM and hide the latency of the double-float chains.
template <int NMAX, bool SMEM>
struct PathState;
template <int NMAX>
struct PathState<NMAX, false> {
    double v[NMAX];
    __device__ __forceinline__ double& operator[](int j) { return v[j]; }
};
template <int NMAX>
struct PathState<NMAX, true> {
    double* col;
    __device__ __forceinline__ double& operator[](int j) { return col[j * kPathThreads]; }
};

// the shared-memory state for up to 40 components (40 KB a block, five blocks an SM)
__host__ __device__ constexpr bool fp64_state_in_smem(int nmax, bool functional) { return functional && nmax <= 40; }
__host__ __device__ constexpr int fp64_min_blocks(int nmax, bool functional)
{
    return fp64_state_in_smem(nmax, functional) ? 5 : 1;
}

// EXACT: the model has exactly NMAX components, so the component loop carries no bound
// checks.  With the state in registers the loop enters its unrolled sequence at the first
// alive component through a jump table (unroll_range.cuh); with the state in shared memory
// it is a rolled loop.
// REPLAY: the adjoint's replay of the steps [rp_n0, rp_n_stop) from the checkpoint rp_ckpt,
// with the same step code, so that the replayed forward rates equal the stored ones bit for
// bit; it writes the rates of every step of the segment (components below rp_n_eff) and no
// numeraire.  EULER (not FUNCTIONAL) restarts exp(Y) from the stored rate: exact when
// uncapped only.
template <int NMAX, int FMAX, bool FUNCTIONAL, bool EXACT, bool REPLAY = false>
__global__ void __launch_bounds__(kPathThreads, fp64_min_blocks(NMAX, FUNCTIONAL)) paths_fp64_kernel(const PathLaunch a)
{
    static_assert(FMAX % 2 == 0, "factors run in pairs");
    constexpr int FPD = fp64_df_pitch(FMAX);
    constexpr bool SMEM = fp64_state_in_smem(NMAX, FUNCTIONAL);
    const int p = blockIdx.x * kPathThreads + threadIdx.x;
    const bool active = p < a.P;
    const int N = EXACT ? NMAX : a.N, F = a.F, P = a.P;
    const long long capbits = __double_as_longlong(a.libor_cap);  // +infinity when uncapped: never caps
    const double* dW = static_cast<const double*>(a.d_dw);
    double* states = static_cast<double*>(a.d_states);

    // exp(k/128), |k| <= 128, in shared memory: every 2nd entry of the exp(k/256) table.  The
    // lanes of a warp gather about twenty distinct entries a component-step; from the L1,
    // beside the shared-memory state, those gathers kept missing
    constexpr int kExpHalf = 128;
    static_assert(kExpTableHalf % kExpHalf == 0, "the shared table takes every n-th entry");
    __shared__ double etab_s[2 * kExpHalf + 1];
    for (int q = threadIdx.x; q <= 2 * kExpHalf; q += kPathThreads)
        etab_s[q] = __ldg(a.d_exp_tab + kExpTableHalf + (q - kExpHalf) * (kExpTableHalf / kExpHalf));
    __syncthreads();
    __shared__ double state_smem[SMEM ? NMAX : 1][kPathThreads];
    PathState<NMAX, SMEM> L;
    if constexpr (SMEM) L.col = &state_smem[0][threadIdx.x];
    double E[FUNCTIONAL ? 1 : NMAX];  // EULER: exp of the uncapped log state Y
    if constexpr (REPLAY) {
#pragma unroll
        for (int j = 0; j < NMAX; j++) {
            const double v = (j < N && active) ? a.rp_ckpt[(size_t)j * P + p] : 0.0;
            L[j] = v;
            if (!FUNCTIONAL) E[FUNCTIONAL ? 0 : j] = v;
            if (j < a.rp_n_eff && active) a.rp_seg[(size_t)j * P + p] = v;
        }
    }
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        if (REPLAY) break;
        if (j < N) {
            // getInitialState (:1081-1093) and applyStateSpaceTransform (:1200-1212):
            // exp(log(max(f,0))), the same for every path, from the host
            const double e0 = __ldg(a.d_init_state + j);
            L[j] = cap_positive(e0, capbits);
            if (!FUNCTIONAL) E[FUNCTIONAL ? 0 : j] = e0;
        } else {
            L[j] = 0.0;
        }
    }
    if (!REPLAY) {
        const int slot = __ldg(a.d_obs_slot + 0);
        if (slot >= 0 && active) {
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) states[((size_t)slot * N + j) * P + p] = L[j];
        }
        if (a.d_ckpt && active) {
            double* ck = static_cast<double*>(a.d_ckpt);
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) ck[(size_t)j * P + p] = L[j];
        }
    }

    const int i_end = REPLAY ? a.rp_n_stop : a.T;
    for (int i = REPLAY ? a.rp_n0 : 0; i < i_end; i++) {
        const int first = __ldg(a.d_first + i);
        const float dth = __ldg(a.d_dt_df + 2 * i), dtl = __ldg(a.d_dt_df + 2 * i + 1);
        const float4* rows = reinterpret_cast<const float4*>(a.d_rows_df + (size_t)i * N * FPD);
        // G_k = dW_k + dt S_k with the drift's running sum S_k = sum_{l<=j} os_l lambda_lk
        // (:1156-1158), carried as double-float pairs (Gp + Gs): the step increment of
        // component j is then  d_j = mu_j dt + sum_k dW_k lambda_jk = sum_k G_k lambda_jk
        // - dt variance_j / 2, two double-float multiply-adds per factor on the FP32 pipe
        // factor pairs (2m, 2m+1) side by side in the lanes of float2 registers
        // (the increments, read once, bypass the L1, which keeps the component rows)
        float2 Gh[FMAX / 2], Gl[FMAX / 2];
#pragma unroll
        for (int m = 0; m < FMAX / 2; m++) {
            float h0 = 0.0f, l0 = 0.0f, h1 = 0.0f, l1 = 0.0f;
            if (2 * m < F && active) df_split_int(__ldcg(dW + ((size_t)i * F + 2 * m) * P + p), h0, l0);
            if (2 * m + 1 < F && active) df_split_int(__ldcg(dW + ((size_t)i * F + 2 * m + 1) * P + p), h1, l1);
            Gh[m] = make_float2(h0, h1);
            Gl[m] = make_float2(l0, l1);
        }
        // the next step's component rows into this SM's L1 (one 128-byte line per thread; the
        // first warp of every SM to reach a step would otherwise wait on their L2 round trips)
        // and this path's next increments into L2
        if (i + 1 < i_end) {
            const int row_lines = (N * FPD * (int)sizeof(float) + 127) / 128;
            const char* nrows = reinterpret_cast<const char*>(a.d_rows_df + (size_t)(i + 1) * N * FPD);
            for (int q = threadIdx.x; q < row_lines; q += kPathThreads)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(nrows + 128 * q));
            if (active)
                for (int k = 0; k < F; k++)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(dW + ((size_t)(i + 1) * F + k) * P + p));
        }
        auto component_step = [&](auto jc) {
            const int j = jc.value;
            if (EXACT || j < N) {
                // the component's row: loadings (hi, lo), the drift term (variance * -0.5) * dt
                // and 1/delta, each as a double-float pair
                float r[FPD];
#pragma unroll
                for (int q = 0; q < FPD / 4; q++) {
                    const float4 v = __ldg(rows + j * (FPD / 4) + q);
                    r[4 * q] = v.x;
                    r[4 * q + 1] = v.y;
                    r[4 * q + 2] = v.z;
                    r[4 * q + 3] = v.w;
                }
                const double Lj = L[j];
                // os = L / (L + 1/delta) (Scalar(delta).discount(L, delta) times L, :1149-1153):
                // the FP32 reciprocal of L + 1/delta refined by one double-float Newton step
                // (about 2^-44 relative; os enters only the drift, a small part of d)
                float Lh, Ll;
                df_split_int(Lj, Lh, Ll);
                float xh, xl;
                two_sum(Lh, r[2 * FMAX + 2], xh, xl);
                xl = xl + (Ll + r[2 * FMAX + 3]);
                const float r0 = rcp_approx_f32(xh);
                const float ph = __fmul_rn(xh, r0);
                float pe = fmaf(xh, r0, -ph);
                pe = fmaf(xl, r0, pe);
                const float er = (1.0f - ph) - pe;
                const float r1 = __fmul_rn(r0, er);
                const float oh = __fmul_rn(Lh, r0);
                float oe = fmaf(Lh, r0, -oh);
                oe = fmaf(Lh, r1, oe);
                oe = fmaf(Ll, r0, oe);
                // os dt
                const float qh = __fmul_rn(oh, dth);
                float qe = fmaf(oh, dth, -qh);
                qe = fmaf(oh, dtl, qe);
                qe = fmaf(oe, dth, qe);
                // Euler step (EulerSchemeFromProcessModel.java:235-255) with the drift of
                // :1159 and :1183-1189: the increment d of the log state.  Two accumulators,
                // even factors in lane x (started at the drift term) and odd ones in lane y, on
                // paired instructions; the rows are zero beyond F, so padded factors add 0
                float2 acc_h = make_float2(r[2 * FMAX], 0.0f), acc_l = make_float2(r[2 * FMAX + 1], 0.0f);
                const float2 q2h = make_float2(qh, qh), q2l = make_float2(qe, qe);
#pragma unroll
                for (int m = 0; m < FMAX / 2; m++) {
                    const float2 bh = make_float2(r[2 * m], r[2 * m + 1]);
                    const float2 bl = make_float2(r[FMAX + 2 * m], r[FMAX + 2 * m + 1]);
                    const float2 bn = __fmul2_rn(bh, make_float2(-1.0f, -1.0f));
                    df_dot_acc2(Gh[m], Gl[m], q2h, q2l, bh, bl, bn);      // G_k += os dt lambda_k
                    df_dot_acc2(acc_h, acc_l, Gh[m], Gl[m], bh, bl, bn);  // d += G_k lambda_k
                }
                const float dp = acc_h.x, ep = acc_h.y, ds = acc_l.x, es = acc_l.y;
                // exp(d) by the table method of exp_small (fp64math.cuh) with k = rint(128 d):
                // the remainder r = rh + dl, rh = dh - k/128 (|rh| <= 1/256, exact in FP32),
                // and exp(r) = 1 + r + r^2 B, B = 1/2 + rh/6 + rh^2/24 + rh^3/120 + dl/2
                // (dl/2: the low part's first-order share of r^3/6, up to 2^-44 with this
                // table; truncation below 2^-57), as a float pair s + low (B - 1/2 in FP32: it
                // enters times r^2 <= 2^-16); then L exp(k/128) (s + low) in three FP64
                // instructions
                float dh, dl;
                {
                    float x, q;
                    two_sum(dp, ep, x, q);
                    two_sum(x, (ds + es) + q, dh, dl);
                }
                const double base = FUNCTIONAL ? Lj : E[FUNCTIONAL ? 0 : j];
                double nv;
                if (fabsf(dh) <= 1.0f) {
                    const float t = fmaf(dh, (float)kExpHalf, 12582912.0f);  // 1.5 2^23 + rint(128 dh)
                    const int kk = __float_as_int(t) - 0x4b400000;
                    const float rh = fmaf(-(t - 12582912.0f), 1.0f / kExpHalf, dh);  // exact
                    const float r2h = __fmul_rn(rh, rh);
                    const float r2e = fmaf(rh, rh, -r2h) + (rh + rh) * dl;  // r^2 - r2h
                    const float bt = fmaf(dl, 0.5f, rh * fmaf(rh, fmaf(rh, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f));
                    const float th = 0.5f * r2h;                      // exact
                    const float tl = fmaf(r2h, bt, 0.5f * r2e);
                    const float s1 = 1.0f + rh;                       // |1| >= |rh|: fast TwoSum
                    const float e1 = rh - (s1 - 1.0f);
                    const float s2 = s1 + th;
                    const float e2 = th - (s2 - s1);
                    const float low = (e1 + e2) + (dl + tl);
                    const double scaled = base * etab_s[kExpHalf + kk];  // L exp(k/128)
                    nv = fma(scaled, f32_to_f64_nz(low), scaled * f32_to_f64_nz(s2));
                } else {
                    nv = base * exp(df_to_double(dh, dl));
                }
                // then L exp(d) (FUNCTIONAL: log L is the state) or exp(Y) exp(d) (EULER)
                if (!FUNCTIONAL) E[FUNCTIONAL ? 0 : j] = nv;
                L[j] = cap_positive(nv, capbits);
            }
        };
        if constexpr (SMEM) {
            // the state lives in shared memory: a rolled loop keeps the step's code inside the
            // instruction cache (the unrolled sequence of 40 components did not fit, and its
            // instruction-fetch stalls cost a third of the kernel's time); two components per
            // iteration let the compiler overlap one's exponential with the next one's sums
#pragma unroll 2
            for (int j = first; j < N; j++) component_step(RuntimeIndex{j});
        } else {
            for_up_from<NMAX>(first, component_step);
        }
        if constexpr (REPLAY) {
            if (active) {
                double* out = a.rp_seg + (size_t)(i + 1 - a.rp_n0) * N * P + p;
#pragma unroll
                for (int j = 0; j < NMAX; j++)
                    if (j < a.rp_n_eff) out[(size_t)j * P] = L[j];
            }
            continue;
        }
        const int slot = __ldg(a.d_obs_slot + i + 1);
        if (slot >= 0 && active) {
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) states[((size_t)slot * N + j) * P + p] = L[j];
        }
        if (a.d_ckpt && active && (i + 1) % a.ckpt_stride == 0) {
            double* ck = static_cast<double*>(a.d_ckpt) + (size_t)((i + 1) / a.ckpt_stride) * N * P;
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) ck[(size_t)j * P + p] = L[j];
        }
    }
    if constexpr (REPLAY) return;

    // Spot numeraire from the frozen fixings L_l(T_l) (:1050-1066): Scalar.accrue while
    // the numeraire is deterministic, RandomVariableFromDoubleArray.accrue afterwards.  The
    // numeraire adjustment's input, mean of N(T)^-1 * N(0) (:869-874), from 1/N by a Newton
    // reciprocal (within an ulp of the division) summed in plain FP64 within each warp
    // (transposed reductions over chunks of eight tenor times) and compensated across warps.
    static_assert(NMAX % 8 == 0, "the transposed reduction works on chunks of eight tenor times");
    __shared__ double wsum[kPathThreads / 32][NMAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double Nv = 1.0;
    if (active) a.d_numeraire[p] = 1.0;
    if (a.d_inv_numeraire && active) a.d_inv_numeraire[p] = 1.0;
#pragma unroll
    for (int c = 0; c < NMAX / 8; c++) {
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int l = 8 * c + q;
            v[q] = 0.0;
            if (l < N) {
                const double delta = __ldg(a.d_delta + l);
                if (l < a.num_det_prefix) Nv = L[l] * (delta * Nv) + Nv;
                else Nv = Nv * (1.0 + L[l] * delta);
                if (active) {
                    a.d_numeraire[(size_t)(l + 1) * P + p] = Nv;
                    v[q] = rcp_newton(Nv);
                    if (a.d_inv_numeraire) a.d_inv_numeraire[(size_t)(l + 1) * P + p] = v[q];
                }
            }
        }
        const double sum = warp_sum8_transposed(v, lane);
        const int idx = 8 * c + ((lane >> 2) & 7);
        if ((lane & 3) == 0 && idx < N) wsum[warp][idx] = sum;
    }
    __syncthreads();
    if ((int)threadIdx.x < N) {
        dd acc{0.0, 0.0};
#pragma unroll
        for (int w = 0; w < kPathThreads / 32; w++) acc = dd_add_d(acc, wsum[w][threadIdx.x]);
        double* o = a.d_inv_num_partials + ((size_t)blockIdx.x * N + threadIdx.x) * 2;
        o[0] = acc.hi;
        o[1] = acc.lo;
    }
}

// ------------------------------------------------------------------ general form
// The rarely used forms (predictor-corrector schemes, TERMINAL measure, NORMAL state space)
// run one kernel with run-time switches.  Its component loops are rolled (the per-path
// vectors live in thread-local memory): it is the coverage path, kept small to compile.
//
// getDrift (LIBORMarketModelFromCovarianceModel.java:1125-1191) for any measure and state
// space: SPOT sums the one-step transforms of l <= j (updated before j reads them), TERMINAL
// those of l > j (walking down, read before j adds to them); LOGNORMAL multiplies the
// transform by L and adds -variance/2.  Scalar(+-delta).discount(L, delta) =
// 1/(L (delta/(+-delta)) + 1/(+-delta)) (stochastic/Scalar.java:321-328).
template <int FMAX>
__device__ void drift_general(const PathLaunch& a, int i, int first, const double* L, double* mu)
{
    const int N = a.N, F = a.F;
    const double* lam = a.d_loadings + (size_t)i * N * F;
    const bool lognormal = a.state_space == 0;
    const bool spot = a.measure == 0;
    double S[FMAX];
#pragma unroll
    for (int k = 0; k < FMAX; k++) S[k] = 0.0;
#pragma unroll 1
    for (int c = 0; c < N - first; c++) {
        const int j = spot ? first + c : N - 1 - c;
        const double delta = __ldg(a.d_delta + j);
        double os = spot ? 1.0 / (L[j] * (delta / delta) + 1.0 / delta) : 1.0 / (L[j] * (delta / -delta) + 1.0 / -delta);
        if (lognormal) os = os * L[j];
        const double* lj = lam + (size_t)j * F;
        double d = 0.0;
        if (spot) {
#pragma unroll
            for (int k = 0; k < FMAX; k++)
                if (k < F) S[k] = S[k] + os * __ldg(lj + k);
#pragma unroll
            for (int k = 0; k < FMAX; k++)
                if (k < F) d = d + S[k] * __ldg(lj + k);
        } else {
#pragma unroll
            for (int k = 0; k < FMAX; k++)
                if (k < F) d = d + S[k] * __ldg(lj + k);
#pragma unroll
            for (int k = 0; k < FMAX; k++)
                if (k < F) S[k] = S[k] + os * __ldg(lj + k);
        }
        if (lognormal) d = d + __ldg(a.d_variance + (size_t)i * N + j) * -0.5;
        mu[j] = d;
    }
}

// applyStateSpaceTransform (:1200-1212): exp for LOGNORMAL, then the cap
__device__ __forceinline__ double transform_general(const PathLaunch& a, double y)
{
    double v = a.state_space == 0 ? exp(y) : y;
    if (!isinf(a.libor_cap) && v > a.libor_cap) v = a.libor_cap;
    return v;
}

// TERMINAL numeraire at tenor index l from the state at the time of T_l
// (getNumerairetUnAdjustedAtLIBORIndex :1029-1048): Scalar.discount steps while deterministic,
// RandomVariableFromDoubleArray.discount (x / (1 + L delta), :1308-1333) afterwards
__device__ double terminal_numeraire(const PathLaunch& a, int l, const double* L, bool deterministic)
{
    double x = 1.0;
#pragma unroll 1
    for (int k = l; k < a.N; k++) {
        const double delta = __ldg(a.d_delta + k);
        if (deterministic || k == l) x = 1.0 / (L[k] * (delta / x) + 1.0 / x);
        else x = x / (1.0 + L[k] * delta);
    }
    return x;
}

// The Euler scheme (EulerSchemeFromProcessModel.java:170-326) for any scheme, measure and state
// space: the predictor-corrector step adds ((mu(predictor) - mu)/2) dt to the state and
// transforms again (:292-314).
template <int NMAX, int FMAX>
__global__ void __launch_bounds__(kPathThreads) paths_fp64_general_kernel(const PathLaunch a)
{
    const int p = blockIdx.x * kPathThreads + threadIdx.x;
    const bool active = p < a.P;
    const int N = a.N, F = a.F, P = a.P;
    const bool functional = a.scheme == 1 || a.scheme == 3;
    const bool pc = a.scheme == 2 || a.scheme == 3;
    const bool lognormal = a.state_space == 0;
    const bool terminal = a.measure == 1;
    const double* dW = static_cast<const double*>(a.d_dw);
    double* states = static_cast<double*>(a.d_states);
    double L[NMAX], Y[NMAX], mu0[NMAX], mu1[NMAX], Ln[NMAX];
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        const double f = __ldg(a.d_init + j);
        Y[j] = lognormal ? log(f > 0.0 ? f : 0.0) : f;
        L[j] = transform_general(a, Y[j]);
    }
    {
        const int slot = __ldg(a.d_obs_slot + 0);
        if (slot >= 0 && active)
            for (int j = 0; j < N; j++) states[((size_t)slot * N + j) * P + p] = L[j];
        if (a.d_ckpt && active)
            for (int j = 0; j < N; j++) static_cast<double*>(a.d_ckpt)[(size_t)j * P + p] = L[j];
        if (terminal && active)
            for (int l = 0; l <= N; l++)
                if (__ldg(a.d_tenor_tidx + l) == 0) a.d_numeraire[(size_t)l * P + p] = terminal_numeraire(a, l, L, true);
    }
#pragma unroll 1
    for (int i = 0; i < a.T; i++) {
        const int first = __ldg(a.d_first + i);
        const double dt = __ldg(a.d_dt + i);
        const double* lam = a.d_loadings + (size_t)i * N * F;
        double dw[FMAX];
#pragma unroll
        for (int k = 0; k < FMAX; k++) dw[k] = (k < F && active) ? dW[((size_t)i * F + k) * P + p] : 0.0;
        drift_general<FMAX>(a, i, first, L, mu0);
#pragma unroll 1
        for (int j = 0; j < N; j++) {
            Ln[j] = L[j];
            if (j >= first) {
                double y = functional ? (lognormal ? log(L[j]) : L[j]) : Y[j];
                y = y + mu0[j] * dt;
#pragma unroll
                for (int k = 0; k < FMAX; k++)
                    if (k < F) y = y + dw[k] * __ldg(lam + (size_t)j * F + k);
                Y[j] = y;
                Ln[j] = transform_general(a, y);
            }
        }
        if (pc) {
            drift_general<FMAX>(a, i, first, Ln, mu1);
#pragma unroll 1
            for (int j = first; j < N; j++) {
                Y[j] = Y[j] + ((mu1[j] - mu0[j]) / 2.0) * dt;
                Ln[j] = transform_general(a, Y[j]);
            }
        }
#pragma unroll 1
        for (int j = 0; j < N; j++) L[j] = Ln[j];
        const int slot = __ldg(a.d_obs_slot + i + 1);
        if (slot >= 0 && active)
            for (int j = 0; j < N; j++) states[((size_t)slot * N + j) * P + p] = L[j];
        if (a.d_ckpt && active && (i + 1) % a.ckpt_stride == 0) {
            double* ck = static_cast<double*>(a.d_ckpt) + (size_t)((i + 1) / a.ckpt_stride) * N * P;
            for (int j = 0; j < N; j++) ck[(size_t)j * P + p] = L[j];
        }
        if (terminal && active)
            for (int l = 0; l <= N; l++)
                if (__ldg(a.d_tenor_tidx + l) == i + 1) a.d_numeraire[(size_t)l * P + p] = terminal_numeraire(a, l, L, false);
    }
    if (!terminal) {
        // SPOT numeraire from the frozen fixings (as paths_fp64_kernel)
        double Nv = 1.0;
        if (active) a.d_numeraire[p] = 1.0;
#pragma unroll 1
        for (int l = 0; l < N; l++) {
            const double delta = __ldg(a.d_delta + l);
            if (l < a.num_det_prefix) Nv = L[l] * (delta * Nv) + Nv;
            else Nv = Nv * (1.0 + L[l] * delta);
            if (active) a.d_numeraire[(size_t)(l + 1) * P + p] = Nv;
        }
    } else if (active && __ldg(a.d_tenor_tidx + N) > a.T) {
        a.d_numeraire[(size_t)N * P + p] = 1.0;
    }
    // block partials of N(T_l)^-1 * N(0) for the numeraire adjustment (:869-874), and 1/N
    // per path for the products
    const double N0 = active ? a.d_numeraire[p] : 1.0;
    if (a.d_inv_numeraire && active) a.d_inv_numeraire[p] = 1.0 / N0;
#pragma unroll 1
    for (int l = 1; l <= N; l++) {
        const double r = active ? 1.0 / a.d_numeraire[(size_t)l * P + p] : 0.0;
        if (a.d_inv_numeraire && active) a.d_inv_numeraire[(size_t)l * P + p] = r;
        block_dd_partial(active ? r * N0 : 0.0, a.d_inv_num_partials + ((size_t)blockIdx.x * N + (l - 1)) * 2);
    }
}

// the fast kernel's template choice of launch_t, as a replay; kReplayNotFast where the
// forward simulation ran another kernel (or EULER with a cap)
template <int NMAX, int FMAX>
int replay_t(const PathLaunch& a, cudaStream_t s, int blocks)
{
    if (a.scheme > 1 || a.measure != 0 || a.state_space != 0) return kReplayNotFast;
    if (a.scheme == 1 && a.N == NMAX)
        paths_fp64_kernel<NMAX, FMAX, true, true, true><<<blocks, kPathThreads, 0, s>>>(a);
    else if (a.scheme == 1)
        paths_fp64_kernel<NMAX, FMAX, true, false, true><<<blocks, kPathThreads, 0, s>>>(a);
    else if (std::isinf(a.libor_cap) && a.libor_cap > 0.0)
        paths_fp64_kernel<NMAX, FMAX, false, false, true><<<blocks, kPathThreads, 0, s>>>(a);
    else
        return kReplayNotFast;
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <int NMAX, int FMAX>
int launch_general(const PathLaunch& a, cudaStream_t s, int blocks)
{
    paths_fp64_general_kernel<NMAX, FMAX><<<blocks, kPathThreads, 0, s>>>(a);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <int NMAX, int FMAX>
int launch_t(const PathLaunch& a, cudaStream_t s, int blocks)
{
    if (a.scheme > 1 || a.measure != 0 || a.state_space != 0)
        paths_fp64_general_kernel<NMAX, FMAX><<<blocks, kPathThreads, 0, s>>>(a);
    else if (a.scheme == 1 && a.N == NMAX)
        paths_fp64_kernel<NMAX, FMAX, true, true><<<blocks, kPathThreads, 0, s>>>(a);
    else if (a.scheme == 1)
        paths_fp64_kernel<NMAX, FMAX, true, false><<<blocks, kPathThreads, 0, s>>>(a);
    else
        paths_fp64_kernel<NMAX, FMAX, false, false><<<blocks, kPathThreads, 0, s>>>(a);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

}  // namespace
}  // namespace lmm
