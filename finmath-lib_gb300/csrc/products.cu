// products.cu -- numeraire adjustment (K3), European swaption, Bermudan backward induction
// with regression (K4/K5) and the compensated mean / standard error of per-path values.
//
// References (finmath-lib, src/main/java/net/finmath/):
//   LIBORMarketModelFromCovarianceModel.getNumeraire            …/models/LIBORMarketModelFromCovarianceModel.java:860-876
//   Swaption.getValue                                           montecarlo/interestrate/products/Swaption.java:137-199
//   BermudanSwaption.getValues / getBasisFunctions              montecarlo/interestrate/products/BermudanSwaption.java:91-157, 215-252
//   MonteCarloConditionalExpectationRegression                  montecarlo/conditionalexpectation/MonteCarloConditionalExpectationRegression.java:98-150
//   RandomVariableFromDoubleArray.getAverage / getStandardError montecarlo/RandomVariableFromDoubleArray.java:287-308, 332-354, 419-428
//
// Compiled with -fmad=false (unfused FP64, as the reference's Java).
#include "lmm_internal.h"
#include "reduce.cuh"
#include "exact_sum.cuh"

#include <math_constants.h>
#include <cstring>
#include <mutex>

namespace lmm {
namespace {

constexpr int kProdThreads = 256;
constexpr int kMaxN = kMaxForwardRates;

struct NumeraireInfo {
    int P;
    int has_discount;
    const double* numeraire;   // [N+1][P] unadjusted
    const double* adj;         // [N+1] mean of 1/N (device)
    const double* inv_numeraire;  // [N+1][P] 1/N from the path kernel (or nullptr)
    double pd[kMaxN + 1];      // P^d(T_l)
    double inv_pd[kMaxN + 1];  // 1 / P^d(T_l)
    unsigned char det[kMaxN + 1];
};

// getNumeraire(T_l) including the discount-curve adjustment (:869-874).
__device__ __forceinline__ double numeraire_adj(const NumeraireInfo& n, int l, int p)
{
    const double Nu = n.numeraire[(size_t)l * n.P + p];
    if (!n.has_discount) return Nu;
    const double a = n.adj[l];
    if (n.det[l]) return (1.0 / n.pd[l]) * (Nu * a);  // Scalar.div: invert, then mult
    return (Nu * a) / n.pd[l];
}

template <typename TS>
__device__ __forceinline__ double state_at(const void* states, int slot, int N, int P, int j, int p)
{
    return (double)static_cast<const TS*>(states)[((size_t)slot * N + j) * P + p];
}

// ------------------------------------------------------------------ numeraire adjustment
__global__ void numeraire_finish_kernel(const double* partials, int blocks, int N, int P, const double* numeraire,
                                        const uint8_t* det, double* adj)
{
    const int l = blockIdx.x;  // numeraire index 0..N
    if (l > N) return;
    if (det[l]) {
        // N(T)^-1 * N(0) of a deterministic numeraire (N(0) = 1 under SPOT)
        if (threadIdx.x == 0) adj[l] = numeraire[0] * (1.0 / numeraire[(size_t)l * P]);
        return;
    }
    dd acc{0.0, 0.0};
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) {
        const double* q = partials + ((size_t)b * N + (l - 1)) * 2;
        acc = dd_add(acc, dd{q[0], q[1]});
    }
    acc = block_dd_sum(acc);
    if (threadIdx.x == 0) adj[l] = (acc.hi + acc.lo) / (double)P;
}

// ------------------------------------------------------------------ mean / standard error
__global__ void sum_partials_kernel(const double* x, int P, const double* center, double* partials)
{
    dd acc{0.0, 0.0};
    const double m = center ? *center : 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const double v = center ? (x[p] - m) * (x[p] - m) : x[p];
        acc = dd_add_d(acc, v);
    }
    acc = block_dd_sum(acc);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = acc.hi;
        partials[2 * blockIdx.x + 1] = acc.lo;
    }
}

__global__ void finish_partials_kernel(const double* partials, int blocks, int P, double* out)
{
    dd acc{0.0, 0.0};
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) acc = dd_add(acc, dd{partials[2 * b], partials[2 * b + 1]});
    acc = block_dd_sum(acc);
    if (threadIdx.x == 0) *out = (acc.hi + acc.lo) / (double)P;
}

// ------------------------------------------------------------------ swaption
struct SwaptionParams {
    SwaptionLaunch s;
    NumeraireInfo num;
    const void* states;
    int N, P, fp32;
    double* values;
};

template <typename TS>
__global__ void __launch_bounds__(kProdThreads) swaption_kernel(const SwaptionParams a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    const double w = 1.0 / (double)a.P;
    double v = 0.0;
    for (int per = a.s.nper - 1; per >= 0; per--) {
        const double L = state_at<TS>(a.states, a.s.period_slot[per], a.N, a.P, a.s.period_index[per], p);
        const double payoff = ((L - a.s.strike[per]) * a.s.period_length[per]) * a.s.notional;
        v = v + payoff;
        v = v / (1.0 + L * a.s.disc_dt[per]);
        v = v * 1.0;
    }
    double x = isnan(v) ? v : (v > 0.0 ? v : 0.0);
    x = x / numeraire_adj(a.num, a.s.num_index, p);
    x = x * w;
    x = x * numeraire_adj(a.num, 0, 0);  // numeraire at evaluation time 0 (exactly 1 under SPOT)
    x = x / w;
    a.values[p] = x;
}

// ------------------------------------------------------------------ European products' adjoint seeds
// Per path the value V = payoff N(0) / N_adj(T_l) of a swaption (kind 0: Swaption.getValue's
// backward recursion U <- (U + A_q) / (1 + L_q tau_q) over the forwards read at the exercise
// slot, floored at 0) or a caplet (kind 1: max(L_m(T_m) - K, 0) times the day count fraction,
// paid at T_{m+1}), and its derivative to every state of the observation slot: through the
// payoff, and through the numeraire N(T_l) = prod_{k<l} (1 + d_k L_k(T_k)) whose adjustment
// factor a_l / P^d_l is held constant.  The recursion's adjoint runs forward over the
// periods: with D_q = 1 + L_q tau_q and U_q the value after period q,
//   dU_q / dL_q = (len_q notional - U_q tau_q) / D_q,   Ubar_{q+1} = Ubar_q / D_q.
struct EuroSeedParams {
    SwaptionLaunch s;
    CapletSeed c;
    int kind, N, P, num_index, state_slot;
    NumeraireInfo num;
    const double* states;
    double delta[kMaxN];
    double* seeds;  // [N][P]: d V_p / d L_j / P
};

__global__ void __launch_bounds__(kProdThreads) european_seed_kernel(const EuroSeedParams a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    double g[kMaxN];
#pragma unroll 1
    for (int j = 0; j < a.N; j++) g[j] = 0.0;
    const double scale = numeraire_adj(a.num, 0, 0) / numeraire_adj(a.num, a.num_index, p);  // N(0) / N_adj(T_l)
    double V;
    if (a.kind == 0) {
        double vout[kMaxN];
        double v = 0.0;
#pragma unroll 1
        for (int per = a.s.nper - 1; per >= 0; per--) {
            const double L = state_at<double>(a.states, a.s.period_slot[per], a.N, a.P, a.s.period_index[per], p);
            const double payoff = ((L - a.s.strike[per]) * a.s.period_length[per]) * a.s.notional;
            v = v + payoff;
            v = v / (1.0 + L * a.s.disc_dt[per]);
            vout[per] = v;
        }
        V = (v > 0.0 ? v : 0.0) * scale;
        double ub = (v >= 0.0 ? 1.0 : 0.0) * scale;
#pragma unroll 1
        for (int per = 0; per < a.s.nper; per++) {
            const double L = state_at<double>(a.states, a.s.period_slot[per], a.N, a.P, a.s.period_index[per], p);
            const double D = 1.0 + L * a.s.disc_dt[per];
            g[a.s.period_index[per]] += ub * (a.s.period_length[per] * a.s.notional - vout[per] * a.s.disc_dt[per]) / D;
            ub = ub / D;
        }
    } else {
        const double L = state_at<double>(a.states, a.c.slot, a.N, a.P, a.c.index, p);
        const double x = L - a.c.strike;
        V = (x > 0.0 ? x : 0.0) * a.c.daycount * scale;
        g[a.c.index] += (x >= 0.0 ? a.c.daycount : 0.0) * scale;
    }
#pragma unroll 1
    for (int k = 0; k < a.num_index; k++) {
        const double Lk = state_at<double>(a.states, a.state_slot, a.N, a.P, k, p);  // L_k(T_k)
        g[k] -= V * a.delta[k] / (1.0 + a.delta[k] * Lk);
    }
    const double invP = 1.0 / (double)a.P;
#pragma unroll 1
    for (int j = 0; j < a.N; j++) a.seeds[(size_t)j * a.P + p] = g[j] * invP;
}

// ------------------------------------------------------------------ Bermudan
// The regression's Gram matrix X^T X at an exercise date depends only on the basis
// functions, not on the backward induction, so (as the reference caches its solver,
// MonteCarloConditionalExpectationRegression.java:125-137) all exercise dates' Gram
// matrices are accumulated in one pass and their SVDs computed in parallel.  The
// backward induction then needs, per date, only the six sums of X^T y and a 6x6 apply.
constexpr int kGram = 20;  // G[0][1..5] and G[1..5][1..5] (i<=j); G[0][0] = 1 exactly
constexpr int kRhs = 6;
constexpr int kSvdStride = 80;  // U[36], s[6], V[36], tol, pad

struct BermShared {
    int basis, callable, N, P, ne;
    NumeraireInfo num;
    const void* states;
    const BermudanPeriod* per;     // [nper] (device)
    const int* ex_period;          // [ne] period index of each exercise date (device)
    const double* tenor_delta;     // [N]
    const int* period_index;       // [nper]
    const double* period_length;   // [nper]
    double* basis_buf;             // [ne][5][P]
};

// the swap periods of one exercise date in FP32 (period index, length), staged per block
struct SwapRows32 {
    int idx[kMaxN];
    float len[kMaxN];
};

template <typename TS>
__device__ __forceinline__ void bermudan_basis(const BermShared& a, const BermudanPeriod& c, int p, double B[5])
{
    if (a.basis == 1) {
        // {S, S^2, N, N^2, S*N}: S = par rate of the remaining periods from L_j(T_ex),
        // S = (prod g_q - 1) / sum_s d_s prod_{r>s} g_r with g_q = 1 + L_q d_q, both by a
        // forward recursion (one division per path instead of one per period)
        double H = 0.0, prod = 1.0;
        for (int q = c.swap_first; q < c.swap_last; q++) {
            const double Lq = state_at<TS>(a.states, c.ex_slot, a.N, a.P, a.period_index[q], p);
            const double dq = a.period_length[q];
            const double g = 1.0 + Lq * dq;
            if (q == c.swap_first) {
                prod = g;
                H = dq;
            } else {
                prod = prod * g;
                H = H * g + dq;
            }
        }
        const double S = (prod - 1.0) / H;
        const double Nn = numeraire_adj(a.num, c.ex_num_index, p);
        B[0] = S;
        B[1] = S * S;
        B[2] = Nn;
        B[3] = Nn * Nn;
        B[4] = S * Nn;
    } else {
        // reference basis {P_short, P_short^2, P_long, P_long^2, 1/N} (BermudanSwaption.java:215-252)
        const double rs = state_at<TS>(a.states, c.ex_slot, a.N, a.P, c.short_index, p);
        const double ds = 1.0 / (rs * c.short_dt + 1.0);
        double rl;
        if (c.long_last == c.long_first + 1) {
            rl = state_at<TS>(a.states, c.ex_slot, a.N, a.P, c.long_first, p);
        } else {
            double acc = 0.0;
            for (int q = c.long_first; q < c.long_last; q++) {
                const double Lq = state_at<TS>(a.states, c.ex_slot, a.N, a.P, q, p);
                const double sub = a.tenor_delta[q];
                acc = (q == c.long_first) ? Lq * sub + 1.0 : acc * (1.0 + Lq * sub);
            }
            rl = (acc - 1.0) / c.long_dt;
        }
        const double dl = 1.0 / (rl * c.long_dt + 1.0);
        B[0] = ds;
        B[1] = ds * ds;
        B[2] = dl;
        B[3] = dl * dl;
        B[4] = 1.0 / numeraire_adj(a.num, c.ex_num_index, p);
    }
}

// Mixed form: the basis in FP32.  The {S, S^2, N, N^2, S*N} basis runs the same par-rate
// recursion in FP32 (the state's precision) over the staged FP32 period table, with the
// adjusted numeraire rounded to FP32 (nfac = adjustment / P^d of the date); the reference
// basis is evaluated in FP64 and rounded.  The Gram matrix and X^T y are accumulated from
// these same rounded values, so the regression is the exact least-squares fit of them.
__device__ __forceinline__ void bermudan_basis32(const BermShared& a, const BermudanPeriod& c, int p, float B[5],
                                 const SwapRows32* rows, float nfac)
{
    if (a.basis == 1) {
        float H = 0.0f, prod = 1.0f;
        const float* st = static_cast<const float*>(a.states) + (size_t)c.ex_slot * a.N * a.P + p;
        const int nq = c.swap_last - c.swap_first;
        for (int q0 = 0; q0 < nq; q0 += 8) {
            float Lb[8];  // eight independent loads in flight per thread
#pragma unroll
            for (int k = 0; k < 8; k++) Lb[k] = q0 + k < nq ? st[(size_t)rows->idx[q0 + k] * a.P] : 0.0f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int q = q0 + k;
                if (q < nq) {
                    const float dq = rows->len[q];
                    const float g = fmaf(Lb[k], dq, 1.0f);
                    if (q == 0) {
                        prod = g;
                        H = dq;
                    } else {
                        prod = prod * g;
                        H = fmaf(H, g, dq);
                    }
                }
            }
        }
        const float S = (prod - 1.0f) / H;
        const float Nn = f64_to_f32_int(a.num.numeraire[(size_t)c.ex_num_index * a.P + p]) * nfac;
        B[0] = S;
        B[1] = S * S;
        B[2] = Nn;
        B[3] = Nn * Nn;
        B[4] = S * Nn;
    } else {
        double Bd[5];
        bermudan_basis<float>(a, c, p, Bd);
#pragma unroll
        for (int i = 0; i < 5; i++) B[i] = (float)Bd[i];
    }
}

// FP64 form, swap-rate basis: the par rate S = (prod g_q - 1) / H of the remaining periods
// by the same forward recursion on float pairs (FP32 pipe): the forwards split into pairs in
// integer operations, the period lengths staged as pairs; g = 1 + L d, prod <- prod g,
// H <- H g + d as double-float products and sums (about 2^-47 relative a step).  The basis
// enters only the regression that estimates the continuation value, so its error moves
// the exercise decisions of paths within ~1e-13 of the boundary only; the adjusted
// numeraire is N times the date's uniform factor adjustment / P^d.
struct SwapRowsDf {
    int idx[kMaxN];
    float len_h[kMaxN], len_l[kMaxN];
};

__device__ __forceinline__ void df_mul_pair(float ah, float al, float bh, float bl, float& ph, float& pl)
{
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    ph = p + e;  // |e| is far below |p|: the renormalised pair
    pl = e - (ph - p);
}

__device__ __forceinline__ void df_add_pair(float ah, float al, float bh, float bl, float& sh, float& sl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    const float t = (al + bl) + e;
    sh = s + t;
    sl = t - (sh - s);
}

__device__ __forceinline__ void bermudan_basis_swaprate_df(const BermShared& a, const BermudanPeriod& c, int p,
                                                           const SwapRowsDf* rows, double nfac, double B[5])
{
    const double* st = static_cast<const double*>(a.states) + (size_t)c.ex_slot * a.N * a.P + p;
    const int nq = c.swap_last - c.swap_first;
    float ph = 1.0f, pl = 0.0f, hh = 0.0f, hl = 0.0f;
    for (int q0 = 0; q0 < nq; q0 += 8) {
        double Lb[8];  // eight independent loads in flight per thread
#pragma unroll
        for (int k = 0; k < 8; k++) Lb[k] = q0 + k < nq ? st[(size_t)rows->idx[q0 + k] * a.P] : 0.0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int q = q0 + k;
            if (q < nq) {
                float Lh, Ll;
                df_split_int(Lb[k], Lh, Ll);
                const float dh = rows->len_h[q], dl = rows->len_l[q];
                // g = 1 + L d: the product's exact error, then 1 + x with |x| < 1
                const float x = __fmul_rn(Lh, dh);
                float xe = fmaf(Lh, dh, -x);
                xe = fmaf(Lh, dl, xe);
                xe = fmaf(Ll, dh, xe);
                const float gh0 = 1.0f + x;
                const float gl0 = (x - (gh0 - 1.0f)) + xe;
                if (q == 0) {
                    ph = gh0;
                    pl = gl0;
                    hh = dh;
                    hl = dl;
                } else {
                    df_mul_pair(ph, pl, gh0, gl0, ph, pl);
                    float th, tl;
                    df_mul_pair(hh, hl, gh0, gl0, th, tl);
                    df_add_pair(th, tl, dh, dl, hh, hl);
                }
            }
        }
    }
    // S = (prod - 1) / H
    float nh, nl;
    df_add_pair(ph, pl, -1.0f, 0.0f, nh, nl);
    const float yh = __fdiv_rn(nh, hh);
    const float pr = __fmul_rn(yh, hh);
    const float pe = fmaf(yh, hh, -pr);
    float res = (nh - pr) - pe;
    res = res + nl;
    res = fmaf(-yh, hl, res);
    const float yl = __fmul_rn(res, __frcp_rn(hh));
    const double S = f32_to_f64_nz(yh) + f32_to_f64_nz(yl);
    const double Nn = a.num.numeraire[(size_t)c.ex_num_index * a.P + p] * nfac;
    B[0] = S;
    B[1] = S * S;
    B[2] = Nn;
    B[3] = Nn * Nn;
    B[4] = S * Nn;
}

// grid (bx, ne): basis functions of exercise date blockIdx.y and their Gram partial sums
template <typename TS>
__global__ void __launch_bounds__(kProdThreads, sizeof(TS) == 4 ? 3 : 1) bermudan_gram_kernel(const BermShared a, double* partials)
{
    const int e = blockIdx.y;
    const BermudanPeriod c = a.per[a.ex_period[e]];
    double acc[kGram];
    if (sizeof(TS) == 4) {
        // mixed form: the basis in FP32 (stored as FP32), the Gram sums in FP64 (plain within
        // a thread and a warp, compensated across warps and blocks)
        __shared__ SwapRows32 rows;
        for (int q = threadIdx.x; q < c.swap_last - c.swap_first; q += blockDim.x) {
            rows.idx[q] = a.period_index[c.swap_first + q];
            rows.len[q] = (float)a.period_length[c.swap_first + q];
        }
        __syncthreads();
        __shared__ float nfac_s;  // adjustment / P^d of the date, once per block (no FP64 per thread)
        if (threadIdx.x == 0) {
            const int l = c.ex_num_index;
            nfac_s = a.num.has_discount ? (float)(a.num.adj[l] * a.num.inv_pd[l]) : 1.0f;
        }
        __syncthreads();
        const float nfac = nfac_s;
#pragma unroll
        for (int k = 0; k < kGram; k++) acc[k] = 0.0;
        float* bb = reinterpret_cast<float*>(a.basis_buf) + (size_t)e * 5 * a.P;
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.P; p += gridDim.x * blockDim.x) {
            float B32[5];
            bermudan_basis32(a, c, p, B32, &rows, nfac);
            double B[5];
#pragma unroll
            for (int i = 0; i < 5; i++) {
                bb[(size_t)i * a.P + p] = B32[i];
                B[i] = f32_to_f64_int(B32[i]);  // exact, in integer operations
            }
#pragma unroll
            for (int i = 0; i < 5; i++) acc[i] = acc[i] + B[i];
            int k = 5;
#pragma unroll
            for (int i = 0; i < 5; i++)
#pragma unroll
                for (int j = i; j < 5; j++, k++) acc[k] = fma(B[i], B[j], acc[k]);  // the product is exact in FP64
        }
        block_sums_warp_plain<kGram>(acc, partials + ((size_t)e * gridDim.x + blockIdx.x) * kGram * 2, 1);
        return;
    }
    // FP64 form: the swap-rate basis on float pairs (above), the reference basis in FP64;
    // the Gram sums by fused multiply-adds, plain within a thread and a warp, compensated
    // across warps and blocks
    __shared__ SwapRowsDf rows;
    __shared__ double nfac_d;
    if (a.basis == 1) {
        for (int q = threadIdx.x; q < c.swap_last - c.swap_first; q += blockDim.x) {
            const double d = a.period_length[c.swap_first + q];
            rows.idx[q] = a.period_index[c.swap_first + q];
            rows.len_h[q] = (float)d;
            rows.len_l[q] = (float)(d - (double)rows.len_h[q]);
        }
        if (threadIdx.x == 0) {
            const int l = c.ex_num_index;
            nfac_d = a.num.has_discount ? a.num.adj[l] / a.num.pd[l] : 1.0;
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < kGram; k++) acc[k] = 0.0;
    double* bb = a.basis_buf + (size_t)e * 5 * a.P;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.P; p += gridDim.x * blockDim.x) {
        double B[5];
        if (a.basis == 1) bermudan_basis_swaprate_df(a, c, p, &rows, nfac_d, B);
        else bermudan_basis<TS>(a, c, p, B);
#pragma unroll
        for (int i = 0; i < 5; i++) bb[(size_t)i * a.P + p] = B[i];
#pragma unroll
        for (int i = 0; i < 5; i++) acc[i] = acc[i] + B[i];  // mean(1 * B_i)
        int k = 5;
#pragma unroll
        for (int i = 0; i < 5; i++)
#pragma unroll
            for (int j = i; j < 5; j++, k++) acc[k] = fma(B[i], B[j], acc[k]);
    }
    block_sums_warp_plain<kGram>(acc, partials + ((size_t)e * gridDim.x + blockIdx.x) * kGram * 2, 1);
}

__device__ void svd6(const double G[36], double U[36], double s[6], double V[36])
{
    for (int i = 0; i < 36; i++) U[i] = G[i];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) V[i * 6 + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        int rotated = 0;
        for (int p = 0; p < 5; p++)
            for (int q = p + 1; q < 6; q++) {
                double alpha = 0.0, beta = 0.0, gamma = 0.0;
                for (int k = 0; k < 6; k++) {
                    const double up = U[k * 6 + p], uq = U[k * 6 + q];
                    alpha += up * up;
                    beta += uq * uq;
                    gamma += up * uq;
                }
                if (gamma == 0.0 || fabs(gamma) <= 0x1.0p-52 * sqrt(alpha * beta)) continue;
                rotated = 1;
                const double zeta = (beta - alpha) / (2.0 * gamma);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
                for (int k = 0; k < 6; k++) {
                    const double up = U[k * 6 + p], uq = U[k * 6 + q];
                    U[k * 6 + p] = cs * up - sn * uq;
                    U[k * 6 + q] = sn * up + cs * uq;
                }
                for (int k = 0; k < 6; k++) {
                    const double vp = V[k * 6 + p], vq = V[k * 6 + q];
                    V[k * 6 + p] = cs * vp - sn * vq;
                    V[k * 6 + q] = sn * vp + cs * vq;
                }
            }
        if (!rotated) break;
    }
    for (int j = 0; j < 6; j++) {
        double nn = 0.0;
        for (int k = 0; k < 6; k++) nn += U[k * 6 + j] * U[k * 6 + j];
        s[j] = sqrt(nn);
        if (s[j] > 0.0)
            for (int k = 0; k < 6; k++) U[k * 6 + j] = U[k * 6 + j] / s[j];
    }
}

// grid ne x 32: reduce the Gram partials of date blockIdx.x, SVD, store U, s, V, cutoff
__global__ void __launch_bounds__(32) bermudan_svd_kernel(const double* partials, int bx, int P, double* svd)
{
    __shared__ double tot[kGram];
    const int e = blockIdx.x, lane = threadIdx.x;
    for (int k = 0; k < kGram; k++) {
        dd acc{0.0, 0.0};
        for (int b = lane; b < bx; b += 32) {
            const double* q = partials + (((size_t)e * bx + b) * kGram + k) * 2;
            acc = dd_add(acc, dd{q[0], q[1]});
        }
        acc = warp_dd_sum(acc);
        if (lane == 0) tot[k] = (acc.hi + acc.lo) / (double)P;
    }
    __syncwarp();
    if (lane == 0) {
        double G[36], U[36], s[6], V[36];
        G[0] = 1.0 * 1.0;
        int k = 0;
        for (int j = 1; j < 6; j++) { G[j] = tot[k]; G[j * 6] = tot[k]; k++; }
        for (int i = 1; i < 6; i++)
            for (int j = i; j < 6; j++) { G[i * 6 + j] = tot[k]; G[j * 6 + i] = tot[k]; k++; }
        svd6(G, U, s, V);
        double smax = 0.0;
        for (int j = 0; j < 6; j++) smax = s[j] > smax ? s[j] : smax;
        double tol = 6.0 * smax * 0x1.0p-52;
        const double tmin = sqrt(0x1.0p-1022);
        if (tol < tmin) tol = tmin;
        double* o = svd + (size_t)e * kSvdStride;
        for (int i = 0; i < 36; i++) o[i] = U[i];
        for (int i = 0; i < 6; i++) o[36 + i] = s[i];
        for (int i = 0; i < 36; i++) o[42 + i] = V[i];
        o[78] = tol;
    }
}

// X^T y sums of one date and beta = V diag(1/s) U^T (X^T y) with the SVD's cutoff,
// in the oracle's order (MonteCarloConditionalExpectationRegression.java:141-147).  Run by
// one block of at least 6 warps (all its threads call it).
__device__ void regression_solve(const double* partials, int blocks, int P, const double* svd, double* beta_out)
{
    __shared__ double b[kRhs];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < kRhs) {
        // the blocks' double-double partials of column `warp`, summed exactly
        const dd acc = warp_exact_pair_sum(partials + (size_t)warp * 2, blocks, kRhs * 2);
        if (lane == 0) b[warp] = (acc.hi + acc.lo) / (double)P;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const double* U = svd;
        const double* s = svd + 36;
        const double* V = svd + 42;
        const double tol = svd[78];
        const int i = threadIdx.x;
        double acc = 0.0;
        for (int j = 0; j < 6; j++) {
            if (!(s[j] > tol)) continue;
            double utb = 0.0;
            for (int r = 0; r < 6; r++) utb += U[r * 6 + j] * b[r];
            acc += V[i * 6 + j] * (utb / s[j]);
        }
        beta_out[i] = acc;
    }
}

// Mixed form: the same solve, the coefficients stored as FP32 pairs (hi, lo) for the
// Dot2 conditional expectation of the next step.
__device__ void regression_solve_mixed(const double* partials, int blocks, int P, const double* svd, double* beta_out)
{
    __shared__ double b[kRhs];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < kRhs) {
        // the blocks' double-double partials of column `warp`, summed exactly
        const dd acc = warp_exact_pair_sum(partials + (size_t)warp * 2, blocks, kRhs * 2);
        if (lane == 0) b[warp] = (acc.hi + acc.lo) / (double)P;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const double* U = svd;
        const double* s = svd + 36;
        const double* V = svd + 42;
        const double tol = svd[78];
        const int i = threadIdx.x;
        double acc = 0.0;
        for (int j = 0; j < 6; j++) {
            if (!(s[j] > tol)) continue;
            double utb = 0.0;
            for (int r = 0; r < 6; r++) utb = fma(U[r * 6 + j], b[r], utb);
            acc = fma(V[i * 6 + j], utb / s[j], acc);
        }
        float hi, lo;
        split_double(acc, hi, lo);
        reinterpret_cast<float*>(beta_out)[2 * i] = hi;
        reinterpret_cast<float*>(beta_out)[2 * i + 1] = lo;
    }
}

struct BermStepParams {
    BermShared sh;
    int cur;                   // period processed by this launch (-1: final pass)
    int cur_ex;                // exercise index of cur (or -1)
    int pending_ex;            // exercise index whose choose is pending (or -1)
    double pending_fixing;
    const double* beta;        // [ne][6]
    double* values;
    double* under;
    double* ex;
    double* partials;          // [blocks][6][2], then an unsigned completion counter
    const double* svd_cur;     // SVD factors of the date cur_ex (when it regresses)
    double* beta_cur;          // its coefficients, written by the launch's last block
    int init;
    double* rec;               // nullptr, or [2][ne][P]: per exercise date the trigger X and Y - Z
                               // (continuation minus underlying) the choice is made on
};

// The last block of a step launch to finish reduces every block's X^T y partials (in block
// order) and solves for the date's coefficients; nothing waits on another block.  All
// threads of every block call it after writing their block's partials.
__device__ void finish_date_last_block(const BermStepParams& a, bool mixed)
{
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    unsigned int* done = reinterpret_cast<unsigned int*>(a.partials + (size_t)gridDim.x * kRhs * 2);
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) {
        __threadfence();
        if (mixed) regression_solve_mixed(a.partials, gridDim.x, a.sh.P, a.svd_cur, a.beta_cur);
        else regression_solve(a.partials, gridDim.x, a.sh.P, a.svd_cur, a.beta_cur);
        if (threadIdx.x == 0) *done = 0u;  // ready for the next date
    }
}

// FP64 form: the reference's backward induction (BermudanSwaption.java:91-157) with fused
// multiply-adds for X beta and X^T y, and the payoff times the path's reciprocal numeraire
// (from the path kernel) and the date's uniform factor P^d / adjustment instead of a
// division per path.
__global__ void __launch_bounds__(kProdThreads) bermudan_step_kernel(const BermStepParams a)
{
    const BermShared& sh = a.sh;
    const double w = 1.0 / (double)sh.P;
    __shared__ double pay_fac;  // (P^d / adjustment) w of the payment date, once per block
    if (a.cur >= 0 && sh.num.inv_numeraire) {
        if (threadIdx.x == 0) {
            const int l = sh.per[a.cur].pay_num_index;
            pay_fac = sh.num.has_discount ? (sh.num.pd[l] / sh.num.adj[l]) * w : w;
        }
        __syncthreads();
    }
    double acc[kRhs];
#pragma unroll
    for (int i = 0; i < kRhs; i++) acc[i] = 0.0;
    double beta[6];
    const double* bprev = nullptr;
    if (a.pending_ex >= 0) {
#pragma unroll
        for (int i = 0; i < 6; i++) beta[i] = a.beta[a.pending_ex * 6 + i];
        bprev = sh.basis_buf + (size_t)a.pending_ex * 5 * sh.P;
    }
    const double* bcur = a.cur_ex >= 0 ? sh.basis_buf + (size_t)a.cur_ex * 5 * sh.P : nullptr;
    BermudanPeriod c;
    if (a.cur >= 0) c = sh.per[a.cur];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < sh.P; p += gridDim.x * blockDim.x) {
        double v, u;
        if (a.init) {
            v = 0.0;
            u = 0.0;
            a.ex[p] = CUDART_INF;
        } else {
            v = a.values[p];
            u = a.under[p];
        }
        if (bprev) {
            // conditional expectation X beta (:104-107), then choose (:139, :141)
            double ce = beta[0];
#pragma unroll
            for (int i = 1; i < 6; i++) ce = fma(bprev[(size_t)(i - 1) * sh.P + p], beta[i], ce);
            const bool cont = ce >= 0.0;
            if (a.rec) {
                a.rec[(size_t)a.pending_ex * sh.P + p] = ce;
                a.rec[((size_t)sh.ne + a.pending_ex) * sh.P + p] = v - u;
            }
            v = cont ? v : u;
            if (!cont) a.ex[p] = a.pending_fixing;
        }
        if (a.cur >= 0) {
            const double L = state_at<double>(sh.states, c.libor_slot, sh.N, sh.P, c.libor_index, p);
            double payoff = ((L - c.strike) * c.period_length) * c.notional;
            if (sh.num.inv_numeraire) {
                payoff = payoff * (sh.num.inv_numeraire[(size_t)c.pay_num_index * sh.P + p] * pay_fac);
            } else {
                payoff = payoff / numeraire_adj(sh.num, c.pay_num_index, p);
                payoff = payoff * w;
            }
            if (sh.callable) u = u + payoff;
            else v = v + payoff;
            if (bcur) {
                const double y = v - u;
                acc[0] = acc[0] + y;
#pragma unroll
                for (int i = 0; i < 5; i++) acc[1 + i] = fma(y, bcur[(size_t)i * sh.P + p], acc[1 + i]);
            }
        } else {
            v = (v * numeraire_adj(sh.num, 0, 0)) / w;  // numeraire at time 0 (exactly 1 under SPOT)
        }
        a.values[p] = v;
        a.under[p] = u;
    }
    if (bcur) {
        // plain within a warp (a thread holds a few paths' sums), compensated across warps
        block_sums_warp_plain<kRhs>(acc, a.partials + (size_t)blockIdx.x * kRhs * 2, 1);
        finish_date_last_block(a, false);
    }
}

// Mixed form: the same backward induction with FP32 path values (continuation v and
// underlying u, kept as two FP32 arrays in the under buffer), FP32 payoffs and the FP32
// basis; the X^T y sums in FP64 (the products of FP32 values exact), the conditional
// expectation X beta in twice FP32 precision (Dot2).  Payoffs are not scaled by 1/P (the reference's weight, which cancels in the
// final value and scales X^T y and beta alike, leaving the exercise decisions unchanged).
// Only the final values are written in FP64.
__global__ void __launch_bounds__(kProdThreads) bermudan_step_mixed_kernel(const BermStepParams a)
{
    const BermShared& sh = a.sh;
    const int P = sh.P;
    float* v32 = reinterpret_cast<float*>(a.under);
    float* u32 = v32 + P;
    double acc[kRhs];
#pragma unroll
    for (int i = 0; i < kRhs; i++) acc[i] = 0.0;
    float bh[6], bl[6];
    const float* bprev = nullptr;
    if (a.pending_ex >= 0) {
        const float* b32 = reinterpret_cast<const float*>(a.beta + a.pending_ex * 6);  // (hi, lo) pairs
#pragma unroll
        for (int i = 0; i < 6; i++) {
            bh[i] = b32[2 * i];
            bl[i] = b32[2 * i + 1];
        }
        bprev = reinterpret_cast<const float*>(sh.basis_buf) + (size_t)a.pending_ex * 5 * P;
    }
    const float* bcur = a.cur_ex >= 0 ? reinterpret_cast<const float*>(sh.basis_buf) + (size_t)a.cur_ex * 5 * P : nullptr;
    const float* Lrow = nullptr;
    const double* inv_num = nullptr;
    const double* num = nullptr;
    // per-date constants, evaluated once per block: FP64 work per thread would load the
    // narrow FP64 pipe more than the paths themselves do
    __shared__ float consts_s[2];
    __shared__ double num0_s;
    if (threadIdx.x == 0) {
        if (a.cur >= 0) {
            const BermudanPeriod c = sh.per[a.cur];
            const int l = c.pay_num_index;
            double f = c.period_length * c.notional;
            if (sh.num.has_discount) f = f * (sh.num.pd[l] / sh.num.adj[l]);  // 1/N_adj = (1/N) P^d / adjustment
            consts_s[0] = (float)c.strike;
            consts_s[1] = (float)f;
        } else {
            num0_s = numeraire_adj(sh.num, 0, 0);  // numeraire at time 0 (exactly 1 under SPOT)
        }
    }
    __syncthreads();
    float strike = 0.0f, fac = 0.0f;
    double num0 = 0.0;
    if (a.cur >= 0) {
        const BermudanPeriod& c = sh.per[a.cur];
        const int l = c.pay_num_index;
        Lrow = static_cast<const float*>(sh.states) + ((size_t)c.libor_slot * sh.N + c.libor_index) * P;
        strike = consts_s[0];
        fac = consts_s[1];
        if (sh.num.inv_numeraire) inv_num = sh.num.inv_numeraire + (size_t)l * P;
        else num = sh.num.numeraire + (size_t)l * P;
    } else {
        num0 = num0_s;
    }
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        float v, u;
        if (a.init) {
            v = 0.0f;
            u = 0.0f;
            a.ex[p] = CUDART_INF;
        } else {
            v = v32[p];
            u = u32[p];
        }
        if (bprev) {
            Sum2 ce{bh[0], bl[0]};
#pragma unroll
            for (int i = 1; i < 6; i++) {
                const float x = bprev[(size_t)(i - 1) * P + p];
                dot2_add(ce, bh[i], x);
                ce.s = fmaf(bl[i], x, ce.s);
            }
            if (a.rec) {
                a.rec[(size_t)a.pending_ex * P + p] = sum2_value(ce);
                a.rec[((size_t)sh.ne + a.pending_ex) * P + p] = f32_to_f64_int(v - u);
            }
            if (!(ce.p + ce.s >= 0.0f)) {
                v = u;
                a.ex[p] = a.pending_fixing;
            }
        }
        if (a.cur >= 0) {
            const float iN = inv_num ? f64_to_f32_int(inv_num[p]) : (float)(1.0 / num[p]);
            const float payoff = ((Lrow[p] - strike) * fac) * iN;
            if (sh.callable) u = u + payoff;
            else v = v + payoff;
            if (bcur) {
                const double y = f32_to_f64_int(v - u);  // widened in integer operations
                acc[0] = acc[0] + y;
#pragma unroll
                for (int i = 0; i < 5; i++) acc[1 + i] = fma(y, f32_to_f64_int(bcur[(size_t)i * P + p]), acc[1 + i]);
            }
            v32[p] = v;
            u32[p] = u;
        } else {
            a.values[p] = (double)v * num0;
        }
    }
    if (bcur) {
        block_sums_warp_plain<kRhs>(acc, a.partials + (size_t)blockIdx.x * kRhs * 2, 1);
        finish_date_last_block(a, true);
    }
}

NumeraireInfo make_numeraire_info(const ProductView& v)
{
    NumeraireInfo n;
    n.P = v.P;
    n.has_discount = v.h_discount != nullptr;
    n.numeraire = v.d_numeraire;
    n.inv_numeraire = v.d_inv_numeraire;
    n.adj = v.d_num_adj;
    for (int l = 0; l <= kMaxN; l++) {
        n.pd[l] = (v.h_discount && l <= v.N) ? v.h_discount[l] : 1.0;
        n.inv_pd[l] = 1.0 / n.pd[l];
        n.det[l] = (l <= v.N) ? v.h_num_det[l] : 0;
    }
    return n;
}

int grid_for(int P, int threads, int max_blocks)
{
    int b = (P + threads - 1) / threads;
    return b < max_blocks ? b : max_blocks;
}

}  // namespace

static int launch_european_seeds(const ProductView& v, EuroSeedParams& e, const double* h_delta, double* d_seeds,
                                 cudaStream_t s)
{
    if (v.state_fp32) return fail(LMM_ERR_INVALID, "the European products' adjoint runs on FP64 processes");
    e.N = v.N;
    e.P = v.P;
    e.num = make_numeraire_info(v);
    e.states = static_cast<const double*>(v.d_states);
    for (int k = 0; k < v.N && k < kMaxN; k++) e.delta[k] = h_delta[k];
    e.seeds = d_seeds;
    KernelTimer kt(K_ADJOINT, s);
    european_seed_kernel<<<(v.P + kProdThreads - 1) / kProdThreads, kProdThreads, 0, s>>>(e);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

int launch_swaption_seeds(const ProductView& v, const SwaptionLaunch& a, int exercise_slot, const double* h_delta,
                          double* d_seeds, cudaStream_t s)
{
    EuroSeedParams e;
    std::memset(&e, 0, sizeof(e));
    e.s = a;
    e.kind = 0;
    e.num_index = a.num_index;
    e.state_slot = exercise_slot;  // the fixings L_k(T_k), k < the exercise index, as of the exercise date
    return launch_european_seeds(v, e, h_delta, d_seeds, s);
}

int launch_caplet_seeds(const ProductView& v, const CapletSeed& c, const double* h_delta, double* d_seeds,
                        cudaStream_t s)
{
    EuroSeedParams e;
    std::memset(&e, 0, sizeof(e));
    e.c = c;
    e.kind = 1;
    e.num_index = c.index + 1;
    e.state_slot = c.slot;
    return launch_european_seeds(v, e, h_delta, d_seeds, s);
}

int launch_numeraire_finish(const double* d_partials, int blocks, int N, int P, const double* d_numeraire,
                            const uint8_t* d_det, double* d_adj, cudaStream_t s)
{
    KernelTimer kt(K_NUMERAIRE_FINISH, s);
    numeraire_finish_kernel<<<N + 1, 256, 0, s>>>(d_partials, blocks, N, P, d_numeraire, d_det, d_adj);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

int reduce_mean_stderr(const double* d_values, int P, double* d_scratch, size_t scratch_bytes, double* h_mean,
                       double* h_stderr, cudaStream_t s)
{
    const int blocks = grid_for(P, 256, 1024);
    if (scratch_bytes < (size_t)(2 * blocks + 2) * sizeof(double)) return fail(LMM_ERR_INVALID, "reduction scratch too small");
    double* partials = d_scratch;
    double* res = d_scratch + 2 * blocks;
    {
        KernelTimer kt(K_VALUE_REDUCE, s, 4);
        sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, nullptr, partials);
        finish_partials_kernel<<<1, 256, 0, s>>>(partials, blocks, P, res);
        sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, res, partials);
        finish_partials_kernel<<<1, 256, 0, s>>>(partials, blocks, P, res + 1);
        LMM_CUDA(cudaGetLastError());
    }
    double h[2];
    LMM_CUDA(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, s));
    LMM_CUDA(cudaStreamSynchronize(s));
    *h_mean = h[0];
    if (h_stderr) *h_stderr = P > 1 ? sqrt(h[1]) / sqrt((double)P) : 0.0;
    return LMM_OK;
}

int launch_swaption(const ProductView& v, const SwaptionLaunch& a, double* d_values, cudaStream_t s)
{
    SwaptionParams prm;
    prm.s = a;
    prm.num = make_numeraire_info(v);
    prm.states = v.d_states;
    prm.N = v.N;
    prm.P = v.P;
    prm.fp32 = v.state_fp32;
    prm.values = d_values;
    const int blocks = (v.P + kProdThreads - 1) / kProdThreads;
    KernelTimer kt(K_SWAPTION, s);
    if (v.state_fp32) swaption_kernel<float><<<blocks, kProdThreads, 0, s>>>(prm);
    else swaption_kernel<double><<<blocks, kProdThreads, 0, s>>>(prm);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

int bermudan_blocks(int P)
{
    static int cap = 0;
    if (!cap) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
        cap = sms * 4;
    }
    return grid_for(P, kProdThreads, cap);
}

// Gram blocks per exercise date.  The mixed form spreads its (latency-bound, unevenly
// sized: early dates have long swaps) dates over four times as many blocks.
int bermudan_gram_blocks(int P, int ne, bool fp32)
{
    const int total = bermudan_blocks(P) * (fp32 ? 4 : 1);
    int bx = (total + ne - 1) / (ne > 0 ? ne : 1);
    const int need = (P + kProdThreads - 1) / kProdThreads;
    if (bx > need) bx = need;
    return bx < 1 ? 1 : bx;
}

int reduce_mean_var_device(const double* d_values, int P, double* d_scratch, double* d_out2, cudaStream_t s)
{
    const int blocks = grid_for(P, 256, 1024);
    KernelTimer kt(K_VALUE_REDUCE, s, 4);
    sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, nullptr, d_scratch);
    finish_partials_kernel<<<1, 256, 0, s>>>(d_scratch, blocks, P, d_out2);
    sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, d_out2, d_scratch);
    finish_partials_kernel<<<1, 256, 0, s>>>(d_scratch, blocks, P, d_out2 + 1);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

namespace {
__global__ void timestamp_kernel(unsigned long long* out)
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}
}  // namespace

int launch_timestamp(unsigned long long* d_out, cudaStream_t s)
{
    timestamp_kernel<<<1, 1, 0, s>>>(d_out);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

int launch_bermudan(const ProductView& v, const BermudanLaunch& a, const BermudanScratch& sc, cudaStream_t s,
                    int* launches)
{
    const int blocks = bermudan_blocks(v.P);
    std::vector<int> ex_period, ex_of_period(a.nper, -1);
    for (int q = 0; q < a.nper; q++)
        if (a.per[q].exercisable) {
            ex_of_period[q] = (int)ex_period.size();
            ex_period.push_back(q);
        }
    const int ne = (int)ex_period.size();
    if (!sc.tables_on_device) {
        LMM_CUDA(cudaMemcpyAsync(sc.d_per, a.per.data(), sizeof(BermudanPeriod) * a.nper, cudaMemcpyHostToDevice, s));
        if (ne) LMM_CUDA(cudaMemcpyAsync(sc.d_ex_period, ex_period.data(), sizeof(int) * ne, cudaMemcpyHostToDevice, s));
        count_h2d(sizeof(BermudanPeriod) * (size_t)a.nper + sizeof(int) * (size_t)ne);
    }
    BermShared sh;
    std::memset(&sh, 0, sizeof(sh));
    sh.basis = a.basis;
    sh.callable = a.callable;
    sh.N = v.N;
    sh.P = v.P;
    sh.ne = ne;
    sh.num = make_numeraire_info(v);
    sh.states = v.d_states;
    sh.per = sc.d_per;
    sh.ex_period = sc.d_ex_period;
    sh.tenor_delta = sc.d_tenor_delta;
    sh.period_index = sc.d_period_index;
    sh.period_length = sc.d_period_length;
    sh.basis_buf = sc.d_basis;
    if (ne > 0) {
        const int bx = sc.gram_blocks > 0 ? sc.gram_blocks : bermudan_gram_blocks(v.P, ne, v.state_fp32 != 0);
        {
            KernelTimer kt(K_BERMUDAN_STEP, s);
            const dim3 grid(bx, ne);
            if (v.state_fp32) bermudan_gram_kernel<float><<<grid, kProdThreads, 0, s>>>(sh, sc.d_gram);
            else bermudan_gram_kernel<double><<<grid, kProdThreads, 0, s>>>(sh, sc.d_gram);
            LMM_CUDA(cudaGetLastError());
        }
        {
            KernelTimer kt(K_BERMUDAN_SOLVE, s);
            bermudan_svd_kernel<<<ne, 32, 0, s>>>(sc.d_gram, bx, v.P, sc.d_svd);
            LMM_CUDA(cudaGetLastError());
        }
        if (launches) (*launches) += 2;
    }
    BermStepParams prm;
    std::memset(&prm, 0, sizeof(prm));
    prm.sh = sh;
    prm.beta = sc.d_beta;
    prm.values = sc.d_values;
    prm.under = sc.d_under;
    prm.ex = sc.d_ex;
    prm.partials = sc.d_partials;
    prm.rec = sc.d_rec;
    int pending = -1;  // exercise index whose choose is pending
    for (int per = a.nper - 1; per >= -1; per--) {
        prm.cur = per;
        prm.cur_ex = per >= 0 ? ex_of_period[per] : -1;
        prm.svd_cur = prm.cur_ex >= 0 ? sc.d_svd + (size_t)prm.cur_ex * kSvdStride : nullptr;
        prm.beta_cur = prm.cur_ex >= 0 ? sc.d_beta + (size_t)prm.cur_ex * 6 : nullptr;
        prm.pending_ex = pending;
        prm.pending_fixing = pending >= 0 ? a.per[ex_period[pending]].fixing : 0.0;
        prm.init = per == a.nper - 1;
        {
            KernelTimer kt(K_BERMUDAN_STEP, s);
            if (v.state_fp32) bermudan_step_mixed_kernel<<<blocks, kProdThreads, 0, s>>>(prm);
            else bermudan_step_kernel<<<blocks, kProdThreads, 0, s>>>(prm);
            LMM_CUDA(cudaGetLastError());
        }
        if (launches) (*launches)++;
        pending = -1;
        if (per >= 0 && prm.cur_ex >= 0) pending = prm.cur_ex;  // its coefficients come from the step's last block
    }
    return LMM_OK;
}

// ------------------------------------------------------------------ AAD weights of the cash flows
// The reverse sweep that finmath-lib's RandomVariableDifferentiableAAD runs over
// BermudanSwaption.getValues (BermudanSwaption.java:91-157) with
// diracDeltaApproximationMethod DISCRETE_DELTA (RandomVariableDifferentiableAAD.java:409-429):
// per path, the adjoint weight omega[q][p] of each period's discounted cash flow.  The choice
// values = X.choose(Y, Z) passes its adjoint to Y where X >= 0 and to Z where X < 0, and to
// the trigger X the term (Y - Z) 1{-eps/2 <= X < eps/2} / eps, eps = width * stdev(X); the
// trigger is the conditional expectation of Y - Z, whose argument receives the conditional
// expectation of the adjoint (:188-192) -- the regression of the trigger's adjoint on the
// date's basis, solved with the date's stored SVD -- so consecutive dates depend on one
// another through a reduction over all paths: one launch per date, whose last block solves
// for the projection coefficients the next launch applies.
namespace {

struct DdSweepParams {
    int P, nper, callable;
    int prev_e, cur_e;           // exercise index applied / processed (-1: none)
    int q_lo, q_hi;              // periods whose weights this launch writes
    double num0;                 // numeraire at time 0: the value's adjoint seed
    const double* rec;           // [2][ne][P]
    const void* basis;           // [ne][5][P] of type TB
    const double* eps;           // [ne]
    const double* svd_cur;       // SVD of the date cur_e
    double* betap;               // [ne][6] projection coefficients
    double* vbar;                // [P] adjoint of the continuation values
    double* ubar;                // [P] adjoint of the underlying
    double* omega;               // [nper][P]
    double* partials;            // [blocks][6][2], then the completion counter
    int ne;
};

// TB: the basis as the forward valuation stored it (double in the FP64 form, float in the mixed
// form); the sweep itself runs in FP64 in both
template <typename TB>
__global__ void __launch_bounds__(kProdThreads) dd_sweep_kernel(const DdSweepParams a)
{
    double acc[kRhs];
#pragma unroll
    for (int i = 0; i < kRhs; i++) acc[i] = 0.0;
    double bp[6];
    const TB* basis = static_cast<const TB*>(a.basis);
    const TB* bprev = nullptr;
    if (a.prev_e >= 0) {
#pragma unroll
        for (int i = 0; i < 6; i++) bp[i] = a.betap[a.prev_e * 6 + i];
        bprev = basis + (size_t)a.prev_e * 5 * a.P;
    }
    const TB* bcur = a.cur_e >= 0 ? basis + (size_t)a.cur_e * 5 * a.P : nullptr;
    const double eps = a.cur_e >= 0 ? a.eps[a.cur_e] : 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.P; p += gridDim.x * blockDim.x) {
        double vb = a.prev_e < 0 && a.q_lo == 0 ? a.num0 : a.vbar[p];
        double ub = a.prev_e < 0 && a.q_lo == 0 ? 0.0 : a.ubar[p];
        if (bprev) {
            // the projection of the previous date's trigger adjoint, as the estimator forms it
            double d = 1.0 * bp[0];
#pragma unroll
            for (int i = 1; i < 6; i++) d = d + (double)bprev[(size_t)(i - 1) * a.P + p] * bp[i];
            vb = vb + d;
            ub = ub - d;
        }
        for (int q = a.q_lo; q < a.q_hi; q++) a.omega[(size_t)q * a.P + p] = a.callable ? ub : vb;
        if (bcur) {
            const double X = a.rec[(size_t)a.cur_e * a.P + p];
            const double D = a.rec[((size_t)a.ne + a.cur_e) * a.P + p];
            double xb = 0.0;
            if (isinf(eps)) xb = vb * D;
            else if (eps > 0.0 && X + eps / 2 >= 0.0 && X - eps / 2 < 0.0) xb = vb * D / eps;
            const bool cont = X >= 0.0;
            ub = ub + (cont ? 0.0 : vb);
            vb = cont ? vb : 0.0;
            acc[0] = acc[0] + xb * 1.0;
#pragma unroll
            for (int i = 0; i < 5; i++) acc[1 + i] = acc[1 + i] + xb * (double)bcur[(size_t)i * a.P + p];
        }
        a.vbar[p] = vb;
        a.ubar[p] = ub;
    }
    if (bcur) {
        block_sums_warp_plain<kRhs>(acc, a.partials + (size_t)blockIdx.x * kRhs * 2, 1);
        __shared__ bool last;
        __threadfence();
        __syncthreads();
        unsigned int* done = reinterpret_cast<unsigned int*>(a.partials + (size_t)gridDim.x * kRhs * 2);
        if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
        __syncthreads();
        if (last) {
            __threadfence();
            regression_solve(a.partials, gridDim.x, a.P, a.svd_cur, a.betap + a.cur_e * 6);
            if (threadIdx.x == 0) *done = 0u;
        }
    }
}

// block partial sums per exercise date of X (pass 0) or of (X - mean)^2 (pass 1)
__global__ void __launch_bounds__(kProdThreads) dd_moment_kernel(const double* rec, int P, const double* mean,
                                                                 double* partials)
{
    const int e = blockIdx.y;
    const double* x = rec + (size_t)e * P;
    const double m = mean ? mean[e] : 0.0;
    double sum = 0.0, err = 0.0;  // the Kahan loop of getAverage / getVariance, per thread
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const double v = (mean ? (x[p] - m) * (x[p] - m) : x[p]) - err;
        const double t = sum + v;
        err = (t - sum) - v;
        sum = t;
    }
    const dd s = block_dd_sum(dd{sum, -err});
    if (threadIdx.x == 0) {
        partials[((size_t)e * gridDim.x + blockIdx.x) * 2] = s.hi;
        partials[((size_t)e * gridDim.x + blockIdx.x) * 2 + 1] = s.lo;
    }
}

// mean (pass 0) or eps = width * sqrt(variance) (pass 1) of every date
__global__ void __launch_bounds__(kProdThreads) dd_moment_finish_kernel(const double* partials, int blocks, int P,
                                                                        int pass, double width, double* out)
{
    const int e = blockIdx.x;
    dd acc{0.0, 0.0};
    for (int b = threadIdx.x; b < blocks; b += blockDim.x)
        acc = dd_add(acc, dd{partials[((size_t)e * blocks + b) * 2], partials[((size_t)e * blocks + b) * 2 + 1]});
    acc = block_dd_sum(acc);
    if (threadIdx.x == 0) {
        const double v = (acc.hi + acc.lo) / (double)P;
        out[e] = pass == 0 ? v : width * sqrt(v);
    }
}

}  // namespace

int launch_bermudan_dd_weights(const BermudanLaunch& a, const BermudanDdScratch& sc, int P, double num0, double width,
                               cudaStream_t s)
{
    std::vector<int> ex_period;
    for (int q = 0; q < a.nper; q++)
        if (a.per[q].exercisable) ex_period.push_back(q);
    const int ne = (int)ex_period.size();
    const int blocks = bermudan_blocks(P);
    KernelTimer kt(K_ADJOINT, s, 2 * (ne > 0 ? 2 : 0) + ne + 1);
    if (ne > 0) {
        const int mb = std::min(64, std::max(1, (P + kProdThreads - 1) / kProdThreads));
        const dim3 grid(mb, ne);
        dd_moment_kernel<<<grid, kProdThreads, 0, s>>>(sc.d_rec, P, nullptr, sc.d_moments);
        dd_moment_finish_kernel<<<ne, kProdThreads, 0, s>>>(sc.d_moments, mb, P, 0, width, sc.d_mean);
        dd_moment_kernel<<<grid, kProdThreads, 0, s>>>(sc.d_rec, P, sc.d_mean, sc.d_moments);
        dd_moment_finish_kernel<<<ne, kProdThreads, 0, s>>>(sc.d_moments, mb, P, 1, width, sc.d_eps);
        LMM_CUDA(cudaGetLastError());
    }
    DdSweepParams prm;
    std::memset(&prm, 0, sizeof(prm));
    prm.P = P;
    prm.nper = a.nper;
    prm.callable = a.callable;
    prm.num0 = num0;
    prm.rec = sc.d_rec;
    prm.basis = sc.d_basis;
    prm.eps = sc.d_eps;
    prm.betap = sc.d_betap;
    prm.vbar = sc.d_vbar;
    prm.ubar = sc.d_ubar;
    prm.omega = sc.d_omega;
    prm.partials = sc.d_partials;
    prm.ne = ne;
    for (int k = 0; k <= ne; k++) {
        prm.prev_e = k - 1;
        prm.cur_e = k < ne ? k : -1;
        prm.q_lo = k == 0 ? 0 : ex_period[k - 1];
        prm.q_hi = k < ne ? ex_period[k] : a.nper;
        prm.svd_cur = k < ne ? sc.d_svd + (size_t)k * kSvdStride : nullptr;
        if (sc.basis_fp32) dd_sweep_kernel<float><<<blocks, kProdThreads, 0, s>>>(prm);
        else dd_sweep_kernel<double><<<blocks, kProdThreads, 0, s>>>(prm);
        LMM_CUDA(cudaGetLastError());
    }
    return LMM_OK;
}

// ------------------------------------------------------------------ allocation-free mean / standard error
// The allocation-free variant of reduce_mean_stderr keeps its scratch (the block partials
// of the two compensated sums and the two results) in this file-scope array instead of
// memory from the pool.  Every GPU that loads the library holds these 8,208 bytes until
// the process exits.
namespace {
constexpr int kNoAllocBlocks = 512;
constexpr int64_t kNoAllocMaxValues = (int64_t)1 << 30;
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocBlocks + 2];

// Device address of the scratch on the current device, looked up once per device with
// that device current.  Host code must not pass g_noalloc_scratch itself to a kernel:
// on the host that name is only a stand-in for the device symbol.
static int noalloc_scratch_address(double** out)
{
    int dev = 0;
    LMM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(LMM_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[dev];
    return LMM_OK;
}

}  // namespace lmm

extern "C" int lmm_values_mean_stderr_noalloc(const double* d_values, int64_t num_values, void* stream,
                                              double* out_mean, double* out_error)
{
    using namespace lmm;
    if (!d_values || !out_mean) return fail(LMM_ERR_INVALID, "lmm_values_mean_stderr_noalloc: null argument");
    if (num_values < 1 || num_values > kNoAllocMaxValues)
        return fail(LMM_ERR_INVALID, "lmm_values_mean_stderr_noalloc: num_values must be in [1, 2^30]");
    double* scratch = nullptr;
    int rc = noalloc_scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int P = (int)num_values;
    const int blocks = grid_for(P, 256, kNoAllocBlocks);
    // Each block overwrites its own partial and the finishing kernels overwrite the
    // results, so nothing left by an earlier call is read and nothing needs clearing.
    double* partials = scratch;
    double* res = scratch + 2 * kNoAllocBlocks;
    sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, nullptr, partials);
    finish_partials_kernel<<<1, 256, 0, s>>>(partials, blocks, P, res);
    sum_partials_kernel<<<blocks, 256, 0, s>>>(d_values, P, res, partials);
    finish_partials_kernel<<<1, 256, 0, s>>>(partials, blocks, P, res + 1);
    LMM_CUDA(cudaGetLastError());
    double h[2];
    LMM_CUDA(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, s));
    LMM_CUDA(cudaStreamSynchronize(s));
    *out_mean = h[0];
    if (out_error) *out_error = P > 1 ? sqrt(h[1]) / sqrt((double)P) : 0.0;
    return LMM_OK;
}
