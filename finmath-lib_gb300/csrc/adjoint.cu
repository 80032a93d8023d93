// adjoint.cu -- K6: adjoint (reverse-mode) sensitivities of the Bermudan swaption value to
// the initial forwards (deltas) and to every volatility-matrix entry sigma_{i,j} (vegas).
//
// This is the GPU counterpart of finmath-lib's RandomVariableDifferentiable.getGradient()
// (montecarlo/automaticdifferentiation/RandomVariableDifferentiable.java:56-75) with the
// initial state and the volatility matrix as leaves, as in the reference's
// LIBORMarketModelNormalAADSensitivitiesTest (:343-355, :431-434).  Instead of a tape of
// random-variable operations (RandomVariableDifferentiableAAD.java:80-219), the adjoint of
// the Euler-log step is written by hand:
//
//   forward  os_j = L_j/(L_j + 1/d_j),  S_k += os_j lam_jk,  mu_j = sum_k S_k lam_jk - sigma_ij^2/2,
//            Y_j' = Y_j + mu_j dt + sum_k dW_k lam_jk,  L_j' = exp(Y_j')          (lam_jk = sigma_ij f_jk)
//   reverse  mubar_j = Ybar'_j dt,  R_k = sum_{l>=j} mubar_l lam_lk (a reverse running sum),
//            osbar_j = sum_k lam_jk R_k,  Ybar_j = Ybar'_j + osbar_j os_j (1 - os_j),
//            lambar_jk = mubar_j S_k^(j) + os_j R_k + Ybar'_j dW_k,
//            sigmabar_ij = sum_k lambar_jk f_jk - mubar_j sigma_ij
//
// so a reverse step costs O(N F) like the forward one.  The forward rates come from the
// path kernel's checkpoints: with stride 1 (the default: HBM holds every state) one sweep
// reads them directly; with a larger stride each segment is regenerated from its
// checkpoint into a global buffer before that segment's sweep, by the path kernels' own
// step (the FP32 component step of euler_fp32.cuh; the FP64 fast kernel's REPLAY
// instantiation), so the regenerated rates are the stored ones bit for bit and the Greeks
// do not depend on the stride.  The Bermudan's exercise
// decisions are frozen from the forward valuation (regression coefficients fixed); the seed
// kernel turns each path's realised cash flows into adjoints of the fixings L_m(T_m),
// through the payment numeraires, their cross-path adjustment a_l = mean(1/N_l)
// (:869-874) and the numeraire chain.
#include <math_constants.h>

#include <algorithm>
#include <cstring>
#include <cmath>

#include "lmm_internal.h"
#include "reduce.cuh"
#include "dfloat.cuh"
#include "euler_fp32.cuh"
#include "unroll_range.cuh"

namespace lmm {
namespace {

constexpr int kMaxStride = 16;

template <typename R>
__device__ __forceinline__ R fexp(R x);
template <>
__device__ __forceinline__ float fexp<float>(float x) { return __expf(x); }
template <>
__device__ __forceinline__ double fexp<double>(double x) { return exp(x); }
template <typename R>
__device__ __forceinline__ R flog(R x);
template <>
__device__ __forceinline__ float flog<float>(float x) { return __logf(x); }
template <>
__device__ __forceinline__ double flog<double>(double x) { return log(x); }
template <typename R>
__device__ __forceinline__ R fdiv(R a, R b);
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }
template <>
__device__ __forceinline__ double fdiv<double>(double a, double b) { return a / b; }

// vector unit of the factor-matrix rows (one 16-byte load)
template <typename R>
struct Vec;
template <>
struct Vec<float> {
    using T = float4;
    static constexpr int W = 4;
    static __device__ __forceinline__ void unpack(const T& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <>
struct Vec<double> {
    using T = double2;
    static constexpr int W = 2;
    static __device__ __forceinline__ void unpack(const T& v, double* o) { o[0] = v.x; o[1] = v.y; }
};

// two factors at a time: FP32 on the paired FMA (__ffma2_rn), FP64 as two scalar FMAs
template <typename R>
struct Pair;
template <>
struct Pair<float> {
    using T = float2;
    static __device__ __forceinline__ T mk(float x, float y) { return make_float2(x, y); }
    static __device__ __forceinline__ T fma(T a, T b, T c) { return __ffma2_rn(a, b, c); }
};
template <>
struct Pair<double> {
    using T = double2;
    static __device__ __forceinline__ T mk(double x, double y) { return make_double2(x, y); }
    static __device__ __forceinline__ T fma(T a, T b, T c) { return make_double2(::fma(a.x, b.x, c.x), ::fma(a.y, b.y, c.y)); }
};

// row pitch of the factor table f[T][N][pitch]: FMAX rounded up to whole 16-byte vectors
template <typename R, int FMAX>
__host__ __device__ constexpr int f_pitch() { return (FMAX + Vec<R>::W - 1) / Vec<R>::W * Vec<R>::W; }

template <typename R>
struct AdjTables {
    const R* lam;       // [T][N][F] factor loadings (replay)
    const R* var_half;  // [T][N] -variance/2 (replay)
    const R* f;         // [T][N][pitch] factor matrix rows f_jk = lam_jk / sigma_j, zero padded
    const R* sigma;     // [T][N]
    const R* inv_delta; // [N]
    const R* dt;        // [T]
    const void* dw;     // [T][F][P] of type R
};

struct RevParams {
    int T, N, F, P;
    int n_lo, n_hi;      // steps [n_lo, n_hi) of this sweep, in reverse
    int t_end, n_eff;    // product horizon: states t_end, components 0..n_eff-1
    int base_step;       // states[] holds the steps base_step, base_step+1, ...
    int seed;            // 1: start from the seeds at t_end, else from ybar
    int capped;
    int normal;          // NORMAL state space: the state is L itself (else log L)
    double cap;
    const int* first;     // [T]
    const double* init;   // [N]
    const void* seeds;    // [N][P] (type R) d value / d L_m(T_m), already divided by P
    const void* states;   // [slots][N][P] forward rates L (type R)
    void* ybar;           // [N][P] (type R): adjoint of log L carried between sweeps
    double* vega_partials;   // [warps][T][N]
    double* delta_partials;  // [warps][N]
};

// Sums over the warp's 32 lanes of eight values a lane holds (v[0..7], overwritten): three
// transposed exchange levels (offsets 16, 8, 4), at each of which a lane keeps half of what it
// holds and adds its partner's copy of that half, then two plain levels (offsets 2, 1).
// Every lane returns the total of value (lane >> 2) & 7; the order of the additions is fixed.
// All 32 lanes must call it.  It takes 7 exchanges and 2 plain shuffles for eight sums, and
// no shared memory (a transpose buffer of the warp's per-component values would hold
// NMAX x 32 values per warp).
template <typename R>
__device__ __forceinline__ R warp_sum8_transposed(R (&v)[8], int lane)
{
    {
        const bool up = (lane & 16) != 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const R send = up ? v[i] : v[i + 4];
            const R keep = up ? v[i + 4] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
    }
    {
        const bool up = (lane & 8) != 0;
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const R send = up ? v[i] : v[i + 2];
            const R keep = up ? v[i + 2] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
    }
    {
        const bool up = (lane & 4) != 0;
        const R send = up ? v[0] : v[1];
        const R keep = up ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    R t = v[0];
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    return t;
}

// FP32 sweeps stage each step's factor table in shared memory; FP64 ones read it from L1/L2
template <typename R>
__host__ __device__ constexpr bool rev_stage_tables() { return sizeof(R) == 4; }

// one 16-byte vector of a factor row (shared memory when staged, else the read-only path)
template <typename R>
__device__ __forceinline__ typename Vec<R>::T load_row(const R* row, int q)
{
    const typename Vec<R>::T* v = reinterpret_cast<const typename Vec<R>::T*>(row) + q;
    if (rev_stage_tables<R>()) return *v;
    return __ldg(v);
}

// asynchronous 4- or 8-byte copy global -> shared (completes at cp_async_wait)
template <typename R>
__device__ __forceinline__ void cp_async(R* dst, const R* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(R) == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// resident warps per SM the grid is sized for (the shared memory of 40 components holds it
// there): 12 in FP32, 8 in FP64
template <typename R>
__host__ __device__ constexpr int rev_warps_per_sm() { return sizeof(R) == 4 ? 12 : 8; }
template <typename R, int TH>
__host__ __device__ constexpr int rev_min_blocks() { return rev_warps_per_sm<R>() * 32 / TH > 0 ? rev_warps_per_sm<R>() * 32 / TH : 1; }

// shared memory of the reverse kernel: the step buffer [NMAX][TH] of one step's forward
// rates, the adjoint buffer [NMAX][TH], two increment buffers [2][FMAX][TH], and (FP32) per
// warp two copies of a step's factor rows and volatilities [2][NMAX*pitch + NMAX]
template <typename R, int NMAX, int FMAX>
__host__ __device__ constexpr int rev_table_elems() { return NMAX * f_pitch<R, FMAX>() + NMAX; }
template <typename R, int NMAX, int FMAX, int TH>
__host__ __device__ constexpr size_t rev_smem_bytes()
{
    return (size_t)(2 * NMAX + 2 * FMAX) * TH * sizeof(R) +
           (rev_stage_tables<R>() ? (size_t)(TH / 32) * 2 * rev_table_elems<R, NMAX, FMAX>() * sizeof(R) : 0);
}

// Reverse sweep over the steps [n_lo, n_hi) of every path, from stored forward rates.
// One thread per path (grid-stride over path batches; the partition is fixed by the grid, so
// the per-warp partial sums and their order do not depend on the checkpoint stride).  The
// path's forward rates of the step and its adjoint vector Ybar live in the thread's own
// columns of shared memory, so that both component passes are rolled loops over the live
// components [first, NE): fully unrolled over 40 components the sweep overflowed the
// instruction cache (a fifth of the fetches missed).  The reverse pass runs over chunks of
// eight components, unrolled within a chunk, and takes the per-warp vega sums of each chunk
// by a transposed shuffle reduction.  Each thread prefetches its path's forward rates and
// increments of the next step (cp.async) once the current step's rates are consumed; the
// increments alternate between two buffers.  In FP32 each warp also stages the next step's
// factor rows and volatilities (16-byte copies by its lanes, two buffers), read back as
// broadcast shared-memory vectors.  The per-warp partial sums are fire-and-forget
// reductions (one lane per entry, so their order is program order).
template <typename R, int NMAX, int FMAX, int TH>
__global__ void __launch_bounds__(TH, rev_min_blocks<R, TH>()) reverse_kernel(const RevParams a, const AdjTables<R> tb)
{
    constexpr int FP = f_pitch<R, FMAX>();
    static_assert(NMAX % 8 == 0, "the per-warp sums work on chunks of eight components");
    using V = Vec<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    R* sbuf = reinterpret_cast<R*>(smem_raw) + tid;  // [NMAX][TH]: the step's forward rates, own column
    R* ybuf = sbuf + NMAX * TH;                       // [NMAX][TH]: Ybar, own column
    R* wbuf = ybuf + NMAX * TH;                       // [2][FMAX][TH]: increments, own column
    constexpr int TE_ = rev_table_elems<R, NMAX, FMAX>();
    R* tbuf = reinterpret_cast<R*>(smem_raw) + (2 * NMAX + 2 * FMAX) * TH +
              (size_t)warp * 2 * TE_;                 // [2][NMAX*FP + NMAX] of this warp
    const int N = a.N, F = a.F, NE = a.n_eff;
    const size_t gw = (size_t)blockIdx.x * (TH / 32) + warp;
    double* vp = a.vega_partials + gw * a.T * N;
    const R* states = static_cast<const R*>(a.states);
    const R* dW = static_cast<const R*>(tb.dw);
    const R cap = (R)a.cap;
    // 1/delta_j, read in every iteration of both component passes
    __shared__ R inv_delta_s[NMAX];
    for (int j = tid; j < NMAX; j += TH) inv_delta_s[j] = j < NE ? tb.inv_delta[j] : R(1);
    __syncthreads();

    for (int base = blockIdx.x * TH; base < a.P; base += gridDim.x * TH) {
        const int p = base + tid;
        const bool active = p < a.P;
        // this path's forward rates (components first..NE-1) and increments of step n, and
        // (FP32) the warp's copy of the step's factor rows and volatilities
        auto prefetch = [&](int n) {
            if (rev_stage_tables<R>()) {
                R* tb_dst = tbuf + (n & 1) * TE_;
                const R* fsrc = tb.f + (size_t)n * N * FP;
                constexpr int kVec = 16 / sizeof(R);
                for (int q = lane; q < NE * FP / kVec; q += 32) cp_async16(tb_dst + q * kVec, fsrc + q * kVec);
                for (int j = lane; j < NE; j += 32) cp_async(tb_dst + NMAX * FP + j, tb.sigma + (size_t)n * N + j);
            }
            if (active) {
                const int fst = __ldg(a.first + n);
                const R* Ls = states + (size_t)(n - a.base_step) * N * a.P + p;
                for (int j = fst; j < NE; j++) cp_async(sbuf + j * TH, Ls + (size_t)j * a.P);
                R* wb = wbuf + (n & 1) * FMAX * TH;
#pragma unroll
                for (int k = 0; k < FMAX; k++)
                    if (k < F) cp_async(wb + k * TH, dW + ((size_t)n * F + k) * a.P + p);
            }
            cp_async_commit();
        };
        prefetch(a.n_hi - 1);
        if (a.seed) {
            const R* Ls = states + (size_t)(a.t_end - a.base_step) * N * a.P;
            for (int j = 0; j < NE; j++) {
                R yb = R(0);
                if (active) {
                    const R sd = static_cast<const R*>(a.seeds)[(size_t)j * a.P + p];
                    if (a.normal) {
                        yb = sd;  // the state is L: its adjoint is the seed
                    } else {
                        const R L = Ls[(size_t)j * a.P + p];
                        if (!(a.capped && L >= cap)) yb = sd * L;
                    }
                }
                ybuf[j * TH] = yb;
            }
        } else {
            const R* yb = static_cast<const R*>(a.ybar);
            for (int j = 0; j < NE; j++) ybuf[j * TH] = active ? yb[(size_t)j * a.P + p] : R(0);
        }

        for (int n = a.n_hi - 1; n >= a.n_lo; n--) {
            const int first = __ldg(a.first + n);
            const R dt = tb.dt[n];
            cp_async_wait();
            if (rev_stage_tables<R>()) __syncwarp();  // the warp's staged table is visible to all its lanes
            const R* sig = rev_stage_tables<R>() ? tbuf + (n & 1) * TE_ + NMAX * FP : tb.sigma + (size_t)n * N;
            const R* frow = rev_stage_tables<R>() ? tbuf + (n & 1) * TE_ : tb.f + (size_t)n * N * FP;
            // factor pairs (2m, 2m+1); the factor rows are zero beyond F, so padded pairs add nothing
            constexpr int FH = (FMAX + 1) / 2;
            using PT = typename Pair<R>::T;
            PT dw[FH], S[FH], Rk[FH];
#pragma unroll
            for (int m = 0; m < FH; m++) {
                const int k0 = 2 * m, k1 = 2 * m + 1;
                dw[m] = Pair<R>::mk((k0 < F && active) ? wbuf[((n & 1) * FMAX + k0) * TH] : R(0),
                                    (k1 < F && active) ? wbuf[((n & 1) * FMAX + (k1 < FMAX ? k1 : 0)) * TH] : R(0));
                S[m] = Pair<R>::mk(R(0), R(0));
                Rk[m] = Pair<R>::mk(R(0), R(0));
            }
            // os_j = L/(L + 1/d) (LOGNORMAL) or d/(1 + d L) = 1/(L + 1/d) (NORMAL)
            auto os_of = [&](int j, R L) { return fdiv<R>(a.normal ? R(1) : L, L + inv_delta_s[j]); };
            // forward pass of the step: S_k = sum_j os_j sigma_j f_jk
            unsigned long long capmask = 0ull;  // capped models have at most 64 components
#pragma unroll 2
            for (int j = first; j < NE; j++) {
                const R L = active ? sbuf[j * TH] : R(0);
                if (a.capped && L >= cap && j < 64) capmask |= 1ull << j;
                const R oss2s = os_of(j, L) * sig[j];
                R fr[FP];
#pragma unroll
                for (int q = 0; q < FP / V::W; q++) V::unpack(load_row<R>(frow + j * FP, q), fr + q * V::W);
                const PT oss2 = Pair<R>::mk(oss2s, oss2s);
#pragma unroll
                for (int m = 0; m < FH; m++) S[m] = Pair<R>::fma(oss2, Pair<R>::mk(fr[2 * m], fr[2 * m + 1]), S[m]);
            }
            // reverse pass over the components, by chunks of eight from the chunk of NE-1 down
            // to the chunk of first; each chunk's per-warp vega sums as it completes
            for (int c = (NE - 1) >> 3; c >= (first >> 3); c--) {
                R vch[8];
#pragma unroll
                for (int i = 7; i >= 0; i--) {
                    const int j = 8 * c + i;
                    vch[i] = R(0);
                    if (j < NE && j >= first) {
                        const R L = active ? sbuf[j * TH] : R(0);
                        const R o = os_of(j, L);
                        const R sg = sig[j];
                        const R yb = ybuf[j * TH];
                        const R mub = yb * dt;
                        const R mubs = mub * sg;
                        const R oss = o * sg;
                        R fr[FP];
#pragma unroll
                        for (int q = 0; q < FP / V::W; q++) V::unpack(load_row<R>(frow + j * FP, q), fr + q * V::W);
                        const PT mubs2 = Pair<R>::mk(mubs, mubs), noss2 = Pair<R>::mk(-oss, -oss);
                        PT A2 = Pair<R>::mk(R(0), R(0)), B2 = A2, D2 = A2;
#pragma unroll
                        for (int m = 0; m < FH; m++) {
                            const PT f2 = Pair<R>::mk(fr[2 * m], fr[2 * m + 1]);
                            Rk[m] = Pair<R>::fma(mubs2, f2, Rk[m]);  // R_k = sum_{l>=j} mubar_l lam_lk
                            A2 = Pair<R>::fma(Rk[m], f2, A2);
                            B2 = Pair<R>::fma(S[m], f2, B2);         // S^(j)
                            D2 = Pair<R>::fma(dw[m], f2, D2);
                            S[m] = Pair<R>::fma(noss2, f2, S[m]);    // S^(j-1)
                        }
                        const R A = A2.x + A2.y, B = B2.x + B2.y, D = D2.x + D2.y;
                        // sigmabar_ij = sum_k lambar_jk f_jk - mubar_j sigma_ij with
                        // lambar_jk = mubar_j S_k + os_j R_k + Ybar'_j dW_k
                        // (NORMAL: no -variance/2 drift term, so no -mubar_j sigma_ij)
                        vch[i] = active ? (mub * B + o * A + yb * D - (a.normal ? R(0) : mubs)) : R(0);
                        // osbar_j = sigma_j A;  d os_j / d Y_j = os_j (1 - os_j) (LOGNORMAL, zero
                        // where capped), d os_j / d L_j = -os_j^2 (NORMAL)
                        if (a.normal) ybuf[j * TH] = yb - (sg * A) * (o * o);
                        else if (!(a.capped && j < 64 && ((capmask >> j) & 1ull))) ybuf[j * TH] = yb + (sg * A) * (o * (R(1) - o));
                    }
                }
                const R sum = warp_sum8_transposed<R>(vch, lane);
                const int r = 8 * c + ((lane >> 2) & 7);
                if ((lane & 3) == 0 && r < NE && r >= first) atomicAdd(vp + (size_t)n * N + r, (double)sum);
            }
            // the step's rates are consumed -- fetch the next step
            if (n - 1 >= a.n_lo) prefetch(n - 1);
        }

        if (a.n_lo > 0) {
            R* yb = static_cast<R*>(a.ybar);
            if (active)
                for (int j = 0; j < NE; j++) yb[(size_t)j * a.P + p] = ybuf[j * TH];
        } else {
            // deltas: Y_0 = log(L_0(0)) -> d value / d L_0 = Ybar / L_0, the uniform division
            // applied to the warp's sum (one division per component and warp, not per path);
            // NORMAL: the state is L_0 itself
            for (int c = 0; 8 * c < NE; c++) {
                R v8[8];
#pragma unroll
                for (int i = 0; i < 8; i++) v8[i] = (8 * c + i < NE && active) ? ybuf[(8 * c + i) * TH] : R(0);
                const R sum = warp_sum8_transposed<R>(v8, lane);
                const int r = 8 * c + ((lane >> 2) & 7);
                if ((lane & 3) == 0 && r < NE) atomicAdd(a.delta_partials + gw * N + r, a.normal ? (double)sum : (double)sum / a.init[r]);
            }
        }
    }
    cp_async_wait();
}

// Replays the Euler-log steps [n0, n_stop) of every path from the checkpoint at n0 (forward
// rates) and stores the forward rates of the steps n0..n_stop in seg[0..n_stop-n0].
struct ReplayParams {
    int T, N, F, P, n0, n_stop, n_eff, capped, normal;
    double cap;
    const int* first;
    const void* ckpt_slot;  // [N][P] forward rates at n0
    void* seg;              // [n_stop-n0+1][N][P]
};

template <typename R, int NMAX, int FMAX>
__global__ void __launch_bounds__(128) replay_kernel(const ReplayParams a, const AdjTables<R> tb)
{
    const int p = blockIdx.x * 128 + threadIdx.x;
    if (p >= a.P) return;
    const int N = a.N, F = a.F, NE = a.n_eff, P = a.P;
    const R* ck = static_cast<const R*>(a.ckpt_slot);
    R* seg = static_cast<R*>(a.seg);
    const R* dW = static_cast<const R*>(tb.dw);
    const R cap = (R)a.cap;
    R Y[NMAX], L[NMAX];
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        L[j] = (j < NE) ? ck[(size_t)j * P + p] : R(0);
        Y[j] = (j < NE) ? (a.normal ? L[j] : flog<R>(L[j])) : R(0);
        if (j < NE) seg[(size_t)j * P + p] = L[j];
    }
    for (int n = a.n0; n < a.n_stop; n++) {
        const int first = __ldg(a.first + n);
        const R dt = tb.dt[n];
        const R* lam = tb.lam + (size_t)n * N * F;
        R dw[FMAX], S[FMAX];
#pragma unroll
        for (int k = 0; k < FMAX; k++) {
            dw[k] = (k < F) ? dW[((size_t)n * F + k) * P + p] : R(0);
            S[k] = R(0);
        }
#pragma unroll
        for (int j = 0; j < NMAX; j++) {
            if (j < NE && j >= first) {
                const R os = fdiv<R>(a.normal ? R(1) : L[j], L[j] + tb.inv_delta[j]);
                R mu = a.normal ? R(0) : tb.var_half[(size_t)n * N + j], diff = R(0);
#pragma unroll
                for (int k = 0; k < FMAX; k++) {
                    if (k < F) {
                        const R l = lam[j * F + k];
                        S[k] = S[k] + os * l;
                        mu = mu + S[k] * l;
                        diff = diff + dw[k] * l;
                    }
                }
                Y[j] = Y[j] + (mu * dt + diff);
                R v = a.normal ? Y[j] : fexp<R>(Y[j]);
                if (a.capped && v > cap) v = cap;
                L[j] = v;
            }
        }
        R* out = seg + (size_t)(n + 1 - a.n0) * N * P;
#pragma unroll
        for (int j = 0; j < NMAX; j++)
            if (j < NE) out[(size_t)j * P + p] = L[j];
    }
}

// ------------------------------------------------------------------ FP64 sweep on float pairs
// The FP64 form's reverse sweep with its arithmetic in double-float pairs on the FP32 pipe
// (about 2^-44 relative per operation; the FP64 adjoint is checked to 1e-6): the FP64 sweep
// ran about 60 FP64 fused multiply-adds per component-step on a pipe that issues at 1/64 of
// the FP32 rate.  Rates, adjoints and increments stay FP64 in memory (split into pairs in
// integer operations as they are read, rebuilt by one FP64 addition as they are written);
// the factor pairs' running sums use the path kernel's paired Dot2 step (df_dot_acc2).  The
// products are explicit __fmul_rn / __fmaf_rn so that FMA contraction cannot break the
// error-free transforms.
struct DF {
    float h, l;
};
__device__ __forceinline__ DF df_of(double x)
{
    DF r;
    df_split_int(x, r.h, r.l);
    return r;
}
__device__ __forceinline__ double df_val(DF a) { return f32_to_f64_int(a.h) + f32_to_f64_int(a.l); }
__device__ __forceinline__ DF df_norm(float s, float e)
{
    DF r;
    r.h = __fadd_rn(s, e);
    r.l = __fsub_rn(e, __fsub_rn(r.h, s));
    return r;
}
__device__ __forceinline__ DF df_mul(DF a, DF b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_norm(p, e);
}
__device__ __forceinline__ DF df_add(DF a, DF b)
{
    const float s = __fadd_rn(a.h, b.h);
    const float z = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, z)), __fsub_rn(b.h, z));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return df_norm(s, e);
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
// n / d for d > 0: the approximate FP32 reciprocal, then the residual's quotient
__device__ __forceinline__ DF df_div(DF n, DF d)
{
    const float r0 = euler32::rcp_approx(d.h);
    const float q0 = __fmul_rn(n.h, r0);
    const float p = __fmul_rn(q0, d.h);
    const float e = __fmaf_rn(q0, d.h, -p);
    float res = __fsub_rn(__fsub_rn(n.h, p), e);
    res = __fadd_rn(res, n.l);
    res = __fmaf_rn(-q0, d.l, res);
    return df_norm(q0, __fmul_rn(res, r0));
}

template <int NMAX, int FMAX, int TH>
__global__ void __launch_bounds__(TH, rev_min_blocks<double, TH>()) reverse_df_kernel(const RevParams a, const AdjTables<double> tb)
{
    using R = double;
    constexpr int FP = f_pitch<R, FMAX>();
    static_assert(NMAX % 8 == 0 && FMAX % 2 == 0, "chunks of eight components, factor pairs");
    using V = Vec<R>;
    constexpr int FH = FMAX / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    R* sbuf = reinterpret_cast<R*>(smem_raw) + tid;  // [NMAX][TH]: the step's forward rates, own column
    R* ybuf = sbuf + NMAX * TH;                       // [NMAX][TH]: Ybar, own column
    R* wbuf = ybuf + NMAX * TH;                       // [2][FMAX][TH]: increments, own column
    const int N = a.N, F = a.F, NE = a.n_eff;
    const size_t gw = (size_t)blockIdx.x * (TH / 32) + warp;
    double* vp = a.vega_partials + gw * a.T * N;
    const R* states = static_cast<const R*>(a.states);
    const R* dW = static_cast<const R*>(tb.dw);
    const R cap = a.cap;
    __shared__ float invd_h[NMAX], invd_l[NMAX];
    for (int j = tid; j < NMAX; j += TH) {
        const DF v = df_of(j < NE ? tb.inv_delta[j] : 1.0);
        invd_h[j] = v.h;
        invd_l[j] = v.l;
    }
    __syncthreads();

    for (int base = blockIdx.x * TH; base < a.P; base += gridDim.x * TH) {
        const int p = base + tid;
        const bool active = p < a.P;
        auto prefetch = [&](int n) {
            if (active) {
                const int fst = __ldg(a.first + n);
                const R* Ls = states + (size_t)(n - a.base_step) * N * a.P + p;
                for (int j = fst; j < NE; j++) cp_async(sbuf + j * TH, Ls + (size_t)j * a.P);
                R* wb = wbuf + (n & 1) * FMAX * TH;
#pragma unroll
                for (int k = 0; k < FMAX; k++)
                    if (k < F) cp_async(wb + k * TH, dW + ((size_t)n * F + k) * a.P + p);
            }
            cp_async_commit();
        };
        prefetch(a.n_hi - 1);
        if (a.seed) {
            const R* Ls = states + (size_t)(a.t_end - a.base_step) * N * a.P;
            for (int j = 0; j < NE; j++) {
                R yb = R(0);
                if (active) {
                    const R sd = static_cast<const R*>(a.seeds)[(size_t)j * a.P + p];
                    if (a.normal) {
                        yb = sd;
                    } else {
                        const R L = Ls[(size_t)j * a.P + p];
                        if (!(a.capped && L >= cap)) yb = sd * L;
                    }
                }
                ybuf[j * TH] = yb;
            }
        } else {
            const R* yb = static_cast<const R*>(a.ybar);
            for (int j = 0; j < NE; j++) ybuf[j * TH] = active ? yb[(size_t)j * a.P + p] : R(0);
        }

        for (int n = a.n_hi - 1; n >= a.n_lo; n--) {
            const int first = __ldg(a.first + n);
            const DF dt = df_of(tb.dt[n]);
            cp_async_wait();
            const R* sig = tb.sigma + (size_t)n * N;
            const R* frow = tb.f + (size_t)n * N * FP;
            // factor pairs (2m, 2m+1) as float pairs: high parts (lanes x, y) and low parts
            float2 dwh[FH], dwl[FH], Sh[FH], Sl[FH], Rh[FH], Rl[FH];
#pragma unroll
            for (int m = 0; m < FH; m++) {
                const int k0 = 2 * m, k1 = 2 * m + 1;
                const DF w0 = df_of((k0 < F && active) ? wbuf[((n & 1) * FMAX + k0) * TH] : R(0));
                const DF w1 = df_of((k1 < F && active) ? wbuf[((n & 1) * FMAX + k1) * TH] : R(0));
                dwh[m] = make_float2(w0.h, w1.h);
                dwl[m] = make_float2(w0.l, w1.l);
                Sh[m] = Sl[m] = Rh[m] = Rl[m] = make_float2(0.0f, 0.0f);
            }
            // os_j = L/(L + 1/d) (LOGNORMAL) or 1/(L + 1/d) (NORMAL)
            auto os_of = [&](int j, DF L) {
                const DF den = df_add(L, DF{invd_h[j], invd_l[j]});
                return df_div(a.normal ? DF{1.0f, 0.0f} : L, den);
            };
            // the factor row of component j as pairs (hi, lo, -hi)
            auto row_of = [&](int j, float2 (&fh)[FH], float2 (&fl)[FH], float2 (&fn)[FH]) {
                R fr[FP];
#pragma unroll
                for (int q = 0; q < FP / V::W; q++) V::unpack(load_row<R>(frow + j * FP, q), fr + q * V::W);
#pragma unroll
                for (int m = 0; m < FH; m++) {
                    const DF f0 = df_of(fr[2 * m]), f1 = df_of(fr[2 * m + 1]);
                    fh[m] = make_float2(f0.h, f1.h);
                    fl[m] = make_float2(f0.l, f1.l);
                    fn[m] = make_float2(-f0.h, -f1.h);
                }
            };
            unsigned long long capmask = 0ull;
#pragma unroll 2
            for (int j = first; j < NE; j++) {
                const R Lr = active ? sbuf[j * TH] : R(0);
                if (a.capped && Lr >= cap && j < 64) capmask |= 1ull << j;
                const DF oss = df_mul(os_of(j, df_of(Lr)), df_of(sig[j]));
                const float2 oh = make_float2(oss.h, oss.h), ol = make_float2(oss.l, oss.l);
                float2 fh[FH], fl[FH], fn[FH];
                row_of(j, fh, fl, fn);
#pragma unroll
                for (int m = 0; m < FH; m++) df_dot_acc2(Sh[m], Sl[m], oh, ol, fh[m], fl[m], fn[m]);  // S_k += os sigma f_k
            }
            for (int c = (NE - 1) >> 3; c >= (first >> 3); c--) {
                R vch[8];
#pragma unroll
                for (int i = 7; i >= 0; i--) {
                    const int j = 8 * c + i;
                    vch[i] = R(0);
                    if (j < NE && j >= first) {
                        const DF L = df_of(active ? sbuf[j * TH] : R(0));
                        const DF o = os_of(j, L);
                        const DF sg = df_of(sig[j]);
                        const DF yb = df_of(ybuf[j * TH]);
                        const DF mub = df_mul(yb, dt);
                        const DF mubs = df_mul(mub, sg);
                        const DF oss = df_mul(o, sg);
                        float2 fh[FH], fl[FH], fn[FH];
                        row_of(j, fh, fl, fn);
                        const float2 mh = make_float2(mubs.h, mubs.h), ml = make_float2(mubs.l, mubs.l);
                        const float2 nh = make_float2(-oss.h, -oss.h), nl = make_float2(-oss.l, -oss.l);
                        float2 Ah = make_float2(0.0f, 0.0f), Al = Ah, Bh = Ah, Bl = Ah, Dh = Ah, Dl = Ah;
#pragma unroll
                        for (int m = 0; m < FH; m++) {
                            df_dot_acc2(Rh[m], Rl[m], mh, ml, fh[m], fl[m], fn[m]);       // R_k += mubar lam_k
                            df_dot_acc2(Ah, Al, Rh[m], Rl[m], fh[m], fl[m], fn[m]);       // A += R_k f_k
                            df_dot_acc2(Bh, Bl, Sh[m], Sl[m], fh[m], fl[m], fn[m]);       // B += S^(j)_k f_k
                            df_dot_acc2(Dh, Dl, dwh[m], dwl[m], fh[m], fl[m], fn[m]);     // D += dW_k f_k
                            df_dot_acc2(Sh[m], Sl[m], nh, nl, fh[m], fl[m], fn[m]);       // S^(j-1)_k
                        }
                        const DF A = df_add(DF{Ah.x, Al.x}, DF{Ah.y, Al.y});
                        const DF B = df_add(DF{Bh.x, Bl.x}, DF{Bh.y, Bl.y});
                        const DF D = df_add(DF{Dh.x, Dl.x}, DF{Dh.y, Dl.y});
                        DF v = df_add(df_add(df_mul(mub, B), df_mul(o, A)), df_mul(yb, D));
                        if (!a.normal) v = df_add(v, df_neg(mubs));
                        vch[i] = active ? df_val(v) : R(0);
                        const DF sa = df_mul(sg, A);
                        if (a.normal) ybuf[j * TH] = df_val(df_add(yb, df_neg(df_mul(sa, df_mul(o, o)))));
                        else if (!(a.capped && j < 64 && ((capmask >> j) & 1ull)))
                            ybuf[j * TH] = df_val(df_add(yb, df_mul(sa, df_mul(o, df_add(DF{1.0f, 0.0f}, df_neg(o))))));
                    }
                }
                const R sum = warp_sum8_transposed<R>(vch, lane);
                const int r = 8 * c + ((lane >> 2) & 7);
                if ((lane & 3) == 0 && r < NE && r >= first) atomicAdd(vp + (size_t)n * N + r, sum);
            }
            if (n - 1 >= a.n_lo) prefetch(n - 1);
        }

        if (a.n_lo > 0) {
            R* yb = static_cast<R*>(a.ybar);
            if (active)
                for (int j = 0; j < NE; j++) yb[(size_t)j * a.P + p] = ybuf[j * TH];
        } else {
            for (int c = 0; 8 * c < NE; c++) {
                R v8[8];
#pragma unroll
                for (int i = 0; i < 8; i++) v8[i] = (8 * c + i < NE && active) ? ybuf[(8 * c + i) * TH] : R(0);
                const R sum = warp_sum8_transposed<R>(v8, lane);
                const int r = 8 * c + ((lane >> 2) & 7);
                if ((lane & 3) == 0 && r < NE) atomicAdd(a.delta_partials + gw * N + r, a.normal ? sum : sum / a.init[r]);
            }
        }
    }
    cp_async_wait();
}

// The mixed form's replay: the steps [n0, n_stop) of every path from the checkpoint at n0 by
// the FP32 path kernel's own component step (euler_fp32.cuh), on its own rows and time
// steps, so that every replayed forward rate is bit for bit the one the path kernel computed
// (components at or beyond n_eff do not enter components below it).  The state lives in
// registers and the component loop enters its unrolled sequence at the step's first live
// component, as in the path kernel.
struct Replay32Params {
    int N, F, P, n0, n_stop, n_eff;
    float cap;
    const int* first;
    const float* ckpt_slot;  // [N][P] forward rates at n0
    const float* rows32;     // [T][N][pitch]
    const float* dt32;       // [T]
    const float* dw;         // [T][F][P]
    float* seg;              // [n_stop-n0+1][N][P]
};

template <int NMAX, int FMAX, bool CAPPED>
__global__ void __launch_bounds__(128) replay32_kernel(const Replay32Params a)
{
    constexpr int FP = euler32::row_pitch(FMAX);
    constexpr int FH = (FMAX + 1) / 2;
    const int p = blockIdx.x * 128 + threadIdx.x;
    if (p >= a.P) return;
    const int N = a.N, F = a.F, NE = a.n_eff, P = a.P;
    float L[NMAX];
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        L[j] = j < NE ? a.ckpt_slot[(size_t)j * P + p] : 0.0f;
        if (j < NE) a.seg[(size_t)j * P + p] = L[j];
    }
    // the increments of step n, loaded one step ahead
    float wn[FMAX];
    auto load_dw = [&](int n) {
#pragma unroll
        for (int k = 0; k < FMAX; k++) wn[k] = k < F ? a.dw[((size_t)n * F + k) * P + p] : 0.0f;
    };
    if (a.n0 < a.n_stop) load_dw(a.n0);
    for (int n = a.n0; n < a.n_stop; n++) {
        const int first = __ldg(a.first + n);
        const float dt = euler32::step_dt(a.dt32, n);
        float2 G2[FH];
#pragma unroll
        for (int m = 0; m < FH; m++) G2[m] = euler32::start_sum(wn[2 * m], 2 * m + 1 < FMAX ? wn[2 * m + 1] : 0.0f);
        if (n + 1 < a.n_stop) {
            load_dw(n + 1);
            // the next step's rows into L1 (one 128-byte line per lane of the first warp)
            const char* nrows = reinterpret_cast<const char*>(a.rows32 + (size_t)(n + 1) * N * FP);
            for (int q = threadIdx.x; q < (N * FP * (int)sizeof(float) + 127) / 128; q += 128)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(nrows + 128 * q));
        }
        const float4* rows = reinterpret_cast<const float4*>(a.rows32 + (size_t)n * N * FP);
        for_up_from<NMAX>(first, [&](auto jc) {
            constexpr int j = decltype(jc)::value;
            if (j < NE) {
                float lr[FP];
#pragma unroll
                for (int q = 0; q < FP / 4; q++) {
                    const float4 v = __ldg(rows + j * (FP / 4) + q);
                    lr[4 * q] = v.x;
                    lr[4 * q + 1] = v.y;
                    lr[4 * q + 2] = v.z;
                    lr[4 * q + 3] = v.w;
                }
                L[j] = euler32::component_step<FMAX, CAPPED>(L[j], lr, dt, G2, a.cap);
            }
        });
        float* out = a.seg + (size_t)(n + 1 - a.n0) * N * P;
#pragma unroll
        for (int j = 0; j < NMAX; j++)
            if (j < NE) out[(size_t)j * P + p] = L[j];
    }
}

// ------------------------------------------------------------------ seeds from the Bermudan cash flows
struct SeedParams {
    int nper, N, P, T_slot, callable, freeze_adjustment, pass;
    int has_discount;
    const BermudanPeriod* per;     // [nper]
    const void* states;            // [nobs][N][P]
    int fp32;
    const double* numeraire;       // [N+1][P]
    const double* inv_numeraire;   // [N+1][P] 1/N
    const double* adj;             // [N+1]
    const double* abar;            // [N+1] (pass 2)
    double inv_pd[kMaxForwardRates + 1];  // 1 / P^d(T_l)
    unsigned char det[kMaxForwardRates + 1];
    double delta[kMaxForwardRates];       // tenor period lengths
    const double* ex_time;         // [P]
    double* abar_partials;         // [blocks][N+1] (pass 1)
    double* seeds;                 // [N][P]: pass 1 the payoff part, pass 2 final (divided by P)
    double* nb;                    // [N+1][P] adjoints of the adjusted numeraires (pass 1 -> 2)
    double* value_partials;        // [blocks] (pass 1): sum of the frozen-decision values
    const double* omega;           // nullptr, or [nper][P]: the cash flows' AAD weights (FP64 form)
};

constexpr int kSeedThreads = 256;

template <typename TS>
__device__ __forceinline__ double st(const SeedParams& a, int slot, int j, int p)
{
    return (double)static_cast<const TS*>(a.states)[((size_t)slot * a.N + j) * a.P + p];
}

// Pass 1: per path the frozen-decision cash flows cf = A / N_adj of the periods paid, their
// adjoints to the fixings (into seeds, not yet divided by P) and to the adjusted numeraires
// (into nb), and per block the sums over paths of cf by payment date and of the value.  With
// N_adj = N a / P^d, the adjoint of the adjustment a_l is
//   abar_l = sum_p nbar_l N_l / P^d_l = -(1/a_l) sum_p (cf of the periods paid at l),
// so the per-date cash-flow sums are all pass 1 has to reduce.
// Pass 2: the numeraire chain N_l = N_{l-1} (1 + L_{l-1} d_{l-1}) downward, and the seeds.
// Both passes are division-free: 1/N comes from the table the path kernel kept.
template <typename TS>
__global__ void __launch_bounds__(kSeedThreads) seed_kernel(const SeedParams a)
{
    constexpr int VC = kMaxForwardRates + 1;                // the value's column of wsum
    __shared__ double r_adj[kMaxForwardRates + 1];          // P^d_l / a_l: 1/N_adj = (1/N) r_adj
    __shared__ double wsum[kSeedThreads / 32][VC + 1];      // per warp: cash-flow sums by date, then the value
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int p = blockIdx.x * kSeedThreads + tid;
    const bool active = p < a.P;
    const int N = a.N, P = a.P;
    if (a.pass == 1) {
        for (int l = tid; l <= N; l += kSeedThreads) {
            r_adj[l] = a.has_discount ? 1.0 / (a.adj[l] * a.inv_pd[l]) : 1.0;
            for (int w = 0; w < kSeedThreads / 32; w++) wsum[w][l] = 0.0;
        }
        __syncthreads();
        const double tau = active ? a.ex_time[p] : 0.0;
        double x = 0.0;
        for (int q = 0; q < a.nper; q++) {
            const BermudanPeriod c = a.per[q];
            // a callable payer receives the periods from its exercise date on; a cancelable one
            // receives the periods before its exercise date
            const bool paid = active && (a.callable ? (c.fixing >= tau) : (c.fixing < tau));
            const int l = c.pay_num_index;
            // the cash flow's adjoint weight: the frozen decision, or the AAD sweep's weight
            const double wgt = a.omega ? (active ? a.omega[(size_t)q * P + p] : 0.0) : (paid ? 1.0 : 0.0);
            double cf = 0.0, wcf = 0.0;
            if (paid || wgt != 0.0) {
                const double L = st<TS>(a, c.libor_slot, c.libor_index, p);
                const double invN = a.inv_numeraire[(size_t)l * P + p] * r_adj[l];
                const double A = ((L - c.strike) * c.period_length) * c.notional;
                cf = paid ? A * invN : 0.0;
                wcf = a.omega ? wgt * (A * invN) : cf;
                a.seeds[(size_t)c.libor_index * P + p] += a.omega ? wgt * ((c.period_length * c.notional) * invN)
                                                                  : (c.period_length * c.notional) * invN;
                if (!a.det[l]) a.nb[(size_t)l * P + p] -= wcf * invN;
            }
            x += cf;
            double v = wcf;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0) wsum[warp][l] += v;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if (lane == 0) wsum[warp][VC] = x;
        __syncthreads();
        // block partials, compensated across the warps (warp order)
        for (int l = tid; l <= N + 1; l += kSeedThreads) {
            const int col = (l <= N) ? l : VC;
            dd acc{0.0, 0.0};
            for (int w = 0; w < kSeedThreads / 32; w++) acc = dd_add_d(acc, wsum[w][col]);
            const double sum = acc.hi + acc.lo;
            if (l <= N) {
                const bool adjusted = a.has_discount && !a.det[l] && l >= 1;
                a.abar_partials[(size_t)blockIdx.x * (N + 1) + l] = adjusted ? -sum / a.adj[l] : 0.0;
            } else {
                a.value_partials[blockIdx.x] = sum;
            }
        }
        return;
    }
    if (!active) return;
    // nb holds adjoints of the adjusted numeraires N_adj = N a / P^d (from the payoffs); convert
    // them to adjoints of the unadjusted N (Nbar = Nbar_adj a / P^d - abar / N^2) and run the
    // chain N_l = N_{l-1} (1 + L_{l-1} d_{l-1}) downward, whose adjoint (un) is already
    // with respect to the unadjusted numeraire.
    const double invP = 1.0 / (double)P;
    double un = 0.0;
    for (int l = N; l >= 1; l--) {
        double t = un;
        if (a.has_discount) {
            if (!a.det[l]) {
                t += (a.nb[(size_t)l * P + p] * a.adj[l]) * a.inv_pd[l];
                if (!a.freeze_adjustment) {
                    const double iN = a.inv_numeraire[(size_t)l * P + p];
                    t -= a.abar[l] * (iN * iN);
                }
            }
        } else {
            t += a.nb[(size_t)l * P + p];
        }
        const double Nprev = a.numeraire[(size_t)(l - 1) * P + p];
        const double Lf = st<TS>(a, a.T_slot, l - 1, p);  // frozen fixing L_{l-1}(T_{l-1})
        double* sd = a.seeds + (size_t)(l - 1) * P + p;
        *sd = (*sd + t * Nprev * a.delta[l - 1]) * invP;
        un = t * (1.0 + Lf * a.delta[l - 1]);
    }
}

// Mixed form: the same two passes in FP32 (seeds and numeraire adjoints kept as FP32
// arrays, which the FP32 reverse sweep reads), with the per-date cash-flow sums and the
// value as Sum2 pairs (twice FP32 precision) and every per-date constant converted once per
// block: on this GPU an FP64 instruction per path would cost more than the pass itself.
// Exercise times are compared as the bit patterns of non-negative doubles (the IEEE order).
struct SeedSmem32 {
    float r_adj[kMaxForwardRates + 1];    // P^d_l / a_l
    float adj_pd[kMaxForwardRates + 1];   // a_l / P^d_l
    float abar[kMaxForwardRates + 1];     // pass 2
    float delta[kMaxForwardRates];
    float strike[kMaxForwardRates], lennot[kMaxForwardRates];
    long long fixbits[kMaxForwardRates];
    int libor_slot[kMaxForwardRates], libor_index[kMaxForwardRates], pay[kMaxForwardRates];
};

__global__ void __launch_bounds__(kSeedThreads) seed_mixed_kernel(const SeedParams a)
{
    constexpr int VC = kMaxForwardRates + 1;          // the value's column of wsum
    __shared__ SeedSmem32 c;
    __shared__ Sum2 wsum[kSeedThreads / 32][VC + 1];  // per warp: cash-flow sums by date, then the value
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int p = blockIdx.x * kSeedThreads + tid;
    const bool active = p < a.P;
    const int N = a.N, P = a.P;
    float* seeds = static_cast<float*>(static_cast<void*>(a.seeds));
    float* nb = static_cast<float*>(static_cast<void*>(a.nb));
    for (int l = tid; l <= N; l += kSeedThreads) {
        const double ap = a.has_discount ? a.adj[l] * a.inv_pd[l] : 1.0;
        c.r_adj[l] = (float)(1.0 / ap);
        c.adj_pd[l] = (float)ap;
        if (a.pass == 2) c.abar[l] = (float)a.abar[l];
        if (l < N) c.delta[l] = (float)a.delta[l];
        for (int w = 0; w < kSeedThreads / 32; w++) wsum[w][l] = Sum2{0.0f, 0.0f};
    }
    for (int q = tid; q < a.nper; q += kSeedThreads) {
        const BermudanPeriod pq = a.per[q];
        c.strike[q] = (float)pq.strike;
        c.lennot[q] = (float)(pq.period_length * pq.notional);
        c.fixbits[q] = __double_as_longlong(pq.fixing);
        c.libor_slot[q] = pq.libor_slot;
        c.libor_index[q] = pq.libor_index;
        c.pay[q] = pq.pay_num_index;
    }
    if (tid < kSeedThreads / 32) wsum[tid][VC] = Sum2{0.0f, 0.0f};
    __syncthreads();
    const float* states = static_cast<const float*>(a.states);
    if (a.pass == 1) {
        const long long taubits = active ? __double_as_longlong(a.ex_time[p]) : 0;
        Sum2 x{0.0f, 0.0f};
        for (int q = 0; q < a.nper; q++) {
            // a callable payer receives the periods from its exercise date on; a cancelable one
            // receives the periods before its exercise date (times >= 0: bit order = value order)
            const bool paid = active && (a.callable ? (c.fixbits[q] >= taubits) : (c.fixbits[q] < taubits));
            const int l = c.pay[q];
            // the cash flow's adjoint weight: the frozen decision, or the AAD sweep's weight
            const float wgt = a.omega ? (active ? (float)a.omega[(size_t)q * P + p] : 0.0f) : (paid ? 1.0f : 0.0f);
            float cf = 0.0f, wcf = 0.0f;
            if (paid || wgt != 0.0f) {
                const float L = states[((size_t)c.libor_slot[q] * N + c.libor_index[q]) * P + p];
                const float invN = f64_to_f32_int(a.inv_numeraire[(size_t)l * P + p]) * c.r_adj[l];
                const float A = __fmul_rn((L - c.strike[q]) * c.lennot[q], invN);  // exact input of the Sum2 below
                cf = paid ? A : 0.0f;
                wcf = a.omega ? wgt * A : cf;
                seeds[(size_t)c.libor_index[q] * P + p] += wgt * (c.lennot[q] * invN);
                if (!a.det[l]) nb[(size_t)l * P + p] -= wcf * invN;
            }
            sum2_add(x, cf);
            Sum2 v{wcf, 0.0f};
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const Sum2 y{__shfl_down_sync(0xffffffffu, v.p, off), __shfl_down_sync(0xffffffffu, v.s, off)};
                v = sum2_merge(v, y);
            }
            if (lane == 0) wsum[warp][l] = sum2_merge(wsum[warp][l], v);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const Sum2 y{__shfl_down_sync(0xffffffffu, x.p, off), __shfl_down_sync(0xffffffffu, x.s, off)};
            x = sum2_merge(x, y);
        }
        if (lane == 0) wsum[warp][VC] = x;
        __syncthreads();
        // block partials, the warps merged in warp order
        for (int l = tid; l <= N + 1; l += kSeedThreads) {
            const int col = (l <= N) ? l : VC;
            Sum2 acc = wsum[0][col];
            for (int w = 1; w < kSeedThreads / 32; w++) acc = sum2_merge(acc, wsum[w][col]);
            const double sum = sum2_value(acc);
            if (l <= N) {
                const bool adjusted = a.has_discount && !a.det[l] && l >= 1;
                a.abar_partials[(size_t)blockIdx.x * (N + 1) + l] = adjusted ? -sum / a.adj[l] : 0.0;
            } else {
                a.value_partials[blockIdx.x] = sum;
            }
        }
        return;
    }
    if (!active) return;
    const float invP = 1.0f / (float)P;
    float un = 0.0f;
    for (int l = N; l >= 1; l--) {
        float t = un;
        if (a.has_discount) {
            if (!a.det[l]) {
                t += nb[(size_t)l * P + p] * c.adj_pd[l];
                if (!a.freeze_adjustment) {
                    const float iN = f64_to_f32_int(a.inv_numeraire[(size_t)l * P + p]);
                    t -= c.abar[l] * (iN * iN);
                }
            }
        } else {
            t += nb[(size_t)l * P + p];
        }
        const float Nprev = f64_to_f32_int(a.numeraire[(size_t)(l - 1) * P + p]);
        const float Lf = states[((size_t)a.T_slot * N + (l - 1)) * P + p];  // frozen fixing L_{l-1}(T_{l-1})
        float* sd = seeds + (size_t)(l - 1) * P + p;
        *sd = (*sd + t * Nprev * c.delta[l - 1]) * invP;
        un = t * (1.0f + Lf * c.delta[l - 1]);
    }
}

// column sums of [rows][cols] partials in fixed order (grid: cols/32 blocks of 1024 threads)
__global__ void __launch_bounds__(1024) column_sum_kernel(const double* in, int rows, int cols, double scale, double* out)
{
    __shared__ double part[32][33];
    const int c = blockIdx.x * 32 + (threadIdx.x & 31), r0 = threadIdx.x >> 5;
    double s = 0.0;
    if (c < cols)
        for (int r = r0; r < rows; r += 32) s += in[(size_t)r * cols + c];
    part[r0][threadIdx.x & 31] = s;
    __syncthreads();
    if (r0 == 0 && c < cols) {
        double t = 0.0;
        for (int k = 0; k < 32; k++) t += part[k][threadIdx.x & 31];
        out[c] = t * scale;
    }
}

template <typename R, int NMAX, int FMAX, int TH>
int launch_rev(const RevParams& a, const AdjTables<R>& tb, int blocks, cudaStream_t s)
{
    const size_t smem = rev_smem_bytes<R, NMAX, FMAX, TH>();
    static bool attr_set = false;  // set once, before any stream capture
    // the FP64 form up to 40 forward rates sweeps on float pairs (the 80-rate, two-factor
    // form keeps the FP64 sweep)
    constexpr bool kDf = sizeof(R) == 8 && NMAX <= 40;
    if (!attr_set) {
        if constexpr (kDf)
            LMM_CUDA(cudaFuncSetAttribute(reverse_df_kernel<NMAX, FMAX, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        else
            LMM_CUDA(cudaFuncSetAttribute(reverse_kernel<R, NMAX, FMAX, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        attr_set = true;
    }
    if constexpr (kDf) reverse_df_kernel<NMAX, FMAX, TH><<<blocks, TH, smem, s>>>(a, tb);
    else reverse_kernel<R, NMAX, FMAX, TH><<<blocks, TH, smem, s>>>(a, tb);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <typename R, int NMAX, int FMAX>
int launch_rev_threads(const RevParams& a, const AdjTables<R>& tb, int threads, int blocks, cudaStream_t s)
{
    if (threads == 64) return launch_rev<R, NMAX, FMAX, 64>(a, tb, blocks, s);
    if (threads == 256) return launch_rev<R, NMAX, FMAX, 256>(a, tb, blocks, s);
    return launch_rev<R, NMAX, FMAX, 128>(a, tb, blocks, s);
}

template <typename R>
int launch_rev_dispatch(const RevParams& a, const AdjTables<R>& tb, int threads, int blocks, cudaStream_t s)
{
    if (a.N <= 24 && a.F <= 4) return launch_rev_threads<R, 24, 4>(a, tb, threads, blocks, s);
    if (a.N <= 40 && a.F <= 10) {
        // the sweep touches components below n_eff only: products that end early (a portfolio's
        // short swaps) take a narrower register-resident state (same factor-row pitch)
        if constexpr (sizeof(R) == 4) {
            if (threads == 128) {
                if (a.n_eff <= 16) return launch_rev<R, 16, 10, 128>(a, tb, blocks, s);
                if (a.n_eff <= 24) return launch_rev<R, 24, 10, 128>(a, tb, blocks, s);
                if (a.n_eff <= 32) return launch_rev<R, 32, 10, 128>(a, tb, blocks, s);
            }
        }
        return launch_rev_threads<R, 40, 10>(a, tb, threads, blocks, s);
    }
    if constexpr (sizeof(R) == 8) {
        // the FP64 form with up to 80 forward rates and two factors (the reference's own
        // sensitivity test: 80 forwards, one factor)
        if (a.N <= kMaxForwardRates && a.F <= 2) return launch_rev<R, 80, 2, 64>(a, tb, blocks, s);
    }
    return fail(LMM_ERR_INVALID, "adjoint supports at most 40 forward rates and 10 factors (FP64: or 80 and 2)");
}

template <typename R>
int launch_replay_dispatch(const ReplayParams& a, const AdjTables<R>& tb, cudaStream_t s)
{
    const int blocks = (a.P + 127) / 128;
    if (a.N <= 24 && a.F <= 4) replay_kernel<R, 24, 4><<<blocks, 128, 0, s>>>(a, tb);
    else if (a.N <= 40 && a.F <= 10) replay_kernel<R, 40, 10><<<blocks, 128, 0, s>>>(a, tb);
    else if (sizeof(R) == 8 && a.N <= kMaxForwardRates && a.F <= 2) replay_kernel<R, 80, 2><<<blocks, 128, 0, s>>>(a, tb);
    else return fail(LMM_ERR_INVALID, "adjoint supports at most 40 forward rates and 10 factors (FP64: or 80 and 2)");
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <int NMAX, int FMAX>
void launch_replay32_t(const Replay32Params& q, bool capped, cudaStream_t s)
{
    const int blocks = (q.P + 127) / 128;
    if (capped) replay32_kernel<NMAX, FMAX, true><<<blocks, 128, 0, s>>>(q);
    else replay32_kernel<NMAX, FMAX, false><<<blocks, 128, 0, s>>>(q);
}

// the row table's pitch follows the path kernel's (forward rates, factors) template, which the
// same bounds select
int launch_replay32(const Replay32Params& q, bool capped, cudaStream_t s)
{
    if (q.N <= 24 && q.F <= 4) launch_replay32_t<24, 4>(q, capped, s);
    else if (q.N <= 40 && q.F <= 10) launch_replay32_t<40, 10>(q, capped, s);
    else return fail(LMM_ERR_INVALID, "adjoint supports at most 40 forward rates and 10 factors");
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <typename R>
int reverse_sweeps(const AdjointLaunch& L, const AdjTables<R>& tb, cudaStream_t s)
{
    RevParams rp;
    std::memset(&rp, 0, sizeof(rp));
    rp.T = L.T;
    rp.N = L.N;
    rp.F = L.F;
    rp.P = L.P;
    rp.t_end = L.t_end;
    rp.n_eff = L.n_eff;
    rp.capped = !std::isinf(L.cap);
    rp.normal = L.normal;
    rp.cap = L.cap;
    rp.first = L.d_first;
    rp.init = L.d_init;
    rp.seeds = L.d_seeds;
    rp.ybar = L.d_ybar;
    rp.vega_partials = L.d_vega_partials;
    rp.delta_partials = L.d_delta_partials;
    if (L.stride == 1) {
        // every step's forward rates are stored: one sweep over [0, t_end)
        rp.n_lo = 0;
        rp.n_hi = L.t_end;
        rp.base_step = 0;
        rp.seed = 1;
        rp.states = L.d_ckpt;
        return launch_rev_dispatch<R>(rp, tb, L.threads, L.blocks, s);
    }
    ReplayParams q;
    std::memset(&q, 0, sizeof(q));
    q.T = L.T;
    q.N = L.N;
    q.F = L.F;
    q.P = L.P;
    q.n_eff = L.n_eff;
    q.capped = rp.capped;
    q.normal = L.normal;
    q.cap = L.cap;
    q.first = L.d_first;
    q.seg = L.d_seg;
    const int nseg = (L.t_end + L.stride - 1) / L.stride;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
        const int n0 = sgi * L.stride, n1 = std::min(n0 + L.stride, L.t_end);
        q.n0 = n0;
        q.n_stop = (sgi == nseg - 1) ? n1 : n1 - 1;  // the last segment also needs the state at t_end
        q.ckpt_slot = static_cast<const R*>(L.d_ckpt) + (size_t)sgi * L.N * L.P;
        int rc;
        if (sizeof(R) == 4 && L.d_rows32 && !L.normal) {
            Replay32Params q32;
            q32.N = L.N;
            q32.F = L.F;
            q32.P = L.P;
            q32.n0 = q.n0;
            q32.n_stop = q.n_stop;
            q32.n_eff = L.n_eff;
            q32.cap = (float)L.cap;
            q32.first = L.d_first;
            q32.ckpt_slot = static_cast<const float*>(q.ckpt_slot);
            q32.rows32 = L.d_rows32;
            q32.dt32 = L.d_dt32;
            q32.dw = static_cast<const float*>(L.d_dw);
            q32.seg = static_cast<float*>(L.d_seg);
            rc = launch_replay32(q32, rp.capped != 0, s);
        } else {
            rc = kReplayNotFast;
            if (sizeof(R) == 8 && L.path64) {
                ReplaySegment seg;
                seg.n0 = q.n0;
                seg.n_stop = q.n_stop;
                seg.n_eff = L.n_eff;
                seg.ckpt = static_cast<const double*>(q.ckpt_slot);
                seg.seg = static_cast<double*>(L.d_seg);
                rc = launch_replay_fp64(*L.path64, seg, s);
            }
            if (rc == kReplayNotFast) rc = launch_replay_dispatch<R>(q, tb, s);
        }
        if (rc) return rc;
        rp.n_lo = n0;
        rp.n_hi = n1;
        rp.base_step = n0;
        rp.seed = sgi == nseg - 1;
        rp.states = L.d_seg;
        if ((rc = launch_rev_dispatch<R>(rp, tb, L.threads, L.blocks, s))) return rc;
    }
    return LMM_OK;
}

}  // namespace

int adjoint_f_pitch(int N, int F, int fp32)
{
    const bool small = N <= 24 && F <= 4;  // the (forward rates, factors) templates of the reverse kernel
    if (fp32) return small ? f_pitch<float, 4>() : f_pitch<float, 10>();
    if (!small && !(N <= 40 && F <= 10)) return f_pitch<double, 2>();  // 41..80 forward rates, <= 2 factors
    return small ? f_pitch<double, 4>() : f_pitch<double, 10>();
}

int adjoint_blocks(int P, int threads, int fp32)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int want = sms * std::max(1, (fp32 ? rev_warps_per_sm<float>() : rev_warps_per_sm<double>()) * 32 / threads);  // the resident blocks of rev_min_blocks
    const int need = (P + threads - 1) / threads;
    return need < want ? need : want;
}

AdjointScratch adjoint_scratch(int T, int N, int P, int threads, int stride, int fp32)
{
    AdjointScratch z;
    z.blocks = adjoint_blocks(P, threads, fp32);
    z.warps = z.blocks * (threads / 32);
    z.vega_partials = (size_t)z.warps * T * N;
    z.delta_partials = (size_t)z.warps * N;
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    z.seg_bytes = stride > 1 ? (size_t)(stride + 1) * N * (size_t)P * esz : 0;
    z.nb_doubles = (size_t)(N + 1) * P;
    z.ybar_bytes = stride > 1 ? (size_t)N * (size_t)P * esz : 0;
    return z;
}

int launch_adjoint(const AdjointLaunch& L, cudaStream_t s)
{
    if (L.stride < 1 || L.stride > kMaxStride) return fail(LMM_ERR_INVALID, "checkpoint stride must be in [1, 16]");
    // ---- seeds: pass 1 (adjustment adjoint partials), reduce, pass 2
    SeedParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.nper = L.nper;
    sp.N = L.N;
    sp.P = L.P;
    sp.T_slot = L.T_slot;
    sp.callable = L.callable;
    sp.freeze_adjustment = L.freeze_adjustment;
    sp.has_discount = L.h_discount != nullptr;
    sp.per = L.d_per;
    sp.states = L.d_states;
    sp.fp32 = L.fp32;
    sp.numeraire = L.d_numeraire;
    sp.adj = L.d_num_adj;
    sp.abar = L.d_abar;
    for (int l = 0; l <= L.N && l <= kMaxForwardRates; l++) {
        sp.inv_pd[l] = L.h_discount ? 1.0 / L.h_discount[l] : 1.0;
        sp.det[l] = L.h_num_det[l];
    }
    for (int j = 0; j < L.N && j < kMaxForwardRates; j++) sp.delta[j] = L.h_delta[j];
    sp.ex_time = L.d_ex;
    sp.abar_partials = L.d_abar_partials;
    sp.seeds = L.d_seeds;
    sp.value_partials = L.d_value_partials;
    sp.nb = L.d_nb;
    sp.inv_numeraire = L.d_inv_numeraire;
    sp.omega = L.d_omega;
    if (!L.d_inv_numeraire || !L.d_nb) return fail(LMM_ERR_STATE, "adjoint: the simulation kept no reciprocal numeraire");
    if (L.nper > 0 && L.N > kMaxForwardRates) return fail(LMM_ERR_INVALID, "adjoint: at most 80 forward rates");
    const int sb = (L.P + kSeedThreads - 1) / kSeedThreads;
    {
        KernelTimer kt(K_ADJOINT, s, 4);
        const size_t esz = L.fp32 ? sizeof(float) : sizeof(double);  // the mixed form keeps FP32 seeds
        LMM_CUDA(cudaMemsetAsync(L.d_seeds, 0, esz * (size_t)L.N * L.P, s));
        LMM_CUDA(cudaMemsetAsync(L.d_nb, 0, esz * (size_t)(L.N + 1) * L.P, s));
        sp.pass = 1;
        if (L.fp32) seed_mixed_kernel<<<sb, kSeedThreads, 0, s>>>(sp);
        else seed_kernel<double><<<sb, kSeedThreads, 0, s>>>(sp);
        column_sum_kernel<<<(L.N + 1 + 31) / 32, 1024, 0, s>>>(L.d_abar_partials, sb, L.N + 1, 1.0 / (double)L.P, L.d_abar);
        column_sum_kernel<<<1, 1024, 0, s>>>(L.d_value_partials, sb, 1, 1.0 / (double)L.P, L.d_value_out);
        sp.pass = 2;
        if (L.fp32) seed_mixed_kernel<<<sb, kSeedThreads, 0, s>>>(sp);
        else seed_kernel<double><<<sb, kSeedThreads, 0, s>>>(sp);
        LMM_CUDA(cudaGetLastError());
    }
    return launch_adjoint_sweeps(L, s);
}

int launch_adjoint_sweeps(const AdjointLaunch& L, cudaStream_t s)
{
    if (L.stride < 1 || L.stride > kMaxStride) return fail(LMM_ERR_INVALID, "checkpoint stride must be in [1, 16]");
    // ---- reverse sweeps over the paths (per-warp partials, then fixed-order column sums)
    const int warps = L.blocks * (L.threads / 32);
    LMM_CUDA(cudaMemsetAsync(L.d_vega_partials, 0, sizeof(double) * (size_t)warps * L.T * L.N, s));
    LMM_CUDA(cudaMemsetAsync(L.d_delta_partials, 0, sizeof(double) * (size_t)warps * L.N, s));
    const int nsweeps = L.stride == 1 ? 1 : 2 * ((L.t_end + L.stride - 1) / L.stride);
    int rc;
    {
        KernelTimer kt(K_ADJOINT, s, nsweeps);
        if (L.fp32) {
            AdjTables<float> tb{static_cast<const float*>(L.d_lam), static_cast<const float*>(L.d_var_half),
                                static_cast<const float*>(L.d_f), static_cast<const float*>(L.d_sigma),
                                static_cast<const float*>(L.d_inv_delta), static_cast<const float*>(L.d_dt), L.d_dw};
            rc = reverse_sweeps<float>(L, tb, s);
        } else {
            AdjTables<double> tb{static_cast<const double*>(L.d_lam), static_cast<const double*>(L.d_var_half),
                                 static_cast<const double*>(L.d_f), static_cast<const double*>(L.d_sigma),
                                 static_cast<const double*>(L.d_inv_delta), static_cast<const double*>(L.d_dt), L.d_dw};
            rc = reverse_sweeps<double>(L, tb, s);
        }
    }
    if (rc) return rc;
    {
        KernelTimer kt(K_ADJOINT, s, 2);
        column_sum_kernel<<<(L.T * L.N + 31) / 32, 1024, 0, s>>>(L.d_vega_partials, warps, L.T * L.N, 1.0, L.d_vegas);
        column_sum_kernel<<<(L.N + 31) / 32, 1024, 0, s>>>(L.d_delta_partials, warps, L.N, 1.0, L.d_deltas);
        LMM_CUDA(cudaGetLastError());
    }
    return LMM_OK;
}

}  // namespace lmm
