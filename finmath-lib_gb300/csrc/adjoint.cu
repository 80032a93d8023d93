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
//            osbar_j = sum_k lam_jk R_k,  Ybar_j = Ybar'_j + osbar_j (1/d_j)/(L_j+1/d_j)^2 L_j,
//            lambar_jk = mubar_j S_k^(j) + os_j R_k + Ybar'_j dW_k,
//            sigmabar_ij = sum_k lambar_jk f_jk - mubar_j sigma_ij
//
// so a reverse step costs O(N F) like the forward one.  The path state is recomputed
// from checkpoints written by the forward kernel every `stride` steps (the states of a
// segment live in thread-local memory).  The Bermudan's exercise decisions are frozen from
// the forward valuation (regression coefficients fixed); the seed kernel turns each path's
// realised cash flows into adjoints of the fixings L_m(T_m), through the payment numeraires,
// their cross-path adjustment a_l = mean(1/N_l) (:869-874) and the numeraire chain.
#include <math_constants.h>

#include "lmm_internal.h"
#include "reduce.cuh"

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
__device__ __forceinline__ R fdiv(R a, R b);
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }
template <>
__device__ __forceinline__ double fdiv<double>(double a, double b) { return a / b; }

template <typename R>
struct AdjTables {
    const R* lam;       // [T][N][F]
    const R* f;         // [T][N][F] lam / sigma
    const R* sigma;     // [T][N]
    const R* var_half;  // [T][N]
    const R* inv_delta; // [N]
    const R* dt;        // [T]
    const void* dw;     // [T][F][P] of type R
    const void* ckpt;   // [T/stride+1][N][P]
};

struct AdjParams {
    int T, N, F, P, stride, ckpt_is_L;
    int t_end;   // last time index the product reads (reverse sweep starts there)
    int n_eff;   // components 0..n_eff-1 influence the product (spot drift of j uses l <= j only)
    int capped;
    double cap;
    const int* first;        // [T]
    const double* init;      // [N]
    const double* seeds;     // [N][P]  d value / d L_m(T_m), already divided by P
    double* vega_partials;   // [blocks][T][N]
    double* delta_partials;  // [blocks][N]
};

template <typename R, int NMAX, int FMAX>
__device__ __forceinline__ void forward_step(const AdjParams& a, const AdjTables<R>& tb, int i, int p, bool active,
                                             const R* Y, R* Yn)
{
    const int N = a.N, F = a.F;
    const int first = __ldg(a.first + i);
    const R dt = tb.dt[i];
    const R* lam = tb.lam + (size_t)i * N * F;
    const R* dW = static_cast<const R*>(tb.dw);
    R dw[FMAX], S[FMAX];
#pragma unroll
    for (int k = 0; k < FMAX; k++) {
        dw[k] = (k < F && active) ? dW[((size_t)i * F + k) * a.P + p] : R(0);
        S[k] = R(0);
    }
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        if (j >= a.n_eff) continue;
        if (j < first) {
            Yn[j] = Y[j];
            continue;
        }
        R L = fexp<R>(Y[j]);
        if (a.capped && L > (R)a.cap) L = (R)a.cap;
        const R os = fdiv<R>(L, L + tb.inv_delta[j]);
        R mu = tb.var_half[(size_t)i * N + j], diff = R(0);
#pragma unroll
        for (int k = 0; k < FMAX; k++) {
            if (k < F) {
                const R l = lam[j * F + k];
                S[k] = S[k] + os * l;
                mu = mu + S[k] * l;
                diff = diff + dw[k] * l;
            }
        }
        Yn[j] = Y[j] + (mu * dt + diff);
    }
}

template <typename R, int NMAX, int FMAX, int kAdjThreads>
__global__ void __launch_bounds__(kAdjThreads) adjoint_kernel(const AdjParams a, const AdjTables<R> tb)
{
    extern __shared__ double smem_adj[];
    double* acc = smem_adj;                                      // [T][N] block vega accumulator
    R* wpart = reinterpret_cast<R*>(smem_adj + (size_t)a.T * a.N);  // [warps][NMAX]
    const int N = a.N, F = a.F, T = a.T, NE = a.n_eff, TE = a.t_end;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int q = tid; q < T * N; q += kAdjThreads) acc[q] = 0.0;
    double dsum[NMAX];
#pragma unroll
    for (int j = 0; j < NMAX; j++) dsum[j] = 0.0;
    const int nseg = (TE + a.stride - 1) / a.stride;
    __syncthreads();

    for (int base = blockIdx.x * kAdjThreads; base < a.P; base += gridDim.x * kAdjThreads) {
        const int p = base + tid;
        const bool active = p < a.P;
        R Ybar[NMAX];
        R seg[kMaxStride + 1][NMAX];
        for (int s = nseg - 1; s >= 0; s--) {
            const int n0 = s * a.stride, n1 = min(n0 + a.stride, TE);
            // state at the checkpoint
#pragma unroll
            for (int j = 0; j < NMAX; j++) {
                R y = R(0);
                if (j < NE && active) {
                    const size_t o = ((size_t)s * N + j) * a.P + p;
                    if (a.ckpt_is_L) y = (R)log(static_cast<const double*>(tb.ckpt)[o]);
                    else y = static_cast<const R*>(tb.ckpt)[o];
                }
                seg[0][j] = y;
            }
            for (int n = n0; n < n1; n++) forward_step<R, NMAX, FMAX>(a, tb, n, p, active, seg[n - n0], seg[n - n0 + 1]);
            if (s == nseg - 1) {
                // seed: d value / d Y_m(T) = d value / d L_m(T_m) * L_m (components are frozen after fixing)
#pragma unroll
                for (int j = 0; j < NMAX; j++) {
                    R yb = R(0);
                    if (j < NE && active) {
                        const R y = seg[n1 - n0][j];
                        const R L = fexp<R>(y);
                        if (!(a.capped && L > (R)a.cap)) yb = (R)a.seeds[(size_t)j * a.P + p] * L;
                    }
                    Ybar[j] = yb;
                }
            }
            for (int n = n1 - 1; n >= n0; n--) {
                const int i = n;
                const R* Y = seg[n - n0];
                const int first = __ldg(a.first + i);
                const R dt = tb.dt[i];
                const R* lam = tb.lam + (size_t)i * N * F;
                const R* fj = tb.f + (size_t)i * N * F;
                const R* dW = static_cast<const R*>(tb.dw);
                R dw[FMAX], S[FMAX], Rk[FMAX];
#pragma unroll
                for (int k = 0; k < FMAX; k++) {
                    dw[k] = (k < F && active) ? dW[((size_t)i * F + k) * a.P + p] : R(0);
                    S[k] = R(0);
                    Rk[k] = R(0);
                }
                // forward pass of the step: running sums S^(N-1) and the measure-change ratios
                R os[NMAX], Lv[NMAX];
#pragma unroll
                for (int j = 0; j < NMAX; j++) {
                    os[j] = R(0);
                    Lv[j] = R(0);
                    if (j < NE && j >= first) {
                        R L = fexp<R>(Y[j]);
                        const bool c = a.capped && L > (R)a.cap;
                        if (c) L = (R)a.cap;
                        Lv[j] = c ? R(-1) : L;  // -1 marks a capped component (no derivative)
                        os[j] = fdiv<R>(L, L + tb.inv_delta[j]);
#pragma unroll
                        for (int k = 0; k < FMAX; k++)
                            if (k < F) S[k] = S[k] + os[j] * lam[j * F + k];
                    }
                }
                // reverse pass
                R contrib[NMAX];
#pragma unroll
                for (int jj = NMAX - 1; jj >= 0; jj--) {
                    const int j = jj;
                    contrib[j] = R(0);
                    if (j < NE && j >= first) {
                        const R yb = Ybar[j];
                        const R mub = yb * dt;
                        R osb = R(0), sg = R(0);
#pragma unroll
                        for (int k = 0; k < FMAX; k++) {
                            if (k < F) {
                                const R l = lam[j * F + k];
                                Rk[k] = Rk[k] + mub * l;
                                osb = osb + l * Rk[k];
                                const R lb = mub * S[k] + os[j] * Rk[k] + yb * dw[k];
                                sg = sg + lb * fj[j * F + k];
                                S[k] = S[k] - os[j] * l;  // S^(j-1)
                            }
                        }
                        sg = sg - mub * tb.sigma[(size_t)i * N + j];
                        contrib[j] = sg;
                        if (Lv[j] > R(0)) {
                            const R c = tb.inv_delta[j];
                            const R den = Lv[j] + c;
                            Ybar[j] = yb + fdiv<R>(osb * c, den * den) * Lv[j];
                        }
                    }
                }
                // block-sum the vega contributions of step i (deterministic order)
#pragma unroll
                for (int j = 0; j < NMAX; j++) {
                    if (j < NE && j >= first) {
                        R v = active ? contrib[j] : R(0);
#pragma unroll
                        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
                        if (lane == 0) wpart[warp * NMAX + j] = v;
                    }
                }
                __syncthreads();
                if (tid < NE && tid >= first) {
                    double t = 0.0;
                    for (int w = 0; w < kAdjThreads / 32; w++) t += (double)wpart[w * NMAX + tid];
                    acc[(size_t)i * N + tid] += t;
                }
                __syncthreads();
            }
        }
        // deltas: Y_0 = log(L_0(0)) -> d value / d L_0 = Ybar / L_0
#pragma unroll
        for (int j = 0; j < NMAX; j++)
            if (j < NE && active) dsum[j] += (double)Ybar[j] / a.init[j];
    }
    // write block partials
    for (int q = tid; q < T * N; q += kAdjThreads) a.vega_partials[(size_t)blockIdx.x * T * N + q] = acc[q];
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        if (j < N) {
            const dd s = block_dd_sum(dd{dsum[j], 0.0});
            if (tid == 0) a.delta_partials[(size_t)blockIdx.x * N + j] = s.hi + s.lo;
        }
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
    const double* adj;             // [N+1]
    const double* abar;            // [N+1] (pass 2)
    double pd[65];
    unsigned char det[65];
    double delta[64];              // tenor period lengths
    const double* ex_time;         // [P]
    double* abar_partials;         // [blocks][N+1] (pass 1)
    double* seeds;                 // [N][P] (pass 2)
    double* value_partials;        // [blocks] (pass 1): sum of the frozen-decision values
};

template <typename TS>
__device__ __forceinline__ double st(const SeedParams& a, int slot, int j, int p)
{
    return (double)static_cast<const TS*>(a.states)[((size_t)slot * a.N + j) * a.P + p];
}

template <typename TS>
__global__ void __launch_bounds__(256) seed_kernel(const SeedParams a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < a.P;
    double nb[65], lb[64];
    for (int l = 0; l <= a.N; l++) nb[l] = 0.0;
    for (int m = 0; m < a.N; m++) lb[m] = 0.0;
    double x = 0.0;
    if (active) {
        const double tau = a.ex_time[p];
        for (int q = 0; q < a.nper; q++) {
            const BermudanPeriod c = a.per[q];
            // a callable payer receives the periods from its exercise date on; a cancelable one
            // receives the periods before its exercise date
            const bool paid = a.callable ? (c.fixing >= tau) : (c.fixing < tau);
            if (!paid) continue;
            const double L = st<TS>(a, c.libor_slot, c.libor_index, p);
            const int l = c.pay_num_index;
            const double Nu = a.numeraire[(size_t)l * a.P + p];
            const double Nadj = a.has_discount ? (a.det[l] ? (1.0 / a.pd[l]) * (Nu * a.adj[l]) : (Nu * a.adj[l]) / a.pd[l]) : Nu;
            const double A = ((L - c.strike) * c.period_length) * c.notional;
            const double cf = A / Nadj;
            x += cf;
            lb[c.libor_index] += c.period_length * c.notional / Nadj;
            if (!a.det[l]) nb[l] += -cf / Nadj;
        }
    }
    if (a.pass == 1) {
        // sum over paths of Nbar_adj,l * N_l / P^d_l: the adjoint of the adjustment a_l
        for (int l = 1; l <= a.N; l++) {
            double v = 0.0;
            if (active && a.has_discount && !a.det[l]) v = nb[l] * a.numeraire[(size_t)l * a.P + p] / a.pd[l];
            const dd s = block_dd_sum(dd{v, 0.0});
            if (threadIdx.x == 0) a.abar_partials[(size_t)blockIdx.x * (a.N + 1) + l] = s.hi + s.lo;
        }
        const dd s = block_dd_sum(dd{active ? x : 0.0, 0.0});
        if (threadIdx.x == 0) a.value_partials[blockIdx.x] = s.hi + s.lo;
        return;
    }
    if (!active) return;
    // nb holds adjoints of the adjusted numeraires N_adj = N a / P^d (from the payoffs); convert
    // them to adjoints of the unadjusted N (Nbar = Nbar_adj a / P^d - abar / N^2) and run the
    // chain N_l = N_{l-1} (1 + L_{l-1} d_{l-1}) downward, whose adjoint (un) is already
    // with respect to the unadjusted numeraire.
    double un = 0.0;
    for (int l = a.N; l >= 1; l--) {
        const double Nl = a.numeraire[(size_t)l * a.P + p];
        double t = un;
        if (a.has_discount) {
            if (!a.det[l]) {
                t += nb[l] * a.adj[l] / a.pd[l];
                if (!a.freeze_adjustment) t -= a.abar[l] / (Nl * Nl);
            }
        } else {
            t += nb[l];
        }
        const double Nprev = a.numeraire[(size_t)(l - 1) * a.P + p];
        const double Lf = st<TS>(a, a.T_slot, l - 1, p);  // frozen fixing L_{l-1}(T_{l-1})
        lb[l - 1] += t * Nprev * a.delta[l - 1];
        un = t * (1.0 + Lf * a.delta[l - 1]);
    }
    const double invP = 1.0 / (double)a.P;
    for (int m = 0; m < a.N; m++) a.seeds[(size_t)m * a.P + p] = lb[m] * invP;
}

// column sums of [rows][cols] partials in fixed order (grid: cols/32 blocks of 256 threads)
__global__ void __launch_bounds__(256) column_sum_kernel(const double* in, int rows, int cols, double scale, double* out)
{
    __shared__ double part[8][33];
    const int c = blockIdx.x * 32 + (threadIdx.x & 31), r0 = threadIdx.x >> 5;
    double s = 0.0;
    if (c < cols)
        for (int r = r0; r < rows; r += 8) s += in[(size_t)r * cols + c];
    part[r0][threadIdx.x & 31] = s;
    __syncthreads();
    if (r0 == 0 && c < cols) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += part[k][threadIdx.x & 31];
        out[c] = t * scale;
    }
}

template <typename R, int NMAX, int FMAX, int TH>
int launch_adj(const AdjParams& a, const AdjTables<R>& tb, int blocks, cudaStream_t s)
{
    const size_t smem = (size_t)a.T * a.N * sizeof(double) + (TH / 32) * NMAX * sizeof(R);
    if (smem > 200 * 1024) return fail(LMM_ERR_INVALID, "adjoint: time steps x forward rates too large");
    static bool attr_set = false;  // set once, before any stream capture
    if (!attr_set) {
        LMM_CUDA(cudaFuncSetAttribute(adjoint_kernel<R, NMAX, FMAX, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      200 * 1024));
        attr_set = true;
    }
    adjoint_kernel<R, NMAX, FMAX, TH><<<blocks, TH, smem, s>>>(a, tb);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <typename R, int NMAX, int FMAX>
int launch_adj_threads(const AdjParams& a, const AdjTables<R>& tb, int threads, int blocks, cudaStream_t s)
{
    if (threads == 64) return launch_adj<R, NMAX, FMAX, 64>(a, tb, blocks, s);
    if (threads == 256) return launch_adj<R, NMAX, FMAX, 256>(a, tb, blocks, s);
    return launch_adj<R, NMAX, FMAX, 128>(a, tb, blocks, s);
}

template <typename R>
int launch_adj_dispatch(const AdjParams& a, const AdjTables<R>& tb, int threads, int blocks, cudaStream_t s)
{
    if (a.N <= 24 && a.F <= 4) return launch_adj_threads<R, 24, 4>(a, tb, threads, blocks, s);
    if (a.N <= 40 && a.F <= 10) return launch_adj_threads<R, 40, 10>(a, tb, threads, blocks, s);
    return fail(LMM_ERR_INVALID, "adjoint supports at most 40 forward rates and 10 factors");
}

}  // namespace

int adjoint_blocks(int P, int threads)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int want = sms * (512 / threads);
    const int need = (P + threads - 1) / threads;
    return need < want ? need : want;
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
    for (int l = 0; l <= L.N && l < 65; l++) {
        sp.pd[l] = L.h_discount ? L.h_discount[l] : 1.0;
        sp.det[l] = L.h_num_det[l];
    }
    for (int j = 0; j < L.N && j < 64; j++) sp.delta[j] = L.h_delta[j];
    sp.ex_time = L.d_ex;
    sp.abar_partials = L.d_abar_partials;
    sp.seeds = L.d_seeds;
    sp.value_partials = L.d_value_partials;
    const int sb = (L.P + 255) / 256;
    {
        KernelTimer kt(K_ADJOINT, s, 4);
        sp.pass = 1;
        if (L.fp32) seed_kernel<float><<<sb, 256, 0, s>>>(sp);
        else seed_kernel<double><<<sb, 256, 0, s>>>(sp);
        column_sum_kernel<<<(L.N + 1 + 31) / 32, 256, 0, s>>>(L.d_abar_partials, sb, L.N + 1, 1.0 / (double)L.P, L.d_abar);
        column_sum_kernel<<<1, 256, 0, s>>>(L.d_value_partials, sb, 1, 1.0 / (double)L.P, L.d_value_out);
        sp.pass = 2;
        if (L.fp32) seed_kernel<float><<<sb, 256, 0, s>>>(sp);
        else seed_kernel<double><<<sb, 256, 0, s>>>(sp);
        LMM_CUDA(cudaGetLastError());
    }
    // ---- reverse sweep over the paths
    AdjParams ap;
    ap.T = L.T;
    ap.N = L.N;
    ap.F = L.F;
    ap.P = L.P;
    ap.stride = L.stride;
    ap.ckpt_is_L = L.ckpt_is_L;
    ap.capped = !std::isinf(L.cap);
    ap.t_end = L.t_end;
    ap.n_eff = L.n_eff;
    ap.cap = L.cap;
    ap.first = L.d_first;
    ap.init = L.d_init;
    ap.seeds = L.d_seeds;
    ap.vega_partials = L.d_vega_partials;
    ap.delta_partials = L.d_delta_partials;
    const int blocks = L.blocks;
    int rc;
    {
        KernelTimer kt(K_ADJOINT, s);
        if (L.fp32) {
            AdjTables<float> tb{static_cast<const float*>(L.d_lam), static_cast<const float*>(L.d_f),
                                static_cast<const float*>(L.d_sigma), static_cast<const float*>(L.d_var_half),
                                static_cast<const float*>(L.d_inv_delta), static_cast<const float*>(L.d_dt), L.d_dw, L.d_ckpt};
            rc = launch_adj_dispatch<float>(ap, tb, L.threads, blocks, s);
        } else {
            AdjTables<double> tb{static_cast<const double*>(L.d_lam), static_cast<const double*>(L.d_f),
                                 static_cast<const double*>(L.d_sigma), static_cast<const double*>(L.d_var_half),
                                 static_cast<const double*>(L.d_inv_delta), static_cast<const double*>(L.d_dt), L.d_dw, L.d_ckpt};
            rc = launch_adj_dispatch<double>(ap, tb, L.threads, blocks, s);
        }
    }
    if (rc) return rc;
    {
        KernelTimer kt(K_ADJOINT, s, 2);
        column_sum_kernel<<<(L.T * L.N + 31) / 32, 256, 0, s>>>(L.d_vega_partials, blocks, L.T * L.N, 1.0, L.d_vegas);
        column_sum_kernel<<<(L.N + 31) / 32, 256, 0, s>>>(L.d_delta_partials, blocks, L.N, 1.0, L.d_deltas);
        LMM_CUDA(cudaGetLastError());
    }
    return LMM_OK;
}

}  // namespace lmm
