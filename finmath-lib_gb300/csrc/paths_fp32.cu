// paths_fp32.cu -- K2 (mixed-precision form): the fused path kernel in FP32 log space.
//
// Same recurrence as paths_fp64.cu (EulerSchemeFromProcessModel.java:170-326 with the
// spot drift of LIBORMarketModelFromCovarianceModel.java:1125-1191), but the path state
// is kept as Y = log L in FP32 (the EULER form in log coordinates), the drift running
// sums use FP32 FMAs, and exp / the measure-change ratio use the SFU (__expf,
// __fdividef).  The numeraire accrual and its adjustment sums stay FP64, as do all
// product arithmetic and payoff sums downstream.  The error against the FP64 form is
// measured and reported, not assumed.
#include "lmm_internal.h"
#include "reduce.cuh"

namespace lmm {
namespace {

constexpr int kPathThreads = 128;

template <int NMAX, int FMAX>
__global__ void __launch_bounds__(kPathThreads) paths_fp32_kernel(const PathLaunch a, const float* __restrict__ lam32,
                                                                  const float* __restrict__ var32)
{
    const int p = blockIdx.x * kPathThreads + threadIdx.x;
    const bool active = p < a.P;
    const int N = a.N, F = a.F, P = a.P;
    const bool capped = !isinf(a.libor_cap);
    const float cap = capped ? (float)a.libor_cap : 0.0f;
    const float* dW = static_cast<const float*>(a.d_dw);
    float* states = static_cast<float*>(a.d_states);

    float Y[NMAX], L[NMAX];
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        if (j < N) {
            Y[j] = __ldg(a.d_init_log32 + j);
            float v = __expf(Y[j]);
            if (capped && v > cap) v = cap;
            L[j] = v;
        } else {
            Y[j] = 0.0f;
            L[j] = 0.0f;
        }
    }
    {
        const int slot = __ldg(a.d_obs_slot + 0);
        if (slot >= 0 && active) {
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) states[((size_t)slot * N + j) * P + p] = L[j];
        }
        if (a.d_ckpt && active) {
            float* ck = static_cast<float*>(a.d_ckpt);
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) ck[(size_t)j * P + p] = L[j];
        }
    }
    for (int i = 0; i < a.T; i++) {
        const int first = __ldg(a.d_first + i);
        const float dt = __ldg(a.d_dt32 + i);
        const float* lam = lam32 + (size_t)i * N * F;
        const float* var = var32 + (size_t)i * N;
        float dw[FMAX], S[FMAX];
#pragma unroll
        for (int k = 0; k < FMAX; k++) {
            dw[k] = (k < F && active) ? dW[((size_t)i * F + k) * P + p] : 0.0f;
            S[k] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < NMAX; j++) {
            if (j < N && j >= first) {
                const float invd = __ldg(a.d_inv_delta32 + j);
                const float os = __fdividef(L[j], L[j] + invd);
                float mu = -0.5f * __ldg(var + j);
                float diff = 0.0f;
#pragma unroll
                for (int k = 0; k < FMAX; k++) {
                    if (k < F) {
                        const float l = __ldg(lam + j * F + k);
                        S[k] = fmaf(os, l, S[k]);
                        mu = fmaf(S[k], l, mu);
                        diff = fmaf(dw[k], l, diff);
                    }
                }
                Y[j] = Y[j] + fmaf(mu, dt, diff);
                float v = __expf(Y[j]);
                if (capped && v > cap) v = cap;
                L[j] = v;
            }
        }
        const int slot = __ldg(a.d_obs_slot + i + 1);
        if (slot >= 0 && active) {
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) states[((size_t)slot * N + j) * P + p] = L[j];
        }
        if (a.d_ckpt && active && (i + 1) % a.ckpt_stride == 0) {
            float* ck = static_cast<float*>(a.d_ckpt) + (size_t)((i + 1) / a.ckpt_stride) * N * P;
#pragma unroll
            for (int j = 0; j < NMAX; j++)
                if (j < N) ck[(size_t)j * P + p] = L[j];
        }
    }
    // FP64 spot numeraire from the frozen fixings (as paths_fp64.cu).  The block partial
    // sums of 1/N_l for the numeraire adjustment: plain FP64 within a warp (lane order),
    // compensated across the block's warps (warp order).
    __shared__ double wsum[kPathThreads / 32][NMAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double Nv = 1.0;
    if (active) a.d_numeraire[p] = 1.0;
#pragma unroll
    for (int l = 0; l < NMAX; l++) {
        if (l < N) {
            const double delta = __ldg(a.d_delta + l);
            const double Ll = (double)L[l];
            if (l < a.num_det_prefix) Nv = Ll * (delta * Nv) + Nv;
            else Nv = Nv * (1.0 + Ll * delta);
            if (active) a.d_numeraire[(size_t)(l + 1) * P + p] = Nv;
            double v = active ? 1.0 / Nv : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0) wsum[warp][l] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < N) {
        dd acc{0.0, 0.0};
#pragma unroll
        for (int w = 0; w < kPathThreads / 32; w++) acc = dd_add_d(acc, wsum[w][threadIdx.x]);
        double* o = a.d_inv_num_partials + ((size_t)blockIdx.x * N + threadIdx.x) * 2;
        o[0] = acc.hi;
        o[1] = acc.lo;
    }
}

template <int NMAX, int FMAX>
int launch_t(const PathLaunch& a, const float* lam32, const float* var32, cudaStream_t s, int blocks)
{
    paths_fp32_kernel<NMAX, FMAX><<<blocks, kPathThreads, 0, s>>>(a, lam32, var32);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

}  // namespace

int launch_paths_fp32(const PathLaunch& a, const float* lam32, const float* var32, cudaStream_t s, int* blocks_out)
{
    const int blocks = path_blocks(a.P);
    if (blocks_out) *blocks_out = blocks;
    KernelTimer kt(K_PATHS_FP32, s);
    if (a.N <= 24 && a.F <= 4) return launch_t<24, 4>(a, lam32, var32, s, blocks);
    if (a.N <= 40 && a.F <= 10) return launch_t<40, 10>(a, lam32, var32, s, blocks);
    if (a.N <= 64 && a.F <= 16) return launch_t<64, 16>(a, lam32, var32, s, blocks);
    return fail(LMM_ERR_INVALID, "mixed path kernel supports at most 64 forward rates and 16 factors");
}

}  // namespace lmm
