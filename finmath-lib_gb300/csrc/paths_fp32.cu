// paths_fp32.cu -- K2 (mixed-precision form): the fused path kernel in FP32.
//
// Same recurrence as paths_fp64.cu (EulerSchemeFromProcessModel.java:170-326 in its default
// EULER_FUNCTIONAL form, with the spot drift of LIBORMarketModelFromCovarianceModel.java:
// 1125-1191): the log-Euler step Y' = log L + d, L' = min(exp(Y'), cap) is carried as
// L' = min(L exp(d), cap) on the forward rates themselves, so the path state is one FP32
// register per component.  The drift running sums (carried with dt and the increments,
// G_k = dW_k + dt S_k) use paired FP32 FMAs, exp and the measure-change ratio one SFU
// instruction each (ex2.approx, rcp.approx).  The numeraire accrual and its adjustment sums stay FP64, as do the
// regression sums and payoff averages downstream.  The error against the FP64 form is
// measured and reported, not assumed.
//
// GB300 layout: one thread per path, the forward vector in registers for all steps.  Each
// warp stages the next step's component rows in shared memory with cp.async while it works
// on the current step -- per component one row of whole float4 vectors: the factor loadings
// (zero padded to FMAX), the step's deterministic drift term (variance * -0.5 * dt) and
// 1/delta, so a component-step reads its row with three 16-byte loads -- and each thread
// prefetches its own path's next increments the same way, so the step loop does not wait on
// global memory.  The sums over factors run on paired FP32 FMAs (__ffma2_rn, two factors
// per instruction), the drift's dot product in two independent accumulators to halve its
// dependency chain.  When the model has exactly NMAX components (EXACT) the component loop
// carries no run-time bound checks.
#include "lmm_internal.h"
#include "fp64math.cuh"
#include "reduce.cuh"
#include "unroll_range.cuh"
#include "euler_fp32.cuh"

namespace lmm {
namespace {

constexpr int kPathThreads = 128;

using euler32::row_pitch;

__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(float* dst, const float* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int NMAX, int FMAX>
struct Smem32 {
    static constexpr int FP = row_pitch(FMAX);
    float table[kPathThreads / 32][2][NMAX * FP];   // per warp, two steps: rows [NMAX][FP]
    float dw[2][FMAX][kPathThreads];                // per thread column, two steps
    double wsum[kPathThreads / 32][NMAX];           // numeraire-adjustment warp sums
};

// resident blocks per SM: the FP32 state of NMAX components, the factor pairs and the
// staged row of one component fit the register budget this leaves
__host__ __device__ constexpr int fp32_min_blocks(int nmax) { return nmax <= 24 ? 8 : nmax <= 40 ? 6 : 3; }

// CAPPED: the model caps the forward rates (one FMNMX per component-step, a compile-time
// variant so that uncapped models pay nothing).
template <int NMAX, int FMAX, bool CAPPED, bool EXACT>
__global__ void __launch_bounds__(kPathThreads, fp32_min_blocks(NMAX))
    paths_fp32_kernel(const PathLaunch a, const float* __restrict__ rows32)
{
    using SM = Smem32<NMAX, FMAX>;
    constexpr int FP = SM::FP;
    constexpr int FH = (FMAX + 1) / 2;  // factor pairs
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SM& sm = *reinterpret_cast<SM*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int p = blockIdx.x * kPathThreads + tid;
    const bool active = p < a.P;
    const int N = EXACT ? NMAX : a.N, F = a.F, P = a.P;
    const float cap = CAPPED ? (float)a.libor_cap : 0.0f;
    const float* dW = static_cast<const float*>(a.d_dw);
    float* states = static_cast<float*>(a.d_states);

    // step i's component rows (pitch FP) into this warp's buffer i&1, and this thread's
    // increments into dw[i&1]
    auto prefetch = [&](int i) {
        float* tb = sm.table[warp][i & 1];
        const float* ls = rows32 + (size_t)i * N * FP;
        for (int q = lane; q < N * FP / 4; q += 32) cp_async16(tb + 4 * q, ls + 4 * q);
        if (active) {
            const float* src = dW + (size_t)i * F * P + p;
            for (int k = 0; k < F; k++) cp_async4(&sm.dw[i & 1][k][tid], src + (size_t)k * P);
        }
        cp_async_commit();
    };
    if (a.T > 0) prefetch(0);

    float L[NMAX];
#pragma unroll
    for (int j = 0; j < NMAX; j++) {
        float v = j < N ? __ldg(a.d_init32 + j) : 0.0f;
        if (CAPPED) v = fminf(v, cap);
        L[j] = v;
    }
    // the forward rates of all components into rows [N][P] starting at dst (a running
    // pointer: one address increment per component)
    auto store_rows = [&](float* dst) {
#pragma unroll
        for (int j = 0; j < NMAX; j++)
            if (EXACT || j < N) {
                *dst = L[j];
                dst += P;
            }
    };
    {
        const int slot = __ldg(a.d_obs_slot + 0);
        if (slot >= 0 && active) store_rows(states + (size_t)slot * N * P + p);
        if (a.d_ckpt && active) store_rows(static_cast<float*>(a.d_ckpt) + p);
    }
    for (int i = 0; i < a.T; i++) {
        const int first = __ldg(a.d_first + i);
        // the step's sums in base-2 units: G and dt carry log2(e), so that exp(d) = exp2(d')
        const float dt = euler32::step_dt(a.d_dt32, i);
        cp_async_wait();
        __syncwarp();  // the warp's staged table of step i is visible to every lane
        // G_k = dW_k + dt S_k, the drift's running sum S_k = sum_{l<=j} os_l lambda_lk carried
        // with dt and the increments: the step increment of component j is
        // sum_k G_k lambda_jk - dt variance_j / 2 (two paired FMAs per factor pair, not three)
        float2 G2[FH];
#pragma unroll
        for (int m = 0; m < FH; m++) {
            const int k0 = 2 * m, k1 = 2 * m + 1;
            G2[m] = euler32::start_sum((k0 < F && active) ? sm.dw[i & 1][k0][tid] : 0.0f,
                                       (k1 < F && k1 < FMAX && active) ? sm.dw[i & 1][k1 < FMAX ? k1 : 0][tid] : 0.0f);
        }
        if (i + 1 < a.T) prefetch(i + 1);  // buffers (i+1)&1 were last read in step i-1
        const float* tb = sm.table[warp][i & 1];
        for_up_from<NMAX>(first, [&](auto jc) {
            constexpr int j = decltype(jc)::value;
            if (EXACT || j < N) {
                float lr[FP];
#pragma unroll
                for (int q = 0; q < FP / 4; q++) {
                    const float4 v = *reinterpret_cast<const float4*>(tb + j * FP + 4 * q);
                    lr[4 * q] = v.x;
                    lr[4 * q + 1] = v.y;
                    lr[4 * q + 2] = v.z;
                    lr[4 * q + 3] = v.w;
                }
                L[j] = euler32::component_step<FMAX, CAPPED>(L[j], lr, dt, G2, cap);
            }
        });
        const int slot = __ldg(a.d_obs_slot + i + 1);
        if (slot >= 0 && active) store_rows(states + (size_t)slot * N * P + p);
        if (a.d_ckpt && active && (i + 1) % a.ckpt_stride == 0)
            store_rows(static_cast<float*>(a.d_ckpt) + (size_t)((i + 1) / a.ckpt_stride) * N * P + p);
    }
    cp_async_wait();
    // FP64 spot numeraire from the frozen fixings (as paths_fp64.cu), the FP32 fixings
    // widened in integer operations, and 1/N by the FP32 reciprocal refined by one Newton
    // step in FP64 (relative error about 2^-46, far below the FP32 path state's).  The warp
    // sums of 1/N_l for the numeraire adjustment are transposed reductions over chunks of
    // eight tenor times: three exchange levels that each halve the values a lane holds
    // (lanes with the level's bit set keep the upper half, the others the lower half, and
    // add what the partner sends), then two plain levels, so a chunk costs 9 FP64 adds per
    // warp instead of 40.  The block partials: compensated across the block's warps.
    static_assert(NMAX % 8 == 0, "the transposed reduction works on chunks of eight tenor times");
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
            if (EXACT || l < N) {
                const double delta = __ldg(a.d_delta + l);
                const double Ll = f32_to_f64_int(L[l]);
                if (l < a.num_det_prefix) Nv = Ll * (delta * Nv) + Nv;
                else Nv = Nv * (1.0 + Ll * delta);
                if (active) {
                    a.d_numeraire[(size_t)(l + 1) * P + p] = Nv;
                    const double r0 = f32_to_f64_int(__frcp_rn(f64_to_f32_int(Nv)));
                    v[q] = fma(r0, fma(-Nv, r0, 1.0), r0);
                    if (a.d_inv_numeraire) a.d_inv_numeraire[(size_t)(l + 1) * P + p] = v[q];
                }
            }
        }
        const double sum = warp_sum8_transposed(v, lane);
        const int idx = 8 * c + ((lane >> 2) & 7);
        if ((lane & 3) == 0 && idx < N) sm.wsum[warp][idx] = sum;
    }
    __syncthreads();
    if (tid < N) {
        dd acc{0.0, 0.0};
#pragma unroll
        for (int w = 0; w < kPathThreads / 32; w++) acc = dd_add_d(acc, sm.wsum[w][tid]);
        double* o = a.d_inv_num_partials + ((size_t)blockIdx.x * N + tid) * 2;
        o[0] = acc.hi;
        o[1] = acc.lo;
    }
}

template <int NMAX, int FMAX, bool CAPPED, bool EXACT>
int launch_t(const PathLaunch& a, const float* rows32, cudaStream_t s, int blocks)
{
    const size_t smem = sizeof(Smem32<NMAX, FMAX>);
    static bool attr_set = false;  // set once, before any stream capture
    if (!attr_set) {
        LMM_CUDA(cudaFuncSetAttribute(paths_fp32_kernel<NMAX, FMAX, CAPPED, EXACT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    paths_fp32_kernel<NMAX, FMAX, CAPPED, EXACT><<<blocks, kPathThreads, smem, s>>>(a, rows32);
    LMM_CUDA(cudaGetLastError());
    return LMM_OK;
}

template <int NMAX, int FMAX>
int launch_c(const PathLaunch& a, const float* rows32, cudaStream_t s, int blocks)
{
    const bool capped = !isinf(a.libor_cap);
    if (a.N == NMAX)
        return capped ? launch_t<NMAX, FMAX, true, true>(a, rows32, s, blocks)
                      : launch_t<NMAX, FMAX, false, true>(a, rows32, s, blocks);
    return capped ? launch_t<NMAX, FMAX, true, false>(a, rows32, s, blocks)
                  : launch_t<NMAX, FMAX, false, false>(a, rows32, s, blocks);
}

int fp32_fmax(int N, int F)
{
    if (N <= 24 && F <= 4) return 4;
    if (N <= 40 && F <= 10) return 10;
    return 16;
}

}  // namespace

int paths_fp32_rows(int N, int F, int* fmax)
{
    const int fm = fp32_fmax(N, F);
    if (fmax) *fmax = fm;
    return row_pitch(fm);
}

int launch_paths_fp32(const PathLaunch& a, const float* rows32, cudaStream_t s, int* blocks_out)
{
    const int blocks = path_blocks(a.P);
    if (blocks_out) *blocks_out = blocks;
    KernelTimer kt(K_PATHS_FP32, s);
    if (a.N <= 24 && a.F <= 4) return launch_c<24, 4>(a, rows32, s, blocks);
    if (a.N <= 40 && a.F <= 10) return launch_c<40, 10>(a, rows32, s, blocks);
    if (a.N <= 64 && a.F <= 16) return launch_c<64, 16>(a, rows32, s, blocks);
    return fail(LMM_ERR_INVALID, "mixed path kernel supports at most 64 forward rates and 16 factors");
}

}  // namespace lmm
