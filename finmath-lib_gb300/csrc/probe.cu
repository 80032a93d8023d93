// probe.cu -- FP64 FMA throughput probe.  The plain-FP64 path kernel is bound by the
// FP64 pipe, whose rate is not among the separately measured peaks (copy bandwidth, bf16
// GEMM); this kernel measures it on the running GPU (independent DFMA chains, enough
// warps to saturate the pipe).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fp64math.cuh"
#include "lmm_internal.h"

namespace lmm {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void dfma_probe_kernel(double seed, double* sink)
{
    double a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed + (double)(threadIdx.x + c);
    const double m = 0.9999999999999, b = 1e-7;
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) a[c] = fma(a[c], m, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += a[c];
    if (s == 12345.678) sink[0] = s;  // keeps the chains live
}

// exp_small against CUDA's exp on a grid of [-1, 1] and rcp_newton against the correctly
// rounded division on [1, 4097); errors in ulps of the reference value
__global__ void fp64_math_check_kernel(const double* tab, int64_t n, double* err_exp, double* err_rcp)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = (double)i / (double)(n - 1);
    const double d = -1.0 + 2.0 * u + 1e-9 * (double)(i & 7);
    const double s = 1.0 + 4096.0 * u + 1e-7 * (double)(i % 13);
    const double e_ref = exp(d), r_ref = 1.0 / s;
    const double e = exp_small(d, tab), r = rcp_newton(s);
    int ex;
    frexp(e_ref, &ex);
    err_exp[i] = fabs(e - e_ref) / ldexp(1.0, ex - 53);
    frexp(r_ref, &ex);
    err_rcp[i] = fabs(r - r_ref) / ldexp(1.0, ex - 53);
}

}  // namespace

void fp64_exp_table(double out[2 * kExpTableHalf + 1])
{
    for (int k = -kExpTableHalf; k <= kExpTableHalf; k++)
        out[k + kExpTableHalf] = (double)expl((long double)k / (long double)kExpTableHalf);
}

}  // namespace lmm

extern "C" int lmm_fp64_math_check(int64_t n, double* max_ulp_exp, double* max_ulp_rcp)
{
    using namespace lmm;
    if (!max_ulp_exp || !max_ulp_rcp || n < 2 || n > (int64_t)1 << 26) return fail(LMM_ERR_INVALID, "need 2 <= n <= 2^26 and outputs");
    double tab[2 * kExpTableHalf + 1];
    fp64_exp_table(tab);
    double *d_tab = nullptr, *d_e = nullptr, *d_r = nullptr;
    LMM_CUDA(cudaMalloc(&d_tab, sizeof(tab)));
    LMM_CUDA(cudaMalloc(&d_e, sizeof(double) * (size_t)n));
    LMM_CUDA(cudaMalloc(&d_r, sizeof(double) * (size_t)n));
    LMM_CUDA(cudaMemcpy(d_tab, tab, sizeof(tab), cudaMemcpyHostToDevice));
    fp64_math_check_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_tab, n, d_e, d_r);
    LMM_CUDA(cudaGetLastError());
    std::vector<double> he((size_t)n), hr((size_t)n);
    LMM_CUDA(cudaMemcpy(he.data(), d_e, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    LMM_CUDA(cudaMemcpy(hr.data(), d_r, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    cudaFree(d_tab);
    cudaFree(d_e);
    cudaFree(d_r);
    double me = 0.0, mr = 0.0;
    for (int64_t i = 0; i < n; i++) {
        me = std::max(me, he[(size_t)i]);
        mr = std::max(mr, hr[(size_t)i]);
    }
    *max_ulp_exp = me;
    *max_ulp_rcp = mr;
    return LMM_OK;
}

extern "C" int lmm_probe_fp64_fma_rate(double* out)
{
    using namespace lmm;
    if (!out) return fail(LMM_ERR_INVALID, "null argument");
    int dev = 0, sms = 0;
    LMM_CUDA(cudaGetDevice(&dev));
    LMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    LMM_CUDA(cudaMalloc(&sink, sizeof(double)));
    cudaEvent_t e0, e1;
    LMM_CUDA(cudaEventCreate(&e0));
    LMM_CUDA(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256;
    dfma_probe_kernel<<<blocks, threads>>>(1.0, sink);  // warm-up
    LMM_CUDA(cudaEventRecord(e0));
    dfma_probe_kernel<<<blocks, threads>>>(1.0, sink);
    LMM_CUDA(cudaEventRecord(e1));
    LMM_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    LMM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    *out = (double)blocks * threads * kChains * (double)kIters / (ms * 1e-3);
    return LMM_OK;
}
