// probe.cu -- FP64 FMA throughput probe.  The plain-FP64 path kernel is bound by the
// FP64 pipe, whose rate is not part of the measured peaks; this kernel measures
// it on the running GPU (independent DFMA chains, enough warps to saturate the pipe).
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

}  // namespace
}  // namespace lmm

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
