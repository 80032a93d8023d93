// paths_fp64.cu -- launchers of the FP64 path kernels (paths_fp64.cuh); the 64-rate
// instantiations compile separately (paths_fp64_n64.cu) so that the two build in parallel.
#include "paths_fp64.cuh"

namespace lmm {

int launch_paths_fp64_n64(const PathLaunch& a, cudaStream_t s, int blocks);
int launch_paths_fp64_n80(const PathLaunch& a, cudaStream_t s, int blocks);

int path_blocks(int P) { return (P + kPathThreads - 1) / kPathThreads; }

int paths_fp64_fmax(int N, int F)
{
    if (N <= 24 && F <= 4) return 4;
    if (N <= 40 && F <= 10) return 10;
    return 16;
}

int launch_paths_fp64(const PathLaunch& a, cudaStream_t s, int* blocks_out)
{
    const int blocks = path_blocks(a.P);
    if (blocks_out) *blocks_out = blocks;
    KernelTimer kt(K_PATHS_FP64, s);
    if (a.N <= 24 && a.F <= 4) return launch_t<24, 4>(a, s, blocks);
    if (a.N <= 40 && a.F <= 10) return launch_t<40, 10>(a, s, blocks);
    if (a.N <= 64 && a.F <= 16) return launch_paths_fp64_n64(a, s, blocks);
    if (a.N <= kMaxForwardRates && a.F <= 16) return launch_paths_fp64_n80(a, s, blocks);
    return fail(LMM_ERR_INVALID, "FP64 path kernel supports at most 80 forward rates and 16 factors");
}

int launch_replay_fp64(const PathLaunch& path, const ReplaySegment& r, cudaStream_t s)
{
    PathLaunch a = path;
    a.rp_n0 = r.n0;
    a.rp_n_stop = r.n_stop;
    a.rp_n_eff = r.n_eff;
    a.rp_ckpt = r.ckpt;
    a.rp_seg = r.seg;
    const int blocks = path_blocks(a.P);
    if (a.N <= 24 && a.F <= 4) return replay_t<24, 4>(a, s, blocks);
    if (a.N <= 40 && a.F <= 10) return replay_t<40, 10>(a, s, blocks);
    return kReplayNotFast;
}

}  // namespace lmm
