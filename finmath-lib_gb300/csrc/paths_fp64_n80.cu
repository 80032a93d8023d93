#include "paths_fp64.cuh"

namespace lmm {

// 65 to 80 forward rates: every scheme, measure and state space on the general kernel
int launch_paths_fp64_n80(const PathLaunch& a, cudaStream_t s, int blocks) { return launch_general<80, 16>(a, s, blocks); }

}  // namespace lmm
