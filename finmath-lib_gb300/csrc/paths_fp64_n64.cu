// paths_fp64_n64.cu -- the FP64 path kernels for up to 64 forward rates and 16 factors
// (their own translation unit: the widest unrolled instantiations take the longest to compile).
#include "paths_fp64.cuh"

namespace lmm {

int launch_paths_fp64_n64(const PathLaunch& a, cudaStream_t s, int blocks) { return launch_t<64, 16>(a, s, blocks); }

}  // namespace lmm
