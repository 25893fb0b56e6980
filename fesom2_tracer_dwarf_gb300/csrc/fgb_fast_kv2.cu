// FP32 kernels for tracer groups of 2.
#include "fgb_fast_launch.cuh"

namespace fgb {
namespace fast {
int launch_fast_kv2(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  return launch_fast<2>(m, a, L, s);
}
}  // namespace fast
}  // namespace fgb
