// FP32 kernels for tracer groups of 4.
#include "fgb_fast_launch.cuh"

namespace fgb {
namespace fast {
int launch_fast_kv4(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  return launch_fast<4>(m, a, L, s);
}
}  // namespace fast
}  // namespace fgb
