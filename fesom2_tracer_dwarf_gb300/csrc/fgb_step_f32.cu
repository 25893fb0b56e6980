// FP32 form of the step (storage and arithmetic in single precision).
#include "fgb_step.cuh"

namespace fgb {
WorkspaceLayout workspace_layout_f32(const DMesh& m, int K) { return workspace_layout<float>(m, K); }
int launch_stages_f32(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err) {
  return launch_stages<float>(m, d, mask, s, nlaunch, err);
}
}  // namespace fgb
