// FP64 form of the step. Compiled with -fmad=false: every product and sum is
// rounded as written, matching the CPU restatement bit for bit.
#include "fgb_step.cuh"

namespace fgb {
WorkspaceLayout workspace_layout_f64(const DMesh& m, int K) { return workspace_layout<double>(m, K); }
int launch_stages_f64(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err) {
  return launch_stages<double>(m, d, mask, s, nlaunch, err);
}
}  // namespace fgb
