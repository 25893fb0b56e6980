// Fast FP64 form of the step: the FP64 kernels compiled with fused
// multiply-add, divisions by constants as products with the reciprocal
// constant, and dt / areasvol and 1 / hnode_new formed once per layer (their
// own inline namespace, fgb::fast64). Not bit-exact against the reference's
// evaluation order; within 1e-12 of it (relative max-norm, tested).
#define FGB_FAST64 1
#include "fgb_step.cuh"

namespace fgb {
int launch_stages_f64fast(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                          std::string* err) {
  return launch_stages<double>(m, d, mask, s, nlaunch, err);
}
}  // namespace fgb
