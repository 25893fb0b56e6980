// Argument checks of fgb_adv_step_static, kept free of CUDA so that they can
// be compiled and tested on a machine without a GPU.
#pragma once
#include <string>

namespace fgb {

// precision: FGB_FP64 (0), FGB_FP32 (1) or FGB_FP64_FAST (2); need: the scratch bytes the mesh
// and tracer count take (fgb_workspace_bytes), cap: the static array's size.
// mesh_device: the device the mesh was uploaded on; current_device: the
// calling thread's current device. Returns 0 when the call may proceed, else
// -1 with the reason in *err.
inline int static_ws_precheck(int precision, int ntracers, long long need, long long cap, int mesh_device,
                              int current_device, std::string* err) {
  if (precision != 0 && precision != 1 && precision != 2) {
    *err = "fgb_adv_step_static: unknown precision " + std::to_string(precision) +
           " (FGB_FP64, FGB_FP32 or FGB_FP64_FAST)";
    return -1;
  }
  if (ntracers < 1) {
    *err = "fgb_adv_step_static: the tracer count must be at least 1";
    return -1;
  }
  if (need < 0) {
    *err = "fgb_adv_step_static: the workspace size of this mesh is unknown";
    return -1;
  }
  if (need > cap) {
    *err = "fgb_adv_step_static: this mesh and tracer count need " + std::to_string(need) +
           " bytes of scratch, more than the static workspace of " + std::to_string(cap) +
           " bytes; use fgb_adv_step with a caller-provided workspace";
    return -1;
  }
  if (mesh_device != current_device) {
    *err = "fgb_adv_step_static: the mesh lives on device " + std::to_string(mesh_device) +
           " but the current device is " + std::to_string(current_device) +
           "; make the mesh's device current before the call";
    return -1;
  }
  return 0;
}

}  // namespace fgb
