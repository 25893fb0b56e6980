// Internal declarations shared by the translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fesom_tracer_gb300.h"
#include "fgb_device.hpp"
#include "fgb_hmesh.hpp"

namespace fgb {

struct WorkspaceLayout {
  long long off[7];
  long long total;
};

WorkspaceLayout workspace_layout_f64(const DMesh& m, int K);
WorkspaceLayout workspace_layout_f32(const DMesh& m, int K);
int launch_stages_f64(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err);
int launch_stages_f32(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err);

void set_error(const std::string& msg);

}  // namespace fgb

struct fgb_hmesh {
  fgb::HostMesh* m;
};

struct fgb_mesh {
  fgb::DMesh d;
  std::vector<void*> allocs;
  int device;
  // device copies that fgb_mesh_update_vertical rewrites
  double *hnode64, *hnode_new64, *helem64;
  float *hnode32, *hnode_new32, *helem32;
};
