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

// Byte offsets of the step's work arrays: vf, an unused slot, adfh, lo, adfv,
// R+/R- (interleaved per layer), the same again. The sizes do not depend on
// the tracer grouping of the FP32 form.
template <typename R>
WorkspaceLayout workspace_layout(const DMesh& m, int K) {
  WorkspaceLayout w;
  const long long E = m.E, N = m.N, LZ = m.LZ, LW = m.LW, s = sizeof(R);
  auto al = [](long long b) { return (b + 255) / 256 * 256; };
  long long off = 0;
  w.off[0] = off; off += al(E * LZ * s);          // vf
  w.off[1] = off;                                         // (unused slot)
  w.off[2] = off; off += al((long long)K * E * LZ * s);  // adfh
  w.off[3] = off; off += al((long long)K * N * LZ * s);  // lo
  w.off[4] = off; off += al((long long)K * N * LW * s);  // adfv
  w.off[5] = off; off += al(2LL * K * N * LZ * s);       // R+, R- interleaved
  w.off[6] = w.off[5];                                    // (same array)
  w.total = off;
  return w;
}

WorkspaceLayout workspace_layout_f64(const DMesh& m, int K);
WorkspaceLayout workspace_layout_f32(const DMesh& m, int K);
int launch_stages_f64(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err);
int launch_stages_f32(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err);
int launch_stages_f64fast(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
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
