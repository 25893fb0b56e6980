// Step entry point that allocates nothing: its scratch lives in a file-scope
// device array instead of a caller-provided workspace.
//
// Some callers cannot allocate device memory themselves: a host model whose
// framework owns all GPU memory through its own pool allocator, and whose
// coupling layer may not call cudaMalloc behind that allocator's back, can
// still pass its tracer, velocity and geometry buffers but has nowhere to put
// the step's temporary arrays. This entry point keeps them in
// g_static_workspace, a fixed array of FGB_STATIC_WORKSPACE_BYTES that every
// GPU loading this library holds until the process exits.
#include <cuda_runtime.h>

#include <string>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"

namespace {

static __device__ __align__(256) unsigned char g_static_workspace[FGB_STATIC_WORKSPACE_BYTES];

constexpr int kMaxDevices = 64;
void* g_ws_addr[kMaxDevices] = {nullptr};  // device address of the array, per device

// The array's name is a host-side stand-in in host code; its device address
// comes from cudaGetSymbolAddress, once per device with that device current.
int static_ws_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    fgb::set_error("fgb_adv_step_static: no usable current device");
    return -1;
  }
  if (!g_ws_addr[dev]) {
    void* p = nullptr;
    cudaError_t ce = cudaGetSymbolAddress(&p, g_static_workspace);
    if (ce != cudaSuccess || !p) {
      fgb::set_error(std::string("fgb_adv_step_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(ce));
      return -1;
    }
    g_ws_addr[dev] = p;
  }
  *out = g_ws_addr[dev];
  return 0;
}

}  // namespace

extern "C" {

long long fgb_static_workspace_bytes(void) { return (long long)FGB_STATIC_WORKSPACE_BYTES; }

int fgb_adv_step_static(const fgb_mesh* m, const fgb_step_desc* d, void* stream) {
  if (!m || !d) {
    fgb::set_error("fgb_adv_step_static: null argument");
    return -1;
  }
  const long long need = fgb_workspace_bytes(m, d->precision, d->ntracers);
  if (need < 0) {
    fgb::set_error("fgb_adv_step_static: bad precision or tracer count");
    return -1;
  }
  if (need > (long long)FGB_STATIC_WORKSPACE_BYTES) {
    fgb::set_error("fgb_adv_step_static: this mesh and tracer count need " + std::to_string(need) +
                   " bytes of scratch, more than the static workspace of " +
                   std::to_string((long long)FGB_STATIC_WORKSPACE_BYTES) +
                   " bytes; use fgb_adv_step with a caller-provided workspace");
    return -1;
  }
  void* ws = nullptr;
  if (static_ws_address(&ws)) return -1;
  fgb_step_desc s = *d;
  s.workspace = ws;
  s.workspace_bytes = (long long)FGB_STATIC_WORKSPACE_BYTES;
  return fgb_adv_step(m, &s, stream);
}

}  // extern "C"
