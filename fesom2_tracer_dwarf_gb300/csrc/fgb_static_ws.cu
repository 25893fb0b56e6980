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

#include <atomic>
#include <string>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"
#include "fgb_static_ws_check.hpp"

namespace {

static __device__ __align__(256) unsigned char g_static_workspace[FGB_STATIC_WORKSPACE_BYTES];

constexpr int kMaxDevices = 64;
// Device address of the array, per device. Two threads making their first
// call on a device at the same time both look it up and store the same
// value; the atomic slots make that well defined.
std::atomic<void*> g_ws_addr[kMaxDevices];

// The array's name is a host-side stand-in in host code; its device address
// comes from cudaGetSymbolAddress, once per device with that device current.
int static_ws_address(int dev, void** out) {
  void* p = g_ws_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    cudaError_t ce = cudaGetSymbolAddress(&p, g_static_workspace);
    if (ce != cudaSuccess || !p) {
      fgb::set_error(std::string("fgb_adv_step_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(ce));
      return -1;
    }
    g_ws_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
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
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    fgb::set_error("fgb_adv_step_static: no usable current device");
    return -1;
  }
  std::string err;
  const long long need = (d->precision == FGB_FP64 || d->precision == FGB_FP32 || d->precision == FGB_FP64_FAST)
                             ? fgb_workspace_bytes(m, d->precision, d->ntracers)
                             : -1;
  if (fgb::static_ws_precheck(d->precision, d->ntracers, need, (long long)FGB_STATIC_WORKSPACE_BYTES, m->device,
                              dev, &err)) {
    fgb::set_error(err);
    return -1;
  }
  void* ws = nullptr;
  if (static_ws_address(dev, &ws)) return -1;
  fgb_step_desc s = *d;
  s.workspace = ws;
  s.workspace_bytes = (long long)FGB_STATIC_WORKSPACE_BYTES;
  return fgb_adv_step(m, &s, stream);
}

}  // extern "C"
