// FP32 form of the step: argument checks and dispatch to the kernels of the
// tracer-group width (fgb_fast.cuh).
#include <cstdint>

#include "fgb_internal.hpp"

namespace fgb {
namespace fast {
int launch_fast_kv1(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s);
int launch_fast_kv2(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s);
int launch_fast_kv4(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s);
}  // namespace fast

WorkspaceLayout workspace_layout_f32(const DMesh& m, int K) { return workspace_layout<float>(m, K); }

int launch_stages_f32(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                      std::string* err) {
  using namespace fast;
  *nlaunch = 0;
  const int K = d.ntracers;
  const int KV = d.tracer_vec <= 1 ? 1 : d.tracer_vec;
  if (K < 1 || K > 65535) { *err = "ntracers must be in 1..65535"; return -1; }
  if (KV != 1 && KV != 2 && KV != 4) { *err = "tracer_vec must be 0, 1, 2 or 4"; return -1; }
  if (K % KV) { *err = "tracer_vec must divide ntracers"; return -1; }
  if (d.hor < 0 || d.hor > 2 || d.ver < 0 || d.ver > 3 || d.lim < 0 || d.lim > 1) {
    *err = "unknown advection scheme";
    return -1;
  }
  if (!d.T || !d.vel || !d.w || !d.we || !d.workspace) { *err = "null device pointer"; return -1; }
  if (d.ab_order < 0 || d.ab_order > 2) { *err = "ab_order must be 0, 1 or 2"; return -1; }
  const WorkspaceLayout wl = workspace_layout<float>(m, K);
  if (d.workspace_bytes < wl.total) { *err = "workspace too small"; return -1; }
  if ((d.ver == FGB_VER_QR4C || d.ver == FGB_VER_PPM) && m.min_layers < 2) {
    *err = "QR4C/PPM need at least two layers in every column";
    return -1;
  }
  if (d.hor != FGB_HOR_UPW1 && !m.fast_tri_ok) {
    *err = "FP32 MUSCL/MFCT: an upwind triangle does not hold its edge node";
    return -1;
  }
  // Offsets inside a group are 32-bit (units of KV floats).
  const long long lim = 1LL << 32;
  if ((long long)m.E * m.LZ >= lim || 2LL * m.N * m.LZ >= lim || (long long)m.N * m.LW >= lim ||
      (long long)m.M * m.LZ >= lim) {
    *err = "mesh too large for the FP32 form (edges x padded layers must stay below 2^32)";
    return -1;
  }
  const uintptr_t al = 4u * KV;
  auto misaligned = [&](const void* p) { return p && (reinterpret_cast<uintptr_t>(p) % al) != 0; };
  if (misaligned(d.T) || misaligned(d.TA) || misaligned(d.TAout) || misaligned(d.del) || misaligned(d.Tlo) ||
      reinterpret_cast<uintptr_t>(d.vel) % 8 != 0 || d.strideT % KV != 0 || (d.TA && d.strideTA % KV != 0)) {
    *err = "FP32 tracer arrays must be aligned to their group (4 * tracer_vec bytes, strides multiples of tracer_vec)";
    return -1;
  }
  // the workspace's arrays start at multiples of 256 bytes from its base; the
  // pairs of limiting factors are read and written 32 bytes at a time
  if (reinterpret_cast<uintptr_t>(d.workspace) % 32 != 0) {
    *err = "the FP32 form's workspace must be 32-byte aligned (cudaMalloc gives 256)";
    return -1;
  }
  const bool wsplit = d.lim == FGB_LIM_FCT && d.wi;
  if (wsplit) {
    if (m.min_layers < 2) { *err = "w_split needs at least two layers in every column"; return -1; }
    if (vimpl_block_bytes(m.LZ, KV) > 227 * 1024) { *err = "w_split: too many layers for one block"; return -1; }
    if (reinterpret_cast<uintptr_t>(d.wi) % 4 != 0) { *err = "wi must be 4-byte aligned"; return -1; }
  }
  char* ws = static_cast<char*>(d.workspace);
  FastPtrs a;
  a.T = static_cast<float*>(d.T);
  a.TA = d.TA ? static_cast<const float*>(d.TA) : a.T;
  a.TAout = static_cast<float*>(d.TAout);
  a.vel = static_cast<const float*>(d.vel);
  a.w = static_cast<const float*>(d.w);
  a.we = static_cast<const float*>(d.we);
  a.wi = wsplit ? static_cast<const float*>(d.wi) : nullptr;
  a.vf = reinterpret_cast<float*>(ws + wl.off[0]);
  a.adfh = reinterpret_cast<float*>(ws + wl.off[2]);
  a.lo = reinterpret_cast<float*>(ws + wl.off[3]);
  a.adfv = reinterpret_cast<float*>(ws + wl.off[4]);
  a.rpm = reinterpret_cast<float*>(ws + wl.off[5]);
  a.del = static_cast<float*>(d.del);
  a.gT = d.strideT;
  a.gTA = d.TA ? d.strideTA : d.strideT;
  a.gE = (long long)m.E * m.LZ * KV;
  a.gN = (long long)m.N * m.LZ * KV;
  a.gW = (long long)m.N * m.LW * KV;
  a.G = K / KV;
  a.dt = (float)d.dt;
  a.ph = (float)d.ph;
  a.pv = (float)d.pv;
  a.wsplit_fused = 0;  // set per launch of the LO kernel
  a.comp = ~d.fp32_plain_sums & 7;
  a.Tlo = d.del ? nullptr : static_cast<float*>(d.Tlo);
  a.ab2 = d.ab_order == 2;
  a.ab_old = (float)(-(0.5 + d.ab_eps));
  a.ab_new = (float)(1.5 + d.ab_eps);
  auto pick = [](int want, int x, int y, int z, int def) { return (want == x || want == y || want == z) ? want : def; };
  LaunchArgs L;
  L.mask = mask;
  L.edge_warps = pick(d.cfg[0], 2, 4, 8, 8);
  L.nw_lo = pick(d.cfg[1], 1, 2, 4, 4);
  L.nw_ratio = pick(d.cfg[2], 1, 2, 4, 4);
  L.nw_upd = pick(d.cfg[3], 1, 2, 4, 4);
  auto ns = [](int want, int def) { return (want == 1 || want == 2) ? want : def; };
  L.ns_h = ns(d.cfg[7], 2);
  // LO: 3 (the default where it applies) the whole-column kernel for columns
  // of at most 64 layers without w_split; 1 or 2 layers per lane per pass
  L.ns_lo = (d.cfg[4] == 1 || d.cfg[4] == 2) ? d.cfg[4] : (m.LZ <= 64 && !(d.lim == FGB_LIM_FCT && d.wi) ? 3 : 2);
  // ratio: 1 or 2 layers per lane with shared-memory staging, or 3 (the default)
  // the whole column per warp without shared memory
  L.ns_ratio = (d.cfg[5] >= 1 && d.cfg[5] <= 4) ? d.cfg[5] : 0;
  L.ns_upd = ns(d.cfg[6], 1);
  L.vimpl_thomas = d.cfg[8] == 1;
  // the tiled edge kernel stages rows with 16-byte asynchronous copies
  auto al16 = [](const void* p) { return p == nullptr || reinterpret_cast<uintptr_t>(p) % 16 == 0; };
  L.hflux_tile = d.cfg[9] == 1 && al16(d.T) && al16(d.TA) && al16(d.workspace) && (d.strideT * 4) % 16 == 0 &&
                 (!d.TA || (d.strideTA * 4) % 16 == 0);
  L.hor = d.hor;
  L.ver = d.ver;
  L.fct = d.lim == FGB_LIM_FCT;
  int n = 0;
  if (KV == 4) n = launch_fast_kv4(m, a, L, s);
  else if (KV == 2) n = launch_fast_kv2(m, a, L, s);
  else n = launch_fast_kv1(m, a, L, s);
  *nlaunch = n;
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    *err = std::string("kernel launch failed: ") + cudaGetErrorString(ce);
    return -1;
  }
  return 0;
}
}  // namespace fgb
