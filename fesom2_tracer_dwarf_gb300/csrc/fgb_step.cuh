// Launch sequence of one tracer-advection step for a batch of tracers
// (do_oce_adv_tra, lib/oce_adv_tra_driver.F90:23-294, plus the caller's
// tendency update). Included by one translation unit per precision.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"
#include "fgb_kernels.cuh"
#include "fgb_vimpl.cuh"

namespace fgb {
#if FGB_FAST64
inline namespace fast64 {
#else
inline namespace exact64 {
#endif

constexpr int kEdgeWarps = 8;  // default edges per block
constexpr int kNodeWarps = 4;  // default node columns per block (the kernels' launch bound)


template <typename R, int HOR>
void launch_hflux(const DMesh& m, const StepPtrs<R>& a, bool fct, int ew, cudaStream_t s) {
  dim3 grid((m.E + ew - 1) / ew), block(ew * kWarp);
  if (fct) k_hflux<R, HOR, true><<<grid, block, 0, s>>>(m, a);
  else k_hflux<R, HOR, false><<<grid, block, 0, s>>>(m, a);
}

// Dynamic shared memory above the 48 KB default needs an opt-in per kernel.
template <typename F>
void allow_smem(F* kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename R, int VER, int KC>
void launch_lo(const DMesh& m, const StepPtrs<R>& a, int nw, cudaStream_t s) {
  dim3 grid((m.N + nw - 1) / nw), block(nw * kWarp);
  const size_t sm = nw * warp_smem<R>(lo_slices(KC), m.LW, 0);
  allow_smem(k_fct_lo<R, VER, KC>, sm);
  k_fct_lo<R, VER, KC><<<grid, block, sm, s>>>(m, a);
}

template <typename R, int KC>
void launch_ratio(const DMesh& m, const StepPtrs<R>& a, int nw, cudaStream_t s) {
  dim3 grid((m.N + nw - 1) / nw), block(nw * kWarp);
  const size_t sm = nw * warp_smem<R>(ratio_slices(KC), m.LW, kClBytes);
  allow_smem(k_fct_ratio<R, KC>, sm);
  k_fct_ratio<R, KC><<<grid, block, sm, s>>>(m, a);
}

template <typename R, int KC>
void launch_update(const DMesh& m, const StepPtrs<R>& a, int nw, cudaStream_t s) {
  dim3 grid((m.N + nw - 1) / nw), block(nw * kWarp);
  const size_t sm = nw * warp_smem<R>(upd_slices(KC), m.LW, 0);
  allow_smem(k_fct_update<R, KC>, sm);
  k_fct_update<R, KC><<<grid, block, sm, s>>>(m, a);
}

template <typename R, int VER, int KC>
void launch_nofct(const DMesh& m, const StepPtrs<R>& a, int nw, cudaStream_t s) {
  dim3 grid((m.N + nw - 1) / nw), block(nw * kWarp);
  const size_t sm = nw * warp_smem<R>(nofct_slices(KC), m.LW, 0);
  allow_smem(k_nofct_update<R, VER, KC>, sm);
  k_nofct_update<R, VER, KC><<<grid, block, sm, s>>>(m, a);
}

template <typename R, int KC>
void launch_lo_ver(const DMesh& m, const StepPtrs<R>& a, int ver, int nw, cudaStream_t s) {
  switch (ver) {
    case FGB_VER_QR4C: launch_lo<R, 1, KC>(m, a, nw, s); break;
    case FGB_VER_CDIFF: launch_lo<R, 2, KC>(m, a, nw, s); break;
    case FGB_VER_PPM: launch_lo<R, 3, KC>(m, a, nw, s); break;
    default: launch_lo<R, 0, KC>(m, a, nw, s); break;
  }
}

template <typename R, int KC>
void launch_nofct_ver(const DMesh& m, const StepPtrs<R>& a, int ver, int nw, cudaStream_t s) {
  switch (ver) {
    case FGB_VER_QR4C: launch_nofct<R, 1, KC>(m, a, nw, s); break;
    case FGB_VER_CDIFF: launch_nofct<R, 2, KC>(m, a, nw, s); break;
    case FGB_VER_PPM: launch_nofct<R, 3, KC>(m, a, nw, s); break;
    default: launch_nofct<R, 0, KC>(m, a, nw, s); break;
  }
}

// Tracers per node-kernel chunk: the requested value if it divides K, else the
// largest of 4, 2, 1 that does.
inline int pick_kc(int K, int want) {
  if ((want == 1 || want == 2 || want == 4) && K % want == 0) return want;
  return (K % 4 == 0) ? 4 : ((K % 2 == 0) ? 2 : 1);
}

template <typename R>
int launch_stages(const DMesh& m, const fgb_step_desc& d, int mask, cudaStream_t s, int* nlaunch,
                  std::string* err) {
  const int K = d.ntracers;
  if (K < 1 || K > 65535) { *err = "ntracers must be in 1..65535"; return -1; }
  if (d.tracer_vec > 1) { *err = "tracer groups (tracer_vec > 1) are a layout of the FP32 form"; return -1; }
  if (d.hor < 0 || d.hor > 2 || d.ver < 0 || d.ver > 3 || d.lim < 0 || d.lim > 1) {
    *err = "unknown advection scheme";
    return -1;
  }
  if (!d.T || !d.vel || !d.w || !d.we || !d.workspace) { *err = "null device pointer"; return -1; }
  if (d.ab_order < 0 || d.ab_order > 2) { *err = "ab_order must be 0, 1 or 2"; return -1; }
  const WorkspaceLayout wl = workspace_layout<R>(m, K);
  if (d.workspace_bytes < wl.total) { *err = "workspace too small"; return -1; }
  if ((d.ver == FGB_VER_QR4C || d.ver == FGB_VER_PPM) && m.min_layers < 2) {
    *err = "QR4C/PPM need at least two layers in every column";
    return -1;
  }
  const bool fct = d.lim == FGB_LIM_FCT;
  const bool wsplit = fct && d.wi;
  if (wsplit) {
    if (const char* why = vert_impl_check<R>(m)) { *err = why; return -1; }
  }
  char* ws = static_cast<char*>(d.workspace);
  StepPtrs<R> a;
  a.T = static_cast<R*>(d.T);
  a.TA = d.TA ? static_cast<const R*>(d.TA) : a.T;
  a.TAout = static_cast<R*>(d.TAout);
  a.vel = static_cast<const R*>(d.vel);
  a.w = static_cast<const R*>(d.w);
  a.we = static_cast<const R*>(d.we);
  a.wi = wsplit ? static_cast<const R*>(d.wi) : nullptr;
  a.vf = reinterpret_cast<R*>(ws + wl.off[0]);
  a.adfh = reinterpret_cast<R*>(ws + wl.off[2]);
  a.lo = reinterpret_cast<R*>(ws + wl.off[3]);
  a.adfv = reinterpret_cast<R*>(ws + wl.off[4]);
  a.rpm = reinterpret_cast<R*>(ws + wl.off[5]);
  a.del = static_cast<R*>(d.del);
  a.sT = d.strideT;
  a.sTA = d.TA ? d.strideTA : d.strideT;
  a.sE = (long long)m.E * m.LZ;
  a.sN = (long long)m.N * m.LZ;
  a.sW = (long long)m.N * m.LW;
  a.dt = (R)d.dt;
  a.ph = (R)d.ph;
  a.pv = (R)d.pv;
  a.K = K;
  a.ab2 = d.ab_order == 2;
  a.ab_old = (R)(-(0.5 + d.ab_eps));
  a.ab_new = (R)(1.5 + d.ab_eps);
  auto pick_w = [](int want, int a, int b, int c, int def) {
    return (want == a || want == b || want == c) ? want : def;
  };
  const int ew = pick_w(d.cfg[0], 2, 4, 8, kEdgeWarps);
  const int nw_lo = pick_w(d.cfg[1], 1, 2, 4, kNodeWarps);
  const int nw_ratio = pick_w(d.cfg[2], 1, 2, 4, kNodeWarps);
  const int nw_upd = pick_w(d.cfg[3], 1, 2, 4, kNodeWarps);
  const int kc_lo = pick_kc(K, d.cfg[4]), kc_ratio = pick_kc(K, d.cfg[5]), kc_upd = pick_kc(K, d.cfg[6]);
  int launches = 0;
  if (mask & FGB_STAGE_VFLUX) {
    dim3 grid((m.E + kEdgeWarps - 1) / kEdgeWarps), block(kEdgeWarps * kWarp);
    k_vflux<R><<<grid, block, 0, s>>>(m, a.vel, a.vf);
    ++launches;
  }
  if (mask & FGB_STAGE_HFLUX) {
    if (d.hor == FGB_HOR_UPW1) launch_hflux<R, 0>(m, a, fct, ew, s);
    else if (d.hor == FGB_HOR_MUSCL) launch_hflux<R, 1>(m, a, fct, ew, s);
    else launch_hflux<R, 2>(m, a, fct, ew, s);
    ++launches;
  }
  if (fct) {
    if (mask & FGB_STAGE_LO) {
      if (kc_lo == 4) launch_lo_ver<R, 4>(m, a, d.ver, nw_lo, s);
      else if (kc_lo == 2) launch_lo_ver<R, 2>(m, a, d.ver, nw_lo, s);
      else launch_lo_ver<R, 1>(m, a, d.ver, nw_lo, s);
      ++launches;
      if (wsplit) {
        launch_vert_impl<R>(m, GeoSel<R>::get(m), a.lo, a.wi, K, 1, a.sN, a.dt, s);
        ++launches;
      }
    }
    if (mask & FGB_STAGE_RATIO) {
      if (kc_ratio == 4) launch_ratio<R, 4>(m, a, nw_ratio, s);
      else if (kc_ratio == 2) launch_ratio<R, 2>(m, a, nw_ratio, s);
      else launch_ratio<R, 1>(m, a, nw_ratio, s);
      ++launches;
    }
    if (mask & FGB_STAGE_UPDATE) {
      if (kc_upd == 4) launch_update<R, 4>(m, a, nw_upd, s);
      else if (kc_upd == 2) launch_update<R, 2>(m, a, nw_upd, s);
      else launch_update<R, 1>(m, a, nw_upd, s);
      ++launches;
    }
  } else if (mask & FGB_STAGE_UPDATE) {
    if (kc_upd == 4) launch_nofct_ver<R, 4>(m, a, d.ver, nw_upd, s);
    else if (kc_upd == 2) launch_nofct_ver<R, 2>(m, a, d.ver, nw_upd, s);
    else launch_nofct_ver<R, 1>(m, a, d.ver, nw_upd, s);
    ++launches;
  }
  *nlaunch = launches;
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    *err = std::string("kernel launch failed: ") + cudaGetErrorString(ce);
    return -1;
  }
  return 0;
}

}  // inline namespace
}  // namespace fgb
