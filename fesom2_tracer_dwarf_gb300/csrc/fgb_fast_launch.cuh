// Launch sequence of the FP32 form for one tracer-group width KV. Included by
// one translation unit per KV (compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "fesom_tracer_gb300.h"
#include "fgb_fast.cuh"

namespace fgb {
namespace fast {

template <typename F>
inline void allow_smem_f(F* kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int KV, int HOR>
void launch_hflux_f(const DMesh& m, const FastPtrs& a, bool fct, int ew, cudaStream_t s) {
  dim3 grid((m.E + ew - 1) / ew), block(ew * kW);
  if (fct) kf_hflux<HOR, true, KV><<<grid, block, 0, s>>>(m, a);
  else kf_hflux<HOR, false, KV><<<grid, block, 0, s>>>(m, a);
}

template <int KV, int VER>
void launch_lo_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const LoCols c = lo_cols(VER, a.we != a.w, a.TA != a.T);
  const size_t sm = nw * warp_bytes<KV>(c.scal, c.vec, m.LW);
  allow_smem_f(kf_lo<VER, KV>, sm);
  kf_lo<VER, KV><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}

template <int KV, int VER>
void launch_nofct_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const LoCols c = nofct_cols(VER);
  const size_t sm = nw * warp_bytes<KV>(c.scal, c.vec, m.LW);
  allow_smem_f(kf_nofct<VER, KV>, sm);
  kf_nofct<VER, KV><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}

template <int KV>
int launch_fast(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  int launches = 0;
  if (L.mask & FGB_STAGE_VFLUX) {
    kf_vflux<<<(m.E + 7) / 8, 256, 0, s>>>(m, a.vel, a.vf);
    ++launches;
  }
  if (L.mask & FGB_STAGE_HFLUX) {
    if (L.hor == FGB_HOR_UPW1) launch_hflux_f<KV, 0>(m, a, L.fct, L.edge_warps, s);
    else if (L.hor == FGB_HOR_MUSCL) launch_hflux_f<KV, 1>(m, a, L.fct, L.edge_warps, s);
    else launch_hflux_f<KV, 2>(m, a, L.fct, L.edge_warps, s);
    ++launches;
  }
  if (L.fct) {
    if (L.mask & FGB_STAGE_LO) {
      switch (L.ver) {
        case FGB_VER_QR4C: launch_lo_f<KV, 1>(m, a, L.nw_lo, s); break;
        case FGB_VER_CDIFF: launch_lo_f<KV, 2>(m, a, L.nw_lo, s); break;
        case FGB_VER_PPM: launch_lo_f<KV, 3>(m, a, L.nw_lo, s); break;
        default: launch_lo_f<KV, 0>(m, a, L.nw_lo, s); break;
      }
      ++launches;
    }
    if (L.mask & FGB_STAGE_RATIO) {
      const size_t sm = L.nw_ratio * warp_bytes<KV>(0, kRatioVec, m.LW);
      allow_smem_f(kf_ratio<KV>, sm);
      kf_ratio<KV><<<(m.N + L.nw_ratio - 1) / L.nw_ratio, L.nw_ratio * kW, sm, s>>>(m, a);
      ++launches;
    }
    if (L.mask & FGB_STAGE_UPDATE) {
      const size_t sm = L.nw_upd * warp_bytes<KV>(0, kUpdVec, m.LW);
      allow_smem_f(kf_update<KV>, sm);
      kf_update<KV><<<(m.N + L.nw_upd - 1) / L.nw_upd, L.nw_upd * kW, sm, s>>>(m, a);
      ++launches;
    }
  } else if (L.mask & FGB_STAGE_UPDATE) {
    switch (L.ver) {
      case FGB_VER_QR4C: launch_nofct_f<KV, 1>(m, a, L.nw_upd, s); break;
      case FGB_VER_CDIFF: launch_nofct_f<KV, 2>(m, a, L.nw_upd, s); break;
      case FGB_VER_PPM: launch_nofct_f<KV, 3>(m, a, L.nw_upd, s); break;
      default: launch_nofct_f<KV, 0>(m, a, L.nw_upd, s); break;
    }
    ++launches;
  }
  return launches;
}

}  // namespace fast
}  // namespace fgb
