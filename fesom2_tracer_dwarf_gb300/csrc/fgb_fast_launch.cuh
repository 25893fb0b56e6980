// Launch sequence of the FP32 form for one tracer-group width KV. Included by
// one translation unit per KV (compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "fesom_tracer_gb300.h"
#include "fgb_fast.cuh"
#include "fgb_fast_lo64.cuh"
#include "fgb_fast_tile.cuh"

namespace fgb {
namespace fast {

template <typename F>
inline void allow_smem_f(F* kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int KV, int HOR, int NS>
void launch_hflux_f(const DMesh& m, const FastPtrs& a, bool fct, int ew, cudaStream_t s) {
  const int per_block = ew * kW;  // edges per block: 32 per warp
  dim3 grid((m.E + per_block - 1) / per_block), block(ew * kW);
  const size_t sm = (size_t)ew * kW * sizeof(EdgeRec);
  if (fct) kf_hflux<HOR, true, KV, NS><<<grid, block, sm, s>>>(m, a);
  else kf_hflux<HOR, false, KV, NS><<<grid, block, sm, s>>>(m, a);
}

template <int KV, int HOR, bool FCT>
void launch_hflux_tile(const DMesh& m, const FastPtrs& a, cudaStream_t s) {
  const size_t sm = tile_smem_bytes(KV, FCT && a.TA != a.T, m.tile_max_nodes);
  allow_smem_f(kf_hflux_tile<HOR, FCT, KV>, sm);
  kf_hflux_tile<HOR, FCT, KV><<<m.ntiles, kTileThreads, sm, s>>>(m, a);
}

template <int KV, int HOR>
void launch_hflux_ns(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  if (L.hflux_tile && m.ntiles > 0) {
    if (L.fct) launch_hflux_tile<KV, HOR, true>(m, a, s);
    else launch_hflux_tile<KV, HOR, false>(m, a, s);
  } else if (L.ns_h == 1) {
    launch_hflux_f<KV, HOR, 1>(m, a, L.fct, L.edge_warps, s);
  } else {
    launch_hflux_f<KV, HOR, 2>(m, a, L.fct, L.edge_warps, s);
  }
}

template <int KV, int VER, int NS, bool WSPLIT, bool COMP>
void launch_lo_fc(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const LoCols c = lo_cols(VER, a.we != a.w, a.TA != a.T);
  const size_t sm = nw * warp_bytes<KV>(c.scal, c.vec, m.LW);
  allow_smem_f(kf_lo<VER, KV, NS, WSPLIT, COMP>, sm);
  kf_lo<VER, KV, NS, WSPLIT, COMP><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}
template <int KV, int VER, int NS>
void launch_lo_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  if (a.wi) {
    if (a.comp & 1) launch_lo_fc<KV, VER, NS, true, true>(m, a, nw, s);
    else launch_lo_fc<KV, VER, NS, true, false>(m, a, nw, s);
  } else {
    if (a.comp & 1) launch_lo_fc<KV, VER, NS, false, true>(m, a, nw, s);
    else launch_lo_fc<KV, VER, NS, false, false>(m, a, nw, s);
  }
}

template <int KV, int VER, int NS>
void launch_nofct_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const LoCols c = nofct_cols(VER);
  const size_t sm = nw * warp_bytes<KV>(c.scal, c.vec, m.LW);
  allow_smem_f(kf_nofct<VER, KV, NS>, sm);
  kf_nofct<VER, KV, NS><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}

template <int KV, int NS, bool COMP>
void launch_ratio_fc(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const size_t sm = nw * warp_bytes<KV>(0, kRatioVec, m.LW);
  allow_smem_f(kf_ratio<KV, NS, COMP>, sm);
  kf_ratio<KV, NS, COMP><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}
template <int KV, int NS>
void launch_ratio_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  if (a.comp & 4) launch_ratio_fc<KV, NS, true>(m, a, nw, s);
  else launch_ratio_fc<KV, NS, false>(m, a, nw, s);
}

template <int KV, int NS, bool DEL, bool COMP, bool RES>
void launch_update_fc(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const size_t sm = nw * warp_bytes<KV>(0, kUpdVec, m.LW);
  allow_smem_f(kf_update<KV, NS, DEL, COMP, RES>, sm);
  kf_update<KV, NS, DEL, COMP, RES><<<(m.N + nw - 1) / nw, nw * kW, sm, s>>>(m, a);
}
template <int KV, int NS>
void launch_update_f(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  if (a.del) {  // the reference C interface: a persistent del_ttf, no residual
    if (a.comp & 2) launch_update_fc<KV, NS, true, true, false>(m, a, nw, s);
    else launch_update_fc<KV, NS, true, false, false>(m, a, nw, s);
  } else if (a.Tlo) {
    if (a.comp & 2) launch_update_fc<KV, NS, false, true, true>(m, a, nw, s);
    else launch_update_fc<KV, NS, false, false, true>(m, a, nw, s);
  } else {
    if (a.comp & 2) launch_update_fc<KV, NS, false, true, false>(m, a, nw, s);
    else launch_update_fc<KV, NS, false, false, false>(m, a, nw, s);
  }
}

template <int KV, bool LEAN>
void launch_ratio64(const DMesh& m, const FastPtrs& a, int nw, cudaStream_t s) {
  const unsigned grid = (m.N + nw - 1) / nw;
  const size_t sm = nw * ratio64_warp_bytes(KV);
  if (a.comp & 4) kf_ratio64<KV, LEAN, true><<<grid, nw * kW, sm, s>>>(m, a);
  else kf_ratio64<KV, LEAN, false><<<grid, nw * kW, sm, s>>>(m, a);
}

template <int KV, int VER, bool TASEP, bool WESEP, bool COMP>
void launch_lo64c(const DMesh& m, const FastPtrs& a, cudaStream_t s) {
  const size_t sm = kLo64Warps * lo64_warp_bytes(KV, VER, TASEP);
  allow_smem_f(kf_lo64<VER, KV, TASEP, WESEP, COMP>, sm);
  kf_lo64<VER, KV, TASEP, WESEP, COMP><<<(m.N + kLo64Warps - 1) / kLo64Warps, kLo64Warps * kW, sm, s>>>(m, a);
}
template <int KV, int VER, bool TASEP, bool WESEP>
void launch_lo64(const DMesh& m, const FastPtrs& a, cudaStream_t s) {
  if (a.comp & 1) launch_lo64c<KV, VER, TASEP, WESEP, true>(m, a, s);
  else launch_lo64c<KV, VER, TASEP, WESEP, false>(m, a, s);
}

template <int KV, int VER>
void launch_lo_ns(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  if (L.ns_lo == 3) {  // whole column per warp (at most 64 layers, no w_split)
    const bool tasep = a.TA != a.T, wesep = a.we != a.w;
    if (tasep) {
      if (wesep) launch_lo64<KV, VER, true, true>(m, a, s);
      else launch_lo64<KV, VER, true, false>(m, a, s);
    } else {
      if (wesep) launch_lo64<KV, VER, false, true>(m, a, s);
      else launch_lo64<KV, VER, false, false>(m, a, s);
    }
  } else if (L.ns_lo == 1) {
    launch_lo_f<KV, VER, 1>(m, a, L.nw_lo, s);
  } else {
    launch_lo_f<KV, VER, 2>(m, a, L.nw_lo, s);
  }
}

template <int KV, int VER>
void launch_nofct_ns(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  if (L.ns_upd == 1) launch_nofct_f<KV, VER, 1>(m, a, L.nw_upd, s);
  else launch_nofct_f<KV, VER, 2>(m, a, L.nw_upd, s);
}

template <int KV>
int launch_fast(const DMesh& m, const FastPtrs& a, const LaunchArgs& L, cudaStream_t s) {
  int launches = 0;
  if (L.mask & FGB_STAGE_VFLUX) {
    kf_vflux<<<(m.E + 8 * kW - 1) / (8 * kW), 8 * kW, 0, s>>>(m, a.vel, a.vf);
    ++launches;
  }
  if (L.mask & FGB_STAGE_HFLUX) {
    if (L.hor == FGB_HOR_UPW1) launch_hflux_ns<KV, 0>(m, a, L, s);
    else if (L.hor == FGB_HOR_MUSCL) launch_hflux_ns<KV, 1>(m, a, L, s);
    else launch_hflux_ns<KV, 2>(m, a, L, s);
    ++launches;
  }
  if (L.fct) {
    if (L.mask & FGB_STAGE_LO) {
      FastPtrs al = a;
      al.wsplit_fused = a.wi && L.ns_lo == 2 && m.LZ <= 2 * kW && !L.vimpl_thomas;
      switch (L.ver) {
        case FGB_VER_QR4C: launch_lo_ns<KV, 1>(m, al, L, s); break;
        case FGB_VER_CDIFF: launch_lo_ns<KV, 2>(m, al, L, s); break;
        case FGB_VER_PPM: launch_lo_ns<KV, 3>(m, al, L, s); break;
        default: launch_lo_ns<KV, 0>(m, al, L, s); break;
      }
      ++launches;
      if (a.wi && !(L.ns_lo == 2 && m.LZ <= 2 * kW && !L.vimpl_thomas)) {
        // w_split: the implicit vertical step on the LO solution (unless the
        // LO kernel solved it in the same pass)
        if (m.LZ <= 2 * kW && !L.vimpl_thomas) {
          kf_vert_pcr<KV><<<(m.N + 7) / 8, 8 * kW, 0, s>>>(m, a);
        } else {
          const size_t sm = vimpl_block_bytes(m.LZ, KV);
          allow_smem_f(kf_vert_impl<KV>, sm);
          const int per_block = kVimplWarpsF * VimplShape<KV>::NPW;
          kf_vert_impl<KV><<<(m.N + per_block - 1) / per_block, kVimplWarpsF * kW, sm, s>>>(m, a);
        }
        ++launches;
      }
    }
    if (L.mask & FGB_STAGE_RATIO) {
      if (m.LZ <= 2 * kW && (L.ns_ratio == 0 || L.ns_ratio >= 3)) {
        // whole column per warp, no shared memory
        if (L.ns_ratio == 4) launch_ratio64<KV, true>(m, a, L.nw_ratio, s);
        else launch_ratio64<KV, false>(m, a, L.nw_ratio, s);
      } else if (L.ns_ratio == 1) {
        launch_ratio_f<KV, 1>(m, a, L.nw_ratio, s);
      } else {
        launch_ratio_f<KV, 2>(m, a, L.nw_ratio, s);
      }
      ++launches;
    }
    if (L.mask & FGB_STAGE_UPDATE) {
      if (L.ns_upd == 2) launch_update_f<KV, 2>(m, a, L.nw_upd, s);
      else launch_update_f<KV, 1>(m, a, L.nw_upd, s);
      ++launches;
    }
  } else if (L.mask & FGB_STAGE_UPDATE) {
    switch (L.ver) {
      case FGB_VER_QR4C: launch_nofct_ns<KV, 1>(m, a, L, s); break;
      case FGB_VER_CDIFF: launch_nofct_ns<KV, 2>(m, a, L, s); break;
      case FGB_VER_PPM: launch_nofct_ns<KV, 3>(m, a, L, s); break;
      default: launch_nofct_ns<KV, 0>(m, a, L, s); break;
    }
    ++launches;
  }
  return launches;
}

}  // namespace fast
}  // namespace fgb
