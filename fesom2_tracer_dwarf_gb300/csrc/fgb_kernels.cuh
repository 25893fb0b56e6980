// Device kernels of the FESOM2 tracer-advection step (do_oce_adv_tra,
// lib/oce_adv_tra_driver.F90:23-294) for GB300 (sm_103a).
//
// Layout: level index fastest, columns padded to LZ layers / LW interfaces.
// Node-column kernels run one warp per node with the column staged in shared
// memory; edge kernels run one warp per edge, lanes over layers (coalesced
// 256-byte rows). The reference's edge scatters (atomics / OpenMP locks) are
// replaced by gathers over each node's incident edges in ascending edge order,
// which reproduces the reference's per-node summation order exactly.
//
// R is the storage and arithmetic type. Every expression keeps the
// reference's evaluation order; the FP64 translation unit is compiled without
// fused multiply-add so the device result equals the CPU restatement bit for bit.
#pragma once
#include <cstdint>

#include "fgb_device.hpp"

namespace fgb {

constexpr int kWarp = 32;

template <typename R>
struct GeoSel;
template <>
struct GeoSel<double> {
  __device__ static const GeoPtrs<double>& get(const DMesh& m) { return m.g64; }
};
template <>
struct GeoSel<float> {
  __device__ static const GeoPtrs<float>& get(const DMesh& m) { return m.g32; }
};

template <typename R>
__device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <typename R>
__device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <typename R>
__device__ __forceinline__ R rabs(R a) { return fabs(a); }

// Layer membership of the horizontal-flux segments A-E of
// lib/oce_adv_tra_hor.F90:171-252 (1-based layer z): which elements' volume
// fluxes contribute at z. Returns 0 (inactive), 1, 2 or 3 (both).
__device__ __forceinline__ int edge_seg(int z, int nu1, int nl1, int nu2, int nl2) {
  const int nl12 = min(nl1, nl2), nu12 = max(nu1, nu2);
  const bool inA = z >= nu1 && z <= nu12 - 1;
  const bool inB = nu2 > 0 && z >= nu2 && z <= nu12 - 1;
  const bool inC = z >= nu12 && z <= nl12;
  const bool inD = z >= nl12 + 1 && z <= nl1;
  const bool inE = z >= nl12 + 1 && z <= nl2;
  return ((inA || inC || inD) ? 1 : 0) | ((inB || inC || inE) ? 2 : 0);
}

// ---------------------------------------------------------------------------
// Volume flux through each edge segment (shared by all tracers of a step):
// vflux of lib/oce_adv_tra_hor.F90:174,194,215-216.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_vflux(DMesh m, const R* __restrict__ vel, R* __restrict__ vf) {
  const int lane = threadIdx.x & (kWarp - 1);
  const int e = blockIdx.x * (blockDim.x / kWarp) + (threadIdx.x / kWarp);
  if (e >= m.E) return;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const int nu1 = m.edge_lev[4 * e], nl1 = m.edge_lev[4 * e + 1];
  const int nu2 = m.edge_lev[4 * e + 2], nl2 = m.edge_lev[4 * e + 3];
  const int el1 = m.edge_tri[2 * e], el2 = m.edge_tri[2 * e + 1];
  const R dX1 = g.edge_cross[4 * e], dY1 = g.edge_cross[4 * e + 1];
  const R dX2 = g.edge_cross[4 * e + 2], dY2 = g.edge_cross[4 * e + 3];
  const size_t LZ = m.LZ;
  for (int k = lane; k < m.LZ; k += kWarp) {
    R v = R(0);
    if (k < m.nz) {
      const int seg = edge_seg(k + 1, nu1, nl1, nu2, nl2);
      R v1 = R(0), v2 = R(0);
      if (seg & 1) {
        const R u = vel[2 * (el1 * LZ + k)], vv = vel[2 * (el1 * LZ + k) + 1];
        v1 = (-(vv * dX1) + u * dY1) * g.helem[el1 * LZ + k];
      }
      if (seg & 2) {
        const R u = vel[2 * (el2 * LZ + k)], vv = vel[2 * (el2 * LZ + k) + 1];
        v2 = (vv * dX2 - u * dY2) * g.helem[el2 * LZ + k];
      }
      v = (seg == 3) ? v1 + v2 : (seg == 1 ? v1 : v2);
    }
    vf[e * LZ + k] = v;
  }
}

// Elemental gradient of T at layer k (tr_xy, coefficients gradient_sca of
// lib/oce_mesh.F90:2512-2534).
template <typename R>
__device__ __forceinline__ void elem_grad(const DMesh& m, const GeoPtrs<R>& g, const R* __restrict__ T, int el,
                                          size_t k, R& gx, R& gy) {
  const size_t LZ = m.LZ;
  const int a = m.elem_nodes[3 * el], b = m.elem_nodes[3 * el + 1], c = m.elem_nodes[3 * el + 2];
  const R ta = T[a * LZ + k], tb = T[b * LZ + k], tc = T[c * LZ + k];
  const R* gs = g.grad_sca + 6 * (size_t)el;
  gx = gs[0] * ta + gs[1] * tb + gs[2] * tc;
  gy = gs[3] * ta + gs[4] * tb + gs[5] * tc;
}

// Area-weighted mean of the element gradients around a node at layer z
// (lib/oce_muscl_adv.F90:393-410).
template <typename R>
__device__ __forceinline__ void node_mean_grad(const DMesh& m, const GeoPtrs<R>& g, const R* __restrict__ T,
                                               int n, int k, R& gx, R& gy) {
  R tvol = R(0), tx = R(0), ty = R(0);
  const int z = k + 1;
  for (int j = m.nie_ptr[n]; j < m.nie_ptr[n + 1]; ++j) {
    const int el = m.nie_idx[j];
    if (m.elem_nlev[el] - 1 < z) continue;
    R ex, ey;
    elem_grad(m, g, T, el, k, ex, ey);
    const R ar = g.elem_area[el];
    tvol = tvol + ar;
    tx = tx + ex * ar;
    ty = ty + ey * ar;
  }
  gx = tx / tvol;
  gy = ty / tvol;
}

// ---------------------------------------------------------------------------
// Horizontal edge fluxes. FCT: writes the low-order flux (adv_tra_hor_upw1 on
// T) and the antidiffusive flux HO(T_AB) - LO; otherwise the HO flux.
// HOR: 0 UPW1, 1 MUSCL (with the nboundary_lay mask c_lo), 2 MFCT.
// ---------------------------------------------------------------------------
template <typename R, int HOR, bool FCT>
__global__ void __launch_bounds__(256) k_hflux(DMesh m, StepPtrs<R> a) {
  const int lane = threadIdx.x & (kWarp - 1);
  const int e = blockIdx.x * (blockDim.x / kWarp) + (threadIdx.x / kWarp);
  if (e >= m.E) return;
  const int t = blockIdx.y;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const R* __restrict__ T = a.T + t * a.sT;
  const R* __restrict__ TA = a.TA + t * a.sTA;
  R* __restrict__ flo = FCT ? a.flo + t * a.sE : nullptr;
  R* __restrict__ adf = a.adfh + t * a.sE;
  const size_t LZ = m.LZ;
  const int n1 = m.edge_nodes[2 * e], n2 = m.edge_nodes[2 * e + 1];
  const int nu1 = m.edge_lev[4 * e], nl1 = m.edge_lev[4 * e + 1];
  const int nu2 = m.edge_lev[4 * e + 2], nl2 = m.edge_lev[4 * e + 3];
  int up = -1, dn = -1, gm0 = -1, gm1 = -1, nb1 = 0, nb2 = 0;
  R ex = R(0), ey = R(0);
  if (HOR != 0) {
    up = m.edge_updn[2 * e];
    dn = m.edge_updn[2 * e + 1];
    gm0 = m.edge_gm[2 * e];
    gm1 = m.edge_gm[2 * e + 1];
    ex = g.edge_dxa[2 * e];
    ey = g.edge_dxa[2 * e + 1];
    nb1 = m.nbl[n1];
    nb2 = m.nbl[n2];
  }
  const R ph = a.ph;
  for (int k = lane; k < m.nz; k += kWarp) {
    const int z = k + 1;
    const int seg = edge_seg(z, nu1, nl1, nu2, nl2);
    if (seg == 0) {
      if (FCT) flo[e * LZ + k] = R(0);
      adf[e * LZ + k] = R(0);
      continue;
    }
    const R v = a.vf[e * LZ + k];
    const R vp = v + rabs(v), vm = v - rabs(v);
    R lo = R(0);
    if (FCT) {
      lo = -(R(0.5) * (T[n1 * LZ + k] * vp + T[n2 * LZ + k] * vm));
      flo[e * LZ + k] = lo;
    }
    const R ta1 = TA[n1 * LZ + k], ta2 = TA[n2 * LZ + k];
    R ho;
    if (HOR == 0) {
      ho = -(R(0.5) * (ta1 * vp + ta2 * vm));
    } else {
      R g1, g2, g3, g4;
      if (gm0 >= 0 && z >= gm0 && z <= gm1 - 1) {
        elem_grad(m, g, TA, up, k, g1, g3);
        elem_grad(m, g, TA, dn, k, g2, g4);
      } else {
        node_mean_grad(m, g, TA, n1, k, g1, g3);
        node_mean_grad(m, g, TA, n2, k, g2, g4);
      }
      R Tm2, Tm1;
      if (HOR == 1) {
        const R c1 = (nb1 - z >= 0) ? R(1) : R(0);
        const R c2 = (nb2 - z >= 0) ? R(1) : R(0);
        Tm2 = ta2 - ((R(2) * (ta2 - ta1) + ex * g2 + ey * g4) / R(6)) * c2;
        Tm1 = ta1 + ((R(2) * (ta2 - ta1) + ex * g1 + ey * g3) / R(6)) * c1;
      } else {
        Tm2 = ta2 - (R(2) * (ta2 - ta1) + ex * g2 + ey * g4) / R(6);
        Tm1 = ta1 + (R(2) * (ta2 - ta1) + ex * g1 + ey * g3) / R(6);
      }
      const R cHO = vp * Tm1 + vm * Tm2;
      ho = -((R(0.5) * (R(1) - ph)) * cHO) - ((v * ph) * R(0.5)) * (Tm1 + Tm2);
    }
    adf[e * LZ + k] = FCT ? ho - lo : ho;
  }
}

// ---------------------------------------------------------------------------
// Vertical fluxes of one column at interface z (1-based), given the staged
// column. flux_old is the value the reference subtracts ("X - flux").
// VER: 0 UPW1, 1 QR4C, 2 CDIFF, 3 PPM (lib/oce_adv_tra_ver.F90:248-712).
// Staged arrays are 0-based by layer/interface.
// ---------------------------------------------------------------------------
template <typename R>
struct Col {
  const R* T;     // tracer at layers
  const R* W;     // vertical velocity at interfaces
  const R* area;  // at interfaces
  const R* hn;    // hnode at layers (PPM)
  const R* hnn;   // hnode_new at layers (PPM)
  const R* Z;     // Z_3d_n at layers (QR4C)
  const R* zb;    // zbar_3d_n at interfaces (QR4C)
  const R* tv;    // PPM edge values at interfaces
};

template <typename R>
__device__ __forceinline__ R ver_upw1(const Col<R>& c, int z, int nzmin, int nzmax, R fold) {
  if (z == nzmin) return -((c.W[z - 1] * c.T[z - 1]) * c.area[z - 1]) - fold;
  if (z == nzmax) return R(0) - fold;
  const R W = c.W[z - 1];
  return -((R(0.5) * (c.T[z - 1] * (W + rabs(W)) + c.T[z - 2] * (W - rabs(W)))) * c.area[z - 1]) - fold;
}

template <typename R>
__device__ __forceinline__ R ver_qr4c(const Col<R>& c, int z, int nzmin, int nzmax, R num_ord, R fold) {
  const R W = c.W[z - 1];
  if (z == nzmin) return -((c.T[z - 1] * W) * c.area[z - 1]) - fold;
  if (z == nzmax) return R(0) - fold;
  if (z == nzmin + 1 || z == nzmax - 1) {
    const R x = -(((R(0.5) * (c.T[z - 2] + c.T[z - 1])) * W) * c.area[z - 1]);
    R f = x - fold;
    if (nzmin + 1 == nzmax - 1) f = x - f;  // written twice (lib/oce_adv_tra_ver.F90:405-411)
    return f;
  }
  const R T0 = c.T[z - 1], Tm1 = c.T[z - 2], Tm2 = c.T[z - 3], Tp1 = c.T[z];
  const R Z0 = c.Z[z - 1], Zm1 = c.Z[z - 2], Zm2 = c.Z[z - 3], Zp1 = c.Z[z];
  const R qc = (Tm1 - T0) / (Zm1 - Z0);
  const R qu = (T0 - Tp1) / (Z0 - Zp1);
  const R qd = (Tm2 - Tm1) / (Zm2 - Zm1);
  const R zb = c.zb[z - 1];
  const R tm1 = T0 + ((R(2) * qc + qu) * (zb - Z0)) / R(3);
  const R tm2 = Tm1 + ((R(2) * qc + qd) * (zb - Zm1)) / R(3);
  const R tm = (W + rabs(W)) * tm1 + (W - rabs(W)) * tm2;
  return (-((R(0.5) * (R(1) - num_ord)) * tm) - (num_ord * (R(0.5) * (tm1 + tm2))) * W) * c.area[z - 1] - fold;
}

template <typename R>
__device__ __forceinline__ R ver_cdiff(const Col<R>& c, int z, int nzmin, int nlev, R fold) {
  const int nzmax = nlev - 1;  // lib/oce_adv_tra_ver.F90:689
  if (z == nzmin) return -((c.W[z - 1] * c.T[z - 1]) * c.area[z - 1]) - fold;
  if (z <= nzmax) {
    const R tv = R(0.5) * (c.T[z - 2] + c.T[z - 1]);
    return -((tv * c.W[z - 1]) * c.area[z - 1]) - fold;
  }
  return fold;  // the bottom interface is left untouched
}

// PPM edge value tv(z) of lib/oce_adv_tra_ver.F90:510-594; the later
// assignment wins where the special cases coincide.
template <typename R>
__device__ __forceinline__ R ppm_tv(const Col<R>& c, int z, int nzmin, int nzmax) {
  const R* T = c.T;
  if (z >= nzmin + 2 && z <= nzmax - 2) {
    const int nz = z - 1;  // layer whose upper neighbour interface is z
    const R dzjm1 = c.hnn[nz - 2], dzj = c.hnn[nz - 1], dzjp1 = c.hnn[nz], dzjp2 = c.hnn[nz + 1];
    const R Tm = T[nz - 2], T0 = T[nz - 1], Tp = T[nz], Tpp = T[nz + 1];
    R deltaj = (dzj / (dzjm1 + dzj + dzjp1)) *
               (((R(2) * dzjm1 + dzj) / (dzjp1 + dzj)) * (Tp - T0) + ((dzj + R(2) * dzjp1) / (dzjm1 + dzj)) * (T0 - Tm));
    R deltajp1 = (dzjp1 / (dzj + dzjp1 + dzjp2)) *
                 (((R(2) * dzj + dzjp1) / (dzjp2 + dzjp1)) * (Tpp - Tp) + ((dzjp1 + R(2) * dzjp2) / (dzj + dzjp1)) * (Tp - T0));
    if ((Tp - T0) * (T0 - Tm) > R(0))
      deltaj = rmin(rmin(rabs(deltaj), R(2) * rabs(Tp - T0)), R(2) * rabs(T0 - Tm)) * copysign(R(1), deltaj);
    else
      deltaj = R(0);
    if ((Tpp - Tp) * (Tp - T0) > R(0))
      deltajp1 = rmin(rmin(rabs(deltajp1), R(2) * rabs(Tpp - Tp)), R(2) * rabs(Tp - T0)) * copysign(R(1), deltajp1);
    else
      deltajp1 = R(0);
    const R inner1 = (((R(2) * dzjp1) * dzj) / (dzj + dzjp1)) *
                     ((dzjm1 + dzj) / (R(2) * dzj + dzjp1) - (dzjp2 + dzjp1) / (R(2) * dzjp1 + dzj)) * (Tp - T0);
    const R inner2 = ((dzj * (dzjm1 + dzj)) / (R(2) * dzj + dzjp1)) * deltajp1;
    const R inner3 = ((dzjp1 * (dzjp1 + dzjp2)) / (dzj + R(2) * dzjp1)) * deltaj;
    return (T0 + (dzj / (dzj + dzjp1)) * (Tp - T0)) + (R(1) / (dzjm1 + dzj + dzjp1 + dzjp2)) * (inner1 - inner2 + inner3);
  }
  if (z == nzmax) return T[nzmax - 2];
  if (z == nzmax - 1) {
    const R s = copysign(R(1), c.W[nzmax - 2]);
    return -(T[nzmax - 3] * rmin(s, R(0))) + T[nzmax - 2] * rmax(s, R(0));
  }
  if (z == nzmin + 1) return R(0.5) * (T[nzmin - 1] + T[nzmin]);
  return T[nzmin - 1];
}

// PPM flux contribution of layer nz to its interface (upper: W(nz) > 0 side,
// lower: W(nz+1) < 0 side), lib/oce_adv_tra_ver.F90:598-632.
template <typename R>
__device__ __forceinline__ R ppm_layer(const Col<R>& c, int nz, bool upper, R dt) {
  R aL = c.tv[nz - 1], aR = c.tv[nz];
  const R T0 = c.T[nz - 1];
  if ((aR - T0) * (T0 - aL) <= R(0)) {
    aL = T0;
    aR = T0;
  }
  if ((aR - aL) * (T0 - R(0.5) * (aL + aR)) > ((aR - aL) * (aR - aL)) / R(6)) aL = R(3) * T0 - R(2) * aR;
  if ((aR - aL) * (T0 - R(0.5) * (aR + aL)) < -(((aR - aL) * (aR - aL)) / R(6))) aR = R(3) * T0 - R(2) * aL;
  const R dzj = c.hn[nz - 1];
  const R aj = R(6) * (T0 - R(0.5) * (aL + aR));
  if (upper) {
    const R W = c.W[nz - 1];
    const R x = rmin((W * dt) / dzj, R(1));
    R tv = -aL - (R(0.5) * x) * ((aR - aL) + (R(1) - (R(2) / R(3)) * x) * aj);
    return (tv * c.area[nz - 1]) * W;
  }
  const R W = c.W[nz];
  const R x = rmin(-((W * dt) / dzj), R(1));
  R tv = -aR + (R(0.5) * x) * ((aR - aL) - (R(1) - (R(2) / R(3)) * x) * aj);
  return (tv * c.area[nz]) * W;
}

template <typename R>
__device__ __forceinline__ R ver_ppm(const Col<R>& c, int z, int nzmin, int nzmax, R dt, R fold) {
  R tvert = R(0);
  if (z == nzmin) {
    tvert = -((c.tv[nzmin - 1] * c.W[nzmin - 1]) * c.area[nzmin - 1]);
  } else if (z < nzmax) {
    const R W = c.W[z - 1];
    if (W > R(0)) tvert = ppm_layer(c, z, true, dt);
    else if (W < R(0)) tvert = ppm_layer(c, z - 1, false, dt);
  }
  return tvert - fold;
}

template <typename R, int VER>
__device__ __forceinline__ R ver_flux(const Col<R>& c, int z, int nzmin, int nzmax, R num_ord, R dt, R fold) {
  if (VER == 1) return ver_qr4c(c, z, nzmin, nzmax, num_ord, fold);
  if (VER == 2) return ver_cdiff(c, z, nzmin, nzmax, fold);
  if (VER == 3) return ver_ppm(c, z, nzmin, nzmax, dt, fold);
  return ver_upw1(c, z, nzmin, nzmax, fold);
}

// Shared-memory slices of one warp's column.
template <typename R>
struct ColSmem {
  R* s;
  int LW;
  __device__ R* slice(int i) const { return s + (size_t)i * LW; }
};

template <typename R>
__device__ __forceinline__ void stage(R* dst, const R* __restrict__ src, int n, int lane) {
  for (int k = lane; k < n; k += kWarp) dst[k] = src[k];
}

// Vertical HO flux of the column into out[iz] (interfaces), PPM edge values
// computed first when needed. fold[iz] holds the value subtracted.
template <typename R, int VER>
__device__ __forceinline__ void column_ver_flux(Col<R>& c, R* tvbuf, const R* fold, R* out, int nl, int nzmin,
                                                int nzmax, R num_ord, R dt, int lane) {
  if (VER == 3) {
    for (int iz = lane; iz < nl; iz += kWarp) {
      const int z = iz + 1;
      tvbuf[iz] = (z >= nzmin && z <= nzmax) ? ppm_tv(c, z, nzmin, nzmax) : R(0);
    }
    __syncwarp();
    c.tv = tvbuf;
  }
  for (int iz = lane; iz < nl; iz += kWarp) {
    const int z = iz + 1;
    const R f0 = fold ? fold[iz] : R(0);
    out[iz] = (z >= nzmin && z <= nzmax) ? ver_flux<R, VER>(c, z, nzmin, nzmax, num_ord, dt, f0) : f0;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// FCT stage 1 (node columns): low-order solution fct_LO
// (lib/oce_adv_tra_driver.F90:91-235) and the vertical antidiffusive flux
// HO(T_AB, w) - LO(T, w_e).
// ---------------------------------------------------------------------------
template <typename R, int VER>
__global__ void k_fct_lo(DMesh m, StepPtrs<R> a) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int n = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (n >= m.N) return;
  const int t = blockIdx.y;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  ColSmem<R> sm{reinterpret_cast<R*>(smem_raw) + (size_t)wib * 10 * LW, (int)LW};
  R *sT = sm.slice(0), *sTA = sm.slice(1), *sW = sm.slice(2), *sWE = sm.slice(3), *sA = sm.slice(4);
  R *sHn = sm.slice(5), *sHnn = sm.slice(6), *sFlo = sm.slice(7), *sX = sm.slice(8), *sZ = sm.slice(9);
  const R* __restrict__ T = a.T + t * a.sT + n * LZ;
  const R* __restrict__ TA = a.TA + t * a.sTA + n * LZ;
  stage(sT, T, nz, lane);
  stage(sTA, TA, nz, lane);
  stage(sW, a.w + n * LW, nl, lane);
  stage(sWE, a.we + n * LW, nl, lane);
  stage(sA, g.area + n * LW, nl, lane);
  if (VER == 3) {
    stage(sHn, g.hnode + n * LZ, nz, lane);
    stage(sHnn, g.hnode_new + n * LZ, nz, lane);
  }
  if (VER == 1) {
    stage(sZ, g.Z3 + n * LZ, nz, lane);
    stage(sX, g.zbar3 + n * LW, nl, lane);
  }
  __syncwarp();
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  // LO vertical flux: adv_tra_ver_upw1(we, ttf) with init zero.
  Col<R> clo{sT, sWE, sA, sHn, sHnn, sZ, sX, nullptr};
  column_ver_flux<R, 0>(clo, nullptr, nullptr, sFlo, nl, nzmin, nzmax, R(1), a.dt, lane);
  // LO solution (lib/oce_adv_tra_driver.F90:202-209)
  R* __restrict__ lo = a.lo + t * a.sN + n * LZ;
  const R* __restrict__ flo = a.flo + t * a.sE;
  const R dt = a.dt;
  for (int k = lane; k < nz; k += kWarp) {
    const int z = k + 1;
    R acc = R(0);
    for (int j = m.ne_ptr[n]; j < m.ne_ptr[n + 1]; ++j) {
      if (z < m.ne_lo[j] || z > m.ne_hi[j]) continue;
      const int code = m.ne_code[j];
      const R f = flo[(size_t)(code >> 1) * LZ + k];
      acc = (code & 1) ? acc - f : acc + f;
    }
    R v = acc;
    if (z >= nzmin && z <= nzmax - 1)
      v = (sT[k] * g.hnode[n * LZ + k] + ((acc + (sFlo[k] - sFlo[k + 1])) * dt) / g.areasvol[n * LZ + k]) /
          g.hnode_new[n * LZ + k];
    lo[k] = v;
  }
  __syncwarp();  // every lane has read the LO fluxes before they are overwritten
  // HO vertical flux on T_AB with w; adf_v = HO - LO ("X - flux").
  Col<R> cho{sTA, sW, sA, sHn, sHnn, sZ, sX, nullptr};
  R* tvbuf = sm.slice(9);  // PPM edge values reuse the Z_3d_n slice (QR4C only)
  R* __restrict__ adfv = a.adfv + t * a.sW + n * LW;
  column_ver_flux<R, VER>(cho, tvbuf, sFlo, sFlo, nl, nzmin, nzmax, a.pv, dt, lane);
  for (int iz = lane; iz < (int)LW; iz += kWarp) adfv[iz] = iz < nl ? sFlo[iz] : R(0);
}

// ---------------------------------------------------------------------------
// FCT stage 2 (node columns): bounds a1-a3, antidiffusive sums b1 and the
// limiting factors b2 (lib/oce_adv_tra_fct.F90:98-374).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_fct_ratio(DMesh m, StepPtrs<R> a) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int n = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (n >= m.N) return;
  const int t = blockIdx.y;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nz = m.nz;
  R* smax = reinterpret_cast<R*>(smem_raw) + (size_t)wib * 3 * LW;
  R* smin = smax + LW;
  R* sadv = smin + LW;
  const R* __restrict__ T = a.T + t * a.sT;
  const R* __restrict__ LO = a.lo + t * a.sN;
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const int c0 = m.cl_ptr[n], c1 = m.cl_ptr[n + 1], minlev = m.cl_minlev[n];
  const R big = R(1e3);
  for (int k = lane; k < nz; k += kWarp) {
    const int z = k + 1;
    R mx = -big, mn = big;
    bool any = z > minlev;  // some element of the cluster lacks layer z: AUX = -/+1e3
    for (int j = c0; j < c1; ++j) {
      if (z > m.cl_lev[j]) continue;
      const size_t v = (size_t)m.cl_node[j] * LZ + k;
      const R lv = LO[v], tv = T[v];
      const R hi = rmax(lv, tv), lw = rmin(lv, tv);
      if (!any) {
        mx = hi;
        mn = lw;
        any = true;
      } else {
        mx = rmax(mx, hi);
        mn = rmin(mn, lw);
      }
    }
    smax[k] = mx;
    smin[k] = mn;
  }
  stage(sadv, a.adfv + t * a.sW + n * LW, m.nl, lane);
  __syncwarp();
  const R* __restrict__ adfh = a.adfh + t * a.sE;
  R* __restrict__ rp = a.rp + t * a.sN + n * LZ;
  R* __restrict__ rm = a.rm + t * a.sN + n * LZ;
  const R dt = a.dt;
  for (int k = lane; k < nz; k += kWarp) {
    const int z = k + 1;
    if (z < nzmin || z > nzmax - 1) continue;
    const R lo = LO[n * LZ + k];
    R bmax, bmin;
    if (z == nzmax - 1 || z == nzmin) {
      bmax = smax[k] - lo;
      bmin = smin[k] - lo;
    } else {
      bmax = rmax(rmax(smax[k - 1], smax[k]), smax[k + 1]) - lo;
      bmin = rmin(rmin(smin[k - 1], smin[k]), smin[k + 1]) - lo;
    }
    R plus = R(0) + (rmax(R(0), sadv[k]) + rmax(R(0), -sadv[k + 1]));
    R minus = R(0) + (rmin(R(0), sadv[k]) + rmin(R(0), -sadv[k + 1]));
    for (int j = m.ne_ptr[n]; j < m.ne_ptr[n + 1]; ++j) {
      if (z < m.ne_lo[j] || z > m.ne_hi[j]) continue;
      const int code = m.ne_code[j];
      R f = adfh[(size_t)(code >> 1) * LZ + k];
      if (code & 1) f = -f;
      plus = plus + rmax(R(0), f);
      minus = minus + rmin(R(0), f);
    }
    const R av = g.areasvol[n * LZ + k];
    R flux = (plus * dt) / av + R(1e-16);
    rp[k] = rmin(R(1), bmax / flux);
    flux = (minus * dt) / av - R(1e-16);
    rm[k] = rmin(R(1), bmin / flux);
  }
}

// ---------------------------------------------------------------------------
// FCT stage 3 (node columns): limiting b3 (lib/oce_adv_tra_fct.F90:396-471),
// flux divergence (oce_tra_adv_flux2dtracer with use_lo,
// lib/oce_adv_tra_driver.F90:298-450) and the caller's tendency update
// (src/fesom_analytic.F90:419-437 or lib/tracer_c_interface.F90:194-214).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_fct_update(DMesh m, StepPtrs<R> a) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int n = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (n >= m.N) return;
  const int t = blockIdx.y;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nz = m.nz, nl = m.nl;
  R* sLv = reinterpret_cast<R*>(smem_raw) + (size_t)wib * 3 * LW;
  R* sRp = sLv + LW;
  R* sRm = sRp + LW;
  const R* __restrict__ rp = a.rp + t * a.sN;
  const R* __restrict__ rm = a.rm + t * a.sN;
  stage(sRp, rp + n * LZ, nz, lane);
  stage(sRm, rm + n * LZ, nz, lane);
  const R* __restrict__ adfv = a.adfv + t * a.sW + n * LW;
  __syncwarp();
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  for (int iz = lane; iz < nl; iz += kWarp) {
    const int z = iz + 1;
    R f = adfv[iz];
    if (z == nzmin) {
      R ae = R(1);
      ae = (f >= R(0)) ? rmin(ae, sRp[iz]) : rmin(ae, sRm[iz]);
      f = ae * f;
    } else if (z > nzmin && z <= nzmax - 1) {
      R ae = R(1);
      if (f >= R(0)) {
        ae = rmin(ae, sRm[iz - 1]);
        ae = rmin(ae, sRp[iz]);
      } else {
        ae = rmin(ae, sRp[iz - 1]);
        ae = rmin(ae, sRm[iz]);
      }
      f = ae * f;
    }
    sLv[iz] = f;
  }
  __syncwarp();
  R* __restrict__ T = a.T + t * a.sT + n * LZ;
  const R* __restrict__ LO = a.lo + t * a.sN + n * LZ;
  const R* __restrict__ adfh = a.adfh + t * a.sE;
  R* __restrict__ del = a.del ? a.del + t * a.sN + n * LZ : nullptr;
  R* __restrict__ TAo = a.TAout ? a.TAout + t * a.sTA + n * LZ : nullptr;
  const R dt = a.dt;
  for (int k = lane; k < nz; k += kWarp) {
    const int z = k + 1;
    if (z < nzmin || z > nzmax - 1) continue;
    const R av = g.areasvol[n * LZ + k];
    const R Tn = T[k];
    R dv = (R(0) - Tn * g.hnode[n * LZ + k]) + LO[k] * g.hnode_new[n * LZ + k];
    dv = dv + ((sLv[k] - sLv[k + 1]) * dt) / av;
    R dh = R(0);
    const R rpn = sRp[k], rmn = sRm[k];
    for (int j = m.ne_ptr[n]; j < m.ne_ptr[n + 1]; ++j) {
      if (z < m.ne_lo[j] || z > m.ne_hi[j]) continue;
      const int code = m.ne_code[j];
      const R f = adfh[(size_t)(code >> 1) * LZ + k];
      const size_t o = (size_t)m.ne_other[j] * LZ + k;
      R ae = R(1);
      if (code & 1) {  // this node is the edge's second node
        if (f >= R(0)) { ae = rmin(ae, rp[o]); ae = rmin(ae, rmn); }
        else { ae = rmin(ae, rm[o]); ae = rmin(ae, rpn); }
        dh = dh - ((ae * f) * dt) / av;
      } else {
        if (f >= R(0)) { ae = rmin(ae, rpn); ae = rmin(ae, rm[o]); }
        else { ae = rmin(ae, rmn); ae = rmin(ae, rp[o]); }
        dh = dh + ((ae * f) * dt) / av;
      }
    }
    R d = del ? del[k] : R(0);
    d = d + dh + dv;
    if (del) del[k] = d;
    const R tn = Tn + d / g.hnode_new[n * LZ + k];
    T[k] = tn;
    if (TAo) TAo[k] = tn;
  }
}

// ---------------------------------------------------------------------------
// Without a limiter: vertical HO flux on T_AB with w_e, flux divergence
// (oce_tra_adv_flux2dtracer) and the tendency update in one pass.
// ---------------------------------------------------------------------------
template <typename R, int VER>
__global__ void k_nofct_update(DMesh m, StepPtrs<R> a) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int n = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (n >= m.N) return;
  const int t = blockIdx.y;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  ColSmem<R> sm{reinterpret_cast<R*>(smem_raw) + (size_t)wib * 10 * LW, (int)LW};
  R *sTA = sm.slice(1), *sW = sm.slice(2), *sA = sm.slice(4);
  R *sHn = sm.slice(5), *sHnn = sm.slice(6), *sF = sm.slice(7), *sX = sm.slice(8), *sZ = sm.slice(9);
  stage(sTA, a.TA + t * a.sTA + n * LZ, nz, lane);
  stage(sW, a.we + n * LW, nl, lane);
  stage(sA, g.area + n * LW, nl, lane);
  if (VER == 3) {
    stage(sHn, g.hnode + n * LZ, nz, lane);
    stage(sHnn, g.hnode_new + n * LZ, nz, lane);
  }
  if (VER == 1) {
    stage(sZ, g.Z3 + n * LZ, nz, lane);
    stage(sX, g.zbar3 + n * LW, nl, lane);
  }
  __syncwarp();
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  Col<R> c{sTA, sW, sA, sHn, sHnn, sZ, sX, nullptr};
  column_ver_flux<R, VER>(c, sm.slice(VER == 3 ? 9 : 0), nullptr, sF, nl, nzmin, nzmax, a.pv, a.dt, lane);
  R* __restrict__ T = a.T + t * a.sT + n * LZ;
  const R* __restrict__ fh = a.adfh + t * a.sE;
  R* __restrict__ del = a.del ? a.del + t * a.sN + n * LZ : nullptr;
  R* __restrict__ TAo = a.TAout ? a.TAout + t * a.sTA + n * LZ : nullptr;
  const R dt = a.dt;
  for (int k = lane; k < nz; k += kWarp) {
    const int z = k + 1;
    if (z < nzmin || z > nzmax - 1) continue;
    const R av = g.areasvol[n * LZ + k];
    const R dv = R(0) + ((sF[k] - sF[k + 1]) * dt) / av;
    R dh = R(0);
    for (int j = m.ne_ptr[n]; j < m.ne_ptr[n + 1]; ++j) {
      if (z < m.ne_lo[j] || z > m.ne_hi[j]) continue;
      const int code = m.ne_code[j];
      const R f = fh[(size_t)(code >> 1) * LZ + k];
      dh = (code & 1) ? dh - (f * dt) / av : dh + (f * dt) / av;
    }
    R d = del ? del[k] : R(0);
    d = d + dh + dv;
    if (del) del[k] = d;
    const R tn = T[k] + d / g.hnode_new[n * LZ + k];
    T[k] = tn;
    if (TAo) TAo[k] = tn;
  }
}

}  // namespace fgb
