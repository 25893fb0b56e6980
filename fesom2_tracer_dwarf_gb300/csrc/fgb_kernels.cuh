// Device kernels of the FESOM2 tracer-advection step (do_oce_adv_tra,
// lib/oce_adv_tra_driver.F90:23-294) for GB300 (sm_103a).
//
// Layout: level index fastest, columns padded to LZ layers / LW interfaces.
// Node-column kernels run one warp per node with the column staged in shared
// memory; edge kernels run one warp per edge, lanes over layers (coalesced
// rows) with two consecutive layers per lane. Node kernels loop over the
// tracers of a launch KC at a time, so the mesh tables, geometry and edge
// volume fluxes they load serve all tracers. The reference's edge scatters (atomics / OpenMP locks) are
// replaced by gathers over each node's incident edges in ascending edge order,
// which reproduces the reference's per-node summation order exactly.
//
// R is the storage and arithmetic type. Every expression keeps the
// reference's evaluation order; the FP64 translation unit is compiled without
// fused multiply-add so the device result equals the CPU restatement bit for bit.
#pragma once
#include <cstdint>

#include "fgb_device.hpp"

#ifndef FGB_FAST64
#define FGB_FAST64 0
#endif

namespace fgb {
// Two compilations of these kernels live side by side, kept apart by their
// inline namespace: the bit-exact FP64 form (no fused multiply-add, every
// division as the reference writes it) and, with FGB_FAST64, the fast FP64
// form (fused multiply-add; divisions by constants become products with the
// reciprocal constant, and dt / areasvol and 1 / hnode_new are formed once
// per layer and shared by the tracers and edges of a node).
#if FGB_FAST64
inline namespace fast64 {
#else
inline namespace exact64 {
#endif

constexpr int kWarp = 32;

template <typename R>
struct GeoSel;
template <>
struct GeoSel<double> {
  __host__ __device__ static const GeoPtrs<double>& get(const DMesh& m) { return m.g64; }
};
template <>
struct GeoSel<float> {
  __host__ __device__ static const GeoPtrs<float>& get(const DMesh& m) { return m.g32; }
};

template <typename R>
__device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <typename R>
__device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <typename R>
__device__ __forceinline__ R rabs(R a) { return fabs(a); }

// Division: correctly rounded in the FP64 form (bit parity with the CPU
// restatement), the fast single-precision reciprocal form (about 2 ulp) in
// the FP32 form.
template <typename R>
__device__ __forceinline__ R fdiv(R a, R b);
template <>
__device__ __forceinline__ double fdiv<double>(double a, double b) { return a / b; }
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }
// a / c for a constant c: the reference's division, or (fast form) the product
// with the reciprocal constant.
template <typename R>
__device__ __forceinline__ R fdivc(R a, R c) {
  if constexpr (FGB_FAST64) return a * (R(1) / c);
  else return fdiv(a, c);
}
// (x dt) / areasvol: the reference's order, or (fast form) x times the
// layer's dt / areasvol, formed once.
template <typename R>
__device__ __forceinline__ R dt_per_vol(R x, R dt, R av, R rdt_av) {
  if constexpr (FGB_FAST64) return x * rdt_av;
  else return fdiv(x * dt, av);
}
// a / g for a geometric g shared by the tracers of a column: the reference's
// division, or (fast form) the product with 1 / g, which the compiler forms
// once for all tracers.
template <typename R>
__device__ __forceinline__ R fdivg(R a, R g) {
  if constexpr (FGB_FAST64) return a * (R(1) / g);
  else return fdiv(a, g);
}
template <typename R>
__device__ __forceinline__ R rdt_vol(R dt, R av) {
  if constexpr (FGB_FAST64) return dt / av;
  else return R(0);  // unused by the exact form
}

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

// A triangle's nodes and gradient coefficients held in registers.
template <typename R>
struct Tri {
  int a, b, c;
  R x0, x1, x2, y0, y1, y2;
};

template <typename R>
__device__ __forceinline__ Tri<R> load_tri(const DMesh& m, const GeoPtrs<R>& g, int el) {
  Tri<R> q;
  q.a = m.elem_nodes[3 * el];
  q.b = m.elem_nodes[3 * el + 1];
  q.c = m.elem_nodes[3 * el + 2];
  const R* gs = g.grad_sca + 6 * (size_t)el;
  q.x0 = gs[0]; q.x1 = gs[1]; q.x2 = gs[2];
  q.y0 = gs[3]; q.y1 = gs[4]; q.y2 = gs[5];
  return q;
}

template <typename R>
__device__ __forceinline__ void tri_grad(const Tri<R>& q, const R* __restrict__ T, size_t LZ, int k, R& gx, R& gy) {
  const R ta = T[q.a * LZ + k], tb = T[q.b * LZ + k], tc = T[q.c * LZ + k];
  gx = q.x0 * ta + q.x1 * tb + q.x2 * tc;
  gy = q.y0 * ta + q.y1 * tb + q.y2 * tc;
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
  gx = fdiv(tx, tvol);
  gy = fdiv(ty, tvol);
}

// Two consecutive layers per lane: vector loads and stores of R pairs.
template <typename R>
struct V2T;
template <>
struct V2T<float> {
  using T = float2;
};
template <>
struct V2T<double> {
  using T = double2;
};
template <typename R>
using vec2 = typename V2T<R>::T;
template <typename R>
__device__ __forceinline__ vec2<R> ld2(const R* p) {
  return *reinterpret_cast<const vec2<R>*>(p);
}
template <typename R>
__device__ __forceinline__ void st2(R* p, R a, R b) {
  vec2<R> v;
  v.x = a;
  v.y = b;
  *reinterpret_cast<vec2<R>*>(p) = v;
}

// Four values per lane (two layers of an interleaved pair array).
template <typename R>
struct Q4 {
  R a, b, c, d;
};
__device__ __forceinline__ Q4<float> ld4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return Q4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Q4<double> ld4(const double* p) {
  const double2 u = *reinterpret_cast<const double2*>(p), v = *reinterpret_cast<const double2*>(p + 2);
  return Q4<double>{u.x, u.y, v.x, v.y};
}
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void st4(double* p, double a, double b, double c, double d) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
  *reinterpret_cast<double2*>(p + 2) = make_double2(c, d);
}

// High-order horizontal flux of one layer: upwind (adv_tra_hor_upw1,
// lib/oce_adv_tra_hor.F90:218-220) or the MUSCL/MFCT edge reconstruction
// (lib/oce_adv_tra_hor.F90:454-497, :748-790); c1, c2 are the c_lo masks.
template <typename R, int HOR>
__device__ __forceinline__ R ho_flux(R v, R vp, R vm, R ta1, R ta2, R g1, R g2, R g3, R g4, R ex, R ey, R c1, R c2,
                                     R ph) {
  if (HOR == 0) return -(R(0.5) * (ta1 * vp + ta2 * vm));
  R Tm2, Tm1;
  if (HOR == 1) {
    Tm2 = ta2 - fdivc(R(2) * (ta2 - ta1) + ex * g2 + ey * g4, R(6)) * c2;
    Tm1 = ta1 + fdivc(R(2) * (ta2 - ta1) + ex * g1 + ey * g3, R(6)) * c1;
  } else {
    Tm2 = ta2 - fdivc(R(2) * (ta2 - ta1) + ex * g2 + ey * g4, R(6));
    Tm1 = ta1 + fdivc(R(2) * (ta2 - ta1) + ex * g1 + ey * g3, R(6));
  }
  const R cHO = vp * Tm1 + vm * Tm2;
  return -((R(0.5) * (R(1) - ph)) * cHO) - ((v * ph) * R(0.5)) * (Tm1 + Tm2);
}

// ---------------------------------------------------------------------------
// Horizontal edge fluxes of all K tracers. FCT: the antidiffusive flux
// HO(T_AB) - LO(T) (adv_tra_hor_* with o_init_zero=.false. after
// adv_tra_hor_upw1, lib/oce_adv_tra_driver.F90:95,244-255); otherwise the HO
// flux. HOR: 0 UPW1, 1 MUSCL (with the nboundary_lay mask c_lo), 2 MFCT.
// One warp per edge, two layers per lane. Edges are visited in edge_order
// (the three edge families interleaved by node) for cache locality; results
// are stored at the edge's own index.
// ---------------------------------------------------------------------------
template <typename R, int HOR, bool FCT>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2)) k_hflux(DMesh m, StepPtrs<R> a) {
  const int lane = threadIdx.x & (kWarp - 1);
  const int w = blockIdx.x * (blockDim.x / kWarp) + (threadIdx.x / kWarp);
  if (w >= m.E) return;
  const int e = m.edge_order ? m.edge_order[w] : w;
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ;
  const int n1 = m.edge_nodes[2 * e], n2 = m.edge_nodes[2 * e + 1];
  const int nu1 = m.edge_lev[4 * e], nl1 = m.edge_lev[4 * e + 1];
  const int nu2 = m.edge_lev[4 * e + 2], nl2 = m.edge_lev[4 * e + 3];
  int gm0 = -1, gm1 = -1, nb1 = 0, nb2 = 0;
  R ex = R(0), ey = R(0);
  Tri<R> tu{}, td{};
  if (HOR != 0) {
    gm0 = m.edge_gm[2 * e];
    gm1 = m.edge_gm[2 * e + 1];
    ex = g.edge_dxa[2 * e];
    ey = g.edge_dxa[2 * e + 1];
    nb1 = m.nbl[n1];
    nb2 = m.nbl[n2];
    if (gm0 >= 0) {
      tu = load_tri(m, g, m.edge_updn[2 * e]);
      td = load_tri(m, g, m.edge_updn[2 * e + 1]);
    }
  }
  const R ph = a.ph;
  const bool ta_sep = a.TA != a.T;
  for (int p = lane; 2 * p < m.LZ; p += kWarp) {
    const int k0 = 2 * p;
    const int z0 = k0 + 1, z1 = k0 + 2;
    const size_t ek = (size_t)e * LZ + k0;
    const bool a0 = k0 < m.nz && edge_seg(z0, nu1, nl1, nu2, nl2) != 0;
    const bool a1 = k0 + 1 < m.nz && edge_seg(z1, nu1, nl1, nu2, nl2) != 0;
    if (!a0 && !a1) {
      for (int t = 0; t < a.K; ++t) st2(a.adfh + t * a.sE + ek, R(0), R(0));
      continue;
    }
    const vec2<R> vv = ld2(a.vf + ek);
    const R v0 = vv.x, v1 = vv.y;
    const R vp0 = v0 + rabs(v0), vm0 = v0 - rabs(v0), vp1 = v1 + rabs(v1), vm1 = v1 - rabs(v1);
    const bool tri0 = gm0 >= 0 && z0 >= gm0 && z0 <= gm1 - 1;
    const bool tri1 = gm0 >= 0 && z1 >= gm0 && z1 <= gm1 - 1;
    const R c10 = (nb1 - z0 >= 0) ? R(1) : R(0), c11 = (nb1 - z1 >= 0) ? R(1) : R(0);
    const R c20 = (nb2 - z0 >= 0) ? R(1) : R(0), c21 = (nb2 - z1 >= 0) ? R(1) : R(0);
    for (int t = 0; t < a.K; ++t) {
      const R* __restrict__ T = a.T + t * a.sT;
      const R* __restrict__ TA = ta_sep ? a.TA + t * a.sTA : T;
      const vec2<R> s1 = ld2(TA + n1 * LZ + k0), s2 = ld2(TA + n2 * LZ + k0);
      R lo0 = R(0), lo1 = R(0);
      if (FCT) {
        const vec2<R> r1 = ta_sep ? ld2(T + n1 * LZ + k0) : s1;
        const vec2<R> r2 = ta_sep ? ld2(T + n2 * LZ + k0) : s2;
        lo0 = -(R(0.5) * (r1.x * vp0 + r2.x * vm0));
        lo1 = -(R(0.5) * (r1.y * vp1 + r2.y * vm1));
      }
      R g10 = R(0), g20 = R(0), g30 = R(0), g40 = R(0), g11 = R(0), g21 = R(0), g31 = R(0), g41 = R(0);
      if (HOR != 0) {
        if (tri0 && tri1) {
          // the upwind triangle holds node 1 and the downwind one node 2: reuse those columns
          const vec2<R> ua = tu.a == n1 ? s1 : ld2(TA + tu.a * LZ + k0);
          const vec2<R> ub = tu.b == n1 ? s1 : ld2(TA + tu.b * LZ + k0);
          const vec2<R> uc = tu.c == n1 ? s1 : ld2(TA + tu.c * LZ + k0);
          const vec2<R> da = td.a == n2 ? s2 : ld2(TA + td.a * LZ + k0);
          const vec2<R> db = td.b == n2 ? s2 : ld2(TA + td.b * LZ + k0);
          const vec2<R> dc = td.c == n2 ? s2 : ld2(TA + td.c * LZ + k0);
          g10 = tu.x0 * ua.x + tu.x1 * ub.x + tu.x2 * uc.x;
          g30 = tu.y0 * ua.x + tu.y1 * ub.x + tu.y2 * uc.x;
          g11 = tu.x0 * ua.y + tu.x1 * ub.y + tu.x2 * uc.y;
          g31 = tu.y0 * ua.y + tu.y1 * ub.y + tu.y2 * uc.y;
          g20 = td.x0 * da.x + td.x1 * db.x + td.x2 * dc.x;
          g40 = td.y0 * da.x + td.y1 * db.x + td.y2 * dc.x;
          g21 = td.x0 * da.y + td.x1 * db.y + td.x2 * dc.y;
          g41 = td.y0 * da.y + td.y1 * db.y + td.y2 * dc.y;
        } else {
          if (a0) {
            if (tri0) {
              tri_grad(tu, TA, LZ, k0, g10, g30);
              tri_grad(td, TA, LZ, k0, g20, g40);
            } else {
              node_mean_grad(m, g, TA, n1, k0, g10, g30);
              node_mean_grad(m, g, TA, n2, k0, g20, g40);
            }
          }
          if (a1) {
            if (tri1) {
              tri_grad(tu, TA, LZ, k0 + 1, g11, g31);
              tri_grad(td, TA, LZ, k0 + 1, g21, g41);
            } else {
              node_mean_grad(m, g, TA, n1, k0 + 1, g11, g31);
              node_mean_grad(m, g, TA, n2, k0 + 1, g21, g41);
            }
          }
        }
      }
      const R h0 = ho_flux<R, HOR>(v0, vp0, vm0, s1.x, s2.x, g10, g20, g30, g40, ex, ey, c10, c20, ph);
      const R h1 = ho_flux<R, HOR>(v1, vp1, vm1, s1.y, s2.y, g11, g21, g31, g41, ex, ey, c11, c21, ph);
      st2(a.adfh + t * a.sE + ek, a0 ? (FCT ? h0 - lo0 : h0) : R(0), a1 ? (FCT ? h1 - lo1 : h1) : R(0));
    }
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
  const R qc = fdivg(Tm1 - T0, Zm1 - Z0);
  const R qu = fdivg(T0 - Tp1, Z0 - Zp1);
  const R qd = fdivg(Tm2 - Tm1, Zm2 - Zm1);
  const R zb = c.zb[z - 1];
  const R tm1 = T0 + fdivc((R(2) * qc + qu) * (zb - Z0), R(3));
  const R tm2 = Tm1 + fdivc((R(2) * qc + qd) * (zb - Zm1), R(3));
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
    R deltaj = fdiv(dzj, dzjm1 + dzj + dzjp1) *
               (fdiv(R(2) * dzjm1 + dzj, dzjp1 + dzj) * (Tp - T0) + fdiv(dzj + R(2) * dzjp1, dzjm1 + dzj) * (T0 - Tm));
    R deltajp1 = fdiv(dzjp1, dzj + dzjp1 + dzjp2) *
                 (fdiv(R(2) * dzj + dzjp1, dzjp2 + dzjp1) * (Tpp - Tp) + fdiv(dzjp1 + R(2) * dzjp2, dzj + dzjp1) * (Tp - T0));
    if ((Tp - T0) * (T0 - Tm) > R(0))
      deltaj = rmin(rmin(rabs(deltaj), R(2) * rabs(Tp - T0)), R(2) * rabs(T0 - Tm)) * copysign(R(1), deltaj);
    else
      deltaj = R(0);
    if ((Tpp - Tp) * (Tp - T0) > R(0))
      deltajp1 = rmin(rmin(rabs(deltajp1), R(2) * rabs(Tpp - Tp)), R(2) * rabs(Tp - T0)) * copysign(R(1), deltajp1);
    else
      deltajp1 = R(0);
    const R inner1 = fdiv((R(2) * dzjp1) * dzj, dzj + dzjp1) *
                     (fdiv(dzjm1 + dzj, R(2) * dzj + dzjp1) - fdiv(dzjp2 + dzjp1, R(2) * dzjp1 + dzj)) * (Tp - T0);
    const R inner2 = fdiv(dzj * (dzjm1 + dzj), R(2) * dzj + dzjp1) * deltajp1;
    const R inner3 = fdiv(dzjp1 * (dzjp1 + dzjp2), dzj + R(2) * dzjp1) * deltaj;
    return (T0 + fdiv(dzj, dzj + dzjp1) * (Tp - T0)) + fdiv(R(1), dzjm1 + dzj + dzjp1 + dzjp2) * (inner1 - inner2 + inner3);
  }
  if (z == nzmax) return T[nzmax - 2];
  if (z == nzmax - 1) {
    const R s = copysign(R(1), c.W[nzmax - 2]);
    return -(T[nzmax - 3] * rmin(s, R(0))) + T[nzmax - 2] * rmax(s, R(0));
  }
  if (z == nzmin + 1) return R(0.5) * (T[nzmin - 1] + T[nzmin]);
  return T[nzmin - 1];
}

// The tracer part of ppm_layer for a given x = min(|W| dt / h, 1) of the layer.
template <typename R>
__device__ __forceinline__ R ppm_layer_x(R aL, R aR, R T0, R x, bool upper, R area, R W) {
  if ((aR - T0) * (T0 - aL) <= R(0)) {
    aL = T0;
    aR = T0;
  }
  if ((aR - aL) * (T0 - R(0.5) * (aL + aR)) > fdivc((aR - aL) * (aR - aL), R(6))) aL = R(3) * T0 - R(2) * aR;
  if ((aR - aL) * (T0 - R(0.5) * (aR + aL)) < -fdivc((aR - aL) * (aR - aL), R(6))) aR = R(3) * T0 - R(2) * aL;
  const R aj = R(6) * (T0 - R(0.5) * (aL + aR));
  if (upper) {
    R tv = -aL - (R(0.5) * x) * ((aR - aL) + (R(1) - fdivc(R(2), R(3)) * x) * aj);
    return (tv * area) * W;
  }
  R tv = -aR + (R(0.5) * x) * ((aR - aL) - (R(1) - fdivc(R(2), R(3)) * x) * aj);
  return (tv * area) * W;
}

// x of ppm_layer: upper side min(W dt / h, 1), lower side min(-(W dt / h), 1).
template <typename R>
__device__ __forceinline__ R ppm_x(R W, R dt, R dzj, bool upper) {
  return upper ? rmin(fdiv(W * dt, dzj), R(1)) : rmin(-fdiv(W * dt, dzj), R(1));
}

// PPM flux contribution of layer nz to its interface (upper: W(nz) > 0 side,
// lower: W(nz+1) < 0 side), lib/oce_adv_tra_ver.F90:598-632.
template <typename R>
__device__ __forceinline__ R ppm_layer(const Col<R>& c, int nz, bool upper, R dt) {
  const R dzj = c.hn[nz - 1];
  if (upper) {
    const R W = c.W[nz - 1];
    return ppm_layer_x(c.tv[nz - 1], c.tv[nz], c.T[nz - 1], ppm_x(W, dt, dzj, true), true, c.area[nz - 1], W);
  }
  const R W = c.W[nz];
  return ppm_layer_x(c.tv[nz - 1], c.tv[nz], c.T[nz - 1], ppm_x(W, dt, dzj, false), false, c.area[nz], W);
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

// PPM vertical HO fluxes of KC tracer columns of one node (column_ver_flux
// with VER = 3 for each tracer), with the geometry-only divisions of the edge
// values and of x done once per interface instead of once per tracer: the
// same operations on the same operands, so the results are bit-identical.
// T, tv, fold and out hold KC columns LW apart; fold == out is allowed.
template <typename R, int KC>
__device__ __forceinline__ void column_ppm_multi(const Col<R>& g, const R* T, R* tv, const R* fold, R* out, int LW,
                                                 int nl, int nzmin, int nzmax, R dt, int lane) {
  const R* hnn = g.hnn;
  for (int iz = lane; iz < nl; iz += kWarp) {
    const int z = iz + 1;
    if (z < nzmin || z > nzmax) {
#pragma unroll
      for (int i = 0; i < KC; ++i) tv[i * LW + iz] = R(0);
      continue;
    }
    if (z >= nzmin + 2 && z <= nzmax - 2) {
      const int nz = z - 1;
      const R dzjm1 = hnn[nz - 2], dzj = hnn[nz - 1], dzjp1 = hnn[nz], dzjp2 = hnn[nz + 1];
      const R ga = fdiv(dzj, dzjm1 + dzj + dzjp1);
      const R gb = fdiv(R(2) * dzjm1 + dzj, dzjp1 + dzj), gc = fdiv(dzj + R(2) * dzjp1, dzjm1 + dzj);
      const R gd = fdiv(dzjp1, dzj + dzjp1 + dzjp2);
      const R ge = fdiv(R(2) * dzj + dzjp1, dzjp2 + dzjp1), gf = fdiv(dzjp1 + R(2) * dzjp2, dzj + dzjp1);
      const R gh = fdiv((R(2) * dzjp1) * dzj, dzj + dzjp1) *
                   (fdiv(dzjm1 + dzj, R(2) * dzj + dzjp1) - fdiv(dzjp2 + dzjp1, R(2) * dzjp1 + dzj));
      const R gi = fdiv(dzj * (dzjm1 + dzj), R(2) * dzj + dzjp1);
      const R gj = fdiv(dzjp1 * (dzjp1 + dzjp2), dzj + R(2) * dzjp1);
      const R gk = fdiv(dzj, dzj + dzjp1), gl = fdiv(R(1), dzjm1 + dzj + dzjp1 + dzjp2);
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const R* Ti = T + i * LW;
        const R Tm = Ti[nz - 2], T0 = Ti[nz - 1], Tp = Ti[nz], Tpp = Ti[nz + 1];
        R deltaj = ga * (gb * (Tp - T0) + gc * (T0 - Tm));
        R deltajp1 = gd * (ge * (Tpp - Tp) + gf * (Tp - T0));
        if ((Tp - T0) * (T0 - Tm) > R(0))
          deltaj = rmin(rmin(rabs(deltaj), R(2) * rabs(Tp - T0)), R(2) * rabs(T0 - Tm)) * copysign(R(1), deltaj);
        else
          deltaj = R(0);
        if ((Tpp - Tp) * (Tp - T0) > R(0))
          deltajp1 = rmin(rmin(rabs(deltajp1), R(2) * rabs(Tpp - Tp)), R(2) * rabs(Tp - T0)) * copysign(R(1), deltajp1);
        else
          deltajp1 = R(0);
        const R inner1 = gh * (Tp - T0);
        const R inner2 = gi * deltajp1;
        const R inner3 = gj * deltaj;
        tv[i * LW + iz] = (T0 + gk * (Tp - T0)) + gl * (inner1 - inner2 + inner3);
      }
    } else {
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const Col<R> ci{T + i * LW, g.W, g.area, g.hn, g.hnn, g.Z, g.zb, nullptr};
        tv[i * LW + iz] = ppm_tv(ci, z, nzmin, nzmax);
      }
    }
  }
  __syncwarp();
  for (int iz = lane; iz < nl; iz += kWarp) {
    const int z = iz + 1;
    R f0[KC];
#pragma unroll
    for (int i = 0; i < KC; ++i) f0[i] = fold ? fold[i * LW + iz] : R(0);
    if (z < nzmin || z > nzmax) {
#pragma unroll
      for (int i = 0; i < KC; ++i) out[i * LW + iz] = f0[i];
      continue;
    }
    if (z == nzmin) {
#pragma unroll
      for (int i = 0; i < KC; ++i)
        out[i * LW + iz] = -((tv[i * LW + nzmin - 1] * g.W[nzmin - 1]) * g.area[nzmin - 1]) - f0[i];
      continue;
    }
    const R W = g.W[z - 1];
    if (z < nzmax && W != R(0)) {
      const bool up = W > R(0);
      const int L = up ? z : z - 1;  // the layer whose parabola crosses the interface
      const R x = ppm_x(W, dt, g.hn[L - 1], up);
#pragma unroll
      for (int i = 0; i < KC; ++i)
        out[i * LW + iz] =
            ppm_layer_x(tv[i * LW + L - 1], tv[i * LW + L], T[i * LW + L - 1], x, up, g.area[z - 1], W) - f0[i];
    } else {
#pragma unroll
      for (int i = 0; i < KC; ++i) out[i * LW + iz] = R(0) - f0[i];
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Node-column kernels. One warp per node, two layers per lane; tracers are
// processed KC at a time. The node's incident edges (ascending edge index,
// the reference's scatter order) and its FCT cluster are staged once in
// shared memory; gathers run edge-outer, tracer-inner, so every edge's
// metadata is read once and the loads of all KC tracers are in flight
// together. Per-(tracer, layer) summation order is the reference's.
// ---------------------------------------------------------------------------
struct Nbr {
  int e, role, other, lo, hi;
};
constexpr int kMaxDeg = 16;  // incident edges staged per node; more are read from global memory
constexpr int kMaxCl = 24;   // cluster nodes staged per node

__device__ __forceinline__ Nbr nbr_global(const DMesh& m, int j) {
  const int code = m.ne_code[j];
  return Nbr{code >> 1, code & 1, m.ne_other[j], m.ne_lo[j], m.ne_hi[j]};
}

struct NbrList {
  const Nbr* s;
  int j0, deg;
  __device__ __forceinline__ Nbr get(const DMesh& m, int j) const {
    return deg <= kMaxDeg ? s[j] : nbr_global(m, j0 + j);
  }
};

__device__ __forceinline__ NbrList stage_nbrs(const DMesh& m, int n, Nbr* s, int lane) {
  NbrList L{s, m.ne_ptr[n], m.ne_ptr[n + 1] - m.ne_ptr[n]};
  if (L.deg <= kMaxDeg)
    for (int j = lane; j < L.deg; j += kWarp) s[j] = nbr_global(m, L.j0 + j);
  return L;
}

// Shared memory of one warp: `slices` columns of LW values, the edge list and
// `extra_bytes` more.
template <typename R>
__host__ __device__ constexpr size_t warp_smem(int slices, int LW, int extra_bytes) {
  return ((size_t)slices * LW * sizeof(R) + kMaxDeg * sizeof(Nbr) + extra_bytes + 15) / 16 * 16;
}
__host__ __device__ constexpr int lo_slices(int KC) { return 7 + 4 * KC; }
__host__ __device__ constexpr int ratio_slices(int KC) { return 3 * KC; }
__host__ __device__ constexpr int upd_slices(int KC) { return 3 * KC; }
__host__ __device__ constexpr int nofct_slices(int KC) { return 7 + 3 * KC; }
constexpr int kClBytes = kMaxCl * 2 * (int)sizeof(int);

// ---------------------------------------------------------------------------
// FCT stage 1: low-order solution fct_LO (lib/oce_adv_tra_driver.F90:91-235)
// and the vertical antidiffusive flux HO(T_AB, w) - LO(T, w_e). The low-order
// horizontal edge fluxes are formed here from T and the edge volume fluxes,
// with the expression adv_tra_hor_upw1 uses (lib/oce_adv_tra_hor.F90:218-220).
// ---------------------------------------------------------------------------
template <typename R, int VER, int KC>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 8 : 4)) k_fct_lo(DMesh m, StepPtrs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int vi = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  unsigned char* base = smem_raw + (size_t)wib * warp_smem<R>(lo_slices(KC), m.LW, 0);
  R* sl = reinterpret_cast<R*>(base);
  R *sW = sl, *sWE = sl + LW, *sA = sl + 2 * LW, *sHn = sl + 3 * LW, *sHnn = sl + 4 * LW, *sX = sl + 5 * LW;
  R* sZ = sl + 6 * LW;
  R* sT = sl + 7 * LW;                 // KC columns
  R* sTA = sT + (size_t)KC * LW;       // KC columns (T_AB when it is a separate field)
  R* sFv = sTA + (size_t)KC * LW;      // KC columns of vertical fluxes
  R* sTv = sFv + (size_t)KC * LW;      // KC columns of PPM edge values
  const NbrList nb = stage_nbrs(m, n, reinterpret_cast<Nbr*>(base + lo_slices(KC) * LW * sizeof(R)), lane);
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
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const bool ta_sep = a.TA != a.T;
  const R dt = a.dt;
  for (int t0 = 0; t0 < a.K; t0 += KC) {
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      stage(sT + i * LW, a.T + (t0 + i) * a.sT + n * LZ, nz, lane);
      if (ta_sep) stage(sTA + i * LW, a.TA + (t0 + i) * a.sTA + n * LZ, nz, lane);
    }
    __syncwarp();
    // LO vertical flux: adv_tra_ver_upw1(we, ttf) with init zero.
    for (int i = 0; i < KC; ++i) {
      Col<R> clo{sT + i * LW, sWE, sA, sHn, sHnn, sZ, sX, nullptr};
      column_ver_flux<R, 0>(clo, nullptr, nullptr, sFv + i * LW, nl, nzmin, nzmax, R(1), dt, lane);
    }
    for (int p = lane; 2 * p < m.LZ; p += kWarp) {
      const int k0 = 2 * p, z0 = k0 + 1, z1 = k0 + 2;
      R acc0[KC], acc1[KC];
#pragma unroll
      for (int i = 0; i < KC; ++i) acc0[i] = acc1[i] = R(0);
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const Nbr q = nb.get(m, j);
        const bool a0 = z0 >= q.lo && z0 <= q.hi, a1 = z1 >= q.lo && z1 <= q.hi;
        const vec2<R> vv = ld2(a.vf + (size_t)q.e * LZ + k0);
        const R vp0 = vv.x + rabs(vv.x), vm0 = vv.x - rabs(vv.x);
        const R vp1 = vv.y + rabs(vv.y), vm1 = vv.y - rabs(vv.y);
#pragma unroll
        for (int i = 0; i < KC; ++i) {
          const vec2<R> to = ld2(a.T + (t0 + i) * a.sT + (size_t)q.other * LZ + k0);
          const R tn0 = sT[i * LW + k0], tn1 = sT[i * LW + k0 + 1];
          if (q.role) {  // this node is the edge's second node
            if (a0) acc0[i] = acc0[i] - (-(R(0.5) * (to.x * vp0 + tn0 * vm0)));
            if (a1) acc1[i] = acc1[i] - (-(R(0.5) * (to.y * vp1 + tn1 * vm1)));
          } else {
            if (a0) acc0[i] = acc0[i] + (-(R(0.5) * (tn0 * vp0 + to.x * vm0)));
            if (a1) acc1[i] = acc1[i] + (-(R(0.5) * (tn1 * vp1 + to.y * vm1)));
          }
        }
      }
      const vec2<R> hn = ld2(g.hnode + n * LZ + k0), hnn = ld2(g.hnode_new + n * LZ + k0);
      const vec2<R> av = ld2(g.areasvol + n * LZ + k0);
      const bool w0 = z0 >= nzmin && z0 <= nzmax - 1, w1 = z1 >= nzmin && z1 <= nzmax - 1;
      // fast form: dt / areasvol and 1 / hnode_new of the two layers, once
      const vec2<R> rd{rdt_vol(dt, av.x), rdt_vol(dt, av.y)};
      const vec2<R> rh{FGB_FAST64 ? R(1) / hnn.x : R(0), FGB_FAST64 ? R(1) / hnn.y : R(0)};
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const R* Ti = sT + i * LW;
        const R* Fi = sFv + i * LW;
        R l0 = acc0[i], l1 = acc1[i];
        if constexpr (FGB_FAST64) {
          if (w0) l0 = (Ti[k0] * hn.x + (acc0[i] + (Fi[k0] - Fi[k0 + 1])) * rd.x) * rh.x;
          if (w1) l1 = (Ti[k0 + 1] * hn.y + (acc1[i] + (Fi[k0 + 1] - Fi[k0 + 2])) * rd.y) * rh.y;
        } else {
          if (w0) l0 = fdiv(Ti[k0] * hn.x + fdiv((acc0[i] + (Fi[k0] - Fi[k0 + 1])) * dt, av.x), hnn.x);
          if (w1) l1 = fdiv(Ti[k0 + 1] * hn.y + fdiv((acc1[i] + (Fi[k0 + 1] - Fi[k0 + 2])) * dt, av.y), hnn.y);
        }
        st2(a.lo + (t0 + i) * a.sN + n * LZ + k0, l0, l1);
      }
    }
    __syncwarp();  // every lane has read the LO fluxes before they are overwritten
    if (a.wi) {
      // w_split: the antidiffusive flux takes the upwind flux of the full w
      // (lib/oce_adv_tra_driver.F90:221-231)
      for (int i = 0; i < KC; ++i) {
        Col<R> clw{sT + i * LW, sW, sA, sHn, sHnn, sZ, sX, nullptr};
        column_ver_flux<R, 0>(clw, nullptr, nullptr, sFv + i * LW, nl, nzmin, nzmax, R(1), dt, lane);
      }
    }
    // HO vertical flux on T_AB with w; adf_v = HO - LO ("X - flux").
    if constexpr (VER == 3) {
      const Col<R> g{nullptr, sW, sA, sHn, sHnn, sZ, sX, nullptr};
      column_ppm_multi<R, KC>(g, ta_sep ? sTA : sT, sTv, sFv, sFv, (int)LW, nl, nzmin, nzmax, dt, lane);
    }
    for (int i = 0; i < KC; ++i) {
      if constexpr (VER != 3) {
        Col<R> cho{(ta_sep ? sTA : sT) + i * LW, sW, sA, sHn, sHnn, sZ, sX, nullptr};
        column_ver_flux<R, VER>(cho, sTv + i * LW, sFv + i * LW, sFv + i * LW, nl, nzmin, nzmax, a.pv, dt, lane);
      }
      R* __restrict__ adfv = a.adfv + (t0 + i) * a.sW + n * LW;
      for (int iz = lane; iz < (int)LW; iz += kWarp) adfv[iz] = iz < nl ? sFv[i * LW + iz] : R(0);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// FCT stage 2: bounds a1-a3, antidiffusive sums b1 and the limiting factors
// b2 (lib/oce_adv_tra_fct.F90:98-374). The cluster bound is the maximum over
// the cluster's elements of the maximum over their nodes; max is exact, so
// the distinct nodes with the deepest layer reaching them give the same value.
// ---------------------------------------------------------------------------
template <typename R, int KC>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 8 : 4)) k_fct_ratio(DMesh m, StepPtrs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int vi = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  unsigned char* base = smem_raw + (size_t)wib * warp_smem<R>(ratio_slices(KC), m.LW, kClBytes);
  R* smax = reinterpret_cast<R*>(base);
  R* smin = smax + (size_t)KC * LW;
  R* sadv = smin + (size_t)KC * LW;
  const NbrList nb = stage_nbrs(m, n, reinterpret_cast<Nbr*>(base + ratio_slices(KC) * LW * sizeof(R)), lane);
  int* scl = reinterpret_cast<int*>(base + ratio_slices(KC) * LW * sizeof(R) + kMaxDeg * sizeof(Nbr));
  const int c0 = m.cl_ptr[n], ncl = m.cl_ptr[n + 1] - c0, minlev = m.cl_minlev[n];
  const bool cl_staged = ncl <= kMaxCl;
  if (cl_staged)
    for (int j = lane; j < ncl; j += kWarp) {
      scl[2 * j] = m.cl_node[c0 + j];
      scl[2 * j + 1] = m.cl_lev[c0 + j];
    }
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const R big = R(1e3), dt = a.dt;
  const R inf = R(INFINITY);
  for (int t0 = 0; t0 < a.K; t0 += KC) {
#pragma unroll
    for (int i = 0; i < KC; ++i) stage(sadv + i * LW, a.adfv + (t0 + i) * a.sW + n * LW, m.nl, lane);
    __syncwarp();
    for (int p = lane; 2 * p < m.LZ; p += kWarp) {
      const int k0 = 2 * p, z0 = k0 + 1, z1 = k0 + 2;
      // AUX = -/+1e3 of elements without the layer joins the bound (lib/oce_adv_tra_fct.F90:139-145)
      const R mx0i = z0 > minlev ? -big : -inf, mx1i = z1 > minlev ? -big : -inf;
      R mx0[KC], mx1[KC], mn0[KC], mn1[KC];
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        mx0[i] = mx0i;
        mx1[i] = mx1i;
        mn0[i] = -mx0i;
        mn1[i] = -mx1i;
      }
#pragma unroll 2
      for (int j = 0; j < ncl; ++j) {
        const int node = cl_staged ? scl[2 * j] : m.cl_node[c0 + j];
        const int lev = cl_staged ? scl[2 * j + 1] : m.cl_lev[c0 + j];
        const bool a0 = z0 <= lev, a1 = z1 <= lev;
#pragma unroll
        for (int i = 0; i < KC; ++i) {
          const size_t v = (size_t)node * LZ + k0;
          const vec2<R> lv = ld2(a.lo + (t0 + i) * a.sN + v), tv = ld2(a.T + (t0 + i) * a.sT + v);
          if (a0) {
            mx0[i] = rmax(mx0[i], rmax(lv.x, tv.x));
            mn0[i] = rmin(mn0[i], rmin(lv.x, tv.x));
          }
          if (a1) {
            mx1[i] = rmax(mx1[i], rmax(lv.y, tv.y));
            mn1[i] = rmin(mn1[i], rmin(lv.y, tv.y));
          }
        }
      }
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        smax[i * LW + k0] = mx0[i];
        smax[i * LW + k0 + 1] = mx1[i];
        smin[i * LW + k0] = mn0[i];
        smin[i * LW + k0 + 1] = mn1[i];
      }
    }
    __syncwarp();
    for (int p = lane; 2 * p < m.LZ; p += kWarp) {
      const int k0 = 2 * p;
      R pl0[KC], pl1[KC], mi0[KC], mi1[KC];
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const R* ad = sadv + i * LW;
        pl0[i] = R(0) + (rmax(R(0), ad[k0]) + rmax(R(0), -ad[k0 + 1]));
        mi0[i] = R(0) + (rmin(R(0), ad[k0]) + rmin(R(0), -ad[k0 + 1]));
        pl1[i] = R(0) + (rmax(R(0), ad[k0 + 1]) + rmax(R(0), -ad[k0 + 2]));
        mi1[i] = R(0) + (rmin(R(0), ad[k0 + 1]) + rmin(R(0), -ad[k0 + 2]));
      }
      const int z0 = k0 + 1, z1 = k0 + 2;
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const Nbr q = nb.get(m, j);
        const bool a0 = z0 >= q.lo && z0 <= q.hi, a1 = z1 >= q.lo && z1 <= q.hi;
#pragma unroll
        for (int i = 0; i < KC; ++i) {
          vec2<R> f = ld2(a.adfh + (t0 + i) * a.sE + (size_t)q.e * LZ + k0);
          if (q.role) {
            f.x = -f.x;
            f.y = -f.y;
          }
          if (a0) {
            pl0[i] = pl0[i] + rmax(R(0), f.x);
            mi0[i] = mi0[i] + rmin(R(0), f.x);
          }
          if (a1) {
            pl1[i] = pl1[i] + rmax(R(0), f.y);
            mi1[i] = mi1[i] + rmin(R(0), f.y);
          }
        }
      }
      const vec2<R> av = ld2(g.areasvol + n * LZ + k0);
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const R* mxs = smax + i * LW;
        const R* mns = smin + i * LW;
        const vec2<R> lo = ld2(a.lo + (t0 + i) * a.sN + n * LZ + k0);
        R out_p[2] = {R(0), R(0)}, out_m[2] = {R(0), R(0)};
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          const int k = k0 + l, z = k + 1;
          if (z < nzmin || z > nzmax - 1) continue;
          const R lov = l ? lo.y : lo.x;
          R bmax, bmin;
          if (z == nzmax - 1 || z == nzmin) {
            bmax = mxs[k] - lov;
            bmin = mns[k] - lov;
          } else {
            bmax = rmax(rmax(mxs[k - 1], mxs[k]), mxs[k + 1]) - lov;
            bmin = rmin(rmin(mns[k - 1], mns[k]), mns[k + 1]) - lov;
          }
          const R avk = l ? av.y : av.x;
          const R rdk = rdt_vol(dt, avk);
          R flux = dt_per_vol((l ? pl1[i] : pl0[i]), dt, avk, rdk) + R(1e-16);
          out_p[l] = rmin(R(1), fdiv(bmax, flux));
          flux = dt_per_vol((l ? mi1[i] : mi0[i]), dt, avk, rdk) - R(1e-16);
          out_m[l] = rmin(R(1), fdiv(bmin, flux));
        }
        st4(a.rpm + 2 * ((t0 + i) * a.sN + n * LZ + k0), out_p[0], out_m[0], out_p[1], out_m[1]);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// FCT stage 3: limiting b3 (lib/oce_adv_tra_fct.F90:396-471), flux divergence
// (oce_tra_adv_flux2dtracer with use_lo, lib/oce_adv_tra_driver.F90:298-450)
// and the caller's tendency update (src/fesom_analytic.F90:419-437 or, with a
// persistent del_ttf, lib/tracer_c_interface.F90:194-214).
// ---------------------------------------------------------------------------
template <typename R, int KC>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 8 : 4)) k_fct_update(DMesh m, StepPtrs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int vi = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nz = m.nz, nl = m.nl;
  unsigned char* base = smem_raw + (size_t)wib * warp_smem<R>(upd_slices(KC), m.LW, 0);
  R* sLv = reinterpret_cast<R*>(base);
  R* sRp = sLv + (size_t)KC * LW;
  R* sRm = sRp + (size_t)KC * LW;
  const NbrList nb = stage_nbrs(m, n, reinterpret_cast<Nbr*>(base + upd_slices(KC) * LW * sizeof(R)), lane);
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const R dt = a.dt;
  for (int t0 = 0; t0 < a.K; t0 += KC) {
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      const R* src = a.rpm + 2 * ((t0 + i) * a.sN + n * LZ);
      for (int k = lane; k < nz; k += kWarp) {
        sRp[i * LW + k] = src[2 * k];
        sRm[i * LW + k] = src[2 * k + 1];
      }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      const R* __restrict__ adfv = a.adfv + (t0 + i) * a.sW + n * LW;
      const R* Rp = sRp + i * LW;
      const R* Rm = sRm + i * LW;
      for (int iz = lane; iz < nl; iz += kWarp) {
        const int z = iz + 1;
        R f = adfv[iz];
        if (z == nzmin) {
          R ae = R(1);
          ae = (f >= R(0)) ? rmin(ae, Rp[iz]) : rmin(ae, Rm[iz]);
          f = ae * f;
        } else if (z > nzmin && z <= nzmax - 1) {
          R ae = R(1);
          if (f >= R(0)) {
            ae = rmin(ae, Rm[iz - 1]);
            ae = rmin(ae, Rp[iz]);
          } else {
            ae = rmin(ae, Rp[iz - 1]);
            ae = rmin(ae, Rm[iz]);
          }
          f = ae * f;
        }
        sLv[i * LW + iz] = f;
      }
    }
    __syncwarp();
    for (int p = lane; 2 * p < m.LZ; p += kWarp) {
      const int k0 = 2 * p, z0 = k0 + 1, z1 = k0 + 2;
      const vec2<R> av = ld2(g.areasvol + n * LZ + k0);
      const vec2<R> rd{rdt_vol(dt, av.x), rdt_vol(dt, av.y)};  // fast form only
      R dh0[KC], dh1[KC];
#pragma unroll
      for (int i = 0; i < KC; ++i) dh0[i] = dh1[i] = R(0);
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const Nbr q = nb.get(m, j);
        const bool a0 = z0 >= q.lo && z0 <= q.hi, a1 = z1 >= q.lo && z1 <= q.hi;
        const size_t o = (size_t)q.other * LZ + k0;
#pragma unroll
        for (int i = 0; i < KC; ++i) {
          const vec2<R> f = ld2(a.adfh + (t0 + i) * a.sE + (size_t)q.e * LZ + k0);
          const Q4<R> ro = ld4(a.rpm + 2 * ((t0 + i) * a.sN + o));
          const vec2<R> rpo{ro.a, ro.c}, rmo{ro.b, ro.d};
          const R rpn0 = sRp[i * LW + k0], rpn1 = sRp[i * LW + k0 + 1];
          const R rmn0 = sRm[i * LW + k0], rmn1 = sRm[i * LW + k0 + 1];
          R ae0 = R(1), ae1 = R(1);
          if (q.role) {  // this node is the edge's second node
            if (f.x >= R(0)) { ae0 = rmin(ae0, rpo.x); ae0 = rmin(ae0, rmn0); }
            else { ae0 = rmin(ae0, rmo.x); ae0 = rmin(ae0, rpn0); }
            if (f.y >= R(0)) { ae1 = rmin(ae1, rpo.y); ae1 = rmin(ae1, rmn1); }
            else { ae1 = rmin(ae1, rmo.y); ae1 = rmin(ae1, rpn1); }
            if (a0) dh0[i] = dh0[i] - dt_per_vol(ae0 * f.x, dt, av.x, rd.x);
            if (a1) dh1[i] = dh1[i] - dt_per_vol(ae1 * f.y, dt, av.y, rd.y);
          } else {
            if (f.x >= R(0)) { ae0 = rmin(ae0, rpn0); ae0 = rmin(ae0, rmo.x); }
            else { ae0 = rmin(ae0, rmn0); ae0 = rmin(ae0, rpo.x); }
            if (f.y >= R(0)) { ae1 = rmin(ae1, rpn1); ae1 = rmin(ae1, rmo.y); }
            else { ae1 = rmin(ae1, rmn1); ae1 = rmin(ae1, rpo.y); }
            if (a0) dh0[i] = dh0[i] + dt_per_vol(ae0 * f.x, dt, av.x, rd.x);
            if (a1) dh1[i] = dh1[i] + dt_per_vol(ae1 * f.y, dt, av.y, rd.y);
          }
        }
      }
      const vec2<R> hn = ld2(g.hnode + n * LZ + k0), hnn = ld2(g.hnode_new + n * LZ + k0);
      const bool w0 = z0 >= nzmin && z0 <= nzmax - 1, w1 = z1 >= nzmin && z1 <= nzmax - 1;
      const vec2<R> rh{FGB_FAST64 ? R(1) / hnn.x : R(0), FGB_FAST64 ? R(1) / hnn.y : R(0)};
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        R* __restrict__ T = a.T + (t0 + i) * a.sT + n * LZ + k0;
        const vec2<R> Tn = ld2(T);
        const vec2<R> lo = ld2(a.lo + (t0 + i) * a.sN + n * LZ + k0);
        const R* Lv = sLv + i * LW;
        R* del = a.del ? a.del + (t0 + i) * a.sN + n * LZ + k0 : nullptr;
        const vec2<R> d0 = del ? ld2(del) : vec2<R>{R(0), R(0)};
        R dv0 = (R(0) - Tn.x * hn.x) + lo.x * hnn.x;
        dv0 = dv0 + dt_per_vol(Lv[k0] - Lv[k0 + 1], dt, av.x, rd.x);
        R dv1 = (R(0) - Tn.y * hn.y) + lo.y * hnn.y;
        dv1 = dv1 + dt_per_vol(Lv[k0 + 1] - Lv[k0 + 2], dt, av.y, rd.y);
        const R e0 = d0.x + dh0[i] + dv0, e1 = d0.y + dh1[i] + dv1;
        R n0 = Tn.x, n1v = Tn.y;
        if constexpr (FGB_FAST64) {
          if (w0) n0 = Tn.x + e0 * rh.x;
          if (w1) n1v = Tn.y + e1 * rh.y;
        } else {
          if (w0) n0 = Tn.x + fdiv(e0, hnn.x);
          if (w1) n1v = Tn.y + fdiv(e1, hnn.y);
        }
        st2(T, n0, n1v);
        if (del) st2(del, w0 ? e0 : d0.x, w1 ? e1 : d0.y);
        if (a.TAout) {
          R* ta = a.TAout + (t0 + i) * a.sTA + n * LZ + k0;
          if (a.ab2) st2(ta, a.ab_old * Tn.x + a.ab_new * n0, a.ab_old * Tn.y + a.ab_new * n1v);
          else st2(ta, n0, n1v);
        }
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Without a limiter: vertical HO flux on T_AB with w_e, flux divergence
// (oce_tra_adv_flux2dtracer) and the tendency update in one pass.
// ---------------------------------------------------------------------------
template <typename R, int VER, int KC>
__global__ void __launch_bounds__(128, (sizeof(R) == 4 ? 8 : 4)) k_nofct_update(DMesh m, StepPtrs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kWarp - 1), wib = threadIdx.x / kWarp;
  const int vi = blockIdx.x * (blockDim.x / kWarp) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<R>& g = GeoSel<R>::get(m);
  const size_t LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  unsigned char* base = smem_raw + (size_t)wib * warp_smem<R>(nofct_slices(KC), m.LW, 0);
  R* sl = reinterpret_cast<R*>(base);
  R *sW = sl, *sA = sl + LW, *sHn = sl + 2 * LW, *sHnn = sl + 3 * LW, *sX = sl + 4 * LW, *sZ = sl + 5 * LW;
  R* sTA = sl + 7 * LW;              // KC columns
  R* sF = sTA + (size_t)KC * LW;     // KC columns
  R* sTv = sF + (size_t)KC * LW;     // KC columns
  const NbrList nb = stage_nbrs(m, n, reinterpret_cast<Nbr*>(base + nofct_slices(KC) * LW * sizeof(R)), lane);
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
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const R dt = a.dt;
  for (int t0 = 0; t0 < a.K; t0 += KC) {
#pragma unroll
    for (int i = 0; i < KC; ++i) stage(sTA + i * LW, a.TA + (t0 + i) * a.sTA + n * LZ, nz, lane);
    __syncwarp();
    if constexpr (VER == 3) {
      const Col<R> gc{nullptr, sW, sA, sHn, sHnn, sZ, sX, nullptr};
      column_ppm_multi<R, KC>(gc, sTA, sTv, nullptr, sF, (int)LW, nl, nzmin, nzmax, dt, lane);
    } else {
      for (int i = 0; i < KC; ++i) {
        Col<R> c{sTA + i * LW, sW, sA, sHn, sHnn, sZ, sX, nullptr};
        column_ver_flux<R, VER>(c, sTv + i * LW, nullptr, sF + i * LW, nl, nzmin, nzmax, a.pv, dt, lane);
      }
    }
    for (int p = lane; 2 * p < m.LZ; p += kWarp) {
      const int k0 = 2 * p, z0 = k0 + 1, z1 = k0 + 2;
      const vec2<R> av = ld2(g.areasvol + n * LZ + k0);
      const vec2<R> rd{rdt_vol(dt, av.x), rdt_vol(dt, av.y)};  // fast form only
      R dh0[KC], dh1[KC];
#pragma unroll
      for (int i = 0; i < KC; ++i) dh0[i] = dh1[i] = R(0);
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const Nbr q = nb.get(m, j);
        const bool a0 = z0 >= q.lo && z0 <= q.hi, a1 = z1 >= q.lo && z1 <= q.hi;
#pragma unroll
        for (int i = 0; i < KC; ++i) {
          const vec2<R> f = ld2(a.adfh + (t0 + i) * a.sE + (size_t)q.e * LZ + k0);
          if (q.role) {
            if (a0) dh0[i] = dh0[i] - dt_per_vol(f.x, dt, av.x, rd.x);
            if (a1) dh1[i] = dh1[i] - dt_per_vol(f.y, dt, av.y, rd.y);
          } else {
            if (a0) dh0[i] = dh0[i] + dt_per_vol(f.x, dt, av.x, rd.x);
            if (a1) dh1[i] = dh1[i] + dt_per_vol(f.y, dt, av.y, rd.y);
          }
        }
      }
      const vec2<R> hnn = ld2(g.hnode_new + n * LZ + k0);
      const bool w0 = z0 >= nzmin && z0 <= nzmax - 1, w1 = z1 >= nzmin && z1 <= nzmax - 1;
      const vec2<R> rh{FGB_FAST64 ? R(1) / hnn.x : R(0), FGB_FAST64 ? R(1) / hnn.y : R(0)};
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        const R* F = sF + i * LW;
        R* __restrict__ T = a.T + (t0 + i) * a.sT + n * LZ + k0;
        const vec2<R> Tn = ld2(T);
        R* del = a.del ? a.del + (t0 + i) * a.sN + n * LZ + k0 : nullptr;
        const vec2<R> d0 = del ? ld2(del) : vec2<R>{R(0), R(0)};
        const R dv0 = R(0) + dt_per_vol(F[k0] - F[k0 + 1], dt, av.x, rd.x);
        const R dv1 = R(0) + dt_per_vol(F[k0 + 1] - F[k0 + 2], dt, av.y, rd.y);
        const R e0 = d0.x + dh0[i] + dv0, e1 = d0.y + dh1[i] + dv1;
        R n0 = Tn.x, n1v = Tn.y;
        if constexpr (FGB_FAST64) {
          if (w0) n0 = Tn.x + e0 * rh.x;
          if (w1) n1v = Tn.y + e1 * rh.y;
        } else {
          if (w0) n0 = Tn.x + fdiv(e0, hnn.x);
          if (w1) n1v = Tn.y + fdiv(e1, hnn.y);
        }
        st2(T, n0, n1v);
        if (del) st2(del, w0 ? e0 : d0.x, w1 ? e1 : d0.y);
        if (a.TAout) {
          R* ta = a.TAout + (t0 + i) * a.sTA + n * LZ + k0;
          if (a.ab2) st2(ta, a.ab_old * Tn.x + a.ab_new * n0, a.ab_old * Tn.y + a.ab_new * n1v);
          else st2(ta, n0, n1v);
        }
      }
    }
    __syncwarp();
  }
}

}  // inline namespace
}  // namespace fgb
