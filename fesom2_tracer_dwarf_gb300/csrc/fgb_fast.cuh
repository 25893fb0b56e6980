// FP32 form of the tracer-advection step (do_oce_adv_tra,
// lib/oce_adv_tra_driver.F90:23-294, and the caller's tendency update) on the
// tracer-grouped layout.
//
// Layout: tracers are stored in groups of KV (1, 2 or 4) that are contiguous
// per node-layer: value (t, n, k) lives at
//   T[(t / KV) * strideT + (n * LZ + k) * KV + t % KV],
// so one 16-byte load brings the four tracers of a node-layer. The edge and
// node work arrays of the step use the same grouping. With KV = 1 this is the
// per-tracer layout of the FP64 form.
//
// Work decomposition: one warp per edge (edge fluxes) or per node column
// (node kernels); lane l handles layers l and l + 32 of each 64-layer pass,
// so every warp load is one contiguous row. What does not depend on the
// tracer is computed once per layer or interface and applied to the KV
// tracers of a group: the PPM and QR4C interface coefficients, the MUSCL
// edge weights (precomputed per edge at mesh upload), the upwind coefficients
// of the low-order edge fluxes and the dt / area factors of the flux
// divergence. Arithmetic is regrouped accordingly, so results agree with the
// reference order to FP32 rounding, not bit for bit. The active-layer tests of
// the edge gathers are dropped: the edge volume fluxes and the antidiffusive
// fluxes are stored as exact zeros outside an edge's layers, so those terms
// add zero; tracer values at stored layers below a node's bottom must
// therefore be finite.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "fgb_device.hpp"

namespace fgb {
namespace fast {

constexpr int kW = 32;
// Each kernel handles NS (1 or 2) layers per lane per pass: a warp covers
// 32 * NS layers of a column or edge per pass.
constexpr int kColChunk = 3 * kW;  // layers / interfaces per unrolled column round
constexpr int kMaxDegF = 16;            // incident edges staged per node
constexpr int kMaxClF = 24;             // cluster nodes staged per node

// ---------------------------------------------------------------------------
// KV tracer values of one node-layer (or edge-layer, or interface).
// ---------------------------------------------------------------------------
template <int KV>
struct alignas(4 * KV) V {
  float v[KV];
};

template <int KV>
__device__ __forceinline__ V<KV> ld(const float* __restrict__ base, unsigned i) {
  return reinterpret_cast<const V<KV>*>(base)[i];
}
template <int KV>
__device__ __forceinline__ void st(float* base, unsigned i, const V<KV>& a) {
  reinterpret_cast<V<KV>*>(base)[i] = a;
}
// The limiting factors R+ and R- of one node-layer are adjacent (the pair
// index i holds R+ at V index 2 i and R- at 2 i + 1): one load or store of
// 2 x 4 KV bytes. For four tracers that is a 32-byte access (ld/st .v8.f32,
// sm_100 and later; the workspace is 32-byte aligned), which halves the L1
// requests of the update kernel's gathers of its neighbours' factors.
template <int KV>
__device__ __forceinline__ void ld_pair(const float* __restrict__ base, unsigned i, V<KV>& p, V<KV>& q) {
  const V<KV>* a = reinterpret_cast<const V<KV>*>(base) + 2 * i;
  if constexpr (KV == 4) {
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(p.v[0]), "=f"(p.v[1]), "=f"(p.v[2]), "=f"(p.v[3]), "=f"(q.v[0]), "=f"(q.v[1]), "=f"(q.v[2]),
          "=f"(q.v[3])
        : "l"(a));
  } else if constexpr (KV == 2) {
    const float4 t = *reinterpret_cast<const float4*>(a);
    p.v[0] = t.x;
    p.v[1] = t.y;
    q.v[0] = t.z;
    q.v[1] = t.w;
  } else {
    const float2 t = *reinterpret_cast<const float2*>(a);
    p.v[0] = t.x;
    q.v[0] = t.y;
  }
}
template <int KV>
__device__ __forceinline__ void st_pair(float* base, unsigned i, const V<KV>& p, const V<KV>& q) {
  V<KV>* a = reinterpret_cast<V<KV>*>(base) + 2 * i;
  if constexpr (KV == 4) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(a), "f"(p.v[0]), "f"(p.v[1]),
                 "f"(p.v[2]), "f"(p.v[3]), "f"(q.v[0]), "f"(q.v[1]), "f"(q.v[2]), "f"(q.v[3])
                 : "memory");
  } else if constexpr (KV == 2) {
    *reinterpret_cast<float4*>(a) = make_float4(p.v[0], p.v[1], q.v[0], q.v[1]);
  } else {
    *reinterpret_cast<float2*>(a) = make_float2(p.v[0], q.v[0]);
  }
}

template <int KV>
__device__ __forceinline__ V<KV> splat(float s) {
  V<KV> r;
#pragma unroll
  for (int j = 0; j < KV; ++j) r.v[j] = s;
  return r;
}

// Element-wise arithmetic; pairs of tracers use the packed FP32x2 instructions.
#define FGB_F2(x, j) make_float2((x).v[j], (x).v[(j) + 1])
template <int KV>
__device__ __forceinline__ V<KV> add(const V<KV>& a, const V<KV>& b) {
  V<KV> r;
  if constexpr (KV % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KV; j += 2) {
      const float2 t = __fadd2_rn(FGB_F2(a, j), FGB_F2(b, j));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
    }
  } else {
    r.v[0] = __fadd_rn(a.v[0], b.v[0]);
  }
  return r;
}
template <int KV>
__device__ __forceinline__ V<KV> sub(const V<KV>& a, const V<KV>& b) {
  V<KV> r;
  if constexpr (KV % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KV; j += 2) {
      const float2 t = __fadd2_rn(FGB_F2(a, j), make_float2(-b.v[j], -b.v[j + 1]));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
    }
  } else {
    r.v[0] = __fsub_rn(a.v[0], b.v[0]);
  }
  return r;
}
template <int KV>
__device__ __forceinline__ V<KV> mul(const V<KV>& a, const V<KV>& b) {
  V<KV> r;
  if constexpr (KV % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KV; j += 2) {
      const float2 t = __fmul2_rn(FGB_F2(a, j), FGB_F2(b, j));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
    }
  } else {
    r.v[0] = __fmul_rn(a.v[0], b.v[0]);
  }
  return r;
}
// a * b + c
template <int KV>
__device__ __forceinline__ V<KV> fma(const V<KV>& a, const V<KV>& b, const V<KV>& c) {
  V<KV> r;
  if constexpr (KV % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KV; j += 2) {
      const float2 t = __ffma2_rn(FGB_F2(a, j), FGB_F2(b, j), FGB_F2(c, j));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
    }
  } else {
    r.v[0] = __fmaf_rn(a.v[0], b.v[0], c.v[0]);
  }
  return r;
}
// a * s + c with a scalar s
template <int KV>
__device__ __forceinline__ V<KV> fmas(const V<KV>& a, float s, const V<KV>& c) {
  return fma(a, splat<KV>(s), c);
}
template <int KV>
__device__ __forceinline__ V<KV> muls(const V<KV>& a, float s) {
  return mul(a, splat<KV>(s));
}
#undef FGB_F2

// Error-free addition (Knuth's TwoSum: six additions, exact for any order of
// magnitudes): s + x = s' + e exactly; s <- s', c <- c + e. Summing with it
// keeps each sum's rounding error in c, so a compensated sum (s, c) of FP32
// terms is exact to the rounding of c.
template <int KV>
__device__ __forceinline__ void two_sum(V<KV>& s, V<KV>& c, const V<KV>& x) {
  const V<KV> t = add(s, x);
  const V<KV> bp = sub(t, s);
  const V<KV> e = add(sub(s, sub(t, bp)), sub(x, bp));
  s = t;
  c = add(c, e);
}

// Division by the fast single-precision reciprocal (about 2 ulp); the FP32
// form's bar is a tolerance against FP64, not bit parity.
__device__ __forceinline__ float fdv(float a, float b) { return __fdividef(a, b); }

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// ---------------------------------------------------------------------------
// Volume flux through each edge segment (lib/oce_adv_tra_hor.F90:174,194,
// 215-216). With ulevels = 1 the segments reduce to: element 1 contributes at
// layers 1..nl1, element 2 at layers 1..nl2.
// ---------------------------------------------------------------------------
//
// Each warp handles 32 consecutive edges of the visit order: lane j loads the
// tables of edge j once, then the warp sweeps the edges' layers.
static __global__ void __launch_bounds__(256) kf_vflux(DMesh m, const float* __restrict__ vel, float* __restrict__ vf) {
  const int lane = threadIdx.x & (kW - 1);
  const int w0 = (blockIdx.x * (blockDim.x / kW) + (threadIdx.x / kW)) * kW;
  if (w0 >= m.E) return;
  const int cnt = min(kW, m.E - w0);
  const GeoPtrs<float>& g = m.g32;
  int e = 0, el1 = 0, el2 = 0, nl1 = 0, nl2 = 0;
  float4 cr = make_float4(0.f, 0.f, 0.f, 0.f);
  if (lane < cnt) {
    e = m.edge_order ? m.edge_order[w0 + lane] : w0 + lane;  // the edges of a node together: element reuse in L2
    el1 = m.edge_tri[2 * e];
    el2 = m.edge_tri[2 * e + 1];
    nl1 = m.edge_lev[4 * e + 1];
    nl2 = m.edge_lev[4 * e + 3];
    cr = reinterpret_cast<const float4*>(g.edge_cross)[e];
  }
  const unsigned LZ = m.LZ;
  const float2* __restrict__ uv = reinterpret_cast<const float2*>(vel);
  // two edges per round: the element loads of both are in flight together
  for (int i0 = 0; i0 < cnt; i0 += 2) {
    const int i1 = min(i0 + 1, cnt - 1);  // a repeat of the last edge when cnt is odd (same value stored)
    int ei[2], e1[2], e2[2], l1[2], l2[2];
    float dX1[2], dY1[2], dX2[2], dY2[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = q ? i1 : i0;
      ei[q] = __shfl_sync(0xffffffffu, e, i);
      e1[q] = __shfl_sync(0xffffffffu, el1, i);
      e2[q] = __shfl_sync(0xffffffffu, el2, i);
      l1[q] = __shfl_sync(0xffffffffu, nl1, i);
      l2[q] = __shfl_sync(0xffffffffu, nl2, i);
      dX1[q] = __shfl_sync(0xffffffffu, cr.x, i);
      dY1[q] = __shfl_sync(0xffffffffu, cr.y, i);
      dX2[q] = __shfl_sync(0xffffffffu, cr.z, i);
      dY2[q] = __shfl_sync(0xffffffffu, cr.w, i);
    }
    for (unsigned k = lane; k < LZ; k += kW) {
      const int z = (int)k + 1;
      float2 u1[2], u2[2];
      float h1[2], h2[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const bool a1 = z <= l1[q], a2 = z <= l2[q];
        u1[q] = a1 ? uv[e1[q] * LZ + k] : make_float2(0.f, 0.f);
        h1[q] = a1 ? g.helem[e1[q] * LZ + k] : 0.f;
        u2[q] = a2 ? uv[e2[q] * LZ + k] : make_float2(0.f, 0.f);
        h2[q] = a2 ? g.helem[e2[q] * LZ + k] : 0.f;
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float v = 0.f;
        if (z <= l1[q]) v = (-(u1[q].y * dX1[q]) + u1[q].x * dY1[q]) * h1[q];
        if (z <= l2[q]) v = v + (u2[q].y * dX2[q] - u2[q].x * dY2[q]) * h2[q];
        vf[ei[q] * LZ + k] = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Horizontal edge fluxes of all tracer groups (FCT: HO(T_AB) - LO(T), else
// HO). HOR: 0 UPW1 (lib/oce_adv_tra_hor.F90:218-220), 1 MUSCL
// (:454-497, with the nboundary_lay mask), 2 MFCT (:748-790).
//
// MUSCL reconstruction at node 1 with the upwind triangle's gradient g_u:
//   Tm1 = T1 + c1 * (2 (T2 - T1) + (dx, dy) . g_u) / 6
//       = T1 + c1 * ((T2 - T1) / 3 + sum_v w_v T_v),
// the weights w_v = ((dx, dy) . grad_sca_v) / 6 of the triangle's vertices
// taken from the per-edge table; likewise Tm2 from the downwind triangle.
// Layers outside the triangles' common window use the area-weighted mean
// gradient of the elements around each node (lib/oce_muscl_adv.F90:393-410).
// ---------------------------------------------------------------------------
template <int KV>
__device__ __forceinline__ void node_grad(const DMesh& m, const float* __restrict__ TA, int n, unsigned k,
                                          V<KV>& gx, V<KV>& gy) {
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ;
  const int z = (int)k + 1;
  float tvol = 0.f;
  V<KV> tx = splat<KV>(0.f), ty = splat<KV>(0.f);
  for (int j = m.nie_ptr[n]; j < m.nie_ptr[n + 1]; ++j) {
    const int el = m.nie_idx[j];
    if (m.elem_nlev[el] - 1 < z) continue;
    const int a = m.elem_nodes[3 * el], b = m.elem_nodes[3 * el + 1], c = m.elem_nodes[3 * el + 2];
    const float* gs = g.grad_sca + 6 * (size_t)el;
    const V<KV> ta = ld<KV>(TA, a * LZ + k), tb = ld<KV>(TA, b * LZ + k), tc = ld<KV>(TA, c * LZ + k);
    const V<KV> ex = fmas(tc, gs[2], fmas(tb, gs[1], muls(ta, gs[0])));
    const V<KV> ey = fmas(tc, gs[5], fmas(tb, gs[4], muls(ta, gs[3])));
    const float ar = g.elem_area[el];
    tvol += ar;
    tx = fmas(ex, ar, tx);
    ty = fmas(ey, ar, ty);
  }
  const float inv = fdv(1.f, tvol);
  gx = muls(tx, inv);
  gy = muls(ty, inv);
}

// Tables of one edge, filled by one lane and read by the whole warp.
struct alignas(16) EdgeRec {
  int e, n1, n2, hi;
  int gm0, gm1, nb1, nb2;
  float ex, ey, pad0, pad1;
  int4 tri;
  float4 wu, wd;
};

template <int HOR>
__device__ __forceinline__ void fill_edge(const DMesh& m, int w, EdgeRec& r) {
  const int e = m.edge_order ? m.edge_order[w] : w;
  r.e = e;
  r.n1 = m.edge_nodes[2 * e];
  r.n2 = m.edge_nodes[2 * e + 1];
  r.hi = max(m.edge_lev[4 * e + 1], m.edge_lev[4 * e + 3]);
  r.gm0 = -1;
  r.gm1 = -1;
  r.nb1 = r.nb2 = 0;
  r.ex = r.ey = r.pad0 = r.pad1 = 0.f;
  r.tri = make_int4(0, 0, 0, 0);
  r.wu = r.wd = make_float4(0.f, 0.f, 0.f, 0.f);
  if (HOR != 0) {
    r.gm0 = m.edge_gm[2 * e];
    r.gm1 = m.edge_gm[2 * e + 1];
    r.nb1 = m.nbl[r.n1];
    r.nb2 = m.nbl[r.n2];
    r.ex = m.g32.edge_dxa[2 * e];
    r.ey = m.g32.edge_dxa[2 * e + 1];
    if (r.gm0 >= 0) {
      r.tri = reinterpret_cast<const int4*>(m.f_tri)[e];
      r.wu = reinterpret_cast<const float4*>(m.f_wu)[e];
      r.wd = reinterpret_cast<const float4*>(m.f_wd)[e];
    }
  }
}

// Each warp handles 32 consecutive edges of the visit order: lane j fills the
// table record of edge j, then the warp computes the edges one after another.
template <int HOR, bool FCT, int KV, int NS>
__global__ void __launch_bounds__(256, (NS == 1 ? 3 : 2)) kf_hflux(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EdgeRec* recs = reinterpret_cast<EdgeRec*>(smem_raw) + (threadIdx.x / kW) * kW;  // this warp's 32 records
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int w0 = (blockIdx.x * (blockDim.x / kW) + wib) * kW;
  if (w0 >= m.E) return;
  const int cnt = min(kW, m.E - w0);
  if (lane < cnt) fill_edge<HOR>(m, w0 + lane, recs[lane]);
  __syncwarp();
  const unsigned LZ = m.LZ;
  const int nz = m.nz;
  for (int ie = 0; ie < cnt; ++ie) {
  const EdgeRec& rec = recs[ie];
  const int e = rec.e, n1 = rec.n1, n2 = rec.n2, hi = rec.hi;
  const int gm0 = rec.gm0, gm1 = rec.gm1, nb1 = rec.nb1, nb2 = rec.nb2;
  const float ex = rec.ex, ey = rec.ey;
  const int4 tri = rec.tri;
  const float4 wu = rec.wu, wd = rec.wd;
  const float A = 0.5f * (1.f - a.ph);
  const bool ta_sep = a.TA != a.T;
  for (unsigned base = 0; base < LZ; base += kW * NS) {
    unsigned kk[NS];
    bool in[NS], act[NS], tri_ok[NS];
    float vp[NS], vm[NS], B[NS], c1[NS], c2[NS];
    bool all_tri = true;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const unsigned k = base + lane + kW * i;
      in[i] = k < LZ;
      kk[i] = in[i] ? k : LZ - 1;
      const int z = (int)k + 1;
      act[i] = in[i] && (int)k < nz && z <= hi;
      const float v = a.vf[e * LZ + kk[i]];
      vp[i] = v + fabsf(v);
      vm[i] = v - fabsf(v);
      B[i] = (v * a.ph) * 0.5f;
      tri_ok[i] = gm0 >= 0 && z >= gm0 && z <= gm1 - 1;
      c1[i] = (HOR == 2 || nb1 - z >= 0) ? 1.f : 0.f;
      c2[i] = (HOR == 2 || nb2 - z >= 0) ? 1.f : 0.f;
      if (HOR != 0 && act[i] && !tri_ok[i]) all_tri = false;
    }
    const bool fast_tri = __all_sync(0xffffffffu, all_tri);
    for (int gi = 0; gi < a.G; ++gi) {
      const float* __restrict__ Tg = a.T + gi * a.gT;
      const float* __restrict__ TAg = ta_sep ? a.TA + gi * a.gTA : Tg;
      float* __restrict__ out = a.adfh + gi * a.gE;
      V<KV> s1[NS], s2[NS], r1[NS], r2[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        s1[i] = ld<KV>(TAg, n1 * LZ + kk[i]);
        s2[i] = ld<KV>(TAg, n2 * LZ + kk[i]);
        if (FCT && ta_sep) {
          r1[i] = ld<KV>(Tg, n1 * LZ + kk[i]);
          r2[i] = ld<KV>(Tg, n2 * LZ + kk[i]);
        } else {
          r1[i] = s1[i];
          r2[i] = s2[i];
        }
      }
      V<KV> h[NS];
      if (HOR == 0) {
#pragma unroll
        for (int i = 0; i < NS; ++i) h[i] = muls(fmas(s2[i], vm[i], muls(s1[i], vp[i])), -0.5f);
      } else {
        V<KV> tm1[NS], tm2[NS];
        if (fast_tri) {
          V<KV> u1[NS], u2[NS], d1[NS], d2[NS];
#pragma unroll
          for (int i = 0; i < NS; ++i) {
            u1[i] = ld<KV>(TAg, tri.x * LZ + kk[i]);
            u2[i] = ld<KV>(TAg, tri.y * LZ + kk[i]);
            d1[i] = ld<KV>(TAg, tri.z * LZ + kk[i]);
            d2[i] = ld<KV>(TAg, tri.w * LZ + kk[i]);
          }
#pragma unroll
          for (int i = 0; i < NS; ++i) {
            const V<KV> dT3 = muls(sub(s2[i], s1[i]), 1.f / 3.f);
            const V<KV> p1 = fmas(u2[i], wu.z, fmas(u1[i], wu.y, fmas(s1[i], wu.x, dT3)));
            const V<KV> p2 = fmas(d2[i], wd.z, fmas(d1[i], wd.y, fmas(s2[i], wd.x, dT3)));
            tm1[i] = fmas(p1, c1[i], s1[i]);
            tm2[i] = fmas(p2, -c2[i], s2[i]);
          }
        } else {
#pragma unroll
          for (int i = 0; i < NS; ++i) {
            const V<KV> dT3 = muls(sub(s2[i], s1[i]), 1.f / 3.f);
            V<KV> p1, p2;
            if (tri_ok[i]) {
              const V<KV> u1 = ld<KV>(TAg, tri.x * LZ + kk[i]), u2 = ld<KV>(TAg, tri.y * LZ + kk[i]);
              const V<KV> d1 = ld<KV>(TAg, tri.z * LZ + kk[i]), d2 = ld<KV>(TAg, tri.w * LZ + kk[i]);
              p1 = fmas(u2, wu.z, fmas(u1, wu.y, fmas(s1[i], wu.x, dT3)));
              p2 = fmas(d2, wd.z, fmas(d1, wd.y, fmas(s2[i], wd.x, dT3)));
            } else if (act[i]) {
              V<KV> gx, gy;
              node_grad<KV>(m, TAg, n1, kk[i], gx, gy);
              p1 = fmas(fmas(gy, ey, muls(gx, ex)), 1.f / 6.f, dT3);
              node_grad<KV>(m, TAg, n2, kk[i], gx, gy);
              p2 = fmas(fmas(gy, ey, muls(gx, ex)), 1.f / 6.f, dT3);
            } else {
              p1 = splat<KV>(0.f);
              p2 = p1;
            }
            tm1[i] = fmas(p1, c1[i], s1[i]);
            tm2[i] = fmas(p2, -c2[i], s2[i]);
          }
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          const V<KV> cho = fmas(tm2[i], vm[i], muls(tm1[i], vp[i]));
          h[i] = fmas(add(tm1[i], tm2[i]), -B[i], muls(cho, -A));
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        V<KV> r = h[i];
        if (FCT) r = fmas(fmas(r2[i], vm[i], muls(r1[i], vp[i])), 0.5f, r);
        if (!act[i]) r = splat<KV>(0.f);
        if (in[i]) st<KV>(out, e * LZ + kk[i], r);
      }
    }
  }
  }
}

// ---------------------------------------------------------------------------
// Column staging and vertical fluxes (lib/oce_adv_tra_ver.F90:248-712).
// ---------------------------------------------------------------------------
struct ColF {
  const float* W;
  const float* area;
  const float* hn;   // PPM
  const float* hnn;  // PPM
  const float* Z;    // QR4C
  const float* zb;   // QR4C
};

__device__ __forceinline__ void stage_f(float* dst, const float* __restrict__ src, int n, int lane) {
  for (int k = lane; k < n; k += kW) dst[k] = src[k];
}
template <int KV>
__device__ __forceinline__ void stage_v(V<KV>* dst, const float* __restrict__ src, unsigned first, int n, int lane) {
  for (int k = lane; k < n; k += kW) dst[k] = ld<KV>(src, first + k);
}

// PPM slope of layer j (0-based) from layers j-1, j, j+1, limited (the
// deltaj / deltaj+1 of lib/oce_adv_tra_ver.F90:525-545).
template <int KV>
__device__ __forceinline__ V<KV> ppm_slope(const V<KV>* T, const float* hnn, int j) {
  const float dzm = hnn[j - 1], dz = hnn[j], dzp = hnn[j + 1];
  const float f = fdv(dz, dzm + dz + dzp);
  const float s1 = f * fdv(2.f * dzm + dz, dzp + dz);
  const float s0 = f * fdv(dz + 2.f * dzp, dzm + dz);
  V<KV> r;
#pragma unroll
  for (int t = 0; t < KV; ++t) {
    const float d1 = T[j + 1].v[t] - T[j].v[t], d0 = T[j].v[t] - T[j - 1].v[t];
    const float s = s1 * d1 + s0 * d0;
    r.v[t] = (d1 * d0 > 0.f) ? copysignf(min3f(fabsf(s), 2.f * fabsf(d1), 2.f * fabsf(d0)), s) : 0.f;
  }
  return r;
}

// PPM edge value at interface z (1-based), lib/oce_adv_tra_ver.F90:510-594;
// the later assignment wins where the special cases coincide.
template <int KV>
__device__ __forceinline__ V<KV> ppm_edge(const V<KV>* T, const V<KV>* D, const ColF& c, int z, int nzmin,
                                          int nzmax) {
  if (z >= nzmin + 2 && z <= nzmax - 2) {
    const int j0 = z - 2;  // layer above the interface
    const float dzm = c.hnn[j0 - 1], dz = c.hnn[j0], dzp = c.hnn[j0 + 1], dzpp = c.hnn[j0 + 2];
    const float c0 = fdv(dz, dz + dzp);
    const float c1 = fdv((2.f * dzp) * dz, dz + dzp) * (fdv(dzm + dz, 2.f * dz + dzp) - fdv(dzpp + dzp, 2.f * dzp + dz));
    const float ci = fdv(1.f, dzm + dz + dzp + dzpp);
    const float P = c0 + ci * c1;
    const float Q2 = ci * fdv(dz * (dzm + dz), 2.f * dz + dzp);
    const float Q3 = ci * fdv(dzp * (dzp + dzpp), dz + 2.f * dzp);
    const V<KV> d = sub(T[j0 + 1], T[j0]);
    return fmas(D[j0], Q3, fmas(D[j0 + 1], -Q2, fmas(d, P, T[j0])));
  }
  if (z == nzmax) return T[nzmax - 2];
  if (z == nzmax - 1) {
    const float s = copysignf(1.f, c.W[nzmax - 2]);
    return fmas(T[nzmax - 2], fmaxf(s, 0.f), muls(T[nzmax - 3], -fminf(s, 0.f)));
  }
  if (z == nzmin + 1) return muls(add(T[nzmin - 1], T[nzmin]), 0.5f);
  return T[nzmin - 1];
}

// PPM flux of layer L (1-based) through its upper (W > 0) or lower (W < 0)
// interface, lib/oce_adv_tra_ver.F90:598-632; x = min(|W| dt / h, 1).
// Two tracers at once: the arithmetic in packed FP32x2 instructions, the
// limiter's tests and selects per tracer.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sel2(bool cx, bool cy, float2 a, float2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}
__device__ __forceinline__ float2 ppm_flux2(float2 aL, float2 aR, const float2 t0, float hx, float cx, bool upper,
                                            float aw) {
  const float2 pr = __fmul2_rn(__fadd2_rn(aR, neg2(t0)), __fadd2_rn(t0, neg2(aL)));
  aL = sel2(pr.x <= 0.f, pr.y <= 0.f, t0, aL);
  aR = sel2(pr.x <= 0.f, pr.y <= 0.f, t0, aR);
  const float2 t3 = __fmul2_rn(t0, make_float2(3.f, 3.f));
  const float2 sixth = make_float2(1.f / 6.f, 1.f / 6.f), mhalf = make_float2(-0.5f, -0.5f);
  float2 d = __fadd2_rn(aR, neg2(aL));
  float2 dm = __fmul2_rn(d, __ffma2_rn(__fadd2_rn(aL, aR), mhalf, t0));
  float2 dd = __fmul2_rn(__fmul2_rn(d, d), sixth);
  aL = sel2(dm.x > dd.x, dm.y > dd.y, __ffma2_rn(aR, make_float2(-2.f, -2.f), t3), aL);
  d = __fadd2_rn(aR, neg2(aL));
  dm = __fmul2_rn(d, __ffma2_rn(__fadd2_rn(aR, aL), mhalf, t0));
  dd = __fmul2_rn(__fmul2_rn(d, d), sixth);
  aR = sel2(dm.x < -dd.x, dm.y < -dd.y, __ffma2_rn(aL, make_float2(-2.f, -2.f), t3), aR);
  const float2 aj = __fmul2_rn(__ffma2_rn(__fadd2_rn(aL, aR), mhalf, t0), make_float2(6.f, 6.f));
  // upper: -aL - hx ((aR - aL) + cx aj); lower: -aR + hx ((aR - aL) - cx aj)
  const float p = upper ? cx : -cx, h = upper ? -hx : hx;
  const float2 q = __ffma2_rn(aj, make_float2(p, p), __fadd2_rn(aR, neg2(aL)));
  const float2 tv = __ffma2_rn(q, make_float2(h, h), neg2(upper ? aL : aR));
  return __fmul2_rn(tv, make_float2(aw, aw));
}

template <int KV>
__device__ __forceinline__ V<KV> ppm_flux(const V<KV>& aL0, const V<KV>& aR0, const V<KV>& T0, float x, bool upper,
                                          float aw) {
  const float hx = 0.5f * x, cx = 1.f - (2.f / 3.f) * x;
  V<KV> r;
  if constexpr (KV % 2 == 0) {
#pragma unroll
    for (int t = 0; t < KV; t += 2) {
      const float2 f = ppm_flux2(make_float2(aL0.v[t], aL0.v[t + 1]), make_float2(aR0.v[t], aR0.v[t + 1]),
                                 make_float2(T0.v[t], T0.v[t + 1]), hx, cx, upper, aw);
      r.v[t] = f.x;
      r.v[t + 1] = f.y;
    }
    return r;
  } else {
#pragma unroll
  for (int t = 0; t < KV; ++t) {
    float aL = aL0.v[t], aR = aR0.v[t];
    const float t0 = T0.v[t];
    if ((aR - t0) * (t0 - aL) <= 0.f) {
      aL = t0;
      aR = t0;
    }
    const float dd = (aR - aL) * (aR - aL) * (1.f / 6.f);
    if ((aR - aL) * (t0 - 0.5f * (aL + aR)) > dd) aL = 3.f * t0 - 2.f * aR;
    if ((aR - aL) * (t0 - 0.5f * (aR + aL)) < -((aR - aL) * (aR - aL) * (1.f / 6.f))) aR = 3.f * t0 - 2.f * aL;
    const float aj = 6.f * (t0 - 0.5f * (aL + aR));
    const float tv = upper ? -aL - hx * ((aR - aL) + cx * aj) : -aR + hx * ((aR - aL) - cx * aj);
    r.v[t] = tv * aw;
  }
  return r;
  }
}

// Vertical flux of the column at every interface into out[iz], minus fold[iz]
// (fold = nullptr: zero). VER: 0 UPW1, 1 QR4C, 2 CDIFF, 3 PPM. T holds the
// column's layers; D and TV are scratch columns for PPM.
// The bottom interface z = nl is never inside a column's stencil: its value
// is set by one lane, so a 64-layer column needs two passes of 32 lanes.
template <int VER, int KV>
__device__ void vert_flux(const ColF& c, const V<KV>* T, V<KV>* D, V<KV>* TV, const V<KV>* fold, V<KV>* out, int nl,
                          int nzmin, int nzmax, float num_ord, float dt, int lane) {
  const int last = nl - 1;
  if (VER == 3) {
    for (int j = lane; j < nl - 2; j += kW)
      if (j >= nzmin && j <= nzmax - 3) D[j] = ppm_slope<KV>(T, c.hnn, j);
    __syncwarp();
    for (int iz = lane; iz < last; iz += kW) {
      const int z = iz + 1;
      if (z >= nzmin && z <= nzmax) TV[iz] = ppm_edge<KV>(T, D, c, z, nzmin, nzmax);
    }
    if (lane == 0 && nzmax == nl) TV[last] = T[nzmax - 2];
    __syncwarp();
  }
  if (lane == 0) {
    // z = nl: the column's last interface (zero flux, CDIFF leaves it) or below the column
    const V<KV> f0 = fold ? fold[last] : splat<KV>(0.f);
    out[last] = (nzmax == nl && VER != 2) ? sub(splat<KV>(0.f), f0) : f0;
  }
  for (int iz = lane; iz < last; iz += kW) {
    const int z = iz + 1;
    const V<KV> f0 = fold ? fold[iz] : splat<KV>(0.f);
    V<KV> r = f0;
    if (z >= nzmin && z <= nzmax) {
      const float W = c.W[iz], ar = c.area[iz];
      if (VER == 0) {
        if (z == nzmin) r = sub(muls(T[z - 1], -(W * ar)), f0);
        else if (z == nzmax) r = sub(splat<KV>(0.f), f0);
        else
          r = sub(fmas(T[z - 2], -0.5f * (W - fabsf(W)) * ar, muls(T[z - 1], -0.5f * (W + fabsf(W)) * ar)), f0);
      } else if (VER == 1) {
        if (z == nzmin) {
          r = sub(muls(T[z - 1], -(W * ar)), f0);
        } else if (z == nzmax) {
          r = sub(splat<KV>(0.f), f0);
        } else if (z == nzmin + 1 || z == nzmax - 1) {
          const V<KV> x = muls(add(T[z - 2], T[z - 1]), -0.5f * W * ar);
          r = sub(x, f0);
          if (nzmin + 1 == nzmax - 1) r = sub(x, r);  // written twice (lib/oce_adv_tra_ver.F90:405-411)
        } else {
          const float Z0 = c.Z[z - 1], Zm1 = c.Z[z - 2], Zm2 = c.Z[z - 3], Zp1 = c.Z[z];
          const float ic = fdv(1.f, Zm1 - Z0), iu = fdv(1.f, Z0 - Zp1), idn = fdv(1.f, Zm2 - Zm1);
          const float zb = c.zb[z - 1];
          const float a1 = (zb - Z0) * (1.f / 3.f), a2 = (zb - Zm1) * (1.f / 3.f);
          const float wp = W + fabsf(W), wm = W - fabsf(W);
          const float cA = -(0.5f * (1.f - num_ord)) * ar, cB = -(num_ord * 0.5f) * W * ar;
          const V<KV> T0 = T[z - 1], Tm1 = T[z - 2], Tm2 = T[z - 3], Tp1 = T[z];
          const V<KV> qc = muls(sub(Tm1, T0), ic), qu = muls(sub(T0, Tp1), iu), qd = muls(sub(Tm2, Tm1), idn);
          const V<KV> tm1 = fmas(fmas(qc, 2.f, qu), a1, T0);
          const V<KV> tm2 = fmas(fmas(qc, 2.f, qd), a2, Tm1);
          const V<KV> tm = fmas(tm2, wm, muls(tm1, wp));
          r = sub(fmas(add(tm1, tm2), cB, muls(tm, cA)), f0);
        }
      } else if (VER == 2) {
        const int nzc = nzmax - 1;  // lib/oce_adv_tra_ver.F90:689
        if (z == nzmin) r = sub(muls(T[z - 1], -(W * ar)), f0);
        else if (z <= nzc) r = sub(muls(add(T[z - 2], T[z - 1]), -0.5f * W * ar), f0);
      } else {
        V<KV> tvert = splat<KV>(0.f);
        if (z == nzmin) {
          tvert = muls(TV[nzmin - 1], -(W * ar));
        } else if (z < nzmax && W != 0.f) {
          // the upwind layer's parabola: layer z (1-based) for W > 0, z - 1 for W < 0
          const bool up = W > 0.f;
          const int zl = up ? z - 1 : z - 2;
          const float x = fminf(fdv(fabsf(W) * dt, c.hn[zl]), 1.f);
          tvert = ppm_flux<KV>(TV[zl], TV[zl + 1], T[zl], x, up, ar * W);
        }
        r = sub(tvert, f0);
      }
    }
    out[iz] = r;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Node kernels: incident edges staged as (edge code, other node).
// ---------------------------------------------------------------------------
struct NbrF {
  const int2* s;
  int j0, deg;
  __device__ __forceinline__ int2 get(const DMesh& m, int j) const {
    return deg <= kMaxDegF ? s[j] : make_int2(m.ne_code[j0 + j], m.ne_other[j0 + j]);
  }
};
__device__ __forceinline__ NbrF stage_nbrs_f(const DMesh& m, int n, int2* s, int lane) {
  NbrF L{s, m.ne_ptr[n], m.ne_ptr[n + 1] - m.ne_ptr[n]};
  if (L.deg <= kMaxDegF)
    for (int j = lane; j < L.deg; j += kW) s[j] = make_int2(m.ne_code[L.j0 + j], m.ne_other[L.j0 + j]);
  return L;
}

// Shared memory of one warp: floats of the scalar columns, vectors, the edge
// list and the cluster list, each 16-byte aligned.
__host__ __device__ constexpr int al4(int v) { return (v + 3) / 4 * 4; }
template <int KV>
__host__ __device__ constexpr size_t warp_bytes(int scalar_cols, int vec_cols, int LW) {
  return (size_t)scalar_cols * al4(LW) * 4 + (size_t)vec_cols * LW * KV * 4 + kMaxDegF * sizeof(int2) +
         kMaxClF * sizeof(int2);
}
// Shared columns per warp (scalars, vectors) of each kernel, from the flags
// that decide which of them a launch needs.
struct LoCols {
  int scal, vec;
};
__host__ __device__ constexpr LoCols lo_cols(int ver, bool we_sep, bool ta_sep) {
  // W, area (+ WE) (+ hn, hnn for PPM) (+ Z, zbar for QR4C);
  // T, Flo, Fho/D, TV (+ TA)
  return LoCols{2 + (we_sep ? 1 : 0) + (ver == 3 ? 2 : 0) + (ver == 1 ? 2 : 0), 4 + (ta_sep ? 1 : 0)};
}
__host__ __device__ constexpr LoCols nofct_cols(int ver) {
  // W, area (+ hn, hnn) (+ Z, zbar); TA, F/D, TV
  return LoCols{2 + (ver == 3 ? 2 : 0) + (ver == 1 ? 2 : 0), 3};
}
constexpr int kRatioVec = 3, kUpdVec = 3;

struct WarpMem {
  unsigned char* p;
  __device__ float* f(int n) {
    float* r = reinterpret_cast<float*>(p);
    p += (size_t)al4(n) * 4;
    return r;
  }
  template <int KV>
  __device__ V<KV>* v(int n) {
    V<KV>* r = reinterpret_cast<V<KV>*>(p);
    p += (size_t)n * KV * 4;
    return r;
  }
};

template <int KV>
__device__ __forceinline__ V<KV> shfl_v(const V<KV>& x, int src) {
  V<KV> r;
#pragma unroll
  for (int t = 0; t < KV; ++t) r.v[t] = __shfl_sync(0xffffffffu, x.v[t], src);
  return r;
}

template <int KV>
struct PcrRow {
  float A, C;
  V<KV> D;
};

template <int KV>
__device__ __forceinline__ PcrRow<KV> pcr_shfl(const PcrRow<KV>& r, int src) {
  return PcrRow<KV>{__shfl_sync(0xffffffffu, r.A, src), __shfl_sync(0xffffffffu, r.C, src), shfl_v<KV>(r.D, src)};
}

template <int KV>
__device__ __forceinline__ void pcr_update(float& a, float& b, float& c, V<KV>& d, PcrRow<KV>& row, bool hm,
                                           const PcrRow<KV>& m, bool hp, const PcrRow<KV>& p) {
  const float Am = hm ? m.A : 0.f, Cm = hm ? m.C : 0.f, Ap = hp ? p.A : 0.f, Cp = hp ? p.C : 0.f;
  const float na = -a, nc = -c;
  b = fmaf(nc, Ap, fmaf(na, Cm, b));
  V<KV> dd = d;
  if (hm) dd = fmas(m.D, na, dd);
  if (hp) dd = fmas(p.D, nc, dd);
  d = dd;
  a = na * Am;
  c = nc * Cp;
  const float rb = fdv(1.f, b);
  row.A = a * rb;
  row.C = c * rb;
  row.D = muls(d, rb);
}

// Parallel cyclic reduction of one column held by a warp, rows lane and
// lane + 32 (a: coupling to the row above, b: diagonal, c: coupling to the row
// below, d: right-hand sides); rows outside the column are identity rows
// (a = c = d = 0, b = 1). Six steps couple rows 1, 2, 4, ..., 32 apart; d
// returns the solution.
template <int KV>
__device__ __forceinline__ void pcr_solve2(float av[2], float bv[2], float cv[2], V<KV> dv[2], int lane) {
  PcrRow<KV> row[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const float rb = fdv(1.f, bv[r]);
    row[r] = PcrRow<KV>{av[r] * rb, cv[r] * rb, muls(dv[r], rb)};
  }
#pragma unroll
  for (int h = 1; h < kW; h *= 2) {
    const int sm = (lane - h) & (kW - 1), sp = (lane + h) & (kW - 1);
    const PcrRow<KV> m0 = pcr_shfl(row[0], sm), m1 = pcr_shfl(row[1], sm);
    const PcrRow<KV> p0 = pcr_shfl(row[0], sp), p1 = pcr_shfl(row[1], sp);
    const bool lo_in = lane >= h, hi_in = lane + h < kW;
    // row lane: k - h from lane - h (row 0) if lane >= h; k + h from lane + h
    // (row 0) or, past 31, from lane + h - 32 (row 1)
    pcr_update(av[0], bv[0], cv[0], dv[0], row[0], lo_in, m0, true, hi_in ? p0 : p1);
    // row lane + 32: k - h from lane - h (row 1) or lane - h + 32 (row 0);
    // k + h from lane + h (row 1) while below 64
    pcr_update(av[1], bv[1], cv[1], dv[1], row[1], true, lo_in ? m1 : m0, hi_in, p1);
  }
  {  // h = 32: the two rows of a lane couple to each other
    const PcrRow<KV> r0 = row[0], r1 = row[1];
    pcr_update(av[0], bv[0], cv[0], dv[0], row[0], false, r0, true, r1);
    pcr_update(av[1], bv[1], cv[1], dv[1], row[1], true, r0, false, r1);
  }
  dv[0] = row[0].D;
  dv[1] = row[1].D;
}

// Row k of the implicit upwind system of w_split (lib/oce_adv_tra_ver.F90:
// 158-190) for a column with layers k0..k1 (0-based): a, b, c from wi at the
// row's two interfaces, the interface areas, areasvol and hnode_new.
__device__ __forceinline__ void vimpl_row(int k, int k0, int k1, float W0, float W1, float ar0, float ar1, float av,
                                          float hnn, float dt, float& a, float& b, float& c) {
  const float rav = fdv(dt, av);
  const float v0 = ar0 * rav, v1 = ar1 * rav;
  a = k == k0 ? 0.f : fminf(W0, 0.f) * v0;
  b = hnn + (k == k0 ? W0 : fmaxf(W0, 0.f)) * v0;
  c = 0.f;
  if (k != k1) {
    b -= fminf(W1, 0.f) * v1;
    c = -fmaxf(W1, 0.f) * v1;
  }
}

// ---------------------------------------------------------------------------
// FCT stage 1: low-order solution and vertical antidiffusive flux
// (lib/oce_adv_tra_driver.F90:91-235). The FP32 form stores the low-order
// solution as its increment LO - T (0 outside the column): rounding it to
// FP32 then costs a rounding of the small increment, not of the value, and
// the later stages add T back, which they read anyway. The low-order edge flux
// -(T1 (v + |v|) + T2 (v - |v|)) / 2 is exactly -v T_up with T_up the value
// at the upwind node; this node adds -v T_up (role 0, the edge's first node)
// or +v T_up (role 1), the same rounded product at both ends of the edge.
// ---------------------------------------------------------------------------
template <int VER, int KV, int NS, bool WSPLIT, bool COMP>
__global__ void __launch_bounds__(128, 7) kf_lo(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int vi = blockIdx.x * (blockDim.x / kW) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  const bool ta_sep = a.TA != a.T, we_sep = a.we != a.w;
  const LoCols cols = lo_cols(VER, we_sep, ta_sep);
  WarpMem wm{smem_raw + (size_t)wib * warp_bytes<KV>(cols.scal, cols.vec, LW)};
  float* sW = wm.f(LW);
  float* sA = wm.f(LW);
  float* sWE = we_sep ? wm.f(LW) : sW;
  float* sHn = VER == 3 ? wm.f(LW) : nullptr;
  float* sHnn = VER == 3 ? wm.f(LW) : nullptr;
  float* sZ = VER == 1 ? wm.f(LW) : nullptr;
  float* sZb = VER == 1 ? wm.f(LW) : nullptr;
  V<KV>* sT = wm.v<KV>(LW);
  V<KV>* sFlo = wm.v<KV>(LW);
  V<KV>* sD = wm.v<KV>(LW);  // PPM slopes, then the HO - LO fluxes
  V<KV>* sTV = wm.v<KV>(LW);
  V<KV>* sTA = ta_sep ? wm.v<KV>(LW) : sT;
  V<KV>* sFho = sD;
  const NbrF nb = stage_nbrs_f(m, n, reinterpret_cast<int2*>(wm.p), lane);
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const float dt = a.dt;
  const ColF clo{sWE, sA, sHn, sHnn, sZ, sZb};
  const ColF cho{sW, sA, sHn, sHnn, sZ, sZb};
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ Tg = a.T + gi * a.gT;
    const float* __restrict__ TAg = ta_sep ? a.TA + gi * a.gTA : Tg;
    // the column (geometry with the first group) in one round of loads
    for (int c0 = 0; c0 < (int)LW; c0 += kColChunk) {
      float w[3], we[3], ar[3], h1[3], h2[3], z1[3], z2[3];
      V<KV> t[3], ta[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int k = c0 + lane + kW * c;
        const int kw = k < nl ? k : nl - 1, kz = k < nz ? k : nz - 1, kt = k < (int)LZ ? k : LZ - 1;
        if (gi == 0) {
          w[c] = a.w[n * LW + kw];
          we[c] = we_sep ? a.we[n * LW + kw] : 0.f;
          ar[c] = g.area[n * LW + kw];
          h1[c] = VER == 3 ? g.hnode[n * LZ + kz] : 0.f;
          h2[c] = VER == 3 ? g.hnode_new[n * LZ + kz] : 0.f;
          z1[c] = VER == 1 ? g.Z3[n * LZ + kz] : 0.f;
          z2[c] = VER == 1 ? g.zbar3[n * LW + kw] : 0.f;
        }
        t[c] = ld<KV>(Tg, n * LZ + kt);
        ta[c] = ta_sep ? ld<KV>(TAg, n * LZ + kt) : t[c];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int k = c0 + lane + kW * c;
        if (gi == 0 && k < nl) {
          sW[k] = w[c];
          if (we_sep) sWE[k] = we[c];
          sA[k] = ar[c];
          if (VER == 1) sZb[k] = z2[c];
        }
        if (gi == 0 && k < nz) {
          if (VER == 3) {
            sHn[k] = h1[c];
            sHnn[k] = h2[c];
          }
          if (VER == 1) sZ[k] = z1[c];
        }
        if (k < (int)LZ) {
          sT[k] = t[c];
          if (ta_sep) sTA[k] = ta[c];
        }
      }
    }
    __syncwarp();
    // LO vertical flux: upwind on T with w_e; under w_split the antidiffusive
    // flux takes the upwind flux of the full w instead
    // (lib/oce_adv_tra_driver.F90:221-231).
    vert_flux<0, KV>(WSPLIT ? cho : clo, sT, nullptr, nullptr, nullptr, sFlo, nl, nzmin, nzmax, 1.f, dt, lane);
    // HO vertical flux on T_AB with w; adf_v = HO - LO.
    vert_flux<VER, KV>(cho, sTA, sD, sTV, sFlo, sFho, nl, nzmin, nzmax, a.pv, dt, lane);
    float* __restrict__ adfv = a.adfv + gi * a.gW;
    for (int iz = lane; iz < nl - 1; iz += kW) st<KV>(adfv, n * LW + iz, sFho[iz]);
    if (lane == 0) st<KV>(adfv, n * LW + nl - 1, sFho[nl - 1]);
    if (WSPLIT) vert_flux<0, KV>(clo, sT, nullptr, nullptr, nullptr, sFlo, nl, nzmin, nzmax, 1.f, dt, lane);
    float* __restrict__ lo = a.lo + gi * a.gN;
    for (unsigned base = 0; base < LZ; base += kW * NS) {
      unsigned kk[NS];
      bool in[NS];
      V<KV> acc[NS], accc[NS], tnk[NS];
      float hnv[NS], hnnv[NS], avv[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        in[i] = k < LZ;
        kk[i] = in[i] ? k : LZ - 1;
        acc[i] = splat<KV>(0.f);
        accc[i] = splat<KV>(0.f);
        tnk[i] = sT[kk[i]];
        hnv[i] = g.hnode[n * LZ + kk[i]];
        hnnv[i] = g.hnode_new[n * LZ + kk[i]];
        avv[i] = g.areasvol[n * LZ + kk[i]];
      }
#pragma unroll 3
      for (int j = 0; j < nb.deg; ++j) {
        const int2 q = nb.get(m, j);
        const unsigned ed = (unsigned)(q.x >> 1);
        const bool role = q.x & 1;
        float v[NS];
        V<KV> to[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          v[i] = a.vf[ed * LZ + kk[i]];
          to[i] = ld<KV>(Tg, q.y * LZ + kk[i]);
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          const bool own_up = (v[i] >= 0.f) != role;  // the flux leaves this node
          V<KV> tu;
#pragma unroll
          for (int c = 0; c < KV; ++c) tu.v[c] = own_up ? tnk[i].v[c] : to[i].v[c];
          const V<KV> p = muls(tu, v[i]);
          // with COMP the sum carries its rounding error (TwoSum)
          if (COMP) two_sum(acc[i], accc[i], role ? p : sub(splat<KV>(0.f), p));
          else acc[i] = role ? add(acc[i], p) : sub(acc[i], p);
        }
      }
      V<KV> lk[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        lk[i] = splat<KV>(0.f);
        if (!in[i]) continue;
        const unsigned k = kk[i];
        const int z = (int)k + 1;
        const V<KV> tn = tnk[i];
        V<KV> l = splat<KV>(0.f);  // the increment LO - T
        if (z >= nzmin && z <= nzmax - 1) {
          const float hn = hnv[i], hnn = hnnv[i], av = avv[i];
          const float ra = hn / hnn, rb = fdv(dt, av * hnn);  // ra IEEE: exactly 1 for an unchanged layer
          l = fmas(add(COMP ? add(acc[i], accc[i]) : acc[i], sub(sFlo[k], sFlo[k + 1])), rb, muls(tn, ra - 1.f));
        }
        if (WSPLIT && NS == 2 && a.wsplit_fused) lk[i] = l;
        else st<KV>(lo, n * LZ + k, l);
      }
      if constexpr (WSPLIT && NS == 2) {
        if (a.wsplit_fused) {
          // w_split: the implicit vertical step on the column just formed (one
          // pass holds all of it: at most 64 layers), by cyclic reduction
          const int k0 = nzmin - 1, k1 = nzmax - 2;
          float ac[2], bc[2], cc[2];
          V<KV> dv[2];
          bool act[2];
#pragma unroll
          for (int r = 0; r < 2; ++r) {
            const int k = (int)base + lane + kW * r;
            act[r] = k >= k0 && k <= k1;
            const int kq = act[r] ? k : k0, kq1 = kq < k1 ? kq + 1 : kq;
            float A_, B_, C_;
            vimpl_row(kq, k0, k1, a.wi[n * LW + kq], a.wi[n * LW + kq1], sA[kq], sA[kq1], avv[r], hnnv[r], dt, A_,
                      B_, C_);
            ac[r] = act[r] ? A_ : 0.f;
            bc[r] = act[r] ? B_ : 1.f;
            cc[r] = act[r] ? C_ : 0.f;
            dv[r] = act[r] ? muls(add(tnk[r], lk[r]), hnnv[r]) : splat<KV>(0.f);  // hnode_new LO
          }
          pcr_solve2<KV>(ac, bc, cc, dv, lane);
#pragma unroll
          for (int r = 0; r < 2; ++r) {
            const unsigned k = base + lane + kW * r;
            if (k < LZ) st<KV>(lo, n * LZ + k, act[r] ? sub(dv[r], tnk[r]) : lk[r]);
          }
        }
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// FCT stage 2: bounds a1-a3, antidiffusive sums b1 and limiting factors b2
// (lib/oce_adv_tra_fct.F90:98-374).
// ---------------------------------------------------------------------------
template <int KV, int NS, bool COMP>
__global__ void __launch_bounds__(128, (NS == 1 ? 10 : 7)) kf_ratio(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int vi = blockIdx.x * (blockDim.x / kW) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ, LW = m.LW;
  const int nl = m.nl;
  WarpMem wm{smem_raw + (size_t)wib * warp_bytes<KV>(0, kRatioVec, LW)};
  V<KV>*sAdv = wm.v<KV>(LW), *sMx = wm.v<KV>(LW), *sMn = wm.v<KV>(LW);
  int2* snb = reinterpret_cast<int2*>(wm.p);
  int2* scl = snb + kMaxDegF;
  const NbrF nb = stage_nbrs_f(m, n, snb, lane);
  const int c0 = m.cl_ptr[n], ncl = m.cl_ptr[n + 1] - c0, minlev = m.cl_minlev[n];
  const bool cl_staged = ncl <= kMaxClF;
  if (cl_staged)
    for (int j = lane; j < ncl; j += kW) scl[j] = make_int2(m.cl_node[c0 + j], m.cl_lev[c0 + j]);
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const float dt = a.dt;
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ Tg = a.T + gi * a.gT;
    const float* __restrict__ Lg = a.lo + gi * a.gN;
    const float* __restrict__ Fg = a.adfh + gi * a.gE;
    stage_v<KV>(sAdv, a.adfv + gi * a.gW, n * LW, nl, lane);
    __syncwarp();
    // cluster bounds per layer
    for (unsigned base = 0; base < LZ; base += kW * NS) {
      unsigned kk[NS];
      V<KV> mx[NS], mn[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        kk[i] = k < LZ ? k : LZ - 1;
        // AUX = -/+1e3 of elements without the layer (lib/oce_adv_tra_fct.F90:139-145)
        const float m0 = (int)k + 1 > minlev ? -1e3f : -INFINITY;
        mx[i] = splat<KV>(m0);
        mn[i] = splat<KV>(-m0);
      }
#pragma unroll (NS == 1 ? 8 : 4)
      for (int j = 0; j < ncl; ++j) {
        const int2 c = cl_staged ? scl[j] : make_int2(m.cl_node[c0 + j], m.cl_lev[c0 + j]);
        V<KV> lv[NS], tv[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          tv[i] = ld<KV>(Tg, c.x * LZ + kk[i]);
          lv[i] = add(tv[i], ld<KV>(Lg, c.x * LZ + kk[i]));  // LO = T + (LO - T)
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if ((int)(base + lane + kW * i) + 1 <= c.y) {
#pragma unroll
            for (int t = 0; t < KV; ++t) {
              mx[i].v[t] = max3f(mx[i].v[t], lv[i].v[t], tv[i].v[t]);
              mn[i].v[t] = min3f(mn[i].v[t], lv[i].v[t], tv[i].v[t]);
            }
          }
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        if (k < LZ) {
          sMx[k] = mx[i];
          sMn[k] = mn[i];
        }
      }
    }
    __syncwarp();
    float* __restrict__ Rg = a.rpm + 2 * gi * a.gN;
    for (unsigned base = 0; base < LZ; base += kW * NS) {
      unsigned kk[NS];
      V<KV> pl[NS], mi[NS], plc[NS], mic[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        kk[i] = k < LZ ? k : LZ - 1;
        const V<KV> ad0 = sAdv[kk[i]], ad1 = sAdv[kk[i] + 1];
#pragma unroll
        for (int t = 0; t < KV; ++t) {
          pl[i].v[t] = fmaxf(0.f, ad0.v[t]) + fmaxf(0.f, -ad1.v[t]);
          mi[i].v[t] = fminf(0.f, ad0.v[t]) + fminf(0.f, -ad1.v[t]);
        }
        plc[i] = splat<KV>(0.f);
        mic[i] = plc[i];
      }
#pragma unroll (NS == 1 ? 6 : 3)
      for (int j = 0; j < nb.deg; ++j) {
        const int2 q = nb.get(m, j);
        const unsigned ed = (unsigned)(q.x >> 1);
        const float sg = (q.x & 1) ? -1.f : 1.f;
        V<KV> f[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) f[i] = ld<KV>(Fg, ed * LZ + kk[i]);
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if (COMP) {
            V<KV> xp, xm;
#pragma unroll
            for (int t = 0; t < KV; ++t) {
              const float x = sg * f[i].v[t];
              xp.v[t] = fmaxf(0.f, x);
              xm.v[t] = fminf(0.f, x);
            }
            two_sum(pl[i], plc[i], xp);
            two_sum(mi[i], mic[i], xm);
          } else {
#pragma unroll
            for (int t = 0; t < KV; ++t) {
              const float x = sg * f[i].v[t];
              pl[i].v[t] += fmaxf(0.f, x);
              mi[i].v[t] += fminf(0.f, x);
            }
          }
        }
      }
      if (COMP) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          pl[i] = add(pl[i], plc[i]);
          mi[i] = add(mi[i], mic[i]);
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        if (k >= LZ) continue;
        const int z = (int)k + 1;
        V<KV> rp = splat<KV>(0.f), rm = rp;
        if (z >= nzmin && z <= nzmax - 1) {
          const float r = fdv(dt, g.areasvol[n * LZ + k]);
          const V<KV> lv = add(ld<KV>(Tg, n * LZ + k), ld<KV>(Lg, n * LZ + k));
          const bool edge = z == nzmax - 1 || z == nzmin;
#pragma unroll
          for (int t = 0; t < KV; ++t) {
            const float bmax = (edge ? sMx[k].v[t] : max3f(sMx[k - 1].v[t], sMx[k].v[t], sMx[k + 1].v[t])) - lv.v[t];
            const float bmin = (edge ? sMn[k].v[t] : min3f(sMn[k - 1].v[t], sMn[k].v[t], sMn[k + 1].v[t])) - lv.v[t];
            rp.v[t] = fminf(1.f, __fdividef(bmax, pl[i].v[t] * r + 1e-16f));
            rm.v[t] = fminf(1.f, __fdividef(bmin, mi[i].v[t] * r - 1e-16f));
          }
        }
        st_pair<KV>(Rg, n * LZ + k, rp, rm);
      }
    }
    __syncwarp();
  }
}

// Shared memory of one warp of kf_ratio64: bmax, bmin of the lane's two layers.
__host__ __device__ constexpr size_t ratio64_warp_bytes(int KV) { return (size_t)4 * kW * KV * 4; }

// Columns of at most 64 layers: one warp holds the whole column (lanes own
// layers l and l + 32), so the vertical bound window (layers k-1, k, k+1) comes
// from neighbouring lanes by shuffles and the kernel needs no shared memory;
// the edge and cluster lists are read through L1. Fewer resources per warp,
// more resident warps.

// LEAN: fewer registers (64, one cluster node and one incident edge in flight:
// with two edges in flight it spilled) for more resident warps.
// COMP: the +/- sums of the antidiffusive fluxes are compensated sums.
// Shared memory: ratio64_warp_bytes per warp, where the finished bounds wait.
template <int KV, bool LEAN, bool COMP>
__global__ void __launch_bounds__(128, LEAN ? 8 : 7) kf_ratio64(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1);
  const int vi = blockIdx.x * (blockDim.x / kW) + threadIdx.x / kW;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  V<KV>* sB = reinterpret_cast<V<KV>*>(smem_raw) + (size_t)(threadIdx.x / kW) * 4 * kW;
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ, LW = m.LW;
  const int j0 = m.ne_ptr[n], deg = m.ne_ptr[n + 1] - j0;
  const int c0 = m.cl_ptr[n], ncl = m.cl_ptr[n + 1] - c0, minlev = m.cl_minlev[n];
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const float dt = a.dt;
  // layers 32..63 are gathered only when the column reaches them; otherwise
  // their limiting factors are stored as zeros (neighbours read them)
  const bool s1 = nzmax - 2 >= kW;
  unsigned kk[2];
  int z[2];
  bool live[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const unsigned k = lane + kW * i;
    kk[i] = k < LZ ? k : LZ - 1;
    z[i] = (int)k + 1;
    live[i] = i == 0 || s1;
  }
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ Tg = a.T + gi * a.gT;
    const float* __restrict__ Lg = a.lo + gi * a.gN;
    const float* __restrict__ Fg = a.adfh + gi * a.gE;
    const float* __restrict__ adfv = a.adfv + gi * a.gW;
    // bounds a1-a3 over the cluster (lib/oce_adv_tra_fct.F90:105-184)
    V<KV> mx[2], mn[2], lo[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      // AUX = -/+1e3 of elements without the layer (lib/oce_adv_tra_fct.F90:139-145)
      const float m0 = z[i] > minlev ? -1e3f : -INFINITY;
      mx[i] = splat<KV>(m0);
      mn[i] = splat<KV>(-m0);
      lo[i] = live[i] ? add(ld<KV>(Tg, n * LZ + kk[i]), ld<KV>(Lg, n * LZ + kk[i])) : splat<KV>(0.f);  // LO = T + (LO - T)
    }
#pragma unroll(LEAN ? 1 : 2)
    for (int j = 0; j < ncl; ++j) {
      const int c = m.cl_node[c0 + j], lev = m.cl_lev[c0 + j];
      V<KV> lv[2], tv[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        tv[i] = live[i] ? ld<KV>(Tg, c * LZ + kk[i]) : splat<KV>(0.f);
        lv[i] = live[i] ? add(tv[i], ld<KV>(Lg, c * LZ + kk[i])) : tv[i];
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
        if (z[i] <= lev) {
#pragma unroll
          for (int t = 0; t < KV; ++t) {
            mx[i].v[t] = max3f(mx[i].v[t], lv[i].v[t], tv[i].v[t]);
            mn[i].v[t] = min3f(mn[i].v[t], lv[i].v[t], tv[i].v[t]);
          }
        }
    }
    // vertical window: layer k-1 from lane - 1 (lane 31 of the first slice for the
    // second), layer k+1 from lane + 1 (lane 0 of the second slice for the first)
    V<KV> bmax[2], bmin[2];
    {
      const int up = (lane + kW - 1) & (kW - 1), dn = (lane + 1) & (kW - 1);
      const bool first = lane == 0, last = lane == kW - 1;
      const bool edge0 = z[0] == nzmax - 1 || z[0] == nzmin, edge1 = z[1] == nzmax - 1 || z[1] == nzmin;
      {
        const V<KV> u0 = shfl_v(mx[0], up), u1 = shfl_v(mx[1], up), d0 = shfl_v(mx[0], dn), d1 = shfl_v(mx[1], dn);
#pragma unroll
        for (int t = 0; t < KV; ++t) {
          bmax[0].v[t] = (edge0 ? mx[0].v[t] : max3f(u0.v[t], mx[0].v[t], last ? d1.v[t] : d0.v[t])) - lo[0].v[t];
          bmax[1].v[t] = (edge1 ? mx[1].v[t] : max3f(first ? u0.v[t] : u1.v[t], mx[1].v[t], d1.v[t])) - lo[1].v[t];
        }
      }
      {
        const V<KV> u0 = shfl_v(mn[0], up), u1 = shfl_v(mn[1], up), d0 = shfl_v(mn[0], dn), d1 = shfl_v(mn[1], dn);
#pragma unroll
        for (int t = 0; t < KV; ++t) {
          bmin[0].v[t] = (edge0 ? mn[0].v[t] : min3f(u0.v[t], mn[0].v[t], last ? d1.v[t] : d0.v[t])) - lo[0].v[t];
          bmin[1].v[t] = (edge1 ? mn[1].v[t] : min3f(first ? u0.v[t] : u1.v[t], mn[1].v[t], d1.v[t])) - lo[1].v[t];
        }
      }
    }
    // the finished bounds wait in this lane's shared-memory slots while the
    // sums are formed (fewer live registers)
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      sB[i * kW + lane] = bmax[i];
      sB[(2 + i) * kW + lane] = bmin[i];
    }
    // antidiffusive sums b1 (lib/oce_adv_tra_fct.F90:255-346)
    V<KV> pl[2], mi[2], plc[2], mic[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const V<KV> ad0 = live[i] ? ld<KV>(adfv, n * LW + kk[i]) : splat<KV>(0.f);
      const V<KV> ad1 = live[i] ? ld<KV>(adfv, n * LW + kk[i] + 1) : splat<KV>(0.f);
#pragma unroll
      for (int t = 0; t < KV; ++t) {
        pl[i].v[t] = fmaxf(0.f, ad0.v[t]) + fmaxf(0.f, -ad1.v[t]);
        mi[i].v[t] = fminf(0.f, ad0.v[t]) + fminf(0.f, -ad1.v[t]);
      }
      plc[i] = splat<KV>(0.f);
      mic[i] = plc[i];
    }
#pragma unroll(LEAN ? 1 : 2)
    for (int j = 0; j < deg; ++j) {
      const int code = m.ne_code[j0 + j];
      const unsigned ed = (unsigned)(code >> 1);
      const float sg = (code & 1) ? -1.f : 1.f;
      V<KV> f[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) f[i] = live[i] ? ld<KV>(Fg, ed * LZ + kk[i]) : splat<KV>(0.f);
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (COMP) {
          V<KV> xp, xm;
#pragma unroll
          for (int t = 0; t < KV; ++t) {
            const float x = sg * f[i].v[t];
            xp.v[t] = fmaxf(0.f, x);
            xm.v[t] = fminf(0.f, x);
          }
          two_sum(pl[i], plc[i], xp);
          two_sum(mi[i], mic[i], xm);
        } else {
#pragma unroll
          for (int t = 0; t < KV; ++t) {
            const float x = sg * f[i].v[t];
            pl[i].v[t] += fmaxf(0.f, x);
            mi[i].v[t] += fminf(0.f, x);
          }
        }
      }
    }
    if (COMP) {
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        pl[i] = add(pl[i], plc[i]);
        mi[i] = add(mi[i], mic[i]);
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      bmax[i] = sB[i * kW + lane];
      bmin[i] = sB[(2 + i) * kW + lane];
    }
    // factors b2 (lib/oce_adv_tra_fct.F90:363-374)
    float* __restrict__ Rg = a.rpm + 2 * gi * a.gN;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const unsigned k = lane + kW * i;
      if (k >= LZ) continue;
      V<KV> rp = splat<KV>(0.f), rm = rp;
      if (z[i] >= nzmin && z[i] <= nzmax - 1) {
        const float r = fdv(dt, g.areasvol[n * LZ + k]);
#pragma unroll
        for (int t = 0; t < KV; ++t) {
          rp.v[t] = fminf(1.f, fdv(bmax[i].v[t], pl[i].v[t] * r + 1e-16f));
          rm.v[t] = fminf(1.f, fdv(bmin[i].v[t], mi[i].v[t] * r - 1e-16f));
        }
      }
      st_pair<KV>(Rg, n * LZ + k, rp, rm);
    }
  }
}

// ---------------------------------------------------------------------------
// FCT stage 3: limiting b3 (lib/oce_adv_tra_fct.F90:396-471), flux divergence
// (lib/oce_adv_tra_driver.F90:298-450) and the tendency update
// (src/fesom_analytic.F90:419-437; lib/tracer_c_interface.F90:194-214 with a
// persistent del_ttf). The limiting factors are at most 1, so min(1, a, b)
// is min(a, b).
// ---------------------------------------------------------------------------
template <int KV>
__device__ __forceinline__ V<KV> vsel_min(const V<KV>& f, const V<KV>& a_pos, const V<KV>& b_pos, const V<KV>& a_neg,
                                          const V<KV>& b_neg) {
  V<KV> r;
#pragma unroll
  for (int t = 0; t < KV; ++t)
    r.v[t] = f.v[t] >= 0.f ? fminf(a_pos.v[t], b_pos.v[t]) : fminf(a_neg.v[t], b_neg.v[t]);
  return r;
}

template <int KV>
__device__ __forceinline__ void finish_node(const DMesh& m, const FastPtrs& a, int gi, int n, unsigned k, int nzmin,
                                            int nzmax, const V<KV>& dh, const V<KV>& dvflux, const V<KV>* lo_or_null,
                                            bool fct) {
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ;
  float* __restrict__ T = a.T + gi * a.gT;
  const V<KV> Tn = ld<KV>(T, n * LZ + k);
  float* del = a.del ? a.del + gi * a.gN : nullptr;
  const V<KV> d0 = del ? ld<KV>(del, n * LZ + k) : splat<KV>(0.f);
  const int z = (int)k + 1;
  const bool act = z >= nzmin && z <= nzmax - 1;
  V<KV> tnew = Tn, enew = d0;
  if (act) {
    const float av = g.areasvol[n * LZ + k], hnn = g.hnode_new[n * LZ + k];
    const float r = fdv(a.dt, av);
    V<KV> dv;
    if (fct) {
      // -T hnode + LO hnode_new as hnode_new (LO - T hnode / hnode_new): exactly
      // zero when LO equals T and the layer keeps its thickness
      const float ra = g.hnode[n * LZ + k] / hnn;  // IEEE: exactly 1 for an unchanged layer
      dv = fmas(sub(*lo_or_null, muls(Tn, ra)), hnn, muls(dvflux, r));
    } else {
      dv = muls(dvflux, r);
    }
    enew = add(add(d0, muls(dh, r)), dv);
    tnew = fmas(enew, fdv(1.f, hnn), Tn);
  }
  st<KV>(T, n * LZ + k, tnew);
  if (del) st<KV>(del, n * LZ + k, enew);
  if (a.TAout) st<KV>(a.TAout + gi * a.gTA, n * LZ + k, a.ab2 ? fmas(Tn, a.ab_old, muls(tnew, a.ab_new)) : tnew);
}

// The kernel is written so that each node needs few dependent rounds of
// memory traffic: the node's own limiting factors and vertical fluxes arrive in
// one round (all layers at once), the values the final update needs are
// fetched together with the first neighbours, and three incident edges are in
// flight per round.
// DEL: a persistent del_ttf is read and written (the reference C interface).
// COMP: the limited edge fluxes are formed as one rounded product p = ae * f,
// the same number at both ends of the edge (+p at the first node, -p at the
// second), and summed with the vertical fluxes of the layer's two interfaces
// (each interface flux once with each sign) as a compensated sum, so the
// divergence cancels between neighbours to the last bit of the sum; without
// DEL the new value is then LO + T (1 - hnode/hnode_new) + S dt / (areasvol
// hnode_new), the update of the reference in exact arithmetic.
// RES (without DEL): each value carries its rounding residual in a.Tlo; the
// new value T + Tlo + increment is split exactly into its FP32 rounding and
// the new residual (TwoSum), so increments below half an FP32 unit of T --
// the rule, not the exception, where the flow is slow -- accumulate instead
// of being rounded away.
template <int KV, int NS, bool DEL, bool COMP, bool RES = false>
__global__ void __launch_bounds__(128, (NS == 1 ? (COMP || RES ? 8 : 9) : 4)) kf_update(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int vi = blockIdx.x * (blockDim.x / kW) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  WarpMem wm{smem_raw + (size_t)wib * warp_bytes<KV>(0, kUpdVec, LW)};
  V<KV>*sLv = wm.v<KV>(LW), *sRp = wm.v<KV>(LW), *sRm = wm.v<KV>(LW);
  const NbrF nb = stage_nbrs_f(m, n, reinterpret_cast<int2*>(wm.p), lane);
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const float dt = a.dt;
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ Rg = a.rpm + 2 * gi * a.gN;
    const float* __restrict__ Fg = a.adfh + gi * a.gE;
    const float* __restrict__ adfv = a.adfv + gi * a.gW;
    // own R+, R- (layers) and vertical antidiffusive fluxes (interfaces), all in one round
    for (int c0 = 0; c0 < nl; c0 += kColChunk) {
      V<KV> rp[3], rm[3], fv[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int k = c0 + lane + kW * c;
        const int kr = k < nz ? k : nz - 1, kv = k < nl ? k : nl - 1;
        const bool need = k <= nzmax - 1;  // layers and interfaces of the column (to its bottom)
        rp[c] = splat<KV>(0.f);
        rm[c] = rp[c];
        if (need) ld_pair<KV>(Rg, n * LZ + kr, rp[c], rm[c]);
        fv[c] = need ? ld<KV>(adfv, n * LW + kv) : splat<KV>(0.f);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int k = c0 + lane + kW * c;
        if (k < nz) {
          sRp[k] = rp[c];
          sRm[k] = rm[c];
        }
        if (k < nl) sLv[k] = fv[c];
      }
    }
    __syncwarp();
    for (int iz = lane; iz < nl; iz += kW) {
      const int z = iz + 1;
      V<KV> f = sLv[iz];
      if (z == nzmin) {
        f = mul(f, vsel_min(f, splat<KV>(1.f), sRp[iz], splat<KV>(1.f), sRm[iz]));
      } else if (z > nzmin && z <= nzmax - 1) {
        f = mul(f, vsel_min(f, sRm[iz - 1], sRp[iz], sRp[iz - 1], sRm[iz]));
      }
      sLv[iz] = f;
    }
    __syncwarp();
    const float* __restrict__ Lg = a.lo + gi * a.gN;
    float* __restrict__ Tg = a.T + gi * a.gT;
    float* del = DEL ? a.del + gi * a.gN : nullptr;
    // passes below the column's deepest layer change nothing: skipped; in the
    // last pass the lanes below the column load, compute and store nothing
    // (their values, and valuesAB there, keep what they hold)
    const unsigned lz_col = min(LZ, (unsigned)max(nzmax - 1, 1));
    for (unsigned base = 0; base < lz_col; base += kW * NS) {
      unsigned kk[NS];
      bool act[NS];
      V<KV> dh[NS], dc[NS], rpn[NS], rmn[NS], lo[NS], Tn[NS], d0[NS], tl[NS];
      float av[NS], hnn[NS], hn[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        kk[i] = k < LZ ? k : LZ - 1;
        act[i] = (int)k + 1 >= nzmin && (int)k + 1 <= nzmax - 1;  // the column's layers (k < nz <= LZ)
        const unsigned kr = kk[i] < (unsigned)nz ? kk[i] : (unsigned)nz - 1;
        dh[i] = splat<KV>(0.f);
        dc[i] = splat<KV>(0.f);
        rpn[i] = sRp[kr];
        rmn[i] = sRm[kr];
        // the final update's inputs travel with the first neighbours
        lo[i] = splat<KV>(0.f);
        Tn[i] = lo[i];
        d0[i] = lo[i];
        tl[i] = lo[i];
        av[i] = hnn[i] = hn[i] = 1.f;
        if (act[i]) {
          lo[i] = ld<KV>(Lg, n * LZ + kk[i]);
          Tn[i] = ld<KV>(Tg, n * LZ + kk[i]);
          if (DEL) d0[i] = ld<KV>(del, n * LZ + kk[i]);
          if (RES) tl[i] = ld<KV>(a.Tlo + gi * a.gT, n * LZ + kk[i]);
          av[i] = g.areasvol[n * LZ + kk[i]];
          hnn[i] = g.hnode_new[n * LZ + kk[i]];
          hn[i] = g.hnode[n * LZ + kk[i]];
        }
      }
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const int2 q = nb.get(m, j);
        const unsigned ed = (unsigned)(q.x >> 1);
        const bool role = q.x & 1;
        V<KV> f[NS], rpo[NS], rmo[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          f[i] = splat<KV>(0.f);
          rpo[i] = f[i];
          rmo[i] = f[i];
          if (act[i]) {
            f[i] = ld<KV>(Fg, ed * LZ + kk[i]);
            ld_pair<KV>(Rg, q.y * LZ + kk[i], rpo[i], rmo[i]);
          }
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          if (COMP) {
            // the same min of the same two factors at both ends: ae and p are equal there
            const V<KV> ae = role ? vsel_min(f[i], rpo[i], rmn[i], rmo[i], rpn[i])
                                  : vsel_min(f[i], rpn[i], rmo[i], rmn[i], rpo[i]);
            const V<KV> p = mul(ae, f[i]);
            two_sum(dh[i], dc[i], role ? sub(splat<KV>(0.f), p) : p);
          } else if (role) {  // this node is the edge's second node
            const V<KV> ae = vsel_min(f[i], rpo[i], rmn[i], rmo[i], rpn[i]);
            dh[i] = sub(dh[i], mul(ae, f[i]));
          } else {
            const V<KV> ae = vsel_min(f[i], rpn[i], rmo[i], rmn[i], rpo[i]);
            dh[i] = fma(ae, f[i], dh[i]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        if (!act[i]) continue;
        V<KV> tnew = Tn[i], enew = d0[i], tlnew = tl[i];
        {
          const float r = fdv(dt, av[i]);
          const float ra = hn[i] / hnn[i];  // IEEE: exactly 1 for an unchanged layer
          // lo holds LO - T, so LO - T hnode / hnode_new = (LO - T) + T (1 - ra),
          // exactly LO - T when the layer keeps its thickness
          const V<KV> dlo = fmas(Tn[i], 1.f - ra, lo[i]);
          V<KV> inc;  // the new value minus T
          if (COMP && !DEL) {
            // S = horizontal + vertical antidiffusive divergence, compensated
            two_sum(dh[i], dc[i], sLv[k]);
            two_sum(dh[i], dc[i], sub(splat<KV>(0.f), sLv[k + 1]));
            const float q = fdv(dt, av[i] * hnn[i]);
            inc = fmas(dh[i], q, fmas(dc[i], q, dlo));
          } else {
            if (COMP) dh[i] = add(dh[i], dc[i]);
            // -T hnode + LO hnode_new as hnode_new (LO - T hnode / hnode_new)
            const V<KV> dv = fmas(dlo, hnn[i], muls(sub(sLv[k], sLv[k + 1]), r));
            enew = add(add(d0[i], muls(dh[i], r)), dv);
            inc = muls(enew, fdv(1.f, hnn[i]));
          }
          if (RES) {
            // T + (Tlo + inc) = tnew + tlnew exactly
            const V<KV> b = add(tl[i], inc);
            tnew = add(Tn[i], b);
            const V<KV> bp = sub(tnew, Tn[i]);
            tlnew = add(sub(Tn[i], sub(tnew, bp)), sub(b, bp));
          } else {
            tnew = add(Tn[i], inc);
          }
        }
        st<KV>(Tg, n * LZ + k, tnew);
        if (RES) st<KV>(a.Tlo + gi * a.gT, n * LZ + k, tlnew);
        if (DEL) st<KV>(del, n * LZ + k, enew);
        if (a.TAout)
          st<KV>(a.TAout + gi * a.gTA, n * LZ + k, a.ab2 ? fmas(Tn[i], a.ab_old, muls(tnew, a.ab_new)) : tnew);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Without a limiter: vertical HO flux on T_AB with w_e, flux divergence and
// the tendency update in one pass.
// ---------------------------------------------------------------------------
template <int VER, int KV, int NS>
__global__ void __launch_bounds__(128, 8) kf_nofct(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int vi = blockIdx.x * (blockDim.x / kW) + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const GeoPtrs<float>& g = m.g32;
  const unsigned LZ = m.LZ, LW = m.LW;
  const int nl = m.nl, nz = m.nz;
  const LoCols cols = nofct_cols(VER);
  WarpMem wm{smem_raw + (size_t)wib * warp_bytes<KV>(cols.scal, cols.vec, LW)};
  float* sW = wm.f(LW);
  float* sA = wm.f(LW);
  float* sHn = VER == 3 ? wm.f(LW) : nullptr;
  float* sHnn = VER == 3 ? wm.f(LW) : nullptr;
  float* sZ = VER == 1 ? wm.f(LW) : nullptr;
  float* sZb = VER == 1 ? wm.f(LW) : nullptr;
  V<KV>* sTA = wm.v<KV>(LW);
  V<KV>* sD = wm.v<KV>(LW);  // PPM slopes, then the fluxes
  V<KV>* sTV = wm.v<KV>(LW);
  V<KV>* sF = sD;
  const NbrF nb = stage_nbrs_f(m, n, reinterpret_cast<int2*>(wm.p), lane);
  stage_f(sW, a.we + n * LW, nl, lane);
  stage_f(sA, g.area + n * LW, nl, lane);
  if (VER == 3) {
    stage_f(sHn, g.hnode + n * LZ, nz, lane);
    stage_f(sHnn, g.hnode_new + n * LZ, nz, lane);
  }
  if (VER == 1) {
    stage_f(sZ, g.Z3 + n * LZ, nz, lane);
    stage_f(sZb, g.zbar3 + n * LW, nl, lane);
  }
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];
  const ColF c{sW, sA, sHn, sHnn, sZ, sZb};
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ TAg = a.TA + gi * a.gTA;
    const float* __restrict__ Fg = a.adfh + gi * a.gE;
    stage_v<KV>(sTA, TAg, n * LZ, nz, lane);
    __syncwarp();
    vert_flux<VER, KV>(c, sTA, sD, sTV, nullptr, sF, nl, nzmin, nzmax, a.pv, a.dt, lane);
    for (unsigned base = 0; base < LZ; base += kW * NS) {
      unsigned kk[NS];
      V<KV> dh[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        kk[i] = k < LZ ? k : LZ - 1;
        dh[i] = splat<KV>(0.f);
      }
#pragma unroll 2
      for (int j = 0; j < nb.deg; ++j) {
        const int2 q = nb.get(m, j);
        const unsigned ed = (unsigned)(q.x >> 1);
        const bool role = q.x & 1;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
          const V<KV> f = ld<KV>(Fg, ed * LZ + kk[i]);
          dh[i] = role ? sub(dh[i], f) : add(dh[i], f);
        }
      }
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        const unsigned k = base + lane + kW * i;
        if (k >= LZ) continue;
        finish_node<KV>(m, a, gi, n, k, nzmin, nzmax, dh[i], sub(sF[k], sF[k + 1]), nullptr, false);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// w_split: implicit vertical advection of the low-order solution with wi
// (adv_tra_vert_impl, lib/oce_adv_tra_ver.F90:90-244), in place, between the
// LO and ratio kernels. Per column the system A y = hnode_new * LO over the
// layers nzmin..nzmax-1 is solved for the new values y directly (the
// reference solves A x = -(A - diag(hnode_new)) LO for the increment x = y - LO;
// the two agree to rounding).
//
// One lane per (node, tracer of the group): a warp holds 32 / KV node
// columns, so the serial Thomas sweeps run on all 32 lanes. The coefficients
// (per node) and the right-hand sides (per lane) are formed layer-parallel
// and staged in shared memory, transposed so that the sweeps read one row of
// consecutive words per layer; the KV lanes of a node repeat the
// tracer-independent pivots in parallel.
// ---------------------------------------------------------------------------
template <int KV>
__global__ void __launch_bounds__(kVimplWarpsF * kW) kf_vert_impl(DMesh m, FastPtrs a) {
  using S = VimplShape<KV>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int n0 = (blockIdx.x * kVimplWarpsF + wib) * S::NPW;
  if (n0 >= m.N) return;
  const int LZ = m.LZ, LW = m.LW;
  const int nn = m.N - n0 < S::NPW ? m.N - n0 : S::NPW;  // columns of this warp
  float* sY = reinterpret_cast<float*>(smem_raw) + (size_t)wib * S::warp_floats(LZ);  // (LZ, RS)
  float* sA = sY + (size_t)LZ * S::RS;                                                // (LZ, CS) each
  float* sB = sA + (size_t)LZ * S::CS;
  float* sC = sB + (size_t)LZ * S::CS;
  float* sCP = sC + (size_t)LZ * S::CS;
  const GeoPtrs<float>& g = m.g32;
  const float dt = a.dt;
  // Tridiagonal coefficients per node and layer (lib/oce_adv_tra_ver.F90:
  // 158-190). Every row is loaded and stored (rows outside a column are
  // never read), so the loads of several iterations are in flight together.
#pragma unroll 8
  for (int i = lane; i < nn * LZ; i += kW) {
    const int j = i / LZ, k = i - j * LZ, n = n0 + j;
    const int k0 = m.ulev[n] - 1, k1 = m.nlev[n] - 2;
    const unsigned iw = (unsigned)n * LW + k, iz = (unsigned)n * LZ + k;
    const unsigned iw1 = iw + (k + 1 < LW ? 1u : 0u);
    const float W0 = a.wi[iw], W1 = a.wi[iw1], ar0 = g.area[iw], ar1 = g.area[iw1];
    const float rav = fdv(dt, g.areasvol[iz]), hnn = g.hnode_new[iz];
    const float v0 = ar0 * rav, v1 = ar1 * rav;
    const float ak = k == k0 ? 0.f : fminf(W0, 0.f) * v0;
    float bk = hnn + (k == k0 ? W0 : fmaxf(W0, 0.f)) * v0, ck = 0.f;
    if (k != k1) {
      bk -= fminf(W1, 0.f) * v1;
      ck = -fmaxf(W1, 0.f) * v1;
    }
    sA[k * S::CS + j] = ak;
    sB[k * S::CS + j] = bk;
    sC[k * S::CS + j] = ck;
  }
  const int j = lane / KV;
  const bool own = j < nn;
  const int k0 = own ? m.ulev[n0 + j] - 1 : 0, k1 = own ? m.nlev[n0 + j] - 2 : -1;
  for (int gi = 0; gi < a.G; ++gi) {
    float* __restrict__ lo = a.lo + gi * a.gN;
    __syncwarp();
    // right-hand sides hnode_new * LO, rows of consecutive node-layers
#pragma unroll 8
    for (int i = lane; i < nn * LZ; i += kW) {
      const int jj = i / LZ, k = i - jj * LZ;
      const unsigned iz = (unsigned)(n0 + jj) * LZ + k;
      *reinterpret_cast<V<KV>*>(sY + k * S::RS + jj * KV) =
          muls(add(ld<KV>(a.T + gi * a.gT, iz), ld<KV>(lo, iz)), g.hnode_new[iz]);  // hnode_new (T + (LO - T))
    }
    __syncwarp();
    if (own) {
      // forward sweep: pivots m = b - cp * a, cp = c / m, tp = (d - tp * a) / m
      float cp = 0.f, tp = 0.f;
#pragma unroll 4
      for (int k = k0; k <= k1; ++k) {
        const float ak = sA[k * S::CS + j];
        const float rm = fdv(1.f, sB[k * S::CS + j] - cp * ak);
        cp = sC[k * S::CS + j] * rm;
        tp = (sY[k * S::RS + lane] - tp * ak) * rm;
        sY[k * S::RS + lane] = tp;
        if (lane % KV == 0) sCP[k * S::CS + j] = cp;
      }
    }
    __syncwarp();
    if (own) {
      // back substitution: y = tp - cp * y(below)
      float y = sY[k1 * S::RS + lane];
#pragma unroll 4
      for (int k = k1 - 1; k >= k0; --k) {
        y = sY[k * S::RS + lane] - sCP[k * S::CS + j] * y;
        sY[k * S::RS + lane] = y;
      }
    }
    __syncwarp();
#pragma unroll 4
    for (int i = lane; i < nn * LZ; i += kW) {
      const int jj = i / LZ, k = i - jj * LZ, n = n0 + jj;
      if (k >= m.ulev[n] - 1 && k <= m.nlev[n] - 2)
        st<KV>(lo, (unsigned)n * LZ + k,
               sub(*reinterpret_cast<const V<KV>*>(sY + k * S::RS + jj * KV), ld<KV>(a.T + gi * a.gT, (unsigned)n * LZ + k)));
    }
  }
}

// The same solve for columns of at most 64 layers: one warp per node, rows
// k = lane and lane + 32 in registers, parallel cyclic reduction (six steps
// coupling rows 1, 2, 4, ..., 32 apart; stable for these diagonally dominant
// systems). No shared memory, all 32 lanes busy. Each row carries its scaled
// couplings A = a / b, C = c / b and D = d / b; a step with distance h forms
//   a' = -a A(k-h), c' = -c C(k+h), b' = b - a C(k-h) - c A(k+h),
//   d' = d - a D(k-h) - c D(k+h),
// rows outside the column being identity rows (a = c = d = 0, b = 1); after
// the last step D is the solution.
template <int KV>
__global__ void __launch_bounds__(256) kf_vert_pcr(DMesh m, FastPtrs a) {
  const int lane = threadIdx.x & (kW - 1);
  const int vi = blockIdx.x * (blockDim.x / kW) + threadIdx.x / kW;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const unsigned LZ = m.LZ, LW = m.LW;
  const int k0 = m.ulev[n] - 1, k1 = m.nlev[n] - 2;
  const GeoPtrs<float>& g = m.g32;
  // coefficients of rows lane and lane + 32 (rows outside the column: identity)
  float a0[2], b0[2], c0[2], hn[2];
  bool act[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int k = lane + kW * r;
    act[r] = k >= k0 && k <= k1;
    const int kk = act[r] ? k : k0;
    const unsigned iw = (unsigned)n * LW + kk, iz = (unsigned)n * LZ + kk;
    const unsigned iw1 = iw + (kk < k1 ? 1u : 0u);
    float ak, bk, ck;
    vimpl_row(kk, k0, k1, a.wi[iw], a.wi[iw1], g.area[iw], g.area[iw1], g.areasvol[iz], g.hnode_new[iz], a.dt, ak,
              bk, ck);
    a0[r] = act[r] ? ak : 0.f;
    b0[r] = act[r] ? bk : 1.f;
    c0[r] = act[r] ? ck : 0.f;
    hn[r] = act[r] ? g.hnode_new[iz] : 0.f;
  }
  for (int gi = 0; gi < a.G; ++gi) {
    float* __restrict__ lo = a.lo + gi * a.gN;
    float av[2] = {a0[0], a0[1]}, bv[2] = {b0[0], b0[1]}, cv[2] = {c0[0], c0[1]};
    V<KV> dv[2];
#pragma unroll
    for (int r = 0; r < 2; ++r)
      dv[r] = act[r] ? muls(add(ld<KV>(a.T + gi * a.gT, (unsigned)n * LZ + lane + kW * r),
                                ld<KV>(lo, (unsigned)n * LZ + lane + kW * r)), hn[r])
                     : splat<KV>(0.f);  // hnode_new (T + (LO - T))
    pcr_solve2<KV>(av, bv, cv, dv, lane);
#pragma unroll
    for (int r = 0; r < 2; ++r)
      if (act[r])
        st<KV>(lo, (unsigned)n * LZ + lane + kW * r, sub(dv[r], ld<KV>(a.T + gi * a.gT, (unsigned)n * LZ + lane + kW * r)));
  }
}

}  // namespace fast
}  // namespace fgb
