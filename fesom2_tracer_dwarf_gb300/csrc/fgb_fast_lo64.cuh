// FCT stage 1 of the FP32 form for columns of at most 64 layers: the
// low-order solution and the vertical antidiffusive flux
// (lib/oce_adv_tra_driver.F90:91-235 with the vertical schemes of
// lib/oce_adv_tra_ver.F90:248-712), the same results as kf_lo to FP32
// rounding with fewer instructions per column.
//
// One warp per node column; lane l owns layers l and l + 32 (slices s = 0, 1)
// and the interfaces above them, so every index is formed once per launch
// and no access needs clamping. The tracer-independent work is done once per
// layer or interface and applied to the KV tracers of a group: the PPM edge
// value of an interface takes four reciprocals (the seven quotients of the
// reference share denominators), a slope two, and the low-order factors
// T hnode / hnode_new and dt / (areasvol hnode_new) one each. Stencils read
// the column from shared memory, one round per phase. The LO workspace holds
// the increment LO - T (the FP32 form's convention, see kf_lo).
#pragma once
#include <cuda_runtime.h>

#include "fgb_fast.cuh"

namespace fgb {
namespace fast {

constexpr int kLo64Warps = 4;  // node columns per block

__device__ __forceinline__ float frcp(float x) { return __fdividef(1.f, x); }

// Shared memory of one warp (bytes), 16-byte aligned pieces: T (64), T_AB
// (64, separate T_AB), PPM slopes (64) and edge values (68), LO vertical
// fluxes (68), PPM layer thicknesses hnode_new and hnode (64 each), QR4C
// Z_3d_n (64) and zbar_3d_n (68), the low-order update factors ra and rb
// (64 each), the incident-edge list.
__host__ __device__ constexpr size_t lo64_warp_bytes(int KV, int ver, bool tasep) {
  return (size_t)KV * 4 * (64 + (tasep ? 64 : 0) + (ver == 3 ? 64 + 68 : 0) + 68) +
         (ver == 3 ? 2 * 64 * 4 : 0) + (ver == 1 ? (64 + 68) * 4 : 0) + 2 * 64 * 4 + kMaxDegF * sizeof(int2);
}

template <int VER, int KV, bool TASEP, bool WESEP, bool COMP>
__global__ void __launch_bounds__(kLo64Warps * kW, 7) kf_lo64(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & (kW - 1), wib = threadIdx.x / kW;
  const int vi = blockIdx.x * kLo64Warps + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  unsigned char* wp = smem_raw + (size_t)wib * lo64_warp_bytes(KV, VER, TASEP);
  V<KV>* sT = reinterpret_cast<V<KV>*>(wp);
  V<KV>* sTA = TASEP ? sT + 64 : sT;
  V<KV>* sD = (TASEP ? sTA : sT) + 64;            // PPM slopes
  V<KV>* sTV = VER == 3 ? sD + 64 : sD;           // PPM edge values
  V<KV>* sF = VER == 3 ? sTV + 68 : sD;           // LO vertical fluxes
  float* sHnn = reinterpret_cast<float*>(sF + 68);  // PPM
  float* sHn = sHnn + (VER == 3 ? 64 : 0);
  float* sZ = sHn + (VER == 3 ? 64 : 0);            // QR4C
  float* sZb = sZ + (VER == 1 ? 64 : 0);
  float* sRa = sZb + (VER == 1 ? 68 : 0);
  float* sRb = sRa + 64;
  int2* sNb = reinterpret_cast<int2*>(sRb + 64);
  const GeoPtrs<float>& g = m.g32;
  const int LZ = m.LZ, LW = m.LW, nl = m.nl;
  const int nzmin = m.ulev[n], nzmax = m.nlev[n];  // 1-based, as the reference
  const int e0 = m.ne_ptr[n], deg = m.ne_ptr[n + 1] - e0;
  const bool nb_staged = deg <= kMaxDegF;
  if (nb_staged && lane < deg) sNb[lane] = make_int2(m.ne_code[e0 + lane], m.ne_other[e0 + lane]);
  const float dt = a.dt;
  // The second slice (layers 32..63) is skipped when the column ends above it
  // (its deepest layer, 0-based nzmax - 2, is above layer 32): no loads, no
  // arithmetic; its interface fluxes are zero (still written: the bottom
  // interface is read by the update) and its LO increments are never read.
  const bool s1 = nzmax - 2 >= kW;
  // per slice: layer / interface index, geometry and velocity (tracer independent)
  int k[2];
  bool lay[2], itf[2];
  float hn[2], hnn[2], av[2], w[2], wl[2], ar[2], zq[2], zbq[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    k[s] = lane + kW * s;
    lay[s] = k[s] < LZ && (s == 0 || s1);
    itf[s] = k[s] < LW && (s == 0 || s1);
    const unsigned iz = (unsigned)n * LZ + k[s], iw = (unsigned)n * LW + k[s];
    hn[s] = lay[s] ? g.hnode[iz] : 1.f;
    hnn[s] = lay[s] ? g.hnode_new[iz] : 1.f;
    av[s] = lay[s] ? g.areasvol[iz] : 1.f;
    w[s] = itf[s] ? a.w[iw] : 0.f;
    wl[s] = WESEP ? (itf[s] ? a.we[iw] : 0.f) : w[s];
    ar[s] = itf[s] ? g.area[iw] : 0.f;
    zq[s] = VER == 1 && lay[s] ? g.Z3[iz] : 0.f;
    zbq[s] = VER == 1 && itf[s] ? g.zbar3[iw] : 0.f;
    if (VER == 3) {
      sHnn[k[s]] = hnn[s];
      sHn[k[s]] = hn[s];
    }
    if (VER == 1) {
      sZ[k[s]] = zq[s];
      sZb[k[s]] = zbq[s];
    }
  }
  // the low-order update factors: ra = hnode / hnode_new (exactly 1 for an
  // unchanged layer), rb = dt / (areasvol hnode_new); kept in shared memory
  // until the epilogue, out of the registers the gather needs. Each lane
  // reads back only its own layers.
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    sRa[k[s]] = hn[s] == hnn[s] ? 1.f : fdv(hn[s], hnn[s]);
    sRb[k[s]] = fdv(dt, av[s] * hnn[s]);
  }
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ Tg = a.T + gi * a.gT;
    const float* __restrict__ TAg = TASEP ? a.TA + gi * a.gTA : Tg;
    V<KV> t[2], ta[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      t[s] = lay[s] ? ld<KV>(Tg, (unsigned)n * LZ + k[s]) : splat<KV>(0.f);
      ta[s] = TASEP ? (lay[s] ? ld<KV>(TAg, (unsigned)n * LZ + k[s]) : splat<KV>(0.f)) : t[s];
    }
    if (gi > 0) __syncwarp();  // the previous group has read the shared column
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      sT[k[s]] = t[s];
      if (TASEP) sTA[k[s]] = ta[s];
    }
    __syncwarp();
    // PPM: slopes of the layers with both neighbours (lib/oce_adv_tra_ver.F90:525-545),
    // then the edge values (:510-594)
    V<KV> tv[2];
    if (VER == 3) {
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int j = k[s];
        if (j >= nzmin && j <= nzmax - 3) {
          const float dzm = sHnn[j - 1], dz = hnn[s], dzp = sHnn[j + 1];
          const float f = fdv(dz, dzm + dz + dzp);
          const float s1 = f * fdv(2.f * dzm + dz, dzp + dz);
          const float s0 = f * fdv(dz + 2.f * dzp, dzm + dz);
          const V<KV> Tm = sTA[j - 1], Tp = sTA[j + 1];
          V<KV> r;
#pragma unroll
          for (int q = 0; q < KV; ++q) {
            const float d1 = Tp.v[q] - ta[s].v[q], d0 = ta[s].v[q] - Tm.v[q];
            const float sl = s1 * d1 + s0 * d0;
            r.v[q] = (d1 * d0 > 0.f) ? copysignf(min3f(fabsf(sl), 2.f * fabsf(d1), 2.f * fabsf(d0)), sl) : 0.f;
          }
          sD[j] = r;
        }
      }
      __syncwarp();
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int z = k[s] + 1;  // interface k[s], 1-based
        V<KV> e = ta[s];
        if (z >= nzmin + 2 && z <= nzmax - 2) {
          const int j0 = z - 2;  // layer above the interface
          const float dzm = sHnn[j0 - 1], dz = sHnn[j0], dzp = hnn[s], dzpp = sHnn[j0 + 2];
          const float r1 = frcp(dz + dzp), r2 = frcp(2.f * dz + dzp), r3 = frcp(2.f * dzp + dz);
          const float r4 = frcp(dzm + dz + dzp + dzpp);
          const float c1 = ((2.f * dzp) * dz) * r1 * ((dzm + dz) * r2 - (dzpp + dzp) * r3);
          const float P = dz * r1 + r4 * c1;
          const float Q2 = r4 * (dz * (dzm + dz)) * r2;
          const float Q3 = r4 * (dzp * (dzp + dzpp)) * r3;
          const V<KV> Tu = sTA[j0];
          e = fmas(sD[j0], Q3, fmas(sD[j0 + 1], -Q2, fmas(sub(ta[s], Tu), P, Tu)));
        } else if (z == nzmax) {
          e = sTA[nzmax - 2];
        } else if (z == nzmax - 1) {
          const float sg = copysignf(1.f, w[s]);
          e = fmas(ta[s], fmaxf(sg, 0.f), muls(sTA[nzmax - 3], -fminf(sg, 0.f)));
        } else if (z == nzmin + 1) {
          e = muls(add(sTA[nzmin - 1], ta[s]), 0.5f);
        }
        // z == nzmin: the layer's own value (e = ta); outside the column: unused
        tv[s] = e;
        sTV[k[s]] = e;
      }
      if (lane == 0 && nl - 1 >= 2 * kW && nzmax == nl) sTV[nl - 1] = sTA[nzmax - 2];
      __syncwarp();
    }
    // vertical fluxes at the own interfaces: LO upwind on T with w_e, HO on T_AB
    // with w, adf_v = HO - LO; the LO fluxes are kept in shared memory only
    // (held in registers across the gather they pushed the compensated
    // variant into local-memory spills)
    float* __restrict__ adfv = a.adfv + gi * a.gW;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int iz = k[s], z = iz + 1;
      const bool in = z >= nzmin && z <= nzmax;
      const V<KV> Tup = iz > 0 ? sT[iz - 1] : t[s];
      V<KV> lo = splat<KV>(0.f), ho = splat<KV>(0.f);
      bool twice = false;  // QR4C: the interface the reference writes twice
      if (in && z < nzmax) {
        const float W = wl[s], A = ar[s];
        lo = z == nzmin ? muls(t[s], -(W * A))
                        : fmas(Tup, -0.5f * (W - fabsf(W)) * A, muls(t[s], -0.5f * (W + fabsf(W)) * A));
      }
      if (in) {
        const float W = w[s], A = ar[s];
        const V<KV> TAup = TASEP ? (iz > 0 ? sTA[iz - 1] : ta[s]) : Tup;
        if (VER == 0) {
          if (z == nzmin) ho = muls(ta[s], -(W * A));
          else if (z < nzmax)
            ho = fmas(TAup, -0.5f * (W - fabsf(W)) * A, muls(ta[s], -0.5f * (W + fabsf(W)) * A));
        } else if (VER == 1) {
          if (z == nzmin) {
            ho = muls(ta[s], -(W * A));
          } else if (z == nzmin + 1 || z == nzmax - 1) {
            if (z < nzmax) {
              ho = muls(add(TAup, ta[s]), -0.5f * W * A);
              // the reference writes this interface twice when the two cases
              // coincide (lib/oce_adv_tra_ver.F90:405-411): HO - LO, then HO - that
              twice = nzmin + 1 == nzmax - 1;
            }
          } else if (z < nzmax) {
            const float Z0 = zq[s], Zm1 = sZ[z - 2], Zm2 = sZ[z - 3], Zp1 = sZ[z];
            const float ic = fdv(1.f, Zm1 - Z0), iu = fdv(1.f, Z0 - Zp1), idn = fdv(1.f, Zm2 - Zm1);
            const float zb = zbq[s];
            const float a1 = (zb - Z0) * (1.f / 3.f), a2 = (zb - Zm1) * (1.f / 3.f);
            const float wp = W + fabsf(W), wm = W - fabsf(W);
            const float cA = -(0.5f * (1.f - a.pv)) * A, cB = -(a.pv * 0.5f) * W * A;
            const V<KV> T0 = ta[s], Tm1 = TAup, Tm2 = sTA[z - 3], Tp1 = sTA[z];
            const V<KV> qc = muls(sub(Tm1, T0), ic), qu = muls(sub(T0, Tp1), iu), qd = muls(sub(Tm2, Tm1), idn);
            const V<KV> tm1 = fmas(fmas(qc, 2.f, qu), a1, T0);
            const V<KV> tm2 = fmas(fmas(qc, 2.f, qd), a2, Tm1);
            const V<KV> tm = fmas(tm2, wm, muls(tm1, wp));
            ho = fmas(add(tm1, tm2), cB, muls(tm, cA));
          }
        } else if (VER == 2) {
          if (z == nzmin) ho = muls(ta[s], -(W * A));
          else if (z <= nzmax - 1) ho = muls(add(TAup, ta[s]), -0.5f * W * A);
          else ho = lo;  // CDIFF leaves the bottom flux as it was
        } else {
          if (z == nzmin) {
            ho = muls(tv[s], -(W * A));
          } else if (z < nzmax && W != 0.f) {
            // the upwind layer's parabola: the layer below (W > 0) or above
            const bool up = W > 0.f;
            const int zl = up ? iz : iz - 1;
            const float h = sHn[zl];
            const float x = fminf(fdv(fabsf(W) * dt, h), 1.f);
            const V<KV> aL = up ? tv[s] : sTV[zl], aR = up ? sTV[zl + 1] : tv[s];
            const V<KV> T0 = up ? ta[s] : TAup;
            ho = ppm_flux<KV>(aL, aR, T0, x, up, A * W);
          }
        }
      }
      sF[iz] = lo;
      const V<KV> d = sub(ho, lo);
      if (iz < nl) st<KV>(adfv, (unsigned)n * LW + iz, twice ? sub(ho, d) : d);
    }
    if (lane == 0 && nl - 1 >= 2 * kW) {  // the bottom interface of 65-interface columns
      sF[nl - 1] = splat<KV>(0.f);
      st<KV>(adfv, (unsigned)n * LW + nl - 1, splat<KV>(0.f));
    }
    __syncwarp();
    // LO horizontal fluxes (upwind, lib/oce_adv_tra_hor.F90:218-220) gathered
    // over the incident edges in ascending edge order. The upwind flux
    // -(T1 (v + |v|) + T2 (v - |v|)) / 2 is exactly -v T_up, T_up the value at
    // the upwind node: each node adds -v T_up (first node) or +v T_up (second
    // node), one rounded product that is the same number at both ends of the
    // edge, so the low-order fluxes cancel between neighbours; with COMP the
    // products are summed with compensation.
    V<KV> acc[2] = {splat<KV>(0.f), splat<KV>(0.f)}, accc[2] = {splat<KV>(0.f), splat<KV>(0.f)};
    const unsigned kc[2] = {(unsigned)min(k[0], LZ - 1), (unsigned)min(k[1], LZ - 1)};
#pragma unroll 2
    for (int j = 0; j < deg; ++j) {
      const int2 q = nb_staged ? sNb[j] : make_int2(m.ne_code[e0 + j], m.ne_other[e0 + j]);
      const unsigned ed = (unsigned)(q.x >> 1);
      const bool role = q.x & 1;
      float v[2];
      V<KV> to[2];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        v[s] = lay[s] ? a.vf[ed * LZ + kc[s]] : 0.f;
        to[s] = lay[s] ? ld<KV>(Tg, (unsigned)q.y * LZ + kc[s]) : splat<KV>(0.f);
      }
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        // this node is upwind when the flux leaves it: v >= 0 at the first node, v < 0 at the second
        const bool own_up = (v[s] >= 0.f) != role;
        V<KV> tu;
#pragma unroll
        for (int c = 0; c < KV; ++c) tu.v[c] = own_up ? t[s].v[c] : to[s].v[c];
        const V<KV> p = muls(tu, v[s]);
        if (COMP) two_sum(acc[s], accc[s], role ? p : sub(splat<KV>(0.f), p));
        else acc[s] = role ? add(acc[s], p) : sub(acc[s], p);
      }
    }
    float* __restrict__ lo = a.lo + gi * a.gN;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (!lay[s]) continue;
      const int z = k[s] + 1;
      // the increment LO - T = (fluxes) dt / (areasvol hnode_new) + T (hnode / hnode_new - 1)
      V<KV> l = splat<KV>(0.f);
      if (z >= nzmin && z <= nzmax - 1)
        l = fmas(add(COMP ? add(acc[s], accc[s]) : acc[s], sub(sF[k[s]], sF[k[s] + 1])), sRb[k[s]],
                 muls(t[s], sRa[k[s]] - 1.f));
      st<KV>(lo, (unsigned)n * LZ + k[s], l);
    }
  }
}

}  // namespace fast
}  // namespace fgb
