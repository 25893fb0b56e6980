// FP32 edge fluxes, tiled (same fluxes as kf_hflux: lib/oce_adv_tra_hor.F90
// UPW1 :218-220, MUSCL :454-497, MFCT :748-790; FCT: high-order minus
// low-order).
//
// The edges' tracer reads are gathers of node rows (layers fastest): the two
// nodes of the edge and the other vertices of its up- and downwind triangles.
// Neighbouring edges of the visit order share most of these nodes, so the
// visit order is cut into tiles (at mesh upload) of at most kTileEdges edges
// touching at most kTileNodes distinct nodes, and one block per tile stages
// each distinct node row once per pass of kTileChunk layers in shared memory
// with asynchronous 16-byte copies, then computes all edges of the tile from
// there, one edge per warp at a time.
#pragma once
#include <cuda_runtime.h>

#include "fgb_fast.cuh"

namespace fgb {
namespace fast {

constexpr int kTileThreads = 128;
constexpr int kTileChunk = 32;  // layers per pass: lane l handles layer k0 + l of one edge

// 16-byte asynchronous copy global -> shared (cp.async, L2 only), and the
// wait for all of this thread's copies.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Shared memory: edge records, the start of each edge's six node rows in the
// staged rows (16 bits each: slot x kTileChunk; 12 bytes per edge, which keeps
// seven blocks of the largest tiles on an SM), the node ids, the TA rows
// (+ T rows when T_AB is separate under FCT) of the mesh's largest tile (maxn
// nodes) and the volume-flux rows of one pass.
__host__ __device__ constexpr size_t tile_smem_bytes(int KV, bool tsep, int maxn) {
  return (size_t)kTileEdges * sizeof(EdgeRec) + (size_t)kTileEdges * 12 + (size_t)kTileNodes * 4 +
         (size_t)(tsep ? 2 : 1) * maxn * kTileChunk * KV * 4 + (size_t)kTileEdges * kTileChunk * 4;
}
static_assert(kTileNodes * kTileChunk < 65536, "row starts are 16-bit");

template <int HOR, bool FCT, int KV>
__global__ void __launch_bounds__(kTileThreads) kf_hflux_tile(DMesh m, FastPtrs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EdgeRec* recs = reinterpret_cast<EdgeRec*>(smem_raw);
  // row starts of n1 | n2 and of the upwind triangle's two other vertices (rsA), of
  // the downwind triangle's two others (rsD)
  uint2* rsA = reinterpret_cast<uint2*>(smem_raw + kTileEdges * sizeof(EdgeRec));
  unsigned* rsD = reinterpret_cast<unsigned*>(rsA + kTileEdges);
  int* nodes = reinterpret_cast<int*>(rsD + kTileEdges);
  const bool ta_sep = a.TA != a.T;
  const bool tsep = FCT && ta_sep;
  V<KV>* rowsA = reinterpret_cast<V<KV>*>(nodes + kTileNodes);  // [node slot][layer of the pass]
  V<KV>* rowsT = tsep ? rowsA + m.tile_max_nodes * kTileChunk : rowsA;
  float* rowsV = reinterpret_cast<float*>(rowsA + (tsep ? 2 : 1) * m.tile_max_nodes * kTileChunk);  // [edge][layer]
  const int tid = threadIdx.x, lane = tid & (kW - 1), warp = tid / kW;
  const int t = blockIdx.x;
  const int p0 = m.tile_ptr[t], ne = m.tile_ptr[t + 1] - p0;
  const int q0 = m.tile_nptr[t], nn = m.tile_nptr[t + 1] - q0;
  __shared__ int s_hi;  // the deepest layer of the tile's edges
  if (tid == 0) s_hi = 0;
  __syncthreads();
  for (int i = tid; i < ne; i += kTileThreads) {
    fill_edge<HOR>(m, p0 + i, recs[i]);
    const uint2 sl = *reinterpret_cast<const uint2*>(m.tile_slots + 8 * (size_t)(p0 + i));
    auto two = [](unsigned a, unsigned b) { return (a * kTileChunk) | ((b * kTileChunk) << 16); };
    rsA[i] = make_uint2(two(sl.x & 0xff, (sl.x >> 8) & 0xff), two((sl.x >> 16) & 0xff, sl.x >> 24));
    rsD[i] = two(sl.y & 0xff, (sl.y >> 8) & 0xff);
    atomicMax(&s_hi, recs[i].hi);
  }
  for (int i = tid; i < nn; i += kTileThreads) nodes[i] = m.tile_nodes[q0 + i];
  const unsigned LZ = m.LZ;
  const int nz = m.nz;
  const float A = 0.5f * (1.f - a.ph);
  for (int gi = 0; gi < a.G; ++gi) {
    const float* __restrict__ TAg = ta_sep ? a.TA + gi * a.gTA : a.T + gi * a.gT;
    const float* __restrict__ Tg = a.T + gi * a.gT;
    float* __restrict__ out = a.adfh + gi * a.gE;
    for (unsigned k0 = 0; k0 < LZ; k0 += kTileChunk) {
      const int rows = (int)min((unsigned)kTileChunk, LZ - k0);
      __syncthreads();  // the previous pass has read the rows (first pass: records filled)
      if ((int)k0 >= s_hi) {
        // below every edge of the tile: the fluxes are zero (the node kernels read them)
        if (lane < rows)
          for (int j = warp; j < ne; j += kTileThreads / kW) st<KV>(out, (unsigned)recs[j].e * LZ + k0 + lane, splat<KV>(0.f));
        continue;
      }
      // Stage the pass with 16-byte asynchronous copies: a node's rows of the
      // pass are rows * KV floats from (node * LZ + k0) * KV, a multiple of 16
      // bytes from a 16-byte boundary (LZ, k0 and rows are multiples of 4).
      {
        // each thread copies the same 16-byte unit u of every (kTileThreads / upr)-th row
        constexpr int upr = kTileChunk * KV / 4;  // 16-byte units per staged node row
        static_assert(kTileThreads % upr == 0, "whole rows per round");
        const int used = rows * KV / 4;
        const int u = tid % upr;
        if (u < used) {
          float* dA = reinterpret_cast<float*>(rowsA) + 4 * u;
          float* dT = reinterpret_cast<float*>(rowsT) + 4 * u;
          for (int j = tid / upr; j < nn; j += kTileThreads / upr) {
            const size_t off = ((size_t)nodes[j] * LZ + k0) * KV + 4 * u;
            cp_async16(dA + (size_t)j * kTileChunk * KV, TAg + off);
            if (tsep) cp_async16(dT + (size_t)j * kTileChunk * KV, Tg + off);
          }
        }
        constexpr int upv = kTileChunk / 4;
        static_assert(kTileThreads % upv == 0, "whole rows per round");
        const int uv = tid % upv;
        if (4 * uv < rows)
          for (int j = tid / upv; j < ne; j += kTileThreads / upv)
            cp_async16(rowsV + j * kTileChunk + 4 * uv, a.vf + (size_t)recs[j].e * LZ + k0 + 4 * uv);
        cp_async_wait_all();
      }
      __syncthreads();
      if (lane >= rows) continue;
      const unsigned k = k0 + lane;
      const int z = (int)k + 1;
      for (int j = warp; j < ne; j += kTileThreads / kW) {
        // the edge's record in vector reads (broadcast to the warp)
        const int4* rv = reinterpret_cast<const int4*>(&recs[j]);
        const int4 r0 = rv[0], r1 = rv[1];  // e, n1, n2, hi | gm0, gm1, nb1, nb2
        const uint2 rs = rsA[j];
        const int e = r0.x, hi = r0.w;
        const bool act = (int)k < nz && z <= hi;
        const float v = rowsV[j * kTileChunk + lane];
        const float vp = v + fabsf(v), vm = v - fabsf(v);
        const V<KV> s1 = rowsA[(rs.x & 0xffff) + lane];
        const V<KV> s2 = rowsA[(rs.x >> 16) + lane];
        V<KV> h;
        if (HOR == 0) {
          h = muls(fmas(s2, vm, muls(s1, vp)), -0.5f);
        } else {
          const float4 wu = reinterpret_cast<const float4*>(&recs[j])[4];
          const float4 wd = reinterpret_cast<const float4*>(&recs[j])[5];
          const bool tri_ok = r1.x >= 0 && z >= r1.x && z <= r1.y - 1;
          const float B = (v * a.ph) * 0.5f;
          const float c1 = (HOR == 2 || r1.z - z >= 0) ? 1.f : 0.f;
          const float c2 = (HOR == 2 || r1.w - z >= 0) ? 1.f : 0.f;
          const V<KV> dT3 = muls(sub(s2, s1), 1.f / 3.f);
          V<KV> p1, p2;
          if (tri_ok) {
            const unsigned rd = rsD[j];
            const V<KV> u1 = rowsA[(rs.y & 0xffff) + lane];
            const V<KV> u2 = rowsA[(rs.y >> 16) + lane];
            const V<KV> d1 = rowsA[(rd & 0xffff) + lane];
            const V<KV> d2 = rowsA[(rd >> 16) + lane];
            p1 = fmas(u2, wu.z, fmas(u1, wu.y, fmas(s1, wu.x, dT3)));
            p2 = fmas(d2, wd.z, fmas(d1, wd.y, fmas(s2, wd.x, dT3)));
          } else if (act) {
            const float2 ex = reinterpret_cast<const float2*>(&recs[j])[4];  // ex, ey: bytes 32-39
            V<KV> gx, gy;
            node_grad<KV>(m, TAg, r0.y, k, gx, gy);
            p1 = fmas(fmas(gy, ex.y, muls(gx, ex.x)), 1.f / 6.f, dT3);
            node_grad<KV>(m, TAg, r0.z, k, gx, gy);
            p2 = fmas(fmas(gy, ex.y, muls(gx, ex.x)), 1.f / 6.f, dT3);
          } else {
            p1 = splat<KV>(0.f);
            p2 = p1;
          }
          const V<KV> tm1 = fmas(p1, c1, s1), tm2 = fmas(p2, -c2, s2);
          const V<KV> cho = fmas(tm2, vm, muls(tm1, vp));
          h = fmas(add(tm1, tm2), -B, muls(cho, -A));
        }
        V<KV> r = h;
        if (FCT) {
          const V<KV> q1 = tsep ? rowsT[(rs.x & 0xffff) + lane] : s1;
          const V<KV> q2 = tsep ? rowsT[(rs.x >> 16) + lane] : s2;
          r = fmas(fmas(q2, vm, muls(q1, vp)), 0.5f, r);
        }
        if (!act) r = splat<KV>(0.f);
        st<KV>(out, (unsigned)e * LZ + k, r);
      }
    }
  }
}

}  // namespace fast
}  // namespace fgb
