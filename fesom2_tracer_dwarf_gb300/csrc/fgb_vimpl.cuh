// Implicit vertical advection of the w_split option (adv_tra_vert_impl,
// lib/oce_adv_tra_ver.F90:90-244), applied in place to the FCT low-order
// solution between the LO and ratio kernels (lib/oce_adv_tra_driver.F90:
// 221-228). Per node column, the upwind scheme with the implicit vertical
// velocity wi is a tridiagonal system over the layers nzmin..nzmax-1, solved
// by the Thomas algorithm in the reference's operation order.
//
// FP64 form (built with -fmad=false: bit-identical to the reference's
// arithmetic, including the solve for the increment). One warp per node.
// Lanes build the coefficients and right-hand sides layer by layer in
// parallel; the pivots m = b - cp*a and the ratios cp = c/m do not depend on
// the tracer and are formed once per node by lane 0; then lane i runs the
// forward and backward sweeps of staged tracer i. (The FP32 form has its own
// kernel with one lane per node column, kf_vert_impl.)
#pragma once
#include <cuda_runtime.h>

#include "fgb_device.hpp"

namespace fgb {
#if FGB_FAST64
inline namespace fast64 {
#else
inline namespace exact64 {
#endif

constexpr int kVimplTracers = 8;  // tracer columns staged per warp and pass
constexpr int kVimplWarps = 4;    // node columns per block

// Column stride in shared memory: odd, so that lanes walking different
// tracers' columns hit different banks.
__host__ __device__ constexpr int vimpl_stride(int LZ) { return LZ | 1; }

// Shared memory of one warp: a, b, c, the pivots and cp, then per staged
// tracer its column and its right-hand side (overwritten by the solution).
template <typename R>
__host__ __device__ constexpr size_t vimpl_warp_bytes(int LZ) {
  return (size_t)(5 + 2 * kVimplTracers) * vimpl_stride(LZ) * sizeof(R);
}

// Tracer t of the launch, node n, layer k is lo[(t / V) * sG + (n * LZ + k) * V + t % V]
// (V = 1: the (K,N,LZ) layout).
template <typename R>
__global__ void __launch_bounds__(kVimplWarps * 32) k_vert_impl(DMesh m, GeoPtrs<R> g, R* lo,
                                                               const R* __restrict__ wi, int K, int V,
                                                               long long sG, R dt) {
  extern __shared__ __align__(16) unsigned char vimpl_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int vi = blockIdx.x * kVimplWarps + wib;
  if (vi >= m.N) return;
  const int n = visit_node(m, vi);
  const int LZ = m.LZ, LW = m.LW, S = vimpl_stride(LZ);
  R* sh = reinterpret_cast<R*>(vimpl_smem + (size_t)wib * vimpl_warp_bytes<R>(LZ));
  R *sa = sh, *sb = sh + S, *sc = sh + 2 * S, *sm = sh + 3 * S, *scp = sh + 4 * S;
  R* sT = sh + 5 * S;                 // staged columns
  R* sR = sT + kVimplTracers * S;     // right-hand sides, then the increments
  const int k0 = m.ulev[n] - 1, k1 = m.nlev[n] - 2;  // first and last layer (0-based)
  const R zinv = R(1) * dt;
  const size_t nw = (size_t)n * LW, nz = (size_t)n * LZ;
  for (int k = k0 + lane; k <= k1; k += 32) {
    const R W0 = wi[nw + k], av = g.areasvol[nz + k], hnn = g.hnode_new[nz + k];
    const R v0 = zinv * g.area[nw + k] / av;
    R a, b, c = R(0);
    if (k == k0) {
      a = R(0);
      b = hnn + W0 * v0;
    } else {
      a = (W0 < R(0) ? W0 : R(0)) * v0;
      b = hnn + (W0 > R(0) ? W0 : R(0)) * v0;
    }
    if (k != k1) {
      const R W1 = wi[nw + k + 1];
      const R v1 = zinv * g.area[nw + k + 1] / av;
      b = b - (W1 < R(0) ? W1 : R(0)) * v1;
      c = -((W1 > R(0) ? W1 : R(0)) * v1);
    }
    sa[k] = a;
    sb[k] = b;
    sc[k] = c;
  }
  __syncwarp();
  if (lane == 0) {
    R cp = sc[k0] / sb[k0];
    scp[k0] = cp;
    sm[k0] = sb[k0];
    for (int k = k0 + 1; k <= k1; ++k) {
      const R mm = sb[k] - cp * sa[k];
      cp = sc[k] / mm;
      scp[k] = cp;
      sm[k] = mm;
    }
  }
  for (int t0 = 0; t0 < K; t0 += kVimplTracers) {
    const int tc = K - t0 < kVimplTracers ? K - t0 : kVimplTracers;
    for (int i = 0; i < tc; ++i) {
      const int t = t0 + i;
      const R* col = lo + (t / V) * sG + nz * V + t % V;
      for (int k = k0 + lane; k <= k1; k += 32) sT[i * S + k] = col[(size_t)k * V];
    }
    __syncwarp();
    for (int k = k0 + lane; k <= k1; k += 32) {
      const R a = sa[k], bd = sb[k] - g.hnode_new[nz + k], c = sc[k];
      for (int i = 0; i < tc; ++i) {
        const R* T = sT + i * S;
        R r;
        if (k == k0) r = -(bd * T[k]) - c * T[k + 1];
        else if (k == k1) r = -(a * T[k - 1]) - bd * T[k];
        else r = -(a * T[k - 1]) - bd * T[k] - c * T[k + 1];
        sR[i * S + k] = r;
      }
    }
    __syncwarp();
    if (lane < tc) {
      R* r = sR + lane * S;
      R tp = r[k0] / sm[k0];
      r[k0] = tp;
      for (int k = k0 + 1; k <= k1; ++k) {
        tp = (r[k] - tp * sa[k]) / sm[k];
        r[k] = tp;
      }
      R x = tp;
      for (int k = k1 - 1; k >= k0; --k) {
        x = r[k] - scp[k] * x;
        r[k] = x;
      }
    }
    __syncwarp();
    for (int i = 0; i < tc; ++i) {
      const int t = t0 + i;
      R* col = lo + (t / V) * sG + nz * V + t % V;
      for (int k = k0 + lane; k <= k1; k += 32) col[(size_t)k * V] = sT[i * S + k] + sR[i * S + k];
    }
    __syncwarp();
  }
}

// Checks of a w_split launch: columns of at least two layers (with one, the
// reference's right-hand side reads the layer above the column) and the
// shared memory of a block. Returns nullptr or the reason.
template <typename R>
inline const char* vert_impl_check(const DMesh& m) {
  if (m.min_layers < 2) return "w_split needs at least two layers in every column";
  if (kVimplWarps * vimpl_warp_bytes<R>(m.LZ) > 227 * 1024) return "w_split: too many layers for one block";
  return nullptr;
}

// Launches k_vert_impl over all nodes (after vert_impl_check).
template <typename R>
inline void launch_vert_impl(const DMesh& m, const GeoPtrs<R>& g, R* lo, const R* wi, int K, int V, long long sG,
                             R dt, cudaStream_t s) {
  const size_t smem = kVimplWarps * vimpl_warp_bytes<R>(m.LZ);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_vert_impl<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid((m.N + kVimplWarps - 1) / kVimplWarps), block(kVimplWarps * 32);
  k_vert_impl<R><<<grid, block, smem, s>>>(m, g, lo, wi, K, V, sG, dt);
}

}  // inline namespace
}  // namespace fgb
