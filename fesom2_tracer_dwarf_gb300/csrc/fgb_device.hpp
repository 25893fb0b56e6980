// Device-resident mesh and per-launch pointer bundles of the tracer step.
#pragma once
#include <cstddef>
#include <cstdint>

namespace fgb {

// Geometry in the storage precision of a form (FP64 and FP32 copies).
template <typename R>
struct GeoPtrs {
  const R* hnode;       // (N,LZ)
  const R* hnode_new;   // (N,LZ)
  const R* areasvol;    // (N,LZ) layer areas
  const R* area;        // (N,LW) interface areas
  const R* Z3;          // (N,LZ) Z_3d_n
  const R* zbar3;       // (N,LW) zbar_3d_n
  const R* helem;       // (M,LZ)
  const R* edge_cross;  // (E,4)
  const R* edge_dxa;    // (E,2)
  const R* grad_sca;    // (M,6)
  const R* elem_area;   // (M)
};

// Everything the kernels read about the mesh; passed by value to kernels.
struct DMesh {
  int N, E, M, nl, nz, LZ, LW;
  int min_layers;        // fewest layers in any node column
  const int* nlev;       // (N) nlevels_nod2D
  const int* ulev;       // (N) ulevels_nod2D
  const int* nbl;        // (N) nboundary_lay
  const int* ne_ptr;     // (N+1) incident edges, ascending edge index
  const int* ne_code;    // 2*edge + role
  const int* ne_other;   // other endpoint
  const int* ne_lo;      // first layer of that edge's scatter range
  const int* ne_hi;      // last layer of that edge's scatter range
  const int* cl_ptr;     // (N+1) FCT cluster
  const int* cl_node;
  const int* cl_lev;
  const int* cl_minlev;  // (N)
  const int* nie_ptr;    // (N+1) nod_in_elem2D
  const int* nie_idx;
  const int* elem_nodes;  // (M,3)
  const int* elem_nlev;   // (M)
  const int* edge_nodes;  // (E,2)
  const int* edge_tri;    // (E,2)
  const int* edge_updn;   // (E,2)
  const int* edge_lev;    // (E,4)
  const int* edge_gm;     // (E,2)
  const int* edge_order;  // (E) order in which edge kernels visit the edges
  const int* node_order;  // (N) order in which node kernels visit the columns; nullptr: node index
  // FP32 form, MUSCL/MFCT: per edge the two other vertices of the upwind and
  // downwind triangles (E,4) and the triangles' edge-direction weights (E,4)
  // each; valid when fast_tri_ok (each triangle holds its edge node).
  const int* f_tri;
  const float* f_wu;
  const float* f_wd;
  int fast_tri_ok;
  // FP32 form, tiled edge kernel: the visit order cut into tiles of at most
  // kTileEdges edges touching at most kTileNodes distinct nodes (the edges'
  // nodes and the f_tri vertices). Tile t holds visit positions
  // tile_ptr[t] .. tile_ptr[t+1]-1 and nodes tile_nodes[tile_nptr[t] ..]; the
  // 8 bytes of tile_slots[p] give the tile slots of position p's n1, n2 and
  // four f_tri vertices.
  int ntiles, tile_max_nodes;
  const int* tile_ptr;
  const int* tile_nptr;
  const int* tile_nodes;
  const unsigned char* tile_slots;
  GeoPtrs<double> g64;
  GeoPtrs<float> g32;
};

// Node column of visit position i of a node kernel (every column is visited
// once; the order only shapes which columns are in flight together).
#ifdef __CUDACC__
__device__ __forceinline__ int visit_node(const DMesh& m, int i) { return m.node_order ? __ldg(m.node_order + i) : i; }
#endif

// Per-launch field pointers. Tracer t of a batch lives at base + t*stride.
template <typename R>
struct StepPtrs {
  R* T;             // (K,N,LZ) tracer values, updated in place
  const R* TA;      // (K,N,LZ) values used for the high-order fluxes (valuesAB)
  R* TAout;         // optional: written with the new values (copy-AB)
  const R* vel;     // (M,LZ,2) horizontal velocity on elements
  const R* w;       // (N,LW) vertical velocity used by the high-order flux under FCT
  const R* we;      // (N,LW) explicit vertical velocity
  const R* wi;      // optional (N,LW) implicit vertical velocity (w_split)
  R* vf;            // (E,LZ) volume flux through the edge segments
  R* adfh;          // (K,E,LZ) antidiffusive (FCT) or high-order horizontal flux
  R* lo;            // (K,N,LZ) low-order solution fct_LO
  R* adfv;          // (K,N,LW) antidiffusive vertical flux
  R* rpm;           // (K,N,LZ,2) limiting factors fct_plus, fct_minus interleaved per layer
  R* del;           // optional (K,N,LZ) persistent del_ttf
  long long sT, sTA, sE, sN, sW;  // strides between tracers (elements)
  int K;            // tracers in this launch
  R dt, ph, pv;
  int ab2;          // TAout = ab_old * T_old + ab_new * T_new (else T_new)
  R ab_old, ab_new;
};

namespace fast {
// Tiles this small keep a block's staged rows near 32 KB, so the register
// limit (seven blocks of 128 threads) rather than shared memory sets the
// kernel's occupancy; at 2048^2 x 64 the edge stage took 7.65 / 6.90 / 6.57 /
// 6.13 ms with tiles of 64/96, 48/72, 40/64 and 32/48 edges/nodes.
constexpr int kTileEdges = 32;  // edges per tile of the tiled edge kernel
constexpr int kTileNodes = 48;  // distinct nodes per tile

// Pointers of one launch. Group g of a per-tracer array starts at
// base + g * stride (floats); offsets inside a group are in units of KV floats.
struct FastPtrs {
  float* T;
  const float* TA;
  float* TAout;
  const float* vel;  // (M,LZ,2)
  const float* w;    // (N,LW)
  const float* we;   // (N,LW)
  const float* wi;   // optional (N,LW): w_split
  float* vf;         // (E,LZ)
  float* adfh;       // (G,E,LZ,KV)
  float* lo;         // (G,N,LZ,KV)
  float* adfv;       // (G,N,LW,KV)
  float* rpm;        // (G,N,LZ,2,KV): R+ then R- per layer
  float* del;        // optional (G,N,LZ,KV)
  long long gT, gTA, gE, gN, gW;  // group strides (floats)
  int G;
  float dt, ph, pv;
  int ab2;  // TAout = ab_old * T_old + ab_new * T_new (else T_new)
  float ab_old, ab_new;
  int wsplit_fused;  // w_split: the LO kernel also solves the implicit vertical step
  int comp;          // compensated sums: bit 1 LO fluxes, 2 update divergence, 4 FCT +/- sums (~fp32_plain_sums)
  float* Tlo;        // optional (G,N,LZ,KV), stride gT: the rounding residual of each value of T
};

// Shared-memory shape of the w_split kernel (kf_vert_impl): a warp holds
// 32 / KV node columns, one lane per (node, tracer of the group).
template <int KV>
struct VimplShape {
  static constexpr int NPW = 32 / KV;  // node columns per warp
  static constexpr int CS = NPW + 1;   // row stride of the per-node arrays (odd: conflict-free)
  static constexpr int RS = 32 + KV;   // row stride of the per-lane array (conflict-free V<KV> rows)
  // floats of one warp: the per-lane array, then a, b, c and the cp ratios
  __host__ __device__ static constexpr size_t warp_floats(int LZ) { return (size_t)LZ * (RS + 4 * CS); }
};
constexpr int kVimplWarpsF = 4;  // warps per block
inline size_t vimpl_block_bytes(int LZ, int KV) {
  const size_t w = KV == 4 ? VimplShape<4>::warp_floats(LZ)
                           : (KV == 2 ? VimplShape<2>::warp_floats(LZ) : VimplShape<1>::warp_floats(LZ));
  return kVimplWarpsF * w * sizeof(float);
}

// Launch shape of one FP32 call.
struct LaunchArgs {
  int mask, edge_warps, nw_lo, nw_ratio, nw_upd, hor, ver, fct;
  int ns_h, ns_lo, ns_ratio, ns_upd;  // layers per lane per pass (1 or 2)
  int vimpl_thomas;  // w_split: lane-per-column Thomas sweeps also for columns of <= 64 layers
  int hflux_tile;    // edge fluxes by the tiled kernel (node rows staged once per tile)
};
}  // namespace fast

}  // namespace fgb
