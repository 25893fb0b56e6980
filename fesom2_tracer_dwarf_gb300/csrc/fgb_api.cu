// Engine C-ABI (fgb_*): host mesh, device mesh upload, workspace, step
// dispatch and tracer statistics.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"

namespace fgb {

static thread_local std::string g_err;
static thread_local int g_last_launches = 0;
void set_error(const std::string& msg) { g_err = msg; }

namespace {

int pad4(int v) { return (v + 3) / 4 * 4; }

template <typename T>
int upload(fgb_mesh* mm, const T* src, size_t n, const T** dst) {
  void* p = nullptr;
  size_t bytes = (n ? n : 1) * sizeof(T);
  cudaError_t ce = cudaMalloc(&p, bytes);
  if (ce != cudaSuccess) {
    set_error(std::string("cudaMalloc failed: ") + cudaGetErrorString(ce));
    return -1;
  }
  mm->allocs.push_back(p);
  if (n) {
    ce = cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
      set_error(std::string("cudaMemcpy failed: ") + cudaGetErrorString(ce));
      return -1;
    }
  } else {
    cudaMemset(p, 0, bytes);
  }
  *dst = static_cast<const T*>(p);
  return 0;
}

// (rows, ncol) host array -> (rows, ld) padded with zeros, converted to T.
template <typename T>
std::vector<T> padded(const std::vector<double>& a, size_t rows, int ncol, int ld) {
  std::vector<T> out(rows * (size_t)ld, T(0));
  for (size_t r = 0; r < rows; ++r)
    for (int k = 0; k < ncol; ++k) out[r * ld + k] = (T)a[r * ncol + k];
  return out;
}

template <typename T>
std::vector<T> conv(const std::vector<double>& a) {
  return std::vector<T>(a.begin(), a.end());
}

template <typename T>
int upload_geo(fgb_mesh* mm, const HostMesh& h, GeoPtrs<T>& g, T** hn, T** hnn, T** he) {
  const int LZ = mm->d.LZ, LW = mm->d.LW;
  // areasvol is allocated (nl, N) in the reference but only layers 1..nl-1 are used.
  std::vector<double> asv((size_t)h.N * h.nz);
  for (int n = 0; n < h.N; ++n)
    for (int k = 0; k < h.nz; ++k) asv[(size_t)n * h.nz + k] = h.areasvol[(size_t)n * h.nl + k];
  auto v_hn = padded<T>(h.hnode, h.N, h.nz, LZ);
  auto v_hnn = padded<T>(h.hnode_new, h.N, h.nz, LZ);
  auto v_asv = padded<T>(asv, h.N, h.nz, LZ);
  auto v_area = padded<T>(h.area, h.N, h.nl, LW);
  auto v_z3 = padded<T>(h.Z3, h.N, h.nz, LZ);
  auto v_zb3 = padded<T>(h.zbar3, h.N, h.nl, LW);
  auto v_he = padded<T>(h.helem, h.M, h.nz, LZ);
  auto v_ec = conv<T>(h.edge_cross);
  auto v_dxa = conv<T>(h.edge_dxa);
  auto v_gs = conv<T>(h.grad_sca);
  auto v_ea = conv<T>(h.elem_area);
  if (upload(mm, v_hn.data(), v_hn.size(), &g.hnode) || upload(mm, v_hnn.data(), v_hnn.size(), &g.hnode_new) ||
      upload(mm, v_asv.data(), v_asv.size(), &g.areasvol) || upload(mm, v_area.data(), v_area.size(), &g.area) ||
      upload(mm, v_z3.data(), v_z3.size(), &g.Z3) || upload(mm, v_zb3.data(), v_zb3.size(), &g.zbar3) ||
      upload(mm, v_he.data(), v_he.size(), &g.helem) || upload(mm, v_ec.data(), v_ec.size(), &g.edge_cross) ||
      upload(mm, v_dxa.data(), v_dxa.size(), &g.edge_dxa) || upload(mm, v_gs.data(), v_gs.size(), &g.grad_sca) ||
      upload(mm, v_ea.data(), v_ea.size(), &g.elem_area))
    return -1;
  *hn = const_cast<T*>(g.hnode);
  *hnn = const_cast<T*>(g.hnode_new);
  *he = const_cast<T*>(g.helem);
  return 0;
}

bool validate(const HostMesh& h, std::string* err) {
  auto bad = [&](const char* what) {
    *err = std::string("mesh validation failed: ") + what;
    return false;
  };
  if (!h.node_order.empty()) {  // a permutation of the nodes
    if ((int)h.node_order.size() != h.N) return bad("node visit order size");
    std::vector<char> seen(h.N, 0);
    for (int n : h.node_order) {
      if (n < 0 || n >= h.N || seen[n]) return bad("node visit order is not a permutation");
      seen[n] = 1;
    }
  }
  for (int e = 0; e < h.E; ++e) {
    for (int r = 0; r < 2; ++r)
      if (h.edges[2 * e + r] < 0 || h.edges[2 * e + r] >= h.N) return bad("edge node index");
    if (h.edge_tri[2 * e] < 0 || h.edge_tri[2 * e] >= h.M) return bad("edge_tri(1) must be a valid element");
    if (h.edge_tri[2 * e + 1] >= h.M) return bad("edge_tri(2) index");
    for (int r = 0; r < 2; ++r)
      if (h.edge_updn[2 * e + r] >= h.M) return bad("edge_up_dn_tri index");
  }
  for (int el = 0; el < h.M; ++el) {
    for (int k = 0; k < 3; ++k)
      if (h.elem_nodes[3 * el + k] < 0 || h.elem_nodes[3 * el + k] >= h.N) return bad("element node index");
    if (h.ulevels[el] != 1) return bad("cavities (ulevels > 1) are not supported");
    if (h.nlevels[el] < 2 || h.nlevels[el] > h.nl) return bad("element nlevels out of 2..nl");
  }
  for (int n = 0; n < h.N; ++n) {
    if (h.ulev_nod[n] != 1) return bad("cavities (ulevels_nod2D > 1) are not supported");
    if (h.nlev_nod[n] < 2 || h.nlev_nod[n] > h.nl) return bad("nlevels_nod2D out of 2..nl");
    if (h.nie_num[n] < 1) return bad("node without elements");
  }
  for (size_t j = 0; j < h.cl_node.size(); ++j)
    if (h.cl_node[j] < 0 || h.cl_node[j] >= h.N) return bad("cluster node index");
  for (size_t j = 0; j < h.nie_idx.size(); ++j)
    if (h.nie_idx[j] < 0 || h.nie_idx[j] >= h.M) return bad("nod_in_elem2D index");
  return true;
}

}  // namespace
}  // namespace fgb

using namespace fgb;

extern "C" {

const char* fgb_last_error(void) { return g_err.c_str(); }
int fgb_version(void) { return 1; }
int fgb_last_launch_count(void) { return g_last_launches; }

int fgb_hmesh_analytic(int nx, int ny, int nl, double Lx, double Ly, double depth, int periodic, int flags,
                       const double* zbar, const int* elem_nlev, fgb_hmesh** out) {
  if (!out) { set_error("null output"); return -1; }
  std::string err;
  HostMesh* m = build_analytic(nx, ny, nl, Lx, Ly, depth, periodic, flags, zbar, elem_nlev, &err);
  if (!m) { set_error(err); return -1; }
  *out = new fgb_hmesh{m};
  return 0;
}

int fgb_hmesh_from_files(const char* dir, int flags, fgb_hmesh** out) {
  if (!out || !dir) { set_error("null argument"); return -1; }
  if (flags & ~15) { set_error("unknown mesh-file flags"); return -1; }
  std::string err;
  HostMesh* m = build_from_files(dir, flags, &err);
  if (!m) { set_error(err); return -1; }
  *out = new fgb_hmesh{m};
  return 0;
}

int fgb_hmesh_from_arrays(int nod2D, int elem2D, int edge2D, int edge2D_in, int nl, const double* lonlat,
                          const int* elem, const int* edges, const int* edge_tri, const int* elvls,
                          const int* nlvls, const double* zbar, int flags, fgb_hmesh** out) {
  if (!out || !lonlat || !elem || !edges || !edge_tri || !elvls || !nlvls || !zbar) {
    set_error("null argument");
    return -1;
  }
  if (flags & ~15) { set_error("unknown mesh-file flags"); return -1; }
  std::string err;
  HostMesh* m = build_from_arrays(nod2D, elem2D, edge2D, edge2D_in, nl, lonlat, elem, edges, edge_tri, elvls, nlvls,
                                  zbar, flags, &err);
  if (!m) { set_error(err); return -1; }
  *out = new fgb_hmesh{m};
  return 0;
}

int fgb_hmesh_union(const fgb_hmesh* const* parts, int count, fgb_hmesh** out) {
  if (!parts || !out || count < 1) { set_error("bad argument"); return -1; }
  std::vector<const HostMesh*> ps(count);
  for (int i = 0; i < count; ++i) {
    if (!parts[i]) { set_error("null part"); return -1; }
    ps[i] = parts[i]->m;
  }
  std::string err;
  HostMesh* m = union_meshes(ps.data(), count, &err);
  if (!m) { set_error(err); return -1; }
  *out = new fgb_hmesh{m};
  return 0;
}

void fgb_hmesh_free(fgb_hmesh* h) {
  if (!h) return;
  delete h->m;
  delete h;
}

int fgb_hmesh_sizes(const fgb_hmesh* h, long long* o) {
  if (!h || !o) { set_error("null argument"); return -1; }
  const HostMesh& m = *h->m;
  o[0] = m.N; o[1] = m.E; o[2] = m.M; o[3] = m.nl; o[4] = m.max_nie; o[5] = m.edge2D_in;
  o[6] = (long long)m.ne_code.size(); o[7] = (long long)m.cl_node.size();
  return 0;
}

long long fgb_hmesh_get(const fgb_hmesh* h, const char* name, void* out, int* kind) {
  if (!h || !name) return -1;
  const HostMesh& m = *h->m;
  const std::vector<int>* vi = nullptr;
  const std::vector<double>* vd = nullptr;
  struct { const char* n; const std::vector<int>* v; } ints[] = {
      {"elem_nodes", &m.elem_nodes}, {"edges", &m.edges}, {"edge_tri", &m.edge_tri}, {"nlevels", &m.nlevels},
      {"ulevels", &m.ulevels}, {"nlevels_nod2D", &m.nlev_nod}, {"ulevels_nod2D", &m.ulev_nod},
      {"nlevels_nod2D_min", &m.nlev_nod_min}, {"ulevels_nod2D_max", &m.ulev_nod_max},
      {"nod_in_elem2D_num", &m.nie_num}, {"nod_in_elem2D", &m.nie}, {"edge_up_dn_tri", &m.edge_updn},
      {"nboundary_lay", &m.nboundary_lay}, {"ne_ptr", &m.ne_ptr}, {"ne_code", &m.ne_code},
      {"ne_other", &m.ne_other}, {"ne_lo", &m.ne_lo}, {"ne_hi", &m.ne_hi}, {"cl_ptr", &m.cl_ptr},
      {"cl_node", &m.cl_node}, {"cl_lev", &m.cl_lev}, {"cl_minlev", &m.cl_minlev}, {"edge_lev", &m.edge_lev},
      {"edge_gm", &m.edge_gm}, {"edge_order", &m.edge_order}, {"node_order", &m.node_order}, {"nie_ptr", &m.nie_ptr}, {"nie_idx", &m.nie_idx}};
  struct { const char* n; const std::vector<double>* v; } dbls[] = {
      {"coord", &m.coord}, {"zbar", &m.zbar}, {"Z", &m.Z}, {"elem_area", &m.elem_area}, {"area", &m.area},
      {"areasvol", &m.areasvol}, {"edge_dxdy", &m.edge_dxdy}, {"edge_cross_dxdy", &m.edge_cross},
      {"elem_cos", &m.elem_cos}, {"gradient_sca", &m.grad_sca}, {"hnode", &m.hnode}, {"hnode_new", &m.hnode_new},
      {"helem", &m.helem}, {"Z_3d_n", &m.Z3}, {"zbar_3d_n", &m.zbar3}, {"edge_dxa", &m.edge_dxa}};
  for (auto& it : ints)
    if (!strcmp(it.n, name)) vi = it.v;
  for (auto& it : dbls)
    if (!strcmp(it.n, name)) vd = it.v;
  if (vi) {
    if (kind) *kind = 0;
    if (out) memcpy(out, vi->data(), vi->size() * sizeof(int));
    return (long long)vi->size();
  }
  if (vd) {
    if (kind) *kind = 1;
    if (out) memcpy(out, vd->data(), vd->size() * sizeof(double));
    return (long long)vd->size();
  }
  return -1;
}

int fgb_hmesh_set_vertical(fgb_hmesh* h, const double* hnode, const double* hnode_new, const double* helem) {
  if (!h) { set_error("null mesh"); return -1; }
  HostMesh& m = *h->m;
  if (hnode) m.hnode.assign(hnode, hnode + (size_t)m.N * m.nz);
  if (hnode_new) m.hnode_new.assign(hnode_new, hnode_new + (size_t)m.N * m.nz);
  if (helem) m.helem.assign(helem, helem + (size_t)m.M * m.nz);
  return 0;
}

void fgb_mesh_free(fgb_mesh* m) {
  if (!m) return;
  for (void* p : m->allocs) cudaFree(p);
  delete m;
}

int fgb_mesh_create(const fgb_hmesh* hm, fgb_mesh** out) {
  if (!hm || !out) { set_error("null argument"); return -1; }
  const HostMesh& h = *hm->m;
  std::string err;
  if (!validate(h, &err)) { set_error(err); return -1; }
  fgb_mesh* mm = new fgb_mesh();
  cudaGetDevice(&mm->device);
  DMesh& d = mm->d;
  d.N = h.N; d.E = h.E; d.M = h.M; d.nl = h.nl; d.nz = h.nz;
  d.LZ = pad4(h.nz);
  d.LW = pad4(h.nl);
  int minl = 1 << 30;
  for (int n = 0; n < h.N; ++n) minl = std::min(minl, h.nlev_nod[n] - h.ulev_nod[n]);
  d.min_layers = minl;
  std::vector<int> elem_nlev(h.nlevels);
  // FP32 MUSCL tables: triangle weights ((dx, dy) . grad_sca) / 6 of the edge
  // node and the two other vertices of the up- and downwind triangles.
  std::vector<int> ftri((size_t)4 * h.E, 0);
  std::vector<float> fwu((size_t)4 * h.E, 0.f), fwd((size_t)4 * h.E, 0.f);
  d.fast_tri_ok = 1;
  for (int e = 0; e < h.E; ++e) {
    const int n1 = h.edges[2 * e], n2 = h.edges[2 * e + 1];
    const int tu = h.edge_updn[2 * e], td = h.edge_updn[2 * e + 1];
    int* o = &ftri[(size_t)4 * e];
    o[0] = o[1] = n1;
    o[2] = o[3] = n2;
    if (tu < 0 || td < 0) continue;
    const double ex = h.edge_dxa[2 * e], ey = h.edge_dxa[2 * e + 1];
    auto fill = [&](int el, int node, int* oo, float* w) {
      int k = 0;
      bool found = false;
      for (int j = 0; j < 3; ++j) {
        const int v = h.elem_nodes[3 * el + j];
        const double wv = (ex * h.grad_sca[6 * (size_t)el + j] + ey * h.grad_sca[6 * (size_t)el + 3 + j]) / 6.0;
        if (v == node && !found) {
          w[0] = (float)wv;
          found = true;
        } else if (k < 2) {
          oo[k] = v;
          w[1 + k] = (float)wv;
          ++k;
        }
      }
      return found;
    };
    if (!fill(tu, n1, o, &fwu[(size_t)4 * e]) || !fill(td, n2, o + 2, &fwd[(size_t)4 * e])) d.fast_tri_ok = 0;
  }
  // Tiles of the visit order for the tiled FP32 edge kernel: consecutive
  // positions while the tile has at most kTileEdges edges and kTileNodes
  // distinct nodes among their n1, n2 and f_tri vertices.
  std::vector<int> tile_ptr(1, 0), tile_nptr(1, 0), tile_nodes;
  std::vector<unsigned char> tile_slots((size_t)8 * h.E, 0);
  {
    std::vector<int> stamp(h.N, -1), slot(h.N, 0);
    int tile = 0, tn = 0, te = 0;
    for (int p = 0; p < h.E; ++p) {
      const int e = h.edge_order[p];
      const int v6[6] = {h.edges[2 * e], h.edges[2 * e + 1], ftri[4 * (size_t)e], ftri[4 * (size_t)e + 1],
                         ftri[4 * (size_t)e + 2], ftri[4 * (size_t)e + 3]};
      int fresh = 0;
      for (int j = 0; j < 6; ++j) {
        bool seen = stamp[v6[j]] == tile;
        for (int i = 0; i < j && !seen; ++i) seen = v6[i] == v6[j];
        fresh += seen ? 0 : 1;
      }
      if (te == fgb::fast::kTileEdges || tn + fresh > fgb::fast::kTileNodes) {
        tile_ptr.push_back(p);
        tile_nptr.push_back((int)tile_nodes.size());
        ++tile;
        tn = te = 0;
      }
      for (int j = 0; j < 6; ++j) {
        const int v = v6[j];
        if (stamp[v] != tile) {
          stamp[v] = tile;
          slot[v] = tn++;
          tile_nodes.push_back(v);
        }
        tile_slots[8 * (size_t)p + j] = (unsigned char)slot[v];
      }
      ++te;
    }
    tile_ptr.push_back(h.E);
    tile_nptr.push_back((int)tile_nodes.size());
    d.ntiles = (int)tile_ptr.size() - 1;
    d.tile_max_nodes = 1;
    for (int t = 0; t < d.ntiles; ++t) d.tile_max_nodes = std::max(d.tile_max_nodes, tile_nptr[t + 1] - tile_nptr[t]);
  }
  bool ok = !upload(mm, tile_ptr.data(), tile_ptr.size(), &d.tile_ptr) &&
            !upload(mm, tile_nptr.data(), tile_nptr.size(), &d.tile_nptr) &&
            !upload(mm, tile_nodes.data(), tile_nodes.size(), &d.tile_nodes) &&
            !upload(mm, tile_slots.data(), tile_slots.size(), &d.tile_slots) &&
            !upload(mm, ftri.data(), ftri.size(), &d.f_tri) && !upload(mm, fwu.data(), fwu.size(), &d.f_wu) &&
            !upload(mm, fwd.data(), fwd.size(), &d.f_wd) &&!upload(mm, h.nlev_nod.data(), h.nlev_nod.size(), &d.nlev) &&
            !upload(mm, h.ulev_nod.data(), h.ulev_nod.size(), &d.ulev) &&
            !upload(mm, h.nboundary_lay.data(), h.nboundary_lay.size(), &d.nbl) &&
            !upload(mm, h.ne_ptr.data(), h.ne_ptr.size(), &d.ne_ptr) &&
            !upload(mm, h.ne_code.data(), h.ne_code.size(), &d.ne_code) &&
            !upload(mm, h.ne_other.data(), h.ne_other.size(), &d.ne_other) &&
            !upload(mm, h.ne_lo.data(), h.ne_lo.size(), &d.ne_lo) &&
            !upload(mm, h.ne_hi.data(), h.ne_hi.size(), &d.ne_hi) &&
            !upload(mm, h.cl_ptr.data(), h.cl_ptr.size(), &d.cl_ptr) &&
            !upload(mm, h.cl_node.data(), h.cl_node.size(), &d.cl_node) &&
            !upload(mm, h.cl_lev.data(), h.cl_lev.size(), &d.cl_lev) &&
            !upload(mm, h.cl_minlev.data(), h.cl_minlev.size(), &d.cl_minlev) &&
            !upload(mm, h.nie_ptr.data(), h.nie_ptr.size(), &d.nie_ptr) &&
            !upload(mm, h.nie_idx.data(), h.nie_idx.size(), &d.nie_idx) &&
            !upload(mm, h.elem_nodes.data(), h.elem_nodes.size(), &d.elem_nodes) &&
            !upload(mm, elem_nlev.data(), elem_nlev.size(), &d.elem_nlev) &&
            !upload(mm, h.edges.data(), h.edges.size(), &d.edge_nodes) &&
            !upload(mm, h.edge_tri.data(), h.edge_tri.size(), &d.edge_tri) &&
            !upload(mm, h.edge_updn.data(), h.edge_updn.size(), &d.edge_updn) &&
            !upload(mm, h.edge_lev.data(), h.edge_lev.size(), &d.edge_lev) &&
            !upload(mm, h.edge_gm.data(), h.edge_gm.size(), &d.edge_gm) &&
            !upload(mm, h.edge_order.data(), h.edge_order.size(), &d.edge_order) &&
            (h.node_order.empty() || !upload(mm, h.node_order.data(), h.node_order.size(), &d.node_order)) &&
            !upload_geo<double>(mm, h, d.g64, &mm->hnode64, &mm->hnode_new64, &mm->helem64) &&
            !upload_geo<float>(mm, h, d.g32, &mm->hnode32, &mm->hnode_new32, &mm->helem32);
  if (!ok) {
    fgb_mesh_free(mm);
    return -1;
  }
  *out = mm;
  return 0;
}

int fgb_mesh_dims(const fgb_mesh* m, int* o) {
  if (!m || !o) { set_error("null argument"); return -1; }
  const DMesh& d = m->d;
  o[0] = d.N; o[1] = d.E; o[2] = d.M; o[3] = d.nl; o[4] = d.nz; o[5] = d.LZ; o[6] = d.LW; o[7] = d.min_layers;
  return 0;
}

int fgb_mesh_update_vertical(fgb_mesh* m, const fgb_hmesh* hm) {
  if (!m || !hm) { set_error("null argument"); return -1; }
  const HostMesh& h = *hm->m;
  const DMesh& d = m->d;
  if (h.N != d.N || h.M != d.M || h.nz != d.nz) { set_error("mesh size mismatch"); return -1; }
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  auto a = padded<double>(h.hnode, h.N, h.nz, d.LZ), b = padded<double>(h.hnode_new, h.N, h.nz, d.LZ);
  auto c = padded<double>(h.helem, h.M, h.nz, d.LZ);
  auto af = padded<float>(h.hnode, h.N, h.nz, d.LZ), bf = padded<float>(h.hnode_new, h.N, h.nz, d.LZ);
  auto cf = padded<float>(h.helem, h.M, h.nz, d.LZ);
  if (!cp(m->hnode64, a.data(), a.size() * 8) || !cp(m->hnode_new64, b.data(), b.size() * 8) ||
      !cp(m->helem64, c.data(), c.size() * 8) || !cp(m->hnode32, af.data(), af.size() * 4) ||
      !cp(m->hnode_new32, bf.data(), bf.size() * 4) || !cp(m->helem32, cf.data(), cf.size() * 4)) {
    set_error("cudaMemcpy failed");
    return -1;
  }
  return 0;
}

long long fgb_workspace_bytes(const fgb_mesh* m, int precision, int ntracers) {
  if (!m || ntracers < 1) return -1;
  return precision == FGB_FP32 ? workspace_layout_f32(m->d, ntracers).total : workspace_layout_f64(m->d, ntracers).total;
}

int fgb_workspace_offsets(const fgb_mesh* m, int precision, int ntracers, long long* o) {
  if (!m || !o || ntracers < 1) { set_error("bad argument"); return -1; }
  WorkspaceLayout w = precision == FGB_FP32 ? workspace_layout_f32(m->d, ntracers) : workspace_layout_f64(m->d, ntracers);
  for (int i = 0; i < 7; ++i) o[i] = w.off[i];
  return 0;
}

int fgb_adv_stages(const fgb_mesh* m, const fgb_step_desc* d, int mask, void* stream) {
  if (!m || !d) { set_error("null argument"); return -1; }
  std::string err;
  int n = 0, rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d->precision == FGB_FP64) rc = launch_stages_f64(m->d, *d, mask, s, &n, &err);
  else if (d->precision == FGB_FP32) rc = launch_stages_f32(m->d, *d, mask, s, &n, &err);
  else if (d->precision == FGB_FP64_FAST) rc = launch_stages_f64fast(m->d, *d, mask, s, &n, &err);
  else { err = "unknown precision"; rc = -1; }
  g_last_launches = n;
  if (rc) set_error(err);
  return rc;
}

int fgb_adv_step(const fgb_mesh* m, const fgb_step_desc* d, void* stream) {
  return fgb_adv_stages(m, d, FGB_STAGE_VFLUX | FGB_STAGE_HFLUX | FGB_STAGE_LO | FGB_STAGE_RATIO | FGB_STAGE_UPDATE,
                        stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Statistics: per block min/max/sum/NaN over a fixed slice, then one block
// combines the partials in block order (deterministic).
// ---------------------------------------------------------------------------
namespace fgb {
namespace {
constexpr int kStatBlocks = 1024;
constexpr int kStatThreads = 256;

// Sum with its rounding error carried (TwoSum, Knuth): s + c is the exact
// sum of the terms added so far up to the rounding of c.
__device__ __forceinline__ void comp_add(double& s, double& c, double x) {
  const double t = s + x, bp = t - s;
  c += (s - (t - bp)) + (x - bp);
  s = t;
}

// Tracer t of a batch in groups of KV (KV = 1: one tracer per stride): min,
// max, compensated sum and NaN count per blockIdx.y; each block's partial
// sum is s + c rounded once (the final sum adds the blocks' partial sums
// compensated again).
template <typename R>
__global__ void k_stats_partial(const R* __restrict__ T, long long sT, int KV, int N, int nz, int LZ,
                                double* __restrict__ part) {
  const int t = blockIdx.y;
  const R* base = T + (t / KV) * sT + t % KV;
  const long long total = (long long)N * nz;
  const long long per = (total + gridDim.x - 1) / gridDim.x;
  const long long lo = blockIdx.x * per, hi = min(total, lo + per);
  double mn = INFINITY, mx = -INFINITY, sm = 0.0, sc = 0.0, nan = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const long long n = i / nz, k = i - n * nz;
    const double v = (double)base[(n * LZ + k) * KV];
    if (v != v) {  // counted; the sum turns NaN as the reference's sum(dble(values)) does
      nan += 1.0;
      sm += v;
      continue;
    }
    mn = fmin(mn, v);
    mx = fmax(mx, v);
    comp_add(sm, sc, v);
  }
  __shared__ double s[5][kStatThreads];
  s[0][threadIdx.x] = mn; s[1][threadIdx.x] = mx; s[2][threadIdx.x] = sm; s[3][threadIdx.x] = nan;
  s[4][threadIdx.x] = sc;
  __syncthreads();
  for (int w = kStatThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + w]);
      s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + w]);
      double a = s[2][threadIdx.x], c = s[4][threadIdx.x] + s[4][threadIdx.x + w];
      comp_add(a, c, s[2][threadIdx.x + w]);
      s[2][threadIdx.x] = a;
      s[4][threadIdx.x] = c;
      s[3][threadIdx.x] += s[3][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 4)
    part[((size_t)t * gridDim.x + blockIdx.x) * 4 + threadIdx.x] =
        threadIdx.x == 2 ? (isinf(s[2][0]) ? s[2][0] : s[2][0] + s[4][0]) : s[threadIdx.x][0];
}

__global__ void k_stats_final(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  const int t = blockIdx.x;
  if (threadIdx.x != 0) return;
  double mn = INFINITY, mx = -INFINITY, sm = 0.0, sc = 0.0, nan = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const double* p = part + ((size_t)t * nblk + b) * 4;
    mn = fmin(mn, p[0]);
    mx = fmax(mx, p[1]);
    comp_add(sm, sc, p[2]);
    nan += p[3];
  }
  // a NaN anywhere makes the sum NaN, as the plain sum; an infinite sum stays
  // infinite (its compensation term is NaN: inf - inf)
  out[4 * t] = mn; out[4 * t + 1] = mx; out[4 * t + 2] = isinf(sm) ? sm : sm + sc; out[4 * t + 3] = nan;
}
}  // namespace
}  // namespace fgb

extern "C" {

long long fgb_stats_scratch_bytes(const fgb_mesh* m, int ntracers) {
  if (!m || ntracers < 1) return -1;
  return (long long)ntracers * kStatBlocks * 4 * (long long)sizeof(double);
}

int fgb_tracer_stats(const fgb_mesh* m, int precision, const void* T, long long strideT, int ntracers, void* scratch,
                     double* out_dev, void* stream) {
  if (!m || !T || !scratch || !out_dev || ntracers < 1) { set_error("bad argument"); return -1; }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(kStatBlocks, ntracers);
  if (precision == FGB_FP32)
    k_stats_partial<float><<<grid, kStatThreads, 0, s>>>(static_cast<const float*>(T), strideT, 1, m->d.N, m->d.nz,
                                                         m->d.LZ, static_cast<double*>(scratch));
  else
    k_stats_partial<double><<<grid, kStatThreads, 0, s>>>(static_cast<const double*>(T), strideT, 1, m->d.N,
                                                          m->d.nz, m->d.LZ, static_cast<double*>(scratch));
  k_stats_final<<<ntracers, 32, 0, s>>>(static_cast<const double*>(scratch), kStatBlocks, out_dev);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) { set_error(std::string("stats launch failed: ") + cudaGetErrorString(ce)); return -1; }
  return 0;
}

int fgb_tracer_stats_grouped(const fgb_mesh* m, const float* T, long long strideT, int ntracers, int tracer_vec,
                             void* scratch, double* out_dev, void* stream) {
  const int KV = tracer_vec <= 1 ? 1 : tracer_vec;
  if (!m || !T || !scratch || !out_dev || ntracers < 1 || (KV != 2 && KV != 4 && KV != 1) || ntracers % KV) {
    set_error("bad argument");
    return -1;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(kStatBlocks, ntracers);
  k_stats_partial<float><<<grid, kStatThreads, 0, s>>>(T, strideT, KV, m->d.N, m->d.nz, m->d.LZ,
                                                       static_cast<double*>(scratch));
  k_stats_final<<<ntracers, 32, 0, s>>>(static_cast<const double*>(scratch), kStatBlocks, out_dev);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) { set_error(std::string("stats launch failed: ") + cudaGetErrorString(ce)); return -1; }
  return 0;
}

}  // extern "C"
