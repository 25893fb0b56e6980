// Host-side set-up of the tracer-advection mesh: the analytic grid of
// lib/analytic_mesh.F90, the geometry of lib/oce_mesh.F90 (mesh_areas,
// mesh_auxiliary_arrays), the MUSCL tables of lib/oce_muscl_adv.F90 and the
// node-centred gather tables the GB300 kernels use in place of the
// reference's edge scatters.
//
// Compiled with -ffp-contract=off: the geometry is bit-identical to the
// reference's statement order, so the device step can match the CPU
// restatement to the last bit.
#include "fgb_hmesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace fgb {
namespace {

constexpr double kCyclic = 360.0;  // lib/gen_modules_config.F90:83 (degrees; a no-op on radians)

double trim_cyclic(double b) {  // lib/gen_modules_rotate_grid.F90:216-224
  if (b > kCyclic / 2.0) b = b - kCyclic;
  if (b < -kCyclic / 2.0) b = b + kCyclic;
  return b;
}

struct Grid {
  int nx, ny, nreal, ntotal;
  bool periodic;
  // Node of grid point (i,j), 1-based grid indices; halo copies for the
  // periodic seam (lib/analytic_mesh.F90:721-733). Returns a 0-based index.
  int node(int i, int j) const {
    if (!periodic) return (j - 1) * nx + (i - 1);
    if (i <= nx - 1 && j <= ny - 1) return (j - 1) * (nx - 1) + (i - 1);
    if (i == nx && j <= ny - 1) return nreal + (j - 1);
    if (i <= nx - 1 && j == ny) return nreal + (ny - 1) + (i - 1);
    return ntotal - 1;
  }
  // Halo node -> real node (lib/analytic_mesh.F90:744-754), 0-based.
  int real_of(int n) const {
    if (n < nreal) return n;
    int h = n - nreal;  // 0-based halo slot
    if (h < ny - 1) return h * (nx - 1);
    if (h < (ny - 1) + (nx - 1)) return h - (ny - 1);
    return 0;
  }
};

}  // namespace

namespace detail {

// Lists of the elements around each node, in element order
// (lib/analytic_mesh.F90:675-694); nodes >= nlimit are skipped.
void node_elem_lists(const std::vector<int>& en, int M, int ntotal, int nlimit, std::vector<int>& num,
                     std::vector<int>& lst, int& maxn) {
  num.assign(ntotal, 0);
  for (int e = 0; e < M; ++e)
    for (int k = 0; k < 3; ++k)
      if (en[3 * e + k] < nlimit) num[en[3 * e + k]]++;
  maxn = 0;
  for (int n = 0; n < ntotal; ++n) maxn = std::max(maxn, num[n]);
  lst.assign((size_t)maxn * ntotal, -1);
  std::fill(num.begin(), num.end(), 0);
  for (int e = 0; e < M; ++e)
    for (int k = 0; k < 3; ++k) {
      int n = en[3 * e + k];
      if (n >= nlimit) continue;
      lst[(size_t)n * maxn + num[n]] = e;
      num[n]++;
    }
}

// Up/downwind triangle search of lib/oce_muscl_adv.F90:245-337 for one node.
// x components are trimmed by the mesh's cyclic_length as the reference does
// (with 360 a no-op on radian coordinates); on periodic analytic meshes the
// vectors are then wrapped to the minimum image.
// The Fortran `cycle` keeps scanning, so the last matching element wins.
int updn_search(const HostMesh& m, int node, const double* x) {
  const double px = m.Lx / kREarth, py = m.Ly / kREarth;
  auto trim = [&](double v) {  // trim of b(1), c(1) by cyclic_length
    if (v > m.cyclic / 2.0) v = v - m.cyclic;
    if (v < -m.cyclic / 2.0) v = v + m.cyclic;
    return v;
  };
  auto wrap = [&](double* v) {
    if (!m.periodic) return;
    if (v[0] > 0.5 * px) v[0] = v[0] - px;
    if (v[0] < -0.5 * px) v[0] = v[0] + px;
    if (v[1] > 0.5 * py) v[1] = v[1] - py;
    if (v[1] < -0.5 * py) v[1] = v[1] + py;
  };
  int found = -1;
  for (int k = 0; k < m.nie_num[node]; ++k) {
    int el = m.nie[(size_t)node * m.max_nie + k];
    const int* en = &m.elem_nodes[3 * el];
    int v1, v2, v3;
    if (en[0] == node) { v1 = en[0]; v2 = en[1]; v3 = en[2]; }
    else if (en[1] == node) { v1 = en[1]; v2 = en[0]; v3 = en[2]; }
    else { v1 = en[2]; v2 = en[0]; v3 = en[1]; }
    double b[2] = {m.coord[2 * v2] - m.coord[2 * v1], m.coord[2 * v2 + 1] - m.coord[2 * v1 + 1]};
    double c[2] = {m.coord[2 * v3] - m.coord[2 * v1], m.coord[2 * v3 + 1] - m.coord[2 * v1 + 1]};
    b[0] = trim(b[0]);
    c[0] = trim(c[0]);
    wrap(b);
    wrap(c);
    double cr = c[0] * c[0] + c[1] * c[1];
    double bx = (b[0] * c[0] + b[1] * c[1]) / cr;
    double by = (-b[0] * c[1] + b[1] * c[0]) / cr;
    double xx = (x[0] * c[0] + x[1] * c[1]) / cr;
    double xy = (-x[0] * c[1] + x[1] * c[0]) / cr;
    double ab = std::atan2(by, bx), ax = std::atan2(xy, xx);
    if ((ab > 0.0 && ax > 0.0 && ax < ab) || (ab < 0.0 && ax < 0.0 && ax > ab) || (ab == ax || ax == 0.0))
      found = el;
  }
  return found;
}

}  // namespace detail

void ale_from_zbar(HostMesh& m) {
  const int N = m.N, M = m.M, nz = m.nz, nl = m.nl;
  m.hnode.assign((size_t)N * nz, 0.0);
  m.hnode_new.assign((size_t)N * nz, 0.0);
  m.helem.assign((size_t)M * nz, 0.0);
  m.Z3.assign((size_t)N * nz, 0.0);
  m.zbar3.assign((size_t)N * nl, 0.0);
  for (int n = 0; n < N; ++n)
    for (int k = 0; k < nz; ++k) {
      m.hnode[(size_t)n * nz + k] = m.zbar[k] - m.zbar[k + 1];
      m.hnode_new[(size_t)n * nz + k] = m.hnode[(size_t)n * nz + k];
      m.Z3[(size_t)n * nz + k] = m.Z[k];
    }
  for (int n = 0; n < N; ++n)
    for (int k = 0; k < nl; ++k) m.zbar3[(size_t)n * nl + k] = m.zbar[k];
  for (int e = 0; e < M; ++e)
    for (int k = 0; k < nz; ++k) m.helem[(size_t)e * nz + k] = m.zbar[k] - m.zbar[k + 1];
}

HostMesh* build_analytic(int nx, int ny, int nl, double Lx, double Ly, double depth, int periodic,
                         int flags, const double* zbar_in, const int* elem_nlev, std::string* err) {
  const int cluster_full = (flags & kClusterFull) ? 1 : 0;
  if (nx < 2 || ny < 2 || nl < 3 || (periodic && (nx < 3 || ny < 3))) {
    if (err) *err = "analytic mesh needs nx,ny >= 2 (3 if periodic) and nl >= 3";
    return nullptr;
  }
  auto* mp = new HostMesh();
  HostMesh& m = *mp;
  m.periodic = periodic;
  m.cluster_full = cluster_full;
  m.orient_left = (flags & kOrientLeft) ? 1 : 0;
  m.Lx = Lx;
  m.Ly = Ly;
  m.nl = nl;
  m.nz = nl - 1;
  Grid g;
  g.nx = nx;
  g.ny = ny;
  g.periodic = periodic != 0;
  g.nreal = periodic ? (nx - 1) * (ny - 1) : nx * ny;
  const int eDim = periodic ? (nx - 1) + (ny - 1) + 1 : 0;
  g.ntotal = g.nreal + eDim;
  const int NT = g.ntotal, N = g.nreal, M = 2 * (nx - 1) * (ny - 1);
  m.N = N;
  m.M = M;

  // Coordinates (lib/analytic_mesh.F90:268-305), halo copies included.
  const double dx = Lx / (double)(nx - 1), dy = Ly / (double)(ny - 1);
  std::vector<double> coord((size_t)2 * NT, 0.0);
  const int ni = periodic ? nx - 1 : nx, nj = periodic ? ny - 1 : ny;
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      int n = g.node(i, j);
      coord[2 * n] = (double)(i - 1) * dx / kREarth;
      coord[2 * n + 1] = (double)(j - 1) * dy / kREarth;
    }
  if (periodic) {
    for (int j = 1; j <= ny - 1; ++j) {
      int n = g.node(nx, j);
      coord[2 * n] = Lx / kREarth;
      coord[2 * n + 1] = (double)(j - 1) * dy / kREarth;
    }
    for (int i = 1; i <= nx - 1; ++i) {
      int n = g.node(i, ny);
      coord[2 * n] = (double)(i - 1) * dx / kREarth;
      coord[2 * n + 1] = Ly / kREarth;
    }
    coord[2 * (NT - 1)] = Lx / kREarth;
    coord[2 * (NT - 1) + 1] = Ly / kREarth;
  }

  // Elements, two per quad, in the reference's clockwise order (:310-354).
  std::vector<int> en((size_t)3 * M);
  for (int j = 1, e = 0; j <= ny - 1; ++j)
    for (int i = 1; i <= nx - 1; ++i, e += 2) {
      int n1 = g.node(i, j), n2 = g.node(i + 1, j), n3 = g.node(i + 1, j + 1), n4 = g.node(i, j + 1);
      en[3 * e] = n1; en[3 * e + 1] = n3; en[3 * e + 2] = n2;
      en[3 * e + 3] = n1; en[3 * e + 4] = n4; en[3 * e + 5] = n3;
    }

  // Levels (:359-373).
  m.zbar.resize(nl);
  m.Z.resize(nl - 1);
  for (int k = 1; k <= nl; ++k) m.zbar[k - 1] = zbar_in ? zbar_in[k - 1] : -(double)(k - 1) * depth / (double)(nl - 1);
  for (int k = 1; k <= nl - 1; ++k) m.Z[k - 1] = 0.5 * (m.zbar[k - 1] + m.zbar[k]);

  // Edges: horizontal, vertical, diagonal (:383-596); element quad index q(i,j).
  auto quad = [&](int i, int j) { return 2 * ((j - 1) * (nx - 1) + (i - 1)); };  // lower tri, 0-based
  std::vector<int> ed, et;
  if (periodic) {
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i + 1, j));
        et.push_back((j >= 2 ? quad(i, j - 1) : quad(i, ny - 1)) + 1); et.push_back(quad(i, j));
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i, j + 1));
        et.push_back(quad(i, j) + 1); et.push_back(i >= 2 ? quad(i - 1, j) : quad(nx - 1, j));
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i + 1, j + 1));
        et.push_back(quad(i, j) + 1); et.push_back(quad(i, j));
      }
    m.edges = ed;
    m.edge_tri = et;
    m.edge2D_in = (int)(ed.size() / 2);
  } else {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i + 1, j));
        et.push_back(j >= 2 ? quad(i, j - 1) + 1 : -1); et.push_back(j <= ny - 1 ? quad(i, j) : -1);
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i, j + 1));
        et.push_back(i <= nx - 1 ? quad(i, j) + 1 : -1); et.push_back(i >= 2 ? quad(i - 1, j) : -1);
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ed.push_back(g.node(i, j)); ed.push_back(g.node(i + 1, j + 1));
        et.push_back(quad(i, j) + 1); et.push_back(quad(i, j));
      }
    const int Eall = (int)(ed.size() / 2);
    for (int n = 0; n < Eall; ++n)  // valid element first (:533-539)
      if (et[2 * n] < 0 && et[2 * n + 1] >= 0) { et[2 * n] = et[2 * n + 1]; et[2 * n + 1] = -1; }
    m.edges.reserve(ed.size());
    m.edge_tri.reserve(et.size());
    for (int pass = 0; pass < 2; ++pass)  // internal edges first, then the wall (:541-588)
      for (int n = 0; n < Eall; ++n) {
        bool internal = et[2 * n] >= 0 && et[2 * n + 1] >= 0;
        if ((pass == 0) != internal) continue;
        m.edges.push_back(ed[2 * n]); m.edges.push_back(ed[2 * n + 1]);
        m.edge_tri.push_back(et[2 * n]); m.edge_tri.push_back(et[2 * n + 1]);
        if (pass == 0) m.edge2D_in = (int)(m.edges.size() / 2);
      }
  }
  const int E = (int)(m.edges.size() / 2);
  m.E = E;
  if (m.orient_left) {
    // The analytic grid puts edge_tri(1) to the right of horizontal and
    // vertical edges and to the left of diagonal ones; FESOM meshes keep it on
    // the left, which makes the upwind volume fluxes of a rotated-gradient
    // flow telescope around every node. Swap the two nodes where needed.
    for (int n = 0; n < E; ++n) {
      const int a = m.edges[2 * n], b = m.edges[2 * n + 1], el = m.edge_tri[2 * n];
      const double cx3 = (coord[2 * en[3 * el]] + coord[2 * en[3 * el + 1]] + coord[2 * en[3 * el + 2]]) / 3.0;
      const double cy3 = (coord[2 * en[3 * el] + 1] + coord[2 * en[3 * el + 1] + 1] + coord[2 * en[3 * el + 2] + 1]) / 3.0;
      const double dx0 = coord[2 * b] - coord[2 * a], dy0 = coord[2 * b + 1] - coord[2 * a + 1];
      double sx = cx3 - coord[2 * a], sy = cy3 - coord[2 * a + 1];
      if (periodic) {  // the element of a seam edge may sit across the domain
        const double px = Lx / kREarth, py = Ly / kREarth;
        if (sx > 0.5 * px) sx = sx - px;
        if (sx < -0.5 * px) sx = sx + px;
        if (sy > 0.5 * py) sy = sy - py;
        if (sy < -0.5 * py) sy = sy + py;
      }
      if (dx0 * sy - dy0 * sx < 0.0) std::swap(m.edges[2 * n], m.edges[2 * n + 1]);
    }
  }

  // Element and node levels; node columns reach the deepest adjacent element.
  m.nlevels.assign(M, nl);
  m.ulevels.assign(M, 1);
  std::vector<int> nlev_t(NT, nl), ulev_t(NT, 1);
  if (elem_nlev) {
    for (int e = 0; e < M; ++e) m.nlevels[e] = elem_nlev[e];
    std::fill(nlev_t.begin(), nlev_t.end(), 0);
    for (int e = 0; e < M; ++e)
      for (int k = 0; k < 3; ++k) {
        int r = g.real_of(en[3 * e + k]);
        nlev_t[r] = std::max(nlev_t[r], m.nlevels[e]);
      }
    for (int n = N; n < NT; ++n) nlev_t[n] = nlev_t[g.real_of(n)];
  }

  // test_tri (lib/oce_mesh.F90:1565-1615): orientation check, a no-op here.
  for (int e = 0; e < M; ++e) {
    int* el = &en[3 * e];
    double a0 = coord[2 * el[0]], a1 = coord[2 * el[0] + 1];
    double b0 = trim_cyclic(coord[2 * el[1]] - a0), b1 = coord[2 * el[1] + 1] - a1;
    double c0 = trim_cyclic(coord[2 * el[2]] - a0), c1 = coord[2 * el[2] + 1] - a1;
    if (b0 * c1 - b1 * c0 > 0.0) std::swap(el[1], el[2]);
  }

  // nod_in_elem2D before the periodic remap (lib/analytic_mesh.F90:675-694).
  std::vector<int> num_t, lst_t;
  int maxn_t = 0;
  detail::node_elem_lists(en, M, NT, NT, num_t, lst_t, maxn_t);

  // mesh_areas (lib/oce_mesh.F90:2043-2309), cartesian, no cavity.
  m.elem_area.assign(M, 0.0);
  for (int e = 0; e < M; ++e) {
    const int* el = &en[3 * e];
    const double ay = 1.0;
    double a0 = trim_cyclic(coord[2 * el[1]] - coord[2 * el[0]]) * ay;
    double a1 = coord[2 * el[1] + 1] - coord[2 * el[0] + 1];
    double b0 = trim_cyclic(coord[2 * el[2]] - coord[2 * el[0]]) * ay;
    double b1 = coord[2 * el[2] + 1] - coord[2 * el[0] + 1];
    m.elem_area[e] = 0.5 * std::fabs(a0 * b1 - b0 * a1);
  }
  std::vector<double> area_t((size_t)NT * nl, 0.0), asv_t((size_t)NT * nl, 0.0);
  for (int n = 0; n < NT; ++n)
    for (int j = 0; j < num_t[n]; ++j) {
      int e = lst_t[(size_t)n * maxn_t + j];
      for (int z = m.ulevels[e]; z <= m.nlevels[e] - 1; ++z)
        area_t[(size_t)n * nl + z - 1] = area_t[(size_t)n * nl + z - 1] + m.elem_area[e] / 3.0;
    }
  for (int n = 0; n < NT; ++n)
    for (int z = ulev_t[n]; z <= nlev_t[n] - 1; ++z) asv_t[(size_t)n * nl + z - 1] = area_t[(size_t)n * nl + z - 1];
  for (auto& v : m.elem_area) v = v * kREarth * kREarth;
  for (auto& v : area_t) v = v * kREarth * kREarth;
  for (auto& v : asv_t) v = v * kREarth * kREarth;

  // mesh_auxiliary_arrays (lib/oce_mesh.F90:2313-2534).
  std::vector<double> cx(M), cy(M);
  m.elem_cos.assign(M, 1.0);  // cartesian
  for (int e = 0; e < M; ++e) {
    const int* el = &en[3 * e];
    double ax[3] = {coord[2 * el[0]], coord[2 * el[1]], coord[2 * el[2]]};
    double amin = std::min(std::min(ax[0], ax[1]), ax[2]);
    for (double& v : ax) {
      if (v - amin >= kCyclic / 2.0) v = v - kCyclic;
      if (v - amin < -kCyclic / 2.0) v = v + kCyclic;
    }
    cx[e] = (ax[0] + ax[1] + ax[2]) / 3.0;
    cy[e] = (coord[2 * el[0] + 1] + coord[2 * el[1] + 1] + coord[2 * el[2] + 1]) / 3.0;
  }
  m.edge_dxdy.assign((size_t)2 * E, 0.0);
  m.edge_cross.assign((size_t)4 * E, 0.0);
  for (int n = 0; n < E; ++n) {
    int e1 = m.edges[2 * n], e2 = m.edges[2 * n + 1];
    m.edge_dxdy[2 * n] = trim_cyclic(coord[2 * e2] - coord[2 * e1]);
    m.edge_dxdy[2 * n + 1] = coord[2 * e2 + 1] - coord[2 * e1 + 1];
    double p0 = coord[2 * e1], p1 = coord[2 * e1 + 1], q0 = coord[2 * e2], q1 = coord[2 * e2 + 1];
    if (p0 - q0 > kCyclic / 2.0) p0 = p0 - kCyclic;
    if (p0 - q0 < -kCyclic / 2.0) q0 = q0 - kCyclic;
    const double ax = 0.5 * (p0 + q0), ay = 0.5 * (p1 + q1);
    for (int s = 0; s < 2; ++s) {
      int el = m.edge_tri[2 * n + s];
      if (el < 0) continue;  // edge_cross_dxdy(3:4) stays 0 on walls
      double b0 = trim_cyclic(cx[el] - ax), b1 = cy[el] - ay;
      b0 = b0 * m.elem_cos[el];
      m.edge_cross[4 * n + 2 * s] = b0 * kREarth;
      m.edge_cross[4 * n + 2 * s + 1] = b1 * kREarth;
    }
  }
  m.grad_sca.assign((size_t)6 * M, 0.0);
  for (int e = 0; e < M; ++e) {
    const int* el = &en[3 * e];
    double dX31 = m.elem_cos[e] * trim_cyclic(coord[2 * el[2]] - coord[2 * el[0]]);
    double dX21 = m.elem_cos[e] * trim_cyclic(coord[2 * el[1]] - coord[2 * el[0]]);
    double dY31 = coord[2 * el[2] + 1] - coord[2 * el[0] + 1];
    double dY21 = coord[2 * el[1] + 1] - coord[2 * el[0] + 1];
    double f = -(0.5 * kREarth / m.elem_area[e]);
    double* gs = &m.grad_sca[6 * e];
    gs[0] = (-dY31 + dY21) * f;
    gs[1] = dY31 * f;
    gs[2] = -dY21 * f;
    gs[3] = (dX31 - dX21) * f;
    gs[4] = -dX31 * f;
    gs[5] = dX21 * f;
  }

  // Periodic post-remap (lib/analytic_mesh.F90:736-827): minimum-image cross
  // distances, halo areas merged into the real nodes (halo order), halo
  // indices replaced by real ones.
  if (periodic) {
    const double hLx = 0.5 * Lx, hLy = 0.5 * Ly;
    for (int n = 0; n < E; ++n)
      for (int k = 0; k < 4; k += 2) {
        double v = m.edge_cross[4 * n + k];
        if (std::fabs(v) > hLx) m.edge_cross[4 * n + k] = v - std::copysign(Lx, v);
        v = m.edge_cross[4 * n + k + 1];
        if (std::fabs(v) > hLy) m.edge_cross[4 * n + k + 1] = v - std::copysign(Ly, v);
      }
    for (int h = N; h < NT; ++h) {
      int r = g.real_of(h);
      for (int z = 0; z < nl - 1; ++z) {
        area_t[(size_t)r * nl + z] = area_t[(size_t)r * nl + z] + area_t[(size_t)h * nl + z];
        asv_t[(size_t)r * nl + z] = asv_t[(size_t)r * nl + z] + asv_t[(size_t)h * nl + z];
      }
    }
    for (auto& v : en) v = g.real_of(v);
    for (auto& v : m.edges) v = g.real_of(v);
  }
  m.elem_nodes = en;
  m.coord.assign(coord.begin(), coord.begin() + 2 * (size_t)N);
  m.area.assign(area_t.begin(), area_t.begin() + (size_t)N * nl);
  m.areasvol.assign(asv_t.begin(), asv_t.begin() + (size_t)N * nl);
  m.nlev_nod.assign(nlev_t.begin(), nlev_t.begin() + N);
  m.ulev_nod.assign(ulev_t.begin(), ulev_t.begin() + N);

  // Element lists around the real nodes: un-remapped (the reference's lists,
  // built before the remap) or full (every element around the folded node).
  if (periodic && cluster_full) {
    detail::node_elem_lists(en, M, N, N, m.nie_num, m.nie, m.max_nie);
  } else {
    m.max_nie = maxn_t;
    m.nie_num.assign(num_t.begin(), num_t.begin() + N);
    m.nie.assign(lst_t.begin(), lst_t.begin() + (size_t)N * maxn_t);
  }
  // find_levels_min_e2n (lib/oce_mesh.F90:1522-1560)
  m.nlev_nod_min.assign(N, 0);
  m.ulev_nod_max.assign(N, 0);
  for (int n = 0; n < N; ++n) {
    int mn = 1 << 30, mx = -(1 << 30);
    for (int k = 0; k < m.nie_num[n]; ++k) {
      int e = m.nie[(size_t)n * m.max_nie + k];
      mn = std::min(mn, m.nlevels[e]);
      mx = std::max(mx, m.ulevels[e]);
    }
    m.nlev_nod_min[n] = mn;
    m.ulev_nod_max[n] = mx;
  }

  ale_from_zbar(m);

  // nboundary_lay (lib/oce_muscl_adv.F90:96-159)
  m.nboundary_lay.assign(N, nl - 1);
  for (int n = 0; n < E; ++n) {
    int t1 = m.edge_tri[2 * n], t2 = m.edge_tri[2 * n + 1], a = m.edges[2 * n], b = m.edges[2 * n + 1];
    if (t1 < 0 || t2 < 0) {
      m.nboundary_lay[a] = 0;
      m.nboundary_lay[b] = 0;
    } else {
      int v = std::min(m.nlevels[t1], m.nlevels[t2]) - 1;
      m.nboundary_lay[a] = std::min(m.nboundary_lay[a], v);
      m.nboundary_lay[b] = std::min(m.nboundary_lay[b], v);
    }
  }
  // up/downwind triangles (lib/oce_muscl_adv.F90:166-357)
  m.edge_updn.assign((size_t)2 * E, -1);
  for (int n = 0; n < E; ++n) {
    int e1 = m.edges[2 * n], e2 = m.edges[2 * n + 1];
    double x[2] = {m.coord[2 * e2] - m.coord[2 * e1], m.coord[2 * e2 + 1] - m.coord[2 * e1 + 1]};
    if (periodic) {
      const double px = Lx / kREarth, py = Ly / kREarth;
      if (x[0] > 0.5 * px) x[0] = x[0] - px;
      if (x[0] < -0.5 * px) x[0] = x[0] + px;
      if (x[1] > 0.5 * py) x[1] = x[1] - py;
      if (x[1] < -0.5 * py) x[1] = x[1] + py;
    }
    double mx[2] = {-x[0], -x[1]};
    m.edge_updn[2 * n] = detail::updn_search(m, e1, mx);
    m.edge_updn[2 * n + 1] = detail::updn_search(m, e2, x);
  }
  build_tables(m);
  if (flags & kVisitHilbert) visit_order_hilbert(m);
  return mp;
}

// Visit order of the edge kernels: by the edge's first-visited node (the
// lower node index without a node visit order), so that the horizontal,
// vertical and diagonal edges of a grid row are swept together.
static void edge_visit_order(HostMesh& m) {
  const int N = m.N, E = m.E;
  std::vector<int> rank;
  if ((int)m.node_order.size() == N) {
    rank.assign(N, 0);
    for (int i = 0; i < N; ++i) rank[m.node_order[i]] = i;
  }
  auto first = [&](int e) {
    const int a = m.edges[2 * e], b = m.edges[2 * e + 1];
    return rank.empty() ? std::min(a, b) : std::min(rank[a], rank[b]);
  };
  m.edge_order.resize(E);
  for (int e = 0; e < E; ++e) m.edge_order[e] = e;
  std::stable_sort(m.edge_order.begin(), m.edge_order.end(), [&](int a, int b) { return first(a) < first(b); });
}

void build_tables(HostMesh& m) {
  const int N = m.N, E = m.E;
  // Per-edge layer windows (1-based layers, nl = nlevels-1).
  m.edge_lev.assign((size_t)4 * E, 0);
  for (int e = 0; e < E; ++e) {
    int t1 = m.edge_tri[2 * e], t2 = m.edge_tri[2 * e + 1];
    m.edge_lev[4 * e + 0] = m.ulevels[t1];
    m.edge_lev[4 * e + 1] = m.nlevels[t1] - 1;
    m.edge_lev[4 * e + 2] = t2 >= 0 ? m.ulevels[t2] : 0;
    m.edge_lev[4 * e + 3] = t2 >= 0 ? m.nlevels[t2] - 1 : 0;
  }
  // Incident edges per node in ascending edge order: the order of the
  // reference's edge loops, so a gather reproduces its summation order.
  m.ne_ptr.assign(N + 1, 0);
  for (int e = 0; e < E; ++e) {
    m.ne_ptr[m.edges[2 * e] + 1]++;
    m.ne_ptr[m.edges[2 * e + 1] + 1]++;
  }
  for (int n = 0; n < N; ++n) m.ne_ptr[n + 1] += m.ne_ptr[n];
  m.ne_code.assign(m.ne_ptr[N], 0);
  m.ne_other.assign(m.ne_ptr[N], 0);
  m.ne_lo.assign(m.ne_ptr[N], 0);
  m.ne_hi.assign(m.ne_ptr[N], 0);
  std::vector<int> fill(m.ne_ptr.begin(), m.ne_ptr.end() - 1);
  for (int e = 0; e < E; ++e) {
    const int nu1 = m.edge_lev[4 * e], nl1 = m.edge_lev[4 * e + 1];
    const int nu2 = m.edge_lev[4 * e + 2], nl2 = m.edge_lev[4 * e + 3];
    const int hi = std::max(nl1, nl2), lo = nu2 > 0 ? std::min(nu1, nu2) : nu1;
    for (int r = 0; r < 2; ++r) {
      int n = m.edges[2 * e + r];
      m.ne_code[fill[n]] = 2 * e + r;
      m.ne_other[fill[n]] = m.edges[2 * e + 1 - r];
      m.ne_lo[fill[n]] = lo;
      m.ne_hi[fill[n]] = hi;
      fill[n]++;
    }
  }
  // nod_in_elem2D as CSR
  m.nie_ptr.assign(N + 1, 0);
  for (int n = 0; n < N; ++n) m.nie_ptr[n + 1] = m.nie_ptr[n] + m.nie_num[n];
  m.nie_idx.resize(m.nie_ptr[N]);
  for (int n = 0; n < N; ++n)
    for (int k = 0; k < m.nie_num[n]; ++k) m.nie_idx[m.nie_ptr[n] + k] = m.nie[(size_t)n * m.max_nie + k];
  // FCT cluster (lib/oce_adv_tra_fct.F90:129-184): the bound at node n, layer z
  // is the max over the elements in nod_in_elem2D(n) of the max over their
  // three nodes, or -1e3 for elements without layer z. Max is exact, so the
  // distinct nodes with the deepest layer that reaches them give the same value.
  m.cl_ptr.assign(N + 1, 0);
  m.cl_node.clear();
  m.cl_lev.clear();
  m.cl_minlev.assign(N, 0);
  for (int n = 0; n < N; ++n) {
    std::vector<std::pair<int, int>> acc;
    int minlev = 1 << 30;
    for (int k = 0; k < m.nie_num[n]; ++k) {
      int e = m.nie[(size_t)n * m.max_nie + k];
      int lev = m.nlevels[e] - 1;
      minlev = std::min(minlev, lev);
      for (int j = 0; j < 3; ++j) {
        int v = m.elem_nodes[3 * e + j];
        auto it = std::find_if(acc.begin(), acc.end(), [&](const std::pair<int, int>& p) { return p.first == v; });
        if (it == acc.end()) acc.push_back({v, lev});
        else it->second = std::max(it->second, lev);
      }
    }
    m.cl_minlev[n] = minlev;
    for (auto& p : acc) {
      m.cl_node.push_back(p.first);
      m.cl_lev.push_back(p.second);
    }
    m.cl_ptr[n + 1] = (int)m.cl_node.size();
  }
  edge_visit_order(m);
  // MUSCL gradient windows and edge lengths scaled to metres.
  m.edge_gm.assign((size_t)2 * E, -1);
  m.edge_dxa.assign((size_t)2 * E, 0.0);
  for (int e = 0; e < E; ++e) {
    int t1 = m.edge_tri[2 * e], t2 = m.edge_tri[2 * e + 1];
    double a = kREarth * m.elem_cos[t1];
    if (t2 >= 0) a = 0.5 * (a + kREarth * m.elem_cos[t2]);
    m.edge_dxa[2 * e] = m.edge_dxdy[2 * e] * a;
    m.edge_dxa[2 * e + 1] = m.edge_dxdy[2 * e + 1] * kREarth;
    if (!m.edge_updn.empty() && m.edge_updn[2 * e] >= 0 && m.edge_updn[2 * e + 1] >= 0) {
      int a1 = m.edges[2 * e], b1 = m.edges[2 * e + 1];
      m.edge_gm[2 * e] = std::max(m.ulev_nod_max[a1], m.ulev_nod_max[b1]);
      m.edge_gm[2 * e + 1] = std::min(m.nlev_nod_min[a1], m.nlev_nod_min[b1]);
    }
  }
}

}  // namespace fgb

namespace fgb {

namespace {
template <typename T>
void append_shift(std::vector<T>& dst, const std::vector<T>& src, T shift, bool keep_negative) {
  for (T v : src) dst.push_back((keep_negative && v < 0) ? v : v + shift);
}
// rows x ncol -> rows x ld, zero padding
void append_rows(std::vector<double>& dst, const std::vector<double>& src, size_t rows, int ncol, int ld) {
  for (size_t r = 0; r < rows; ++r) {
    dst.insert(dst.end(), src.begin() + r * ncol, src.begin() + (r + 1) * ncol);
    dst.insert(dst.end(), (size_t)(ld - ncol), 0.0);
  }
}
}  // namespace

HostMesh* union_meshes(const HostMesh* const* parts, int count, std::string* err) {
  if (count < 1 || !parts) {
    if (err) *err = "union of no meshes";
    return nullptr;
  }
  auto* up = new HostMesh();
  HostMesh& u = *up;
  const HostMesh* deepest = parts[0];
  u.periodic = 1;
  for (int p = 0; p < count; ++p) {
    const HostMesh& m = *parts[p];
    u.N += m.N;
    u.E += m.E;
    u.M += m.M;
    u.edge2D_in += m.edge2D_in;
    u.max_nie = std::max(u.max_nie, m.max_nie);
    if (m.nl > deepest->nl) deepest = &m;
    u.periodic = u.periodic && m.periodic;
  }
  u.nl = deepest->nl;
  u.nz = u.nl - 1;
  u.cluster_full = parts[0]->cluster_full;
  u.orient_left = parts[0]->orient_left;
  u.zbar = deepest->zbar;
  u.Z = deepest->Z;
  u.nie.assign((size_t)u.N * u.max_nie, -1);
  int no = 0, mo = 0;
  for (int p = 0; p < count; ++p) {
    const HostMesh& m = *parts[p];
    u.coord.insert(u.coord.end(), m.coord.begin(), m.coord.end());
    append_shift(u.elem_nodes, m.elem_nodes, no, false);
    append_shift(u.edges, m.edges, no, false);
    append_shift(u.edge_tri, m.edge_tri, mo, true);
    u.nlevels.insert(u.nlevels.end(), m.nlevels.begin(), m.nlevels.end());
    u.ulevels.insert(u.ulevels.end(), m.ulevels.begin(), m.ulevels.end());
    u.nlev_nod.insert(u.nlev_nod.end(), m.nlev_nod.begin(), m.nlev_nod.end());
    u.ulev_nod.insert(u.ulev_nod.end(), m.ulev_nod.begin(), m.ulev_nod.end());
    u.nlev_nod_min.insert(u.nlev_nod_min.end(), m.nlev_nod_min.begin(), m.nlev_nod_min.end());
    u.ulev_nod_max.insert(u.ulev_nod_max.end(), m.ulev_nod_max.begin(), m.ulev_nod_max.end());
    u.nie_num.insert(u.nie_num.end(), m.nie_num.begin(), m.nie_num.end());
    for (int n = 0; n < m.N; ++n)
      for (int k = 0; k < m.nie_num[n]; ++k)
        u.nie[(size_t)(no + n) * u.max_nie + k] = m.nie[(size_t)n * m.max_nie + k] + mo;
    u.elem_area.insert(u.elem_area.end(), m.elem_area.begin(), m.elem_area.end());
    append_rows(u.area, m.area, m.N, m.nl, u.nl);
    append_rows(u.areasvol, m.areasvol, m.N, m.nl, u.nl);
    u.edge_dxdy.insert(u.edge_dxdy.end(), m.edge_dxdy.begin(), m.edge_dxdy.end());
    u.edge_cross.insert(u.edge_cross.end(), m.edge_cross.begin(), m.edge_cross.end());
    u.elem_cos.insert(u.elem_cos.end(), m.elem_cos.begin(), m.elem_cos.end());
    u.grad_sca.insert(u.grad_sca.end(), m.grad_sca.begin(), m.grad_sca.end());
    append_rows(u.hnode, m.hnode, m.N, m.nz, u.nz);
    append_rows(u.hnode_new, m.hnode_new, m.N, m.nz, u.nz);
    append_rows(u.helem, m.helem, m.M, m.nz, u.nz);
    append_rows(u.Z3, m.Z3, m.N, m.nz, u.nz);
    append_rows(u.zbar3, m.zbar3, m.N, m.nl, u.nl);
    append_shift(u.edge_updn, m.edge_updn, mo, true);
    u.nboundary_lay.insert(u.nboundary_lay.end(), m.nboundary_lay.begin(), m.nboundary_lay.end());
    no += m.N;
    mo += m.M;
  }
  // each part keeps its own visit order, the parts one after another
  bool any_order = false;
  for (int p = 0; p < count; ++p) any_order = any_order || !parts[p]->node_order.empty();
  if (any_order) {
    int off = 0;
    for (int p = 0; p < count; ++p) {
      const HostMesh& m = *parts[p];
      for (int i = 0; i < m.N; ++i) u.node_order.push_back(off + (m.node_order.empty() ? i : m.node_order[i]));
      off += m.N;
    }
  }
  build_tables(u);
  return up;
}

namespace {

// Position of cell (x, y) of a side x side grid (side a power of two) along
// the Hilbert curve that fills it: two bits per level, the quadrant's place
// on the curve, with the cell's coordinates reflected and swapped into the
// quadrant's own frame before the next level (the curve's sub-squares are
// rotated copies of the whole).
uint64_t hilbert_index(uint32_t side, uint32_t x, uint32_t y) {
  uint64_t d = 0;
  for (uint32_t s = side / 2; s > 0; s /= 2) {
    const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
    d += (uint64_t)s * s * ((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = side - 1 - x;
        y = side - 1 - y;
      }
      std::swap(x, y);
    }
  }
  return d;
}

}  // namespace

void visit_order_hilbert(HostMesh& m) {
  const int N = m.N;
  if (N <= 0) return;
  double lo[2] = {m.coord[0], m.coord[1]}, hi[2] = {m.coord[0], m.coord[1]};
  for (int n = 0; n < N; ++n)
    for (int c = 0; c < 2; ++c) {
      lo[c] = std::min(lo[c], m.coord[2 * n + c]);
      hi[c] = std::max(hi[c], m.coord[2 * n + c]);
    }
  constexpr uint32_t kSide = 1u << 16;
  std::vector<std::pair<uint64_t, int>> key(N);
  for (int n = 0; n < N; ++n) {
    uint32_t q[2];
    for (int c = 0; c < 2; ++c) {
      const double span = hi[c] - lo[c];
      const double t = span > 0 ? (m.coord[2 * n + c] - lo[c]) / span : 0.0;
      q[c] = (uint32_t)std::min<double>(kSide - 1, std::max(0.0, t * (kSide - 1)));
    }
    key[n] = {hilbert_index(kSide, q[0], q[1]), n};
  }
  std::sort(key.begin(), key.end());
  m.node_order.resize(N);
  for (int i = 0; i < N; ++i) m.node_order[i] = key[i].second;
  edge_visit_order(m);
}

}  // namespace fgb
