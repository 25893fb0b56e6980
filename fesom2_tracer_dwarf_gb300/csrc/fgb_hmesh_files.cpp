// FESOM mesh files on the host: the global mesh of a mesh directory read as
// one partition, with the set-up of lib/oce_mesh.F90 mesh_setup (read_mesh,
// test_tri, load_edges, find_neighbors, find_levels, find_levels_min_e2n,
// mesh_areas, mesh_auxiliary_arrays) on the sphere, the ALE arrays of
// tracer_init_ale_arrays (lib/tracer_c_interface.F90:875-925) and the MUSCL
// set-up of lib/oce_muscl_adv.F90.
//
// The reference reads no namelist, so its defaults hold
// (lib/gen_modules_config.F90:81-88): cartesian = .false., force_rotation =
// .true., the Euler angles 50, 15, -90 passed to cos/sin as they are, and
// cyclic_length = 360 against radian coordinates (the trims never fire).
// The flags select FESOM2's namelist handling instead (no rotation, angles in
// degrees, cyclic_length = 2*pi).
//
// Compiled with -ffp-contract=off, statement order as in the reference.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "fgb_hmesh.hpp"

namespace fgb {
namespace {

// Record-oriented reader of a list-directed Fortran input file: `record(k)`
// takes the first k items of the next line (the rest of the line is skipped,
// as read(unit,*) does); `items(n)` takes n items across lines.
class ListFile {
 public:
  bool open(const std::string& path, std::string* err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
      if (err) *err = "can not open file " + path;
      return false;
    }
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf_.assign(n > 0 ? (size_t)n : 0, '\0');
    size_t got = n > 0 ? std::fread(&buf_[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    buf_.resize(got);
    path_ = path;
    pos_ = 0;
    return true;
  }
  // Next item of the current line; false at the end of the line.
  bool item_in_line(std::string& tok) {
    while (pos_ < buf_.size() && (buf_[pos_] == ' ' || buf_[pos_] == '\t' || buf_[pos_] == ',' || buf_[pos_] == '\r'))
      ++pos_;
    if (pos_ >= buf_.size() || buf_[pos_] == '\n') return false;
    size_t b = pos_;
    while (pos_ < buf_.size() && !std::strchr(" \t,\r\n", buf_[pos_])) ++pos_;
    tok.assign(buf_, b, pos_ - b);
    return true;
  }
  void next_line() {
    while (pos_ < buf_.size() && buf_[pos_] != '\n') ++pos_;
    if (pos_ < buf_.size()) ++pos_;
  }
  bool eof() const { return pos_ >= buf_.size(); }
  template <typename T>
  bool record(T* out, int k, std::string* err) {
    for (;;) {  // list-directed input skips empty lines
      size_t mark = pos_;
      std::string tok;
      if (item_in_line(tok)) {
        pos_ = mark;
        break;
      }
      if (eof()) return fail(err);
      next_line();
    }
    for (int i = 0; i < k; ++i) {
      std::string tok;
      if (!item_in_line(tok) || !parse(tok, out[i])) return fail(err);
    }
    next_line();
    return true;
  }
  template <typename T>
  bool items(T* out, long n, std::string* err) {
    for (long i = 0; i < n;) {
      std::string tok;
      if (item_in_line(tok)) {
        if (!parse(tok, out[i])) return fail(err);
        ++i;
      } else {
        if (eof()) return fail(err);
        next_line();
      }
    }
    next_line();
    return true;
  }

 private:
  bool fail(std::string* err) {
    if (err) *err = "unexpected end of data or bad value in " + path_;
    return false;
  }
  static bool parse(const std::string& t, int& v) {
    char* e = nullptr;
    errno = 0;
    long x = std::strtol(t.c_str(), &e, 10);
    if (errno || *e || x < -2147483647L || x > 2147483647L) return false;
    v = (int)x;
    return true;
  }
  static bool parse(const std::string& t, double& v) {
    std::string s = t;
    for (char& c : s)  // Fortran exponent letters
      if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
    char* e = nullptr;
    errno = 0;
    v = std::strtod(s.c_str(), &e);
    return !errno && !*e;
  }
  std::string buf_, path_;
  size_t pos_ = 0;
};

// set_mesh_transform_matrix and g2r, lib/gen_modules_rotate_grid.F90:12-88.
struct Rotation {
  double r[9];
  explicit Rotation(bool degrees) {
    double al = 50.0, be = 15.0, ga = -90.0;  // lib/gen_modules_config.F90:86-88
    if (degrees) {
      al = al * (kPiRef / 180.0);
      be = be * (kPiRef / 180.0);
      ga = ga * (kPiRef / 180.0);
    }
    r[0] = std::cos(ga) * std::cos(al) - std::sin(ga) * std::cos(be) * std::sin(al);
    r[1] = std::cos(ga) * std::sin(al) + std::sin(ga) * std::cos(be) * std::cos(al);
    r[2] = std::sin(ga) * std::sin(be);
    r[3] = -std::sin(ga) * std::cos(al) - std::cos(ga) * std::cos(be) * std::sin(al);
    r[4] = -std::sin(ga) * std::sin(al) + std::cos(ga) * std::cos(be) * std::cos(al);
    r[5] = std::cos(ga) * std::sin(be);
    r[6] = std::sin(be) * std::sin(al);
    r[7] = -std::sin(be) * std::cos(al);
    r[8] = std::cos(be);
  }
  void g2r(double glon, double glat, double& rlon, double& rlat) const {
    const double xg = std::cos(glat) * std::cos(glon), yg = std::cos(glat) * std::sin(glon), zg = std::sin(glat);
    const double xr = r[0] * xg + r[1] * yg + r[2] * zg;
    const double yr = r[3] * xg + r[4] * yg + r[5] * zg;
    const double zr = r[6] * xg + r[7] * yg + r[8] * zg;
    rlat = std::asin(zr);
    rlon = (yr == 0.0 && xr == 0.0) ? 0.0 : std::atan2(yr, xr);
  }
};

}  // namespace

HostMesh* build_from_files(const std::string& dir_in, int flags, std::string* err) {
  std::string dir = dir_in;
  if (!dir.empty() && dir.back() != '/') dir += '/';  // the reference appends names to MeshPath as given
  auto bad = [&](const std::string& msg) -> HostMesh* {
    if (err) *err = msg;
    return nullptr;
  };
  ListFile f;
  std::string e;

  // nod2d.out (read_mesh, lib/oce_mesh.F90:230-330)
  if (!f.open(dir + "nod2d.out", &e)) return bad(e);
  int N = 0;
  if (!f.record(&N, 1, &e)) return bad(e);
  if (N < 3) return bad("nod2d.out: fewer than 3 nodes");
  std::vector<double> lonlat((size_t)2 * N);
  for (int n = 0; n < N; ++n) {
    double rec[3];  // id, lon, lat (the coast flag is not used by the step)
    if (!f.record(rec, 3, &e)) return bad(e);
    lonlat[2 * n] = rec[1];
    lonlat[2 * n + 1] = rec[2];
  }
  // elem2d.out
  if (!f.open(dir + "elem2d.out", &e)) return bad(e);
  int M = 0;
  if (!f.record(&M, 1, &e)) return bad(e);
  if (M < 1) return bad("elem2d.out: no elements");
  std::vector<int> en((size_t)3 * M);
  for (int k = 0; k < M; ++k)
    if (!f.record(&en[3 * k], 3, &e)) return bad(e);
  // aux3d.out: levels (lib/oce_mesh.F90:425-455)
  if (!f.open(dir + "aux3d.out", &e)) return bad(e);
  int nl = 0;
  if (!f.record(&nl, 1, &e)) return bad(e);
  if (nl < 3) return bad("aux3d.out: number of levels is less than 3");
  std::vector<double> zbar(nl);
  if (!f.items(zbar.data(), nl, &e)) return bad(e);
  // edgenum.out, edges.out, edge_tri.out (load_edges, lib/oce_mesh.F90:1617-1848)
  if (!f.open(dir + "edgenum.out", &e)) return bad(e);
  int E = 0, Ein = 0;
  if (!f.record(&E, 1, &e) || !f.record(&Ein, 1, &e)) return bad(e);
  if (E < 3 || Ein < 0 || Ein > E) return bad("edgenum.out: bad edge counts");
  std::vector<int> edges((size_t)2 * E), edge_tri((size_t)2 * E);
  ListFile g;
  if (!f.open(dir + "edges.out", &e) || !g.open(dir + "edge_tri.out", &e)) return bad(e);
  for (int k = 0; k < E; ++k)
    if (!f.record(&edges[2 * k], 2, &e) || !g.record(&edge_tri[2 * k], 2, &e)) return bad(e);
  // elvls.out, nlvls.out (find_levels, lib/oce_mesh.F90:807-1001)
  std::vector<int> elvls(M), nlvls(N);
  if (!f.open(dir + "elvls.out", &e)) return bad(e);
  for (int k = 0; k < M; ++k)
    if (!f.record(&elvls[k], 1, &e)) return bad(e);
  if (!f.open(dir + "nlvls.out", &e)) return bad(e);
  for (int k = 0; k < N; ++k)
    if (!f.record(&nlvls[k], 1, &e)) return bad(e);
  return build_from_arrays(N, M, E, Ein, nl, lonlat.data(), en.data(), edges.data(), edge_tri.data(), elvls.data(),
                           nlvls.data(), zbar.data(), flags, err);
}

HostMesh* build_from_arrays(int N, int M, int E, int Ein, int nl, const double* lonlat, const int* elem,
                            const int* edges_in, const int* edge_tri_in, const int* elvls, const int* nlvls,
                            const double* zbar_in, int flags, std::string* err) {
  auto bad = [&](const std::string& msg) -> HostMesh* {
    if (err) *err = msg;
    return nullptr;
  };
  if (N < 3 || M < 1 || nl < 3 || E < 3 || Ein < 0 || Ein > E) return bad("bad mesh sizes");
  std::vector<int> en((size_t)3 * M);
  for (size_t i = 0; i < (size_t)3 * M; ++i) {
    if (elem[i] < 1 || elem[i] > N) return bad("elem2d.out: node index out of range");
    en[i] = elem[i] - 1;
  }
  auto* mp = new HostMesh();
  HostMesh& m = *mp;
  auto bad_m = [&](const std::string& msg) -> HostMesh* {
    delete mp;
    return bad(msg);
  };
  m.nl = nl;
  m.nz = nl - 1;
  m.zbar.assign(zbar_in, zbar_in + nl);
  if (m.zbar[1] > 0.0)  // zbar is negative (lib/oce_mesh.F90:447)
    for (double& z : m.zbar) z = -z;
  m.Z.resize(nl - 1);
  for (int k = 0; k < nl - 1; ++k) m.Z[k] = 0.5 * (m.zbar[k] + m.zbar[k + 1]);
  m.edges.resize((size_t)2 * E);
  m.edge_tri.resize((size_t)2 * E);
  for (int k = 0; k < E; ++k) {
    for (int j = 0; j < 2; ++j) {
      const int a = edges_in[2 * k + j], t = edge_tri_in[2 * k + j];
      if (a < 1 || a > N) return bad_m("edges.out: node index out of range");
      if (t > M) return bad_m("edge_tri.out: element index out of range");
      m.edges[2 * k + j] = a - 1;
      m.edge_tri[2 * k + j] = t > 0 ? t - 1 : -1;  // where (edge_tri < 0) edge_tri = 0
    }
    if (m.edge_tri[2 * k] < 0) return bad_m("edge_tri.out: an edge without its first element");
  }
  // levels (find_levels); ulevels = 1
  m.nlevels.assign(elvls, elvls + M);
  m.ulevels.assign(M, 1);
  m.nlev_nod.assign(nlvls, nlvls + N);
  m.ulev_nod.assign(N, 1);
  for (int k = 0; k < M; ++k)
    if (m.nlevels[k] < 2 || m.nlevels[k] > nl) return bad_m("elvls.out: levels outside 2..nl");
  for (int k = 0; k < N; ++k)
    if (m.nlev_nod[k] < 2 || m.nlev_nod[k] > nl) return bad_m("nlvls.out: levels outside 2..nl");
  m.N = N;
  m.M = M;
  m.E = E;
  m.edge2D_in = Ein;
  std::vector<double> ll(lonlat, lonlat + (size_t)2 * N);
  m.periodic = 0;
  m.cyclic = (flags & kFileCyclic2Pi) ? 2.0 * kPiRef : 360.0;
  const double cyc = m.cyclic;
  auto trim = [cyc](double b) {  // trim_cyclic_mp, lib/gen_modules_rotate_grid.F90:216-224
    if (b > cyc / 2.0) b = b - cyc;
    if (b < -cyc / 2.0) b = b + cyc;
    return b;
  };

  // coordinates: degrees -> radians, rotated when force_rotation (:296-310)
  const Rotation rot((flags & kFileEulerDegrees) != 0);
  const double rad = kPiRef / 180.0;  // lib/oce_modules.F90:20
  m.coord.resize((size_t)2 * N);
  for (int n = 0; n < N; ++n) {
    double x = ll[2 * n] * rad, y = ll[2 * n + 1] * rad;
    if (!(flags & kFileNoRotation)) {
      const double rx = x, ry = y;
      rot.g2r(rx, ry, x, y);
    }
    m.coord[2 * n] = x;
    m.coord[2 * n + 1] = y;
  }
  const std::vector<double>& coord = m.coord;

  // test_tri (lib/oce_mesh.F90:1565-1615)
  for (int k = 0; k < M; ++k) {
    int* el = &en[3 * k];
    const double a0 = coord[2 * el[0]], a1 = coord[2 * el[0] + 1];
    const double b0 = trim(coord[2 * el[1]] - a0), b1 = coord[2 * el[1] + 1] - a1;
    const double c0 = trim(coord[2 * el[2]] - a0), c1 = coord[2 * el[2] + 1] - a1;
    if (b0 * c1 - b1 * c0 > 0.0) std::swap(el[1], el[2]);
  }
  m.elem_nodes = en;
  // nod_in_elem2D (find_neighbors) and find_levels_min_e2n (lib/oce_mesh.F90:1522-1560)
  detail::node_elem_lists(en, M, N, N, m.nie_num, m.nie, m.max_nie);
  m.nlev_nod_min.assign(N, 0);
  m.ulev_nod_max.assign(N, 0);
  for (int n = 0; n < N; ++n) {
    int mn = 1 << 30, mx = -(1 << 30);
    for (int k = 0; k < m.nie_num[n]; ++k) {
      const int el = m.nie[(size_t)n * m.max_nie + k];
      mn = std::min(mn, m.nlevels[el]);
      mx = std::max(mx, m.ulevels[el]);
    }
    m.nlev_nod_min[n] = mn;
    m.ulev_nod_max[n] = mx;
  }

  // mesh_areas (lib/oce_mesh.F90:2043-2309), no cavity
  m.elem_area.assign(M, 0.0);
  for (int k = 0; k < M; ++k) {
    const int* el = &en[3 * k];
    double ay = (coord[2 * el[0] + 1] + coord[2 * el[1] + 1] + coord[2 * el[2] + 1]) / 3.0;
    ay = std::cos(ay);
    double a0 = trim(coord[2 * el[1]] - coord[2 * el[0]]), a1 = coord[2 * el[1] + 1] - coord[2 * el[0] + 1];
    double b0 = trim(coord[2 * el[2]] - coord[2 * el[0]]), b1 = coord[2 * el[2] + 1] - coord[2 * el[0] + 1];
    a0 = a0 * ay;
    b0 = b0 * ay;
    m.elem_area[k] = 0.5 * std::fabs(a0 * b1 - b0 * a1);
  }
  m.area.assign((size_t)N * nl, 0.0);
  m.areasvol.assign((size_t)N * nl, 0.0);
  for (int n = 0; n < N; ++n)
    for (int j = 0; j < m.nie_num[n]; ++j) {
      const int el = m.nie[(size_t)n * m.max_nie + j];
      for (int z = m.ulevels[el]; z <= m.nlevels[el] - 1; ++z)
        m.area[(size_t)n * nl + z - 1] = m.area[(size_t)n * nl + z - 1] + m.elem_area[el] / 3.0;
    }
  for (int n = 0; n < N; ++n)
    for (int z = m.ulev_nod[n]; z <= m.nlev_nod[n] - 1; ++z)
      m.areasvol[(size_t)n * nl + z - 1] = m.area[(size_t)n * nl + z - 1];
  for (auto& v : m.elem_area) v = v * kREarth * kREarth;
  for (auto& v : m.area) v = v * kREarth * kREarth;
  for (auto& v : m.areasvol) v = v * kREarth * kREarth;

  // mesh_auxiliary_arrays (lib/oce_mesh.F90:2313-2534): element centres
  // (elem_center :2021-2041), elem_cos, edge_dxdy, edge_cross_dxdy
  // (edge_center :2001-2019), gradient_sca.
  std::vector<double> cx(M), cy(M);
  m.elem_cos.resize(M);
  for (int k = 0; k < M; ++k) {
    const int* el = &en[3 * k];
    double ax[3] = {coord[2 * el[0]], coord[2 * el[1]], coord[2 * el[2]]};
    const double amin = std::min(std::min(ax[0], ax[1]), ax[2]);
    for (double& v : ax) {
      if (v - amin >= cyc / 2.0) v = v - cyc;
      if (v - amin < -cyc / 2.0) v = v + cyc;
    }
    cx[k] = (ax[0] + ax[1] + ax[2]) / 3.0;
    cy[k] = (coord[2 * el[0] + 1] + coord[2 * el[1] + 1] + coord[2 * el[2] + 1]) / 3.0;
    m.elem_cos[k] = std::cos(cy[k]);
  }
  m.edge_dxdy.assign((size_t)2 * E, 0.0);
  m.edge_cross.assign((size_t)4 * E, 0.0);
  for (int n = 0; n < E; ++n) {
    const int e1 = m.edges[2 * n], e2 = m.edges[2 * n + 1];
    m.edge_dxdy[2 * n] = trim(coord[2 * e2] - coord[2 * e1]);
    m.edge_dxdy[2 * n + 1] = coord[2 * e2 + 1] - coord[2 * e1 + 1];
    double p0 = coord[2 * e1], q0 = coord[2 * e2];
    if (p0 - q0 > cyc / 2.0) p0 = p0 - cyc;
    if (p0 - q0 < -cyc / 2.0) q0 = q0 - cyc;
    const double ax = 0.5 * (p0 + q0), ay = 0.5 * (coord[2 * e1 + 1] + coord[2 * e2 + 1]);
    for (int s = 0; s < 2; ++s) {
      const int el = m.edge_tri[2 * n + s];
      if (el < 0) continue;  // edge_cross_dxdy(3:4) = 0 on the coast
      double b0 = trim(cx[el] - ax), b1 = cy[el] - ay;
      b0 = b0 * m.elem_cos[el];
      m.edge_cross[4 * n + 2 * s] = b0 * kREarth;
      m.edge_cross[4 * n + 2 * s + 1] = b1 * kREarth;
    }
  }
  m.grad_sca.assign((size_t)6 * M, 0.0);
  for (int k = 0; k < M; ++k) {
    const int* el = &en[3 * k];
    const double dX31 = m.elem_cos[k] * trim(coord[2 * el[2]] - coord[2 * el[0]]);
    const double dX21 = m.elem_cos[k] * trim(coord[2 * el[1]] - coord[2 * el[0]]);
    const double dY31 = coord[2 * el[2] + 1] - coord[2 * el[0] + 1];
    const double dY21 = coord[2 * el[1] + 1] - coord[2 * el[0] + 1];
    const double fct = -(0.5 * kREarth / m.elem_area[k]);
    double* gs = &m.grad_sca[6 * k];
    gs[0] = (-dY31 + dY21) * fct;
    gs[1] = dY31 * fct;
    gs[2] = -dY21 * fct;
    gs[3] = (dX31 - dX21) * fct;
    gs[4] = -dX31 * fct;
    gs[5] = dX21 * fct;
  }

  ale_from_zbar(m);

  // nboundary_lay and the up/downwind triangles (lib/oce_muscl_adv.F90:96-357)
  m.nboundary_lay.assign(N, nl - 1);
  for (int n = 0; n < E; ++n) {
    const int t1 = m.edge_tri[2 * n], t2 = m.edge_tri[2 * n + 1], a = m.edges[2 * n], b = m.edges[2 * n + 1];
    if (t1 < 0 || t2 < 0) {
      m.nboundary_lay[a] = 0;
      m.nboundary_lay[b] = 0;
    } else {
      const int v = std::min(m.nlevels[t1], m.nlevels[t2]) - 1;
      m.nboundary_lay[a] = std::min(m.nboundary_lay[a], v);
      m.nboundary_lay[b] = std::min(m.nboundary_lay[b], v);
    }
  }
  m.edge_updn.assign((size_t)2 * E, -1);
  for (int n = 0; n < E; ++n) {
    const int e1 = m.edges[2 * n], e2 = m.edges[2 * n + 1];
    double x[2] = {trim(coord[2 * e2] - coord[2 * e1]), coord[2 * e2 + 1] - coord[2 * e1 + 1]};
    const double mx[2] = {-x[0], -x[1]};
    m.edge_updn[2 * n] = detail::updn_search(m, e1, mx);
    m.edge_updn[2 * n + 1] = detail::updn_search(m, e2, x);
  }
  build_tables(m);
  if (!(flags & kFileKeepOrder)) visit_order_hilbert(m);
  return mp;
}

}  // namespace fgb
