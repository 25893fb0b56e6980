// Derived-type binary restarts (see fgb_restart.hpp for the format).
#include "fgb_restart.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "fgb_hmesh.hpp"

namespace fgb {
namespace restart {

size_t Field::count() const {
  if (dims.empty()) return 0;
  size_t n = 1;
  for (int32_t d : dims) n *= d > 0 ? (size_t)d : 0;
  return n;
}

Field* Record::get(const std::string& name) {
  for (Field& f : fields)
    if (f.name == name) return &f;
  return nullptr;
}

const Field* Record::get(const std::string& name) const {
  for (const Field& f : fields)
    if (f.name == name) return &f;
  return nullptr;
}

Field& Record::add(const std::string& name, Kind kind, int rank) {
  Field f;
  f.name = name;
  f.kind = kind;
  f.rank = rank;
  if (kind == Kind::ArrI4 || kind == Kind::ArrR8) f.dims.assign(rank, 0);
  if (kind == Kind::C20) f.c.assign(20, ' ');
  fields.push_back(std::move(f));
  return fields.back();
}

// ---------------------------------------------------------------------------
// Record framing
// ---------------------------------------------------------------------------
bool read_record_file(const std::string& path, std::vector<uint8_t>* bytes, std::string* err) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) {
    *err = "cannot open " + path;
    return false;
  }
  bytes->clear();
  bool ok = true, more = true;
  while (ok && more) {
    int32_t lead = 0, trail = 0;
    if (std::fread(&lead, 4, 1, fp) != 1) {
      *err = path + ": missing record marker";
      ok = false;
      break;
    }
    const int64_t len = lead < 0 ? -(int64_t)lead : lead;
    const size_t at = bytes->size();
    bytes->resize(at + (size_t)len);
    if (len && std::fread(bytes->data() + at, 1, (size_t)len, fp) != (size_t)len) {
      *err = path + ": record shorter than its marker";
      ok = false;
      break;
    }
    if (std::fread(&trail, 4, 1, fp) != 1 || (trail < 0 ? -(int64_t)trail : trail) != len) {
      *err = path + ": record markers disagree";
      ok = false;
      break;
    }
    more = lead < 0;
  }
  if (ok && std::fgetc(fp) != EOF) {
    *err = path + ": bytes after the record (one record per file expected)";
    ok = false;
  }
  std::fclose(fp);
  return ok;
}

bool write_record_file(const std::string& path, const std::vector<uint8_t>& bytes, std::string* err,
                       int64_t max_sub) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) {
    *err = "cannot create " + path;
    return false;
  }
  const int64_t total = (int64_t)bytes.size();
  const int64_t nsub = total == 0 ? 1 : (total + max_sub - 1) / max_sub;
  bool ok = true;
  for (int64_t s = 0; s < nsub && ok; ++s) {
    const int64_t off = s * max_sub, len = std::min<int64_t>(max_sub, total - off);
    const int32_t lead = (int32_t)(s + 1 < nsub ? -len : len), trail = (int32_t)(s > 0 ? -len : len);
    ok = std::fwrite(&lead, 4, 1, fp) == 1 && (len == 0 || std::fwrite(bytes.data() + off, 1, (size_t)len, fp) == (size_t)len) &&
         std::fwrite(&trail, 4, 1, fp) == 1;
  }
  if (std::fclose(fp) != 0) ok = false;
  if (!ok) *err = "write failed: " + path;
  return ok;
}

// ---------------------------------------------------------------------------
// Field decoding / encoding
// ---------------------------------------------------------------------------
namespace {

struct Reader {
  explicit Reader(const std::vector<uint8_t>& bytes) : b(bytes) {}
  const std::vector<uint8_t>& b;
  size_t pos = 0;
  std::string err;
  bool need(size_t n, const std::string& what) {
    if (!err.empty()) return false;
    if (b.size() - pos < n) {
      err = "record ends inside " + what;
      return false;
    }
    return true;
  }
  template <typename T>
  T scalar(const std::string& what) {
    T v{};
    if (need(sizeof(T), what)) {
      std::memcpy(&v, b.data() + pos, sizeof(T));
      pos += sizeof(T);
    }
    return v;
  }
  void field(Field& f) {
    switch (f.kind) {
      case Kind::I4: f.i = scalar<int32_t>(f.name); break;
      case Kind::L4: f.i = scalar<int32_t>(f.name) != 0; break;
      case Kind::R8: f.r = scalar<double>(f.name); break;
      case Kind::C20:
        if (need(20, f.name)) {
          f.c.assign(reinterpret_cast<const char*>(b.data() + pos), 20);
          pos += 20;
        }
        break;
      case Kind::ArrI4:
      case Kind::ArrR8: {
        f.dims.assign(f.rank, 0);
        for (int d = 0; d < f.rank; ++d) {
          f.dims[d] = scalar<int32_t>(f.name);
          if (f.dims[d] < 0 && err.empty()) err = f.name + ": negative extent";
        }
        // the extents' product, refused once it exceeds what the record can hold
        const size_t w = f.kind == Kind::ArrI4 ? 4 : 8, cap = b.size() / w + 1;
        size_t n = 1;
        for (int32_t d : f.dims) {
          const size_t e = d > 0 ? (size_t)d : 0;
          if (e && n > cap / e) {
            if (err.empty()) err = f.name + ": extents larger than the record";
            n = 0;
            break;
          }
          n *= e;
        }
        if (n && need(n * w, f.name)) {
          if (f.kind == Kind::ArrI4) {
            f.vi.resize(n);
            std::memcpy(f.vi.data(), b.data() + pos, n * 4);
          } else {
            f.vr.resize(n);
            std::memcpy(f.vr.data(), b.data() + pos, n * 8);
          }
          pos += n * w;
        }
        break;
      }
    }
  }
};

struct Spec {
  const char* name;
  Kind kind;
  int rank;
};

// t_mesh, in the order of write_t_mesh (lib/MOD_MESH.F90:185-275).
const Spec kMesh[] = {
    {"nod2D", Kind::I4, 0}, {"ocean_area", Kind::R8, 0}, {"ocean_areawithcav", Kind::R8, 0},
    {"edge2D", Kind::I4, 0}, {"edge2D_in", Kind::I4, 0}, {"elem2D", Kind::I4, 0},
    {"elem2D_nodes", Kind::ArrI4, 2}, {"edges", Kind::ArrI4, 2}, {"edge_tri", Kind::ArrI4, 2},
    {"elem_edges", Kind::ArrI4, 2}, {"elem_area", Kind::ArrR8, 1}, {"edge_dxdy", Kind::ArrR8, 2},
    {"edge_cross_dxdy", Kind::ArrR8, 2}, {"elem_cos", Kind::ArrR8, 1}, {"metric_factor", Kind::ArrR8, 1},
    {"elem_neighbors", Kind::ArrI4, 2}, {"nod_in_elem2D", Kind::ArrI4, 2}, {"x_corners", Kind::ArrR8, 2},
    {"y_corners", Kind::ArrR8, 2}, {"nod_in_elem2D_num", Kind::ArrI4, 1}, {"depth", Kind::ArrR8, 1},
    {"gradient_vec", Kind::ArrR8, 2}, {"gradient_sca", Kind::ArrR8, 2}, {"bc_index_nod2D", Kind::ArrI4, 1},
    {"nl", Kind::I4, 0}, {"zbar", Kind::ArrR8, 1}, {"Z", Kind::ArrR8, 1}, {"elem_depth", Kind::ArrR8, 1},
    {"ulevels", Kind::ArrI4, 1}, {"ulevels_nod2D", Kind::ArrI4, 1}, {"ulevels_nod2D_max", Kind::ArrI4, 1},
    {"nlevels", Kind::ArrI4, 1}, {"nlevels_nod2D", Kind::ArrI4, 1}, {"nlevels_nod2D_min", Kind::ArrI4, 1},
    {"area", Kind::ArrR8, 2}, {"area_inv", Kind::ArrR8, 2}, {"areasvol", Kind::ArrR8, 2},
    {"areasvol_inv", Kind::ArrR8, 2}, {"mesh_resolution", Kind::ArrR8, 1}, {"cavity_flag_n", Kind::ArrI4, 1},
    {"cavity_flag_e", Kind::ArrI4, 1}, {"cavity_depth", Kind::ArrR8, 1},
    {"cavity_nrst_cavlpnt_xyz", Kind::ArrR8, 2}, {"ssh_stiff%dim", Kind::I4, 0}, {"ssh_stiff%nza", Kind::I4, 0},
    {"ssh_stiff%rowptr", Kind::ArrI4, 1}, {"ssh_stiff%colind", Kind::ArrI4, 1},
    {"ssh_stiff%values", Kind::ArrR8, 1}, {"ssh_stiff%colind_loc", Kind::ArrI4, 1},
    {"ssh_stiff%rowptr_loc", Kind::ArrI4, 1}, {"lump2d_south", Kind::ArrR8, 1},
    {"lump2d_north", Kind::ArrR8, 1}, {"ind_south", Kind::ArrI4, 1}, {"ind_north", Kind::ArrI4, 1},
    {"nn_size", Kind::I4, 0}, {"nn_num", Kind::ArrI4, 1}, {"nn_pos", Kind::ArrI4, 2}, {"hnode", Kind::ArrR8, 2},
    {"hnode_new", Kind::ArrR8, 2}, {"zbar_3d_n", Kind::ArrR8, 2}, {"Z_3d_n", Kind::ArrR8, 2},
    {"Z_3d_n_ib", Kind::ArrR8, 2}, {"helem", Kind::ArrR8, 2}, {"bottom_elem_thickness", Kind::ArrR8, 1},
    {"bottom_node_thickness", Kind::ArrR8, 1}, {"dhe", Kind::ArrR8, 1}, {"hbar", Kind::ArrR8, 1},
    {"hbar_old", Kind::ArrR8, 1}, {"zbar_n_bot", Kind::ArrR8, 1}, {"zbar_e_bot", Kind::ArrR8, 1},
    {"zbar_n_srf", Kind::ArrR8, 1}, {"zbar_e_srf", Kind::ArrR8, 1}, {"coriolis", Kind::ArrR8, 1},
    {"coriolis_node", Kind::ArrR8, 1}};

// com_struct (lib/MOD_PARTIT.F90:113-133): the fixed-size lists are written
// like allocatable ones (extent, then elements).
const Spec kCom[] = {{"rPEnum", Kind::I4, 0}, {"rPE", Kind::ArrI4, 1},   {"rptr", Kind::ArrI4, 1},
                     {"rlist", Kind::ArrI4, 1}, {"sPEnum", Kind::I4, 0}, {"sPE", Kind::ArrI4, 1},
                     {"sptr", Kind::ArrI4, 1},  {"slist", Kind::ArrI4, 1}, {"nreq", Kind::I4, 0}};
const char* const kComNames[] = {"com_nod2D", "com_elem2D", "com_elem2D_full"};
const Spec kPartit[] = {{"npes", Kind::I4, 0},          {"mype", Kind::I4, 0},          {"maxPEnum", Kind::I4, 0},
                        {"part", Kind::ArrI4, 1},        {"myDim_nod2D", Kind::I4, 0},   {"eDim_nod2D", Kind::I4, 0},
                        {"myList_nod2D", Kind::ArrI4, 1}, {"myDim_elem2D", Kind::I4, 0}, {"eDim_elem2D", Kind::I4, 0},
                        {"eXDim_elem2D", Kind::I4, 0},   {"myList_elem2D", Kind::ArrI4, 1},
                        {"myDim_edge2D", Kind::I4, 0},   {"eDim_edge2D", Kind::I4, 0},
                        {"myList_edge2D", Kind::ArrI4, 1}, {"pe_status", Kind::I4, 0}};

// t_tracer_data (lib/MOD_TRACER.F90:104-124) and t_tracer_work (:146-168).
const Spec kTracerData[] = {
    {"values", Kind::ArrR8, 2},       {"valuesold", Kind::ArrR8, 3},   {"valuesAB", Kind::ArrR8, 2},
    {"smooth_bh_tra", Kind::L4, 0},   {"gamma0_tra", Kind::R8, 0},     {"gamma1_tra", Kind::R8, 0},
    {"gamma2_tra", Kind::R8, 0},      {"i_vert_diff", Kind::L4, 0},    {"tra_adv_hor", Kind::C20, 0},
    {"tra_adv_ver", Kind::C20, 0},    {"tra_adv_lim", Kind::C20, 0},   {"tra_adv_ph", Kind::R8, 0},
    {"tra_adv_pv", Kind::R8, 0},      {"ID", Kind::I4, 0}};
const Spec kTracerWork[] = {
    {"work%del_ttf", Kind::ArrR8, 2},       {"work%del_ttf_advhoriz", Kind::ArrR8, 2},
    {"work%del_ttf_advvert", Kind::ArrR8, 2}, {"work%dvd_trflx_hor", Kind::ArrR8, 3},
    {"work%dvd_trflx_ver", Kind::ArrR8, 3}, {"work%fct_LO", Kind::ArrR8, 2},
    {"work%adv_flux_hor", Kind::ArrR8, 2},  {"work%adv_flux_ver", Kind::ArrR8, 2},
    {"work%fct_ttf_max", Kind::ArrR8, 2},   {"work%fct_ttf_min", Kind::ArrR8, 2},
    {"work%fct_plus", Kind::ArrR8, 2},      {"work%fct_minus", Kind::ArrR8, 2},
    {"work%edge_up_dn_grad", Kind::ArrR8, 3}, {"work%nboundary_lay", Kind::ArrI4, 1},
    {"work%edge_up_dn_tri", Kind::ArrI4, 2}};

// t_dyn (lib/MOD_DYN.F90:256-300) with t_solverinfo (:189-206) and
// t_dyn_work (:222-232).
const Spec kDynHead[] = {{"opt_visc", Kind::I4, 0},          {"visc_gamma0", Kind::R8, 0},
                         {"visc_gamma1", Kind::R8, 0},       {"visc_gamma2", Kind::R8, 0},
                         {"visc_easybsreturn", Kind::R8, 0}, {"use_ivertvisc", Kind::L4, 0},
                         {"momadv_opt", Kind::I4, 0},        {"use_freeslip", Kind::L4, 0},
                         {"use_wsplit", Kind::L4, 0},        {"wsplit_maxcfl", Kind::R8, 0},
                         {"use_ssh_se_subcycl", Kind::L4, 0},
                         {"solverinfo%ident", Kind::I4, 0},  {"solverinfo%maxiter", Kind::I4, 0},
                         {"solverinfo%restart", Kind::I4, 0}, {"solverinfo%fillin", Kind::I4, 0},
                         {"solverinfo%lutype", Kind::I4, 0}, {"solverinfo%droptol", Kind::R8, 0},
                         {"solverinfo%soltol", Kind::R8, 0}, {"solverinfo%rr", Kind::ArrR8, 1},
                         {"solverinfo%zz", Kind::ArrR8, 1},  {"solverinfo%pp", Kind::ArrR8, 1},
                         {"solverinfo%App", Kind::ArrR8, 1}, {"work%uvnode_rhs", Kind::ArrR8, 3},
                         {"work%u_c", Kind::ArrR8, 2},       {"work%v_c", Kind::ArrR8, 2},
                         {"work%u_b", Kind::ArrR8, 2},       {"work%v_b", Kind::ArrR8, 2},
                         {"uv", Kind::ArrR8, 3},             {"uv_rhs", Kind::ArrR8, 3},
                         {"uv_rhsAB", Kind::ArrR8, 4},       {"uvnode", Kind::ArrR8, 3},
                         {"w", Kind::ArrR8, 2},              {"w_e", Kind::ArrR8, 2},
                         {"w_i", Kind::ArrR8, 2},            {"cfl_z", Kind::ArrR8, 2}};
const Spec kDynGM[] = {{"fer_w", Kind::ArrR8, 2}, {"fer_uv", Kind::ArrR8, 3}};
const Spec kDynSE[] = {{"se_uvh", Kind::ArrR8, 3},           {"se_uvBT_rhs", Kind::ArrR8, 2},
                       {"se_uvBT_4AB", Kind::ArrR8, 2},      {"se_uvBT", Kind::ArrR8, 2},
                       {"se_uvBT_theta", Kind::ArrR8, 2},    {"se_uvBT_mean", Kind::ArrR8, 2},
                       {"se_uvBT_12", Kind::ArrR8, 2},       {"se_uvBT_stab_hvisc", Kind::ArrR8, 2},
                       {"se_uvBT_stab_bdrag", Kind::ArrR8, 1}};

template <size_t N>
void read_specs(Reader& rd, const Spec (&specs)[N], const std::string& prefix, Record* out) {
  for (const Spec& s : specs) {
    if (!rd.err.empty()) return;
    rd.field(out->add(prefix + s.name, s.kind, s.rank));
  }
}

template <size_t N>
void add_specs(const Spec (&specs)[N], const std::string& prefix, Record* out) {
  for (const Spec& s : specs) out->add(prefix + s.name, s.kind, s.rank);
}

bool finish(Reader& rd, const char* type, std::string* err) {
  if (rd.err.empty() && rd.pos != rd.b.size())
    rd.err = std::to_string(rd.b.size() - rd.pos) + " bytes left after the last field";
  if (!rd.err.empty()) {
    *err = std::string(type) + " record: " + rd.err;
    return false;
  }
  return true;
}

}  // namespace

bool decode_mesh(const std::vector<uint8_t>& b, Record* out, std::string* err) {
  Reader rd(b);
  out->fields.clear();
  read_specs(rd, kMesh, "", out);
  return finish(rd, "t_mesh", err);
}

bool decode_partit(const std::vector<uint8_t>& b, Record* out, std::string* err) {
  Reader rd(b);
  out->fields.clear();
  for (const char* c : kComNames) read_specs(rd, kCom, std::string(c) + "%", out);
  read_specs(rd, kPartit, "", out);
  return finish(rd, "t_partit", err);
}

bool decode_tracer(const std::vector<uint8_t>& b, Record* out, std::string* err) {
  Reader rd(b);
  out->fields.clear();
  Field& nt = out->add("num_tracers", Kind::I4);
  rd.field(nt);
  if (rd.err.empty() && (nt.i < 0 || nt.i > 100000)) rd.err = "implausible num_tracers " + std::to_string(nt.i);
  for (int t = 0; t < nt.i && rd.err.empty(); ++t) read_specs(rd, kTracerData, "data(" + std::to_string(t + 1) + ")%", out);
  read_specs(rd, kTracerWork, "", out);
  return finish(rd, "t_tracer", err);
}

bool decode_dynamics(const std::vector<uint8_t>& b, Record* out, std::string* err, bool fer_gm) {
  Reader rd(b);
  out->fields.clear();
  read_specs(rd, kDynHead, "", out);
  if (fer_gm) read_specs(rd, kDynGM, "", out);
  const Field* se = out->get("use_ssh_se_subcycl");
  if (rd.err.empty() && se && se->i) read_specs(rd, kDynSE, "", out);
  return finish(rd, "t_dynamics", err);
}

std::vector<uint8_t> encode(const Record& r) {
  std::vector<uint8_t> b;
  auto put = [&](const void* p, size_t n) {
    const uint8_t* q = static_cast<const uint8_t*>(p);
    b.insert(b.end(), q, q + n);
  };
  for (const Field& f : r.fields) {
    switch (f.kind) {
      case Kind::I4: put(&f.i, 4); break;
      case Kind::L4: {
        const int32_t v = f.i ? 1 : 0;
        put(&v, 4);
        break;
      }
      case Kind::R8: put(&f.r, 8); break;
      case Kind::C20: {
        std::string s = f.c.substr(0, 20);
        s.resize(20, ' ');
        put(s.data(), 20);
        break;
      }
      case Kind::ArrI4:
      case Kind::ArrR8: {
        for (int d = 0; d < f.rank; ++d) {
          const int32_t e = d < (int)f.dims.size() ? f.dims[d] : 0;
          put(&e, 4);
        }
        const size_t n = f.count();
        if (f.kind == Kind::ArrI4) put(f.vi.data(), n * 4);
        else put(f.vr.data(), n * 8);
        break;
      }
    }
  }
  return b;
}

// ---------------------------------------------------------------------------
// Records of a state <-> host mesh
// ---------------------------------------------------------------------------
namespace {

void set_i(Record& r, const char* name, int32_t v) { r.get(name)->i = v; }
void set_r(Record& r, const char* name, double v) { r.get(name)->r = v; }

void set_arr(Record& r, const std::string& name, std::vector<int32_t> dims, const std::vector<int>& v, int shift = 0) {
  Field* f = r.get(name);
  f->dims = std::move(dims);
  f->vi.resize(f->count());
  for (size_t i = 0; i < f->vi.size(); ++i) f->vi[i] = v[i] + shift;
}

void set_arr(Record& r, const std::string& name, std::vector<int32_t> dims, const std::vector<double>& v) {
  Field* f = r.get(name);
  f->dims = std::move(dims);
  f->vr.assign(v.begin(), v.begin() + f->count());
}

// 0-based index with -1 for none <-> 1-based with 0 for none.
std::vector<int> to_fortran_opt(const std::vector<int>& v) {
  std::vector<int> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = v[i] >= 0 ? v[i] + 1 : 0;
  return o;
}

}  // namespace

Record mesh_record(const HostMesh& m) {
  Record r;
  add_specs(kMesh, "", &r);
  const int N = m.N, M = m.M, E = m.E, nl = m.nl, nz = m.nz;
  set_i(r, "nod2D", N);
  set_i(r, "edge2D", E);
  set_i(r, "edge2D_in", m.edge2D_in);
  set_i(r, "elem2D", M);
  set_i(r, "nl", nl);
  double ocean = 0.0;
  for (int n = 0; n < N; ++n) ocean += m.area[(size_t)n * nl];
  set_r(r, "ocean_area", ocean);
  set_r(r, "ocean_areawithcav", ocean);
  set_arr(r, "elem2D_nodes", {3, M}, m.elem_nodes, 1);
  set_arr(r, "edges", {2, E}, m.edges, 1);
  set_arr(r, "edge_tri", {2, E}, to_fortran_opt(m.edge_tri));
  set_arr(r, "elem_area", {M}, m.elem_area);
  set_arr(r, "edge_dxdy", {2, E}, m.edge_dxdy);
  set_arr(r, "edge_cross_dxdy", {4, E}, m.edge_cross);
  set_arr(r, "elem_cos", {M}, m.elem_cos);
  set_arr(r, "nod_in_elem2D", {m.max_nie, N}, to_fortran_opt(m.nie));
  set_arr(r, "nod_in_elem2D_num", {N}, m.nie_num);
  set_arr(r, "gradient_sca", {6, M}, m.grad_sca);
  set_arr(r, "zbar", {nl}, m.zbar);
  set_arr(r, "Z", {nz}, m.Z);
  set_arr(r, "ulevels", {M}, m.ulevels);
  set_arr(r, "ulevels_nod2D", {N}, m.ulev_nod);
  set_arr(r, "ulevels_nod2D_max", {N}, m.ulev_nod_max);
  set_arr(r, "nlevels", {M}, m.nlevels);
  set_arr(r, "nlevels_nod2D", {N}, m.nlev_nod);
  set_arr(r, "nlevels_nod2D_min", {N}, m.nlev_nod_min);
  set_arr(r, "area", {nl, N}, m.area);
  set_arr(r, "areasvol", {nl, N}, m.areasvol);
  set_arr(r, "hnode", {nz, N}, m.hnode);
  set_arr(r, "hnode_new", {nz, N}, m.hnode_new);
  set_arr(r, "zbar_3d_n", {nl, N}, m.zbar3);
  set_arr(r, "Z_3d_n", {nz, N}, m.Z3);
  set_arr(r, "helem", {nz, M}, m.helem);
  return r;
}

Record partit_record(int N, int M, int E) {
  Record r;
  for (const char* c : kComNames) {
    add_specs(kCom, std::string(c) + "%", &r);
    const std::string p = std::string(c) + "%";
    // no neighbouring partitions: the fixed lists at their declared sizes (32, 33, 32, 32), zero
    for (const char* nm : {"rPE", "sPE", "sptr"}) {
      Field* f = r.get(p + nm);
      f->dims = {32};
      f->vi.assign(32, 0);
    }
    Field* rp = r.get(p + "rptr");
    rp->dims = {33};
    rp->vi.assign(33, 0);
  }
  add_specs(kPartit, "", &r);
  auto iota1 = [](int n) {
    std::vector<int> v(n);
    for (int i = 0; i < n; ++i) v[i] = i + 1;
    return v;
  };
  set_i(r, "npes", 1);
  set_i(r, "mype", 0);
  set_i(r, "maxPEnum", 100);  // the type's default (lib/MOD_PARTIT.F90:53)
  set_i(r, "myDim_nod2D", N);
  set_arr(r, "myList_nod2D", {N}, iota1(N));
  set_i(r, "myDim_elem2D", M);
  set_arr(r, "myList_elem2D", {M}, iota1(M));
  set_i(r, "myDim_edge2D", E);
  set_arr(r, "myList_edge2D", {E}, iota1(E));
  return r;
}

Record tracer_record(const HostMesh& m, int ntracers) {
  Record r;
  r.add("num_tracers", Kind::I4).i = ntracers;
  const int N = m.N, E = m.E, nz = m.nz;
  const std::vector<double> zeros((size_t)nz * N, 0.0);
  for (int t = 0; t < ntracers; ++t) {
    const std::string p = "data(" + std::to_string(t + 1) + ")%";
    add_specs(kTracerData, p, &r);
    set_arr(r, p + "values", {nz, N}, zeros);
    set_arr(r, p + "valuesAB", {nz, N}, zeros);
    r.get(p + "ID")->i = t + 1;
    r.get(p + "tra_adv_ph")->r = 1.0;
    r.get(p + "tra_adv_pv")->r = 1.0;
  }
  add_specs(kTracerWork, "", &r);
  set_arr(r, "work%del_ttf", {nz, N}, zeros);
  set_arr(r, "work%nboundary_lay", {N}, m.nboundary_lay);
  set_arr(r, "work%edge_up_dn_tri", {2, E}, to_fortran_opt(m.edge_updn));
  return r;
}

Record dynamics_record(int nl, int N, int M) {
  Record r;
  add_specs(kDynHead, "", &r);
  // the types' defaults (lib/MOD_DYN.F90:9-17, :67-90)
  set_i(r, "opt_visc", 5);
  set_r(r, "visc_gamma0", 0.03);
  set_r(r, "visc_gamma1", 0.1);
  set_r(r, "visc_gamma2", 0.285);
  set_r(r, "visc_easybsreturn", 1.5);
  set_i(r, "use_ivertvisc", 1);
  set_i(r, "momadv_opt", 2);
  set_r(r, "wsplit_maxcfl", 1.0);
  set_i(r, "solverinfo%ident", 1);
  set_i(r, "solverinfo%maxiter", 2000);
  set_i(r, "solverinfo%restart", 15);
  set_i(r, "solverinfo%fillin", 3);
  set_i(r, "solverinfo%lutype", 2);
  set_r(r, "solverinfo%droptol", 1.e-8);
  set_r(r, "solverinfo%soltol", 1e-5);
  const int nz = nl - 1;
  set_arr(r, "uv", {2, nz, M}, std::vector<double>((size_t)2 * nz * M, 0.0));
  for (const char* w : {"w", "w_e", "w_i"}) set_arr(r, w, {nl, N}, std::vector<double>((size_t)nl * N, 0.0));
  return r;
}

HostMesh* mesh_from_records(const Record& r, const Record* tr, std::string* err) {
  auto bad = [&](const std::string& what) -> HostMesh* {
    *err = "t_mesh restart: " + what;
    return nullptr;
  };
  auto arr = [&](const std::string& name, std::vector<int32_t> dims) -> const Field* {
    const Field* f = r.get(name);
    if (!f || f->dims != dims) return nullptr;
    return f;
  };
  const Field *fn = r.get("nod2D"), *fe = r.get("edge2D"), *fm = r.get("elem2D"), *fl = r.get("nl");
  const Field* fen = r.get("elem2D_nodes");
  if (!fn || !fe || !fm || !fl || !fen) return bad("missing sizes");
  // Array extents are the local (partition) sizes; a one-process restart has the global ones.
  const int M = fen->dims.size() == 2 ? fen->dims[1] : -1;
  const Field* fed = r.get("edges");
  const int E = fed && fed->dims.size() == 2 ? fed->dims[1] : -1;
  const Field* fnl = r.get("nlevels_nod2D");
  const int N = fnl && fnl->dims.size() == 1 ? fnl->dims[0] : -1;
  const int nl = fl->i, nz = nl - 1;
  if (N < 3 || M < 1 || E < 3 || nl < 3) return bad("bad sizes");
  const Field *en = arr("elem2D_nodes", {3, M}), *ed = arr("edges", {2, E}), *et = arr("edge_tri", {2, E});
  const Field *ea = arr("elem_area", {M}), *dxdy = arr("edge_dxdy", {2, E}), *cr = arr("edge_cross_dxdy", {4, E});
  const Field *ec = arr("elem_cos", {M}), *gs = arr("gradient_sca", {6, M}), *nie_num = arr("nod_in_elem2D_num", {N});
  const Field* nie = r.get("nod_in_elem2D");
  const Field *zb = arr("zbar", {nl}), *Z = arr("Z", {nz}), *ul = arr("ulevels", {M}), *uln = arr("ulevels_nod2D", {N});
  const Field *ulx = arr("ulevels_nod2D_max", {N}), *nle = arr("nlevels", {M}), *nln = arr("nlevels_nod2D", {N});
  const Field *nlm = arr("nlevels_nod2D_min", {N}), *ar = arr("area", {nl, N}), *asv = arr("areasvol", {nl, N});
  const Field *hn = arr("hnode", {nz, N}), *hnn = arr("hnode_new", {nz, N}), *z3 = arr("zbar_3d_n", {nl, N});
  const Field *Z3 = arr("Z_3d_n", {nz, N}), *he = arr("helem", {nz, M});
  const Field* need[] = {en, ed, et, ea, dxdy, cr, ec, gs, nie_num, zb, Z, ul, uln, ulx, nle, nln, nlm, ar, asv, hn, hnn, z3, Z3, he};
  for (const Field* f : need)
    if (!f) return bad("an array the step needs is missing or has other extents than the mesh sizes");
  if (!nie || nie->dims.size() != 2 || nie->dims[1] != N || nie->dims[0] < 1) return bad("nod_in_elem2D extents");
  HostMesh* mp = new HostMesh();
  HostMesh& m = *mp;
  m.N = N;
  m.E = E;
  m.M = M;
  m.nl = nl;
  m.nz = nz;
  m.edge2D_in = r.get("edge2D_in") ? r.get("edge2D_in")->i : E;
  m.max_nie = nie->dims[0];
  auto from1 = [](const std::vector<int32_t>& v) {
    std::vector<int> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = v[i] > 0 ? v[i] - 1 : -1;
    return o;
  };
  m.elem_nodes = from1(en->vi);
  m.edges = from1(ed->vi);
  m.edge_tri = from1(et->vi);
  m.nie = from1(nie->vi);
  m.nie_num.assign(nie_num->vi.begin(), nie_num->vi.end());
  m.nlevels.assign(nle->vi.begin(), nle->vi.end());
  m.ulevels.assign(ul->vi.begin(), ul->vi.end());
  m.nlev_nod.assign(nln->vi.begin(), nln->vi.end());
  m.ulev_nod.assign(uln->vi.begin(), uln->vi.end());
  m.nlev_nod_min.assign(nlm->vi.begin(), nlm->vi.end());
  m.ulev_nod_max.assign(ulx->vi.begin(), ulx->vi.end());
  m.elem_area = ea->vr;
  m.edge_dxdy = dxdy->vr;
  m.edge_cross = cr->vr;
  m.elem_cos = ec->vr;
  m.grad_sca = gs->vr;
  m.zbar = zb->vr;
  m.Z = Z->vr;
  m.area = ar->vr;
  m.areasvol = asv->vr;
  m.hnode = hn->vr;
  m.hnode_new = hnn->vr;
  m.zbar3 = z3->vr;
  m.Z3 = Z3->vr;
  m.helem = he->vr;
  for (int v : m.elem_nodes)
    if (v < 0 || v >= N) {
      delete mp;
      return bad("element node index out of range");
    }
  for (int e = 0; e < E; ++e)
    if (m.edges[2 * e] < 0 || m.edges[2 * e] >= N || m.edges[2 * e + 1] < 0 || m.edges[2 * e + 1] >= N ||
        m.edge_tri[2 * e] < 0 || m.edge_tri[2 * e] >= M || m.edge_tri[2 * e + 1] >= M) {
      delete mp;
      return bad("edge index out of range");
    }
  for (int v : m.nie)
    if (v >= M) {
      delete mp;
      return bad("nod_in_elem2D index out of range");
    }
  // The MUSCL tables of the tracer restart (muscl_adv_init's results), or
  // nboundary_lay as muscl_adv_init forms it (lib/oce_muscl_adv.F90:96-119)
  // and no up/downwind triangles when there is none.
  const Field* nb = tr ? tr->get("work%nboundary_lay") : nullptr;
  const Field* ud = tr ? tr->get("work%edge_up_dn_tri") : nullptr;
  if (nb && nb->dims == std::vector<int32_t>{N}) {
    m.nboundary_lay.assign(nb->vi.begin(), nb->vi.end());
  } else {
    m.nboundary_lay.assign(N, nl - 1);
    for (int e = 0; e < E; ++e) {
      const int t1 = m.edge_tri[2 * e], t2 = m.edge_tri[2 * e + 1], a = m.edges[2 * e], b = m.edges[2 * e + 1];
      const int v = (t1 < 0 || t2 < 0) ? 0 : std::min(m.nlevels[t1], m.nlevels[t2]) - 1;
      m.nboundary_lay[a] = std::min(m.nboundary_lay[a], v);
      m.nboundary_lay[b] = std::min(m.nboundary_lay[b], v);
    }
  }
  if (ud && ud->dims == std::vector<int32_t>{2, E}) {
    m.edge_updn = from1(ud->vi);
    for (int v : m.edge_updn)
      if (v >= M) {
        delete mp;
        return bad("edge_up_dn_tri index out of range");
      }
  } else {
    m.edge_updn.assign((size_t)2 * E, -1);
  }
  build_tables(m);
  return mp;
}

bool write_meta(const std::string& path, int cstep, int ctime, int cyear, bool tracers, bool dynamics,
                std::string* err) {
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) {
    *err = "cannot create " + path;
    return false;
  }
  // lib/io_restart_derivedtype.F90:57-59 and the '!   t_<type>' lines after each file
  std::fprintf(fp, "%d\n%d\n! year: %d\n!   t_mesh\n!   t_partit\n", cstep, ctime, cyear);
  if (tracers) std::fprintf(fp, "!   t_tracer\n");
  if (dynamics) std::fprintf(fp, "!   t_dynamics\n");
  const bool ok = std::fclose(fp) == 0;
  if (!ok) *err = "write failed: " + path;
  return ok;
}

}  // namespace restart
}  // namespace fgb
