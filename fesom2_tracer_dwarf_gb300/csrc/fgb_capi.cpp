// The reference's C interface (lib/tracer_c_interface.F90) on the GB300
// engine: one module-global system, host copies of what the caller sets,
// device buffers owned by the library, the step launched on the engine.
//
// Behaviour kept from the reference (a caller relinking against this
// library sees the same results and status codes):
//  - tracer_advect_step advances tracer 1 only; it zeroes the advective
//    tendencies but not del_ttf, which accumulates across calls (:179-214);
//  - tracer_set_velocity stores uv as (nl-1,edge2D,2) and the step reads the
//    same memory as vel(2,nl-1,elem2D) (:697 vs lib/oce_adv_tra_driver.F90:42);
//    w_e and w_i are zero (:735-736), so the low-order vertical flux and,
//    without FCT, the whole vertical advection see w_e = 0;
//  - valuesAB is set by tracer_set_values only (frozen time level);
//  - tracer_set_thickness sets hnode_new only; tracer_init_ale_arrays sets
//    hnode, hnode_new and helem from zbar.
//  - tracer_load_mesh_from_files reads the FESOM mesh files of the directory
//    as one partition (the reference reads dist_<npes>/ partition lists with
//    MPI; a single-GPU library owns every node), with the reference's
//    geometry defaults; a missing '/' at the end of the path is added.
//  - tracer_init / tracer_load_mesh_partition read, and tracer_finalize
//    writes, the derived-type binary restarts of <dir>/np1/ (one process:
//    npes = 1, rank text "0"; fgb_restart.hpp has the format). After
//    tracer_init the step uses the restart's w_e, w_i (under use_wsplit)
//    and del_ttf, as the reference's step uses global_dyn and the tracer
//    work arrays; tracer_set_velocity zeroes w_e and w_i again (:735-736).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"
#include "fgb_restart.hpp"

namespace {

struct Tracer {
  std::vector<double> values, valuesAB;  // (nl-1, node_size)
  int hor = FGB_HOR_UPW1, ver = FGB_VER_UPW1, lim = FGB_LIM_NONE;
  double ph = 1.0, pv = 1.0;
};

struct State {
  bool initialized = false;
  int mpi_comm = 0, npes = 1;
  int nl = 0, nod2D = 0, edge2D = 0, elem2D = 0;  // tracer_set_mesh_dims
  int myDim = 0, eDim = 0;                        // tracer_set_partition
  fgb_hmesh* hmesh = nullptr;
  fgb_mesh* dmesh = nullptr;
  std::vector<int> set_nlev, set_ulev;            // tracer_set_levels
  bool have_hnode = false, have_hnode_new = false, have_helem = false;
  std::vector<double> hnode, hnode_new, helem;    // host copies (nl-1, n)
  int ab_order = 2;
  std::vector<Tracer> tr;
  bool have_uv = false, have_w = false;
  int uv_nl = 0, uv_edge2D = 0;
  std::vector<double> uv, w;                      // (nl-1,edge2D,2), (nl,nod2D)
  // from a restart (t_dynamics): w_e, w_i (nl,nod2D) and use_wsplit; del_ttf (nl-1,nod2D)
  bool have_we = false, use_wsplit = false, del_pending = false;
  std::vector<double> we, wi, del;
  // the records a restart was read from: written back with the state's arrays
  bool from_restart = false;
  fgb::restart::Record rmesh, rpartit, rtracer, rdyn;
  int precision = FGB_FP64;
  bool input_checks = false;  // tracer_set_input_checks
  // device
  void *dT = nullptr, *dTA = nullptr, *dvel = nullptr, *dw = nullptr, *dwe = nullptr, *ddel = nullptr;
  void *dwi = nullptr, *dws = nullptr;
  long long ws_bytes = 0;
  bool device_ready = false;   // device buffers allocated for the current configuration
  bool mesh_dirty = true;      // levels or thicknesses changed: rebuild the device mesh
  bool inputs_dirty = true;    // fields changed since the last upload
  bool values_on_device = false;  // tracer 1 values newer on the device than on the host
  int dev_precision = -1;
};

State g;

int fail(const char* msg) {
  std::fprintf(stderr, "### error: %s\n", msg);
  fgb::set_error(msg);
  return -1;
}

std::string c2s(const char* s) {
  std::string out;
  if (!s) return out;
  for (int i = 0; i < 4096 && s[i]; ++i) out.push_back(s[i]);  // MAX_PATH, lib/oce_modules.F90:16
  return out;
}

bool dir_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

void free_device() {
  void* ps[] = {g.dT, g.dTA, g.dvel, g.dw, g.dwe, g.ddel, g.dwi, g.dws};
  for (void* p : ps)
    if (p) cudaFree(p);
  g.dT = g.dTA = g.dvel = g.dw = g.dwe = g.ddel = g.dwi = g.dws = nullptr;
  g.device_ready = false;
  g.dev_precision = -1;
}

int node_size() { return g.myDim + g.eDim; }

const fgb::HostMesh* hm() { return g.hmesh ? g.hmesh->m : nullptr; }

// Host (nl-1, n) column-major -> device (n, LZ) padded, in the form's precision.
template <typename R>
std::vector<R> pad_cols(const double* src, int n, int nrow, int ld) {
  std::vector<R> out((size_t)n * ld, R(0));
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < nrow; ++i) out[(size_t)j * ld + i] = (R)src[(size_t)j * nrow + i];
  return out;
}

int copy_to_device(void* dst, const void* src, size_t bytes) {
  return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? 0 : -1;
}

template <typename R>
int upload_inputs() {
  const fgb::HostMesh& h = *hm();
  int dims[8];
  fgb_mesh_dims(g.dmesh, dims);
  const int N = dims[0], M = dims[2], nz = dims[4], LZ = dims[5], LW = dims[6], nl = nz + 1;
  const Tracer& t = g.tr[0];
  auto T = pad_cols<R>(t.values.data(), N, nz, LZ);
  auto TA = pad_cols<R>(t.valuesAB.data(), N, nz, LZ);
  // The step reads the uv buffer as vel(2, nl-1, elem2D) (sequence association).
  std::vector<R> vel((size_t)M * LZ * 2, R(0));
  if (g.have_uv)
    for (int el = 0; el < M; ++el)
      for (int z = 0; z < nz; ++z)
        for (int c = 0; c < 2; ++c) vel[((size_t)el * LZ + z) * 2 + c] = (R)g.uv[(size_t)c + 2 * ((size_t)z + (size_t)nz * el)];
  std::vector<R> w((size_t)N * LW, R(0)), we((size_t)N * LW, R(0)), wi((size_t)N * LW, R(0));
  auto cols = [&](const std::vector<double>& src, std::vector<R>& dst) {
    for (int n = 0; n < N; ++n)
      for (int z = 0; z < nl; ++z) dst[(size_t)n * LW + z] = (R)src[(size_t)n * nl + z];
  };
  if (g.have_w) cols(g.w, w);
  if (g.have_we) cols(g.we, we);
  if (g.use_wsplit && g.wi.size() == (size_t)N * nl) cols(g.wi, wi);
  (void)h;
  if (copy_to_device(g.dT, T.data(), T.size() * sizeof(R)) || copy_to_device(g.dTA, TA.data(), TA.size() * sizeof(R)) ||
      copy_to_device(g.dvel, vel.data(), vel.size() * sizeof(R)) || copy_to_device(g.dw, w.data(), w.size() * sizeof(R)) ||
      copy_to_device(g.dwe, we.data(), we.size() * sizeof(R)) || copy_to_device(g.dwi, wi.data(), wi.size() * sizeof(R)))
    return fail("cudaMemcpy to the device failed");
  if (g.del_pending) {  // the restart's del_ttf, once
    auto del = pad_cols<R>(g.del.data(), N, nz, LZ);
    if (copy_to_device(g.ddel, del.data(), del.size() * sizeof(R))) return fail("cudaMemcpy to the device failed");
    g.del_pending = false;
  }
  return 0;
}

// del_ttf of the device (the step's accumulated tendency) into g.del.
template <typename R>
int download_del() {
  int dims[8];
  fgb_mesh_dims(g.dmesh, dims);
  const int N = dims[0], nz = dims[4], LZ = dims[5];
  std::vector<R> D((size_t)N * LZ);
  if (cudaMemcpy(D.data(), g.ddel, D.size() * sizeof(R), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail("cudaMemcpy from the device failed");
  g.del.assign((size_t)N * nz, 0.0);
  for (int n = 0; n < N; ++n)
    for (int z = 0; z < nz; ++z) g.del[(size_t)n * nz + z] = (double)D[(size_t)n * LZ + z];
  return 0;
}

template <typename R>
int download_values() {
  int dims[8];
  fgb_mesh_dims(g.dmesh, dims);
  const int N = dims[0], nz = dims[4], LZ = dims[5];
  std::vector<R> T((size_t)N * LZ);
  if (cudaMemcpy(T.data(), g.dT, T.size() * sizeof(R), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail("cudaMemcpy from the device failed");
  std::vector<double>& v = g.tr[0].values;
  for (int n = 0; n < N; ++n)
    for (int z = 0; z < nz; ++z) v[(size_t)n * nz + z] = (double)T[(size_t)n * LZ + z];
  return 0;
}

int sync_values_to_host() {
  if (!g.values_on_device) return 0;
  int rc = g.dev_precision == FGB_FP32 ? download_values<float>() : download_values<double>();
  if (rc == 0) g.values_on_device = false;
  return rc;
}

// Applies the caller's level and thickness arrays to the host mesh and
// (re)creates the device mesh and buffers when needed.
int prepare_device() {
  if (!g.hmesh) return fail("no mesh: call tracer_load_mesh_from_files or tracer_generate_analytic_mesh first");
  fgb::HostMesh& h = *g.hmesh->m;
  if (g.tr.empty()) return fail("no tracers: call tracer_allocate_tracers first");
  if (node_size() != h.N) return fail("partition size (myDim+eDim) does not match the mesh nodes");
  if ((int)g.tr[0].values.size() != (h.nl - 1) * h.N) return fail("tracer arrays do not match the mesh");
  if (g.have_uv && (long long)g.uv.size() < 2LL * (h.nl - 1) * h.M)
    return fail("uv holds fewer values than vel(2,nl-1,elem2D) reads");
  if (g.have_w && (long long)g.w.size() != (long long)h.nl * h.N) return fail("w does not match the mesh");
  const bool need_new = !g.device_ready || g.dev_precision != g.precision || g.mesh_dirty;
  if (g.mesh_dirty || !g.dmesh) {
    if (!g.set_nlev.empty()) {
      if ((int)g.set_nlev.size() != h.N) return fail("tracer_set_levels size does not match the mesh");
      h.nlev_nod.assign(g.set_nlev.begin(), g.set_nlev.end());
      h.ulev_nod.assign(g.set_ulev.begin(), g.set_ulev.end());
    }
    if (g.have_hnode) h.hnode = g.hnode;
    if (g.have_hnode_new) h.hnode_new = g.hnode_new;
    if (g.have_helem) h.helem = g.helem;
    if (g.dmesh) {
      fgb_mesh_free(g.dmesh);
      g.dmesh = nullptr;
    }
    if (fgb_mesh_create(g.hmesh, &g.dmesh)) return fail(fgb_last_error());
    g.mesh_dirty = false;
  }
  if (need_new) {
    free_device();
    int dims[8];
    fgb_mesh_dims(g.dmesh, dims);
    const size_t N = dims[0], M = dims[2], LZ = dims[5], LW = dims[6];
    const size_t s = g.precision == FGB_FP32 ? 4 : 8;
    g.ws_bytes = fgb_workspace_bytes(g.dmesh, g.precision, 1);
    void** bufs[] = {&g.dT, &g.dTA, &g.dvel, &g.dw, &g.dwe, &g.ddel, &g.dwi, &g.dws};
    size_t sizes[] = {N * LZ * s, N * LZ * s, M * LZ * 2 * s, N * LW * s, N * LW * s, N * LZ * s, N * LW * s,
                      (size_t)g.ws_bytes};
    for (int i = 0; i < 8; ++i) {
      if (cudaMalloc(bufs[i], sizes[i]) != cudaSuccess) {
        free_device();
        return fail("cudaMalloc failed");
      }
      cudaMemset(*bufs[i], 0, sizes[i]);
    }
    g.device_ready = true;
    g.dev_precision = g.precision;
    g.inputs_dirty = true;
  }
  if (g.inputs_dirty) {
    int rc = g.precision == FGB_FP32 ? upload_inputs<float>() : upload_inputs<double>();
    if (rc) return rc;
    g.inputs_dirty = false;
    g.values_on_device = false;
  }
  return 0;
}

const char* const kHorNames[] = {"UPW1", "MUSCL", "MFCT"};
const char* const kVerNames[] = {"UPW1", "QR4C", "CDIFF", "PPM"};
const char* const kLimNames[] = {"NONE", "FCT"};

std::string trimmed(const std::string& s) {
  size_t e = s.find_last_not_of(' ');
  return e == std::string::npos ? std::string() : s.substr(0, e + 1);
}

int scheme_index(const std::string& s, const char* const* names, int n) {
  const std::string v = trimmed(s);
  for (int i = 0; i < n; ++i)
    if (v == names[i]) return i;
  return -1;
}

// <dir>/np<npes>/t_<type>.<rank> of a one-process run (rank text "0":
// mpirank_to_txt pads to the digits of npes, lib/fortran_utils.F90:45-56).
std::string restart_file(const std::string& npepath, const char* type) { return npepath + "/" + type + ".0"; }

bool read_type(const std::string& npepath, const char* type, fgb::restart::Record* out, std::string* err,
               bool (*decode)(const std::vector<uint8_t>&, fgb::restart::Record*, std::string*)) {
  std::vector<uint8_t> bytes;
  return fgb::restart::read_record_file(restart_file(npepath, type), &bytes, err) && decode(bytes, out, err);
}

bool decode_dyn(const std::vector<uint8_t>& b, fgb::restart::Record* r, std::string* err) {
  return fgb::restart::decode_dynamics(b, r, err, false);
}

bool file_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// Replaces the mesh and the velocities by those of the restart records
// (t_mesh with the MUSCL tables of t_tracer when given, t_partit, t_dynamics).
int adopt_restart(const std::string& npepath, fgb::restart::Record&& rm, fgb::restart::Record&& rp,
                  fgb::restart::Record* rt, fgb::restart::Record&& rd) {
  using fgb::restart::Field;
  std::string err;
  fgb::HostMesh* hm = fgb::restart::mesh_from_records(rm, rt, &err);
  if (!hm) return fail(err.c_str());
  const Field *md = rp.get("myDim_nod2D"), *ed = rp.get("eDim_nod2D"), *np = rp.get("npes");
  if (!md || !ed || md->i + ed->i != hm->N || (np && np->i != 1)) {
    delete hm;
    return fail((npepath + ": t_partit does not describe one process owning every node of t_mesh").c_str());
  }
  const int N = hm->N, M = hm->M, nl = hm->nl, nz = nl - 1;
  const Field *uv = rd.get("uv"), *w = rd.get("w"), *we = rd.get("w_e"), *wi = rd.get("w_i"), *ws = rd.get("use_wsplit");
  const std::vector<int32_t> dim_uv = {2, nz, M}, dim_w = {nl, N};
  if (!uv || uv->dims != dim_uv || !w || w->dims != dim_w) {
    delete hm;
    return fail((npepath + ": t_dynamics uv/w do not match the mesh").c_str());
  }
  if (sync_values_to_host()) {
    delete hm;
    return -1;
  }
  free_device();
  if (g.dmesh) fgb_mesh_free(g.dmesh);
  if (g.hmesh) fgb_hmesh_free(g.hmesh);
  g.dmesh = nullptr;
  g.hmesh = new fgb_hmesh{hm};
  g.nl = nl;
  g.nod2D = rm.get("nod2D")->i;
  g.edge2D = hm->E;
  g.elem2D = hm->M;
  g.myDim = md->i;
  g.eDim = ed->i;
  g.hnode = hm->hnode;
  g.hnode_new = hm->hnode_new;
  g.helem = hm->helem;
  g.have_hnode = g.have_hnode_new = g.have_helem = false;
  g.set_nlev.clear();
  g.set_ulev.clear();
  g.uv = uv->vr;  // vel(2, nl-1, elem2D), the layout the step reads
  g.w = w->vr;
  g.have_uv = g.have_w = true;
  g.have_we = we && we->dims == dim_w;
  g.we = g.have_we ? we->vr : std::vector<double>();
  g.use_wsplit = ws && ws->i;
  g.wi = (wi && wi->dims == dim_w) ? wi->vr : std::vector<double>((size_t)nl * N, 0.0);
  g.from_restart = true;
  g.rmesh = std::move(rm);
  g.rpartit = std::move(rp);
  g.rdyn = std::move(rd);
  g.rtracer = rt ? std::move(*rt) : fgb::restart::Record();
  g.initialized = true;
  g.mesh_dirty = g.inputs_dirty = true;
  return 0;
}

// The tracers of a t_tracer record (values, valuesAB, schemes, del_ttf).
int adopt_tracers(const fgb::restart::Record& rt) {
  using fgb::restart::Field;
  const Field* nt = rt.get("num_tracers");
  const int N = node_size(), nz = g.nl - 1;
  const std::vector<int32_t> dim_v = {nz, N};
  if (!nt || nt->i < 1) return fail("t_tracer restart holds no tracer");
  std::vector<Tracer> tr(nt->i);
  for (int t = 0; t < nt->i; ++t) {
    const std::string p = "data(" + std::to_string(t + 1) + ")%";
    const Field *v = rt.get(p + "values"), *vab = rt.get(p + "valuesAB");
    if (!v || v->dims != dim_v) return fail("t_tracer restart: values do not match the mesh");
    tr[t].values = v->vr;
    tr[t].valuesAB = (vab && vab->dims == dim_v) ? vab->vr : v->vr;
    const int a = scheme_index(rt.get(p + "tra_adv_hor")->c, kHorNames, 3);
    const int b = scheme_index(rt.get(p + "tra_adv_ver")->c, kVerNames, 4);
    const int c = scheme_index(rt.get(p + "tra_adv_lim")->c, kLimNames, 2);
    // the reference aborts on an unknown scheme (lib/oce_adv_tra_driver.F90:252-254)
    if (a < 0) return fail("Unknown horizontal advection type");
    if (b < 0) return fail("Unknown vertical advection type");
    if (c < 0) return fail("Unknown limiter type");
    tr[t].hor = a;
    tr[t].ver = b;
    tr[t].lim = c;
    tr[t].ph = rt.get(p + "tra_adv_ph")->r;
    tr[t].pv = rt.get(p + "tra_adv_pv")->r;
  }
  g.tr = std::move(tr);
  const Field* del = rt.get("work%del_ttf");
  g.del_pending = del && del->dims == dim_v;
  g.del = g.del_pending ? del->vr : std::vector<double>();
  g.values_on_device = false;
  g.inputs_dirty = true;
  return 0;
}

int parse_scheme(const char* s, const char* const* names, int n) {
  std::string v = c2s(s);
  while (!v.empty() && v.back() == ' ') v.pop_back();  // Fortran character(20) is blank padded
  for (int i = 0; i < n; ++i)
    if (v == names[i]) return i;
  return -1;
}

}  // namespace

extern "C" {

int tracer_init_mpi(int mpi_comm) {
  g.mpi_comm = mpi_comm;
  g.npes = 1;
  return 0;
}

int tracer_finalize_mpi(void) { return 0; }

int tracer_init(const char* restart_dir) {
  const std::string npepath = c2s(restart_dir) + "/np" + std::to_string(g.npes);
  if (!dir_exists(npepath)) {
    std::fprintf(stderr, "### error: could not find restart directory: %s\n", npepath.c_str());
    fgb::set_error("could not find restart directory");
    return -1;
  }
  // read_all_bin_restarts(npepath, partit, mesh, dynamics, tracers)
  fgb::restart::Record rm, rp, rt, rd;
  std::string err;
  if (!read_type(npepath, "t_mesh", &rm, &err, fgb::restart::decode_mesh) ||
      !read_type(npepath, "t_partit", &rp, &err, fgb::restart::decode_partit) ||
      !read_type(npepath, "t_tracer", &rt, &err, fgb::restart::decode_tracer) ||
      !read_type(npepath, "t_dynamics", &rd, &err, decode_dyn))
    return fail(err.c_str());
  if (adopt_restart(npepath, std::move(rm), std::move(rp), &rt, std::move(rd))) return -1;  // keeps rt
  if (adopt_tracers(g.rtracer)) {
    g.initialized = false;
    return -1;
  }
  std::printf("Tracer initialized from: %s\n", npepath.c_str());  // :150-152
  std::fflush(stdout);
  return 0;
}

int tracer_advect_step(double dt) {
  if (!g.initialized) return fail("tracer not initialized. Call tracer_init first.");
  // Setters copy device values back first, so dirty inputs never hide newer device values.
  if (prepare_device()) return -1;
  const Tracer& t = g.tr[0];
  int dims[8];
  fgb_mesh_dims(g.dmesh, dims);
  fgb_step_desc d;
  std::memset(&d, 0, sizeof(d));
  d.precision = g.precision;
  d.ntracers = 1;
  d.hor = t.hor;
  d.ver = t.ver;
  d.lim = t.lim;
  d.ph = t.ph;
  d.pv = t.pv;
  d.dt = dt;
  d.T = g.dT;
  d.strideT = (long long)dims[0] * dims[5];
  d.TA = g.dTA;
  d.strideTA = d.strideT;
  d.vel = g.dvel;
  d.w = g.dw;   // the high-order flux under FCT uses w
  d.we = g.dwe;  // w_e: zero after tracer_set_velocity
  d.wi = g.use_wsplit ? g.dwi : nullptr;  // w_split (a restart's use_wsplit)
  d.del = g.ddel;
  d.workspace = g.dws;
  d.workspace_bytes = g.ws_bytes;
  if (g.input_checks) {
    int flags = 0;
    if (fgb_check_inputs(g.dmesh, &d, nullptr, &flags)) return fail(fgb_last_error());
    if (flags) {
      std::string what = "non-finite input values:";
      const std::pair<int, const char*> names[] = {{FGB_CHECK_T, " values"}, {FGB_CHECK_TA, " valuesAB"},
                                                   {FGB_CHECK_VEL, " uv"},    {FGB_CHECK_W, " w"},
                                                   {FGB_CHECK_WE, " w_e"},    {FGB_CHECK_WI, " w_i"}};
      for (const auto& nm : names)
        if (flags & nm.first) what += nm.second;
      return fail(what.c_str());
    }
  }
  if (fgb_adv_step(g.dmesh, &d, nullptr)) return fail(fgb_last_error());
  if (cudaDeviceSynchronize() != cudaSuccess) return fail("device error during the step");
  g.values_on_device = true;
  return 0;
}

int tracer_get_stats(double* tmin, double* tmax, double* tsum) {
  if (!g.initialized || g.tr.empty()) {
    std::fprintf(stderr, "### error: tracer not initialized.\n");
    if (tmin) *tmin = 0.0;
    if (tmax) *tmax = 0.0;
    if (tsum) *tsum = 0.0;
    return -1;
  }
  if (sync_values_to_host()) return -1;
  const std::vector<double>& v = g.tr[0].values;
  double mn = INFINITY, mx = -INFINITY, sm = 0.0;
  for (double x : v) {
    mn = std::fmin(mn, x);
    mx = std::fmax(mx, x);
    sm += x;
  }
  *tmin = mn;
  *tmax = mx;
  *tsum = sm;
  return 0;
}

int tracer_get_size(int* nz, int* nn) {
  if (!g.initialized) {
    std::fprintf(stderr, "### error: tracer not initialized.\n");
    if (nz) *nz = 0;
    if (nn) *nn = 0;
    return -1;
  }
  *nz = g.nl - 1;
  *nn = g.myDim;
  return 0;
}

int tracer_get_values(double* values, int nz, int nn) {
  if (!g.initialized || g.tr.empty()) return fail("tracer not initialized.");
  if (nz > g.nl - 1 || nn > node_size() || nz < 0 || nn < 0) return fail("requested size exceeds the tracer array");
  if (sync_values_to_host()) return -1;
  const std::vector<double>& v = g.tr[0].values;
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < nz; ++i) values[(size_t)j * nz + i] = v[(size_t)j * (g.nl - 1) + i];
  return 0;
}

int tracer_finalize(const char* output_dir) {
  if (!g.initialized) return fail("tracer not initialized.");
  if (!g.hmesh) return fail("no mesh");
  using fgb::restart::Field;
  using fgb::restart::Record;
  const fgb::HostMesh& h = *g.hmesh->m;
  if (sync_values_to_host()) return -1;
  if (g.device_ready && g.ddel) {
    const int rc = g.dev_precision == FGB_FP32 ? download_del<float>() : download_del<double>();
    if (rc) return rc;
  }
  const std::string out = c2s(output_dir), npepath = out + "/np" + std::to_string(g.npes);
  mkdir(out.c_str(), 0777);  // like the reference's mkdir: an existing directory is fine
  mkdir(npepath.c_str(), 0777);
  if (!dir_exists(npepath)) return fail(("cannot create " + npepath).c_str());
  const int N = h.N, M = h.M, E = h.E, nl = h.nl, nz = nl - 1;
  const int ntr = (int)g.tr.size();
  // the records read at tracer_init, else those of this state with the types' defaults
  Record rm = g.from_restart ? g.rmesh : fgb::restart::mesh_record(h);
  Record rp = g.from_restart ? g.rpartit : fgb::restart::partit_record(N, M, E);
  Record rd = g.from_restart ? g.rdyn : fgb::restart::dynamics_record(nl, N, M);
  const Field* nt = g.rtracer.get("num_tracers");
  Record rt = (g.from_restart && nt && nt->i == ntr) ? g.rtracer : fgb::restart::tracer_record(h, ntr);
  // the state's arrays
  auto set = [](Record& r, const std::string& name, std::vector<int32_t> dims, const std::vector<double>& v) {
    Field* f = r.get(name);
    if (!f) return;
    f->dims = std::move(dims);
    f->vr.assign(v.begin(), v.begin() + std::min(v.size(), f->count()));
    f->vr.resize(f->count(), 0.0);
  };
  set(rm, "hnode", {nz, N}, h.hnode);
  set(rm, "hnode_new", {nz, N}, h.hnode_new);
  set(rm, "helem", {nz, M}, h.helem);
  for (int t = 0; t < ntr; ++t) {
    const std::string p = "data(" + std::to_string(t + 1) + ")%";
    set(rt, p + "values", {nz, N}, g.tr[t].values);
    set(rt, p + "valuesAB", {nz, N}, g.tr[t].valuesAB);
    rt.get(p + "tra_adv_hor")->c = kHorNames[g.tr[t].hor];
    rt.get(p + "tra_adv_ver")->c = kVerNames[g.tr[t].ver];
    rt.get(p + "tra_adv_lim")->c = kLimNames[g.tr[t].lim];
    rt.get(p + "tra_adv_ph")->r = g.tr[t].ph;
    rt.get(p + "tra_adv_pv")->r = g.tr[t].pv;
  }
  set(rt, "work%del_ttf", {nz, N}, g.del.empty() ? std::vector<double>((size_t)nz * N, 0.0) : g.del);
  // the step's velocity: vel(2, nl-1, elem2D) as the step reads it
  set(rd, "uv", {2, nz, M}, g.uv);
  set(rd, "w", {nl, N}, g.w);
  set(rd, "w_e", {nl, N}, g.have_we ? g.we : std::vector<double>((size_t)nl * N, 0.0));
  set(rd, "w_i", {nl, N}, g.wi.size() == (size_t)nl * N ? g.wi : std::vector<double>((size_t)nl * N, 0.0));
  std::string err;
  const std::pair<const char*, const Record*> files[] = {
      {"t_mesh", &rm}, {"t_partit", &rp}, {"t_tracer", &rt}, {"t_dynamics", &rd}};
  for (const auto& f : files)
    if (!fgb::restart::write_record_file(restart_file(npepath, f.first), fgb::restart::encode(*f.second), &err))
      return fail(err.c_str());
  if (!fgb::restart::write_meta(out + "/meta.time", 0, 0, 0, true, true, &err)) return fail(err.c_str());
  std::printf("Restart files written to: %s\n", npepath.c_str());  // :339-341
  std::fflush(stdout);
  g.initialized = false;
  return 0;
}

int tracer_run_workflow(const char* restart_dir, int nsteps, double dt) {
  int status = tracer_init(restart_dir);
  if (status != 0) return status;
  for (int step = 1; step <= nsteps; ++step) {
    double tmin, tmax, tsum;
    if ((status = tracer_advect_step(dt)) != 0) return status;
    if ((status = tracer_get_stats(&tmin, &tmax, &tsum)) != 0) return status;
    std::printf("Step %3d: min/max/sum = %15.6E%15.6E%15.6E\n", step, tmin, tmax, tsum);
  }
  return tracer_finalize(restart_dir);
}

int tracer_cleanup(void) {
  free_device();
  if (g.dmesh) fgb_mesh_free(g.dmesh);
  if (g.hmesh) fgb_hmesh_free(g.hmesh);
  g = State();
  return 0;
}

int tracer_set_mesh_dims(int nl, int nod2D, int edge2D, int elem2D) {
  g.nl = nl;
  g.nod2D = nod2D;
  g.edge2D = edge2D;
  g.elem2D = elem2D;
  return 0;
}

int tracer_set_levels(const int* nlevels, const int* ulevels, int nod2D) {
  if (nod2D < 0 || (nod2D > 0 && (!nlevels || !ulevels))) return fail("bad level arrays");
  if (sync_values_to_host()) return -1;
  g.set_nlev.assign(nlevels, nlevels + nod2D);
  g.set_ulev.assign(ulevels, ulevels + nod2D);
  g.mesh_dirty = g.inputs_dirty = true;
  return 0;
}

int tracer_set_thickness(const double* hnode, int nl, int nod2D) {
  if (nl < 2 || nod2D < 0 || !hnode) return fail("bad thickness array");
  if (sync_values_to_host()) return -1;
  g.hnode_new.assign(hnode, hnode + (size_t)(nl - 1) * nod2D);
  g.have_hnode_new = true;
  g.mesh_dirty = g.inputs_dirty = true;
  return 0;
}

int tracer_set_partition(int myDim_nod2D, int eDim_nod2D) {
  g.myDim = myDim_nod2D;
  g.eDim = eDim_nod2D;
  return 0;
}

int tracer_allocate_tracers(int num_tracers, int nl, int nod2D, int AB_order) {
  (void)nod2D;
  if (num_tracers < 1 || nl < 2) return fail("bad tracer dimensions");
  const size_t n = (size_t)(nl - 1) * node_size();
  g.tr.assign(num_tracers, Tracer());
  for (Tracer& t : g.tr) {
    t.values.assign(n, 0.0);
    t.valuesAB.assign(n, 0.0);
  }
  g.ab_order = AB_order;
  if (g.nl == 0) g.nl = nl;
  g.values_on_device = false;
  g.inputs_dirty = true;
  g.del_pending = false;
  g.del.clear();
  if (g.device_ready && g.ddel) {  // del_ttf is re-zeroed with the work arrays
    int dims[8];
    if (g.dmesh && fgb_mesh_dims(g.dmesh, dims) == 0)
      cudaMemset(g.ddel, 0, (size_t)dims[0] * dims[5] * (g.dev_precision == FGB_FP32 ? 4 : 8));
  }
  return 0;
}

int tracer_set_values(int tracer_id, const double* values, int nl, int nod2D) {
  if (tracer_id < 1 || tracer_id > (int)g.tr.size()) {
    std::fprintf(stderr, "### error: invalid tracer_id %3d, num_tracers=%3d\n", tracer_id, (int)g.tr.size());
    fgb::set_error("invalid tracer_id");
    return -1;
  }
  Tracer& t = g.tr[tracer_id - 1];
  const size_t n = (size_t)(nl - 1) * nod2D;
  if (n > t.values.size()) return fail("values larger than the tracer array");
  if (tracer_id == 1 && sync_values_to_host()) return -1;
  for (size_t i = 0; i < n; ++i) {
    t.values[i] = values[i];
    t.valuesAB[i] = values[i];
  }
  g.inputs_dirty = true;
  return 0;
}

int tracer_set_velocity_zero(int nl, int nod2D, int edge2D) {
  if (sync_values_to_host()) return -1;
  if (!g.have_uv) {
    g.uv.assign((size_t)(nl - 1) * edge2D * 2, 0.0);
    g.uv_nl = nl;
    g.uv_edge2D = edge2D;
  } else {
    std::fill(g.uv.begin(), g.uv.end(), 0.0);
  }
  if (!g.have_w) g.w.assign((size_t)nl * nod2D, 0.0);
  else std::fill(g.w.begin(), g.w.end(), 0.0);
  g.have_uv = g.have_w = true;
  g.have_we = false;
  std::fill(g.wi.begin(), g.wi.end(), 0.0);
  g.inputs_dirty = true;
  return 0;
}

int tracer_set_velocity(const double* uv, const double* w, int nl, int nod2D, int edge2D) {
  if (!uv || !w || nl < 2) return fail("bad velocity arrays");
  if (sync_values_to_host()) return -1;
  if (!g.have_uv) {
    g.uv_nl = nl;
    g.uv_edge2D = edge2D;
  }
  g.uv.assign(uv, uv + (size_t)(nl - 1) * edge2D * 2);
  g.w.assign(w, w + (size_t)nl * nod2D);
  g.have_uv = g.have_w = true;
  g.have_we = false;  // w_e = w_i = 0 (:735-736)
  std::fill(g.wi.begin(), g.wi.end(), 0.0);
  g.inputs_dirty = true;
  return 0;
}

int tracer_init_complete(void) {
  g.initialized = true;
  return 0;
}

int tracer_load_mesh_partition(const char* restart_dir) {
  const std::string npepath = c2s(restart_dir) + "/np" + std::to_string(g.npes);
  if (!dir_exists(npepath)) {
    std::fprintf(stderr, "### error: could not find mesh partition directory: %s\n", npepath.c_str());
    fgb::set_error("could not find mesh partition directory");
    return -1;
  }
  // read_all_bin_restarts(npepath, partit, mesh, dynamics): no tracers. The
  // MUSCL tables come from t_tracer when the directory holds one.
  fgb::restart::Record rm, rp, rt, rd;
  std::string err;
  if (!read_type(npepath, "t_mesh", &rm, &err, fgb::restart::decode_mesh) ||
      !read_type(npepath, "t_partit", &rp, &err, fgb::restart::decode_partit) ||
      !read_type(npepath, "t_dynamics", &rd, &err, decode_dyn))
    return fail(err.c_str());
  const bool have_tr = file_exists(restart_file(npepath, "t_tracer")) &&
                       read_type(npepath, "t_tracer", &rt, &err, fgb::restart::decode_tracer);
  if (adopt_restart(npepath, std::move(rm), std::move(rp), have_tr ? &rt : nullptr, std::move(rd))) return -1;
  g.rtracer = fgb::restart::Record();
  const fgb::HostMesh& m = *g.hmesh->m;
  std::printf("Loaded mesh partition from: %s\n", npepath.c_str());  // :819-826
  std::printf("  Mesh: nl=%8d, nod2D=%8d, edge2D=%8d\n", m.nl, g.nod2D, m.E);
  std::printf("  Partition: myDim=%8d, eDim=%8d\n", g.myDim, g.eDim);
  std::fflush(stdout);
  return 0;
}

int tracer_load_mesh_from_files(const char* mesh_path) {
  const std::string path = c2s(mesh_path);
  std::printf("Loading mesh from partition files: %s\n", path.c_str());  // lib/tracer_c_interface.F90:849-851
  fgb_hmesh* h = nullptr;
  if (fgb_hmesh_from_files(path.c_str(), 0, &h)) return fail(fgb_last_error());
  if (sync_values_to_host()) {
    fgb_hmesh_free(h);
    return -1;
  }
  free_device();
  if (g.dmesh) fgb_mesh_free(g.dmesh);
  if (g.hmesh) fgb_hmesh_free(g.hmesh);
  g.dmesh = nullptr;
  g.hmesh = h;
  const fgb::HostMesh& m = *g.hmesh->m;
  g.nl = m.nl;
  g.nod2D = m.N;
  g.edge2D = m.E;
  g.elem2D = m.M;
  g.myDim = m.N;
  g.eDim = 0;
  g.hnode = m.hnode;
  g.hnode_new = m.hnode_new;
  g.helem = m.helem;
  g.have_hnode = g.have_hnode_new = g.have_helem = false;
  g.set_nlev.clear();
  g.set_ulev.clear();
  g.initialized = true;  // :856-857
  g.mesh_dirty = g.inputs_dirty = true;
  std::printf("Mesh loaded successfully from partition files\n");
  std::printf("  Mesh: nl=%8d, nod2D=%8d, edge2D=%8d\n", m.nl, m.N, m.E);
  std::printf("  Partition: myDim=%8d, eDim=%8d\n", m.N, 0);
  std::fflush(stdout);
  return 0;
}

int tracer_init_ale_arrays(void) {
  if (!g.initialized) return fail("tracer_init_ale_arrays called before initialization");
  if (!g.hmesh) return fail("no mesh");
  fgb::HostMesh& h = *g.hmesh->m;
  if (sync_values_to_host()) return -1;
  fgb::ale_from_zbar(h);
  g.hnode = h.hnode;
  g.hnode_new = h.hnode_new;
  g.helem = h.helem;
  g.have_hnode = g.have_hnode_new = g.have_helem = true;
  g.mesh_dirty = g.inputs_dirty = true;
  return 0;
}

int tracer_init_for_advection(void) {
  if (!g.initialized) return fail("tracer_init_for_advection called before mesh loaded");
  if (!g.hmesh) return fail("no mesh");
  const fgb::HostMesh& h = *g.hmesh->m;
  if (!g.have_uv) {
    g.uv.assign((size_t)2 * (h.nl - 1) * h.M, 0.0);
    g.have_uv = true;
  }
  if (!g.have_w) {
    g.w.assign((size_t)h.nl * h.N, 0.0);
    g.have_w = true;
  }
  if (g.tr.empty()) return 0;  // work arrays are sized by tracer_allocate_tracers
  return prepare_device();
}

int tracer_generate_analytic_mesh(int nx, int ny, int nl, int periodic) {
  if (sync_values_to_host()) return -1;
  free_device();
  if (g.dmesh) fgb_mesh_free(g.dmesh);
  if (g.hmesh) fgb_hmesh_free(g.hmesh);
  g.dmesh = nullptr;
  g.hmesh = nullptr;
  // Domain and depth of the analytic dwarf, src/fesom_analytic.F90:69-71.
  if (fgb_hmesh_analytic(nx, ny, nl, 100000.0, 100000.0, 1000.0, periodic, 0, nullptr, nullptr, &g.hmesh))
    return fail(fgb_last_error());
  const fgb::HostMesh& h = *g.hmesh->m;
  g.nl = h.nl;
  g.nod2D = h.N;
  g.edge2D = h.E;
  g.elem2D = h.M;
  g.myDim = h.N;
  g.eDim = 0;
  g.hnode = h.hnode;
  g.hnode_new = h.hnode_new;
  g.helem = h.helem;
  g.have_hnode = g.have_hnode_new = g.have_helem = false;
  g.set_nlev.clear();
  g.set_ulev.clear();
  g.initialized = true;  // a loaded mesh marks the system initialised (:856-857)
  g.mesh_dirty = g.inputs_dirty = true;
  return 0;
}

int tracer_set_schemes(int tracer_id, const char* hor, const char* ver, const char* lim, double ph, double pv) {
  static const char* H[] = {"UPW1", "MUSCL", "MFCT"};
  static const char* V[] = {"UPW1", "QR4C", "CDIFF", "PPM"};
  static const char* L[] = {"NONE", "FCT"};
  if (tracer_id < 1 || tracer_id > (int)g.tr.size()) return fail("invalid tracer_id");
  int a = parse_scheme(hor, H, 3), b = parse_scheme(ver, V, 4), c = parse_scheme(lim, L, 2);
  if (a < 0) return fail("Unknown horizontal advection type");
  if (b < 0) return fail("Unknown vertical advection type");
  if (c < 0) return fail("Unknown limiter type");
  Tracer& t = g.tr[tracer_id - 1];
  t.hor = a;
  t.ver = b;
  t.lim = c;
  t.ph = ph;
  t.pv = pv;
  return 0;
}

int tracer_set_input_checks(int on) {
  g.input_checks = on != 0;
  return 0;
}

int tracer_set_precision(int precision) {
  if (precision != FGB_FP64 && precision != FGB_FP32) return fail("precision must be 0 (FP64) or 1 (FP32)");
  if (sync_values_to_host()) return -1;
  g.precision = precision;
  g.inputs_dirty = true;
  return 0;
}

}  // extern "C"
