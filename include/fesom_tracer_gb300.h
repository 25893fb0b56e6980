/*
 * libfesom_tracer_gb300.so -- GB300-native FESOM2 tracer-advection step.
 *
 * Two C-ABI layers, both plain pointers and sizes:
 *
 *  1. The reference's own C interface (lib/tracer_c_interface.F90), same
 *     symbol names, argument types and status codes, so a caller of
 *     libfesom_tracer_Fortran.so can relink against this library. Each
 *     declaration cites the Fortran function it replaces.
 *
 *  2. The fgb_* engine interface: an explicit mesh handle and caller-owned
 *     device buffers (tracers, velocities, workspace) with a CUDA stream, so
 *     that hosts such as PyTorch keep the allocation and the stream. It adds
 *     what the reference interface cannot express: building the analytic
 *     mesh, choosing schemes, stepping many tracers per launch, the FP32
 *     form, and the individual stages of the step.
 *
 * Status codes: 0 success, -1 error (message on stderr for tracer_*; the
 * text of the last error from fgb_last_error() for fgb_*).
 * Array layouts of layer 1 are the reference's Fortran column-major ones.
 */
#ifndef FESOM_TRACER_GB300_H
#define FESOM_TRACER_GB300_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===================================================================== */
/* 1. Reference interface (lib/tracer_c_interface.F90)                    */
/* ===================================================================== */

/* lib/tracer_c_interface.F90:46. One GPU, one rank: records the
 * communicator and returns 0; no MPI is initialised. */
int tracer_init_mpi(int mpi_comm);
/* lib/tracer_c_interface.F90:89. Returns 0. */
int tracer_finalize_mpi(void);
/* lib/tracer_c_interface.F90:113. Reads the derived-type binary restarts
 * <dir>/np1/t_mesh.0, t_partit.0, t_tracer.0 and t_dynamics.0
 * (read_all_bin_restarts, lib/io_restart_derivedtype.F90:132-199; one
 * process, so npes = 1): mesh, tracers with their schemes, del_ttf, uv, w,
 * w_e and (under use_wsplit) w_i. -1 with the reference's message when
 * <dir>/np<npes> is missing; -1 with the file and field when a record does
 * not parse or does not fit the mesh. */
int tracer_init(const char* restart_dir);
/* lib/tracer_c_interface.F90:163. One do_oce_adv_tra for tracer 1 plus the
 * tendency update; del_ttf accumulates across calls as in the reference. */
int tracer_advect_step(double dt);
/* lib/tracer_c_interface.F90:228. min, max and plain sum of tracer 1. */
int tracer_get_stats(double* tmin, double* tmax, double* tsum);
/* lib/tracer_c_interface.F90:255. nz = nl-1 layers, nn = owned nodes. */
int tracer_get_size(int* nz, int* nn);
/* lib/tracer_c_interface.F90:280. Copies tracer 1 into values(nz,nn). */
int tracer_get_values(double* values, int nz, int nn);
/* lib/tracer_c_interface.F90:308. Writes <dir>/np1/t_mesh.0, t_partit.0,
 * t_tracer.0, t_dynamics.0 and <dir>/meta.time (write_all_bin_restarts,
 * lib/io_restart_derivedtype.F90:33-125) and marks the system
 * uninitialised. After tracer_init the records read are written back with
 * the state's values, valuesAB, schemes, del_ttf, thicknesses and
 * velocities; otherwise the fields the step does not keep are written
 * unallocated and the types' scalars at their defaults. */
int tracer_finalize(const char* output_dir);
/* lib/tracer_c_interface.F90:356. init + nsteps x (step, stats) + finalize. */
int tracer_run_workflow(const char* restart_dir, int nsteps, double dt);
/* lib/tracer_c_interface.F90:391. Resets the module state, frees device memory. */
int tracer_cleanup(void);
/* lib/tracer_c_interface.F90:415 */
int tracer_set_mesh_dims(int nl, int nod2D, int edge2D, int elem2D);
/* lib/tracer_c_interface.F90:441. Sets nodal levels only (as the reference). */
int tracer_set_levels(const int* nlevels, const int* ulevels, int nod2D);
/* lib/tracer_c_interface.F90:477. Sets hnode_new only (as the reference). */
int tracer_set_thickness(const double* hnode, int nl, int nod2D);
/* lib/tracer_c_interface.F90:510 */
int tracer_set_partition(int myDim_nod2D, int eDim_nod2D);
/* lib/tracer_c_interface.F90:539. Defaults UPW1/UPW1/NONE, ph=pv=1. */
int tracer_allocate_tracers(int num_tracers, int nl, int nod2D, int AB_order);
/* lib/tracer_c_interface.F90:613. Sets values and valuesAB of one tracer. */
int tracer_set_values(int tracer_id, const double* values, int nl, int nod2D);
/* lib/tracer_c_interface.F90:652 */
int tracer_set_velocity_zero(int nl, int nod2D, int edge2D);
/* lib/tracer_c_interface.F90:694. uv is stored as given, (nl-1,edge2D,2),
 * and read by the step as vel(2,nl-1,elem2D) -- the reference reinterprets
 * the same memory. w_e and w_i are set to zero, as in the reference. */
int tracer_set_velocity(const double* uv, const double* w, int nl, int nod2D, int edge2D);
/* lib/tracer_c_interface.F90:749 */
int tracer_init_complete(void);
/* lib/tracer_c_interface.F90:769. Reads t_mesh.0, t_partit.0 and
 * t_dynamics.0 of <dir>/np1 (no tracers; the MUSCL tables come from
 * t_tracer.0 when the directory holds one). */
int tracer_load_mesh_partition(const char* restart_dir);
/* lib/tracer_c_interface.F90:830. Reads the FESOM mesh files of mesh_path
 * (nod2d.out, elem2d.out, aux3d.out, edgenum.out, edges.out, edge_tri.out,
 * elvls.out, nlvls.out) as one partition with mesh_setup's set-up and the
 * reference's defaults (fgb_hmesh_from_files with flags 0) and marks the
 * system initialised; the dist_<npes>/ lists are not read. -1 with a message
 * if a file is missing or malformed. */
int tracer_load_mesh_from_files(const char* mesh_path);
/* lib/tracer_c_interface.F90:875. Layer thicknesses from zbar. */
int tracer_init_ale_arrays(void);
/* lib/tracer_c_interface.F90:931. Allocates work arrays (device). */
int tracer_init_for_advection(void);

/* Extensions of the reference interface (no Fortran counterpart). */
/* Analytic mesh of lib/analytic_mesh.F90:114 (what the analytic dwarf
 * src/fesom_analytic.F90:188 builds); replaces loading a mesh. */
int tracer_generate_analytic_mesh(int nx, int ny, int nl, int periodic);
/* Advection schemes of one tracer: hor "UPW1"|"MUSCL"|"MFCT", ver
 * "UPW1"|"QR4C"|"CDIFF"|"PPM", lim "NONE"|"FCT" (T_TRACER_DATA fields,
 * lib/MOD_TRACER.F90:18-20). */
int tracer_set_schemes(int tracer_id, const char* hor, const char* ver, const char* lim, double ph,
                       double pv);
/* Device form of the step: 0 = FP64 (default), 1 = FP32. */
int tracer_set_precision(int precision);
/* on != 0: every tracer_advect_step first checks that its inputs (values,
 * valuesAB, uv, w, w_e, w_i) are finite on the device (fgb_check_inputs)
 * and returns -1 with the arrays named instead of stepping. Off by default,
 * as in the reference, which carries NaN and Inf through the step. */
int tracer_set_input_checks(int on);

/* ===================================================================== */
/* 2. Engine interface                                                    */
/* ===================================================================== */

typedef struct fgb_hmesh fgb_hmesh; /* host-side mesh (set-up) */
typedef struct fgb_mesh fgb_mesh;   /* device-resident mesh */

enum { FGB_HOR_UPW1 = 0, FGB_HOR_MUSCL = 1, FGB_HOR_MFCT = 2 };
enum { FGB_VER_UPW1 = 0, FGB_VER_QR4C = 1, FGB_VER_CDIFF = 2, FGB_VER_PPM = 3 };
enum { FGB_LIM_NONE = 0, FGB_LIM_FCT = 1 };
/* FGB_FP64: the bit-exact FP64 form (the reference's evaluation order, no
 * fused multiply-add). FGB_FP32: FP32 storage and arithmetic, tracers grouped
 * by fgb_step_desc.tracer_vec. FGB_FP64_FAST: FP64 storage and arithmetic with
 * fused multiply-add and divisions by constants and by the layer volumes
 * replaced by products with reciprocals formed once per layer; the FP64
 * layout and workspace, results within 1e-12 (relative) of FGB_FP64. */
enum { FGB_FP64 = 0, FGB_FP32 = 1, FGB_FP64_FAST = 2 };

/* Stages of one step (bit mask for fgb_adv_stages). */
enum {
  FGB_STAGE_VFLUX = 1,  /* edge volume fluxes from the velocity (per step) */
  FGB_STAGE_HFLUX = 2,  /* horizontal LO / antidiffusive edge fluxes */
  FGB_STAGE_LO = 4,     /* FCT low-order solution + vertical antidiffusive flux */
  FGB_STAGE_RATIO = 8,  /* FCT bounds, sums and limiting factors */
  FGB_STAGE_UPDATE = 16 /* limiting, flux divergence, tracer update */
};

const char* fgb_last_error(void);
int fgb_version(void);

/* Analytic mesh (lib/analytic_mesh.F90:114-829 + geometry). zbar: nl values
 * or NULL (uniform to depth); elem_nlev: nlevels per element or NULL (flat).
 * flags = 0 reproduces the reference mesh exactly. FGB_MESH_CLUSTER_FULL
 * replaces the reference's un-remapped nod_in_elem2D of periodic meshes
 * (lib/analytic_mesh.F90:675-707) by the full lists; FGB_MESH_ORIENT_LEFT
 * swaps an edge's nodes where edge_tri(1) lies to the right of
 * node1 -> node2 (the analytic grid does so for horizontal and vertical
 * edges, lib/analytic_mesh.F90:386-426; FESOM mesh files keep it left).
 * FGB_MESH_VISIT_HILBERT makes the kernels visit node columns along a
 * Hilbert curve through the node coordinates, and edges by their
 * first-visited node (the default for file meshes, below); it changes the
 * order of the work only, never an index, a layout or a result. */
enum { FGB_MESH_CLUSTER_FULL = 1, FGB_MESH_ORIENT_LEFT = 2, FGB_MESH_VISIT_HILBERT = 4 };
int fgb_hmesh_analytic(int nx, int ny, int nl, double Lx, double Ly, double depth, int periodic, int flags,
                       const double* zbar, const int* elem_nlev, fgb_hmesh** out);
/* A FESOM mesh directory (nod2d.out, elem2d.out, aux3d.out, edgenum.out,
 * edges.out, edge_tri.out, elvls.out, nlvls.out) as one partition, with the
 * set-up of lib/oce_mesh.F90:49-94 (mesh_setup) on the sphere and the ALE
 * arrays of tracer_init_ale_arrays. flags = 0 keeps the reference's defaults
 * (lib/gen_modules_config.F90:81-88: rotation on, the Euler angles 50/15/-90
 * used as given, cyclic_length = 360 against radian coordinates);
 * FGB_MESH_FILE_NO_ROTATION, FGB_MESH_FILE_EULER_DEGREES and
 * FGB_MESH_FILE_CYCLIC_2PI select FESOM2's namelist handling instead.
 * The kernels visit the node columns of a file mesh along a Hilbert curve
 * through the (rotated) node coordinates and each edge with its
 * first-visited node, whatever the file order (a partitioner's or a mesh
 * generator's numbering); nodes, edges, elements and every array keep the
 * file's numbering, and results do not depend on the visit order.
 * FGB_MESH_FILE_KEEP_ORDER visits them in file order instead. */
enum {
  FGB_MESH_FILE_NO_ROTATION = 1,
  FGB_MESH_FILE_EULER_DEGREES = 2,
  FGB_MESH_FILE_CYCLIC_2PI = 4,
  FGB_MESH_FILE_KEEP_ORDER = 8
};
int fgb_hmesh_from_files(const char* dir, int flags, fgb_hmesh** out);
/* The same from arrays laid out as the files are (a host that holds its mesh
 * in memory): lonlat (nod2D,2) degrees, elem (elem2D,3), edges and edge_tri
 * (edge2D,2) 1-based with edge_tri <= 0 for none, elvls (elem2D), nlvls
 * (nod2D), zbar (nl). */
int fgb_hmesh_from_arrays(int nod2D, int elem2D, int edge2D, int edge2D_in, int nl, const double* lonlat,
                          const int* elem, const int* edges, const int* edge_tri, const int* elvls,
                          const int* nlvls, const double* zbar, int flags, fgb_hmesh** out);
void fgb_hmesh_free(fgb_hmesh* h);
/* No counterpart in the reference (the batching form): the disjoint union of
 * `count` host meshes as one mesh, parts in order (node, edge and element
 * indices offset by the sizes of the parts before). Layers are padded to the
 * deepest part; each part keeps its own levels. */
int fgb_hmesh_union(const fgb_hmesh* const* parts, int count, fgb_hmesh** out);
/* out[0..7] = N, E, M, nl, max_nie, edge2D_in, incident-edge entries, cluster entries */
int fgb_hmesh_sizes(const fgb_hmesh* h, long long* out8);
/* Copies a named array (0-based indices) into out; returns its element
 * count (out may be NULL to query), -1 for an unknown name. *kind is set to
 * 0 for int32, 1 for float64. */
long long fgb_hmesh_get(const fgb_hmesh* h, const char* name, void* out, int* kind);
/* Replaces the vertical arrays (N,nl-1) hnode, hnode_new and (M,nl-1)
 * helem; any may be NULL to keep it. */
int fgb_hmesh_set_vertical(fgb_hmesh* h, const double* hnode, const double* hnode_new, const double* helem);

/* Uploads the mesh to the current device (FP64 and FP32 geometry). */
int fgb_mesh_create(const fgb_hmesh* h, fgb_mesh** out);
void fgb_mesh_free(fgb_mesh* m);
/* out[0..7] = N, E, M, nl, nz, LZ, LW, fewest layers in a column. Device
 * arrays are padded: layers to LZ, interfaces to LW (multiples of 4). */
int fgb_mesh_dims(const fgb_mesh* m, int* out8);
/* Re-uploads hnode/hnode_new/helem from the host mesh. */
int fgb_mesh_update_vertical(fgb_mesh* m, const fgb_hmesh* h);

/* Workspace of a step: bytes, and the byte offsets of its arrays
 * (vf, an unused slot, adfh, lo, adfv, R+/R- interleaved per layer, the
 * same again). */
long long fgb_workspace_bytes(const fgb_mesh* m, int precision, int ntracers);
int fgb_workspace_offsets(const fgb_mesh* m, int precision, int ntracers, long long* out7);

/* One call of the step for a batch of tracers. Device pointers:
 *   T      (K,N,LZ) values, updated in place (strideT elements apart)
 *   TA     (K,N,LZ) valuesAB used by the high-order fluxes, or NULL for T
 *   TAout  optional, receives the new values (copy-AB time level)
 *   vel    (M,LZ,2) velocity on elements; w, we (N,LW) vertical velocities
 *   del    optional (K,N,LZ) persistent tendency (reference C-ABI semantics)
 *   workspace of fgb_workspace_bytes (32-byte aligned for the FP32 form).
 * Tracer grouping (FP32 form only): with tracer_vec = V in {2, 4} (V divides
 * ntracers) the per-tracer arrays T, TA, TAout and del hold groups of V
 * tracers interleaved per node-layer: tracer t, node n, layer k is element
 * (t / V) * stride + (n * LZ + k) * V + t % V, each group 16-byte aligned;
 * strideT / strideTA then count the elements between groups. tracer_vec 0
 * or 1 is the (K,N,LZ) layout above, the only one of the FP64 form. */
typedef struct {
  int precision;
  int ntracers;
  int hor, ver, lim;
  double ph, pv, dt;
  void* T;
  long long strideT;
  const void* TA;
  long long strideTA;
  void* TAout;
  const void* vel;
  const void* w;
  const void* we;
  void* del;
  void* workspace;
  long long workspace_bytes;
  int tracer_vec; /* tracers per group of the FP32 layout: 0 or 1, 2, 4 */
  /* Launch configuration; 0 picks the default. Results do not depend on it.
   * cfg[0]     warps (edges) per block of the edge-flux kernel: 2, 4, 8 (default 8)
   * cfg[1..3]  warps (node columns) per block of the LO, ratio and update
   *            kernels: 1, 2, 4 (default 4)
   * cfg[4..6]  FP64 form: tracers per chunk of the same three kernels: 1, 2,
   *            4, used when it divides ntracers (default: the largest of 4, 2,
   *            1 that does). FP32 form (one tracer group at a time): layers
   *            per lane per pass, 1 or 2 with the column staged in shared
   *            memory (defaults: LO 2, update 1), or for the ratio kernel
   *            3 (its default) / 4 without shared memory, 4 with fewer
   *            registers (columns of at most 64 layers).
   * cfg[7]     FP32 form: layers per lane per pass of the edge-flux kernel, 1 or 2
   * cfg[8]     FP32 form, w_split: 0 parallel cyclic reduction, one warp per
   *            column (columns of at most 64 layers; deeper ones always use
   *            the other solver), 1 Thomas sweeps, one lane per column
   * cfg[9]     FP32 form: 1 edge fluxes by the tiled kernel (each tile's node
   *            rows staged once in shared memory)
   * cfg[10..11] unused, 0 */
  int cfg[12];
  /* w_split (dynamics%use_wsplit, lib/oce_adv_tra_driver.F90:221-231): NULL
   * for off, else the implicit vertical velocity wi (N,LW). Under FCT the
   * low-order solution then gets the implicit vertical step with wi
   * (adv_tra_vert_impl, lib/oce_adv_tra_ver.F90:90-244; columns of at least
   * two layers) and the antidiffusive vertical flux takes the upwind flux of
   * w instead of we. Without FCT it has no effect, as in the reference. */
  const void* wi;
  /* What TAout receives: ab_order 0 or 1 the new values; 2 the second-order
   * Adams-Bashforth time level of the next step's high-order fluxes,
   * -(0.5 + ab_eps) * T_old + (1.5 + ab_eps) * T_new, on every stored layer
   * (FESOM2's tracer AB2 with offset epsilon; the reference declares
   * epsilon = 0.1, lib/oce_modules.F90:75, and allocates valuesold,
   * lib/tracer_c_interface.F90:561). TAout may alias TA: the update stage
   * runs after every stage that reads TA. */
  int ab_order;
  double ab_eps;
  /* FP32 form: which sums are plain FP32 sums instead of compensated ones
   * (FP32 pairs with error-free additions, of one rounded product per edge
   * that is the same number at both ends, so the edge fluxes cancel between
   * neighbouring nodes to the last bit of the sum). Bit mask, 0 (default): all
   * compensated. 1: the low-order fluxes of the LO stage; 2: the flux
   * divergence of the update; 4: the FCT +/- sums of the limiter (these only
   * scale each edge's flux, the same factor at both ends, so they never
   * affect conservation); 7: all plain. With Tlo set, 6 (the LO sums
   * compensated) keeps the tracer sum to ~1e-12 over 100 steps at a few
   * per cent of the step's time. The FP64 forms ignore it. */
  int fp32_plain_sums;
  /* FP32 form, optional (NULL: off): the rounding residual of every tracer
   * value, an array of T's layout and strideT. The value of a cell is
   * T + Tlo; the update stage forms T + Tlo + increment and stores its FP32
   * rounding in T and the (exact) remainder in Tlo, so that increments below
   * half an FP32 unit of T are kept. Ignored with del (the reference C
   * interface's persistent del_ttf) and by the FP64 forms. */
  void* Tlo;
} fgb_step_desc;

/* Full step: vflux, hflux, and the FCT (lo, ratio, update) or plain update. */
int fgb_adv_step(const fgb_mesh* m, const fgb_step_desc* d, void* stream);
/* Selected stages only (FGB_STAGE_* mask), in pipeline order. */
int fgb_adv_stages(const fgb_mesh* m, const fgb_step_desc* d, int stage_mask, void* stream);

/* Min, max, plain sum (FP64) and NaN count of values (K,N,LZ) over the
 * first nz layers of every node (src/fesom_analytic.F90:441-445; min and max
 * skip NaN, the sum is NaN when a value is): out_dev
 * receives 4 doubles per tracer; scratch of fgb_stats_scratch_bytes. */
long long fgb_stats_scratch_bytes(const fgb_mesh* m, int ntracers);
int fgb_tracer_stats(const fgb_mesh* m, int precision, const void* T, long long strideT, int ntracers,
                     void* scratch, double* out_dev, void* stream);
/* The same for FP32 values in the grouped layout of fgb_step_desc.tracer_vec
 * (strideT: elements between groups). */
int fgb_tracer_stats_grouped(const fgb_mesh* m, const float* T, long long strideT, int ntracers, int tracer_vec,
                             void* scratch, double* out_dev, void* stream);

/* Number of kernels the last fgb_adv_step / fgb_adv_stages call launched. */
int fgb_last_launch_count(void);

/* No counterpart in the reference: a variant of fgb_adv_step for callers that
 * cannot allocate device memory -- for example a host model whose framework
 * owns all GPU memory through its own pool allocator and must not see
 * cudaMalloc called behind its back. It allocates nothing: the step's scratch
 * is a file-scope device array of FGB_STATIC_WORKSPACE_BYTES (64 MiB) that
 * every GPU loading this library holds until the process exits; d->workspace
 * is ignored. The caller still passes T, TA, vel, w and we.
 * - Meshes whose fgb_workspace_bytes(m, precision, ntracers) exceeds
 *   FGB_STATIC_WORKSPACE_BYTES are rejected with -1 and a message, and so is
 *   a call whose current device is not the device the mesh was uploaded on.
 * - The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress) with that device current; make that first call
 *   before any stream capture.
 * - Under CUDA's default lazy module loading the array's device memory is
 *   reserved when this library's module first loads on a device, which is
 *   that first call at the latest. A host framework whose pool claims the
 *   free device memory first can make that call fail with out-of-memory:
 *   make a first (warm-up) call on each device before the pool reserves its
 *   memory, or load modules eagerly (CUDA_MODULE_LOADING=EAGER).
 * - Every call shares the one array and overwrites it; nothing in it needs to
 *   start at zero (each call writes every scratch value before reading it).
 *   Calls that overlap on the GPU (concurrent streams, or two threads) race on
 *   it: serialise them. */
#define FGB_STATIC_WORKSPACE_BYTES (64LL * 1024 * 1024)
long long fgb_static_workspace_bytes(void);
int fgb_adv_step_static(const fgb_mesh* m, const fgb_step_desc* d, void* stream);

/* No counterpart in the reference: checks that every value of the arrays the
 * step described by d reads is finite (T and TA per tracer group, Tlo, vel,
 * w, we, wi; padding layers included, which the step requires finite). One
 * device reduction per array into a status word; synchronises `stream`.
 * *flags_out: 0 when all are finite, else the FGB_CHECK_* bits of the arrays
 * that hold a NaN or an infinity. Returns 0, or -1 with a message on a bad
 * argument or a CUDA error. */
enum {
  FGB_CHECK_T = 1,
  FGB_CHECK_TA = 2,
  FGB_CHECK_VEL = 4,
  FGB_CHECK_W = 8,
  FGB_CHECK_WE = 16,
  FGB_CHECK_WI = 32,
  FGB_CHECK_TLO = 64
};
int fgb_check_inputs(const fgb_mesh* m, const fgb_step_desc* d, void* stream, int* flags_out);

/* No counterpart in the reference: the current device's FP64 rates, the bound
 * of the FP64 forms. out3 receives fused multiply-add TFLOP/s, IEEE double
 * divisions per second (in G/s) and the milliseconds the two timed launches
 * took. Synchronises `stream`; 0 on success, -1 with a message. */
int fgb_probe_fp64(double* out3, void* stream);

#ifdef __cplusplus
}
#endif
#endif
