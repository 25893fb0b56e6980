// Host-side mesh of the tracer-advection step: connectivity, geometry and the
// derived gather tables the device kernels read. All indices are 0-based,
// -1 meaning "none"; level counts keep the reference's 1-based meaning
// (a column holds layers ulevels..nlevels-1).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fgb {

struct HostMesh {
  // sizes
  int N = 0, E = 0, M = 0, nl = 0, nz = 0, max_nie = 0, edge2D_in = 0;
  int periodic = 0, cluster_full = 0, orient_left = 0;
  double Lx = 0, Ly = 0;
  double cyclic = 360.0;  // cyclic_length, lib/gen_modules_config.F90:83 (degrees, never converted)

  // connectivity (reference names, lib/MOD_MESH.F90:24-184)
  std::vector<double> coord;          // (N,2) radians
  std::vector<int> elem_nodes;        // (M,3)
  std::vector<int> edges;             // (E,2)
  std::vector<int> edge_tri;          // (E,2), second -1 on walls
  std::vector<int> nlevels, ulevels;  // (M)
  std::vector<int> nlev_nod, ulev_nod;          // (N)
  std::vector<int> nlev_nod_min, ulev_nod_max;  // (N)
  std::vector<int> nie_num;           // (N) nod_in_elem2D_num
  std::vector<int> nie;               // (N,max_nie) nod_in_elem2D

  // geometry
  std::vector<double> zbar, Z;        // (nl), (nl-1)
  std::vector<double> elem_area;      // (M) m^2
  std::vector<double> area, areasvol; // (N,nl) m^2
  std::vector<double> edge_dxdy;      // (E,2) radians
  std::vector<double> edge_cross;     // (E,4) m
  std::vector<double> elem_cos;       // (M)
  std::vector<double> grad_sca;       // (M,6) 1/m

  // vertical (ALE) arrays
  std::vector<double> hnode, hnode_new;  // (N,nz)
  std::vector<double> helem;             // (M,nz)
  std::vector<double> Z3;                // (N,nz) Z_3d_n
  std::vector<double> zbar3;             // (N,nl) zbar_3d_n

  // MUSCL support
  std::vector<int> edge_updn;         // (E,2) up/downwind triangles
  std::vector<int> nboundary_lay;     // (N)

  // derived gather tables
  std::vector<int> ne_ptr;            // (N+1) incident edges, ascending edge index
  std::vector<int> ne_code;           // 2*edge + role (role 1: node is the edge's second node)
  std::vector<int> ne_other;          // other endpoint of that edge
  std::vector<int> ne_lo, ne_hi;      // that edge's scatter layer range (lib/oce_adv_tra_driver.F90:134-136)
  std::vector<int> nie_ptr;           // (N+1) CSR form of nod_in_elem2D
  std::vector<int> nie_idx;
  std::vector<int> cl_ptr;            // (N+1) distinct cluster nodes of the FCT bounds
  std::vector<int> cl_node, cl_lev;   // node, deepest layer reached through the cluster
  std::vector<int> cl_minlev;         // (N) shallowest element bottom layer in the cluster
  std::vector<int> edge_lev;          // (E,4) nu1,nl1,nu2,nl2 (1-based layers; nl = nlevels-1)
  std::vector<int> edge_gm;           // (E,2) layer window using the triangle gradients, -1 if none
  std::vector<double> edge_dxa;       // (E,2) edge_dxdy(1)*a, edge_dxdy(2)*r_earth
  std::vector<int> edge_order;        // (E) edges sorted by their first-visited node (locality of edge sweeps)
  std::vector<int> node_order;        // (N) order in which node kernels visit the columns; empty: node index
};

// Analytic mesh of lib/analytic_mesh.F90:114-829 with its geometry.
// Returns nullptr and sets err on invalid parameters.
// flags: kClusterFull (un-remapped nod_in_elem2D replaced by the full
// periodic lists), kOrientLeft (edge nodes swapped where edge_tri(1) lies on
// the right of node1 -> node2, the orientation of FESOM mesh files).
constexpr int kClusterFull = 1;
constexpr int kOrientLeft = 2;
constexpr int kVisitHilbert = 4;  // node and edge visit order along a Hilbert curve (visit_order_hilbert)
HostMesh* build_analytic(int nx, int ny, int nl, double Lx, double Ly, double depth, int periodic,
                         int flags, const double* zbar, const int* elem_nlev, std::string* err);

// A FESOM mesh from its files (nod2d.out, elem2d.out, aux3d.out, edgenum.out,
// edges.out, edge_tri.out, elvls.out, nlvls.out) as one partition, with the
// geometry of lib/oce_mesh.F90 on the sphere. flags: kFileNoRotation,
// kFileEulerDegrees, kFileCyclic2Pi (FESOM2's namelist handling instead of
// the reference's defaults).
constexpr int kFileNoRotation = 1;
constexpr int kFileEulerDegrees = 2;
constexpr int kFileCyclic2Pi = 4;
constexpr int kFileKeepOrder = 8;  // visit nodes and edges in file order (default: along a Hilbert curve)
HostMesh* build_from_files(const std::string& dir, int flags, std::string* err);
// The same from arrays laid out as the files are: lonlat (N,2) degrees, elem
// (M,3), edges and edge_tri (E,2) 1-based (edge_tri <= 0: none), elvls (M),
// nlvls (N), zbar (nl).
HostMesh* build_from_arrays(int N, int M, int E, int Ein, int nl, const double* lonlat, const int* elem,
                            const int* edges, const int* edge_tri, const int* elvls, const int* nlvls,
                            const double* zbar, int flags, std::string* err);

// Derived tables (CSR, cluster, per-edge level windows). Called by the builders.
void build_tables(HostMesh& m);

// Visit order of the kernels along a Hilbert curve through the nodes'
// coordinates: node_order, and edge_order by the first-visited node of each
// edge. Only the order of the work changes, not any index, array or result.
void visit_order_hilbert(HostMesh& m);

// Recompute the vertical arrays from zbar (the analytic driver's ALE set-up).
void ale_from_zbar(HostMesh& m);

// Disjoint union of independent meshes (the batching form: one launch
// advances all of them). Node, edge and element arrays are concatenated in
// part order with index offsets; per-layer arrays are padded to the largest
// nl, whose extra layers lie below every column of the shallower parts.
// Derived tables are rebuilt, so each part's gathers keep their order.
HostMesh* union_meshes(const HostMesh* const* parts, int count, std::string* err);

namespace detail {
// nod_in_elem2D in element order for nodes < nlimit (lib/oce_mesh.F90:1850-1999).
void node_elem_lists(const std::vector<int>& en, int M, int ntotal, int nlimit, std::vector<int>& num,
                     std::vector<int>& lst, int& maxn);
// Up/downwind triangle at `node` for the edge vector x (lib/oce_muscl_adv.F90:245-337).
int updn_search(const HostMesh& m, int node, const double* x);
}  // namespace detail

constexpr double kREarth = 6367500.0;   // lib/oce_modules.F90:24
constexpr double kPiRef = 3.14159265358979;  // lib/oce_modules.F90:19

}  // namespace fgb
