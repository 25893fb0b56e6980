/*
 * CPU oracle for the FESOM2 tracer-advection step (do_oce_adv_tra).
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C, loop-by-loop restatement of the
 * reference Fortran, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py as the checker. The product path never links it.
 *
 * Parity pin: the analytic dwarf configuration (20x20 periodic, nl=10,
 * UPW1/UPW1/NONE, frozen valuesAB, 10 steps) reproduces the golden per-step
 * T min/max/sum printed in the reference README.md:51-52 (tests/test_oracle.py).
 * MUSCL, FCT, QR4C, PPM and CDIFF are not exercised by any reference test:
 * for those the oracle follows the Fortran statement by statement, and parity
 * against the Fortran build itself is unpinned (no Fortran compiler exists on
 * either machine of this project).
 *
 * Index conventions: every array mirrors the Fortran column-major layout with
 * the first (level / component) index fastest; node, element and edge indices
 * stored inside arrays are 1-based, 0 meaning "none" (edge_tri(2,e) on walls).
 */
#ifndef FESOM_ORACLE_H
#define FESOM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { OM_HOR_UPW1 = 0, OM_HOR_MUSCL = 1, OM_HOR_MFCT = 2 };
enum { OM_VER_UPW1 = 0, OM_VER_QR4C = 1, OM_VER_CDIFF = 2, OM_VER_PPM = 3 };
enum { OM_LIM_NONE = 0, OM_LIM_FCT = 1 };

typedef struct omesh omesh;

/* Analytic mesh, lib/analytic_mesh.F90:114-829 plus the oce_mesh.F90 geometry it
 * calls. zbar (nl values, 0 at the surface, negative downwards) and elem_nlev
 * (nlevels per element, 1..nl) are optional overrides of the uniform flat
 * bottom; node levels are then the maximum over the adjacent elements (the
 * convention of the FESOM mesh files nlvls.out/elvls.out).
 * cluster_full=0 keeps nod_in_elem2D un-remapped on periodic meshes as the
 * reference does (lib/analytic_mesh.F90:675-694 runs before the remap at :705). */
omesh* om_mesh_analytic(int nx, int ny, int nl, double Lx, double Ly, double max_depth,
                        int periodic, int cluster_full, const double* zbar, const int* elem_nlev);
/* As om_mesh_analytic; orient_left=1 swaps the nodes of every edge whose
 * edge_tri(1) lies to the right of node1 -> node2 (FESOM mesh-file
 * orientation; the analytic grid, lib/analytic_mesh.F90:386-426, has it on
 * the right for horizontal and vertical edges). */
omesh* om_mesh_analytic2(int nx, int ny, int nl, double Lx, double Ly, double max_depth, int periodic,
                         int cluster_full, int orient_left, const double* zbar, const int* elem_nlev);
/* A FESOM mesh read from its files (the global mesh as one partition):
 * read_mesh, test_tri, load_edges, find_neighbors, find_levels,
 * find_levels_min_e2n, mesh_areas and mesh_auxiliary_arrays of
 * lib/oce_mesh.F90 with the reference's defaults (cartesian = .false.,
 * force_rotation = .true., the Euler angles 50/15/-90 used as given,
 * cyclic_length = 360), then the ALE arrays of tracer_init_ale_arrays and the
 * MUSCL set-up. lonlat (2,N) degrees as in nod2d.out; elem (3,M), edges (2,E),
 * edge_tri (2,E) 1-based as in elem2d.out, edges.out, edge_tri.out; elvls (M),
 * nlvls (N); zbar (nl) as in aux3d.out. Flags select FESOM2's namelist
 * handling instead: no rotation, Euler angles in degrees, cyclic_length 2*pi. */
enum { OM_FILE_NO_ROTATION = 1, OM_FILE_EULER_DEGREES = 2, OM_FILE_CYCLIC_2PI = 4 };
omesh* om_mesh_from_arrays(int nod2D, int elem2D, int edge2D, int edge2D_in, int nl, const double* lonlat,
                           const int* elem, const int* edges, const int* edge_tri, const int* elvls,
                           const int* nlvls, const double* zbar, int flags);
void om_mesh_free(omesh* m);
/* sizes: [nod2D, nod2D_total, elem2D, edge2D, edge2D_in, nl, max_nie] */
void om_mesh_sizes(const omesh* m, int* out7);
/* Copy a named mesh array into out (Fortran order). Returns element count or -1. */
long om_mesh_get_int(const omesh* m, const char* name, int* out);
long om_mesh_get_dbl(const omesh* m, const char* name, double* out);

/* Work arrays of one tracer step (T_TRACER_WORK, lib/MOD_TRACER.F90:30-62). */
typedef struct omwork omwork;
omwork* om_work_new(const omesh* m);
void om_work_free(omwork* w);
long om_work_get(const omwork* w, const char* name, double* out);

/* do_oce_adv_tra (lib/oce_adv_tra_driver.F90:23-294) for one tracer.
 * vel(2,nl-1,elem2D), w/wi/we(nl,nod2D), ttf/ttfAB(nl-1,nod2D).
 * dttf_h/dttf_v (nl-1,nod2D) are accumulated into (callers zero them). */
int om_do_oce_adv_tra(const omesh* m, omwork* wk, double dt, const double* vel,
                      const double* w, const double* wi, const double* we,
                      const double* ttf, const double* ttfAB, int hor, int ver, int lim,
                      double ph, double pv, int use_wsplit, double* dttf_h, double* dttf_v);

/* One step of the analytic driver loop for ntr tracers
 * (src/fesom_analytic.F90:404-437): zero tendencies, advect, accumulate, apply.
 * values/valuesAB are ntr consecutive (nl-1,nod2D) blocks. copy_ab=1 sets
 * valuesAB=values after each tracer update (frozen-AB when 0). */
int om_analytic_step(const omesh* m, omwork* wk, int ntr, double dt, const double* vel,
                     const double* w, double* values, double* valuesAB, const int* hor,
                     const int* ver, const int* lim, const double* ph, const double* pv,
                     int copy_ab, double* del_ttf);
/* The same with separate implicit / explicit vertical velocities: use_wsplit
 * applies adv_tra_vert_impl with wi to the FCT low-order solution
 * (lib/oce_adv_tra_driver.F90:221-231); we feeds the LO vertical flux.
 * copy_ab: 0 valuesAB frozen, 1 valuesAB = new values, 2 valuesAB =
 * -(0.5+ab_eps) old + (1.5+ab_eps) new (second-order Adams-Bashforth). */
int om_analytic_step_split(const omesh* m, omwork* wk, int ntr, double dt, const double* vel,
                           const double* w, const double* wi, const double* we, int use_wsplit,
                           double* values, double* valuesAB, const int* hor, const int* ver,
                           const int* lim, const double* ph, const double* pv, int copy_ab,
                           double ab_eps, double* del_ttf);

/* tracer_advect_step semantics (lib/tracer_c_interface.F90:163-220): tracer 1 only,
 * del_ttf accumulates across calls. */
int om_cabi_step(const omesh* m, omwork* wk, double dt, const double* vel, const double* w,
                 const double* wi, const double* we, double* values, double* valuesAB,
                 int hor, int ver, int lim, double ph, double pv, double* del_ttf);

/* Analytic initial fields of the dwarf (src/fesom_analytic.F90:306-331). */
void om_init_dwarf_fields(const omesh* m, double Lx, double Ly, double* T, double* S);

/* Step statistics (src/fesom_analytic.F90:441-445): min, max, plain sum, NaN count
 * over values(:, 1:myDim_nod2D). */
void om_stats(const omesh* m, const double* values, double* out4);

/* Threads of the parallel loops (OpenMP; 1 when built without it). Results
 * do not depend on the thread count. */
void om_set_threads(int n);
int om_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
