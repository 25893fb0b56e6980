/*
 * CPU oracle for the FESOM2 tracer-advection step. TEST INFRASTRUCTURE ONLY:
 * imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
 * as the checker; the product never links or calls it.
 *
 * Each routine restates the reference Fortran statement by statement and keeps
 * its floating-point evaluation order (the file is compiled with
 * -ffp-contract=off so that no multiply-add is fused). Citations are
 * path:line inside the reference project.
 *
 * Threads (OpenMP, om_set_threads) change no result: loops whose iterations
 * write disjoint data (per node column, per edge, per element) are split
 * across threads, and every edge scatter keeps the reference's order per
 * node -- each thread owns a contiguous range of nodes and walks all edges in
 * ascending index, applying only the updates of its own nodes.
 */
#include "fesom_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void om_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int om_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

#define OMP_FOR _Pragma("omp parallel for schedule(static)")
/* inside a scatter region: does this thread apply the updates of node n? */
#define OWNS(n) ((n) >= own_lo && (n) < own_hi)

/* Node range [*lo, *hi) (1-based) whose scatter updates the calling thread
 * applies: the whole mesh outside a parallel region. */
static void owner_range(int N, int* lo, int* hi) {
#ifdef _OPENMP
  const long t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
  const long t = 0, nt = 1;
#endif
  *lo = 1 + (int)(N * t / nt);
  *hi = 1 + (int)(N * (t + 1) / nt);
}

#define R_EARTH 6367500.0              /* lib/oce_modules.F90:24 */
#define PI_F 3.14159265358979          /* lib/oce_modules.F90:19 (truncated literal) */
#define CYCLIC_LENGTH 360.0            /* lib/gen_modules_config.F90:83 */

/* 1-based Fortran-style accessors: first index fastest. */
#define A2(a, ld, i, j) (a)[(size_t)((j)-1) * (size_t)(ld) + (size_t)((i)-1)]
#define A3(a, l1, l2, i, j, k) \
  (a)[((size_t)((k)-1) * (size_t)(l2) + (size_t)((j)-1)) * (size_t)(l1) + (size_t)((i)-1)]

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }

struct omesh {
  int nx, ny, nl, periodic, cluster_full;
  int cartesian;            /* lib/gen_modules_config.F90:81 (.true. for the analytic mesh) */
  double cyclic;            /* cyclic_length, lib/gen_modules_config.F90:83 */
  int nod2D, eDim, nod2D_total, elem2D, edge2D, edge2D_in, max_nie;
  double Lx, Ly;
  double* coord;            /* (2, nod2D_total) radians */
  int* elem2D_nodes;        /* (3, elem2D) */
  int* edges;               /* (2, edge2D) */
  int* edge_tri;            /* (2, edge2D) */
  int* nod_in_elem2D_num;   /* (nod2D_total) */
  int* nod_in_elem2D;       /* (max_nie, nod2D_total) */
  int* nlevels;             /* (elem2D) */
  int* ulevels;             /* (elem2D) */
  int* nlevels_nod2D;       /* (nod2D_total) */
  int* ulevels_nod2D;       /* (nod2D_total) */
  int* nlevels_nod2D_min;   /* (nod2D_total) */
  int* ulevels_nod2D_max;   /* (nod2D_total) */
  double* zbar;             /* (nl) */
  double* Z;                /* (nl-1) */
  double* elem_area;        /* (elem2D) m^2 */
  double* area;             /* (nl, nod2D_total) m^2 */
  double* areasvol;         /* (nl, nod2D_total) m^2 */
  double* edge_dxdy;        /* (2, edge2D) radians */
  double* edge_cross_dxdy;  /* (4, edge2D) m */
  double* elem_cos;         /* (elem2D) */
  double* gradient_sca;     /* (6, elem2D) 1/m */
  double* hnode;            /* (nl-1, nod2D) */
  double* hnode_new;        /* (nl-1, nod2D) */
  double* helem;            /* (nl-1, elem2D) */
  double* Z_3d_n;           /* (nl-1, nod2D) */
  double* zbar_3d_n;        /* (nl, nod2D) */
  int* edge_up_dn_tri;      /* (2, edge2D) */
  int* nboundary_lay;       /* (nod2D) */
};

struct omwork {
  int nl, N, E, M;
  double* fct_LO;           /* (nl-1, N) */
  double* adv_flux_hor;     /* (nl-1, E) */
  double* adv_flux_ver;     /* (nl, N) */
  double* fct_ttf_max;      /* (nl-1, N) */
  double* fct_ttf_min;
  double* fct_plus;
  double* fct_minus;
  double* tvert_max;        /* (nl-1, N) automatic array in the Fortran */
  double* tvert_min;
  double* aux;              /* (2, nl-1, M): the AUX of oce_tra_adv_fct */
  double* edge_up_dn_grad;  /* (4, nl-1, E) */
  double* tr_xy;            /* (2, nl-1, M) */
  double* adf_h_raw;        /* (nl-1, E) antidiffusive flux before limiting */
  double* adf_v_raw;        /* (nl, N) */
};

static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s);
  if (!p) abort();
  return p;
}

/* ------------------------------------------------------------------------- */
/* Mesh generation: lib/analytic_mesh.F90:114-829                             */
/* ------------------------------------------------------------------------- */

typedef struct { int nx, ny, nod2D, nod2D_total; } pctx;

/* pnode, lib/analytic_mesh.F90:721-733 */
static int pnode(const pctx* c, int i, int j) {
  if (i <= c->nx - 1 && j <= c->ny - 1) return (j - 1) * (c->nx - 1) + i;
  if (i == c->nx && j <= c->ny - 1) return c->nod2D + j;
  if (i <= c->nx - 1 && j == c->ny) return c->nod2D + (c->ny - 1) + i;
  return c->nod2D_total;
}

/* trim_cyclic_mp, lib/gen_modules_rotate_grid.F90:216-224. With the
 * reference's cyclic_length = 360 (degrees, never converted) it never fires on
 * radian coordinates. */
static double trim_cyc(const omesh* m, double b) {
  if (b > m->cyclic / 2.0) b = b - m->cyclic;
  if (b < -m->cyclic / 2.0) b = b + m->cyclic;
  return b;
}

static void build_nod_in_elem(omesh* m, int nnodes) {
  free(m->nod_in_elem2D_num);
  free(m->nod_in_elem2D);
  m->nod_in_elem2D_num = (int*)xcalloc((size_t)m->nod2D_total, sizeof(int));
  for (int n = 1; n <= m->elem2D; ++n)
    for (int j = 1; j <= 3; ++j) {
      int node = A2(m->elem2D_nodes, 3, j, n);
      if (node <= nnodes) m->nod_in_elem2D_num[node - 1] += 1;
    }
  int mx = 0;
  for (int n = 0; n < m->nod2D_total; ++n) mx = imax(mx, m->nod_in_elem2D_num[n]);
  m->max_nie = mx;
  m->nod_in_elem2D = (int*)xcalloc((size_t)mx * (size_t)m->nod2D_total, sizeof(int));
  memset(m->nod_in_elem2D_num, 0, sizeof(int) * (size_t)m->nod2D_total);
  for (int n = 1; n <= m->elem2D; ++n)
    for (int j = 1; j <= 3; ++j) {
      int node = A2(m->elem2D_nodes, 3, j, n);
      if (node > nnodes) continue;
      m->nod_in_elem2D_num[node - 1] += 1;
      A2(m->nod_in_elem2D, mx, m->nod_in_elem2D_num[node - 1], node) = n;
    }
}

/* find_levels_min_e2n, lib/oce_mesh.F90:1522-1560 */
static void find_levels_min_e2n(omesh* m) {
  for (int node = 1; node <= m->nod2D; ++node) {
    int k = m->nod_in_elem2D_num[node - 1];
    int mn = 1 << 30, mx = -(1 << 30);
    for (int j = 1; j <= k; ++j) {
      int el = A2(m->nod_in_elem2D, m->max_nie, j, node);
      mn = imin(mn, m->nlevels[el - 1]);
      mx = imax(mx, m->ulevels[el - 1]);
    }
    m->nlevels_nod2D_min[node - 1] = mn;
    m->ulevels_nod2D_max[node - 1] = mx;
  }
}

/* test_tri, lib/oce_mesh.F90:1565-1615 */
static void test_tri(omesh* m) {
  for (int n = 1; n <= m->elem2D; ++n) {
    int* el = &A2(m->elem2D_nodes, 3, 1, n);
    double a0 = A2(m->coord, 2, 1, el[0]), a1 = A2(m->coord, 2, 2, el[0]);
    double b0 = A2(m->coord, 2, 1, el[1]) - a0, b1 = A2(m->coord, 2, 2, el[1]) - a1;
    double c0 = A2(m->coord, 2, 1, el[2]) - a0, c1 = A2(m->coord, 2, 2, el[2]) - a1;
    b0 = trim_cyc(m, b0);
    c0 = trim_cyc(m, c0);
    double r = b0 * c1 - b1 * c0;
    if (r > 0.0) {
      int t = el[1];
      el[1] = el[2];
      el[2] = t;
    }
  }
}

/* mesh_areas, lib/oce_mesh.F90:2043-2309 (no cavity) */
static void mesh_areas(omesh* m) {
  const int nl = m->nl;
  for (int n = 1; n <= m->elem2D; ++n) {
    const int* el = &A2(m->elem2D_nodes, 3, 1, n);
    double ay = (A2(m->coord, 2, 2, el[0]) + A2(m->coord, 2, 2, el[1]) + A2(m->coord, 2, 2, el[2])) / 3.0;
    ay = cos(ay);
    if (m->cartesian) ay = 1.0; /* lib/oce_mesh.F90:2091-2093 */
    double a0 = A2(m->coord, 2, 1, el[1]) - A2(m->coord, 2, 1, el[0]);
    double a1 = A2(m->coord, 2, 2, el[1]) - A2(m->coord, 2, 2, el[0]);
    double b0 = A2(m->coord, 2, 1, el[2]) - A2(m->coord, 2, 1, el[0]);
    double b1 = A2(m->coord, 2, 2, el[2]) - A2(m->coord, 2, 2, el[0]);
    a0 = trim_cyc(m, a0);
    b0 = trim_cyc(m, b0);
    a0 = a0 * ay;
    b0 = b0 * ay;
    m->elem_area[n - 1] = 0.5 * fabs(a0 * b1 - b0 * a1);
  }
  for (int n = 1; n <= m->nod2D_total; ++n) {
    for (int j = 1; j <= m->nod_in_elem2D_num[n - 1]; ++j) {
      int elem = A2(m->nod_in_elem2D, m->max_nie, j, n);
      int nzmin = m->ulevels[elem - 1], nzmax = m->nlevels[elem - 1] - 1;
      for (int nz = nzmin; nz <= nzmax; ++nz)
        A2(m->area, nl, nz, n) = A2(m->area, nl, nz, n) + m->elem_area[elem - 1] / 3.0;
    }
  }
  for (int n = 1; n <= m->nod2D_total; ++n) {
    int nzmin = m->ulevels_nod2D[n - 1], nzmax = m->nlevels_nod2D[n - 1] - 1;
    for (int nz = nzmin; nz <= nzmax; ++nz) A2(m->areasvol, nl, nz, n) = A2(m->area, nl, nz, n);
  }
  for (int n = 0; n < m->elem2D; ++n) m->elem_area[n] = m->elem_area[n] * R_EARTH * R_EARTH;
  for (size_t i = 0; i < (size_t)nl * (size_t)m->nod2D_total; ++i) {
    m->area[i] = m->area[i] * R_EARTH * R_EARTH;
    m->areasvol[i] = m->areasvol[i] * R_EARTH * R_EARTH;
  }
}

/* elem_center, lib/oce_mesh.F90:2021-2041 */
static void elem_center(const omesh* m, int elem, double* x, double* y) {
  const int* el = &A2(m->elem2D_nodes, 3, 1, elem);
  double ax[3];
  for (int k = 0; k < 3; ++k) ax[k] = A2(m->coord, 2, 1, el[k]);
  double amin = dmin(dmin(ax[0], ax[1]), ax[2]);
  for (int k = 0; k < 3; ++k) {
    if (ax[k] - amin >= m->cyclic / 2.0) ax[k] = ax[k] - m->cyclic;
    if (ax[k] - amin < -m->cyclic / 2.0) ax[k] = ax[k] + m->cyclic;
  }
  *x = (ax[0] + ax[1] + ax[2]) / 3.0;
  *y = (A2(m->coord, 2, 2, el[0]) + A2(m->coord, 2, 2, el[1]) + A2(m->coord, 2, 2, el[2])) / 3.0;
}

/* mesh_auxiliary_arrays, lib/oce_mesh.F90:2313-2534 (the parts the step reads) */
static void mesh_auxiliary_arrays(omesh* m) {
  double* cx = (double*)xcalloc((size_t)m->elem2D, sizeof(double));
  double* cy = (double*)xcalloc((size_t)m->elem2D, sizeof(double));
  for (int n = 1; n <= m->elem2D; ++n) {
    elem_center(m, n, &cx[n - 1], &cy[n - 1]);
    m->elem_cos[n - 1] = m->cartesian ? 1.0 : cos(cy[n - 1]); /* :2408-2421 */
  }
  for (int n = 1; n <= m->edge2D; ++n) {
    int e1 = A2(m->edges, 2, 1, n), e2 = A2(m->edges, 2, 2, n);
    double a0 = A2(m->coord, 2, 1, e2) - A2(m->coord, 2, 1, e1);
    double a1 = A2(m->coord, 2, 2, e2) - A2(m->coord, 2, 2, e1);
    a0 = trim_cyc(m, a0);
    A2(m->edge_dxdy, 2, 1, n) = a0;
    A2(m->edge_dxdy, 2, 2, n) = a1;
  }
  for (int n = 1; n <= m->edge2D; ++n) {
    int e1 = A2(m->edges, 2, 1, n), e2 = A2(m->edges, 2, 2, n);
    int el1 = A2(m->edge_tri, 2, 1, n), el2 = A2(m->edge_tri, 2, 2, n);
    /* edge_center, lib/oce_mesh.F90:2001-2019 */
    double p0 = A2(m->coord, 2, 1, e1), p1 = A2(m->coord, 2, 2, e1);
    double q0 = A2(m->coord, 2, 1, e2), q1 = A2(m->coord, 2, 2, e2);
    if (p0 - q0 > m->cyclic / 2.0) p0 = p0 - m->cyclic;
    if (p0 - q0 < -m->cyclic / 2.0) q0 = q0 - m->cyclic;
    double ax = 0.5 * (p0 + q0), ay = 0.5 * (p1 + q1);
    double b0 = cx[el1 - 1] - ax, b1 = cy[el1 - 1] - ay;
    b0 = trim_cyc(m, b0);
    b0 = b0 * m->elem_cos[el1 - 1];
    b0 = b0 * R_EARTH;
    b1 = b1 * R_EARTH;
    A2(m->edge_cross_dxdy, 4, 1, n) = b0;
    A2(m->edge_cross_dxdy, 4, 2, n) = b1;
    if (el2 > 0) {
      b0 = cx[el2 - 1] - ax;
      b1 = cy[el2 - 1] - ay;
      b0 = trim_cyc(m, b0);
      b0 = b0 * m->elem_cos[el2 - 1];
      b0 = b0 * R_EARTH;
      b1 = b1 * R_EARTH;
      A2(m->edge_cross_dxdy, 4, 3, n) = b0;
      A2(m->edge_cross_dxdy, 4, 4, n) = b1;
    } else {
      A2(m->edge_cross_dxdy, 4, 3, n) = 0.0;
      A2(m->edge_cross_dxdy, 4, 4, n) = 0.0;
    }
  }
  for (int elem = 1; elem <= m->elem2D; ++elem) {
    const int* el = &A2(m->elem2D_nodes, 3, 1, elem);
    double dX31 = A2(m->coord, 2, 1, el[2]) - A2(m->coord, 2, 1, el[0]);
    dX31 = trim_cyc(m, dX31);
    dX31 = m->elem_cos[elem - 1] * dX31;
    double dX21 = A2(m->coord, 2, 1, el[1]) - A2(m->coord, 2, 1, el[0]);
    dX21 = trim_cyc(m, dX21);
    dX21 = m->elem_cos[elem - 1] * dX21;
    double dY31 = A2(m->coord, 2, 2, el[2]) - A2(m->coord, 2, 2, el[0]);
    double dY21 = A2(m->coord, 2, 2, el[1]) - A2(m->coord, 2, 2, el[0]);
    double dfactor = -(0.5 * R_EARTH / m->elem_area[elem - 1]);
    double* g = &A2(m->gradient_sca, 6, 1, elem);
    g[0] = (-dY31 + dY21) * dfactor;
    g[1] = dY31 * dfactor;
    g[2] = -dY21 * dfactor;
    g[3] = (dX31 - dX21) * dfactor;
    g[4] = -dX31 * dfactor;
    g[5] = dX21 * dfactor;
  }
  free(cx);
  free(cy);
}

/* periodic_post_remap, lib/analytic_mesh.F90:736-827 */
static void periodic_post_remap(omesh* m) {
  const int nx = m->nx, ny = m->ny, eDim = m->eDim, nl = m->nl;
  int* h2r = (int*)xcalloc((size_t)eDim, sizeof(int));
  for (int h = 1; h <= ny - 1; ++h) h2r[h - 1] = (h - 1) * (nx - 1) + 1;
  for (int h = 1; h <= nx - 1; ++h) h2r[(ny - 1) + h - 1] = h;
  h2r[eDim - 1] = 1;
  double half_Lx = 0.5 * m->Lx, half_Ly = 0.5 * m->Ly;
  for (int n = 1; n <= m->edge2D; ++n) {
    for (int k = 1; k <= 3; k += 2) {
      double val = A2(m->edge_cross_dxdy, 4, k, n);
      if (fabs(val) > half_Lx) A2(m->edge_cross_dxdy, 4, k, n) = val - copysign(m->Lx, val);
      val = A2(m->edge_cross_dxdy, 4, k + 1, n);
      if (fabs(val) > half_Ly) A2(m->edge_cross_dxdy, 4, k + 1, n) = val - copysign(m->Ly, val);
    }
  }
  for (int h = 1; h <= eDim; ++h) {
    int r = h2r[h - 1];
    for (int nz = 1; nz <= nl - 1; ++nz) {
      A2(m->area, nl, nz, r) = A2(m->area, nl, nz, r) + A2(m->area, nl, nz, m->nod2D + h);
      A2(m->areasvol, nl, nz, r) = A2(m->areasvol, nl, nz, r) + A2(m->areasvol, nl, nz, m->nod2D + h);
    }
  }
  for (int n = 1; n <= m->elem2D; ++n)
    for (int k = 1; k <= 3; ++k) {
      int h = A2(m->elem2D_nodes, 3, k, n);
      if (h > m->nod2D) A2(m->elem2D_nodes, 3, k, n) = h2r[h - m->nod2D - 1];
    }
  for (int n = 1; n <= m->edge2D; ++n)
    for (int k = 1; k <= 2; ++k) {
      int h = A2(m->edges, 2, k, n);
      if (h > m->nod2D) A2(m->edges, 2, k, n) = h2r[h - m->nod2D - 1];
    }
  free(h2r);
}

/* nboundary_lay part of muscl_adv_init, lib/oce_muscl_adv.F90:96-159 */
static void muscl_nboundary_lay(omesh* m) {
  for (int n = 0; n < m->nod2D; ++n) m->nboundary_lay[n] = m->nl - 1;
  for (int n = 1; n <= m->edge2D; ++n) {
    int t1 = A2(m->edge_tri, 2, 1, n), t2 = A2(m->edge_tri, 2, 2, n);
    int e1 = A2(m->edges, 2, 1, n), e2 = A2(m->edges, 2, 2, n);
    if (t1 <= 0 || t2 <= 0) {
      m->nboundary_lay[e1 - 1] = 0;
      m->nboundary_lay[e2 - 1] = 0;
    } else {
      int mn = imin(m->nlevels[t1 - 1], m->nlevels[t2 - 1]) - 1;
      m->nboundary_lay[e1 - 1] = imin(m->nboundary_lay[e1 - 1], mn);
      m->nboundary_lay[e2 - 1] = imin(m->nboundary_lay[e2 - 1], mn);
    }
  }
}

/* Minimum-image wrap used by the up/downwind triangle search on periodic meshes.
 * The reference trims only x and with cyclic_length=360 (a no-op in radians);
 * the analytic periodic domain has periods Lx/r_earth and Ly/r_earth. */
static void wrap_mi(const omesh* m, double* v) {
  if (!m->periodic) return;
  double px = m->Lx / R_EARTH, py = m->Ly / R_EARTH;
  if (v[0] > 0.5 * px) v[0] = v[0] - px;
  if (v[0] < -0.5 * px) v[0] = v[0] + px;
  if (v[1] > 0.5 * py) v[1] = v[1] - py;
  if (v[1] < -0.5 * py) v[1] = v[1] + py;
}

/* find_up_downwind_triangles, lib/oce_muscl_adv.F90:166-357. The Fortran
 * `cycle` continues the search, so the LAST matching element is kept. */
static int updn_search(const omesh* m, int node, const double* x) {
  int found = 0;
  for (int k = 1; k <= m->nod_in_elem2D_num[node - 1]; ++k) {
    int elem = A2(m->nod_in_elem2D, m->max_nie, k, node);
    const int* en = &A2(m->elem2D_nodes, 3, 1, elem);
    int v1, v2, v3;
    if (en[0] == node) { v1 = en[0]; v2 = en[1]; v3 = en[2]; }
    else if (en[1] == node) { v1 = en[1]; v2 = en[0]; v3 = en[2]; }
    else { v1 = en[2]; v2 = en[0]; v3 = en[1]; }
    double b[2] = {A2(m->coord, 2, 1, v2) - A2(m->coord, 2, 1, v1), A2(m->coord, 2, 2, v2) - A2(m->coord, 2, 2, v1)};
    double c[2] = {A2(m->coord, 2, 1, v3) - A2(m->coord, 2, 1, v1), A2(m->coord, 2, 2, v3) - A2(m->coord, 2, 2, v1)};
    b[0] = trim_cyc(m, b[0]);
    c[0] = trim_cyc(m, c[0]);
    wrap_mi(m, b);
    wrap_mi(m, c);
    double cr = c[0] * c[0] + c[1] * c[1];
    double bx = (b[0] * c[0] + b[1] * c[1]) / cr;
    double by = (-b[0] * c[1] + b[1] * c[0]) / cr;
    double xx = (x[0] * c[0] + x[1] * c[1]) / cr;
    double xy = (-x[0] * c[1] + x[1] * c[0]) / cr;
    double ab = atan2(by, bx);
    double ax = atan2(xy, xx);
    if (ab > 0.0 && ax > 0.0 && ax < ab) { found = elem; continue; }
    if (ab < 0.0 && ax < 0.0 && ax > ab) { found = elem; continue; }
    if (ab == ax || ax == 0.0) { found = elem; continue; }
  }
  return found;
}

static void find_up_downwind_triangles(omesh* m) {
  for (int n = 1; n <= m->edge2D; ++n) {
    int e1 = A2(m->edges, 2, 1, n), e2 = A2(m->edges, 2, 2, n);
    double x[2] = {A2(m->coord, 2, 1, e2) - A2(m->coord, 2, 1, e1), A2(m->coord, 2, 2, e2) - A2(m->coord, 2, 2, e1)};
    x[0] = trim_cyc(m, x[0]);
    wrap_mi(m, x);
    x[0] = -x[0];
    x[1] = -x[1];
    A2(m->edge_up_dn_tri, 2, 1, n) = updn_search(m, e1, x);
    x[0] = -x[0];
    x[1] = -x[1];
    A2(m->edge_up_dn_tri, 2, 2, n) = updn_search(m, e2, x);
  }
}

/* ALE arrays from zbar (src/fesom_analytic.F90:206-244, the same as
 * tracer_init_ale_arrays, lib/tracer_c_interface.F90:875-925) and the MUSCL
 * set-up (lib/oce_muscl_adv.F90:38-357). */
static void finish_mesh(omesh* m) {
  const int N = m->nod2D, M = m->elem2D, E = m->edge2D, nl = m->nl, nz = nl - 1;
  m->hnode = (double*)xcalloc((size_t)nz * N, sizeof(double));
  m->hnode_new = (double*)xcalloc((size_t)nz * N, sizeof(double));
  m->helem = (double*)xcalloc((size_t)nz * M, sizeof(double));
  m->Z_3d_n = (double*)xcalloc((size_t)nz * N, sizeof(double));
  m->zbar_3d_n = (double*)xcalloc((size_t)nl * N, sizeof(double));
  for (int n = 1; n <= N; ++n)
    for (int k = 1; k <= nz; ++k) {
      A2(m->hnode, nz, k, n) = m->zbar[k - 1] - m->zbar[k];
      A2(m->hnode_new, nz, k, n) = A2(m->hnode, nz, k, n);
    }
  for (int n = 1; n <= M; ++n)
    for (int k = 1; k <= nz; ++k) A2(m->helem, nz, k, n) = m->zbar[k - 1] - m->zbar[k];
  for (int n = 1; n <= N; ++n) {
    for (int k = 1; k <= nl; ++k) A2(m->zbar_3d_n, nl, k, n) = m->zbar[k - 1];
    for (int k = 1; k <= nz; ++k) A2(m->Z_3d_n, nz, k, n) = m->Z[k - 1];
  }

  /* MUSCL set-up (lib/oce_muscl_adv.F90:38-357) */
  m->nboundary_lay = (int*)xcalloc((size_t)N, sizeof(int));
  m->edge_up_dn_tri = (int*)xcalloc((size_t)2 * E, sizeof(int));
  muscl_nboundary_lay(m);
  find_up_downwind_triangles(m);
}


omesh* om_mesh_analytic(int nx, int ny, int nl, double Lx, double Ly, double max_depth,
                        int periodic, int cluster_full, const double* zbar_in, const int* elem_nlev) {
  return om_mesh_analytic2(nx, ny, nl, Lx, Ly, max_depth, periodic, cluster_full, 0, zbar_in, elem_nlev);
}

omesh* om_mesh_analytic2(int nx, int ny, int nl, double Lx, double Ly, double max_depth, int periodic,
                         int cluster_full, int orient_left, const double* zbar_in, const int* elem_nlev) {
  if (nx < 2 || ny < 2 || nl < 3) return NULL;
  if (periodic && (nx < 3 || ny < 3)) return NULL;
  omesh* m = (omesh*)xcalloc(1, sizeof(omesh));
  m->nx = nx; m->ny = ny; m->nl = nl; m->periodic = periodic; m->cluster_full = cluster_full;
  m->cartesian = 1; /* lib/analytic_mesh.F90:162 */
  m->cyclic = CYCLIC_LENGTH;
  m->Lx = Lx; m->Ly = Ly;
  int n_horiz, n_vert, n_diag;
  if (periodic) {
    m->nod2D = (nx - 1) * (ny - 1);
    m->eDim = (nx - 1) + (ny - 1) + 1;
    n_horiz = n_vert = n_diag = (nx - 1) * (ny - 1);
  } else {
    m->nod2D = nx * ny;
    m->eDim = 0;
    n_horiz = (nx - 1) * ny;
    n_vert = nx * (ny - 1);
    n_diag = (nx - 1) * (ny - 1);
  }
  m->nod2D_total = m->nod2D + m->eDim;
  m->elem2D = 2 * (nx - 1) * (ny - 1);
  m->edge2D = n_horiz + n_vert + n_diag;
  const int NT = m->nod2D_total, M = m->elem2D, E = m->edge2D;
  pctx pc = {nx, ny, m->nod2D, NT};

  /* 1c. coordinates, lib/analytic_mesh.F90:268-305 */
  double dx = Lx / (double)(nx - 1), dy = Ly / (double)(ny - 1);
  m->coord = (double*)xcalloc((size_t)2 * NT, sizeof(double));
  if (periodic) {
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        int n = (j - 1) * (nx - 1) + i;
        A2(m->coord, 2, 1, n) = (double)(i - 1) * dx / R_EARTH;
        A2(m->coord, 2, 2, n) = (double)(j - 1) * dy / R_EARTH;
      }
    for (int j = 1; j <= ny - 1; ++j) {
      int n = m->nod2D + j;
      A2(m->coord, 2, 1, n) = Lx / R_EARTH;
      A2(m->coord, 2, 2, n) = (double)(j - 1) * dy / R_EARTH;
    }
    for (int i = 1; i <= nx - 1; ++i) {
      int n = m->nod2D + (ny - 1) + i;
      A2(m->coord, 2, 1, n) = (double)(i - 1) * dx / R_EARTH;
      A2(m->coord, 2, 2, n) = Ly / R_EARTH;
    }
    A2(m->coord, 2, 1, NT) = Lx / R_EARTH;
    A2(m->coord, 2, 2, NT) = Ly / R_EARTH;
  } else {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        int n = (j - 1) * nx + i;
        A2(m->coord, 2, 1, n) = (double)(i - 1) * dx / R_EARTH;
        A2(m->coord, 2, 2, n) = (double)(j - 1) * dy / R_EARTH;
      }
  }

  /* 1d. elements (CW), :310-354 */
  m->elem2D_nodes = (int*)xcalloc((size_t)3 * M, sizeof(int));
  {
    int e = 0;
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        int n1, n2, n3, n4;
        if (periodic) {
          n1 = pnode(&pc, i, j); n2 = pnode(&pc, i + 1, j);
          n3 = pnode(&pc, i + 1, j + 1); n4 = pnode(&pc, i, j + 1);
        } else {
          n1 = (j - 1) * nx + i; n2 = (j - 1) * nx + i + 1;
          n3 = j * nx + i + 1; n4 = j * nx + i;
        }
        e += 1;
        A2(m->elem2D_nodes, 3, 1, e) = n1; A2(m->elem2D_nodes, 3, 2, e) = n3; A2(m->elem2D_nodes, 3, 3, e) = n2;
        e += 1;
        A2(m->elem2D_nodes, 3, 1, e) = n1; A2(m->elem2D_nodes, 3, 2, e) = n4; A2(m->elem2D_nodes, 3, 3, e) = n3;
      }
  }

  /* 1e. vertical levels, :359-373 */
  m->zbar = (double*)xcalloc((size_t)nl, sizeof(double));
  m->Z = (double*)xcalloc((size_t)nl, sizeof(double));
  for (int k = 1; k <= nl; ++k)
    m->zbar[k - 1] = zbar_in ? zbar_in[k - 1] : -(double)(k - 1) * max_depth / (double)(nl - 1);
  for (int k = 1; k <= nl - 1; ++k) m->Z[k - 1] = 0.5 * (m->zbar[k - 1] + m->zbar[k]);

  /* 1f. edges and edge_tri, :378-596 */
  int* en = (int*)xcalloc((size_t)2 * E, sizeof(int));
  int* ee = (int*)xcalloc((size_t)2 * E, sizeof(int));
  int ec = 0;
  if (periodic) {
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ec++;
        A2(en, 2, 1, ec) = pnode(&pc, i, j);
        A2(en, 2, 2, ec) = pnode(&pc, i + 1, j);
        int e_lower = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 1;
        int e_upper = (j >= 2) ? 2 * ((j - 2) * (nx - 1) + (i - 1)) + 2 : 2 * ((ny - 2) * (nx - 1) + (i - 1)) + 2;
        A2(ee, 2, 1, ec) = e_upper; A2(ee, 2, 2, ec) = e_lower;
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ec++;
        A2(en, 2, 1, ec) = pnode(&pc, i, j);
        A2(en, 2, 2, ec) = pnode(&pc, i, j + 1);
        int e_upper = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 2;
        int e_lower = (i >= 2) ? 2 * ((j - 1) * (nx - 1) + (i - 2)) + 1 : 2 * ((j - 1) * (nx - 1) + (nx - 2)) + 1;
        A2(ee, 2, 1, ec) = e_upper; A2(ee, 2, 2, ec) = e_lower;
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ec++;
        A2(en, 2, 1, ec) = pnode(&pc, i, j);
        A2(en, 2, 2, ec) = pnode(&pc, i + 1, j + 1);
        A2(ee, 2, 1, ec) = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 2;
        A2(ee, 2, 2, ec) = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 1;
      }
    m->edges = en;
    m->edge_tri = ee;
    m->edge2D_in = E;
  } else {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ec++;
        A2(en, 2, 1, ec) = (j - 1) * nx + i;
        A2(en, 2, 2, ec) = (j - 1) * nx + i + 1;
        int e_lower = (j <= ny - 1) ? 2 * ((j - 1) * (nx - 1) + (i - 1)) + 1 : 0;
        int e_upper = (j >= 2) ? 2 * ((j - 2) * (nx - 1) + (i - 1)) + 2 : 0;
        A2(ee, 2, 1, ec) = e_upper; A2(ee, 2, 2, ec) = e_lower;
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        ec++;
        A2(en, 2, 1, ec) = (j - 1) * nx + i;
        A2(en, 2, 2, ec) = j * nx + i;
        int e_upper = (i <= nx - 1) ? 2 * ((j - 1) * (nx - 1) + (i - 1)) + 2 : 0;
        int e_lower = (i >= 2) ? 2 * ((j - 1) * (nx - 1) + (i - 2)) + 1 : 0;
        A2(ee, 2, 1, ec) = e_upper; A2(ee, 2, 2, ec) = e_lower;
      }
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        ec++;
        A2(en, 2, 1, ec) = (j - 1) * nx + i;
        A2(en, 2, 2, ec) = j * nx + i + 1;
        A2(ee, 2, 1, ec) = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 2;
        A2(ee, 2, 2, ec) = 2 * ((j - 1) * (nx - 1) + (i - 1)) + 1;
      }
    for (int n = 1; n <= E; ++n)
      if (A2(ee, 2, 1, n) == 0 && A2(ee, 2, 2, n) > 0) {
        A2(ee, 2, 1, n) = A2(ee, 2, 2, n);
        A2(ee, 2, 2, n) = 0;
      }
    m->edges = (int*)xcalloc((size_t)2 * E, sizeof(int));
    m->edge_tri = (int*)xcalloc((size_t)2 * E, sizeof(int));
    int eidx = 0;
    for (int pass = 0; pass < 2; ++pass)
      for (int n = 1; n <= E; ++n) {
        int internal = A2(ee, 2, 1, n) > 0 && A2(ee, 2, 2, n) > 0;
        if ((pass == 0) != internal) continue;
        eidx++;
        A2(m->edges, 2, 1, eidx) = A2(en, 2, 1, n);
        A2(m->edges, 2, 2, eidx) = A2(en, 2, 2, n);
        A2(m->edge_tri, 2, 1, eidx) = A2(ee, 2, 1, n);
        A2(m->edge_tri, 2, 2, eidx) = A2(ee, 2, 2, n);
        if (pass == 0) m->edge2D_in = eidx;
      }
    free(en);
    free(ee);
  }

  if (orient_left) {
    for (int n = 1; n <= E; ++n) {
      int a = A2(m->edges, 2, 1, n), b = A2(m->edges, 2, 2, n), el = A2(m->edge_tri, 2, 1, n);
      const int* v = &A2(m->elem2D_nodes, 3, 1, el);
      double cx = (A2(m->coord, 2, 1, v[0]) + A2(m->coord, 2, 1, v[1]) + A2(m->coord, 2, 1, v[2])) / 3.0;
      double cy = (A2(m->coord, 2, 2, v[0]) + A2(m->coord, 2, 2, v[1]) + A2(m->coord, 2, 2, v[2])) / 3.0;
      double dx0 = A2(m->coord, 2, 1, b) - A2(m->coord, 2, 1, a), dy0 = A2(m->coord, 2, 2, b) - A2(m->coord, 2, 2, a);
      double s[2] = {cx - A2(m->coord, 2, 1, a), cy - A2(m->coord, 2, 2, a)};
      wrap_mi(m, s);
      double sx = s[0], sy = s[1];
      if (dx0 * sy - dy0 * sx < 0.0) {
        A2(m->edges, 2, 1, n) = b;
        A2(m->edges, 2, 2, n) = a;
      }
    }
  }

  /* 1g. levels, :601-608 (element overrides: see header) */
  m->nlevels = (int*)xcalloc((size_t)M, sizeof(int));
  m->ulevels = (int*)xcalloc((size_t)M, sizeof(int));
  m->nlevels_nod2D = (int*)xcalloc((size_t)NT, sizeof(int));
  m->ulevels_nod2D = (int*)xcalloc((size_t)NT, sizeof(int));
  m->nlevels_nod2D_min = (int*)xcalloc((size_t)NT, sizeof(int));
  m->ulevels_nod2D_max = (int*)xcalloc((size_t)NT, sizeof(int));
  for (int e = 0; e < M; ++e) {
    m->nlevels[e] = elem_nlev ? elem_nlev[e] : nl;
    m->ulevels[e] = 1;
  }
  for (int n = 0; n < NT; ++n) {
    m->nlevels_nod2D[n] = elem_nlev ? 0 : nl;
    m->ulevels_nod2D[n] = 1;
  }
  if (elem_nlev) {
    for (int e = 1; e <= M; ++e)
      for (int k = 1; k <= 3; ++k) {
        int node = A2(m->elem2D_nodes, 3, k, e);
        m->nlevels_nod2D[node - 1] = imax(m->nlevels_nod2D[node - 1], m->nlevels[e - 1]);
      }
    if (periodic) { /* a halo copy and its real node are one column */
      int* h2r = (int*)xcalloc((size_t)m->eDim, sizeof(int));
      for (int h = 1; h <= ny - 1; ++h) h2r[h - 1] = (h - 1) * (nx - 1) + 1;
      for (int h = 1; h <= nx - 1; ++h) h2r[(ny - 1) + h - 1] = h;
      h2r[m->eDim - 1] = 1;
      for (int h = 1; h <= m->eDim; ++h) {
        int r = h2r[h - 1];
        m->nlevels_nod2D[r - 1] = imax(m->nlevels_nod2D[r - 1], m->nlevels_nod2D[m->nod2D + h - 1]);
      }
      for (int h = 1; h <= m->eDim; ++h) m->nlevels_nod2D[m->nod2D + h - 1] = m->nlevels_nod2D[h2r[h - 1] - 1];
      free(h2r);
    }
  }

  /* 1i. mesh computation routines, :653-700 */
  test_tri(m);
  build_nod_in_elem(m, NT);
  find_levels_min_e2n(m);
  m->elem_area = (double*)xcalloc((size_t)M, sizeof(double));
  m->area = (double*)xcalloc((size_t)nl * NT, sizeof(double));
  m->areasvol = (double*)xcalloc((size_t)nl * NT, sizeof(double));
  mesh_areas(m);
  m->edge_dxdy = (double*)xcalloc((size_t)2 * E, sizeof(double));
  m->edge_cross_dxdy = (double*)xcalloc((size_t)4 * E, sizeof(double));
  m->elem_cos = (double*)xcalloc((size_t)M, sizeof(double));
  m->gradient_sca = (double*)xcalloc((size_t)6 * M, sizeof(double));
  mesh_auxiliary_arrays(m);

  /* 1j. periodic post-remap, :705-707 */
  if (periodic) periodic_post_remap(m);
  if (periodic && cluster_full) {
    build_nod_in_elem(m, m->nod2D);
    find_levels_min_e2n(m);
  }

  finish_mesh(m);
  return m;
}

/* g2r with the rotation matrix of set_mesh_transform_matrix,
 * lib/gen_modules_rotate_grid.F90:12-88: geographic (glon, glat) -> rotated. */
static void g2r(const double* r, double glon, double glat, double* rlon, double* rlat) {
  double xg = cos(glat) * cos(glon), yg = cos(glat) * sin(glon), zg = sin(glat);
  double xr = r[0] * xg + r[1] * yg + r[2] * zg;
  double yr = r[3] * xg + r[4] * yg + r[5] * zg;
  double zr = r[6] * xg + r[7] * yg + r[8] * zg;
  *rlat = asin(zr);
  *rlon = (yr == 0.0 && xr == 0.0) ? 0.0 : atan2(yr, xr);
}

omesh* om_mesh_from_arrays(int nod2D, int elem2D, int edge2D, int edge2D_in, int nl, const double* lonlat,
                           const int* elem, const int* edges, const int* edge_tri, const int* elvls,
                           const int* nlvls, const double* zbar_in, int flags) {
  if (nod2D < 3 || elem2D < 1 || edge2D < 3 || nl < 3) return NULL;
  omesh* m = (omesh*)xcalloc(1, sizeof(omesh));
  m->nl = nl;
  m->cartesian = 0; /* lib/gen_modules_config.F90:81 */
  m->cyclic = (flags & OM_FILE_CYCLIC_2PI) ? 2.0 * PI_F : CYCLIC_LENGTH;
  m->nod2D = m->nod2D_total = nod2D;
  m->elem2D = elem2D;
  m->edge2D = edge2D;
  m->edge2D_in = edge2D_in;
  const int N = nod2D, M = elem2D, E = edge2D;

  /* read_mesh, lib/oce_mesh.F90:230-330: degrees -> radians, then the
   * rotation when force_rotation (default .true., lib/gen_modules_config.F90:85).
   * The Euler angles 50, 15, -90 (:86-88) enter cos/sin as they are. */
  double rm[9];
  {
    double al = 50.0, be = 15.0, ga = -90.0;
    if (flags & OM_FILE_EULER_DEGREES) {
      al = al * (PI_F / 180.0);
      be = be * (PI_F / 180.0);
      ga = ga * (PI_F / 180.0);
    }
    rm[0] = cos(ga) * cos(al) - sin(ga) * cos(be) * sin(al);
    rm[1] = cos(ga) * sin(al) + sin(ga) * cos(be) * cos(al);
    rm[2] = sin(ga) * sin(be);
    rm[3] = -sin(ga) * cos(al) - cos(ga) * cos(be) * sin(al);
    rm[4] = -sin(ga) * sin(al) + cos(ga) * cos(be) * cos(al);
    rm[5] = cos(ga) * sin(be);
    rm[6] = sin(be) * sin(al);
    rm[7] = -sin(be) * cos(al);
    rm[8] = cos(be);
  }
  const double rad = PI_F / 180.0; /* lib/oce_modules.F90:20 */
  m->coord = (double*)xcalloc((size_t)2 * N, sizeof(double));
  for (int n = 1; n <= N; ++n) {
    double x = A2(lonlat, 2, 1, n) * rad, y = A2(lonlat, 2, 2, n) * rad;
    if (!(flags & OM_FILE_NO_ROTATION)) {
      double rx = x, ry = y;
      g2r(rm, rx, ry, &x, &y);
    }
    A2(m->coord, 2, 1, n) = x;
    A2(m->coord, 2, 2, n) = y;
  }
  m->elem2D_nodes = (int*)xcalloc((size_t)3 * M, sizeof(int));
  memcpy(m->elem2D_nodes, elem, (size_t)3 * M * sizeof(int));
  /* aux3d.out: zbar negative downwards, Z the mid-depths (lib/oce_mesh.F90:445-455) */
  m->zbar = (double*)xcalloc((size_t)nl, sizeof(double));
  m->Z = (double*)xcalloc((size_t)nl, sizeof(double));
  for (int k = 0; k < nl; ++k) m->zbar[k] = zbar_in[k];
  if (m->zbar[1] > 0.0)
    for (int k = 0; k < nl; ++k) m->zbar[k] = -m->zbar[k];
  for (int k = 0; k < nl - 1; ++k) m->Z[k] = 0.5 * (m->zbar[k] + m->zbar[k + 1]);

  test_tri(m);
  /* load_edges, lib/oce_mesh.F90:1617-1848 (negative edge_tri -> 0) */
  m->edges = (int*)xcalloc((size_t)2 * E, sizeof(int));
  m->edge_tri = (int*)xcalloc((size_t)2 * E, sizeof(int));
  for (size_t i = 0; i < (size_t)2 * E; ++i) {
    m->edges[i] = edges[i];
    m->edge_tri[i] = edge_tri[i] < 0 ? 0 : edge_tri[i];
  }
  build_nod_in_elem(m, N);
  /* find_levels, lib/oce_mesh.F90:807-1001 */
  m->nlevels = (int*)xcalloc((size_t)M, sizeof(int));
  m->ulevels = (int*)xcalloc((size_t)M, sizeof(int));
  m->nlevels_nod2D = (int*)xcalloc((size_t)N, sizeof(int));
  m->ulevels_nod2D = (int*)xcalloc((size_t)N, sizeof(int));
  m->nlevels_nod2D_min = (int*)xcalloc((size_t)N, sizeof(int));
  m->ulevels_nod2D_max = (int*)xcalloc((size_t)N, sizeof(int));
  for (int e = 0; e < M; ++e) {
    m->nlevels[e] = elvls[e];
    m->ulevels[e] = 1;
  }
  for (int n = 0; n < N; ++n) {
    m->nlevels_nod2D[n] = nlvls[n];
    m->ulevels_nod2D[n] = 1;
  }
  find_levels_min_e2n(m);
  m->elem_area = (double*)xcalloc((size_t)M, sizeof(double));
  m->area = (double*)xcalloc((size_t)nl * N, sizeof(double));
  m->areasvol = (double*)xcalloc((size_t)nl * N, sizeof(double));
  mesh_areas(m);
  m->edge_dxdy = (double*)xcalloc((size_t)2 * E, sizeof(double));
  m->edge_cross_dxdy = (double*)xcalloc((size_t)4 * E, sizeof(double));
  m->elem_cos = (double*)xcalloc((size_t)M, sizeof(double));
  m->gradient_sca = (double*)xcalloc((size_t)6 * M, sizeof(double));
  mesh_auxiliary_arrays(m);
  finish_mesh(m);
  return m;
}

void om_mesh_free(omesh* m) {
  if (!m) return;
  void* ptrs[] = {m->coord, m->elem2D_nodes, m->edges, m->edge_tri, m->nod_in_elem2D_num,
                  m->nod_in_elem2D, m->nlevels, m->ulevels, m->nlevels_nod2D, m->ulevels_nod2D,
                  m->nlevels_nod2D_min, m->ulevels_nod2D_max, m->zbar, m->Z, m->elem_area, m->area,
                  m->areasvol, m->edge_dxdy, m->edge_cross_dxdy, m->elem_cos, m->gradient_sca,
                  m->hnode, m->hnode_new, m->helem, m->Z_3d_n, m->zbar_3d_n, m->edge_up_dn_tri,
                  m->nboundary_lay};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  free(m);
}

void om_mesh_sizes(const omesh* m, int* out) {
  out[0] = m->nod2D; out[1] = m->nod2D_total; out[2] = m->elem2D; out[3] = m->edge2D;
  out[4] = m->edge2D_in; out[5] = m->nl; out[6] = m->max_nie;
}

long om_mesh_get_int(const omesh* m, const char* name, int* out) {
  const int* src = NULL;
  size_t n = 0;
  const size_t NT = (size_t)m->nod2D_total, N = (size_t)m->nod2D, M = (size_t)m->elem2D, E = (size_t)m->edge2D;
  if (!strcmp(name, "elem2D_nodes")) { src = m->elem2D_nodes; n = 3 * M; }
  else if (!strcmp(name, "edges")) { src = m->edges; n = 2 * E; }
  else if (!strcmp(name, "edge_tri")) { src = m->edge_tri; n = 2 * E; }
  else if (!strcmp(name, "nod_in_elem2D_num")) { src = m->nod_in_elem2D_num; n = N; }
  else if (!strcmp(name, "nod_in_elem2D")) { src = m->nod_in_elem2D; n = (size_t)m->max_nie * N; }
  else if (!strcmp(name, "nlevels")) { src = m->nlevels; n = M; }
  else if (!strcmp(name, "ulevels")) { src = m->ulevels; n = M; }
  else if (!strcmp(name, "nlevels_nod2D")) { src = m->nlevels_nod2D; n = N; }
  else if (!strcmp(name, "ulevels_nod2D")) { src = m->ulevels_nod2D; n = N; }
  else if (!strcmp(name, "nlevels_nod2D_min")) { src = m->nlevels_nod2D_min; n = N; }
  else if (!strcmp(name, "ulevels_nod2D_max")) { src = m->ulevels_nod2D_max; n = N; }
  else if (!strcmp(name, "edge_up_dn_tri")) { src = m->edge_up_dn_tri; n = 2 * E; }
  else if (!strcmp(name, "nboundary_lay")) { src = m->nboundary_lay; n = N; }
  else return -1;
  (void)NT;
  if (out) memcpy(out, src, n * sizeof(int));
  return (long)n;
}

long om_mesh_get_dbl(const omesh* m, const char* name, double* out) {
  const double* src = NULL;
  size_t n = 0;
  const size_t N = (size_t)m->nod2D, M = (size_t)m->elem2D, E = (size_t)m->edge2D, nl = (size_t)m->nl;
  if (!strcmp(name, "coord")) { src = m->coord; n = 2 * N; }
  else if (!strcmp(name, "zbar")) { src = m->zbar; n = nl; }
  else if (!strcmp(name, "Z")) { src = m->Z; n = nl - 1; }
  else if (!strcmp(name, "elem_area")) { src = m->elem_area; n = M; }
  else if (!strcmp(name, "area")) { src = m->area; n = nl * N; }
  else if (!strcmp(name, "areasvol")) { src = m->areasvol; n = nl * N; }
  else if (!strcmp(name, "edge_dxdy")) { src = m->edge_dxdy; n = 2 * E; }
  else if (!strcmp(name, "edge_cross_dxdy")) { src = m->edge_cross_dxdy; n = 4 * E; }
  else if (!strcmp(name, "elem_cos")) { src = m->elem_cos; n = M; }
  else if (!strcmp(name, "gradient_sca")) { src = m->gradient_sca; n = 6 * M; }
  else if (!strcmp(name, "hnode")) { src = m->hnode; n = (nl - 1) * N; }
  else if (!strcmp(name, "hnode_new")) { src = m->hnode_new; n = (nl - 1) * N; }
  else if (!strcmp(name, "helem")) { src = m->helem; n = (nl - 1) * M; }
  else if (!strcmp(name, "Z_3d_n")) { src = m->Z_3d_n; n = (nl - 1) * N; }
  else if (!strcmp(name, "zbar_3d_n")) { src = m->zbar_3d_n; n = nl * N; }
  else return -1;
  if (out) memcpy(out, src, n * sizeof(double));
  return (long)n;
}

/* ------------------------------------------------------------------------- */
/* Work arrays                                                                */
/* ------------------------------------------------------------------------- */

omwork* om_work_new(const omesh* m) {
  omwork* w = (omwork*)xcalloc(1, sizeof(omwork));
  const size_t nl = (size_t)m->nl, N = (size_t)m->nod2D, E = (size_t)m->edge2D, M = (size_t)m->elem2D;
  w->nl = m->nl; w->N = m->nod2D; w->E = m->edge2D; w->M = m->elem2D;
  w->fct_LO = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->adv_flux_hor = (double*)xcalloc((nl - 1) * E, sizeof(double));
  w->adv_flux_ver = (double*)xcalloc(nl * N, sizeof(double));
  w->fct_ttf_max = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->fct_ttf_min = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->fct_plus = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->fct_minus = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->tvert_max = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->tvert_min = (double*)xcalloc((nl - 1) * N, sizeof(double));
  w->aux = (double*)xcalloc(2 * (nl - 1) * M, sizeof(double));
  w->edge_up_dn_grad = (double*)xcalloc(4 * (nl - 1) * E, sizeof(double));
  w->tr_xy = (double*)xcalloc(2 * (nl - 1) * M, sizeof(double));
  w->adf_h_raw = (double*)xcalloc((nl - 1) * E, sizeof(double));
  w->adf_v_raw = (double*)xcalloc(nl * N, sizeof(double));
  return w;
}

void om_work_free(omwork* w) {
  if (!w) return;
  void* ptrs[] = {w->fct_LO, w->adv_flux_hor, w->adv_flux_ver, w->fct_ttf_max, w->fct_ttf_min,
                  w->fct_plus, w->fct_minus, w->tvert_max, w->tvert_min, w->aux,
                  w->edge_up_dn_grad, w->tr_xy, w->adf_h_raw, w->adf_v_raw};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  free(w);
}

long om_work_get(const omwork* w, const char* name, double* out) {
  const double* src = NULL;
  size_t n = 0;
  const size_t nl = (size_t)w->nl, N = (size_t)w->N, E = (size_t)w->E, M = (size_t)w->M;
  if (!strcmp(name, "fct_LO")) { src = w->fct_LO; n = (nl - 1) * N; }
  else if (!strcmp(name, "adv_flux_hor")) { src = w->adv_flux_hor; n = (nl - 1) * E; }
  else if (!strcmp(name, "adv_flux_ver")) { src = w->adv_flux_ver; n = nl * N; }
  else if (!strcmp(name, "fct_ttf_max")) { src = w->fct_ttf_max; n = (nl - 1) * N; }
  else if (!strcmp(name, "fct_ttf_min")) { src = w->fct_ttf_min; n = (nl - 1) * N; }
  else if (!strcmp(name, "fct_plus")) { src = w->fct_plus; n = (nl - 1) * N; }
  else if (!strcmp(name, "fct_minus")) { src = w->fct_minus; n = (nl - 1) * N; }
  else if (!strcmp(name, "edge_up_dn_grad")) { src = w->edge_up_dn_grad; n = 4 * (nl - 1) * E; }
  else if (!strcmp(name, "tr_xy")) { src = w->tr_xy; n = 2 * (nl - 1) * M; }
  else if (!strcmp(name, "adf_h_raw")) { src = w->adf_h_raw; n = (nl - 1) * E; }
  else if (!strcmp(name, "adf_v_raw")) { src = w->adf_v_raw; n = nl * N; }
  else return -1;
  if (out) memcpy(out, src, n * sizeof(double));
  return (long)n;
}

/* ------------------------------------------------------------------------- */
/* Horizontal fluxes, lib/oce_adv_tra_hor.F90                                 */
/* ------------------------------------------------------------------------- */

typedef struct {
  int n1, n2, el1, el2, nl1, nu1, nl2, nu2, nl12, nu12;
  double dX1, dY1, dX2, dY2, a;
} edgeinfo;

static void edge_info(const omesh* m, int edge, edgeinfo* s) {
  s->n1 = A2(m->edges, 2, 1, edge);
  s->n2 = A2(m->edges, 2, 2, edge);
  s->el1 = A2(m->edge_tri, 2, 1, edge);
  s->el2 = A2(m->edge_tri, 2, 2, edge);
  s->nl1 = m->nlevels[s->el1 - 1] - 1;
  s->nu1 = m->ulevels[s->el1 - 1];
  s->dX1 = A2(m->edge_cross_dxdy, 4, 1, edge);
  s->dY1 = A2(m->edge_cross_dxdy, 4, 2, edge);
  s->a = R_EARTH * m->elem_cos[s->el1 - 1];
  s->nl2 = 0;
  s->nu2 = 0;
  s->dX2 = 0.0;
  s->dY2 = 0.0;
  if (s->el2 > 0) {
    s->dX2 = A2(m->edge_cross_dxdy, 4, 3, edge);
    s->dY2 = A2(m->edge_cross_dxdy, 4, 4, edge);
    s->nl2 = m->nlevels[s->el2 - 1] - 1;
    s->nu2 = m->ulevels[s->el2 - 1];
    s->a = 0.5 * (s->a + R_EARTH * m->elem_cos[s->el2 - 1]);
  }
  s->nl12 = imin(s->nl1, s->nl2);
  s->nu12 = imax(s->nu1, s->nu2);
}

#define VEL(c, nz, el) A3(vel, 2, nzl, c, nz, el)

/* adv_tra_hor_upw1, lib/oce_adv_tra_hor.F90:64-261 */
static void hor_upw1(const omesh* m, const double* vel, const double* ttf, double* flux, int init_zero) {
  const int nzl = m->nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nzl * m->edge2D);
  OMP_FOR
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    edgeinfo s;
    edge_info(m, edge, &s);
#define UPW_FLUX(VF)                                                                               \
  {                                                                                                \
    double vf = (VF);                                                                              \
    A2(flux, nzl, nz, edge) = -(0.5 * (A2(ttf, nzl, nz, s.n1) * (vf + fabs(vf)) +                  \
                                       A2(ttf, nzl, nz, s.n2) * (vf - fabs(vf)))) -                \
                              A2(flux, nzl, nz, edge);                                             \
  }
#define VF1 ((-(VEL(2, nz, s.el1) * s.dX1) + VEL(1, nz, s.el1) * s.dY1) * A2(m->helem, nzl, nz, s.el1))
#define VF2 ((VEL(2, nz, s.el2) * s.dX2 - VEL(1, nz, s.el2) * s.dY2) * A2(m->helem, nzl, nz, s.el2))
    for (int nz = s.nu1; nz <= s.nu12 - 1; ++nz) UPW_FLUX(VF1)
    if (s.nu2 > 0)
      for (int nz = s.nu2; nz <= s.nu12 - 1; ++nz) UPW_FLUX(VF2)
    for (int nz = s.nu12; nz <= s.nl12; ++nz) UPW_FLUX(VF1 + VF2)
    for (int nz = s.nl12 + 1; nz <= s.nl1; ++nz) UPW_FLUX(VF1)
    for (int nz = s.nl12 + 1; nz <= s.nl2; ++nz) UPW_FLUX(VF2)
#undef UPW_FLUX
  }
}

/* adv_tra_hor_muscl (:265-550) when use_clo=1, adv_tra_hor_mfct (:554-846) when 0 */
static void hor_muscl(const omesh* m, const double* vel, const double* ttf, double num_ord, double* flux,
                      const double* grad, int use_clo, int init_zero) {
  const int nzl = m->nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nzl * m->edge2D);
  OMP_FOR
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    edgeinfo s;
    edge_info(m, edge, &s);
    const double ex = A2(m->edge_dxdy, 2, 1, edge), ey = A2(m->edge_dxdy, 2, 2, edge);
#define MUSCL_FLUX(VF)                                                                             \
  {                                                                                                \
    double c1 = 1.0, c2 = 1.0;                                                                     \
    if (use_clo) {                                                                                 \
      c1 = (m->nboundary_lay[s.n1 - 1] - nz >= 0) ? 1.0 : 0.0;                                     \
      c2 = (m->nboundary_lay[s.n2 - 1] - nz >= 0) ? 1.0 : 0.0;                                     \
    }                                                                                              \
    double T1 = A2(ttf, nzl, nz, s.n1), T2 = A2(ttf, nzl, nz, s.n2);                               \
    const double* g = &A3(grad, 4, nzl, 1, nz, edge);                                              \
    double Tm2 = T2 - ((2.0 * (T2 - T1) + ex * s.a * g[1] + ey * R_EARTH * g[3]) / 6.0) * c2;      \
    double Tm1 = T1 + ((2.0 * (T2 - T1) + ex * s.a * g[0] + ey * R_EARTH * g[2]) / 6.0) * c1;      \
    double vf = (VF);                                                                              \
    double cHO = (vf + fabs(vf)) * Tm1 + (vf - fabs(vf)) * Tm2;                                    \
    A2(flux, nzl, nz, edge) = (-((0.5 * (1.0 - num_ord)) * cHO) - ((vf * num_ord) * 0.5) * (Tm1 + Tm2)) - \
                              A2(flux, nzl, nz, edge);                                             \
  }
    for (int nz = s.nu1; nz <= s.nu12 - 1; ++nz) MUSCL_FLUX(VF1)
    if (s.nu2 > 0)
      for (int nz = s.nu2; nz <= s.nu12 - 1; ++nz) MUSCL_FLUX(VF2)
    for (int nz = s.nu12; nz <= s.nl12; ++nz) MUSCL_FLUX(VF1 + VF2)
    for (int nz = s.nl12 + 1; nz <= s.nl1; ++nz) MUSCL_FLUX(VF1)
    for (int nz = s.nl12 + 1; nz <= s.nl2; ++nz) MUSCL_FLUX(VF2)
#undef MUSCL_FLUX
  }
}
#undef VF1
#undef VF2

/* Elemental P1 gradient tr_xy (declared lib/oce_modules.F90:212; its producer is
 * in upstream FESOM2, not in the reference): tr_xy(1)=sum(gradient_sca(1:3)*T),
 * tr_xy(2)=sum(gradient_sca(4:6)*T) over the element's nodes, levels
 * ulevels..nlevels-1 (coefficients lib/oce_mesh.F90:2512-2534). */
static void tracer_gradient_elements(const omesh* m, const double* ttf, double* tr_xy) {
  const int nzl = m->nl - 1;
  OMP_FOR
  for (int elem = 1; elem <= m->elem2D; ++elem) {
    const int* en = &A2(m->elem2D_nodes, 3, 1, elem);
    const double* g = &A2(m->gradient_sca, 6, 1, elem);
    for (int nz = m->ulevels[elem - 1]; nz <= m->nlevels[elem - 1] - 1; ++nz) {
      double t1 = A2(ttf, nzl, nz, en[0]), t2 = A2(ttf, nzl, nz, en[1]), t3 = A2(ttf, nzl, nz, en[2]);
      A3(tr_xy, 2, nzl, 1, nz, elem) = g[0] * t1 + g[1] * t2 + g[2] * t3;
      A3(tr_xy, 2, nzl, 2, nz, elem) = g[3] * t1 + g[4] * t2 + g[5] * t3;
    }
  }
}

/* Area-weighted mean of the element gradients around one node at level nz
 * (lib/oce_muscl_adv.F90:394-409 and its repeats). */
static void node_mean_grad(const omesh* m, const double* tr_xy, int node, int nz, double* gx, double* gy) {
  const int nzl = m->nl - 1;
  double tvol = 0.0, tx = 0.0, ty = 0.0;
  for (int k = 1; k <= m->nod_in_elem2D_num[node - 1]; ++k) {
    int elem = A2(m->nod_in_elem2D, m->max_nie, k, node);
    if (m->nlevels[elem - 1] - 1 < nz || nz < m->ulevels[elem - 1]) continue;
    tvol = tvol + m->elem_area[elem - 1];
    tx = tx + A3(tr_xy, 2, nzl, 1, nz, elem) * m->elem_area[elem - 1];
    ty = ty + A3(tr_xy, 2, nzl, 2, nz, elem) * m->elem_area[elem - 1];
  }
  *gx = tx / tvol;
  *gy = ty / tvol;
}

/* fill_up_dn_grad, lib/oce_muscl_adv.F90:361-530 */
static void fill_up_dn_grad(const omesh* m, const double* tr_xy, double* grad) {
  const int nzl = m->nl - 1;
  OMP_FOR
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    int n1 = A2(m->edges, 2, 1, edge), n2 = A2(m->edges, 2, 2, edge);
    int up = A2(m->edge_up_dn_tri, 2, 1, edge), dn = A2(m->edge_up_dn_tri, 2, 2, edge);
    double gx, gy;
    if (up != 0 && dn != 0) {
      int nzmin = imax(m->ulevels_nod2D_max[n1 - 1], m->ulevels_nod2D_max[n2 - 1]);
      int nzmax = imin(m->nlevels_nod2D_min[n1 - 1], m->nlevels_nod2D_min[n2 - 1]);
      for (int nz = m->ulevels_nod2D[n1 - 1]; nz <= nzmin - 1; ++nz) {
        node_mean_grad(m, tr_xy, n1, nz, &gx, &gy);
        A3(grad, 4, nzl, 1, nz, edge) = gx;
        A3(grad, 4, nzl, 3, nz, edge) = gy;
      }
      for (int nz = m->ulevels_nod2D[n2 - 1]; nz <= nzmin - 1; ++nz) {
        node_mean_grad(m, tr_xy, n2, nz, &gx, &gy);
        A3(grad, 4, nzl, 2, nz, edge) = gx;
        A3(grad, 4, nzl, 4, nz, edge) = gy;
      }
      for (int nz = nzmin; nz <= nzmax - 1; ++nz) {
        A3(grad, 4, nzl, 1, nz, edge) = A3(tr_xy, 2, nzl, 1, nz, up);
        A3(grad, 4, nzl, 2, nz, edge) = A3(tr_xy, 2, nzl, 1, nz, dn);
        A3(grad, 4, nzl, 3, nz, edge) = A3(tr_xy, 2, nzl, 2, nz, up);
        A3(grad, 4, nzl, 4, nz, edge) = A3(tr_xy, 2, nzl, 2, nz, dn);
      }
      for (int nz = nzmax; nz <= m->nlevels_nod2D[n1 - 1] - 1; ++nz) {
        node_mean_grad(m, tr_xy, n1, nz, &gx, &gy);
        A3(grad, 4, nzl, 1, nz, edge) = gx;
        A3(grad, 4, nzl, 3, nz, edge) = gy;
      }
      for (int nz = nzmax; nz <= m->nlevels_nod2D[n2 - 1] - 1; ++nz) {
        node_mean_grad(m, tr_xy, n2, nz, &gx, &gy);
        A3(grad, 4, nzl, 2, nz, edge) = gx;
        A3(grad, 4, nzl, 4, nz, edge) = gy;
      }
    } else {
      for (int nz = m->ulevels_nod2D[n1 - 1]; nz <= m->nlevels_nod2D[n1 - 1] - 1; ++nz) {
        node_mean_grad(m, tr_xy, n1, nz, &gx, &gy);
        A3(grad, 4, nzl, 1, nz, edge) = gx;
        A3(grad, 4, nzl, 3, nz, edge) = gy;
      }
      for (int nz = m->ulevels_nod2D[n2 - 1]; nz <= m->nlevels_nod2D[n2 - 1] - 1; ++nz) {
        node_mean_grad(m, tr_xy, n2, nz, &gx, &gy);
        A3(grad, 4, nzl, 2, nz, edge) = gx;
        A3(grad, 4, nzl, 4, nz, edge) = gy;
      }
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Vertical fluxes, lib/oce_adv_tra_ver.F90                                   */
/* ------------------------------------------------------------------------- */

#define TT(nz) A2(ttf, nzl, nz, n)
#define WW(nz) A2(W, nl, nz, n)
#define AREA(nz) A2(m->area, nl, nz, n)
#define FV(nz) A2(flux, nl, nz, n)

/* adv_tra_ver_upw1, :248-335 */
static void ver_upw1(const omesh* m, const double* W, const double* ttf, double* flux, int init_zero) {
  const int nl = m->nl, nzl = nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nl * m->nod2D);
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n) {
    int nzmax = m->nlevels_nod2D[n - 1], nzmin = m->ulevels_nod2D[n - 1];
    int nz = nzmin;
    FV(nz) = -((WW(nz) * TT(nz)) * AREA(nz)) - FV(nz);
    nz = nzmax;
    FV(nz) = 0.0 - FV(nz);
    for (nz = nzmin + 1; nz <= nzmax - 1; ++nz)
      FV(nz) = -((0.5 * (TT(nz) * (WW(nz) + fabs(WW(nz))) + TT(nz - 1) * (WW(nz) - fabs(WW(nz))))) * AREA(nz)) -
               FV(nz);
  }
}

/* adv_tra_ver_qr4c, :339-444 */
static void ver_qr4c(const omesh* m, const double* W, const double* ttf, double num_ord, double* flux,
                     int init_zero) {
  const int nl = m->nl, nzl = nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nl * m->nod2D);
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n) {
    int nzmax = m->nlevels_nod2D[n - 1], nzmin = m->ulevels_nod2D[n - 1];
    int nz = nzmin;
    FV(nz) = -((TT(nz) * WW(nz)) * AREA(nz)) - FV(nz);
    nz = nzmin + 1;
    FV(nz) = -(((0.5 * (TT(nz - 1) + TT(nz))) * WW(nz)) * AREA(nz)) - FV(nz);
    nz = nzmax - 1;
    FV(nz) = -(((0.5 * (TT(nz - 1) + TT(nz))) * WW(nz)) * AREA(nz)) - FV(nz);
    nz = nzmax;
    FV(nz) = 0.0 - FV(nz);
    for (nz = nzmin + 2; nz <= nzmax - 2; ++nz) {
      double Zm2 = A2(m->Z_3d_n, nzl, nz - 2, n), Zm1 = A2(m->Z_3d_n, nzl, nz - 1, n);
      double Z0 = A2(m->Z_3d_n, nzl, nz, n), Zp1 = A2(m->Z_3d_n, nzl, nz + 1, n);
      double zb = A2(m->zbar_3d_n, nl, nz, n);
      double qc = (TT(nz - 1) - TT(nz)) / (Zm1 - Z0);
      double qu = (TT(nz) - TT(nz + 1)) / (Z0 - Zp1);
      double qd = (TT(nz - 2) - TT(nz - 1)) / (Zm2 - Zm1);
      double Tm1 = TT(nz) + ((2.0 * qc + qu) * (zb - Z0)) / 3.0;
      double Tm2 = TT(nz - 1) + ((2.0 * qc + qd) * (zb - Zm1)) / 3.0;
      double Tm = (WW(nz) + fabs(WW(nz))) * Tm1 + (WW(nz) - fabs(WW(nz))) * Tm2;
      FV(nz) = (-((0.5 * (1.0 - num_ord)) * Tm) - (num_ord * (0.5 * (Tm1 + Tm2))) * WW(nz)) * AREA(nz) - FV(nz);
    }
  }
}

/* adv_tra_vert_ppm, :448-644 */
static void ver_ppm(const omesh* m, double dt, const double* W, const double* ttf, double* flux, int init_zero) {
  const int nl = m->nl, nzl = nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nl * m->nod2D);
#pragma omp parallel
  {
  double* tv = (double*)xcalloc((size_t)nl + 1, sizeof(double)) - 1;
  double* tvert = (double*)xcalloc((size_t)nl + 1, sizeof(double)) - 1;
#pragma omp for schedule(static)
  for (int n = 1; n <= m->nod2D; ++n) {
    int nzmax = m->nlevels_nod2D[n - 1], nzmin = m->ulevels_nod2D[n - 1];
#define HN(nz) A2(m->hnode_new, nzl, nz, n)
    tv[nzmin] = TT(nzmin);
    tv[nzmin + 1] = 0.5 * (TT(nzmin) + TT(nzmin + 1));
    {
      double s = copysign(1.0, WW(nzmax - 1));
      tv[nzmax - 1] = -(TT(nzmax - 2) * dmin(s, 0.0)) + TT(nzmax - 1) * dmax(s, 0.0);
    }
    tv[nzmax] = TT(nzmax - 1);
    for (int nz = nzmin + 1; nz <= nzmax - 3; ++nz) {
      double dzjm1 = HN(nz - 1), dzj = HN(nz), dzjp1 = HN(nz + 1), dzjp2 = HN(nz + 2);
      double deltaj = (dzj / (dzjm1 + dzj + dzjp1)) *
                      (((2.0 * dzjm1 + dzj) / (dzjp1 + dzj)) * (TT(nz + 1) - TT(nz)) +
                       ((dzj + 2.0 * dzjp1) / (dzjm1 + dzj)) * (TT(nz) - TT(nz - 1)));
      double deltajp1 = (dzjp1 / (dzj + dzjp1 + dzjp2)) *
                        (((2.0 * dzj + dzjp1) / (dzjp2 + dzjp1)) * (TT(nz + 2) - TT(nz + 1)) +
                         ((dzjp1 + 2.0 * dzjp2) / (dzj + dzjp1)) * (TT(nz + 1) - TT(nz)));
      if ((TT(nz + 1) - TT(nz)) * (TT(nz) - TT(nz - 1)) > 0.0)
        deltaj = dmin(dmin(fabs(deltaj), 2.0 * fabs(TT(nz + 1) - TT(nz))), 2.0 * fabs(TT(nz) - TT(nz - 1))) *
                 copysign(1.0, deltaj);
      else
        deltaj = 0.0;
      if ((TT(nz + 2) - TT(nz + 1)) * (TT(nz + 1) - TT(nz)) > 0.0)
        deltajp1 = dmin(dmin(fabs(deltajp1), 2.0 * fabs(TT(nz + 2) - TT(nz + 1))), 2.0 * fabs(TT(nz + 1) - TT(nz))) *
                   copysign(1.0, deltajp1);
      else
        deltajp1 = 0.0;
      double inner1 = (((2.0 * dzjp1) * dzj) / (dzj + dzjp1)) *
                      ((dzjm1 + dzj) / (2.0 * dzj + dzjp1) - (dzjp2 + dzjp1) / (2.0 * dzjp1 + dzj)) *
                      (TT(nz + 1) - TT(nz));
      double inner2 = ((dzj * (dzjm1 + dzj)) / (2.0 * dzj + dzjp1)) * deltajp1;
      double inner3 = ((dzjp1 * (dzjp1 + dzjp2)) / (dzj + 2.0 * dzjp1)) * deltaj;
      tv[nz + 1] = (TT(nz) + (dzj / (dzj + dzjp1)) * (TT(nz + 1) - TT(nz))) +
                   (1.0 / (dzjm1 + dzj + dzjp1 + dzjp2)) * (inner1 - inner2 + inner3);
    }
#undef HN
    for (int k = 1; k <= nzmax; ++k) tvert[k] = 0.0;
    for (int nz = nzmin; nz <= nzmax - 1; ++nz) {
      if ((WW(nz) <= 0.0) && (WW(nz + 1) >= 0.0)) continue;
      double aL = tv[nz], aR = tv[nz + 1], T0 = TT(nz);
      if ((aR - T0) * (T0 - aL) <= 0.0) {
        aL = T0;
        aR = T0;
      }
      if ((aR - aL) * (T0 - 0.5 * (aL + aR)) > ((aR - aL) * (aR - aL)) / 6.0) aL = 3.0 * T0 - 2.0 * aR;
      if ((aR - aL) * (T0 - 0.5 * (aR + aL)) < -(((aR - aL) * (aR - aL)) / 6.0)) aR = 3.0 * T0 - 2.0 * aL;
      double dzj = A2(m->hnode, nzl, nz, n);
      double aj = 6.0 * (T0 - 0.5 * (aL + aR));
      if (WW(nz) > 0.0) {
        double x = dmin((WW(nz) * dt) / dzj, 1.0);
        tvert[nz] = -aL - (0.5 * x) * ((aR - aL) + (1.0 - (2.0 / 3.0) * x) * aj);
        tvert[nz] = (tvert[nz] * AREA(nz)) * WW(nz);
      }
      if (WW(nz + 1) < 0.0) {
        double x = dmin(-((WW(nz + 1) * dt) / dzj), 1.0);
        tvert[nz + 1] = -aR + (0.5 * x) * ((aR - aL) - (1.0 - (2.0 / 3.0) * x) * aj);
        tvert[nz + 1] = (tvert[nz + 1] * AREA(nz + 1)) * WW(nz + 1);
      }
    }
    tvert[nzmin] = -((tv[nzmin] * WW(nzmin)) * AREA(nzmin));
    tvert[nzmax] = 0.0;
    for (int nz = nzmin; nz <= nzmax; ++nz) FV(nz) = tvert[nz] - FV(nz);
  }
  free(tv + 1);
  free(tvert + 1);
  }
}

/* adv_tra_ver_cdiff, :648-712 */
static void ver_cdiff(const omesh* m, const double* W, const double* ttf, double* flux, int init_zero) {
  const int nl = m->nl, nzl = nl - 1;
  if (init_zero) memset(flux, 0, sizeof(double) * (size_t)nl * m->nod2D);
#pragma omp parallel
  {
  double* tvert = (double*)xcalloc((size_t)nl + 1, sizeof(double)) - 1;
#pragma omp for schedule(static)
  for (int n = 1; n <= m->nod2D; ++n) {
    int nzmax = m->nlevels_nod2D[n - 1] - 1, nzmin = m->ulevels_nod2D[n - 1];
    tvert[nzmin] = -((WW(nzmin) * TT(nzmin)) * AREA(nzmin));
    tvert[nzmax + 1] = 0.0;
    for (int nz = nzmin + 1; nz <= nzmax; ++nz) {
      double tv = 0.5 * (TT(nz - 1) + TT(nz));
      tvert[nz] = -((tv * WW(nz)) * AREA(nz));
    }
    for (int nz = nzmin; nz <= nzmax; ++nz) FV(nz) = tvert[nz] - FV(nz);
  }
  free(tvert + 1);
  }
}

#undef TT
#undef WW
#undef AREA
#undef FV

/* ------------------------------------------------------------------------- */
/* FCT, lib/oce_adv_tra_fct.F90:53-483                                        */
/* ------------------------------------------------------------------------- */

static void edge_scatter_range(const omesh* m, int edge, int* n1, int* n2, int* nu12, int* nl12) {
  int el1 = A2(m->edge_tri, 2, 1, edge), el2 = A2(m->edge_tri, 2, 2, edge);
  *n1 = A2(m->edges, 2, 1, edge);
  *n2 = A2(m->edges, 2, 2, edge);
  int nl1 = m->nlevels[el1 - 1] - 1, nu1 = m->ulevels[el1 - 1], nl2 = 0, nu2 = 0;
  if (el2 > 0) {
    nl2 = m->nlevels[el2 - 1] - 1;
    nu2 = m->ulevels[el2 - 1];
  }
  *nl12 = imax(nl1, nl2);
  *nu12 = nu1;
  if (nu2 > 0) *nu12 = imin(nu1, nu2);
}

static void oce_tra_adv_fct(const omesh* m, omwork* wk, double dt, const double* ttf, const double* LO,
                            double* adf_h, double* adf_v) {
  const int nl = m->nl, nzl = nl - 1;
  const double flux_eps = 1e-16, bignumber = 1e3;
  double *fmax = wk->fct_ttf_max, *fmin = wk->fct_ttf_min, *fplus = wk->fct_plus, *fminus = wk->fct_minus;
  double *tmax = wk->tvert_max, *tmin = wk->tvert_min, *AUX = wk->aux;
  /* a1 */
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz) {
      A2(fmax, nzl, nz, n) = dmax(A2(LO, nzl, nz, n), A2(ttf, nzl, nz, n));
      A2(fmin, nzl, nz, n) = dmin(A2(LO, nzl, nz, n), A2(ttf, nzl, nz, n));
    }
  /* a2 */
  OMP_FOR
  for (int elem = 1; elem <= m->elem2D; ++elem) {
    const int* en = &A2(m->elem2D_nodes, 3, 1, elem);
    int nu1 = m->ulevels[elem - 1], nl1 = m->nlevels[elem - 1];
    for (int nz = nu1; nz <= nl1 - 1; ++nz) {
      A3(AUX, 2, nzl, 1, nz, elem) =
          dmax(dmax(A2(fmax, nzl, nz, en[0]), A2(fmax, nzl, nz, en[1])), A2(fmax, nzl, nz, en[2]));
      A3(AUX, 2, nzl, 2, nz, elem) =
          dmin(dmin(A2(fmin, nzl, nz, en[0]), A2(fmin, nzl, nz, en[1])), A2(fmin, nzl, nz, en[2]));
    }
    if (nl1 <= nl - 1)
      for (int nz = nl1; nz <= nl - 1; ++nz) {
        A3(AUX, 2, nzl, 1, nz, elem) = -bignumber;
        A3(AUX, 2, nzl, 2, nz, elem) = bignumber;
      }
  }
  /* a3 */
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n) {
    int nu1 = m->ulevels_nod2D[n - 1], nl1 = m->nlevels_nod2D[n - 1];
    for (int nz = nu1; nz <= nl1 - 1; ++nz) {
      int e0 = A2(m->nod_in_elem2D, m->max_nie, 1, n);
      A2(tmax, nzl, nz, n) = A3(AUX, 2, nzl, 1, nz, e0);
      A2(tmin, nzl, nz, n) = A3(AUX, 2, nzl, 2, nz, e0);
      for (int k = 2; k <= m->nod_in_elem2D_num[n - 1]; ++k) {
        int el = A2(m->nod_in_elem2D, m->max_nie, k, n);
        A2(tmax, nzl, nz, n) = dmax(A2(tmax, nzl, nz, n), A3(AUX, 2, nzl, 1, nz, el));
        A2(tmin, nzl, nz, n) = dmin(A2(tmin, nzl, nz, n), A3(AUX, 2, nzl, 2, nz, el));
      }
    }
  }
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n) {
    int nu1 = m->ulevels_nod2D[n - 1], nl1 = m->nlevels_nod2D[n - 1];
    A2(fmax, nzl, nu1, n) = A2(tmax, nzl, nu1, n) - A2(LO, nzl, nu1, n);
    A2(fmin, nzl, nu1, n) = A2(tmin, nzl, nu1, n) - A2(LO, nzl, nu1, n);
    for (int nz = nu1 + 1; nz <= nl1 - 2; ++nz) {
      A2(fmax, nzl, nz, n) =
          dmax(dmax(A2(tmax, nzl, nz - 1, n), A2(tmax, nzl, nz, n)), A2(tmax, nzl, nz + 1, n)) - A2(LO, nzl, nz, n);
      A2(fmin, nzl, nz, n) =
          dmin(dmin(A2(tmin, nzl, nz - 1, n), A2(tmin, nzl, nz, n)), A2(tmin, nzl, nz + 1, n)) - A2(LO, nzl, nz, n);
    }
    int nz = nl1 - 1;
    A2(fmax, nzl, nz, n) = A2(tmax, nzl, nz, n) - A2(LO, nzl, nz, n);
    A2(fmin, nzl, nz, n) = A2(tmin, nzl, nz, n) - A2(LO, nzl, nz, n);
  }
  /* b1 */
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz) {
      A2(fplus, nzl, nz, n) = 0.0;
      A2(fminus, nzl, nz, n) = 0.0;
    }
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz) {
      double a = A2(adf_v, nl, nz, n), b = A2(adf_v, nl, nz + 1, n);
      A2(fplus, nzl, nz, n) = A2(fplus, nzl, nz, n) + (dmax(0.0, a) + dmax(0.0, -b));
      A2(fminus, nzl, nz, n) = A2(fminus, nzl, nz, n) + (dmin(0.0, a) + dmin(0.0, -b));
    }
#pragma omp parallel
  {
  int own_lo, own_hi;
  owner_range(m->nod2D, &own_lo, &own_hi);
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    const int o1 = OWNS(A2(m->edges, 2, 1, edge)), o2 = OWNS(A2(m->edges, 2, 2, edge));
    if (!o1 && !o2) continue;
    int n1, n2, nu12, nl12;
    edge_scatter_range(m, edge, &n1, &n2, &nu12, &nl12);
    for (int nz = nu12; nz <= nl12; ++nz) {
      double f = A2(adf_h, nzl, nz, edge);
      if (o1) {
        A2(fplus, nzl, nz, n1) = A2(fplus, nzl, nz, n1) + dmax(0.0, f);
        A2(fminus, nzl, nz, n1) = A2(fminus, nzl, nz, n1) + dmin(0.0, f);
      }
      if (o2) {
        A2(fplus, nzl, nz, n2) = A2(fplus, nzl, nz, n2) + dmax(0.0, -f);
        A2(fminus, nzl, nz, n2) = A2(fminus, nzl, nz, n2) + dmin(0.0, -f);
      }
    }
  }
  }
  /* b2 */
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz) {
      double av = A2(m->areasvol, nl, nz, n);
      double flux = (A2(fplus, nzl, nz, n) * dt) / av + flux_eps;
      A2(fplus, nzl, nz, n) = dmin(1.0, A2(fmax, nzl, nz, n) / flux);
      flux = (A2(fminus, nzl, nz, n) * dt) / av - flux_eps;
      A2(fminus, nzl, nz, n) = dmin(1.0, A2(fmin, nzl, nz, n) / flux);
    }
  /* b3 vertical */
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n) {
    int nu1 = m->ulevels_nod2D[n - 1], nl1 = m->nlevels_nod2D[n - 1];
    int nz = nu1;
    double ae = 1.0, flux = A2(adf_v, nl, nz, n);
    if (flux >= 0.0) ae = dmin(ae, A2(fplus, nzl, nz, n));
    else ae = dmin(ae, A2(fminus, nzl, nz, n));
    A2(adf_v, nl, nz, n) = ae * A2(adf_v, nl, nz, n);
    for (nz = nu1 + 1; nz <= nl1 - 1; ++nz) {
      ae = 1.0;
      flux = A2(adf_v, nl, nz, n);
      if (flux >= 0.0) {
        ae = dmin(ae, A2(fminus, nzl, nz - 1, n));
        ae = dmin(ae, A2(fplus, nzl, nz, n));
      } else {
        ae = dmin(ae, A2(fplus, nzl, nz - 1, n));
        ae = dmin(ae, A2(fminus, nzl, nz, n));
      }
      A2(adf_v, nl, nz, n) = ae * A2(adf_v, nl, nz, n);
    }
  }
  /* b3 horizontal */
  OMP_FOR
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    int n1, n2, nu12, nl12;
    edge_scatter_range(m, edge, &n1, &n2, &nu12, &nl12);
    for (int nz = nu12; nz <= nl12; ++nz) {
      double ae = 1.0, flux = A2(adf_h, nzl, nz, edge);
      if (flux >= 0.0) {
        ae = dmin(ae, A2(fplus, nzl, nz, n1));
        ae = dmin(ae, A2(fminus, nzl, nz, n2));
      } else {
        ae = dmin(ae, A2(fminus, nzl, nz, n1));
        ae = dmin(ae, A2(fplus, nzl, nz, n2));
      }
      A2(adf_h, nzl, nz, edge) = ae * A2(adf_h, nzl, nz, edge);
    }
  }
}

/* oce_tra_adv_flux2dtracer, lib/oce_adv_tra_driver.F90:298-450 */
static void flux2dtracer(const omesh* m, double dt, double* dttf_h, double* dttf_v, const double* flux_h,
                         const double* flux_v, int use_lo, const double* ttf, const double* lo) {
  const int nl = m->nl, nzl = nl - 1;
  if (use_lo) {
    OMP_FOR
    for (int n = 1; n <= m->nod2D; ++n)
      for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz)
        A2(dttf_v, nzl, nz, n) = A2(dttf_v, nzl, nz, n) - A2(ttf, nzl, nz, n) * A2(m->hnode, nzl, nz, n) +
                                 A2(lo, nzl, nz, n) * A2(m->hnode_new, nzl, nz, n);
  }
  OMP_FOR
  for (int n = 1; n <= m->nod2D; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz)
      A2(dttf_v, nzl, nz, n) = A2(dttf_v, nzl, nz, n) +
                               ((A2(flux_v, nl, nz, n) - A2(flux_v, nl, nz + 1, n)) * dt) / A2(m->areasvol, nl, nz, n);
#pragma omp parallel
  {
  int own_lo, own_hi;
  owner_range(m->nod2D, &own_lo, &own_hi);
  for (int edge = 1; edge <= m->edge2D; ++edge) {
    const int o1 = OWNS(A2(m->edges, 2, 1, edge)), o2 = OWNS(A2(m->edges, 2, 2, edge));
    if (!o1 && !o2) continue;
    int n1, n2, nu12, nl12;
    edge_scatter_range(m, edge, &n1, &n2, &nu12, &nl12);
    for (int nz = nu12; nz <= nl12; ++nz) {
      if (o1)
        A2(dttf_h, nzl, nz, n1) =
            A2(dttf_h, nzl, nz, n1) + (A2(flux_h, nzl, nz, edge) * dt) / A2(m->areasvol, nl, nz, n1);
      if (o2)
        A2(dttf_h, nzl, nz, n2) =
            A2(dttf_h, nzl, nz, n2) - (A2(flux_h, nzl, nz, edge) * dt) / A2(m->areasvol, nl, nz, n2);
    }
  }
  }
}

/* adv_tra_vert_impl, lib/oce_adv_tra_ver.F90:90-244: implicit upwind
 * vertical advection with W (the w_split part) applied to ttf in place, one
 * tridiagonal (Thomas) solve per column. Columns need at least two layers
 * (with one, the reference reads ttf(nzmin-1)). The zbar_n / Z_n profile the
 * reference computes first is not used by the coefficients and is omitted. */
static void vert_impl(const omesh* m, double dt, const double* W, double* ttf) {
  const int nl = m->nl, nzl = nl - 1;
#pragma omp parallel
  {
  double* a = (double*)xcalloc(nl + 1, sizeof(double));
  double* b = (double*)xcalloc(nl + 1, sizeof(double));
  double* c = (double*)xcalloc(nl + 1, sizeof(double));
  double* tr = (double*)xcalloc(nl + 1, sizeof(double));
  double* cp = (double*)xcalloc(nl + 1, sizeof(double));
  double* tp = (double*)xcalloc(nl + 1, sizeof(double));
#pragma omp for schedule(static)
  for (int n = 1; n <= m->nod2D; ++n) {
    for (int k = 0; k <= nl; ++k) a[k] = b[k] = c[k] = tr[k] = tp[k] = cp[k] = 0.0;
    const int nzmax = m->nlevels_nod2D[n - 1], nzmin = m->ulevels_nod2D[n - 1];
    const double zinv = 1.0 * dt;
    double v_adv;
    int nz = nzmin;
    a[nz] = 0.0;
    v_adv = zinv * A2(m->area, nl, nz, n) / A2(m->areasvol, nl, nz, n);
    b[nz] = A2(m->hnode_new, nzl, nz, n) + A2(W, nl, nz, n) * v_adv;
    v_adv = zinv * A2(m->area, nl, nz + 1, n) / A2(m->areasvol, nl, nz, n);
    b[nz] = b[nz] - dmin(0.0, A2(W, nl, nz + 1, n)) * v_adv;
    c[nz] = -(dmax(0.0, A2(W, nl, nz + 1, n)) * v_adv);
    for (nz = nzmin + 1; nz <= nzmax - 2; ++nz) {
      v_adv = zinv * A2(m->area, nl, nz, n) / A2(m->areasvol, nl, nz, n);
      a[nz] = dmin(0.0, A2(W, nl, nz, n)) * v_adv;
      b[nz] = A2(m->hnode_new, nzl, nz, n) + dmax(0.0, A2(W, nl, nz, n)) * v_adv;
      v_adv = zinv * A2(m->area, nl, nz + 1, n) / A2(m->areasvol, nl, nz, n);
      b[nz] = b[nz] - dmin(0.0, A2(W, nl, nz + 1, n)) * v_adv;
      c[nz] = -(dmax(0.0, A2(W, nl, nz + 1, n)) * v_adv);
    }
    nz = nzmax - 1;
    v_adv = zinv * A2(m->area, nl, nz, n) / A2(m->areasvol, nl, nz, n);
    a[nz] = dmin(0.0, A2(W, nl, nz, n)) * v_adv;
    b[nz] = A2(m->hnode_new, nzl, nz, n) + dmax(0.0, A2(W, nl, nz, n)) * v_adv;
    c[nz] = 0.0;
    nz = nzmin;
    double dz = A2(m->hnode_new, nzl, nz, n);
    tr[nz] = -((b[nz] - dz) * A2(ttf, nzl, nz, n)) - c[nz] * A2(ttf, nzl, nz + 1, n);
    for (nz = nzmin + 1; nz <= nzmax - 2; ++nz) {
      dz = A2(m->hnode_new, nzl, nz, n);
      tr[nz] = -(a[nz] * A2(ttf, nzl, nz - 1, n)) - (b[nz] - dz) * A2(ttf, nzl, nz, n) - c[nz] * A2(ttf, nzl, nz + 1, n);
    }
    nz = nzmax - 1;
    dz = A2(m->hnode_new, nzl, nz, n);
    tr[nz] = -(a[nz] * A2(ttf, nzl, nz - 1, n)) - (b[nz] - dz) * A2(ttf, nzl, nz, n);
    nz = nzmin;
    cp[nz] = c[nz] / b[nz];
    tp[nz] = tr[nz] / b[nz];
    for (nz = nzmin + 1; nz <= nzmax - 1; ++nz) {
      const double mm = b[nz] - cp[nz - 1] * a[nz];
      cp[nz] = c[nz] / mm;
      tp[nz] = (tr[nz] - tp[nz - 1] * a[nz]) / mm;
    }
    tr[nzmax - 1] = tp[nzmax - 1];
    for (nz = nzmax - 2; nz >= nzmin; --nz) tr[nz] = tp[nz] - cp[nz] * tr[nz + 1];
    for (nz = nzmin; nz <= nzmax - 1; ++nz) A2(ttf, nzl, nz, n) = A2(ttf, nzl, nz, n) + tr[nz];
  }
  free(a);
  free(b);
  free(c);
  free(tr);
  free(cp);
  free(tp);
  }
}

/* ------------------------------------------------------------------------- */
/* do_oce_adv_tra, lib/oce_adv_tra_driver.F90:23-294                           */
/* ------------------------------------------------------------------------- */

int om_do_oce_adv_tra(const omesh* m, omwork* wk, double dt, const double* vel, const double* w,
                      const double* wi, const double* we, const double* ttf, const double* ttfAB, int hor,
                      int ver, int lim, double ph, double pv, int use_wsplit, double* dttf_h, double* dttf_v) {
  const int nl = m->nl, nzl = nl - 1;
  if (hor < 0 || hor > 2 || ver < 0 || ver > 3 || lim < 0 || lim > 1) return -1;
  if (use_wsplit && lim == OM_LIM_FCT) {
    for (int n = 1; n <= m->nod2D; ++n)
      if (m->nlevels_nod2D[n - 1] - m->ulevels_nod2D[n - 1] < 2) return -2; /* see vert_impl */
  }
  double *LO = wk->fct_LO, *Fh = wk->adv_flux_hor, *Fv = wk->adv_flux_ver;
  if (lim == OM_LIM_FCT) {
    hor_upw1(m, vel, ttf, Fh, 1);
    memset(LO, 0, sizeof(double) * (size_t)nzl * m->nod2D);
#pragma omp parallel
    {
    int own_lo, own_hi;
    owner_range(m->nod2D, &own_lo, &own_hi);
    for (int edge = 1; edge <= m->edge2D; ++edge) {
      const int o1 = OWNS(A2(m->edges, 2, 1, edge)), o2 = OWNS(A2(m->edges, 2, 2, edge));
      if (!o1 && !o2) continue;
      int n1, n2, nu12, nl12;
      edge_scatter_range(m, edge, &n1, &n2, &nu12, &nl12);
      for (int nz = nu12; nz <= nl12; ++nz) {
        if (o1) A2(LO, nzl, nz, n1) = A2(LO, nzl, nz, n1) + A2(Fh, nzl, nz, edge);
        if (o2) A2(LO, nzl, nz, n2) = A2(LO, nzl, nz, n2) - A2(Fh, nzl, nz, edge);
      }
    }
    }
    ver_upw1(m, we, ttf, Fv, 1);
    OMP_FOR
    for (int n = 1; n <= m->nod2D; ++n)
      for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz)
        A2(LO, nzl, nz, n) =
            (A2(ttf, nzl, nz, n) * A2(m->hnode, nzl, nz, n) +
             ((A2(LO, nzl, nz, n) + (A2(Fv, nl, nz, n) - A2(Fv, nl, nz + 1, n))) * dt) / A2(m->areasvol, nl, nz, n)) /
            A2(m->hnode_new, nzl, nz, n);
    if (use_wsplit) {
      /* implicit part with wi, then the LO vertical flux of the full w for the
       * antidiffusive vertical flux (lib/oce_adv_tra_driver.F90:221-231) */
      vert_impl(m, dt, wi, LO);
      ver_upw1(m, w, ttf, Fv, 1);
    }
  }
  int zero = (lim != OM_LIM_FCT);
  if (hor == OM_HOR_UPW1) {
    hor_upw1(m, vel, ttfAB, Fh, zero);
  } else {
    tracer_gradient_elements(m, ttfAB, wk->tr_xy);
    fill_up_dn_grad(m, wk->tr_xy, wk->edge_up_dn_grad);
    hor_muscl(m, vel, ttfAB, ph, Fh, wk->edge_up_dn_grad, hor == OM_HOR_MUSCL, zero);
  }
  const double* pw = (lim == OM_LIM_FCT) ? w : we;
  switch (ver) {
    case OM_VER_QR4C: ver_qr4c(m, pw, ttfAB, pv, Fv, zero); break;
    case OM_VER_CDIFF: ver_cdiff(m, pw, ttfAB, Fv, zero); break;
    case OM_VER_PPM: ver_ppm(m, dt, pw, ttfAB, Fv, zero); break;
    default: ver_upw1(m, pw, ttfAB, Fv, zero); break;
  }
  memcpy(wk->adf_h_raw, Fh, sizeof(double) * (size_t)nzl * m->edge2D);
  memcpy(wk->adf_v_raw, Fv, sizeof(double) * (size_t)nl * m->nod2D);
  if (lim == OM_LIM_FCT) {
    oce_tra_adv_fct(m, wk, dt, ttf, LO, Fh, Fv);
    flux2dtracer(m, dt, dttf_h, dttf_v, Fh, Fv, 1, ttf, LO);
  } else {
    flux2dtracer(m, dt, dttf_h, dttf_v, Fh, Fv, 0, NULL, NULL);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Driver loops                                                               */
/* ------------------------------------------------------------------------- */

int om_analytic_step(const omesh* m, omwork* wk, int ntr, double dt, const double* vel, const double* w,
                     double* values, double* valuesAB, const int* hor, const int* ver, const int* lim,
                     const double* ph, const double* pv, int copy_ab, double* del_ttf) {
  return om_analytic_step_split(m, wk, ntr, dt, vel, w, w, w, 0, values, valuesAB, hor, ver, lim, ph, pv, copy_ab,
                                0.0, del_ttf);
}

int om_analytic_step_split(const omesh* m, omwork* wk, int ntr, double dt, const double* vel, const double* w,
                           const double* wi, const double* we, int use_wsplit, double* values, double* valuesAB,
                           const int* hor, const int* ver, const int* lim, const double* ph, const double* pv,
                           int copy_ab, double ab_eps, double* del_ttf) {
  const int nzl = m->nl - 1, N = m->nod2D;
  const size_t blk = (size_t)nzl * N;
  double* dh = (double*)xcalloc(blk, sizeof(double));
  double* dv = (double*)xcalloc(blk, sizeof(double));
  double* old = copy_ab == 2 ? (double*)xcalloc(blk, sizeof(double)) : NULL;
  int rc = 0;
  for (int t = 0; t < ntr && rc == 0; ++t) {
    memset(dh, 0, blk * sizeof(double));
    memset(dv, 0, blk * sizeof(double));
    memset(del_ttf, 0, blk * sizeof(double));
    double* val = values + t * blk;
    double* vab = valuesAB + t * blk;
    rc = om_do_oce_adv_tra(m, wk, dt, vel, w, wi, we, val, vab, hor[t], ver[t], lim[t], ph[t], pv[t], use_wsplit, dh,
                           dv);
    if (old) memcpy(old, val, blk * sizeof(double));
    OMP_FOR
    for (int k = 1; k <= N; ++k)
      for (int kz = m->ulevels_nod2D[k - 1]; kz <= m->nlevels_nod2D[k - 1] - 1; ++kz)
        A2(del_ttf, nzl, kz, k) = A2(del_ttf, nzl, kz, k) + A2(dh, nzl, kz, k) + A2(dv, nzl, kz, k);
    OMP_FOR
    for (int k = 1; k <= N; ++k)
      for (int kz = m->ulevels_nod2D[k - 1]; kz <= m->nlevels_nod2D[k - 1] - 1; ++kz)
        A2(val, nzl, kz, k) = A2(val, nzl, kz, k) + A2(del_ttf, nzl, kz, k) / A2(m->hnode_new, nzl, kz, k);
    if (copy_ab == 2) {
      /* second-order Adams-Bashforth time level of the next step's high-order
       * fluxes with offset epsilon (FESOM2's tracer AB2; the reference
       * declares epsilon = 0.1 at lib/oce_modules.F90:75 and allocates
       * valuesold, lib/tracer_c_interface.F90:561) */
      for (size_t i = 0; i < blk; ++i) vab[i] = -(0.5 + ab_eps) * old[i] + (1.5 + ab_eps) * val[i];
    } else if (copy_ab) {
      memcpy(vab, val, blk * sizeof(double));
    }
  }
  free(dh);
  free(dv);
  free(old);
  return rc;
}

int om_cabi_step(const omesh* m, omwork* wk, double dt, const double* vel, const double* w, const double* wi,
                 const double* we, double* values, double* valuesAB, int hor, int ver, int lim, double ph,
                 double pv, double* del_ttf) {
  const int nzl = m->nl - 1, N = m->nod2D;
  const size_t blk = (size_t)nzl * N;
  double* dh = (double*)xcalloc(blk, sizeof(double));
  double* dv = (double*)xcalloc(blk, sizeof(double));
  int rc = om_do_oce_adv_tra(m, wk, dt, vel, w, wi, we, values, valuesAB, hor, ver, lim, ph, pv, 0, dh, dv);
  for (int n = 1; n <= N; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz)
      A2(del_ttf, nzl, nz, n) = A2(del_ttf, nzl, nz, n) + A2(dh, nzl, nz, n) + A2(dv, nzl, nz, n);
  for (int n = 1; n <= N; ++n)
    for (int nz = m->ulevels_nod2D[n - 1]; nz <= m->nlevels_nod2D[n - 1] - 1; ++nz)
      A2(values, nzl, nz, n) = A2(values, nzl, nz, n) + A2(del_ttf, nzl, nz, n) / A2(m->hnode_new, nzl, nz, n);
  free(dh);
  free(dv);
  return rc;
}

void om_init_dwarf_fields(const omesh* m, double Lx, double Ly, double* T, double* S) {
  const int nzl = m->nl - 1;
  const double xc = 0.5 * Lx, yc = 0.5 * Ly;
  for (int n = 1; n <= m->nod2D; ++n) {
    double xn = A2(m->coord, 2, 1, n) * R_EARTH, yn = A2(m->coord, 2, 2, n) * R_EARTH;
    double r = sqrt((xn - xc) * (xn - xc) + (yn - yc) * (yn - yc));
    for (int k = 1; k <= nzl; ++k) {
      double zn = (double)(k - 1) / (double)(nzl - 1);
      if (T)
        A2(T, nzl, k, n) = 15.0 + (5.0 * sin(((2.0 * PI_F) * xn) / Lx)) * cos(((2.0 * PI_F) * yn) / Ly) - 10.0 * zn;
      if (S) A2(S, nzl, k, n) = 34.0 + (2.0 * exp(-(r * r) / ((0.1 * Lx) * (0.1 * Lx)))) * (1.0 - zn);
    }
  }
}

void om_stats(const omesh* m, const double* values, double* out) {
  const size_t cnt = (size_t)(m->nl - 1) * m->nod2D;
  double mn = INFINITY, mx = -INFINITY, sm = 0.0;
  long nan = 0;
  for (size_t i = 0; i < cnt; ++i) {
    double v = values[i];
    if (v != v) { nan++; sm = sm + v; continue; } /* minval/maxval skip NaN; sum(dble()) turns NaN */
    if (v < mn) mn = v;
    if (v > mx) mx = v;
    sm = sm + v;
  }
  out[0] = mn; out[1] = mx; out[2] = sm; out[3] = (double)nan;
}
