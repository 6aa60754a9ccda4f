/*
 * otfem_oracle.c -- CPU oracle (plain C restatement) of OpenTissue's
 * stiffness-warped tetrahedral FEM step.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py as the checker / reported CPU baseline.  The
 * product (libotfem_gpu.so) never links or calls this file.
 *
 * Each function restates one reference function and cites it (paths are
 * relative to the OpenTissue source tree).  The floating-point operations
 * are written in the same order and association as the reference's
 * Vector3 / Matrix3x3 operators (core/math/math_vector3.h,
 * core/math/math_matrix3x3.h), so a build with -ffp-contract=off gives
 * results bit-identical to the reference headers built the same way.  The
 * node K_row maps (std::map<int,Matrix3x3>, fem_node_traits.h:30-36) are
 * stored as one CSR pattern with ascending columns, which is the map's
 * iteration order.
 */
#include "otfem_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc_mesh {
  int N, T;
  int *tets; /* 4*T: t4mesh_t4tetrahedron.h:39 node indices i,j,k,m */
  /* node fields (fem_node_traits.h:37-52) */
  double *coord, *model, *vel, *fext, *mass, *f0, *b, *update, *prev, *residual;
  unsigned char *fixed;
  /* tet fields (fem_tetrahedron_traits.h:18-49) */
  double *young, *poisson, *density, *Ke /*T*144*/, *Re /*T*9*/, *V, *e10, *e20, *e30;
  double *B /*T*12*/, *D /*T*3*/, *plastic /*T*6*/, *yield, *creep, *cmax;
  /* K_row / A_row maps as CSR; built on the first stiffness assembly */
  int k_built;
  int *row_ptr, *cols;
  double *K, *A; /* 9 per block */
};

/* ----------------------------------------------------------------------- */
/* 3x3 helpers with the reference's association (math_matrix3x3.h).       */

/* Matrix3x3 * Vector3: row(r) * v = x*v0 + y*v1 + z*v2 (math_matrix3x3.h:151,
 * math_vector3.h:194). */
static void mv(const double *M, const double *v, double *out) {
  double a = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
  double b = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
  double c = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
  out[0] = a;
  out[1] = b;
  out[2] = c;
}

/* Matrix3x3 * Matrix3x3 (math_matrix3x3.h:254-266): each entry starts at zero
 * and accumulates A(r,i)*B(i,c) for i = 0,1,2. */
static void mm(const double *A, const double *B, double *C) {
  double tmp[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
      for (int i = 0; i < 3; ++i) s += A[r * 3 + i] * B[i * 3 + c];
      tmp[r * 3 + c] = s;
    }
  memcpy(C, tmp, sizeof(tmp));
}

static void transpose(const double *M, double *Mt) {
  double t[9] = {M[0], M[3], M[6], M[1], M[4], M[7], M[2], M[5], M[8]};
  memcpy(Mt, t, sizeof(t));
}

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* ortonormalize (math_matrix3x3.h:536-558): row Gram-Schmidt, row2 = row0 x row1. */
static void ortonormalize(double *A) {
  double r0[3] = {A[0], A[1], A[2]}, r1[3] = {A[3], A[4], A[5]}, r2[3];
  double l0 = sqrt(dot3(r0, r0));
  if (l0 != 0.0) {
    r0[0] /= l0;
    r0[1] /= l0;
    r0[2] /= l0;
  }
  double d = dot3(r0, r1);
  r1[0] -= r0[0] * d;
  r1[1] -= r0[1] * d;
  r1[2] -= r0[2] * d;
  double l1 = sqrt(dot3(r1, r1));
  if (l1 != 0.0) {
    r1[0] /= l1;
    r1[1] /= l1;
    r1[2] /= l1;
  }
  /* cross (math_vector3.h:375-378) */
  r2[0] = r0[1] * r1[2] - r1[1] * r0[2];
  r2[1] = -r0[0] * r1[2] + r1[0] * r0[2];
  r2[2] = r0[0] * r1[1] - r1[0] * r0[1];
  A[0] = r0[0]; A[1] = r0[1]; A[2] = r0[2];
  A[3] = r1[0]; A[4] = r1[1]; A[5] = r1[2];
  A[6] = r2[0]; A[7] = r2[1]; A[8] = r2[2];
}

/* ----------------------------------------------------------------------- */

/* t4mesh_block_generator.h:32-110 */
void orc_generate_blocks(int I, int J, int K, double w, double h, double d, int *tets, double *coord) {
  long n = 0;
  for (int x = 0; x <= I; ++x)
    for (int y = 0; y <= J; ++y)
      for (int z = 0; z <= K; ++z) {
        coord[3 * n + 0] = w * (double)x;
        coord[3 * n + 2] = d * (double)y;
        coord[3 * n + 1] = h * (double)z;
        ++n;
      }
  long t = 0;
  for (int i = 0; i < I; ++i)
    for (int j = 0; j < J; ++j)
      for (int k = 0; k < K; ++k) {
        int p0 = (i * (J + 1) + j) * (K + 1) + k;
        int p1 = p0 + 1;
        int p3 = ((i + 1) * (J + 1) + j) * (K + 1) + k;
        int p2 = p3 + 1;
        int p7 = ((i + 1) * (J + 1) + (j + 1)) * (K + 1) + k;
        int p6 = p7 + 1;
        int p4 = (i * (J + 1) + (j + 1)) * (K + 1) + k;
        int p5 = p4 + 1;
        int q[20];
        if ((i + j + k) % 2 == 1) {
          int a[20] = {p1, p2, p6, p3, p3, p6, p4, p7, p1, p4, p6, p5, p1, p3, p4, p0, p1, p6, p4, p3};
          memcpy(q, a, sizeof(a));
        } else {
          int a[20] = {p2, p0, p5, p1, p2, p7, p0, p3, p2, p5, p7, p6, p0, p7, p5, p4, p2, p0, p7, p5};
          memcpy(q, a, sizeof(a));
        }
        memcpy(tets + 4 * t, q, sizeof(q));
        t += 5;
      }
}

static double *zalloc(long n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

orc_mesh *orc_create(int n_nodes, int n_tets, const int *tets, const double *coord,
                     const double *model_coord, const unsigned char *fixed) {
  orc_mesh *m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
  m->N = n_nodes;
  m->T = n_tets;
  m->tets = (int *)malloc(sizeof(int) * 4 * (size_t)(n_tets > 0 ? n_tets : 1));
  memcpy(m->tets, tets, sizeof(int) * 4 * (size_t)n_tets);
  long N = n_nodes, T = n_tets;
  m->coord = zalloc(3 * N);
  m->model = zalloc(3 * N);
  m->vel = zalloc(3 * N);
  m->fext = zalloc(3 * N);
  m->mass = zalloc(N);
  m->f0 = zalloc(3 * N);
  m->b = zalloc(3 * N);
  m->update = zalloc(3 * N);
  m->prev = zalloc(3 * N);
  m->residual = zalloc(3 * N);
  m->fixed = (unsigned char *)calloc((size_t)(N > 0 ? N : 1), 1);
  if (coord) memcpy(m->coord, coord, sizeof(double) * 3 * N);
  if (model_coord) memcpy(m->model, model_coord, sizeof(double) * 3 * N);
  if (fixed) memcpy(m->fixed, fixed, (size_t)N);
  m->young = zalloc(T);
  m->poisson = zalloc(T);
  m->density = zalloc(T);
  m->Ke = zalloc(144 * T);
  m->Re = zalloc(9 * T);
  m->V = zalloc(T);
  m->e10 = zalloc(3 * T);
  m->e20 = zalloc(3 * T);
  m->e30 = zalloc(3 * T);
  m->B = zalloc(12 * T);
  m->D = zalloc(3 * T);
  m->plastic = zalloc(6 * T);
  m->yield = zalloc(T);
  m->creep = zalloc(T);
  m->cmax = zalloc(T);
  return m;
}

void orc_destroy(orc_mesh *m) {
  if (!m) return;
  void *p[] = {m->tets, m->coord, m->model, m->vel, m->fext, m->mass, m->f0, m->b, m->update,
               m->prev, m->residual, m->fixed, m->young, m->poisson, m->density, m->Ke, m->Re,
               m->V, m->e10, m->e20, m->e30, m->B, m->D, m->plastic, m->yield, m->creep,
               m->cmax, m->row_ptr, m->cols, m->K, m->A};
  for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); ++i) free(p[i]);
  free(m);
}

void orc_set_fixed(orc_mesh *m, const unsigned char *fixed) { memcpy(m->fixed, fixed, (size_t)m->N); }

static double *field_ptr(orc_mesh *m, int field) {
  switch (field) {
    case ORC_COORD: return m->coord;
    case ORC_MODEL_COORD: return m->model;
    case ORC_VELOCITY: return m->vel;
    case ORC_F_EXTERNAL: return m->fext;
    case ORC_MASS: return m->mass;
    case ORC_F0: return m->f0;
    case ORC_B: return m->b;
    default: return NULL;
  }
}

void orc_set_field(orc_mesh *m, int field, const double *src) {
  double *p = field_ptr(m, field);
  if (p && field <= ORC_F_EXTERNAL) memcpy(p, src, sizeof(double) * 3 * (size_t)m->N);
}

void orc_get_field(orc_mesh *m, int field, double *dst) {
  double *p = field_ptr(m, field);
  if (!p) return;
  memcpy(dst, p, sizeof(double) * (size_t)m->N * (field == ORC_MASS ? 1 : 3));
}

/* ----------------------------------------------------------------------- */
/* init                                                                    */

/* compute_Ke (fem_compute_ke.h:29-100) */
static void compute_Ke(const double *p0, const double *p1, const double *p2, const double *p3,
                       double E, double nu, double *Ke /*144*/) {
  double d = p0[0], d4 = p0[1], d8 = p0[2];
  double d1 = p1[0] - d, d5 = p1[1] - d4, d9 = p1[2] - d8;
  double d2 = p2[0] - d, d6 = p2[1] - d4, d10 = p2[2] - d8;
  double d3 = p3[0] - d, d7 = p3[1] - d4, d11 = p3[2] - d8;
  double d12 = (d1 * d6 * d11 + d2 * d7 * d9 + d3 * d5 * d10) - d1 * d7 * d10 - d2 * d5 * d11 - d3 * d6 * d9;
  double d13 = 1.0 / d12;
  double d14 = fabs(d12 / 6.0);
  double B[4][3];
  B[1][0] = (d10 * d7 - d6 * d11) * d13;
  B[2][0] = (d5 * d11 - d9 * d7) * d13;
  B[3][0] = (d9 * d6 - d5 * d10) * d13;
  B[0][0] = -B[1][0] - B[2][0] - B[3][0];
  B[1][1] = (d2 * d11 - d10 * d3) * d13;
  B[2][1] = (d9 * d3 - d1 * d11) * d13;
  B[3][1] = (d1 * d10 - d9 * d2) * d13;
  B[0][1] = -B[1][1] - B[2][1] - B[3][1];
  B[1][2] = (d6 * d3 - d2 * d7) * d13;
  B[2][2] = (d1 * d7 - d5 * d3) * d13;
  B[3][2] = (d5 * d2 - d1 * d6) * d13;
  B[0][2] = -B[1][2] - B[2][2] - B[3][2];
  double d15 = E / (1.0 + nu) / (1.0 - 2.0 * nu);
  double d16 = (1.0 - nu) * d15;
  double d17 = nu * d15;
  double d18 = E / 2.0 / (1.0 + nu);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double d19 = B[i][0], d20 = B[i][1], d21 = B[i][2];
      double d22 = B[j][0], d23 = B[j][1], d24 = B[j][2];
      double *k = Ke + (i * 4 + j) * 9;
      k[0] = d16 * d19 * d22 + d18 * (d20 * d23 + d21 * d24);
      k[1] = d17 * d19 * d23 + d18 * (d20 * d22);
      k[2] = d17 * d19 * d24 + d18 * (d21 * d22);
      k[3] = d17 * d20 * d22 + d18 * (d19 * d23);
      k[4] = d16 * d20 * d23 + d18 * (d19 * d22 + d21 * d24);
      k[5] = d17 * d20 * d24 + d18 * (d21 * d23);
      k[6] = d17 * d21 * d22 + d18 * (d19 * d24);
      k[7] = d17 * d21 * d23 + d18 * (d20 * d24);
      k[8] = d16 * d21 * d24 + d18 * (d20 * d23 + d19 * d22);
      for (int q = 0; q < 9; ++q) k[q] *= d14;
    }
}

/* compute_B (fem_compute_b.h:28-400) */
static void compute_B(const double *e10, const double *e20, const double *e30, double volume, double *B) {
  double div6V = 1.0 / (6.0 * volume);
  B[1 * 3 + 0] = (e20[2] * e30[1] - e20[1] * e30[2]) * div6V;
  B[2 * 3 + 0] = (e10[1] * e30[2] - e10[2] * e30[1]) * div6V;
  B[3 * 3 + 0] = (e10[2] * e20[1] - e10[1] * e20[2]) * div6V;
  B[0 * 3 + 0] = -B[1 * 3 + 0] - B[2 * 3 + 0] - B[3 * 3 + 0];
  B[1 * 3 + 1] = (e20[0] * e30[2] - e20[2] * e30[0]) * div6V;
  B[2 * 3 + 1] = (e10[2] * e30[0] - e10[0] * e30[2]) * div6V;
  B[3 * 3 + 1] = (e10[0] * e20[2] - e10[2] * e20[0]) * div6V;
  B[0 * 3 + 1] = -B[1 * 3 + 1] - B[2 * 3 + 1] - B[3 * 3 + 1];
  B[1 * 3 + 2] = (e20[1] * e30[0] - e20[0] * e30[1]) * div6V;
  B[2 * 3 + 2] = (e10[0] * e30[1] - e10[1] * e30[0]) * div6V;
  B[3 * 3 + 2] = (e10[1] * e20[0] - e10[0] * e20[1]) * div6V;
  B[0 * 3 + 2] = -B[1 * 3 + 2] - B[2 * 3 + 2] - B[3 * 3 + 2];
}

/* clear_stiffness_assembly (fem_clear_stiffness_assembly.h:23-33) */
static void clear_stiffness_assembly(orc_mesh *m) {
  memset(m->f0, 0, sizeof(double) * 3 * (size_t)m->N);
  if (m->k_built) memset(m->K, 0, sizeof(double) * 9 * (size_t)m->row_ptr[m->N]);
}

void orc_init(orc_mesh *m, double young, double poisson, double density, double c_yield,
              double c_creep, double c_max) {
  int T = m->T;
  /* uniform_young / uniform_poisson / uniform_density (fem_uniform_*.h) */
  for (int t = 0; t < T; ++t) {
    m->young[t] = young;
    m->poisson[t] = poisson;
    m->density[t] = density;
  }
  /* initialize_stiffness_elements (fem_initialize_stiffness_elements.h:30-62) */
  for (int t = 0; t < T; ++t) {
    const int *n = m->tets + 4 * t;
    const double *x0 = m->model + 3 * n[0], *x1 = m->model + 3 * n[1];
    const double *x2 = m->model + 3 * n[2], *x3 = m->model + 3 * n[3];
    double *e10 = m->e10 + 3 * t, *e20 = m->e20 + 3 * t, *e30 = m->e30 + 3 * t;
    for (int c = 0; c < 3; ++c) {
      e10[c] = x1[c] - x0[c];
      e20[c] = x2[c] - x0[c];
      e30[c] = x3[c] - x0[c];
    }
    /* compute_volume (fem_compute_volume.h:27-39): e10 * (e20 % e30) / 6 */
    double cr[3] = {e20[1] * e30[2] - e30[1] * e20[2], e30[0] * e20[2] - e20[0] * e30[2],
                    e20[0] * e30[1] - e30[0] * e20[1]};
    m->V[t] = dot3(e10, cr) / 6.0;
    double *R = m->Re + 9 * t;
    memset(R, 0, 9 * sizeof(double));
    R[0] = R[4] = R[8] = 1.0;
    compute_Ke(x0, x1, x2, x3, m->young[t], m->poisson[t], m->Ke + 144 * t);
  }
  clear_stiffness_assembly(m);
  /* compute_mass (fem_compute_mass.h:30-172) */
  for (int i = 0; i < m->N; ++i) m->mass[i] = m->fixed[i] ? DBL_MAX : 0.0;
  for (int t = 0; t < T; ++t) {
    double amount = m->density[t] * m->V[t] * .25;
    for (int a = 0; a < 4; ++a) m->mass[m->tets[4 * t + a]] += amount;
  }
  /* initialize_plastic (fem_initialize_plastic.h:33-57) */
  for (int t = 0; t < T; ++t) {
    m->yield[t] = c_yield;
    m->creep[t] = c_creep;
    m->cmax[t] = c_max;
    for (int i = 0; i < 6; ++i) m->plastic[6 * t + i] = 0.0;
    compute_B(m->e10 + 3 * t, m->e20 + 3 * t, m->e30 + 3 * t, m->V[t], m->B + 12 * t);
    /* compute_isotropic_elasticity_vector (fem_compute_isotropic_elasticity.h:25-51) */
    double p2 = 2.0 * m->poisson[t];
    double scale = m->young[t] / ((1.0 + m->poisson[t]) * (1.0 - p2));
    m->D[3 * t + 0] = (1.0 - m->poisson[t]) * scale;
    m->D[3 * t + 1] = m->poisson[t] * scale;
    m->D[3 * t + 2] = m->young[t] / (2.0 + p2);
  }
}

/* ----------------------------------------------------------------------- */
/* simulate phases                                                         */

/* update_orientation (fem_update_orientation.h:22-215) */
static void update_orientation(orc_mesh *m) {
  for (int t = 0; t < m->T; ++t) {
    double div6V = 1.0 / m->V[t] * 6.0;
    const double *a = m->e10 + 3 * t, *b = m->e20 + 3 * t, *c = m->e30 + 3 * t;
    double e1x = a[0], e1y = a[1], e1z = a[2];
    double e2x = b[0], e2y = b[1], e2z = b[2];
    double e3x = c[0], e3y = c[1], e3z = c[2];
    double n1x = (e2y * e3z - e3y * e2z) * div6V;
    double n1y = (e3x * e2z - e2x * e3z) * div6V;
    double n1z = (e2x * e3y - e3x * e2y) * div6V;
    double n2x = (e1z * e3y - e1y * e3z) * div6V;
    double n2y = (e1x * e3z - e1z * e3x) * div6V;
    double n2z = (e1y * e3x - e1x * e3y) * div6V;
    double n3x = (e1y * e2z - e1z * e2y) * div6V;
    double n3y = (e1z * e2x - e1x * e2z) * div6V;
    double n3z = (e1x * e2y - e1y * e2x) * div6V;
    const int *n = m->tets + 4 * t;
    const double *p0 = m->coord + 3 * n[0], *p1 = m->coord + 3 * n[1];
    const double *p2 = m->coord + 3 * n[2], *p3 = m->coord + 3 * n[3];
    e1x = p1[0] - p0[0]; e1y = p1[1] - p0[1]; e1z = p1[2] - p0[2];
    e2x = p2[0] - p0[0]; e2y = p2[1] - p0[1]; e2z = p2[2] - p0[2];
    e3x = p3[0] - p0[0]; e3y = p3[1] - p0[1]; e3z = p3[2] - p0[2];
    double *R = m->Re + 9 * t;
    R[0] = e1x * n1x + e2x * n2x + e3x * n3x;
    R[1] = e1x * n1y + e2x * n2y + e3x * n3y;
    R[2] = e1x * n1z + e2x * n2z + e3x * n3z;
    R[3] = e1y * n1x + e2y * n2x + e3y * n3x;
    R[4] = e1y * n1y + e2y * n2y + e3y * n3y;
    R[5] = e1y * n1z + e2y * n2z + e3y * n3z;
    R[6] = e1z * n1x + e2z * n2x + e3z * n3x;
    R[7] = e1z * n1y + e2z * n2y + e3z * n3y;
    R[8] = e1z * n1z + e2z * n2z + e3z * n3z;
    ortonormalize(R);
  }
}

/* reset_orientation (fem_reset_orientation.h:22-27) */
static void reset_orientation(orc_mesh *m) {
  for (int t = 0; t < m->T; ++t) {
    double *R = m->Re + 9 * t;
    memset(R, 0, 9 * sizeof(double));
    R[0] = R[4] = R[8] = 1.0;
  }
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* The K_row key sets: every ordered node pair sharing a tet, which is what
 * p_i->K(p_j->idx()) creates on first touch (fem_stiffness_assembly.h:199-201). */
static void build_pattern(orc_mesh *m) {
  int N = m->N;
  int *deg = (int *)calloc((size_t)N + 1, sizeof(int));
  for (int t = 0; t < m->T; ++t)
    for (int a = 0; a < 4; ++a) deg[m->tets[4 * t + a]] += 4;
  int *start = (int *)calloc((size_t)N + 1, sizeof(int));
  for (int i = 0; i < N; ++i) start[i + 1] = start[i] + deg[i];
  int *buf = (int *)malloc(sizeof(int) * (size_t)(start[N] > 0 ? start[N] : 1));
  int *fill = (int *)calloc((size_t)N, sizeof(int));
  for (int t = 0; t < m->T; ++t)
    for (int a = 0; a < 4; ++a) {
      int i = m->tets[4 * t + a];
      for (int b = 0; b < 4; ++b) buf[start[i] + fill[i]++] = m->tets[4 * t + b];
    }
  m->row_ptr = (int *)calloc((size_t)N + 1, sizeof(int));
  int total = 0;
  for (int i = 0; i < N; ++i) {
    int *s = buf + start[i];
    int n = deg[i];
    qsort(s, (size_t)n, sizeof(int), cmp_int);
    int u = 0;
    for (int q = 0; q < n; ++q)
      if (q == 0 || s[q] != s[q - 1]) s[u++] = s[q];
    deg[i] = u;
    total += u;
  }
  m->cols = (int *)malloc(sizeof(int) * (size_t)(total > 0 ? total : 1));
  for (int i = 0; i < N; ++i) {
    m->row_ptr[i + 1] = m->row_ptr[i] + deg[i];
    memcpy(m->cols + m->row_ptr[i], buf + start[i], sizeof(int) * (size_t)deg[i]);
  }
  m->K = zalloc(9L * total);
  m->A = zalloc(9L * total);
  m->k_built = 1;
  free(deg);
  free(start);
  free(buf);
  free(fill);
}

static double *block(orc_mesh *m, double *vals, int i, int j) {
  int lo = m->row_ptr[i], hi = m->row_ptr[i + 1];
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (m->cols[mid] < j) lo = mid + 1;
    else hi = mid;
  }
  return vals + 9L * lo;
}

/* stiffness_assembly (fem_stiffness_assembly.h:171-209) */
static void stiffness_assembly(orc_mesh *m) {
  if (!m->k_built) build_pattern(m);
  for (int t = 0; t < m->T; ++t) {
    const double *Re = m->Re + 9 * t;
    double ReT[9];
    transpose(Re, ReT);
    const int *n = m->tets + 4 * t;
    for (int i = 0; i < 4; ++i) {
      double f[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < 4; ++j) {
        const double *Ke = m->Ke + 144 * t + (i * 4 + j) * 9;
        double kx[3];
        mv(Ke, m->model + 3 * n[j], kx);
        f[0] += kx[0];
        f[1] += kx[1];
        f[2] += kx[2];
        if (j >= i) {
          double tmp[9];
          mm(Re, Ke, tmp);
          mm(tmp, ReT, tmp);
          double *Kij = block(m, m->K, n[i], n[j]);
          for (int q = 0; q < 9; ++q) Kij[q] += tmp[q];
          if (j > i) {
            double tt[9];
            transpose(tmp, tt);
            double *Kji = block(m, m->K, n[j], n[i]);
            for (int q = 0; q < 9; ++q) Kji[q] += tt[q];
          }
        }
      }
      double rf[3];
      mv(Re, f, rf);
      double *f0 = m->f0 + 3 * n[i];
      f0[0] -= rf[0];
      f0[1] -= rf[1];
      f0[2] -= rf[2];
    }
  }
}

/* add_plasticity_force (fem_add_plasticity_force.h:26-204) */
static void add_plasticity_force(orc_mesh *m, double dt) {
  for (int t = 0; t < m->T; ++t) {
    const double *Re = m->Re + 9 * t;
    double ReT[9];
    transpose(Re, ReT);
    const int *n = m->tets + 4 * t;
    const double *B = m->B + 12 * t;
    double *plastic = m->plastic + 6 * t;
    double e_total[6], e_elastic[6];
    for (int i = 0; i < 6; ++i) e_elastic[i] = e_total[i] = 0.0;
    for (int j = 0; j < 4; ++j) {
      double rx[3], tmp[3];
      mv(ReT, m->coord + 3 * n[j], rx);
      const double *x0 = m->model + 3 * n[j];
      tmp[0] = rx[0] - x0[0];
      tmp[1] = rx[1] - x0[1];
      tmp[2] = rx[2] - x0[2];
      double bj = B[3 * j + 0], cj = B[3 * j + 1], dj = B[3 * j + 2];
      e_total[0] += bj * tmp[0];
      e_total[1] += cj * tmp[1];
      e_total[2] += dj * tmp[2];
      e_total[3] += cj * tmp[0] + bj * tmp[1];
      e_total[4] += dj * tmp[0] + bj * tmp[2];
      e_total[5] += dj * tmp[1] + cj * tmp[2];
    }
    for (int i = 0; i < 6; ++i) e_elastic[i] = e_total[i] - plastic[i];
    double norm_elastic = 0.0;
    for (int i = 0; i < 6; ++i) norm_elastic += e_elastic[i] * e_elastic[i];
    norm_elastic = sqrt(norm_elastic);
    if (norm_elastic > m->yield[t]) {
      double inv = 1.0 / dt;
      double amount = dt * ((inv < m->creep[t]) ? inv : m->creep[t]); /* std::min */
      for (int i = 0; i < 6; ++i) plastic[i] += amount * e_elastic[i];
    }
    double norm_plastic = 0.0;
    for (int i = 0; i < 6; ++i) norm_plastic += plastic[i] * plastic[i];
    norm_plastic = sqrt(norm_plastic);
    if (norm_plastic > m->cmax[t]) {
      double scale = m->cmax[t] / norm_plastic;
      for (int i = 0; i < 6; ++i) plastic[i] *= scale;
    }
    for (int j = 0; j < 4; ++j) {
      double bj = B[3 * j + 0], cj = B[3 * j + 1], dj = B[3 * j + 2];
      double E0 = m->D[3 * t + 0], E1 = m->D[3 * t + 1], E2 = m->D[3 * t + 2];
      double bjE0 = bj * E0, bjE1 = bj * E1, bjE2 = bj * E2;
      double cjE0 = cj * E0, cjE1 = cj * E1, cjE2 = cj * E2;
      double djE0 = dj * E0, djE1 = dj * E1, djE2 = dj * E2;
      double f[3];
      f[0] = bjE0 * plastic[0] + bjE1 * plastic[1] + bjE1 * plastic[2] + cjE2 * plastic[3] + djE2 * plastic[4];
      f[1] = cjE1 * plastic[0] + cjE0 * plastic[1] + cjE1 * plastic[2] + bjE2 * plastic[3] + djE2 * plastic[5];
      f[2] = djE1 * plastic[0] + djE1 * plastic[1] + djE0 * plastic[2] + bjE2 * plastic[4] + cjE2 * plastic[5];
      f[0] *= m->V[t];
      f[1] *= m->V[t];
      f[2] *= m->V[t];
      double rf[3];
      mv(Re, f, rf);
      double *fe = m->fext + 3 * n[j];
      fe[0] += rf[0];
      fe[1] += rf[1];
      fe[2] += rf[2];
    }
  }
}

/* dynamics_assembly (fem_dynamics_assembly.h:47-93) */
static void dynamics_assembly(orc_mesh *m, double mass_damping, double dt) {
  for (int i = 0; i < m->N; ++i) {
    double *b = m->b + 3 * i;
    double mi = m->mass[i];
    b[0] = b[1] = b[2] = 0.0;
    for (int q = m->row_ptr[i]; q < m->row_ptr[i + 1]; ++q) {
      int j = m->cols[q];
      const double *K = m->K + 9L * q;
      double *A = m->A + 9L * q;
      double s = dt * dt;
      for (int e = 0; e < 9; ++e) A[e] = K[e] * s;
      double kx[3];
      mv(K, m->coord + 3 * j, kx);
      b[0] -= kx[0];
      b[1] -= kx[1];
      b[2] -= kx[2];
      if (i == j) {
        double c_i = mass_damping * mi;
        double tmp = mi + dt * c_i;
        A[0] += tmp;
        A[4] += tmp;
        A[8] += tmp;
      }
    }
    const double *f0 = m->f0 + 3 * i, *fe = m->fext + 3 * i, *v = m->vel + 3 * i;
    for (int c = 0; c < 3; ++c) b[c] -= f0[c];
    for (int c = 0; c < 3; ++c) b[c] += fe[c];
    for (int c = 0; c < 3; ++c) b[c] *= dt;
    for (int c = 0; c < 3; ++c) b[c] += v[c] * mi;
  }
}

/* r_i = b_i - sum_j A_ij x_j over the row's keys in ascending order. */
static void residual_row(orc_mesh *m, int i, const double *x, double *r) {
  r[0] = m->b[3 * i + 0];
  r[1] = m->b[3 * i + 1];
  r[2] = m->b[3 * i + 2];
  for (int q = m->row_ptr[i]; q < m->row_ptr[i + 1]; ++q) {
    double ax[3];
    mv(m->A + 9L * q, x + 3 * m->cols[q], ax);
    r[0] -= ax[0];
    r[1] -= ax[1];
    r[2] -= ax[2];
  }
}

static void apply_row(orc_mesh *m, int i, const double *x, double *u) {
  u[0] = u[1] = u[2] = 0.0;
  for (int q = m->row_ptr[i]; q < m->row_ptr[i + 1]; ++q) {
    double ax[3];
    mv(m->A + 9L * q, x + 3 * m->cols[q], ax);
    u[0] += ax[0];
    u[1] += ax[1];
    u[2] += ax[2];
  }
}

/* conjugate_gradients (fem_conjugate_gradients.h:25-133) */
static void conjugate_gradients(orc_mesh *m, unsigned min_it, unsigned max_it) {
  const double tiny = 1e-010, tolerence = 0.001;
  int N = m->N;
  for (int i = 0; i < N; ++i) {
    if (m->fixed[i]) continue;
    residual_row(m, i, m->vel, m->residual + 3 * i);
    memcpy(m->prev + 3 * i, m->residual + 3 * i, 3 * sizeof(double));
  }
  for (unsigned it = 0; it < max_it; ++it) {
    double d = 0.0, d2 = 0.0;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      apply_row(m, i, m->prev, m->update + 3 * i);
      d += dot3(m->residual + 3 * i, m->residual + 3 * i);
      d2 += dot3(m->prev + 3 * i, m->update + 3 * i);
    }
    if (fabs(d2) < tiny) d2 = tiny;
    double d3 = d / d2, d1 = 0.0;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      double *v = m->vel + 3 * i, *p = m->prev + 3 * i, *r = m->residual + 3 * i, *u = m->update + 3 * i;
      for (int c = 0; c < 3; ++c) v[c] += p[c] * d3;
      for (int c = 0; c < 3; ++c) r[c] -= u[c] * d3;
      d1 += dot3(r, r);
    }
    if (it >= min_it && d1 < tolerence) break;
    if (fabs(d) < tiny) d = tiny;
    double d4 = d1 / d;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      double *p = m->prev + 3 * i, *r = m->residual + 3 * i;
      for (int c = 0; c < 3; ++c) p[c] = r[c] + p[c] * d4;
    }
  }
}

/* Clamp-free relative-residual CG on the same fixed-row / fixed-column
 * semantics as conjugate_gradients above; stopping rule ||r||^2 <= eps^2 * ref^2
 * as in core/math/big/big_conjugate_gradient.h:92-94 with ref = ||b||. */
static void conjugate_gradients_converged(orc_mesh *m, double rtol, int max_it, int *iters,
                                          double *rel_res) {
  int N = m->N;
  double bb = 0.0, rr = 0.0;
  for (int i = 0; i < N; ++i) {
    if (m->fixed[i]) continue;
    residual_row(m, i, m->vel, m->residual + 3 * i);
    memcpy(m->prev + 3 * i, m->residual + 3 * i, 3 * sizeof(double));
    bb += dot3(m->b + 3 * i, m->b + 3 * i);
    rr += dot3(m->residual + 3 * i, m->residual + 3 * i);
  }
  double thresh = rtol * rtol * bb;
  int it = 0;
  while (it < max_it && rr > thresh) {
    double pq = 0.0;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      apply_row(m, i, m->prev, m->update + 3 * i);
      pq += dot3(m->prev + 3 * i, m->update + 3 * i);
    }
    double alpha = rr / pq, rr_new = 0.0;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      double *v = m->vel + 3 * i, *p = m->prev + 3 * i, *r = m->residual + 3 * i, *u = m->update + 3 * i;
      for (int c = 0; c < 3; ++c) v[c] += p[c] * alpha;
      for (int c = 0; c < 3; ++c) r[c] -= u[c] * alpha;
      rr_new += dot3(r, r);
    }
    double beta = rr_new / rr;
    rr = rr_new;
    for (int i = 0; i < N; ++i) {
      if (m->fixed[i]) continue;
      double *p = m->prev + 3 * i, *r = m->residual + 3 * i;
      for (int c = 0; c < 3; ++c) p[c] = r[c] + p[c] * beta;
    }
    ++it;
  }
  double tr = 0.0;
  for (int i = 0; i < N; ++i) {
    if (m->fixed[i]) continue;
    double r[3];
    residual_row(m, i, m->vel, r);
    tr += dot3(r, r);
  }
  if (iters) *iters = it;
  if (rel_res) *rel_res = bb > 0.0 ? sqrt(tr / bb) : sqrt(tr);
}

/* position_update (fem_position_update.h:25-39) */
static void position_update(orc_mesh *m, double dt) {
  for (int i = 0; i < m->N; ++i) {
    if (m->fixed[i]) continue;
    for (int c = 0; c < 3; ++c) m->coord[3 * i + c] += m->vel[3 * i + c] * dt;
  }
}

static void step_front(orc_mesh *m, double dt, int use_warping, double mass_damping) {
  clear_stiffness_assembly(m);
  if (use_warping) update_orientation(m);
  else reset_orientation(m);
  stiffness_assembly(m);
  add_plasticity_force(m, dt);
  dynamics_assembly(m, mass_damping, dt);
}

/* simulate (fem_simulate.h:49-113) */
void orc_simulate(orc_mesh *m, double dt, int use_warping) {
  step_front(m, dt, use_warping, 2.0);
  conjugate_gradients(m, 20u, 20u);
  position_update(m, dt);
}

void orc_simulate_converged(orc_mesh *m, double dt, int use_warping, double mass_damping,
                            double rtol, int max_iterations, int *iterations, double *rel_residual) {
  step_front(m, dt, use_warping, mass_damping);
  conjugate_gradients_converged(m, rtol, max_iterations, iterations, rel_residual);
  position_update(m, dt);
}

void orc_update_original_coord(orc_mesh *m) {
  memcpy(m->model, m->coord, sizeof(double) * 3 * (size_t)m->N);
}

/* export_K (fem_export_k.h:23-68) */
long orc_export_k_count(orc_mesh *m) {
  long n = 0;
  for (int i = 0; i < m->N; ++i) {
    if (m->fixed[i]) {
      n += 3;
      continue;
    }
    if (!m->k_built) continue;
    for (int q = m->row_ptr[i]; q < m->row_ptr[i + 1]; ++q)
      if (!m->fixed[m->cols[q]]) n += 9;
  }
  return n;
}

void orc_export_k(orc_mesh *m, int *rows, int *cols, double *vals) {
  long n = 0;
  for (int i = 0; i < m->N; ++i)
    for (int r = 0; r < 3; ++r) {
      int row = 3 * i + r;
      if (m->fixed[i]) {
        rows[n] = row;
        cols[n] = row;
        vals[n] = 1.0;
        ++n;
        continue;
      }
      if (!m->k_built) continue;
      for (int q = m->row_ptr[i]; q < m->row_ptr[i + 1]; ++q) {
        int j = m->cols[q];
        if (m->fixed[j]) continue;
        for (int c = 0; c < 3; ++c) {
          rows[n] = row;
          cols[n] = 3 * j + c;
          vals[n] = m->K[9L * q + 3 * r + c];
          ++n;
        }
      }
    }
}

long orc_k_nnz(orc_mesh *m) { return m->k_built ? m->row_ptr[m->N] : 0; }

void orc_k_pattern(orc_mesh *m, int *row_ptr, int *cols) {
  if (!m->k_built) {
    memset(row_ptr, 0, sizeof(int) * ((size_t)m->N + 1));
    return;
  }
  memcpy(row_ptr, m->row_ptr, sizeof(int) * ((size_t)m->N + 1));
  memcpy(cols, m->cols, sizeof(int) * (size_t)m->row_ptr[m->N]);
}

void orc_k_values(orc_mesh *m, double *vals) {
  if (m->k_built) memcpy(vals, m->K, sizeof(double) * 9 * (size_t)m->row_ptr[m->N]);
}

void orc_get_re(orc_mesh *m, double *re) { memcpy(re, m->Re, sizeof(double) * 9 * (size_t)m->T); }
void orc_get_plastic(orc_mesh *m, double *pl) { memcpy(pl, m->plastic, sizeof(double) * 6 * (size_t)m->T); }
void orc_get_volume(orc_mesh *m, double *vol) { memcpy(vol, m->V, sizeof(double) * (size_t)m->T); }
