// otfem_exact.cu -- the reference solver's kernels in FP64 with the
// reference's operation order.  Built with -fmad=false: no multiply-add
// contraction, so every kernel below performs the same IEEE operations as the
// OpenTissue headers and produces bit-identical values.  Sums that the
// reference accumulates over tets (K_row blocks, f0, mass, plastic forces) are
// gathered per output in ascending tet order, the reference's loop order,
// instead of being scattered with atomics.
#include <cfloat>

#include "otfem_internal.h"
#include "otfem_refmath.cuh"

namespace otfem {
namespace {

constexpr int kThreads = 256;
inline int blocks_for(long n) { return int((n + kThreads - 1) / kThreads) > 0 ? int((n + kThreads - 1) / kThreads) : 1; }

// compute_Ke (fem_compute_ke.h:29-100), compute_volume (fem_compute_volume.h:27-39),
// compute_B (fem_compute_b.h:28-400), compute_isotropic_elasticity_vector
// (fem_compute_isotropic_elasticity.h:25-51); one thread per tet.
__global__ void k_init_elements(int T, const int4* __restrict__ tets, const double* __restrict__ x0,
                                double young_u, double poisson_u, double density_u, double c_yield,
                                double c_creep, double c_max, double* Ke, double* Re, double* V,
                                double* E, double* Bv, double* D, double* plastic, double* yng,
                                double* poi, double* den, double* yld, double* crp, double* cmx,
                                const double* __restrict__ young_t, const double* __restrict__ poisson_t,
                                const double* __restrict__ density_t) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  // uniform materials (fem_uniform_young.h etc.), or per tet when given
  const double young = young_t ? young_t[t] : young_u;
  const double poisson = poisson_t ? poisson_t[t] : poisson_u;
  const double density = density_t ? density_t[t] : density_u;
  int4 n = tets[t];
  const double* p0 = x0 + 3 * n.x;
  const double* p1 = x0 + 3 * n.y;
  const double* p2 = x0 + 3 * n.z;
  const double* p3 = x0 + 3 * n.w;
  yng[t] = young;
  poi[t] = poisson;
  den[t] = density;
  double* e = E + 9 * t;
  for (int c = 0; c < 3; ++c) {
    e[c] = p1[c] - p0[c];
    e[3 + c] = p2[c] - p0[c];
    e[6 + c] = p3[c] - p0[c];
  }
  const double* e10 = e;
  const double* e20 = e + 3;
  const double* e30 = e + 6;
  double cr0 = e20[1] * e30[2] - e30[1] * e20[2];
  double cr1 = e30[0] * e20[2] - e20[0] * e30[2];
  double cr2 = e20[0] * e30[1] - e30[0] * e20[1];
  double vol = (e10[0] * cr0 + e10[1] * cr1 + e10[2] * cr2) / 6.0;
  V[t] = vol;
  double* R = Re + 9 * t;
  for (int q = 0; q < 9; ++q) R[q] = 0.0;
  R[0] = R[4] = R[8] = 1.0;

  // element stiffness from the model coordinates
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
  double d15 = young / (1.0 + poisson) / (1.0 - 2.0 * poisson);
  double d16 = (1.0 - poisson) * d15;
  double d17 = poisson * d15;
  double d18 = young / 2.0 / (1.0 + poisson);
  double* ke = Ke + 144L * t;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double d19 = B[i][0], d20 = B[i][1], d21 = B[i][2];
      double d22 = B[j][0], d23 = B[j][1], d24 = B[j][2];
      double* k = ke + (i * 4 + j) * 9;
      double k0 = d16 * d19 * d22 + d18 * (d20 * d23 + d21 * d24);
      double k1 = d17 * d19 * d23 + d18 * (d20 * d22);
      double k2 = d17 * d19 * d24 + d18 * (d21 * d22);
      double k3 = d17 * d20 * d22 + d18 * (d19 * d23);
      double k4 = d16 * d20 * d23 + d18 * (d19 * d22 + d21 * d24);
      double k5 = d17 * d20 * d24 + d18 * (d21 * d23);
      double k6 = d17 * d21 * d22 + d18 * (d19 * d24);
      double k7 = d17 * d21 * d23 + d18 * (d20 * d24);
      double k8 = d16 * d21 * d24 + d18 * (d20 * d23 + d19 * d22);
      k[0] = k0 * d14; k[1] = k1 * d14; k[2] = k2 * d14;
      k[3] = k3 * d14; k[4] = k4 * d14; k[5] = k5 * d14;
      k[6] = k6 * d14; k[7] = k7 * d14; k[8] = k8 * d14;
    }

  // initialize_plastic (fem_initialize_plastic.h:33-57)
  yld[t] = c_yield;
  crp[t] = c_creep;
  cmx[t] = c_max;
  for (int q = 0; q < 6; ++q) plastic[6 * t + q] = 0.0;
  double div6V = 1.0 / (6.0 * vol);
  double* b = Bv + 12 * t;
  b[3 + 0] = (e20[2] * e30[1] - e20[1] * e30[2]) * div6V;
  b[6 + 0] = (e10[1] * e30[2] - e10[2] * e30[1]) * div6V;
  b[9 + 0] = (e10[2] * e20[1] - e10[1] * e20[2]) * div6V;
  b[0] = -b[3] - b[6] - b[9];
  b[3 + 1] = (e20[0] * e30[2] - e20[2] * e30[0]) * div6V;
  b[6 + 1] = (e10[2] * e30[0] - e10[0] * e30[2]) * div6V;
  b[9 + 1] = (e10[0] * e20[2] - e10[2] * e20[0]) * div6V;
  b[1] = -b[4] - b[7] - b[10];
  b[3 + 2] = (e20[1] * e30[0] - e20[0] * e30[1]) * div6V;
  b[6 + 2] = (e10[0] * e30[1] - e10[1] * e30[0]) * div6V;
  b[9 + 2] = (e10[1] * e20[0] - e10[0] * e20[1]) * div6V;
  b[2] = -b[5] - b[8] - b[11];
  double poisson2 = 2.0 * poisson;
  double scale = young / ((1.0 + poisson) * (1.0 - poisson2));
  D[3 * t + 0] = (1.0 - poisson) * scale;
  D[3 * t + 1] = poisson * scale;
  D[3 * t + 2] = young / (2.0 + poisson2);
}

// compute_mass (fem_compute_mass.h:152-171): fixed nodes get DBL_MAX, then
// each tet adds rho*V/4 to its nodes (gathered in ascending tet order).
__global__ void k_mass(int N, const int* __restrict__ inc_ptr, const int* __restrict__ inc_ent,
                       const unsigned char* __restrict__ fixed, const double* __restrict__ den,
                       const double* __restrict__ V, double* mass) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double m = fixed[i] ? DBL_MAX : 0.0;
  for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
    int t = inc_ent[q] >> 2;
    m += den[t] * V[t] * .25;
  }
  mass[i] = m;
}

// update_orientation (fem_update_orientation.h:22-215) / reset_orientation
// (fem_reset_orientation.h:22-27); one thread per tet.
__global__ void k_orientation(int T, int warp, const int4* __restrict__ tets, const double* __restrict__ x,
                              const double* __restrict__ E, const double* __restrict__ V, double* Re) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double R[9];
  if (warp) {
    int4 n = tets[t];
    ref::orientation(E + 9 * t, V[t], x + 3 * n.x, x + 3 * n.y, x + 3 * n.z, x + 3 * n.w, R);
  } else {
    for (int q = 0; q < 9; ++q) R[q] = 0.0;
    R[0] = R[4] = R[8] = 1.0;
  }
  for (int q = 0; q < 9; ++q) Re[9 * t + q] = R[q];
}

// stiffness_assembly (fem_stiffness_assembly.h:179-208), K_row part: block
// (a,b) = sum over tets containing a and b, in ascending tet order, of
// tmp = (Re*Ke_ij)*trans(Re) when local i <= j, else trans(Re*Ke_ji*trans(Re)).
__global__ void k_assemble_K(long nnz, const int* __restrict__ bc_ptr, const int* __restrict__ bc_ent,
                             const double* __restrict__ Re, const double* __restrict__ Ke, double* K) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= nnz) return;
  double acc[9];
  for (int e = 0; e < 9; ++e) acc[e] = 0.0;
  for (int s = bc_ptr[q]; s < bc_ptr[q + 1]; ++s) {
    int ent = bc_ent[s];
    int t = ent >> 4, li = (ent >> 2) & 3, lj = ent & 3;
    const double* R = Re + 9 * t;
    double RT[9], tmp[9];
    ref::transpose(R, RT);
    if (li <= lj) {
      ref::mm(R, Ke + 144L * t + (li * 4 + lj) * 9, tmp);
      ref::mm(tmp, RT, tmp);
      for (int e = 0; e < 9; ++e) acc[e] += tmp[e];
    } else {
      ref::mm(R, Ke + 144L * t + (lj * 4 + li) * 9, tmp);
      ref::mm(tmp, RT, tmp);
      double tt[9];
      ref::transpose(tmp, tt);
      for (int e = 0; e < 9; ++e) acc[e] += tt[e];
    }
  }
  for (int e = 0; e < 9; ++e) K[9 * q + e] = acc[e];
}

// stiffness_assembly, f0 part (fem_stiffness_assembly.h:186-205):
// f0_i -= Re * sum_j Ke_ij x0_j, over tets containing i in ascending order.
__global__ void k_assemble_f0(int N, const int* __restrict__ inc_ptr, const int* __restrict__ inc_ent,
                              const int4* __restrict__ tets, const double* __restrict__ x0,
                              const double* __restrict__ Re, const double* __restrict__ Ke, double* f0) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int q = inc_ptr[a]; q < inc_ptr[a + 1]; ++q) {
    int t = inc_ent[q] >> 2, i = inc_ent[q] & 3;
    int4 n4 = tets[t];
    int nn[4] = {n4.x, n4.y, n4.z, n4.w};
    double f[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < 4; ++j) {
      double kx[3];
      ref::mv(Ke + 144L * t + (i * 4 + j) * 9, x0 + 3 * nn[j], kx);
      f[0] += kx[0];
      f[1] += kx[1];
      f[2] += kx[2];
    }
    double rf[3];
    ref::mv(Re + 9 * t, f, rf);
    acc[0] -= rf[0];
    acc[1] -= rf[1];
    acc[2] -= rf[2];
  }
  f0[3 * a + 0] = acc[0];
  f0[3 * a + 1] = acc[1];
  f0[3 * a + 2] = acc[2];
}

// add_plasticity_force (fem_add_plasticity_force.h:75-200), per-tet part:
// strain, yield/creep/clamp update of m_plastic, and the four node forces
// Re*f_j stored for the ascending-order gather below.
__global__ void k_plastic_tet(int T, double dt, const int4* __restrict__ tets, const double* __restrict__ x,
                              const double* __restrict__ x0, const double* __restrict__ Re,
                              const double* __restrict__ Bv, const double* __restrict__ D,
                              const double* __restrict__ V, const double* __restrict__ yld,
                              const double* __restrict__ crp, const double* __restrict__ cmx,
                              double* plastic, double* tet_force) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int4 n4 = tets[t];
  int nn[4] = {n4.x, n4.y, n4.z, n4.w};
  const double* R = Re + 9 * t;
  double RT[9];
  ref::transpose(R, RT);
  const double* B = Bv + 12 * t;
  double pl[6];
  for (int i = 0; i < 6; ++i) pl[i] = plastic[6 * t + i];
  double et[6], ee[6];
  for (int i = 0; i < 6; ++i) ee[i] = et[i] = 0.0;
  for (int j = 0; j < 4; ++j) {
    double rx[3], tmp[3];
    ref::mv(RT, x + 3 * nn[j], rx);
    const double* xm = x0 + 3 * nn[j];
    tmp[0] = rx[0] - xm[0];
    tmp[1] = rx[1] - xm[1];
    tmp[2] = rx[2] - xm[2];
    double bj = B[3 * j + 0], cj = B[3 * j + 1], dj = B[3 * j + 2];
    et[0] += bj * tmp[0];
    et[1] += cj * tmp[1];
    et[2] += dj * tmp[2];
    et[3] += cj * tmp[0] + bj * tmp[1];
    et[4] += dj * tmp[0] + bj * tmp[2];
    et[5] += dj * tmp[1] + cj * tmp[2];
  }
  for (int i = 0; i < 6; ++i) ee[i] = et[i] - pl[i];
  double ne = 0.0;
  for (int i = 0; i < 6; ++i) ne += ee[i] * ee[i];
  ne = sqrt(ne);
  if (ne > yld[t]) {
    double inv = 1.0 / dt;
    double amount = dt * ((inv < crp[t]) ? inv : crp[t]);
    for (int i = 0; i < 6; ++i) pl[i] += amount * ee[i];
  }
  double np = 0.0;
  for (int i = 0; i < 6; ++i) np += pl[i] * pl[i];
  np = sqrt(np);
  if (np > cmx[t]) {
    double scale = cmx[t] / np;
    for (int i = 0; i < 6; ++i) pl[i] *= scale;
  }
  for (int i = 0; i < 6; ++i) plastic[6 * t + i] = pl[i];
  double E0 = D[3 * t + 0], E1 = D[3 * t + 1], E2 = D[3 * t + 2];
  for (int j = 0; j < 4; ++j) {
    double bj = B[3 * j + 0], cj = B[3 * j + 1], dj = B[3 * j + 2];
    double bjE0 = bj * E0, bjE1 = bj * E1, bjE2 = bj * E2;
    double cjE0 = cj * E0, cjE1 = cj * E1, cjE2 = cj * E2;
    double djE0 = dj * E0, djE1 = dj * E1, djE2 = dj * E2;
    double f[3];
    f[0] = bjE0 * pl[0] + bjE1 * pl[1] + bjE1 * pl[2] + cjE2 * pl[3] + djE2 * pl[4];
    f[1] = cjE1 * pl[0] + cjE0 * pl[1] + cjE1 * pl[2] + bjE2 * pl[3] + djE2 * pl[5];
    f[2] = djE1 * pl[0] + djE1 * pl[1] + djE0 * pl[2] + bjE2 * pl[4] + cjE2 * pl[5];
    f[0] *= V[t];
    f[1] *= V[t];
    f[2] *= V[t];
    double rf[3];
    ref::mv(R, f, rf);
    for (int c = 0; c < 3; ++c) tet_force[12L * t + 3 * j + c] = rf[c];
  }
}

// add_plasticity_force, node part (fem_add_plasticity_force.h:198):
// m_f_external += Re*f in ascending tet order.
__global__ void k_plastic_gather(int N, const int* __restrict__ inc_ptr, const int* __restrict__ inc_ent,
                                 const double* __restrict__ tet_force, double* fext) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  double f[3] = {fext[3 * a], fext[3 * a + 1], fext[3 * a + 2]};
  for (int q = inc_ptr[a]; q < inc_ptr[a + 1]; ++q) {
    int t = inc_ent[q] >> 2, j = inc_ent[q] & 3;
    const double* tf = tet_force + 12L * t + 3 * j;
    f[0] += tf[0];
    f[1] += tf[1];
    f[2] += tf[2];
  }
  fext[3 * a] = f[0];
  fext[3 * a + 1] = f[1];
  fext[3 * a + 2] = f[2];
}

// dynamics_assembly (fem_dynamics_assembly.h:47-93), one thread per node row.
__global__ void k_dynamics(int N, double mass_damping, double dt, const int* __restrict__ row_ptr,
                           const int* __restrict__ cols, const double* __restrict__ K,
                           const double* __restrict__ x, const double* __restrict__ f0,
                           const double* __restrict__ fext, const double* __restrict__ v,
                           const double* __restrict__ mass, double* A, double* b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double mi = mass[i];
  double bb[3] = {0.0, 0.0, 0.0};
  double s = dt * dt;
  for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) {
    int j = cols[q];
    const double* k = K + 9L * q;
    double a[9];
    for (int e = 0; e < 9; ++e) a[e] = k[e] * s;
    double kx[3];
    ref::mv(k, x + 3 * j, kx);
    bb[0] -= kx[0];
    bb[1] -= kx[1];
    bb[2] -= kx[2];
    if (i == j) {
      double c_i = mass_damping * mi;
      double tmp = mi + dt * c_i;
      a[0] += tmp;
      a[4] += tmp;
      a[8] += tmp;
    }
    for (int e = 0; e < 9; ++e) A[9L * q + e] = a[e];
  }
  for (int c = 0; c < 3; ++c) bb[c] -= f0[3 * i + c];
  for (int c = 0; c < 3; ++c) bb[c] += fext[3 * i + c];
  for (int c = 0; c < 3; ++c) bb[c] *= dt;
  for (int c = 0; c < 3; ++c) bb[c] += v[3 * i + c] * mi;
  for (int c = 0; c < 3; ++c) b[3 * i + c] = bb[c];
}

// ---- conjugate_gradients (fem_conjugate_gradients.h:25-133) --------------

struct RefCG {
  double d, d3, d4;
  int done, it;
};

// r = b - sum_j A_ij v_j, p = r for free rows (fem_conjugate_gradients.h:48-67).
__global__ void k_cg_init(int N, const unsigned char* __restrict__ fixed, const int* __restrict__ row_ptr,
                          const int* __restrict__ cols, const double* __restrict__ A,
                          const double* __restrict__ b, const double* __restrict__ v, double* r,
                          double* p, RefCG* s) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    s->done = 0;
    s->it = 0;
  }
  if (i >= N || fixed[i]) return;
  double ri[3] = {b[3 * i], b[3 * i + 1], b[3 * i + 2]};
  for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) {
    double ax[3];
    ref::mv(A + 9L * q, v + 3 * cols[q], ax);
    ri[0] -= ax[0];
    ri[1] -= ax[1];
    ri[2] -= ax[2];
  }
  for (int c = 0; c < 3; ++c) {
    r[3 * i + c] = ri[c];
    p[3 * i + c] = ri[c];
  }
}

// u = A p for free rows, with the per-node terms of d = r.r and d2 = p.u.
__global__ void k_cg_apply(int N, const unsigned char* __restrict__ fixed, const int* __restrict__ row_ptr,
                           const int* __restrict__ cols, const double* __restrict__ A,
                           const double* __restrict__ p, const double* __restrict__ r, double* u,
                           double* dots, const RefCG* __restrict__ s) {
  if (s->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (fixed[i]) {
    dots[i] = 0.0;
    dots[N + i] = 0.0;
    return;
  }
  double ui[3] = {0.0, 0.0, 0.0};
  for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) {
    double ax[3];
    ref::mv(A + 9L * q, p + 3 * cols[q], ax);
    ui[0] += ax[0];
    ui[1] += ax[1];
    ui[2] += ax[2];
  }
  for (int c = 0; c < 3; ++c) u[3 * i + c] = ui[c];
  dots[i] = ref::dot3(r + 3 * i, r + 3 * i);
  dots[N + i] = ref::dot3(p + 3 * i, ui);
}

// Sum of n per-node terms: node order on one thread (sequential == true,
// bit-identical to the reference's running sum) or a fixed-shape tree.
__device__ double block_sum(const double* a, int n, bool sequential) {
  __shared__ double sh[1024];
  double s = 0.0;
  if (sequential) {
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) s += a[i];
    return s;  // valid on thread 0
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += a[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  double out = sh[0];
  __syncthreads();
  return out;
}

// d, d2, clamps, d3 = d/d2 (fem_conjugate_gradients.h:101-104).
__global__ void k_cg_reduce1(int N, const double* __restrict__ dots, int sequential, RefCG* s) {
  if (s->done) return;
  const double tiny = 1e-010;
  double d = block_sum(dots, N, sequential != 0);
  double d2 = block_sum(dots + N, N, sequential != 0);
  if (threadIdx.x == 0) {
    if (fabs(d2) < tiny) d2 = tiny;
    s->d = d;
    s->d3 = d / d2;
  }
}

// v += p*d3, r -= u*d3 and the terms of d1 = r.r (fem_conjugate_gradients.h:110-117).
__global__ void k_cg_update(int N, const unsigned char* __restrict__ fixed, double* v, double* r,
                            const double* __restrict__ p, const double* __restrict__ u, double* dots,
                            const RefCG* __restrict__ s) {
  if (s->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (fixed[i]) {
    dots[i] = 0.0;
    return;
  }
  double d3 = s->d3;
  for (int c = 0; c < 3; ++c) v[3 * i + c] += p[3 * i + c] * d3;
  for (int c = 0; c < 3; ++c) r[3 * i + c] -= u[3 * i + c] * d3;
  dots[i] = ref::dot3(r + 3 * i, r + 3 * i);
}

// d1, the break test and d4 = d1/d (fem_conjugate_gradients.h:118-124).
__global__ void k_cg_reduce2(int N, const double* __restrict__ dots, int sequential, int min_it, RefCG* s) {
  if (s->done) return;
  const double tiny = 1e-010, tolerence = 0.001;
  double d1 = block_sum(dots, N, sequential != 0);
  if (threadIdx.x == 0) {
    int it = s->it;
    s->it = it + 1;
    if (it >= min_it && d1 < tolerence) {
      s->done = 1;
      return;
    }
    double d = s->d;
    if (fabs(d) < tiny) d = tiny;
    s->d4 = d1 / d;
  }
}

// p = r + p*d4 (fem_conjugate_gradients.h:126-131).
__global__ void k_cg_direction(int N, const unsigned char* __restrict__ fixed, const double* __restrict__ r,
                               double* p, const RefCG* __restrict__ s) {
  if (s->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || fixed[i]) return;
  double d4 = s->d4;
  for (int c = 0; c < 3; ++c) p[3 * i + c] = r[3 * i + c] + p[3 * i + c] * d4;
}

__global__ void k_cg_stats(const RefCG* __restrict__ s, DeviceStats* st) {
  st->iterations = s->it;
  st->applies = s->it + 1;
  st->status = 0;
  st->rr = 0.0;
  st->rr0 = 0.0;
  st->bb = 0.0;
}

// position_update (fem_position_update.h:25-39).
__global__ void k_position_update(int N, double dt, const unsigned char* __restrict__ fixed,
                                  const double* __restrict__ v, double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || fixed[i]) return;
  for (int c = 0; c < 3; ++c) x[3 * i + c] += v[3 * i + c] * dt;
}

// export_K (fem_export_k.h:36-56): per-row block counts of the exported CSR.
__global__ void k_export_counts(int N, int assembled, const unsigned char* __restrict__ fixed,
                                const int* __restrict__ row_ptr, const int* __restrict__ cols, int* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (fixed[i]) {
    cnt[i] = 1;
    return;
  }
  int n = 0;
  if (assembled)
    for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) n += fixed[cols[q]] ? 0 : 1;
  cnt[i] = n;
}

__global__ void k_export_fill(int N, int assembled, const unsigned char* __restrict__ fixed,
                              const int* __restrict__ row_ptr, const int* __restrict__ cols,
                              const double* __restrict__ K, const int* __restrict__ out_ptr,
                              int* out_cols, double* out_vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int o = out_ptr[i];
  if (fixed[i]) {
    out_cols[o] = i;
    for (int e = 0; e < 9; ++e) out_vals[9L * o + e] = (e == 0 || e == 4 || e == 8) ? 1.0 : 0.0;
    return;
  }
  if (!assembled) return;
  for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) {
    int j = cols[q];
    if (fixed[j]) continue;
    out_cols[o] = j;
    for (int e = 0; e < 9; ++e) out_vals[9L * o + e] = K[9L * q + e];
    ++o;
  }
}

}  // namespace

// ---- host launch wrappers ---------------------------------------------------

cudaError_t launch_init_elements(Context& c, double young, double poisson, double density,
                                 double c_yield, double c_creep, double c_max, const double* young_t,
                                 const double* poisson_t, const double* density_t) {
  k_init_elements<<<blocks_for(c.T), kThreads, 0, c.stream>>>(
      c.T, c.tets, c.x0, young, poisson, density, c_yield, c_creep, c_max, c.Ke, c.Re, c.V, c.E,
      c.Bv, c.D, c.plastic, c.young, c.poisson, c.density, c.yield, c.creep, c.cmax, young_t, poisson_t,
      density_t);
  k_mass<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.inc_ptr, c.inc_ent, c.fixed, c.density,
                                                     c.V, c.mass);
  return cudaGetLastError();
}

cudaError_t launch_orientation(Context& c, bool warp) {
  k_orientation<<<blocks_for(c.T), kThreads, 0, c.stream>>>(c.T, warp ? 1 : 0, c.tets, c.x, c.E, c.V,
                                                             c.Re);
  return cudaGetLastError();
}

cudaError_t launch_assembly(Context& c) {
  if (c.nnz > 0)
    k_assemble_K<<<blocks_for(c.nnz), kThreads, 0, c.stream>>>(c.nnz, c.bc_ptr, c.bc_ent, c.Re, c.Ke,
                                                                c.K);
  k_assemble_f0<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.inc_ptr, c.inc_ent, c.tets, c.x0,
                                                            c.Re, c.Ke, c.f0);
  return cudaGetLastError();
}

cudaError_t launch_plasticity(Context& c, double dt) {
  k_plastic_tet<<<blocks_for(c.T), kThreads, 0, c.stream>>>(c.T, dt, c.tets, c.x, c.x0, c.Re, c.Bv,
                                                            c.D, c.V, c.yield, c.creep, c.cmax,
                                                            c.plastic, c.tet_force);
  k_plastic_gather<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.inc_ptr, c.inc_ent, c.tet_force,
                                                               c.fext);
  return cudaGetLastError();
}

cudaError_t launch_dynamics_assembly(Context& c, double mass_damping, double dt) {
  k_dynamics<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, mass_damping, dt, c.row_ptr, c.cols, c.K,
                                                         c.x, c.f0, c.fext, c.v, c.mass, c.A, c.b);
  return cudaGetLastError();
}

cudaError_t launch_reference_cg(Context& c, int min_it, int max_it, bool sequential) {
  RefCG* s = reinterpret_cast<RefCG*>(c.scal);
  int nb = blocks_for(c.N);
  int red_threads = sequential ? 32 : 1024;
  k_cg_init<<<nb, kThreads, 0, c.stream>>>(c.N, c.fixed, c.row_ptr, c.cols, c.A, c.b, c.v, c.residual,
                                           c.prev, s);
  for (int it = 0; it < max_it; ++it) {
    k_cg_apply<<<nb, kThreads, 0, c.stream>>>(c.N, c.fixed, c.row_ptr, c.cols, c.A, c.prev, c.residual,
                                              c.update, c.node_dots, s);
    k_cg_reduce1<<<1, red_threads, 0, c.stream>>>(c.N, c.node_dots, sequential ? 1 : 0, s);
    k_cg_update<<<nb, kThreads, 0, c.stream>>>(c.N, c.fixed, c.v, c.residual, c.prev, c.update,
                                               c.node_dots, s);
    k_cg_reduce2<<<1, red_threads, 0, c.stream>>>(c.N, c.node_dots, sequential ? 1 : 0, min_it, s);
    k_cg_direction<<<nb, kThreads, 0, c.stream>>>(c.N, c.fixed, c.residual, c.prev, s);
  }
  k_cg_stats<<<1, 1, 0, c.stream>>>(s, c.stats);
  return cudaGetLastError();
}

cudaError_t launch_position_update(Context& c, double dt) {
  k_position_update<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, dt, c.fixed, c.v, c.x);
  return cudaGetLastError();
}

cudaError_t launch_export_k_counts(Context& c, int* row_cnt) {
  k_export_counts<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.k_assembled ? 1 : 0, c.fixed,
                                                              c.row_ptr, c.cols, row_cnt);
  return cudaGetLastError();
}

cudaError_t launch_export_k(Context& c, int* row_ptr_out, int* cols_out, double* vals_out) {
  k_export_fill<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.k_assembled ? 1 : 0, c.fixed,
                                                            c.row_ptr, c.cols, c.K, row_ptr_out,
                                                            cols_out, vals_out);
  return cudaGetLastError();
}

}  // namespace otfem
