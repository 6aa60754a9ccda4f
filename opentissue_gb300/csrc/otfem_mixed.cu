// otfem_mixed.cu -- matrix-free implicit step (OTFEM_SOLVER_MIXED / _FP64).
//
// Same step as fem::simulate (fem_simulate.h:94-112) without assembling K:
//   A v = b,  A = M(1 + dt*alpha) + dt^2 * sum_e Re Ke Re^T,
//   b = M v + dt (f_ext - sum_e Re Ke (Re^T x - x0))   (fem_dynamics_assembly.h:79-91)
// with Ke = V B^T D B in the B-form of fem_compute_ke.h:133-292.
//
// K1 k_orient_rhs   one thread per tet, FP64: Re by the reference's
//                   Gram-Schmidt (fem_update_orientation.h), the elastic node
//                   forces Re Ke (Re^T x - x0) of the tet, Re rounded to FP32.
// K2 k_cg_persistent one cooperative launch per step: b, the initial residual,
//                   all CG iterations with FP32 (or FP64) element apply,
//                   FP64 vectors and reductions, residual replacement every
//                   refresh_period iterations, and the position update
//                   (fem_position_update.h).  CTAs meet at a bounded grid
//                   barrier; a wait that exceeds its limit sets
//                   OTFEM_ERR_TIMEOUT and the kernel returns.
//
// Element apply for a tet with nodes 0..3 and operand u (world frame):
//   G = sum_{k=1..3} (u_k - u_0) (x) b_k,  H = Re^T G,
//   sigma_aa = c0 H_aa + c1 tr(H),  sigma_ab = c2 (H_ab + H_ba),
//   S = Re sigma,  f_k = dt^2 S b_k (k = 1..3),  f_0 = -(f_1 + f_2 + f_3)
// with b_k the B-vectors of fem_compute_b.h and (c0, c1, c2) = V (D0 - D1, D1, D2)
// from fem_compute_isotropic_elasticity.h.  b_0 = -(b_1 + b_2 + b_3) is
// implied, so a rigid translation gives exactly zero force.
//
// FP32 operands are stored as (hi, lo) float pairs, hi = float(x) and
// lo = float(x - hi), and the element apply forms u_k - u_0 as
// (hi_k - hi_0) + (lo_k - lo_0).  The stiffness sees only these tet-local
// differences, which for a translating or swinging body are orders of
// magnitude smaller than |u|: a single float(x) would keep ~1e-7 of |u| and
// lose most digits of the differences, capping the attainable residual near
// 1e-6.  The hi difference is exact for nearby values (Sterbenz), so the
// differences keep full FP32 relative precision without FP64 arithmetic.
#include <cfloat>

#include "otfem_internal.h"
#include "otfem_refmath.cuh"

namespace otfem {
namespace {

constexpr int kBlock = 512;

struct MixedArgs {
  int N, T;
  const int4* tets;
  const unsigned char* fixed;
  const int* inc_ptr;
  const int* inc_ent;
  const double* tet_force;  // 12 per tet: elastic node forces (K1)
  const double* mass;
  const double* fext;
  double* x;
  double* v;
  double* bvec;
  double* r;
  double* p;
  double* diag;
  // FP32 apply
  const float* re_f;
  const float* b_f;
  const float* c_f;
  float4* p_f;
  float4* v_f;
  float4* q_f;
  float4* p_lo;
  float4* v_lo;
  // FP64 apply
  const double* re_d;
  const double* b_d;
  const double* c_d;
  double4* p_d;
  double4* v_d;
  double4* q_d;
  double dt, alpha, rtol;
  int max_it, refresh;
  double* partials;
  DeviceSync* sync;
  DeviceStats* stats;
  double* trace;  // kTraceRows x kTraceCols (see otfem_internal.h)
  long long spin_limit;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_status(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_add(float4* q, float a, float b, float c) {
  asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(q), "f"(a), "f"(b),
               "f"(c), "f"(0.0f)
               : "memory");
}
__device__ __forceinline__ void red_add(double4* q, double a, double b, double c) {
  atomicAdd(&q->x, a);
  atomicAdd(&q->y, b);
  atomicAdd(&q->z, c);
}

// Grid barrier with a bounded wait.  Every thread first fences its own
// writes and posted reductions at GPU scope (a fence only covers the issuing
// thread's operations); then thread 0 of each CTA arrives on a counter, and
// the last arrival resets it and advances the generation.  Returns false on
// every thread of the CTA if the wait timed out or any CTA has set an error
// status.
__device__ bool grid_barrier(DeviceSync* s, long long spin_limit) {
  __shared__ int ok;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    unsigned gen = ld_acquire(&s->gen);
    __threadfence();
    unsigned arrived = atomicAdd(&s->count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&s->count, 0u);
      __threadfence();
      atomicAdd(&s->gen, 1u);
    } else {
      long long start = clock64();
      while (ld_acquire(&s->gen) == gen) {
        if (clock64() - start > spin_limit) {
          atomicCAS(&s->status, 0, OTFEM_ERR_TIMEOUT);
          good = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (ld_status(&s->status) != 0) good = 0;
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Sums NV per-thread values over the whole grid in a fixed order (warp
// shuffles, CTA tree, then CTA partials in index order), so every CTA obtains
// bit-identical results.  Includes a grid barrier.  Consecutive calls use
// alternating halves of the partials array (`parity`, flipped on every call):
// a CTA may start writing the next sum's partial while slower CTAs are still
// reading this sum's, and the barrier inside the next call separates the
// reads of call k from the writes of call k + 2.
template <int NV>
__device__ bool grid_sum(const MixedArgs& a, double (&val)[NV], int& parity) {
  static_assert(2 * NV <= kMaxPartials, "partials too small");
  __shared__ double s_warp[kBlock / 32][NV];
  __shared__ double s_out[NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = val[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) s_warp[warp][k] = x;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < (int)(blockDim.x >> 5) ? s_warp[lane][k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) a.partials[(parity * (kMaxPartials / 2) + k) * gridDim.x + blockIdx.x] = x;
    }
  }
  if (!grid_barrier(a.sync, a.spin_limit)) return false;
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32)
        x += __ldcg(a.partials + (parity * (kMaxPartials / 2) + k) * gridDim.x + b);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) s_out[k] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) val[k] = s_out[k];
  __syncthreads();
  parity ^= 1;
  return true;
}

// Coherent (L2) load of node data written by other CTAs within the launch
// (accumulators filled by their atomics, operands they rewrote).
__device__ __forceinline__ float4 load_acc(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ double4 load_acc(const double4* p) {
  double2 lo = __ldcg(reinterpret_cast<const double2*>(p));
  double2 hi = __ldcg(reinterpret_cast<const double2*>(p) + 1);
  return make_double4(lo.x, lo.y, hi.x, hi.y);
}

template <typename R>
struct ApplyOps;
template <>
struct ApplyOps<float> {
  typedef float4 V4;
};
template <>
struct ApplyOps<double> {
  typedef double4 V4;
};

// One element apply (see the file comment).  u: operands of the 4 nodes.
template <typename R>
__device__ __forceinline__ void element_apply(const R* Re, const R* b, R c0, R c1, R c2, R scale,
                                              const R (&du)[3][3], R (&f)[4][3]) {
  R G[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) G[a][c] = du[0][a] * b[c] + du[1][a] * b[3 + c] + du[2][a] * b[6 + c];
  R H[3][3];  // Re^T G
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) H[a][c] = Re[a] * G[0][c] + Re[3 + a] * G[1][c] + Re[6 + a] * G[2][c];
  R tr = c1 * (H[0][0] + H[1][1] + H[2][2]);
  R s[3][3];
  s[0][0] = c0 * H[0][0] + tr;
  s[1][1] = c0 * H[1][1] + tr;
  s[2][2] = c0 * H[2][2] + tr;
  s[0][1] = s[1][0] = c2 * (H[0][1] + H[1][0]);
  s[0][2] = s[2][0] = c2 * (H[0][2] + H[2][0]);
  s[1][2] = s[2][1] = c2 * (H[1][2] + H[2][1]);
  R S[3][3];  // scale * Re sigma
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      S[a][c] = scale * (Re[3 * a] * s[0][c] + Re[3 * a + 1] * s[1][c] + Re[3 * a + 2] * s[2][c]);
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int a = 0; a < 3; ++a)
      f[k + 1][a] = S[a][0] * b[3 * k] + S[a][1] * b[3 * k + 1] + S[a][2] * b[3 * k + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) f[0][a] = -(f[1][a] + f[2][a] + f[3][a]);
}

// u_k - u_0 (k = 1..3) of one tet from the gathered operands.
template <typename R>
__device__ __forceinline__ void local_differences(const typename ApplyOps<R>::V4 (&w)[4],
                                                  const typename ApplyOps<R>::V4* ulo, int4 n, R (&du)[3][3]);
template <>
__device__ __forceinline__ void local_differences<float>(const float4 (&w)[4], const float4* ulo, int4 n,
                                                         float (&du)[3][3]) {
  float4 l0 = load_acc(ulo + n.x), l1 = load_acc(ulo + n.y), l2 = load_acc(ulo + n.z), l3 = load_acc(ulo + n.w);
  du[0][0] = (w[1].x - w[0].x) + (l1.x - l0.x);
  du[0][1] = (w[1].y - w[0].y) + (l1.y - l0.y);
  du[0][2] = (w[1].z - w[0].z) + (l1.z - l0.z);
  du[1][0] = (w[2].x - w[0].x) + (l2.x - l0.x);
  du[1][1] = (w[2].y - w[0].y) + (l2.y - l0.y);
  du[1][2] = (w[2].z - w[0].z) + (l2.z - l0.z);
  du[2][0] = (w[3].x - w[0].x) + (l3.x - l0.x);
  du[2][1] = (w[3].y - w[0].y) + (l3.y - l0.y);
  du[2][2] = (w[3].z - w[0].z) + (l3.z - l0.z);
}
template <>
__device__ __forceinline__ void local_differences<double>(const double4 (&w)[4], const double4*, int4,
                                                          double (&du)[3][3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    du[k][0] = w[k + 1].x - w[0].x;
    du[k][1] = w[k + 1].y - w[0].y;
    du[k][2] = w[k + 1].z - w[0].z;
  }
}

// Stores operand x (and its free flag in w) for the apply: FP32 as (hi, lo).
__device__ __forceinline__ void store_operand(float4* hi, float4* lo, long i, double x, double y, double z,
                                              double w) {
  float hx = float(x), hy = float(y), hz = float(z);
  hi[i] = make_float4(hx, hy, hz, float(w));
  lo[i] = make_float4(float(x - double(hx)), float(y - double(hy)), float(z - double(hz)), 0.0f);
}
__device__ __forceinline__ void store_operand(double4* hi, double4*, long i, double x, double y, double z,
                                              double w) {
  hi[i] = make_double4(x, y, z, w);
}

// q += dt^2 K' u over the tets of this thread (grid-stride).  Contributions to
// nodes whose operand w == 0 (fixed rows, never read) are skipped.  The
// operand u4 is rewritten by other CTAs between sweeps of the same launch, so
// it is read with L2 loads (no read-only or L1 path); the per-tet data is
// constant during the launch and may use the read-only path.
template <typename R>
__device__ void apply_tets(const MixedArgs& a, const typename ApplyOps<R>::V4* u4,
                           const typename ApplyOps<R>::V4* ulo, typename ApplyOps<R>::V4* q4,
                           const R* __restrict__ re, const R* __restrict__ bb, const R* __restrict__ cc,
                           R scale) {
  const int T = a.T;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
    int4 n = a.tets[t];
    typename ApplyOps<R>::V4 w[4] = {load_acc(u4 + n.x), load_acc(u4 + n.y), load_acc(u4 + n.z),
                                     load_acc(u4 + n.w)};
    R Re[9], b[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      Re[k] = re[(long)k * T + t];
      b[k] = bb[(long)k * T + t];
    }
    R c0 = cc[t], c1 = cc[T + t], c2 = cc[2L * T + t];
    R du[3][3], f[4][3];
    local_differences<R>(w, ulo, n, du);
    element_apply<R>(Re, b, c0, c1, c2, scale, du, f);
    int nn[4] = {n.x, n.y, n.z, n.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (w[k].w != R(0)) red_add(q4 + nn[k], f[k][0], f[k][1], f[k][2]);
  }
}

template <typename V4, typename R>
__device__ __forceinline__ V4 make_v4(R x, R y, R z, R w);
template <>
__device__ __forceinline__ float4 make_v4<float4, double>(double x, double y, double z, double w) {
  return make_float4(float(x), float(y), float(z), float(w));
}
template <>
__device__ __forceinline__ double4 make_v4<double4, double>(double x, double y, double z, double w) {
  return make_double4(x, y, z, w);
}

// K2: the persistent CG of one step.  R = element-apply precision.
template <typename R>
__global__ void __launch_bounds__(kBlock, 2) k_cg_persistent(MixedArgs a) {
  typedef typename ApplyOps<R>::V4 V4;
  const int N = a.N;
  const long gstride = (long)gridDim.x * blockDim.x;
  const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  V4* pv = sizeof(R) == 4 ? (V4*)a.p_f : (V4*)a.p_d;
  V4* vv = sizeof(R) == 4 ? (V4*)a.v_f : (V4*)a.v_d;
  V4* plo = sizeof(R) == 4 ? (V4*)a.p_lo : nullptr;
  V4* vlo = sizeof(R) == 4 ? (V4*)a.v_lo : nullptr;
  V4* qv = sizeof(R) == 4 ? (V4*)a.q_f : (V4*)a.q_d;
  const R* re = sizeof(R) == 4 ? (const R*)a.re_f : (const R*)a.re_d;
  const R* bb = sizeof(R) == 4 ? (const R*)a.b_f : (const R*)a.b_d;
  const R* cc = sizeof(R) == 4 ? (const R*)a.c_f : (const R*)a.c_d;
  const R scale = R(a.dt * a.dt);
  const V4 zero4 = make_v4<V4, double>(0.0, 0.0, 0.0, 0.0);
  int parity = 0;  // alternates the halves of a.partials between grid sums
  const bool tracer = blockIdx.x == 0 && threadIdx.x == 0;
  const unsigned long long t_start = tracer ? global_ns() : 0ull;
  double stamp[6] = {0, 0, 0, 0, 0, 0};

  // Phase 0: b = M v + dt (f_ext - g) with g gathered in ascending tet order;
  // diagonal M(1 + dt*alpha) as in fem_dynamics_assembly.h:84-85.
  double bbsum[1] = {0.0};
  for (long i = gtid; i < N; i += gstride) {
    double g[3] = {0.0, 0.0, 0.0};
    for (int q = a.inc_ptr[i]; q < a.inc_ptr[i + 1]; ++q) {
      int e = a.inc_ent[q];
      const double* tf = a.tet_force + 12L * (e >> 2) + 3 * (e & 3);
      g[0] += tf[0];
      g[1] += tf[1];
      g[2] += tf[2];
    }
    bool fx = a.fixed[i] != 0;
    double m = a.mass[i];
    double vi[3] = {a.v[3 * i], a.v[3 * i + 1], a.v[3 * i + 2]};
    if (!fx) {
      double b3[3];
      for (int c = 0; c < 3; ++c) b3[c] = m * vi[c] + a.dt * (a.fext[3 * i + c] - g[c]);
      for (int c = 0; c < 3; ++c) a.bvec[3 * i + c] = b3[c];
      bbsum[0] += b3[0] * b3[0] + b3[1] * b3[1] + b3[2] * b3[2];
      a.diag[i] = m + a.dt * (a.alpha * m);
    } else {
      a.diag[i] = 0.0;
    }
    // fixed columns keep their velocity in the initial residual (the reference
    // multiplies A_ij by the fixed node's m_velocity); rows of fixed nodes are
    // never accumulated (w = 0).
    store_operand(vv, vlo, i, vi[0], vi[1], vi[2], fx ? 0.0 : 1.0);
    qv[i] = zero4;
  }
  if (!grid_sum<1>(a, bbsum, parity)) return;
  const double bnorm2 = bbsum[0];
  const double thresh = a.rtol * a.rtol * bnorm2;

  // Initial residual r = b - A v, p = r.
  apply_tets<R>(a, vv, vlo, qv, re, bb, cc, scale);
  if (!grid_barrier(a.sync, a.spin_limit)) return;
  double rr[1] = {0.0};
  for (long i = gtid; i < N; i += gstride) {
    if (a.fixed[i]) {
      store_operand(pv, plo, i, 0.0, 0.0, 0.0, 0.0);
      for (int c = 0; c < 3; ++c) a.p[3 * i + c] = 0.0, a.r[3 * i + c] = 0.0;
      continue;
    }
    V4 q4 = load_acc(qv + i);
    double qa[3] = {double(q4.x), double(q4.y), double(q4.z)};
    double d = a.diag[i];
    double ri[3];
    for (int c = 0; c < 3; ++c) ri[c] = a.bvec[3 * i + c] - (d * a.v[3 * i + c] + qa[c]);
    for (int c = 0; c < 3; ++c) a.r[3 * i + c] = ri[c], a.p[3 * i + c] = ri[c];
    store_operand(pv, plo, i, ri[0], ri[1], ri[2], 1.0);
    qv[i] = zero4;
    rr[0] += ri[0] * ri[0] + ri[1] * ri[1] + ri[2] * ri[2];
  }
  if (!grid_sum<1>(a, rr, parity)) return;
  double rho = rr[0];
  const double rho0 = rho;
  int it = 0, applies = 1;
  bool converged = rho <= thresh;
  bool v_fresh = false;

  while (!converged && it < a.max_it) {
    // q += dt^2 K' p
    apply_tets<R>(a, pv, plo, qv, re, bb, cc, scale);
    ++applies;
    if (tracer) stamp[0] = double(global_ns() - t_start);
    if (!grid_barrier(a.sync, a.spin_limit)) return;
    if (tracer) stamp[1] = double(global_ns() - t_start);
    // q = diag p + q; p.q, r.q, q.q
    double s3[3] = {0.0, 0.0, 0.0};
    for (long i = gtid; i < N; i += gstride) {
      if (a.fixed[i]) continue;
      V4 q4 = load_acc(qv + i);
      double d = a.diag[i];
      double qi[3] = {d * a.p[3 * i] + double(q4.x), d * a.p[3 * i + 1] + double(q4.y),
                      d * a.p[3 * i + 2] + double(q4.z)};
      for (int c = 0; c < 3; ++c) {
        s3[0] += a.p[3 * i + c] * qi[c];
        s3[1] += a.r[3 * i + c] * qi[c];
        s3[2] += qi[c] * qi[c];
      }
    }
    if (tracer) stamp[2] = double(global_ns() - t_start);
    if (!grid_sum<3>(a, s3, parity)) return;
    if (tracer) stamp[3] = double(global_ns() - t_start);
    const double pq = s3[0];
    const double alpha = rho / pq;
    // ||r - alpha q||^2 from the three sums: the new beta is known before the
    // vector update, so v, r and p are updated in one pass.
    double rho_est = rho - 2.0 * alpha * s3[1] + alpha * alpha * s3[2];
    if (rho_est < 0.0) rho_est = 0.0;
    const double beta = rho_est / rho;
    if (!isfinite(pq) || !isfinite(rho) || !isfinite(s3[1]) || !isfinite(s3[2])) {
      // NaN/Inf in the system (e.g. a non-finite force): an error
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&a.sync->status, 0, OTFEM_ERR_NONFINITE);
      break;
    }
    // finite breakdown (p.Ap <= 0 from rounding at the precision floor):
    // stop; the step reports OTFEM_WARN_NOT_CONVERGED with its residual
    if (!(pq > 0.0) || !isfinite(alpha) || !isfinite(beta)) break;
    const int row = it;
    ++it;
    const bool want_refresh = (a.refresh > 0 && it % a.refresh == 0) || rho_est <= 4.0 * thresh;
    double rn[1] = {0.0};
    for (long i = gtid; i < N; i += gstride) {
      if (a.fixed[i]) continue;
      V4 q4 = load_acc(qv + i);
      double d = a.diag[i];
      double pn[3], vn[3];
      for (int c = 0; c < 3; ++c) {
        double pi = a.p[3 * i + c];
        double qi = d * pi + double(c == 0 ? q4.x : (c == 1 ? q4.y : q4.z));
        vn[c] = a.v[3 * i + c] + alpha * pi;
        double ri = a.r[3 * i + c] - alpha * qi;
        a.v[3 * i + c] = vn[c];
        a.r[3 * i + c] = ri;
        rn[0] += ri * ri;
        pn[c] = ri + beta * pi;
        a.p[3 * i + c] = pn[c];
      }
      store_operand(pv, plo, i, pn[0], pn[1], pn[2], 1.0);
      qv[i] = zero4;
      if (want_refresh) store_operand(vv, vlo, i, vn[0], vn[1], vn[2], 1.0);
    }
    v_fresh = want_refresh;
    if (tracer) stamp[4] = double(global_ns() - t_start);
    if (!grid_sum<1>(a, rn, parity)) return;
    if (tracer && row < kTraceRows) {
      double* tr = a.trace + kTraceCols * row;
      tr[0] = rho;
      tr[1] = pq;
      tr[2] = alpha;
      tr[3] = beta;
      for (int k = 0; k < 5; ++k) tr[4 + k] = stamp[k];
      tr[9] = double(global_ns() - t_start);
    }
    rho = rn[0];
    bool refresh = (a.refresh > 0 && it % a.refresh == 0) || rho <= thresh;
    if (refresh) {
      if (!v_fresh) {
        for (long i = gtid; i < N; i += gstride)
          if (!a.fixed[i]) store_operand(vv, vlo, i, a.v[3 * i], a.v[3 * i + 1], a.v[3 * i + 2], 1.0);
        if (!grid_barrier(a.sync, a.spin_limit)) return;
      }
      // r = b - A v (residual replacement); q is zero here.
      apply_tets<R>(a, vv, vlo, qv, re, bb, cc, scale);
      ++applies;
      if (!grid_barrier(a.sync, a.spin_limit)) return;
      double tr[1] = {0.0};
      for (long i = gtid; i < N; i += gstride) {
        if (a.fixed[i]) continue;
        V4 q4 = load_acc(qv + i);
        double d = a.diag[i];
        double qa[3] = {double(q4.x), double(q4.y), double(q4.z)};
        for (int c = 0; c < 3; ++c) {
          double ri = a.bvec[3 * i + c] - (d * a.v[3 * i + c] + qa[c]);
          a.r[3 * i + c] = ri;
          tr[0] += ri * ri;
        }
        qv[i] = zero4;
      }
      if (!grid_sum<1>(a, tr, parity)) return;
      rho = tr[0];
    }
    converged = rho <= thresh;
  }

  // position_update (fem_position_update.h:25-39)
  for (long i = gtid; i < N; i += gstride) {
    if (a.fixed[i]) continue;
    for (int c = 0; c < 3; ++c) a.x[3 * i + c] += a.v[3 * i + c] * a.dt;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int st = ld_status(&a.sync->status);
    if (st == 0 && !converged) st = OTFEM_WARN_NOT_CONVERGED;
    a.stats->iterations = it;
    a.stats->applies = applies;
    a.stats->status = st;
    a.stats->rr = rho;
    a.stats->rr0 = rho0;
    a.stats->bb = bnorm2;
  }
}

// K1: orientation (FP64, reference Gram-Schmidt) and the elastic forces
// g_k = Re Ke (Re^T x - x0) of the tet's nodes, via displacements relative to
// node 0: d_k = Re^T (x_k - x_0) - (x0_k - x0_0).
__global__ void k_orient_rhs(int T, int warp, const int4* __restrict__ tets, const double* __restrict__ x,
                             const double* __restrict__ x0, const double* __restrict__ E,
                             const double* __restrict__ V, const double* __restrict__ Bv,
                             const double* __restrict__ D, double* Re, float* re_f, double* re_d,
                             double* tet_force) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int4 n = tets[t];
  const double* xs[4] = {x + 3 * n.x, x + 3 * n.y, x + 3 * n.z, x + 3 * n.w};
  const double* ms[4] = {x0 + 3 * n.x, x0 + 3 * n.y, x0 + 3 * n.z, x0 + 3 * n.w};
  double R[9];
  if (warp) {
    ref::orientation(E + 9 * t, V[t], xs[0], xs[1], xs[2], xs[3], R);
  } else {
    for (int q = 0; q < 9; ++q) R[q] = 0.0;
    R[0] = R[4] = R[8] = 1.0;
  }
  for (int q = 0; q < 9; ++q) {
    Re[9 * t + q] = R[q];
    re_f[(long)q * T + t] = float(R[q]);
    re_d[(long)q * T + t] = R[q];
  }
  // rest-frame displacements relative to node 0
  double d[3][3];
  for (int k = 0; k < 3; ++k) {
    double e[3] = {xs[k + 1][0] - xs[0][0], xs[k + 1][1] - xs[0][1], xs[k + 1][2] - xs[0][2]};
    for (int a = 0; a < 3; ++a)
      d[k][a] = (R[a] * e[0] + R[3 + a] * e[1] + R[6 + a] * e[2]) - (ms[k + 1][a] - ms[0][a]);
  }
  const double* b = Bv + 12 * t + 3;  // b_1, b_2, b_3
  double H[3][3];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) H[a][c] = d[0][a] * b[c] + d[1][a] * b[3 + c] + d[2][a] * b[6 + c];
  double vol = V[t];
  double c0 = vol * (D[3 * t] - D[3 * t + 1]), c1 = vol * D[3 * t + 1], c2 = vol * D[3 * t + 2];
  double tr = c1 * (H[0][0] + H[1][1] + H[2][2]);
  double s[3][3];
  s[0][0] = c0 * H[0][0] + tr;
  s[1][1] = c0 * H[1][1] + tr;
  s[2][2] = c0 * H[2][2] + tr;
  s[0][1] = s[1][0] = c2 * (H[0][1] + H[1][0]);
  s[0][2] = s[2][0] = c2 * (H[0][2] + H[2][0]);
  s[1][2] = s[2][1] = c2 * (H[1][2] + H[2][1]);
  double S[3][3];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) S[a][c] = R[3 * a] * s[0][c] + R[3 * a + 1] * s[1][c] + R[3 * a + 2] * s[2][c];
  double f[4][3];
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 3; ++a) f[k + 1][a] = S[a][0] * b[3 * k] + S[a][1] * b[3 * k + 1] + S[a][2] * b[3 * k + 2];
  for (int a = 0; a < 3; ++a) f[0][a] = -(f[1][a] + f[2][a] + f[3][a]);
  for (int k = 0; k < 4; ++k)
    for (int a = 0; a < 3; ++a) tet_force[12L * t + 3 * k + a] = f[k][a];
}

// FP32/FP64 apply operands b_k (k = 1..3) and (c0, c1, c2) from the init data.
__global__ void k_prepare(int T, const double* __restrict__ Bv, const double* __restrict__ D,
                          const double* __restrict__ V, float* b_f, float* c_f, double* b_d, double* c_d) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  for (int q = 0; q < 9; ++q) {
    double val = Bv[12 * t + 3 + q];
    b_f[(long)q * T + t] = float(val);
    b_d[(long)q * T + t] = val;
  }
  double vol = V[t];
  double c[3] = {vol * (D[3 * t] - D[3 * t + 1]), vol * D[3 * t + 1], vol * D[3 * t + 2]};
  for (int q = 0; q < 3; ++q) {
    c_f[(long)q * T + t] = float(c[q]);
    c_d[(long)q * T + t] = c[q];
  }
}

// Standalone y = A x (diagnostics and the apply-only roofline measurement):
// pack, one element-apply sweep, finalize.
template <typename V4>
__global__ void k_pack_operand(int N, const unsigned char* __restrict__ fixed, const double* __restrict__ x,
                               V4* u, V4* ulo, V4* q) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  store_operand(u, ulo, i, x[3 * i], x[3 * i + 1], x[3 * i + 2], fixed[i] ? 0.0 : 1.0);
  q[i] = make_v4<V4, double>(0.0, 0.0, 0.0, 0.0);
}

template <typename R>
__global__ void __launch_bounds__(kBlock, 2) k_apply_sweep(MixedArgs a, const typename ApplyOps<R>::V4* u,
                                                           const typename ApplyOps<R>::V4* ulo,
                                                           typename ApplyOps<R>::V4* q) {
  const R* re = sizeof(R) == 4 ? (const R*)a.re_f : (const R*)a.re_d;
  const R* bb = sizeof(R) == 4 ? (const R*)a.b_f : (const R*)a.b_d;
  const R* cc = sizeof(R) == 4 ? (const R*)a.c_f : (const R*)a.c_d;
  apply_tets<R>(a, u, ulo, q, re, bb, cc, R(a.dt * a.dt));
}

template <typename V4>
__global__ void k_finalize_operand(int N, const unsigned char* __restrict__ fixed, const double* __restrict__ mass,
                                   double dt, double alpha, const double* __restrict__ x, const V4* q, double* y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (fixed[i]) {
    y[3 * i] = y[3 * i + 1] = y[3 * i + 2] = 0.0;
    return;
  }
  double m = mass[i];
  double d = m + dt * (alpha * m);
  V4 qq = q[i];
  y[3 * i] = d * x[3 * i] + double(qq.x);
  y[3 * i + 1] = d * x[3 * i + 1] + double(qq.y);
  y[3 * i + 2] = d * x[3 * i + 2] + double(qq.z);
}

template <typename R>
const void* cg_kernel() {
  return reinterpret_cast<const void*>(&k_cg_persistent<R>);
}

}  // namespace

int mixed_grid_shape(Context& c, int* grid, int* block) {
  int occ32 = 0, occ64 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, k_cg_persistent<float>, kBlock, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, k_cg_persistent<double>, kBlock, 0);
  int occ = occ32 < occ64 ? occ32 : occ64;
  if (occ < 1) occ = 1;
  if (occ > 2) occ = 2;
  *grid = c.num_sms * occ;
  *block = kBlock;
  return occ;
}

cudaError_t mixed_prepare(Context& c) {
  int nb = (c.T + 255) / 256;
  if (nb < 1) nb = 1;
  k_prepare<<<nb, 256, 0, c.stream>>>(c.T, c.Bv, c.D, c.V, c.b_f, c.c_f, c.b_d, c.c_d);
  return cudaGetLastError();
}

cudaError_t launch_mixed_orient(Context& c, double dt, bool warp) {
  int nb = (c.T + 255) / 256;
  if (nb < 1) nb = 1;
  k_orient_rhs<<<nb, 256, 0, c.stream>>>(c.T, warp ? 1 : 0, c.tets, c.x, c.x0, c.E, c.V, c.Bv, c.D, c.Re,
                                         c.re_f, c.re_d, c.tet_force);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // add_plasticity_force (fem_simulate.h:102) runs between the assembly and
  // the right-hand side, as in the reference; it only changes f_ext when
  // creep and max are both positive, which the host records at init.
  if (c.plastic_active && (e = launch_plasticity(c, dt)) != cudaSuccess) return e;
  return cudaSuccess;
}

cudaError_t launch_mixed_solve(Context& c, double dt, const otfem_solver_params& prm) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(c.sync, 0, sizeof(DeviceSync), c.stream)) != cudaSuccess) return e;
  MixedArgs a;
  a.N = c.N;
  a.T = c.T;
  a.tets = c.tets;
  a.fixed = c.fixed;
  a.inc_ptr = c.inc_ptr;
  a.inc_ent = c.inc_ent;
  a.tet_force = c.tet_force;
  a.mass = c.mass;
  a.fext = c.fext;
  a.x = c.x;
  a.v = c.v;
  a.bvec = c.bvec;
  a.r = c.r;
  a.p = c.p;
  a.diag = c.diag;
  a.re_f = c.re_f;
  a.b_f = c.b_f;
  a.c_f = c.c_f;
  a.p_f = c.p_f;
  a.v_f = c.v_f;
  a.q_f = c.q_f;
  a.p_lo = c.p_lo;
  a.v_lo = c.v_lo;
  a.re_d = c.re_d;
  a.b_d = c.b_d;
  a.c_d = c.c_d;
  a.p_d = c.p_d4;
  a.v_d = c.v_d4;
  a.q_d = c.q_d;
  a.dt = dt;
  a.alpha = prm.mass_damping;
  a.rtol = prm.rtol;
  a.max_it = prm.max_iterations;
  a.refresh = prm.refresh_period;
  a.partials = c.partials;
  a.sync = c.sync;
  a.stats = c.stats;
  a.trace = c.trace;
  a.spin_limit = 4000000000LL;  // clock cycles, about two seconds
  void* args[] = {&a};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.mf_grid);
  cfg.blockDim = dim3(c.mf_block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const void* fn = prm.solver == OTFEM_SOLVER_FP64 ? cg_kernel<double>() : cg_kernel<float>();
  return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_apply_sweeps(Context& c, int solver, double dt, int sweeps) {
  MixedArgs a = {};
  a.N = c.N;
  a.T = c.T;
  a.tets = c.tets;
  a.re_f = c.re_f;
  a.b_f = c.b_f;
  a.c_f = c.c_f;
  a.re_d = c.re_d;
  a.b_d = c.b_d;
  a.c_d = c.c_d;
  a.dt = dt;
  for (int k = 0; k < sweeps; ++k) {
    if (solver == OTFEM_SOLVER_FP64)
      k_apply_sweep<double><<<c.mf_grid, kBlock, 0, c.stream>>>(a, c.p_d4, nullptr, c.q_d);
    else
      k_apply_sweep<float><<<c.mf_grid, kBlock, 0, c.stream>>>(a, c.p_f, c.p_lo, c.q_f);
  }
  return cudaGetLastError();
}

cudaError_t launch_apply_operator(Context& c, int solver, double dt, double mass_damping, const double* x,
                                  double* y) {
  MixedArgs a = {};
  a.N = c.N;
  a.T = c.T;
  a.tets = c.tets;
  a.re_f = c.re_f;
  a.b_f = c.b_f;
  a.c_f = c.c_f;
  a.re_d = c.re_d;
  a.b_d = c.b_d;
  a.c_d = c.c_d;
  a.dt = dt;
  int nb = (c.N + 255) / 256 > 0 ? (c.N + 255) / 256 : 1;
  if (solver == OTFEM_SOLVER_FP64) {
    k_pack_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, c.v_d4, nullptr, c.q_d);
    k_apply_sweep<double><<<c.mf_grid, kBlock, 0, c.stream>>>(a, c.v_d4, nullptr, c.q_d);
    k_finalize_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, c.q_d, y);
  } else {
    k_pack_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, c.v_f, c.v_lo, c.q_f);
    k_apply_sweep<float><<<c.mf_grid, kBlock, 0, c.stream>>>(a, c.v_f, c.v_lo, c.q_f);
    k_finalize_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, c.q_f, y);
  }
  return cudaGetLastError();
}

}  // namespace otfem
