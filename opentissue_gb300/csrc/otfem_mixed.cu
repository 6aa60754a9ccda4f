// otfem_mixed.cu -- matrix-free implicit step (OTFEM_SOLVER_MIXED / _FP64).
//
// Same step as fem::simulate (fem_simulate.h:94-112) without assembling K:
//   A v = b,  A = M(1 + dt*alpha) + dt^2 * sum_e Re Ke Re^T,
//   b = M v + dt (f_ext - sum_e Re Ke (Re^T x - x0))   (fem_dynamics_assembly.h:79-91)
// with Ke = V B^T D B in the B-form of fem_compute_ke.h:133-292.
//
// Kernels of one step:
//   K1 k_orient_rhs_f32 (mixed) / k_orient_rhs (FP64 solver), one thread per
//      tet: Re by the reference's row Gram-Schmidt (fem_update_orientation.h,
//      math_matrix3x3.h ortonormalize) and the elastic node forces
//      Re Ke (Re^T x - x0) of the tet.
//   K2 k_cg_mixed / k_cg_fp64: one cooperative persistent launch: b, the
//      initial residual, all CG iterations, residual replacement every
//      refresh_period iterations, the position update (fem_position_update.h).
//
// Element apply for a tet with nodes 0..3 and operand u (world frame):
//   G = sum_{k=1..3} (u_k - u_0) (x) b_k,  H = Re^T G,
//   sigma_aa = c0 H_aa + c1 tr(H),  sigma_ab = c2 (H_ab + H_ba),
//   S = Re sigma,  f_k = dt^2 S b_k (k = 1..3),  f_0 = -(f_1 + f_2 + f_3)
// with b_k the B-vectors of fem_compute_b.h and (c0, c1, c2) = V (D0 - D1, D1, D2)
// from fem_compute_isotropic_elasticity.h.  b_0 = -(b_1 + b_2 + b_3) is
// implied, so a rigid translation gives exactly zero force.
//
// Precision of the mixed solver.  GB300 executes FP64 at ~1/64 of the FP32
// rate, and every FP64 instruction (conversions and compares included) holds
// the issuing SM sub-partition for ~64 cycles, so the mixed solver runs no
// FP64 arithmetic: where cancellation needs more than FP32 it uses (hi, lo)
// float pairs, and FP64 node data is split into pairs and joined back by
// integer instructions (otfem_df.h).
//  * Element apply, search direction p, residual r: FP32.
//  * Velocity v: a (hi, lo) float pair, updated with an exact two-sum, which
//    is also the apply operand when the residual is recomputed.  The stiffness
//    sees only tet-local differences u_k - u_0, which for a translating or
//    swinging body are orders of magnitude smaller than |u|; they are formed
//    as (hi_k - hi_0) + (lo_k - lo_0), exact for nearby values (Sterbenz), so
//    they keep full FP32 relative precision.
//  * Dot products: FP32 node terms accumulated as (hi, lo) float pairs
//    (~48-bit mantissa, the accuracy of FP64 summation) and added up over the
//    grid in CTA order; alpha, beta and the estimates in FP32-pair arithmetic,
//    computed by every CTA from the same totals.
//  * b, the mass diagonal and the residual recompute b - A v: (hi, lo) pairs
//    (once per step / every refresh_period iterations); the position update
//    x += dt v keeps one FP64 addition per coordinate.
//  * K1: FP32, with the edges of the current positions from their (hi, lo)
//    split and the rest edges from a per-tet FP32 table.
// The FP64 solver keeps every vector and reduction in FP64 (accuracy
// reference).
#include <algorithm>
#include <cfloat>
#include <type_traits>
#include <vector>

#include "otfem_internal.h"
#include "otfem_df.h"
#include "otfem_refmath.cuh"

namespace otfem {
namespace {

// Threads per CTA of the persistent kernels: one CTA of 1024 threads per SM
// (measured on GB300 against two CTAs of 512: the CG iteration 2-4% and the
// cold sweep over 4M tets 5% faster; no priority between the CTAs sharing an
// SM leaves one of them finishing a sweep microseconds after the other).
constexpr int kBlock = 1024;
// Tets per apply patch: one tet per thread of a CTA.
constexpr int kPatchTets = kBlock;
// Element-apply variants, chosen per mesh by the autotuner at otfem_init.
constexpr int kApplyAtomics = 0;  // patches, shared-memory atomic accumulation
constexpr int kApplyGather = 1;   // patches, per-node gather over patch-local incidence (deterministic)
constexpr int kApplyTets = 2;     // grid-stride over tets, global vector reductions
constexpr int kApplyStaged = 3;   // tiles of tets staged in shared memory by bulk copies, global reductions
constexpr int kApplyVariants = kNumApplyVariants;
static_assert(kTileMaxTets <= kBlock, "a tile's tets fit one CTA (one tet per thread)");
// Staged apply: two tile buffers and their two mbarriers.
constexpr size_t kStageBytes = size_t(kTileMaxTets) * kTileWords * sizeof(float);
constexpr size_t kStagedSmem = 2 * kStageBytes + 2 * sizeof(unsigned long long);
// Largest persistent grid (CTAs): the last CTA of a grid sum loads one
// partial per thread, so the grid may not exceed the CTA size.
constexpr int kMaxGrid = kBlock;

struct MixedArgs {
  int N, T;
  const int4* tets;
  const unsigned char* fixed;
  const int* inc_ptr;
  const int* inc_ent;
  const double* tet_force;  // FP64 solver: 12 per tet, elastic node forces (K1)
  const float4* g_f;        // mixed: 4 per tet, elastic node forces (K1)
  const double* mass;
  const double* fext;
  double* x;
  double* v;
  double* bvec;
  double* r;
  double* p;
  double* diag;
  float* diag_f;         // the same as (hi, lo) pairs: hi (the mixed loop's vector passes)
  float* diag_lo;        //   and lo
  float4* b_hi;          // b as (hi, lo) pairs (the mixed solver's residual refreshes)
  float4* b_lo;
  const double* node_k;  // tr(sum_e Ke_ii) / 3 per node (Jacobi preconditioner)
  int precond;           // 1: CG preconditioned by the node scalars 1 / (diag + dt^2 node_k)
  // FP32 apply
  const float* re_f;
  const float* b_f;
  const float* c_f;
  float4* p_f;
  float4* v_f;
  float4* q_f;
  float4* p_lo;
  float4* v_lo;
  float4* r_f;
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
  int num_patches;
  int patch_max_nodes_padded;
  const int* patch_node_ptr;
  const int* patch_nodes;
  const ushort4* lconn;
  const int* patch_inc_ptr;             // per patch node: offsets into patch_inc
  const unsigned short* patch_inc;      // (patch-local tet << 2) | slot, ascending tet
  int apply_variant;                    // kApplyAtomics / kApplyGather / kApplyTets / kApplyStaged
  int stream_tiles;                     // tiled sweeps read the tile words past L1 (tiles beyond L2)
  const float* tile_f;                  // staged apply tiles (see Context::tile_f)
  int tile_tets, num_tiles;
  unsigned long long tile_magic;        // tile_of(t, tile_magic) = t / tile_tets
  int ordered_sums;                     // grid sums of the CTA totals in CTA order
  const float4* warm_dv;                // learned guess v + warm_dv (null: plain start from v)
  float4* dv_last;                      // in: dv_prev; out: v_new - v_old per free node
  // projected / learned start of one mesh (see Context::warm_hist)
  float4* hist;                         // difference basis: hi parts (8 x N), then lo parts (8 x N); null: none
  float4* wprod;                        // products A W_j (slots 0..8), the network's correction (slot 9)
  double* wpart;                        // per-CTA partial sums of the Gram system (ordered sums)
  double* wbacc;                        // batch: per-mesh Gram totals (num_meshes x kMaxWarmSums)
  int hist_k;                           // basis vectors searched this step
  int hist_rec;                         // basis vectors the step records
  int nwarm;                            // search directions this step (0: start from v)
  int extrap_k;                         // extrapolated start: the polynomial degree (0: none)
  int* hist_fill;                       // history levels holding the last steps' differences
  float4* v_keep;                       // kept iterates: copy k at v_keep[2kN + i] (hi), [(2k+1)N + i] (lo)
  // batched solve (see Context)
  int num_meshes;
  const int* mesh_of_node;
  const int* mesh_of_tet;
  const int* mesh_tet_start;            // num_meshes + 1: the first tet of each mesh (batches)
  const int* mesh_node_start;           // num_meshes + 1: the first node of each mesh (batches)
  BatchMesh* bm;
  double* bacc;
  unsigned char* bmask;
  const unsigned char* sweep_mask;      // standalone sweeps of a batch (autotuner): meshes to apply
  long long spin_limit;
};

// ---- synchronisation ---------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_status(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Stamps of the trace: SM clock cycles (the GPU timer's resolution is far
// coarser than one CG phase).  All stamps come from one CTA's SM (is_tracer).
__device__ __forceinline__ long long cycles_now() { return clock64(); }
// The stamping thread: thread 0 of the middle CTA, whose node ranges hold
// free nodes (a mesh whose fixed nodes come first, the usual numbering of a
// clamped end, leaves the first CTAs little node work), so the node phases
// it stamps show a full CTA's work.
__device__ __forceinline__ bool is_tracer() { return blockIdx.x == gridDim.x / 2 && threadIdx.x == 0; }

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

// ---- bulk copies into shared memory (staged apply) ----------------------
// One thread arms an mbarrier with the byte count of a tile and issues the
// bulk copy; the copy engine completes the transaction on the barrier, and
// every thread waits for the barrier's phase with a bounded spin.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arm(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Orders this thread's earlier generic-proxy accesses of shared memory (made
// visible to it by a CTA barrier) before its following bulk copies into it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for phase `parity` of the barrier to complete; false after
// spin_limit cycles.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, long long spin_limit) {
  long long start = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - start > spin_limit) return false;
  return true;
}

// Rotation <-> unit quaternion (x, y, z, w).  The quaternion of a rotation
// matrix by Shepperd's method (the largest of the four squared components
// first, for accuracy); the matrix of a quaternion by the standard product
// formula (Hamilton convention, v' = R v).
__device__ __forceinline__ float4 rotation_to_quaternion(const float* R) {
  const float tr = R[0] + R[4] + R[8];
  float x, y, z, w;
  if (tr > 0.f) {
    const float s = 2.f * sqrtf(tr + 1.f);
    w = 0.25f * s, x = (R[7] - R[5]) / s, y = (R[2] - R[6]) / s, z = (R[3] - R[1]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    const float s = 2.f * sqrtf(1.f + R[0] - R[4] - R[8]);
    w = (R[7] - R[5]) / s, x = 0.25f * s, y = (R[1] + R[3]) / s, z = (R[2] + R[6]) / s;
  } else if (R[4] > R[8]) {
    const float s = 2.f * sqrtf(1.f + R[4] - R[0] - R[8]);
    w = (R[2] - R[6]) / s, x = (R[1] + R[3]) / s, y = 0.25f * s, z = (R[5] + R[7]) / s;
  } else {
    const float s = 2.f * sqrtf(1.f + R[8] - R[0] - R[4]);
    w = (R[3] - R[1]) / s, x = (R[2] + R[6]) / s, y = (R[5] + R[7]) / s, z = 0.25f * s;
  }
  const float n = rsqrtf(x * x + y * y + z * z + w * w);
  return make_float4(x * n, y * n, z * n, w * n);
}

// Grid barriers and grid reductions.  Every CTA passes the same sequence of
// barriers, numbered 1, 2, ... (`round`), each counted once per CTA on one
// monotonic arrival counter.  Thread 0 of each CTA arrives after a CTA
// barrier with a release operation (by the PTX memory model's causality
// order this publishes every write the CTA made before the barrier).  A plain
// barrier or atomic-sum reduction (sync_round) then polls the counter with
// acquire loads until the round's gridDim.x arrivals are in.  Rounds that
// hand a result from one CTA to the others (the ordered sums and the batch's
// per-mesh scalars) arrive with an acq_rel atomic instead: the CTA whose
// ticket completes round r computes the result, publishes it and then r in
// `gen` with a release store, and the others wait for `gen` with acquire
// loads.  Waits are bounded: past `spin_limit` cycles the waiter sets
// OTFEM_ERR_TIMEOUT, and every barrier returns false on every thread of the
// CTA once any CTA has set an error status.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 only: arrive; returns true if this CTA is the last of the round.
__device__ __forceinline__ bool arrive(DeviceSync* s, unsigned round) {
  unsigned ticket = atom_add_acq_rel(&s->count, 1u);
  return ticket + 1u == round * gridDim.x;
}

// Thread 0 only: wait until round `round` is released; false on timeout or
// when another CTA has recorded an error (checked every 64 polls, off the
// fast path).
__device__ __forceinline__ bool wait_released(DeviceSync* s, unsigned round, long long spin_limit) {
  long long start = clock64();
  unsigned polls = 0;
  while (int(ld_acquire(&s->gen) - round) < 0) {
    if ((++polls & 63u) == 0u && ld_status(&s->status) != 0) return false;
    if (clock64() - start > spin_limit) {
      atomicCAS(&s->status, 0, OTFEM_ERR_TIMEOUT);
      return false;
    }
  }
  return true;
}

// The accumulator set of round - 1: every CTA read it before arriving at
// round `round`, and round + 2 uses it again, so it is cleared in between.
__device__ __forceinline__ void clear_stale_acc(DeviceSync* s, unsigned round) {
  double* acc = &s->acc[(round + 2u) % 3u][0][0];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k * kAccStride] = 0.0;
}

// Thread 0 only, the last CTA of round `round` (rounds that hand a result
// from the last CTA to the others): clears the stale accumulator set and
// releases the round.
__device__ __forceinline__ void release_round(DeviceSync* s, unsigned round) {
  clear_stale_acc(s, round);
  st_release(&s->gen, round);
}

// Thread 0 only: one grid synchronisation.  Every CTA adds its arrival to the
// counter with release semantics and polls the counter itself (acquire) until
// all gridDim.x arrivals of the round are in: one L2 round trip fewer than a
// last-arriver release (measured on GB300 with 304 CTAs: 2,900 against 3,700
// SM cycles per barrier).  The status word sits next to the counter and every
// poll reads both, so an error recorded anywhere ends the wait (a CTA that
// stopped arriving leaves the others waiting only until they see its error),
// and no separate status read precedes the arrival.  The first CTA clears
// the stale accumulator set once the round is complete; its next arrival (a
// release) publishes the clear before any CTA can pass round + 1.
__device__ __forceinline__ bool sync_round(DeviceSync* s, unsigned round, long long spin_limit) {
  red_add_release(&s->count, 1u);
  const unsigned target = round * gridDim.x;
  const long long start = clock64();
  for (;;) {
    // the counter and the status word in one acquire load
    unsigned long long w;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(&s->count) : "memory");
    if (unsigned(w >> 32) != 0u) return false;
    if (int(unsigned(w) - target) >= 0) break;
    if (clock64() - start > spin_limit) {
      atomicCAS(&s->status, 0, OTFEM_ERR_TIMEOUT);
      return false;
    }
  }
  if (blockIdx.x == 0) clear_stale_acc(s, round);
  return true;
}

__device__ bool grid_barrier(DeviceSync* s, long long spin_limit, unsigned& round) {
  __shared__ int ok;
  ++round;
  __syncthreads();
  if (threadIdx.x == 0) ok = sync_round(s, round, spin_limit) ? 1 : 0;
  __syncthreads();
  return ok != 0;
}

// (hi, lo) float pair: a value hi + lo with |lo| <= ulp(hi)/2.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  float h = s + e;
  return DF{h, e - (h - s)};
}
// (hi, lo) x b, renormalised (the product's rounding error by an FMA).
__device__ __forceinline__ DF df_mul(DF a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  const float h = p + e;
  return DF{h, e - (h - p)};
}
// a x b for two pairs, renormalised.
__device__ __forceinline__ DF df_mul2(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float h = p + e;
  return DF{h, e - (h - p)};
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
// FP64 <-> pair by integer instructions (otfem_df.h)
__device__ __forceinline__ DF df_of(double x) {
  DF r;
  dfbits::split(x, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ double f64_of(DF a) { return dfbits::join(a.hi, a.lo); }
// One component of b - (d v + q) in pair arithmetic, rounded to FP32: b and d
// as pairs, v the (hi, lo) iterate, q the FP32 element sum.
__device__ __forceinline__ float residual_df(DF b, DF d, DF v, float q) {
  const DF t = df_add(df_mul2(d, v), DF{q, 0.f});
  const DF r = df_add(b, df_neg(t));
  return r.hi + r.lo;
}
// a / b rounded to FP32: a fast approximate quotient of the high parts, then
// one correction step q + (a - q b) / b with q b formed exactly by an FMA,
// which also absorbs the approximation's few-ulp error.
__device__ __forceinline__ float df_div(DF a, DF b) {
  const float q = __fdividef(a.hi, b.hi);
  const float p = q * b.hi;
  const float e = fmaf(q, b.hi, -p);
  const float r = (((a.hi - p) - e) + a.lo) - q * b.lo;
  return q + __fdividef(r, b.hi);
}
// (hi, lo) += inc
__device__ __forceinline__ void df_inc(float& hi, float& lo, float inc) {
  float s, e;
  two_sum(hi, inc, s, e);
  e += lo;
  hi = s + e;
  lo = e - (hi - s);
}

// Accumulators of the reductions: FP64, or (hi, lo) float pairs.
template <typename Acc>
struct AccOps;
template <>
struct AccOps<double> {
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double shfl_down(double a, int o) { return __shfl_down_sync(0xffffffffu, a, o); }
  static __device__ __forceinline__ double to_double(double a) { return a; }
  static __device__ __forceinline__ double shfl_xor(double a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
  static __device__ __forceinline__ double from_double(double a) { return a; }
  static __device__ __forceinline__ double zero() { return 0.0; }
};
template <>
struct AccOps<DF> {
  static __device__ __forceinline__ DF add(DF a, DF b) { return df_add(a, b); }
  static __device__ __forceinline__ DF shfl_down(DF a, int o) {
    return DF{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
  }
  static __device__ __forceinline__ DF shfl_xor(DF a, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
  }
  static __device__ __forceinline__ double to_double(DF a) { return double(a.hi) + double(a.lo); }
  static __device__ __forceinline__ DF from_double(double a) {
    float h = float(a);
    return DF{h, float(a - double(h))};
  }
  static __device__ __forceinline__ DF zero() { return DF{0.f, 0.f}; }
};

// Warp sums of NV values per lane by a reduce-scatter butterfly: with the
// values padded to P = 2^S, each of the first S exchange steps (lane
// distance 16, 8, ...) sends half of the remaining values to the partner
// lane and adds the other half, so lane groups of 32 / P end up with one
// value each, which the remaining steps sum over the group.  That is P - 1 +
// 5 - S additions per lane instead of 5 NV.  Returns the value index this
// lane holds (its warp total) or -1 when the lane holds no total to publish.
template <typename Acc, int NV>
__device__ __forceinline__ int warp_totals(const Acc (&val)[NV], Acc& total) {
  typedef AccOps<Acc> Ops;
  static_assert(NV >= 1 && NV <= 8, "1..8 values");
  constexpr int S = NV > 4 ? 3 : NV > 2 ? 2 : NV > 1 ? 1 : 0;
  constexpr int P = 1 << S;
  const int lane = threadIdx.x & 31;
  Acc x[P];
#pragma unroll
  for (int k = 0; k < P; ++k) x[k] = k < NV ? val[k] : Ops::zero();
#pragma unroll
  for (int lvl = 0; lvl < S; ++lvl) {
    const int o = 16 >> lvl;
    const int h = P >> (lvl + 1);
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const Acc send = upper ? x[j] : x[j + h];
      const Acc keep = upper ? x[j + h] : x[j];
      x[j] = Ops::add(keep, Ops::shfl_xor(send, o));
    }
  }
#pragma unroll
  for (int o = 16 >> S; o > 0; o >>= 1) x[0] = Ops::add(x[0], Ops::shfl_xor(x[0], o));
  total = x[0];
  const int idx = lane >> (5 - S);
  return (lane & ((32 >> S) - 1)) == 0 && idx < NV ? idx : -1;
}

// Sums NV per-thread values over the grid: warp shuffles, then the warp
// totals (NV warps in parallel, one value each), then the CTA totals, and
// gives every thread of every CTA the NO outputs of fin(totals, outputs).
// Includes a grid synchronisation.
//  * Default: each CTA adds its totals into FP64 accumulators with atomic
//    reductions (sums in arrival order; each value on its own 128-byte line),
//    and once all arrivals are in every CTA reads the totals and runs fin
//    itself, so nothing but the arrivals sits between the last CTA's sums
//    and the next phase.  Accumulator sets rotate over three rounds: the set
//    of round r is read by every CTA before it arrives at round r + 1, after
//    which it is cleared for round r + 3 (clear_stale_acc).
//  * a.ordered_sums: the CTA totals go to per-CTA partials that the last CTA
//    to arrive adds up in CTA order (a fixed order), runs fin and publishes
//    the outputs; partials and outputs alternate between two halves by round
//    parity, so the writes of round r + 2 cannot overtake the reads of r.
template <typename Acc, int NV, int NO, typename Fin>
__device__ bool grid_reduce(const MixedArgs& a, const Acc (&val)[NV], double (&out)[NO], unsigned& round,
                            Fin fin) {
  static_assert(2 * NV <= kMaxPartials && NO <= 8 && NV <= 8, "partials too small");
  typedef AccOps<Acc> Ops;
  constexpr int kWarps = kBlock / 32;
  __shared__ Acc s_warp[kWarps][NV];
  __shared__ double s_tot[8];
  __shared__ double s_res[8];
  __shared__ int s_flag;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ++round;
  const int half = int(round & 1u);
  double* part = a.partials + half * (kMaxPartials / 2) * gridDim.x;
  double* acc = &a.sync->acc[round % 3u][0][0];
  {
    Acc x;
    const int k = warp_totals<Acc, NV>(val, x);
    if (k >= 0) s_warp[warp][k] = x;
  }
  __syncthreads();
  if (warp < NV) {
    // warp k: value k over the kWarps warp totals
    Acc x = lane < kWarps ? s_warp[lane][warp] : Ops::zero();
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) x = Ops::add(x, Ops::shfl_down(x, o));
    if (lane == 0) {
      if (a.ordered_sums) part[warp * gridDim.x + blockIdx.x] = Ops::to_double(x);
      else atomicAdd(acc + warp * kAccStride, Ops::to_double(x));
    }
  }
  __syncthreads();
  if (!a.ordered_sums) {
    if (threadIdx.x == 0) s_flag = sync_round(a.sync, round, a.spin_limit) ? 1 : 0;
    __syncthreads();
    const bool good = s_flag != 0;
    if (good && threadIdx.x < NV) s_tot[threadIdx.x] = __ldcg(acc + threadIdx.x * kAccStride);
    __syncthreads();
    if (good && threadIdx.x == 0) {
      double tot[NV], res[NO];
#pragma unroll
      for (int k = 0; k < NV; ++k) tot[k] = s_tot[k];
      fin(tot, res);
#pragma unroll
      for (int k = 0; k < NO; ++k) s_res[k] = res[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NO; ++k) out[k] = s_res[k];
    __syncthreads();
    return good;
  }
  if (threadIdx.x == 0) {
    // 2: last CTA, 1: wait for the release (0 once the wait failed); an
    // error recorded earlier ends the wait or the next synchronisation
    s_flag = arrive(a.sync, round) ? 2 : 1;
  }
  __syncthreads();
  if (s_flag == 2) {
    // one partial per thread (gridDim.x <= blockDim.x), then a fixed-order tree
    Acc pv[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k)
      pv[k] = threadIdx.x < gridDim.x ? Ops::from_double(__ldcg(part + k * gridDim.x + threadIdx.x)) : Ops::zero();
    {
      Acc x;
      const int k = warp_totals<Acc, NV>(pv, x);
      if (k >= 0) s_warp[warp][k] = x;
    }
    __syncthreads();
    if (warp < NV) {
      Acc x = lane < kWarps ? s_warp[lane][warp] : Ops::zero();
#pragma unroll
      for (int o = kWarps / 2; o > 0; o >>= 1) x = Ops::add(x, Ops::shfl_down(x, o));
      if (lane == 0) s_tot[warp] = Ops::to_double(x);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot[NV], res[NO];
#pragma unroll
      for (int k = 0; k < NV; ++k) tot[k] = s_tot[k];
      fin(tot, res);
      for (int k = 0; k < NO; ++k) {
        s_res[k] = res[k];
        a.sync->result[half][k] = res[k];
      }
      release_round(a.sync, round);
    }
  } else if (threadIdx.x == 0 && s_flag == 1) {
    const int ok = wait_released(a.sync, round, a.spin_limit) ? 1 : 0;
    if (ok)
      for (int k = 0; k < NO; ++k) s_res[k] = __ldcg(&a.sync->result[half][k]);
    s_flag = ok;
  }
  __syncthreads();
  const bool good = s_flag != 0;
#pragma unroll
  for (int k = 0; k < NO; ++k) out[k] = s_res[k];
  __syncthreads();
  return good;
}

// Grid sums of NV per-thread (hi, lo) values for the mixed solver, in a fixed
// order and without FP64 instructions.  On GB300 every FP64 instruction
// (arithmetic, conversion or compare) holds the issuing SM sub-partition for
// ~64 cycles, so the scalar work between two phases stays in FP32 pairs: warp
// shuffles, the warp totals, one (hi, lo) partial per CTA and value, a grid
// synchronisation, then every CTA adds up all partials in CTA order by the
// same tree, and one warp evaluates fin(totals, outputs) for the CTA.  The
// sums are bit-identical in every CTA, and for the same node values from run
// to run (the element apply's float reductions into q are unordered, so a
// whole solve is not bit-reproducible).  Partials alternate between two
// halves by round parity: a CTA writes the partials of round r + 2 only
// after every CTA has arrived at round r + 1, i.e. has read those of round r.
template <int NV, int NO, typename Fin>
__device__ bool grid_reduce_df(const MixedArgs& a, const DF (&val)[NV], float (&out)[NO], unsigned& round,
                               Fin fin) {
  static_assert(NV <= kMaxPartials / 2 && NV <= 8 && NO <= 8, "partials too small");
  constexpr int kWarps = kBlock / 32;
  __shared__ DF s_warp[kWarps][NV];
  __shared__ DF s_tot[NV];
  __shared__ int s_flag;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ++round;
  const int half = int(round & 1u);
  float2* part = reinterpret_cast<float2*>(a.partials) + size_t(half) * (kMaxPartials / 2) * gridDim.x;
  {
    DF x;
    const int k = warp_totals<DF, NV>(val, x);
    if (k >= 0) s_warp[warp][k] = x;
  }
  __syncthreads();
  if (warp < NV) {
    DF x = lane < kWarps ? s_warp[lane][warp] : DF{0.f, 0.f};
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) x = df_add(x, AccOps<DF>::shfl_down(x, o));
    if (lane == 0) part[size_t(warp) * gridDim.x + blockIdx.x] = make_float2(x.hi, x.lo);
  }
  __syncthreads();
  if (threadIdx.x == 0) s_flag = sync_round(a.sync, round, a.spin_limit) ? 1 : 0;
  __syncthreads();
  if (s_flag == 0) return false;
  DF pv[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) pv[k] = DF{0.f, 0.f};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float2 p = __ldcg(part + size_t(k) * gridDim.x + b);
      pv[k] = df_add(pv[k], DF{p.x, p.y});
    }
  }
  {
    DF x;
    const int k = warp_totals<DF, NV>(pv, x);
    if (k >= 0) s_warp[warp][k] = x;
  }
  __syncthreads();
  if (warp < NV) {
    DF x = lane < kWarps ? s_warp[lane][warp] : DF{0.f, 0.f};
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) x = df_add(x, AccOps<DF>::shfl_down(x, o));
    if (lane == 0) s_tot[warp] = x;
  }
  __syncthreads();
  // the scalar step by one warp, its outputs through shared memory
  __shared__ float s_out[NO];
  if (warp == 0) {
    DF t[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] = s_tot[k];
    float o[NO];
    fin(t, o);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NO; ++k) s_out[k] = o[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NO; ++k) out[k] = s_out[k];
  return true;
}

// The mixed solver's scalar step from its seven (hi, lo) totals, in FP32
// pairs (pcg_scalars restated without FP64 instructions): alpha = r.z / p.q;
// the updated r.z and r.r from the one-reduction identities
//   r'.z' = r.z - 2 alpha z.q + alpha^2 q.Sq,  r'.r' = r.r - 2 alpha r.q + alpha^2 q.q
// for the alpha actually applied; beta = r'.z' / r.z, or 0 on a restart or when
// the recurrence has drifted from the previous estimate by more than 25%;
// flag 1 for non-finite totals, 2 for a finite breakdown (p.q <= 0).
// Outputs: alpha, beta, the r'.r' estimate, flag, the r'.z' estimate.
struct FinPcgF {
  float prev_est;
  bool restart;
  __device__ void operator()(const DF* t, float* o) const {
    const DF pq = t[0], zq = t[1], qsq = t[2], rz = t[3], rq = t[4], qq = t[5], rr = t[6];
    const float alpha = df_div(rz, pq);
    const DF azq = df_mul(zq, alpha), aaqsq = df_mul(df_mul(qsq, alpha), alpha);
    const DF arq = df_mul(rq, alpha), aaqq = df_mul(df_mul(qq, alpha), alpha);
    DF est_z = df_add(df_add(rz, DF{-2.f * azq.hi, -2.f * azq.lo}), aaqsq);
    DF est_r = df_add(df_add(rr, DF{-2.f * arq.hi, -2.f * arq.lo}), aaqq);
    if (est_z.hi < 0.f) est_z = DF{0.f, 0.f};
    if (est_r.hi < 0.f) est_r = DF{0.f, 0.f};
    float beta = df_div(est_z, rz);
    float flag = 0.f;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 7; ++k) finite = finite && isfinite(t[k].hi) && isfinite(t[k].lo);
    if (!finite) flag = 1.f;
    else if (!(pq.hi > 0.f) || !isfinite(alpha) || !isfinite(beta)) flag = 2.f;
    if (restart || (prev_est >= 0.f && fabsf(prev_est - rz.hi) > 0.25f * rz.hi)) beta = 0.f;
    o[0] = alpha;
    o[1] = beta;
    o[2] = est_r.hi + est_r.lo;
    o[3] = flag;
    o[4] = est_z.hi + est_z.lo;
  }
};
struct FinIdentityF1 {
  __device__ void operator()(const DF* t, float* o) const { o[0] = t[0].hi + t[0].lo; }
};
struct FinIdentityF2 {
  __device__ void operator()(const DF* t, float* o) const {
    o[0] = t[0].hi + t[0].lo;
    o[1] = t[1].hi + t[1].lo;
  }
};

struct FinIdentity1 {
  __device__ void operator()(const double* t, double* o) const { o[0] = t[0]; }
};
struct FinIdentity2 {
  __device__ void operator()(const double* t, double* o) const {
    o[0] = t[0];
    o[1] = t[1];
  }
};

// Preconditioned CG (z = S r, S the node scalars; S = I without the
// preconditioner) with both CG scalars from one grid sum.  Totals: p.q,
// z.q, q.Sq, the exact r.z, r.q, q.q and the exact r.r of the current r.
// alpha = r.z / p.q; the new r' = r - alpha q has
//   r'.z' = r.z - 2 alpha z.q + alpha^2 q.Sq   (sets beta = r'.z' / r.z)
//   r'.r' = r.r - 2 alpha r.q + alpha^2 q.q    (the convergence estimate)
// so the vector update can form p' = z' + beta p in the same pass.  Outputs:
// alpha, beta, the r'.r' estimate, flag (0 ok, 1 non-finite system, 2 finite
// breakdown), the r'.z' estimate.  The previous iteration's r'.z' estimate
// (prev_est < 0: none) checks the recurrence against the exact r.z: when they
// disagree by more than a quarter, or on `restart`, beta = 0 restarts the
// search direction from z (preconditioned steepest descent, which cannot grow
// the error) instead of letting an inaccurate recurrence near the precision
// floor amplify itself.
__device__ __forceinline__ void pcg_scalars(const double* t, double prev_est, bool restart, double* o) {
  const double pq = t[0], zq = t[1], qsq = t[2], rz = t[3], rq = t[4], qq = t[5], rr = t[6];
  // independent reciprocals instead of dependent divisions
  const double inv_pq = 1.0 / pq, inv_rz = 1.0 / rz;
  const double alpha = rz * inv_pq;
  double est_z = rz - 2.0 * alpha * zq + alpha * alpha * qsq;
  double est_r = rr - 2.0 * alpha * rq + alpha * alpha * qq;
  if (est_z < 0.0) est_z = 0.0;
  if (est_r < 0.0) est_r = 0.0;
  double beta = est_z * inv_rz;
  double flag = 0.0;
  bool finite = true;
  for (int k = 0; k < 7; ++k) finite = finite && isfinite(t[k]);
  if (!finite) flag = 1.0;
  else if (!(pq > 0.0) || !isfinite(alpha) || !isfinite(beta)) flag = 2.0;
  if (restart || (prev_est >= 0.0 && fabs(prev_est - rz) > 0.25 * rz)) beta = 0.0;
  o[0] = alpha;
  o[1] = beta;
  o[2] = est_r;
  o[3] = flag;
  o[4] = est_z;
}
// The FP64 solver's scalar step, whose exact r.z (t_rz) and r.r come from the
// grid sum after the vector update: totals p.q, z.q, q.Sq, r.q, q.q; outputs
// alpha, beta, the r'.r' estimate, flag.
struct FinPcgFp64 {
  double rz, rr;
  __device__ void operator()(const double* t, double* o) const {
    const double u[7] = {t[0], t[1], t[2], rz, t[3], t[4], rr};
    double w[5];
    pcg_scalars(u, -1.0, false, w);
    for (int k = 0; k < 4; ++k) o[k] = w[k];
  }
};

// Jacobi scalar of a free node whose mass term is dg (1 without the preconditioner).
__device__ __forceinline__ double jacobi_scale(const MixedArgs& a, long i, double dg) {
  return a.precond ? 1.0 / (dg + a.dt * a.dt * a.node_k[i]) : 1.0;
}

// Coherent (L2) load of node data written by other CTAs within the launch.
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

template <typename R>
struct SmemOperand;
template <>
struct SmemOperand<float> {  // per patch node: hi, lo, accumulator
  static constexpr size_t bytes = sizeof(float4) * 2 + sizeof(float) * 3;
};
template <>
struct SmemOperand<double> {
  static constexpr size_t bytes = sizeof(double4) + sizeof(double) * 3;
};

// One element-apply sweep q += dt^2 K' u, by patches.  A CTA takes patches
// blockIdx.x, blockIdx.x + gridDim.x, ...: it loads its tet's data, stages
// the patch's nodes (the operand, as hi/lo pairs for FP32) in shared memory
// once, computes one tet per thread, adds the four node forces into
// shared-memory accumulators, and writes each node back once: a plain store
// when no other patch touches the node, a global vector reduction otherwise.
// Nodes whose operand w == 0 (fixed rows, never read) are not written.  ulo
// may be null (operand exactly FP32).  The operand is rewritten by other
// CTAs between sweeps of a launch, so it is loaded with plain (coherent)
// loads, ordered after the writers by the grid barrier; the per-tet data is
// constant during a launch.
template <typename R>
__device__ void apply_patches(const MixedArgs& a, const typename ApplyOps<R>::V4* u4,
                              const typename ApplyOps<R>::V4* ulo, typename ApplyOps<R>::V4* q4,
                              const R* __restrict__ re, const R* __restrict__ bb, const R* __restrict__ cc,
                              R scale, unsigned char* smem) {
  typedef typename ApplyOps<R>::V4 V4;
  V4* s_hi = reinterpret_cast<V4*>(smem);
  const int cap = a.patch_max_nodes_padded;
  float4* s_lo = reinterpret_cast<float4*>(s_hi + cap);
  R* s_acc = sizeof(R) == 4 ? reinterpret_cast<R*>(s_lo + cap) : reinterpret_cast<R*>(s_hi + cap);
  const int T = a.T;
  const bool has_lo = sizeof(R) == 4 && ulo != nullptr;
  for (int patch = blockIdx.x; patch < a.num_patches; patch += gridDim.x) {
    const int t = patch * kPatchTets + threadIdx.x;
    const bool active = t < T;
    // per-tet data first: independent of the staging, so the loads overlap it
    ushort4 l = make_ushort4(0, 0, 0, 0);
    R Re[9], b[9], c0 = R(0), c1 = R(0), c2 = R(0);
    if (active) {
      l = a.lconn[t];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        Re[k] = re[(long)k * T + t];
        b[k] = bb[(long)k * T + t];
      }
      c0 = cc[t];
      c1 = cc[T + t];
      c2 = cc[2L * T + t];
    }
    const int nb = a.patch_node_ptr[patch];
    const int nn = a.patch_node_ptr[patch + 1] - nb;
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      int id = a.patch_nodes[nb + j] & 0x7fffffff;
      s_hi[j] = u4[id];
      if (sizeof(R) == 4)
        s_lo[j] = has_lo ? reinterpret_cast<const float4*>(ulo)[id] : make_float4(0.f, 0.f, 0.f, 0.f);
      s_acc[3 * j] = R(0);
      s_acc[3 * j + 1] = R(0);
      s_acc[3 * j + 2] = R(0);
    }
    __syncthreads();
    if (active) {
      const int ln[4] = {l.x, l.y, l.z, l.w};
      V4 w[4] = {s_hi[l.x], s_hi[l.y], s_hi[l.z], s_hi[l.w]};
      R du[3][3];
      if (sizeof(R) == 4) {
        float4 lo[4] = {s_lo[l.x], s_lo[l.y], s_lo[l.z], s_lo[l.w]};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          du[k][0] = R((float(w[k + 1].x) - float(w[0].x)) + (lo[k + 1].x - lo[0].x));
          du[k][1] = R((float(w[k + 1].y) - float(w[0].y)) + (lo[k + 1].y - lo[0].y));
          du[k][2] = R((float(w[k + 1].z) - float(w[0].z)) + (lo[k + 1].z - lo[0].z));
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          du[k][0] = R(w[k + 1].x - w[0].x);
          du[k][1] = R(w[k + 1].y - w[0].y);
          du[k][2] = R(w[k + 1].z - w[0].z);
        }
      }
      R f[4][3];
      element_apply<R>(Re, b, c0, c1, c2, scale, du, f);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (w[k].w != 0) {
          atomicAdd(s_acc + 3 * ln[k], f[k][0]);
          atomicAdd(s_acc + 3 * ln[k] + 1, f[k][1]);
          atomicAdd(s_acc + 3 * ln[k] + 2, f[k][2]);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      if (s_hi[j].w == 0) continue;
      const int raw = a.patch_nodes[nb + j];
      const int id = raw & 0x7fffffff;
      R x = s_acc[3 * j], y = s_acc[3 * j + 1], z = s_acc[3 * j + 2];
      if (raw < 0) {
        red_add(q4 + id, x, y, z);
      } else {
        V4 v;
        v.x = x;
        v.y = y;
        v.z = z;
        v.w = R(0);
        q4[id] = v;
      }
    }
    __syncthreads();
  }
}

// u_k - u_0 of one tet from the four (hi, lo) operands (FP32) or FP64 operands.
template <typename R, typename V4>
__device__ __forceinline__ void tet_differences(const V4 (&w)[4], const float4 (&lo)[4], R (&du)[3][3]) {
  if (sizeof(R) == 4) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      du[k][0] = R((float(w[k + 1].x) - float(w[0].x)) + (lo[k + 1].x - lo[0].x));
      du[k][1] = R((float(w[k + 1].y) - float(w[0].y)) + (lo[k + 1].y - lo[0].y));
      du[k][2] = R((float(w[k + 1].z) - float(w[0].z)) + (lo[k + 1].z - lo[0].z));
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      du[k][0] = R(w[k + 1].x - w[0].x);
      du[k][1] = R(w[k + 1].y - w[0].y);
      du[k][2] = R(w[k + 1].z - w[0].z);
    }
  }
}

// Variant kApplyGather: as apply_patches, but each thread writes its tet's
// four node forces to shared memory and each node then sums its own entries
// in ascending tet order (patch_inc): no atomics, deterministic.
template <typename R>
__device__ void apply_patches_gather(const MixedArgs& a, const typename ApplyOps<R>::V4* u4,
                                     const typename ApplyOps<R>::V4* ulo, typename ApplyOps<R>::V4* q4,
                                     const R* __restrict__ re, const R* __restrict__ bb, const R* __restrict__ cc,
                                     R scale, unsigned char* smem) {
  typedef typename ApplyOps<R>::V4 V4;
  V4* s_hi = reinterpret_cast<V4*>(smem);
  const int cap = a.patch_max_nodes_padded;
  float4* s_lo = reinterpret_cast<float4*>(s_hi + cap);
  R* s_f = sizeof(R) == 4 ? reinterpret_cast<R*>(s_lo + cap) : reinterpret_cast<R*>(s_hi + cap);
  const int T = a.T;
  const bool has_lo = sizeof(R) == 4 && ulo != nullptr;
  for (int patch = blockIdx.x; patch < a.num_patches; patch += gridDim.x) {
    const int t = patch * kPatchTets + threadIdx.x;
    const bool active = t < T;
    ushort4 l = make_ushort4(0, 0, 0, 0);
    R Re[9], b[9], c0 = R(0), c1 = R(0), c2 = R(0);
    if (active) {
      l = a.lconn[t];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        Re[k] = re[(long)k * T + t];
        b[k] = bb[(long)k * T + t];
      }
      c0 = cc[t];
      c1 = cc[T + t];
      c2 = cc[2L * T + t];
    }
    const int nb = a.patch_node_ptr[patch];
    const int nn = a.patch_node_ptr[patch + 1] - nb;
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      int id = a.patch_nodes[nb + j] & 0x7fffffff;
      s_hi[j] = u4[id];
      if (sizeof(R) == 4)
        s_lo[j] = has_lo ? reinterpret_cast<const float4*>(ulo)[id] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    if (active) {
      V4 w[4] = {s_hi[l.x], s_hi[l.y], s_hi[l.z], s_hi[l.w]};
      float4 lo[4];
      if (sizeof(R) == 4) {
        lo[0] = s_lo[l.x];
        lo[1] = s_lo[l.y];
        lo[2] = s_lo[l.z];
        lo[3] = s_lo[l.w];
      }
      R du[3][3], f[4][3];
      tet_differences<R>(w, lo, du);
      element_apply<R>(Re, b, c0, c1, c2, scale, du, f);
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) s_f[(k * 3 + c) * kPatchTets + threadIdx.x] = f[k][c];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      if (s_hi[j].w == 0) continue;
      R x = R(0), y = R(0), z = R(0);
      for (int e = a.patch_inc_ptr[nb + j]; e < a.patch_inc_ptr[nb + j + 1]; ++e) {
        const int ent = a.patch_inc[e], lt = ent >> 2, sl = ent & 3;
        x += s_f[(sl * 3) * kPatchTets + lt];
        y += s_f[(sl * 3 + 1) * kPatchTets + lt];
        z += s_f[(sl * 3 + 2) * kPatchTets + lt];
      }
      const int raw = a.patch_nodes[nb + j];
      const int id = raw & 0x7fffffff;
      if (raw < 0) {
        red_add(q4 + id, x, y, z);
      } else {
        V4 v;
        v.x = x;
        v.y = y;
        v.z = z;
        v.w = R(0);
        q4[id] = v;
      }
    }
    __syncthreads();
  }
}

// First item (tet or node) of this thread in a grid-stride sweep (stride
// gridDim.x * blockDim.x).  Warps are numbered across the CTAs first (warp k
// of CTA b is warp k * gridDim.x + b) and each covers 32 consecutive items, so
// a partial last round spreads over every SM instead of falling on the first
// CTAs (whose SMs the next barrier would wait for), while each round still
// covers one contiguous range of items.
__device__ __forceinline__ long sweep_first() {
  return ((long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
}

// Variant kApplyTets: one tet per thread over the whole mesh (grid-stride),
// operands gathered from global memory, node forces added with global vector
// reductions (the accumulator must be zero for every written node).
template <typename R>
__device__ void apply_tets(const MixedArgs& a, const typename ApplyOps<R>::V4* u4,
                           const typename ApplyOps<R>::V4* ulo, typename ApplyOps<R>::V4* q4,
                           const R* __restrict__ re, const R* __restrict__ bb, const R* __restrict__ cc,
                           R scale, const unsigned char* mask) {
  typedef typename ApplyOps<R>::V4 V4;
  const int T = a.T;
  const bool has_lo = sizeof(R) == 4 && ulo != nullptr;
  for (int t = int(sweep_first()); t < T; t += gridDim.x * blockDim.x) {
    if (mask && !mask[a.mesh_of_tet[t]]) continue;  // batched solve: mesh not in this sweep
    const int4 n = a.tets[t];
    V4 w[4] = {u4[n.x], u4[n.y], u4[n.z], u4[n.w]};
    float4 lo[4];
    if (sizeof(R) == 4) {
      if (has_lo) {
        const float4* l4 = reinterpret_cast<const float4*>(ulo);
        lo[0] = l4[n.x];
        lo[1] = l4[n.y];
        lo[2] = l4[n.z];
        lo[3] = l4[n.w];
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) lo[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    R Re[9], b[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      Re[k] = re[(long)k * T + t];
      b[k] = bb[(long)k * T + t];
    }
    R du[3][3], f[4][3];
    tet_differences<R>(w, lo, du);
    element_apply<R>(Re, b, cc[t], cc[T + t], cc[2L * T + t], scale, du, f);
    const int nn[4] = {n.x, n.y, n.z, n.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (w[k].w != 0) red_add(q4 + nn[k], f[k][0], f[k][1], f[k][2]);
  }
}

// Staged-apply tile claims.  Tickets come from one monotonic counter that is
// zero at the start of a launch, and every CTA's claims in a sweep end with
// exactly one ticket past the last tile, so a sweep consumes num_tiles +
// gridDim.x tickets and ticket k is tile k mod (num_tiles + gridDim.x) of
// its sweep (values >= num_tiles: no tile left).  Sweeps of a launch are
// separated by grid barriers, so their tickets do not interleave.
__device__ __forceinline__ int claim_tile(const MixedArgs& a) {
  const unsigned span = unsigned(a.num_tiles) + gridDim.x;
  const unsigned k = atomicAdd(&a.sync->tile_ticket, 1u) % span;
  return k < unsigned(a.num_tiles) ? int(k) : -1;
}

// Variant kApplyStaged (FP32): as kApplyTets, but the per-tet data (node
// ids, rotation quaternion, b_1..b_3, c0..c2: 80 bytes per tet) arrives in
// shared memory by bulk copies, a tile of tile_tets tets at a time and one
// tile ahead of the computation, so no thread waits on DRAM for it.  Each
// sweep initialises its two mbarriers and invalidates them at the end (a
// valid mbarrier must not be initialised again).  CTAs
// claim tiles dynamically (claim_tile), so SMs that see more memory
// bandwidth take more tiles.  On a copy that does not complete within
// spin_limit cycles the CTA sets OTFEM_ERR_TIMEOUT, stops, and waits (again
// bounded) for the copies it still has in flight before returning.
// Batched solve: whether any mesh with tets in `tile` is in the sweep
// (meshes own contiguous tet ranges, so the tile's first and last tets bound
// them).
__device__ __forceinline__ bool tile_in_sweep(const MixedArgs& a, int tile, const unsigned char* mask) {
  const int first = tile * a.tile_tets;
  const int last = min(a.T, first + a.tile_tets) - 1;
  for (int m = a.mesh_of_tet[first]; m <= a.mesh_of_tet[last]; ++m)
    if (mask[m]) return true;
  return false;
}

// The next tile of this sweep whose meshes take part (every tile is drawn
// exactly once; -1: none left).
__device__ __forceinline__ int claim_sweep_tile(const MixedArgs& a, const unsigned char* mask) {
  for (;;) {
    const int tile = claim_tile(a);
    if (tile < 0 || !mask || tile_in_sweep(a, tile, mask)) return tile;
  }
}

template <typename Body>
__device__ void staged_sweep(const MixedArgs& a, unsigned char* smem, const unsigned char* mask, Body body) {
  const int TT = a.tile_tets;
  const unsigned tile_bytes = unsigned(TT) * kTileWords * sizeof(float);
  auto stage = [smem](int sb) { return reinterpret_cast<float*>(smem + sb * kStageBytes); };
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + 2 * kStageBytes);
  __shared__ int s_tile[2];  // tile in each buffer, -1: none
  __shared__ int s_more;     // thread 0 has not yet drawn the sweep's last ticket
  const int tid = threadIdx.x;
  __syncthreads();  // the buffers' previous readers are done
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    int more = 1;
    for (int sb = 0; sb < 2; ++sb) {
      const int tile = more ? claim_sweep_tile(a, mask) : -1;
      if (tile < 0) more = 0;
      s_tile[sb] = tile;
      if (tile >= 0) {
        mbar_arm(&bar[sb], tile_bytes);
        bulk_copy_g2s(stage(sb), a.tile_f + size_t(tile) * kTileWords * TT, tile_bytes, &bar[sb]);
      }
    }
    s_more = more;
  }
  __syncthreads();
  int j = 0;
  bool failed = false;
  for (;; ++j) {
    const int sb = j & 1;
    const int tile = s_tile[sb];  // written before the previous CTA barrier
    if (tile < 0) break;
    const bool ok = mbar_wait(&bar[sb], (j >> 1) & 1, a.spin_limit);
    const int t = tile * TT + tid;
    if (ok && tid < TT && t < a.T && (!mask || mask[a.mesh_of_tet[t]])) body(stage(sb), TT, tid);
    // every thread is done with buffer sb: refill it with the next claim
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (tid == 0) {
      const int next = s_more ? claim_sweep_tile(a, mask) : -1;
      if (next < 0) s_more = 0;
      s_tile[sb] = next;
      if (next >= 0) {
        fence_proxy_async_smem();
        mbar_arm(&bar[sb], tile_bytes);
        bulk_copy_g2s(stage(sb), a.tile_f + size_t(next) * kTileWords * TT, tile_bytes, &bar[sb]);
      }
    }
  }
  if (failed && tid == 0) {
    atomicCAS(&a.sync->status, 0, OTFEM_ERR_TIMEOUT);
    // the copies of claims j and j + 1 may still be arriving
    for (int k = j; k < j + 2; ++k)
      if (s_tile[k & 1] >= 0) mbar_wait(&bar[k & 1], (k >> 1) & 1, a.spin_limit);
  }
  // end of the barriers' life: the next sweep initialises them afresh
  __syncthreads();
  if (tid == 0) {
    mbar_inval(&bar[0]);
    mbar_inval(&bar[1]);
  }
}

// One tile word.  Stream: for sweeps whose tiles do not fit in L2 and stream
// from HBM, the word is read past L1 and marked first to be evicted from L2
// (ld.global.nc.L1::no_allocate with an L2::evict_first cache policy): a tile
// word is read once per sweep, so L2 is left to the node vectors, which the
// sweep gathers and accumulates and the node passes read again.
template <bool Stream>
__device__ __forceinline__ float ld_tile_word(const float* p) {
  if constexpr (Stream) {
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    float v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
  } else {
    return *p;
  }
}

// A staged tile's words for tet `tid`: node ids, rotation, B-vectors, constants.
template <bool Stream = false>
struct StagedTetT {
  int nn[4];
  float Re[9], b[9], c0, c1, c2;
  __device__ __forceinline__ StagedTetT(const float* w, int TT, int tid) {
#pragma unroll
    for (int k = 0; k < 4; ++k) nn[k] = __float_as_int(ld_tile_word<Stream>(w + k * TT + tid));
    load_rest(w, TT, tid);
  }
  // with the node ids already loaded (the tets variant loads them one tet ahead)
  __device__ __forceinline__ StagedTetT(const float* w, int TT, int tid, const int4& ids) {
    nn[0] = ids.x;
    nn[1] = ids.y;
    nn[2] = ids.z;
    nn[3] = ids.w;
    load_rest(w, TT, tid);
  }
  __device__ __forceinline__ void load_rest(const float* w, int TT, int tid) {
    quaternion_to_rotation(make_float4(ld_tile_word<Stream>(w + 4 * TT + tid), ld_tile_word<Stream>(w + 5 * TT + tid),
                                       ld_tile_word<Stream>(w + 6 * TT + tid), ld_tile_word<Stream>(w + 7 * TT + tid)),
                           Re);
#pragma unroll
    for (int k = 0; k < 9; ++k) b[k] = ld_tile_word<Stream>(w + (8 + k) * TT + tid);
    c0 = ld_tile_word<Stream>(w + 17 * TT + tid);
    c1 = ld_tile_word<Stream>(w + 18 * TT + tid);
    c2 = ld_tile_word<Stream>(w + 19 * TT + tid);
  }
};
using StagedTet = StagedTetT<false>;

// Node ids of tet t from its tile (words 0..3), or zeros past the end.
template <bool Stream = false>
__device__ __forceinline__ int4 tile_node_ids(const MixedArgs& a, int t) {
  if (t >= a.T) return make_int4(0, 0, 0, 0);
  const int TT = a.tile_tets, tile = tile_of(t, a.tile_magic);
  const float* w = a.tile_f + size_t(tile) * kTileWords * TT + (t - tile * TT);
  return make_int4(__float_as_int(ld_tile_word<Stream>(w)), __float_as_int(ld_tile_word<Stream>(w + TT)),
                   __float_as_int(ld_tile_word<Stream>(w + 2 * TT)), __float_as_int(ld_tile_word<Stream>(w + 3 * TT)));
}

// q += dt^2 K_e u for one tet (FP32; u with an optional lo part).
__device__ __forceinline__ void tet_apply(const float* Re, const float* b, float c0, float c1, float c2, float scale,
                                          const int (&nn)[4], const float4* u4, const float4* ulo, float4* q4) {
  float4 wv[4], lo[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) wv[k] = u4[nn[k]];
  if (ulo) {
#pragma unroll
    for (int k = 0; k < 4; ++k) lo[k] = ulo[nn[k]];
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) lo[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float du[3][3], f[4][3];
  tet_differences<float>(wv, lo, du);
  element_apply<float>(Re, b, c0, c1, c2, scale, du, f);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (wv[k].w != 0) red_add(q4 + nn[k], f[k][0], f[k][1], f[k][2]);
}

__device__ void apply_staged(const MixedArgs& a, const float4* u4, const float4* ulo, float4* q4, float scale,
                             unsigned char* smem, const unsigned char* mask) {
  staged_sweep(a, smem, mask, [&](const float* w, int TT, int tid) {
    const StagedTet e(w, TT, tid);
    tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, u4, ulo, q4);
  });
}

// Tets variant in FP32: one tet per thread, grid-stride, its words read
// straight from the tiles (node ids, quaternion, B-vectors, constants: 80 B).
// The node ids of the thread's next tet are loaded one tet ahead, so that
// their L2 round trip overlaps this tet's gathers and arithmetic instead of
// preceding the next tet's gathers.  In a batch (mask) a tet of a mesh not in
// the sweep is skipped before anything but its mesh id is loaded.
__device__ __forceinline__ bool tet_in_sweep(const MixedArgs& a, const unsigned char* mask, int t) {
  return t < a.T && (!mask || mask[a.mesh_of_tet[t]]);
}
// The meshes of a batch selected by a mask (at most kBlock meshes), as one
// virtual range of their tets or nodes: every CTA lists them with a CTA-wide
// scan of the mask (meshes without elements left out), list entry j holding
// mesh mesh[j] whose elements starts[m] ... lie at [pref[j], pref[j + 1]) of
// the virtual range.  The lists live in shared memory until the next call.
struct MeshList {
  const int* beg;   // first element of entry j's mesh
  const int* pref;  // n + 1 virtual offsets
  const int* mesh;  // mesh id of entry j
  int n, total;
  // the list entry holding virtual element v < total: the last j with
  // pref[j] <= v (the counts are positive, so pref increases strictly)
  __device__ __forceinline__ int entry(int v) const {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pref[mid] <= v) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
};
__device__ MeshList masked_meshes(const MixedArgs& a, const int* starts, const unsigned char* mask) {
  __shared__ int s_beg[kBlock], s_pref[kBlock + 1], s_mesh[kBlock], s_wsum[kBlock / 32], s_wcnt[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, m = threadIdx.x;
  __syncthreads();  // the previous list's readers are done
  int beg = 0, cnt = 0;
  if (m < a.num_meshes && mask[m]) {
    beg = starts[m];
    cnt = starts[m + 1] - beg;
  }
  // CTA-wide inclusive scans of the flags and of the counts (warp shuffles,
  // then the warp totals by warp 0)
  int f = cnt > 0 ? 1 : 0, c = f ? cnt : 0;
  int fi = f, ci = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int yf = __shfl_up_sync(0xffffffffu, fi, o), yc = __shfl_up_sync(0xffffffffu, ci, o);
    if (lane >= o) fi += yf, ci += yc;
  }
  if (lane == 31) s_wsum[warp] = fi, s_wcnt[warp] = ci;
  __syncthreads();
  if (warp == 0) {
    int tf = lane < kBlock / 32 ? s_wsum[lane] : 0, tc = lane < kBlock / 32 ? s_wcnt[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int yf = __shfl_up_sync(0xffffffffu, tf, o), yc = __shfl_up_sync(0xffffffffu, tc, o);
      if (lane >= o) tf += yf, tc += yc;
    }
    if (lane < kBlock / 32) s_wsum[lane] = tf, s_wcnt[lane] = tc;  // inclusive totals through each warp
  }
  __syncthreads();
  const int f_before = (warp ? s_wsum[warp - 1] : 0) + fi - f, c_before = (warp ? s_wcnt[warp - 1] : 0) + ci - c;
  MeshList L;
  L.n = s_wsum[kBlock / 32 - 1];
  L.total = s_wcnt[kBlock / 32 - 1];
  if (f) {
    s_beg[f_before] = beg;
    s_pref[f_before] = c_before;
    s_mesh[f_before] = m;
  }
  if (threadIdx.x == 0) s_pref[L.n] = L.total;
  __syncthreads();
  L.beg = s_beg;
  L.pref = s_pref;
  L.mesh = s_mesh;
  return L;
}

// Tets of an unmasked sweep streaming from HBM, handed out dynamically:
// warps claim 32-element chunks blockIdx.x + k * gridDim.x (k = 0, 1, ...)
// from a counter of their CTA, so that the CTA's warps finish together
// whatever their issue priority and the memory latency they meet (measured
// on GB300: the cold sweep over 4M tets 5% faster than the static
// grid-stride interleave; with the tiles resident in L2, and in a batch's
// masked sweeps inside the solve, the static interleave is faster).
// body(v, pre) runs for every element v < n, with the next chunk claimed and
// prefetch(v) issued one chunk ahead.
template <typename Prefetch, typename Body>
__device__ __forceinline__ void claimed_chunks(int n, Prefetch prefetch, Body body) {
  __shared__ int s_next;
  const int lane = threadIdx.x & 31;
  __syncthreads();  // the previous sweep's claims are done
  if (threadIdx.x == 0) s_next = 0;
  __syncthreads();
  const int nchunks = (n + 31) >> 5;
  auto claim = [&]() -> int {
    int k = 0;
    if (lane == 0) k = atomicAdd(&s_next, 1);
    k = __shfl_sync(0xffffffffu, k, 0);
    const long c = long(blockIdx.x) + long(k) * gridDim.x;
    return c < nchunks ? int(c) : -1;
  };
  int chunk = claim();
  int v = chunk >= 0 ? chunk * 32 + lane : n;
  auto pre = prefetch(v);
  while (chunk >= 0) {
    const int cur_v = v;
    const auto cur = pre;
    chunk = claim();
    v = chunk >= 0 ? chunk * 32 + lane : n;
    pre = prefetch(v);
    if (cur_v < n) body(cur_v, cur);
  }
}

// A batch's masked sweep over the meshes in the sweep only: their tets as
// one virtual range, so that a sweep late in a step, when a few meshes still
// iterate, costs in proportion to their tets instead of reading the mesh id
// of every tet of the batch.
template <bool Stream>
__device__ void apply_active_meshes(const MixedArgs& a, const float4* u4, const float4* ulo, float4* q4, float scale,
                                    const unsigned char* mask) {
  const MeshList L = masked_meshes(a, a.mesh_tet_start, mask);
  const int TT = a.tile_tets, stride = gridDim.x * blockDim.x;
  // every mesh in the sweep: the virtual range is the tet range itself
  const bool all = L.n == a.num_meshes;
  auto tet_of = [&](int v) {
    if (all) return v;
    const int j = L.entry(v);
    return L.beg[j] + (v - L.pref[j]);
  };
  // the next tet's node ids are loaded one tet ahead (as in the tets sweep)
  int v = int(sweep_first());
  int t = v < L.total ? tet_of(v) : 0;
  int4 ids = v < L.total ? tile_node_ids<Stream>(a, t) : make_int4(0, 0, 0, 0);
  for (; v < L.total; v += stride) {
    const int cur_t = t;
    const int4 cur = ids;
    if (v + stride < L.total) {
      t = tet_of(v + stride);
      ids = tile_node_ids<Stream>(a, t);
    }
    const int tile = tile_of(cur_t, a.tile_magic);
    const StagedTetT<Stream> e(a.tile_f + size_t(tile) * kTileWords * TT, TT, cur_t - tile * TT, cur);
    tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, u4, ulo, q4);
  }
}

template <bool Stream>
__device__ void apply_tets_tiled_impl(const MixedArgs& a, const float4* u4, const float4* ulo, float4* q4,
                                      float scale, const unsigned char* mask) {
  if (mask && a.mesh_tet_start && a.num_meshes <= kBlock && blockDim.x == kBlock) {
    apply_active_meshes<Stream>(a, u4, ulo, q4, scale, mask);
    return;
  }
  const int T = a.T, TT = a.tile_tets, stride = gridDim.x * blockDim.x;
  if (Stream && !mask) {
    claimed_chunks(
        T, [&](int t) { return t < T ? tile_node_ids<Stream>(a, t) : make_int4(0, 0, 0, 0); },
        [&](int t, const int4& ids) {
          const int tile = tile_of(t, a.tile_magic);
          const StagedTetT<Stream> e(a.tile_f + size_t(tile) * kTileWords * TT, TT, t - tile * TT, ids);
          tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, u4, ulo, q4);
        });
    return;
  }
  int t = int(sweep_first());
  bool act = tet_in_sweep(a, mask, t);
  int4 ids = act ? tile_node_ids<Stream>(a, t) : make_int4(0, 0, 0, 0);
  for (; t < T; t += stride) {
    const int4 cur = ids;
    const bool cur_act = act;
    act = tet_in_sweep(a, mask, t + stride);
    ids = act ? tile_node_ids<Stream>(a, t + stride) : make_int4(0, 0, 0, 0);
    if (!cur_act) continue;
    const int tile = tile_of(t, a.tile_magic);
    const StagedTetT<Stream> e(a.tile_f + size_t(tile) * kTileWords * TT, TT, t - tile * TT, cur);
    tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, u4, ulo, q4);
  }
}
// AllowStream: the caller may meet tiles beyond L2 (batches, standalone
// sweeps); the single-mesh solver keeps one, non-streaming, copy of the sweep.
template <bool AllowStream>
__device__ void apply_tets_tiled(const MixedArgs& a, const float4* u4, const float4* ulo, float4* q4, float scale,
                                 const unsigned char* mask) {
  if (AllowStream && a.stream_tiles) apply_tets_tiled_impl<true>(a, u4, ulo, q4, scale, mask);
  else apply_tets_tiled_impl<false>(a, u4, ulo, q4, scale, mask);
}

// Search direction j of the projected start: basis vector j of the
// velocity-change history, then the network's correction.
__device__ __forceinline__ const float4* warm_dir(const MixedArgs& a, int j) {
  return j < a.hist_k ? a.hist + size_t(j) * a.N : a.wprod + size_t(kMaxWarmDirs) * a.N;
}

// Projected start: A v (the (hi, lo) iterate, into q) and A W_j for every
// search direction in one pass over the tets, whose data is loaded (staged)
// once for all operands.
__device__ void apply_staged_dirs(const MixedArgs& a, float scale, unsigned char* smem) {
  staged_sweep(a, smem, nullptr, [&](const float* w, int TT, int tid) {
    const StagedTet e(w, TT, tid);
    tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, a.v_f, a.v_lo, a.q_f);
    for (int j = 0; j < a.nwarm; ++j)
      tet_apply(e.Re, e.b, e.c0, e.c1, e.c2, scale, e.nn, warm_dir(a, j), nullptr, a.wprod + size_t(j) * a.N);
  });
}
// dir_mask (batches; null: every mesh): the meshes whose tets also apply A
// to the search directions.
__device__ void apply_tets_dirs(const MixedArgs& a, float scale, const unsigned char* dir_mask) {
  const int T = a.T, TT = a.tile_tets, stride = gridDim.x * blockDim.x;
  int t = int(sweep_first());
  int4 ids = tile_node_ids(a, t);
  for (; t < T; t += stride) {
    const int4 cur = ids;
    ids = tile_node_ids(a, t + stride);
    const int nw = !dir_mask || dir_mask[a.mesh_of_tet[t]] ? a.nwarm : 0;
    const int tile = tile_of(t, a.tile_magic);
    const float* w = a.tile_f + size_t(tile) * kTileWords * TT + (t - tile * TT);
    const float4 quat = make_float4(w[4 * TT], w[5 * TT], w[6 * TT], w[7 * TT]);
    float b[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) b[k] = w[(8 + k) * TT];
    const float c0 = w[17 * TT], c1 = w[18 * TT], c2 = w[19 * TT];
    const int nn[4] = {cur.x, cur.y, cur.z, cur.w};
    for (int j = -1; j < nw; ++j) {
      float Re[9];
      quaternion_to_rotation(quat, Re);
      if (j < 0) tet_apply(Re, b, c0, c1, c2, scale, nn, a.v_f, a.v_lo, a.q_f);
      else tet_apply(Re, b, c0, c1, c2, scale, nn, warm_dir(a, j), nullptr, a.wprod + size_t(j) * a.N);
    }
  }
}

// One element-apply sweep with the mesh's variant.  `mask` (batched solves
// only, variants kApplyTets and kApplyStaged) selects the meshes whose tets
// take part.
template <typename R, bool AllowStream = true>
__device__ __forceinline__ void apply_sweep(const MixedArgs& a, const typename ApplyOps<R>::V4* u4,
                                            const typename ApplyOps<R>::V4* ulo, typename ApplyOps<R>::V4* q4,
                                            const R* re, const R* bb, const R* cc, R scale, unsigned char* smem,
                                            const unsigned char* mask = nullptr) {
  if constexpr (sizeof(R) == 4) {
    if (a.apply_variant == kApplyStaged) {
      apply_staged(a, u4, ulo, q4, scale, smem, mask);
      return;
    }
    if (a.apply_variant == kApplyTets || mask) {
      apply_tets_tiled<AllowStream>(a, u4, ulo, q4, scale, mask);
      return;
    }
  }
  if (a.apply_variant == kApplyTets || a.apply_variant == kApplyStaged || mask)
    apply_tets<R>(a, u4, ulo, q4, re, bb, cc, scale, mask);
  else if (a.apply_variant == kApplyGather) apply_patches_gather<R>(a, u4, ulo, q4, re, bb, cc, scale, smem);
  else apply_patches<R>(a, u4, ulo, q4, re, bb, cc, scale, smem);
}

// Projected start: A v (into q) and A W_j for every search direction
// (products into a.wprod).  Tets and staged variants do all operands in one
// pass; the patch variants sweep once per operand.  dir_mask (batches, tets
// variant): only the meshes it marks apply the directions (the staged
// variant applies them for every mesh).
template <bool AllowStream>
__device__ bool apply_start_operands(const MixedArgs& a, float scale, unsigned char* smem, unsigned& round,
                                     const unsigned char* dir_mask = nullptr) {
  if (a.apply_variant == kApplyStaged) {
    apply_staged_dirs(a, scale, smem);
    return true;
  }
  if (a.apply_variant == kApplyTets) {
    apply_tets_dirs(a, scale, dir_mask);
    return true;
  }
  apply_sweep<float, AllowStream>(a, a.v_f, a.v_lo, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem);
  for (int j = 0; j < a.nwarm; ++j) {
    if (!grid_barrier(a.sync, a.spin_limit, round)) return false;
    apply_sweep<float, AllowStream>(a, warm_dir(a, j), nullptr, a.wprod + size_t(j) * a.N, a.re_f, a.b_f, a.c_f, scale, smem);
  }
  return true;
}

// Phase stamps of the last mixed solve (the tracer CTA; SM clock cycles since the
// kernel started), after the trace rows: 0 b, 1 start sweeps, 2 start ready,
// 3 CG loop, 4 position update; 5-7 (projected and learned starts) Gram sums
// begun, Gram totals in, coefficients solved, else 0.
constexpr int kPhaseStamps = 8;
__device__ __forceinline__ void phase_stamp(const MixedArgs& a, int k, long long t_start) {
  a.trace[kTraceCols * kTraceRows + k] = double(cycles_now() - t_start);
}
__device__ __forceinline__ void clear_phase_stamps(const MixedArgs& a) {
  for (int k = 0; k < kPhaseStamps; ++k) a.trace[kTraceCols * kTraceRows + k] = 0.0;
}

// Grid sums of nv <= kMaxWarmSums values per free node (value m of node i:
// val(i, m)) for the projected start; every CTA receives the totals in
// tot[].  Each thread accumulates (hi, lo) pairs for chunks of 8 values,
// warp butterflies and the CTA sum follow, then FP64: atomic reductions
// into sync->wacc (zero at launch), or with a.ordered_sums per-CTA partials
// that every CTA adds up in CTA order.
template <typename Val>
__device__ bool grid_sum_wide(const MixedArgs& a, int nv, Val val, double* tot, unsigned& round) {
  constexpr int kWarps = kBlock / 32;
  __shared__ DF s_w[kWarps][kMaxWarmSums];
  __shared__ int s_ok;
  const long N = a.N, n0 = sweep_first(), gstride = (long)gridDim.x * blockDim.x;  // as the node passes
  const int warp = threadIdx.x >> 5;
  for (int c0 = 0; c0 < nv; c0 += 8) {
    DF acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = DF{0.f, 0.f};
    for (long i = n0; i < N; i += gstride) {
      if (a.fixed[i]) continue;
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (c0 + k < nv) acc[k] = df_add(acc[k], DF{val(i, c0 + k), 0.f});
    }
    DF x;
    const int k = warp_totals<DF, 8>(acc, x);
    if (k >= 0 && c0 + k < nv) s_w[warp][c0 + k] = x;
  }
  __syncthreads();
  // warp w: values w, w + kWarps, ... over the kWarps warp totals
  for (int m = warp; m < nv; m += kWarps) {
    const int lane = threadIdx.x & 31;
    DF t = lane < kWarps ? s_w[lane][m] : DF{0.f, 0.f};
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) t = df_add(t, AccOps<DF>::shfl_down(t, o));
    if (lane == 0) {
      const double d = AccOps<DF>::to_double(t);
      if (a.ordered_sums) a.wpart[size_t(m) * gridDim.x + blockIdx.x] = d;
      else atomicAdd(&a.sync->wacc[m][0], d);
    }
  }
  __syncthreads();
  ++round;
  if (threadIdx.x == 0) s_ok = sync_round(a.sync, round, a.spin_limit) ? 1 : 0;
  __syncthreads();
  const bool ok = s_ok != 0;
  if (ok) {
    for (int m = threadIdx.x; m < nv; m += blockDim.x) {
      if (a.ordered_sums) {
        double t = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) t += __ldcg(a.wpart + size_t(m) * gridDim.x + b);
        tot[m] = t;
      } else {
        tot[m] = __ldcg(&a.sync->wacc[m][0]);
      }
    }
  }
  __syncthreads();
  return ok;
}

// FP32 value of an FP64 number by bit manipulation: the exponent rebiased,
// the mantissa truncated to 23 bits (at most 1 ulp of FP32 low).  Integer
// instructions only: a conversion instruction would run on GB300's FP64 pipe.
// Magnitudes below the FP32 normal range become 0, above it infinity; NaN
// stays NaN.
__device__ __forceinline__ float f32_of_f64(double d) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(d));
  const unsigned sign = unsigned(u >> 32) & 0x80000000u;
  const int e = int((u >> 52) & 0x7ffu);
  const unsigned mant = unsigned(u >> 29) & 0x7fffffu;
  if (e == 0x7ff) return (u & 0xfffffffffffffull) != 0ull ? __uint_as_float(0x7fc00000u) : __uint_as_float(sign | 0x7f800000u);
  const int fe = e - 1023 + 127;
  if (fe <= 0) return __uint_as_float(sign);
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | (unsigned(fe) << 23) | mant);
}

// The projected start's coefficients: the least-energy point of v + span{W_j}
// solves G g = h with G_ij = W_i.A W_j and h_i = W_i.(b - A v).  `tot` holds
// G's upper triangle row by row, then h (FP64 sums).  The system is scaled to
// a unit diagonal and solved in FP32 by Gauss-Jordan elimination with the
// diagonal pivots in order (no FP64 instruction; the coefficients only
// choose where CG starts, and an error e in g costs e^T G e / 2 of the
// start's energy).  Directions are taken in order (the newest velocity
// change first); one whose A-norm is not positive and finite, or that lies
// (nearly) in the span of the ones before it (pivot, a Schur complement of
// the unit-diagonal G, below kWarmPivot), gets g_j = 0 and leaves the system.
constexpr float kWarmPivot = 1e-5f;

// One thread per system (the batch: one per mesh).
__device__ void warm_solve(const double* tot, int n, float* g) {
  float M[kMaxWarmDirs][kMaxWarmDirs + 1], sc[kMaxWarmDirs], piv[kMaxWarmDirs];
  bool live[kMaxWarmDirs];
  auto G = [&](int i, int j) {
    if (i > j) {
      const int t = i;
      i = j;
      j = t;
    }
    return f32_of_f64(tot[i * n - i * (i - 1) / 2 + (j - i)]);
  };
  const double* h = tot + n * (n + 1) / 2;
  for (int i = 0; i < n; ++i) {
    const float d = G(i, i), hv = f32_of_f64(h[i]);
    live[i] = d > 0.f && isfinite(d) && isfinite(hv);
    sc[i] = live[i] ? rsqrtf(d) : 0.f;
  }
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) M[i][j] = G(i, j) * sc[i] * sc[j];
    M[i][n] = f32_of_f64(h[i]) * sc[i];
  }
  for (int j = 0; j < n; ++j) {
    piv[j] = M[j][j];
    if (!live[j] || !(piv[j] > kWarmPivot)) {
      live[j] = false;
      continue;
    }
    for (int i = 0; i < n; ++i) {
      if (i == j) continue;
      const float f = M[i][j] / piv[j];
      for (int k = j + 1; k <= n; ++k) M[i][k] = fmaf(-f, M[j][k], M[i][k]);
    }
  }
  for (int i = 0; i < n; ++i) {
    const float x = M[i][n] / piv[i] * sc[i];
    g[i] = live[i] && isfinite(x) ? x : 0.f;
  }
}

// The same by one warp, for a system every CTA solves for itself: lane i
// owns row i of the augmented system [G | h] in shared memory, and each
// elimination step reads the pivot row from there.  The loops are left
// rolled: this code runs once per step, where every instruction is fetched
// cold, so its length, not its dependency chain, sets its time.  Called by
// the 32 lanes of one warp; g[j] is written for j < n.
__device__ void warm_solve_warp(const double* tot, int n, float* g) {
  constexpr unsigned kAll = 0xffffffffu;
  __shared__ float s_m[kMaxWarmDirs][kMaxWarmDirs + 1];
  __shared__ float s_sc[kMaxWarmDirs];
  const int lane = threadIdx.x & 31;
  const int n1 = n + 1, tri = n * (n + 1) / 2;
  bool live = false;
  if (lane < n) {
    const float d = f32_of_f64(tot[lane * n - lane * (lane - 1) / 2]), hv = f32_of_f64(tot[tri + lane]);
    live = d > 0.f && isfinite(d) && isfinite(hv);
    s_sc[lane] = live ? rsqrtf(d) : 0.f;
  }
  __syncwarp();
#pragma unroll 1
  for (int e = lane; e < n * n1; e += 32) {
    const int i = e / n1, j = e - i * n1;
    const int lo = min(i, j), hi = max(i, j);
    s_m[i][j] = j < n ? f32_of_f64(tot[lo * n - lo * (lo - 1) / 2 + (hi - lo)]) * s_sc[i] * s_sc[j]
                      : f32_of_f64(tot[tri + i]) * s_sc[i];
  }
  __syncwarp();
  float piv = 1.f;
#pragma unroll 1
  for (int j = 0; j < n; ++j) {
    const float pj = s_m[j][j];
    const bool use = __shfl_sync(kAll, live ? 1 : 0, j) != 0 && pj > kWarmPivot;
    if (lane == j) {
      live = use;
      piv = pj;
    }
    if (use && lane < n && lane != j) {
      const float f = s_m[lane][j] / pj;
#pragma unroll 1
      for (int k = j + 1; k <= n; ++k) s_m[lane][k] = fmaf(-f, s_m[j][k], s_m[lane][k]);
    }
    __syncwarp();
  }
  if (lane < n) {
    const float x = s_m[lane][n] / piv * s_sc[lane];
    g[lane] = live && isfinite(x) ? x : 0.f;
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

__device__ __forceinline__ void trace_row(const MixedArgs& a, int row, double rho, double pq, double alpha,
                                          double beta, const double* stamp, long long t_start) {
  if (row >= kTraceRows) return;
  double* tr = a.trace + kTraceCols * row;
  tr[0] = rho;
  tr[1] = pq;
  tr[2] = alpha;
  tr[3] = beta;
  for (int k = 0; k < 5; ++k) tr[4 + k] = stamp[k];
  tr[9] = double(cycles_now() - t_start);
}

// The elastic forces g of node i: its incident tets' corner forces in
// ascending tet order, summed as (hi, lo) pairs.  The incidence entries and
// then the forces are loaded eight at a time ahead of the sums, so that a
// node's ~24 dependent gathers overlap instead of queuing one L2 round trip
// after the other.
__device__ __forceinline__ void gather_forces(const MixedArgs& a, long i, DF (&g)[3]) {
  const int q0 = a.inc_ptr[i], q1 = a.inc_ptr[i + 1];
  for (int c = 0; c < 3; ++c) g[c] = DF{0.f, 0.f};
  for (int q = q0; q < q1; q += 8) {
    int e[8];
    float4 f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) e[k] = q + k < q1 ? a.inc_ent[q + k] : -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) f[k] = e[k] >= 0 ? a.g_f[4L * (e[k] >> 2) + (e[k] & 3)] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (e[k] < 0) break;
      df_inc(g[0].hi, g[0].lo, f[k].x);
      df_inc(g[1].hi, g[1].lo, f[k].y);
      df_inc(g[2].hi, g[2].lo, f[k].z);
    }
  }
}

// A W_j += diag W_j (the mass term) for the search directions of node i, four
// directions at a time: their loads are issued ahead of the stores (which the
// compiler may not move across, not knowing that they touch other
// directions), so they overlap.
__device__ __forceinline__ void add_mass_term(const MixedArgs& a, long i, float df) {
  const long N = a.N;
  for (int j0 = 0; j0 < a.nwarm; j0 += 4) {
    float4 w[4], aw[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k < a.nwarm) {
        w[k] = warm_dir(a, j0 + k)[i];
        aw[k] = load_acc(a.wprod + size_t(j0 + k) * N + i);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k < a.nwarm)
        a.wprod[size_t(j0 + k) * N + i] =
            make_float4(df * w[k].x + aw[k].x, df * w[k].y + aw[k].y, df * w[k].z + aw[k].z, 0.f);
    }
  }
}

// The start v + sum_j g_j W_j (two-sums into the (hi, lo) iterate) and its
// residual r - sum_j g_j A W_j at node i, directions in order, four loaded at
// a time.
__device__ __forceinline__ void move_to_start(const MixedArgs& a, long i, const float* gam, float4& vh, float4& vl,
                                              float (&rf)[3]) {
  const long N = a.N;
  for (int j0 = 0; j0 < a.nwarm; j0 += 4) {
    float4 w[4], aw[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k < a.nwarm && gam[j0 + k] != 0.f) {
        w[k] = warm_dir(a, j0 + k)[i];
        aw[k] = a.wprod[size_t(j0 + k) * N + i];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k >= a.nwarm) break;
      const float g = gam[j0 + k];
      if (g == 0.f) continue;
      df_inc(vh.x, vl.x, g * w[k].x);
      df_inc(vh.y, vl.y, g * w[k].y);
      df_inc(vh.z, vl.z, g * w[k].z);
      rf[0] -= g * aw[k].x;
      rf[1] -= g * aw[k].y;
      rf[2] -= g * aw[k].z;
    }
  }
}

// The velocity-change history as a difference basis: D_0 = the newest change,
// D_j = the j-th backward difference of the last changes (new D_j = new
// D_{j-1} - old D_{j-1}), kept as (hi, lo) float pairs.  The basis spans the
// same space as the last kMaxHistory changes, but for a smooth trajectory its
// vectors are far from parallel, so their Gram system stays well conditioned
// in FP32; the pairs keep the differences exact to ~1e-14 of each level.
__device__ __forceinline__ void record_velocity_change(const MixedArgs& a, long i, const DF (&dv)[3]) {
  const long N = a.N;
  float hi[3], lo[3];
  for (int c = 0; c < 3; ++c) {
    hi[c] = dv[c].hi;
    lo[c] = dv[c].lo;
  }
  // four levels at a time: their old values are loaded before any is
  // overwritten, so the loads overlap
  for (int j0 = 0; j0 < a.hist_rec; j0 += 4) {
    float4 oh[4], ol[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k < a.hist_rec) {
        oh[k] = a.hist[size_t(j0 + k) * N + i];
        ol[k] = a.hist[size_t(kMaxHistory + j0 + k) * N + i];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k >= a.hist_rec) break;
      a.hist[size_t(j0 + k) * N + i] = make_float4(hi[0], hi[1], hi[2], 1.f);
      a.hist[size_t(kMaxHistory + j0 + k) * N + i] = make_float4(lo[0], lo[1], lo[2], 0.f);
      // next level: this level's new value minus its old one
      const float ohc[3] = {oh[k].x, oh[k].y, oh[k].z}, olc[3] = {ol[k].x, ol[k].y, ol[k].z};
      for (int c = 0; c < 3; ++c) {
        const DF d = df_add(DF{hi[c], lo[c]}, DF{-ohc[c], -olc[c]});
        hi[c] = d.hi;
        lo[c] = d.lo;
      }
    }
  }
}

// Extrapolated start: v + D_0 + ... + D_{deg-1}, the polynomial of degree deg
// through the last deg + 1 velocities evaluated at the next step (Newton's
// backward-difference form: the next change is the sum of the newest
// change's backward differences), in (hi, lo) pairs from the stored levels.
__device__ __forceinline__ void extrapolate(const MixedArgs& a, long i, int deg, DF (&v)[3]) {
  const long N = a.N;
  for (int j0 = 0; j0 < deg; j0 += 4) {
    float4 h[4], l[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k < deg) {
        h[k] = a.hist[size_t(j0 + k) * N + i];
        l[k] = a.hist[size_t(kMaxHistory + j0 + k) * N + i];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (j0 + k >= deg) break;
      v[0] = df_add(v[0], DF{h[k].x, l[k].x});
      v[1] = df_add(v[1], DF{h[k].y, l[k].y});
      v[2] = df_add(v[2], DF{h[k].z, l[k].z});
    }
  }
}
// The degree the extrapolated start uses: at most the levels that hold
// differences of recorded steps.
__device__ __forceinline__ int extrap_degree(const MixedArgs& a) {
  if (a.extrap_k <= 0 || !a.hist_fill) return 0;
  const int fill = *a.hist_fill;
  return fill < a.extrap_k ? fill : a.extrap_k;
}
// One thread, after every CTA read the count: a step that recorded R levels
// leaves min(fill + 1, R) of them holding differences of recorded steps.
__device__ __forceinline__ void advance_fill(const MixedArgs& a) {
  if (!a.hist_fill || a.hist_rec <= 0) return;
  const int f = *a.hist_fill + 1;
  *a.hist_fill = f < a.hist_rec ? f : a.hist_rec;
}

__device__ __forceinline__ void finish_stats(const MixedArgs& a, int it, int applies, bool converged, double rho,
                                             double rho0, double bnorm2) {
  int st = ld_status(&a.sync->status);
  if (st == 0 && !converged) st = OTFEM_WARN_NOT_CONVERGED;
  a.stats->iterations = it;
  a.stats->applies = applies;
  a.stats->status = st;
  a.stats->rr = rho;
  a.stats->rr0 = rho0;
  a.stats->bb = bnorm2;
}

// r = b - (d v + q) of node i, rounded to FP32: the FP64 subtraction of the
// dynamics assembly (fem_dynamics_assembly.h:88-91) in (hi, lo) pairs, from
// the pairs of b and d the first phase stores.
__device__ __forceinline__ void node_residual(const MixedArgs& a, long i, float4 vh, float4 vl, float4 q4,
                                              float (&r)[3]) {
  const float4 bh = a.b_hi[i], bl = a.b_lo[i];
  const DF d{a.diag_f[i], a.diag_lo[i]};
  r[0] = residual_df(DF{bh.x, bl.x}, d, DF{vh.x, vl.x}, q4.x);
  r[1] = residual_df(DF{bh.y, bl.y}, d, DF{vh.y, vl.y}, q4.y);
  r[2] = residual_df(DF{bh.z, bl.z}, d, DF{vh.z, vl.z}, q4.z);
}

// K2, mixed precision (see the file comment).
__global__ void __launch_bounds__(kBlock, 1) k_cg_mixed(MixedArgs a) {
  const int N = a.N;
  // this thread's nodes (sweep_first); every node pass uses the same
  // mapping, so a node's data passes between phases within one thread
  const long n0 = sweep_first(), gstride = (long)gridDim.x * blockDim.x;
  const float scale = float(a.dt * a.dt);
  // dt and 1 + dt alpha as (hi, lo) pairs
  const DF dt2[2] = {df_of(a.dt), df_add(DF{1.f, 0.f}, df_mul2(df_of(a.dt), df_of(a.alpha)))};
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  unsigned round = 0;  // grid barriers and reductions passed so far
  extern __shared__ __align__(16) unsigned char smem[];  // patch staging of the apply
  const bool tracer = is_tracer();
  const long long t_start = tracer ? cycles_now() : 0ll;
  if (tracer) clear_phase_stamps(a);
  __shared__ double stamp[6];  // trace stamps, written by the tracer thread only

  // Phase 0: b = M v + dt (f_ext - g), g = the elastic forces gathered in
  // ascending tet order and summed as (hi, lo) pairs; the diagonal
  // M(1 + dt*alpha) of fem_dynamics_assembly.h:84-85; v split into (hi, lo).
  DF bbsum[1] = {{0.f, 0.f}};
  const int deg = extrap_degree(a);
  for (long i = n0; i < N; i += gstride) {
    DF g[3];
    gather_forces(a, i, g);
    // in (hi, lo) pairs: no FP64 instruction
    const bool fx = a.fixed[i] != 0;
    const DF m = df_of(a.mass[i]);
    const DF vi[3] = {df_of(a.v[3 * i]), df_of(a.v[3 * i + 1]), df_of(a.v[3 * i + 2])};
    float sp = 0.f;
    if (!fx) {
      DF b3[3];
      for (int c = 0; c < 3; ++c) {
        b3[c] = df_add(df_mul2(m, vi[c]), df_mul2(dt2[0], df_add(df_of(a.fext[3 * i + c]), df_neg(g[c]))));
        a.bvec[3 * i + c] = f64_of(b3[c]);
      }
      a.b_hi[i] = make_float4(b3[0].hi, b3[1].hi, b3[2].hi, 0.f);
      a.b_lo[i] = make_float4(b3[0].lo, b3[1].lo, b3[2].lo, 0.f);
      float bf[3] = {b3[0].hi + b3[0].lo, b3[1].hi + b3[1].lo, b3[2].hi + b3[2].lo};
      bbsum[0] = df_add(bbsum[0], DF{bf[0] * bf[0] + bf[1] * bf[1] + bf[2] * bf[2], 0.f});
      const DF dg = df_mul2(m, dt2[1]);  // m (1 + dt alpha)
      a.diag[i] = f64_of(dg);
      a.diag_f[i] = dg.hi;
      a.diag_lo[i] = dg.lo;
      sp = a.precond ? 1.f / (dg.hi + scale * dfbits::trunc_f32(a.node_k[i])) : 1.f;
    } else {
      a.diag[i] = 0.0;
      a.diag_f[i] = 0.f;
      a.diag_lo[i] = 0.f;
    }
    // r.w carries the node's preconditioner scalar through the solve
    a.r_f[i] = make_float4(0.f, 0.f, 0.f, sp);
    // fixed columns keep their velocity in the initial residual (the reference
    // multiplies A_ij by the fixed node's m_velocity); rows of fixed nodes are
    // never accumulated (w = 0).  The extrapolated start moves free nodes'
    // iterates (b above keeps m v).
    DF v0[3] = {vi[0], vi[1], vi[2]};
    if (deg > 0 && !fx) extrapolate(a, i, deg, v0);
    a.v_f[i] = make_float4(v0[0].hi, v0[1].hi, v0[2].hi, fx ? 0.f : 1.f);
    a.v_lo[i] = make_float4(v0[0].lo, v0[1].lo, v0[2].lo, 0.f);
    a.q_f[i] = zero4;
    if (a.nwarm) {
      // learned start: the network's correction c = its dv - dv_prev is the
      // last search direction
      if (a.nwarm > a.hist_k) {
        const float4 d = fx ? zero4 : a.dv_last[i], w = fx ? zero4 : a.warm_dv[i];
        a.wprod[size_t(kMaxWarmDirs) * N + i] = make_float4(w.x - d.x, w.y - d.y, w.z - d.z, fx ? 0.f : 1.f);
      }
      for (int j = 0; j < a.nwarm; ++j) a.wprod[size_t(j) * N + i] = zero4;
    }
  }
  // The loop's scalars are FP32 (pairs inside the reductions): no FP64
  // instruction sits between two phases of an iteration.  |b|^2 is first
  // needed at the convergence test after the start, so its sums ride along
  // with the start's |r|^2 reduction; here a barrier suffices (the sweep
  // gathers the operand of other CTAs' nodes).
  if (!grid_barrier(a.sync, a.spin_limit, round)) return;
  if (tracer) phase_stamp(a, 0, t_start);

  // Initial residual r = b - A v (FP64), p = S r.  Projected and learned
  // starts: also A W_j for the search directions W_j, and the start moves to
  // the least-energy point v + sum_j g_j W_j (warm_solve), whose residual is
  // r - sum_j g_j A W_j.
  int applies = 1;
  if (a.nwarm) {
    if (!apply_start_operands<false>(a, scale, smem, round)) return;
    applies += a.nwarm;
  } else {
    apply_sweep<float, false>(a, a.v_f, a.v_lo, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem);
  }
  if (!grid_barrier(a.sync, a.spin_limit, round)) return;
  if (tracer) phase_stamp(a, 1, t_start);
  __shared__ float s_gam[kMaxWarmDirs];
  if (a.nwarm) {
    const int nw = a.nwarm;
    // r = b - A v; A W_j += diag W_j (the mass term)
    for (long i = n0; i < N; i += gstride) {
      if (a.fixed[i]) continue;
      const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
      float rf[3];
      node_residual(a, i, vh, vl, q4, rf);
      a.r_f[i] = make_float4(rf[0], rf[1], rf[2], a.r_f[i].w);
      add_mass_term(a, i, a.diag_f[i]);
    }
    // Gram system: W_i.A W_j (i <= j) row by row, then W_i.r
    __shared__ signed char s_pi[kMaxWarmSums], s_pj[kMaxWarmSums];
    __shared__ double s_tot[kMaxWarmSums];
    if (threadIdx.x == 0) {
      int m = 0;
      for (int i = 0; i < nw; ++i)
        for (int j = i; j < nw; ++j, ++m) s_pi[m] = (signed char)i, s_pj[m] = (signed char)j;
      for (int i = 0; i < nw; ++i, ++m) s_pi[m] = (signed char)i, s_pj[m] = -1;
    }
    __syncthreads();
    const int nv = nw * (nw + 1) / 2 + nw;
    auto gram = [&](long i, int m) -> float {
      const float4 w = warm_dir(a, s_pi[m])[i];
      const float4 q = s_pj[m] >= 0 ? a.wprod[size_t(s_pj[m]) * N + i] : a.r_f[i];
      return w.x * q.x + w.y * q.y + w.z * q.z;
    };
    if (tracer) phase_stamp(a, 5, t_start);
    if (!grid_sum_wide(a, nv, gram, s_tot, round)) return;
    if (tracer) phase_stamp(a, 6, t_start);
    if (threadIdx.x < 32) warm_solve_warp(s_tot, nw, s_gam);
    if (tracer) phase_stamp(a, 7, t_start);
    __syncthreads();
  }
  DF rr[1] = {{0.f, 0.f}};
  for (long i = n0; i < N; i += gstride) {
    if (a.fixed[i]) {
      a.p_f[i] = zero4;
      a.r_f[i] = zero4;
      continue;
    }
    const float sp = a.r_f[i].w;
    float rf[3];
    if (a.nwarm) {
      // v += sum_j g_j W_j (exact two-sums); r -= sum_j g_j A W_j
      const float4 r4 = a.r_f[i];
      float4 vh = a.v_f[i], vl = a.v_lo[i];
      rf[0] = r4.x;
      rf[1] = r4.y;
      rf[2] = r4.z;
      move_to_start(a, i, s_gam, vh, vl, rf);
      a.v_f[i] = vh;
      a.v_lo[i] = vl;
    } else {
      const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
      node_residual(a, i, vh, vl, q4, rf);
    }
    a.r_f[i] = make_float4(rf[0], rf[1], rf[2], sp);
    a.p_f[i] = make_float4(sp * rf[0], sp * rf[1], sp * rf[2], 1.f);  // p = z = S r
    a.q_f[i] = zero4;
    a.v_keep[i] = a.v_f[i];  // the start is the first kept iterate
    a.v_keep[N + i] = a.v_lo[i];
    rr[0] = df_add(rr[0], DF{rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2], 0.f});
  }
  float tot[2];
  {
    const DF sums[2] = {rr[0], bbsum[0]};
    if (!grid_reduce_df<2, 2>(a, sums, tot, round, FinIdentityF2())) return;
  }
  if (tracer) phase_stamp(a, 2, t_start);
  const float bnorm2 = tot[1];
  const float thresh = float(a.rtol * a.rtol) * bnorm2;
  float rho = tot[0];
  const float rho0 = rho;
  int it = 0;
  int best_buf = 0;      // kept iterate with the smallest true residual
  bool stalled = false;  // stopped at the precision floor: return the kept iterate
  bool converged = rho <= thresh;
  // recurrence check and restarts (FinPcgF); stagnation of the
  // true residual at the refreshes ends the solve unconverged
  float prev_est = -1.f, best_true = rho0;
  bool restart = false;
  int stalls = 0;

  // With at most one node per thread (N <= threads), the thread's node values
  // that the sweep does not change (p, r, the diagonal, v) are loaded before
  // the barrier after the sweep and stay in registers until the update.
  const bool one_node = long(N) <= gstride;
  auto node_dots = [&](const float4& q4, const float4& p4, const float4& r4, float d, DF (&s7)[7]) {
    const float qx = d * p4.x + q4.x, qy = d * p4.y + q4.y, qz = d * p4.z + q4.z;
    const float rq = r4.x * qx + r4.y * qy + r4.z * qz, qq = qx * qx + qy * qy + qz * qz;
    const float rr2 = r4.x * r4.x + r4.y * r4.y + r4.z * r4.z, sp = r4.w;
    s7[0] = df_add(s7[0], DF{p4.x * qx + p4.y * qy + p4.z * qz, 0.f});
    s7[1] = df_add(s7[1], DF{sp * rq, 0.f});
    s7[2] = df_add(s7[2], DF{sp * qq, 0.f});
    s7[3] = df_add(s7[3], DF{sp * rr2, 0.f});
    s7[4] = df_add(s7[4], DF{rq, 0.f});
    s7[5] = df_add(s7[5], DF{qq, 0.f});
    s7[6] = df_add(s7[6], DF{rr2, 0.f});
  };
  auto node_update = [&](long i, const float4& q4, const float4& p4, const float4& r4, float d, float4 vh, float4 vl,
                         float alpha, float beta) {
    const float qx = d * p4.x + q4.x, qy = d * p4.y + q4.y, qz = d * p4.z + q4.z;
    df_inc(vh.x, vl.x, alpha * p4.x);
    df_inc(vh.y, vl.y, alpha * p4.y);
    df_inc(vh.z, vl.z, alpha * p4.z);
    const float rx = r4.x - alpha * qx, ry = r4.y - alpha * qy, rz = r4.z - alpha * qz;
    const float sp = r4.w;
    a.v_f[i] = vh;
    a.v_lo[i] = vl;
    a.r_f[i] = make_float4(rx, ry, rz, sp);
    a.p_f[i] = make_float4(sp * rx + beta * p4.x, sp * ry + beta * p4.y, sp * rz + beta * p4.z, 1.f);
    a.q_f[i] = zero4;
  };

  while (!converged && it < a.max_it) {
    // q += dt^2 K' p
    apply_sweep<float, false>(a, a.p_f, nullptr, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem);
    ++applies;
    if (tracer) stamp[0] = double(cycles_now() - t_start);
    const bool mine = one_node && n0 < N && !a.fixed[n0];
    float4 np4 = zero4, nr4 = zero4, nq4 = zero4, nvh = zero4, nvl = zero4;
    float nd = 0.f;
    if (mine) {
      np4 = a.p_f[n0];
      nr4 = a.r_f[n0];
      nd = a.diag_f[n0];
      nvh = a.v_f[n0];
      nvl = a.v_lo[n0];
    }
    if (!grid_barrier(a.sync, a.spin_limit, round)) return;
    if (tracer) stamp[1] = double(cycles_now() - t_start);
    // q = diag p + q; the totals of FinPcgF (r.w = the node's scalar s)
    DF s7[7] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (one_node) {
      if (mine) {
        nq4 = load_acc(a.q_f + n0);
        node_dots(nq4, np4, nr4, nd, s7);
      }
    } else {
      for (long i = n0; i < N; i += gstride) {
        if (a.fixed[i]) continue;
        node_dots(load_acc(a.q_f + i), a.p_f[i], a.r_f[i], a.diag_f[i], s7);
      }
    }
    if (tracer) stamp[2] = double(cycles_now() - t_start);
    float sc[5];
    if (!grid_reduce_df<7, 5>(a, s7, sc, round, FinPcgF{prev_est, restart})) return;
    prev_est = sc[4];
    restart = false;
    if (tracer) stamp[3] = double(cycles_now() - t_start);
    if (sc[3] != 0.f) {
      // 1: NaN/Inf in the system (e.g. a non-finite force), an error;
      // 2: finite breakdown (p.Ap <= 0 from rounding at the precision
      // floor): stop, the step reports OTFEM_WARN_NOT_CONVERGED
      if (sc[3] == 1.f && blockIdx.x == 0 && threadIdx.x == 0)
        atomicCAS(&a.sync->status, 0, OTFEM_ERR_NONFINITE);
      break;
    }
    const float alpha = sc[0], beta = sc[1];
    const int row = it;
    ++it;
    if (one_node) {
      if (mine) node_update(n0, nq4, np4, nr4, nd, nvh, nvl, alpha, beta);
    } else {
      for (long i = n0; i < N; i += gstride) {
        if (a.fixed[i]) continue;
        node_update(i, load_acc(a.q_f + i), a.p_f[i], a.r_f[i], a.diag_f[i], a.v_f[i], a.v_lo[i], alpha, beta);
      }
    }
    if (tracer) stamp[4] = double(cycles_now() - t_start);
    // The exact r.r of the new r comes with the next reduction; here the
    // update needs only a barrier (p must be complete before the next
    // apply).  The estimate of the new r.r triggers the residual recompute,
    // which alone declares convergence.
    const bool periodic = a.refresh > 0 && it % a.refresh == 0;
    const bool refresh_now = periodic || sc[2] <= thresh;
    if (!grid_barrier(a.sync, a.spin_limit, round)) return;
    if (tracer) trace_row(a, row, rho, 0.0, sc[0], sc[1], stamp, t_start);
    rho = sc[2];
    if (refresh_now) {
      // r = b - A v (residual replacement, FP64); q is zero here and the
      // (hi, lo) velocity is the apply operand.
      apply_sweep<float, false>(a, a.v_f, a.v_lo, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem);
      ++applies;
      if (!grid_barrier(a.sync, a.spin_limit, round)) return;
      DF tr[1] = {{0.f, 0.f}};
      const long cand = 2L * (best_buf ^ 1) * N;  // the kept copy that is not the best
      for (long i = n0; i < N; i += gstride) {
        if (a.fixed[i]) continue;
        const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
        float rr3[3];
        node_residual(a, i, vh, vl, q4, rr3);
        const float rx = rr3[0], ry = rr3[1], rz = rr3[2];
        a.r_f[i] = make_float4(rx, ry, rz, a.r_f[i].w);
        a.q_f[i] = zero4;
        a.v_keep[cand + i] = vh;
        a.v_keep[cand + N + i] = vl;
        tr[0] = df_add(tr[0], DF{rx * rx + ry * ry + rz * rz, 0.f});
      }
      float tt[1];
      if (!grid_reduce_df<1, 1>(a, tr, tt, round, FinIdentityF1())) return;
      // the true residual well above the recursive one: the recurrence has
      // decoupled from the system, restart the direction
      restart = tt[0] > 4.f * sc[2];
      prev_est = -1.f;
      rho = tt[0];
      // stagnation is judged at the periodic refreshes only (16 iterations
      // apart), not at the convergence checks in between
      if (rho < best_true) {
        best_true = rho;
        best_buf ^= 1;
        stalls = 0;
      } else if ((periodic || a.refresh <= 0) && ++stalls >= 3) {
        stalled = true;  // at the precision floor: no progress over three periods
        rho = best_true;
        break;
      }
    }
    converged = rho <= thresh;
  }

  if (tracer) phase_stamp(a, 3, t_start);
  // v back to FP64 (the kept best iterate when stopped at the floor);
  // position_update (fem_position_update.h:25-39); the velocity change is
  // kept for the warm starts
  for (long i = n0; i < N; i += gstride) {
    if (a.fixed[i]) continue;
    const long kb = 2L * best_buf * N;
    float4 vh = stalled ? a.v_keep[kb + i] : a.v_f[i], vl = stalled ? a.v_keep[kb + N + i] : a.v_lo[i];
    // in pairs, with one FP64 addition per coordinate (x keeps its 53 bits)
    const DF v3[3] = {{vh.x, vl.x}, {vh.y, vl.y}, {vh.z, vl.z}};
    DF dv[3];
    for (int c = 0; c < 3; ++c) {
      dv[c] = df_add(v3[c], df_neg(df_of(a.v[3 * i + c])));
      a.v[3 * i + c] = f64_of(v3[c]);
      a.x[3 * i + c] += f64_of(df_mul2(v3[c], dt2[0]));
    }
    a.dv_last[i] = make_float4(dv[0].hi, dv[1].hi, dv[2].hi, 0.f);
    if (a.hist) record_velocity_change(a, i, dv);
  }
  if (tracer) phase_stamp(a, 4, t_start);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    finish_stats(a, it, applies, converged, rho, rho0, bnorm2);
    advance_fill(a);
  }
}

// K2, FP64 solver: every vector and reduction in FP64.
__global__ void __launch_bounds__(kBlock, 1) k_cg_fp64(MixedArgs a) {
  typedef double4 V4;
  const int N = a.N;
  // this thread's nodes (sweep_first); every node pass uses the same
  // mapping, so a node's data passes between phases within one thread
  const long n0 = sweep_first(), gstride = (long)gridDim.x * blockDim.x;
  V4* pv = a.p_d;
  V4* vv = a.v_d;
  V4* qv = a.q_d;
  const double scale = a.dt * a.dt;
  const V4 zero4 = make_double4(0.0, 0.0, 0.0, 0.0);
  unsigned round = 0;
  extern __shared__ __align__(16) unsigned char smem[];
  const bool tracer = is_tracer();
  const long long t_start = tracer ? cycles_now() : 0ll;
  __shared__ double stamp[6];

  double bbsum[1] = {0.0};
  for (long i = n0; i < N; i += gstride) {
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
    vv[i] = make_double4(vi[0], vi[1], vi[2], fx ? 0.0 : 1.0);
    qv[i] = zero4;
  }
  double tot[1];
  if (!grid_reduce<double, 1, 1>(a, bbsum, tot, round, FinIdentity1())) return;
  const double bnorm2 = tot[0];
  const double thresh = a.rtol * a.rtol * bnorm2;

  apply_sweep<double>(a, vv, nullptr, qv, a.re_d, a.b_d, a.c_d, scale, smem);
  if (!grid_barrier(a.sync, a.spin_limit, round)) return;
  double rr[2] = {0.0, 0.0};
  for (long i = n0; i < N; i += gstride) {
    if (a.fixed[i]) {
      pv[i] = zero4;
      for (int c = 0; c < 3; ++c) a.p[3 * i + c] = 0.0, a.r[3 * i + c] = 0.0;
      continue;
    }
    V4 q4 = load_acc(qv + i);
    double qa[3] = {q4.x, q4.y, q4.z};
    double d = a.diag[i];
    const double sp = jacobi_scale(a, i, d);
    double ri[3];
    for (int c = 0; c < 3; ++c) ri[c] = a.bvec[3 * i + c] - (d * a.v[3 * i + c] + qa[c]);
    for (int c = 0; c < 3; ++c) a.r[3 * i + c] = ri[c], a.p[3 * i + c] = sp * ri[c];  // p = z = S r
    pv[i] = make_double4(sp * ri[0], sp * ri[1], sp * ri[2], 1.0);
    qv[i] = zero4;
    const double r2 = ri[0] * ri[0] + ri[1] * ri[1] + ri[2] * ri[2];
    rr[0] += r2;
    rr[1] += sp * r2;
  }
  double tot2[2];
  if (!grid_reduce<double, 2, 2>(a, rr, tot2, round, FinIdentity2())) return;
  double rho = tot2[0], rz = tot2[1];
  const double rho0 = rho;
  int it = 0, applies = 1;
  bool converged = rho <= thresh;

  while (!converged && it < a.max_it) {
    apply_sweep<double>(a, pv, nullptr, qv, a.re_d, a.b_d, a.c_d, scale, smem);
    ++applies;
    if (tracer) stamp[0] = double(cycles_now() - t_start);
    if (!grid_barrier(a.sync, a.spin_limit, round)) return;
    if (tracer) stamp[1] = double(cycles_now() - t_start);
    double s5[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (long i = n0; i < N; i += gstride) {
      if (a.fixed[i]) continue;
      V4 q4 = load_acc(qv + i);
      double d = a.diag[i];
      double qi[3] = {d * a.p[3 * i] + q4.x, d * a.p[3 * i + 1] + q4.y, d * a.p[3 * i + 2] + q4.z};
      double pq = 0.0, rq = 0.0, qq = 0.0;
      for (int c = 0; c < 3; ++c) {
        pq += a.p[3 * i + c] * qi[c];
        rq += a.r[3 * i + c] * qi[c];
        qq += qi[c] * qi[c];
      }
      const double sp = jacobi_scale(a, i, d);
      s5[0] += pq;
      s5[1] += sp * rq;
      s5[2] += sp * qq;
      s5[3] += rq;
      s5[4] += qq;
    }
    if (tracer) stamp[2] = double(cycles_now() - t_start);
    double sc[4];
    if (!grid_reduce<double, 5, 4>(a, s5, sc, round, FinPcgFp64{rz, rho})) return;
    if (tracer) stamp[3] = double(cycles_now() - t_start);
    if (sc[3] != 0.0) {
      if (sc[3] == 1.0 && blockIdx.x == 0 && threadIdx.x == 0)
        atomicCAS(&a.sync->status, 0, OTFEM_ERR_NONFINITE);
      break;
    }
    const double alpha = sc[0], beta = sc[1];
    const int row = it;
    ++it;
    double rn[2] = {0.0, 0.0};
    for (long i = n0; i < N; i += gstride) {
      if (a.fixed[i]) continue;
      V4 q4 = load_acc(qv + i);
      double d = a.diag[i];
      const double sp = jacobi_scale(a, i, d);
      double pn[3], vn[3];
      const double qq[3] = {q4.x, q4.y, q4.z};
      for (int c = 0; c < 3; ++c) {
        double pi = a.p[3 * i + c];
        double qi = d * pi + qq[c];
        vn[c] = a.v[3 * i + c] + alpha * pi;
        double ri = a.r[3 * i + c] - alpha * qi;
        a.v[3 * i + c] = vn[c];
        a.r[3 * i + c] = ri;
        rn[0] += ri * ri;
        rn[1] += sp * ri * ri;
        pn[c] = sp * ri + beta * pi;
        a.p[3 * i + c] = pn[c];
      }
      pv[i] = make_double4(pn[0], pn[1], pn[2], 1.0);
      vv[i] = make_double4(vn[0], vn[1], vn[2], 1.0);
      qv[i] = zero4;
    }
    if (tracer) stamp[4] = double(cycles_now() - t_start);
    if (!grid_reduce<double, 2, 2>(a, rn, tot2, round, FinIdentity2())) return;
    if (tracer) trace_row(a, row, rho, 0.0, alpha, beta, stamp, t_start);
    rho = tot2[0];
    rz = tot2[1];
    if ((a.refresh > 0 && it % a.refresh == 0) || rho <= thresh) {
      apply_sweep<double>(a, vv, nullptr, qv, a.re_d, a.b_d, a.c_d, scale, smem);
      ++applies;
      if (!grid_barrier(a.sync, a.spin_limit, round)) return;
      double tr[2] = {0.0, 0.0};
      for (long i = n0; i < N; i += gstride) {
        if (a.fixed[i]) continue;
        V4 q4 = load_acc(qv + i);
        double d = a.diag[i];
        const double sp = jacobi_scale(a, i, d);
        const double qa[3] = {q4.x, q4.y, q4.z};
        for (int c = 0; c < 3; ++c) {
          double ri = a.bvec[3 * i + c] - (d * a.v[3 * i + c] + qa[c]);
          a.r[3 * i + c] = ri;
          tr[0] += ri * ri;
          tr[1] += sp * ri * ri;
        }
        qv[i] = zero4;
      }
      if (!grid_reduce<double, 2, 2>(a, tr, tot2, round, FinIdentity2())) return;
      rho = tot2[0];
      rz = tot2[1];
    }
    converged = rho <= thresh;
  }
  for (long i = n0; i < N; i += gstride) {
    if (a.fixed[i]) continue;
    for (int c = 0; c < 3; ++c) a.x[3 * i + c] += a.v[3 * i + c] * a.dt;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) finish_stats(a, it, applies, converged, rho, rho0, bnorm2);
}

// ---- batched solve -------------------------------------------------------
// Every mesh of a batch runs its own CG (own alpha, beta, residuals,
// recurrence checks and convergence) in lock-step with the others inside one
// persistent launch: the apply and node phases skip the meshes that are not
// in the current sweep (masks), the grid sums are per mesh, and the last CTA
// to arrive at a reduction updates the scalars of all meshes at once (one
// thread per mesh).  Node phases walk one contiguous node range per warp, so
// a warp meets each mesh boundary at most once and adds its per-mesh sums
// with one FP64 atomic per value and mesh (the batch's per-mesh sums).

constexpr int kMaskApply = 0, kMaskUpdate = 1, kMaskRefresh = 2;
constexpr int kBatchSlots = 8;  // accumulators per mesh and round

struct NodeRange {
  long beg, end;
};
__device__ __forceinline__ NodeRange warp_node_range(int N) {
  const long nw = (long)gridDim.x * (blockDim.x >> 5);
  const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long chunk = ((N + nw - 1) / nw + 31) / 32 * 32;
  NodeRange r;
  r.beg = w * chunk < N ? w * chunk : N;
  r.end = r.beg + chunk < N ? r.beg + chunk : N;
  return r;
}

// Walks the nodes of the meshes selected by `mask` in contiguous chunks per
// warp, 32 lanes at a time, calling fn(valid, i, m) on every lane with the
// node i and its mesh m (used only where valid); the mesh ids grow along each
// warp's walk.  With at most kBlock meshes the walk covers the selected
// meshes' nodes only (masked_meshes), so that a pass late in a step, when a
// few meshes still iterate, costs in proportion to their nodes; otherwise it
// reads the mesh of every node of the batch.
template <typename Fn>
__device__ __forceinline__ void masked_node_walk(const MixedArgs& a, const unsigned char* mask, Fn fn) {
  const int lane = threadIdx.x & 31;
  if (a.num_meshes <= kBlock && blockDim.x == kBlock) {
    const MeshList L = masked_meshes(a, a.mesh_node_start, mask);
    const NodeRange vr = warp_node_range(L.total);
    // the lane's list entry: searched once, then advanced as the walk
    // passes mesh boundaries
    int j = vr.beg + lane < vr.end ? L.entry(int(vr.beg + lane)) : 0;
    for (long base = vr.beg; base < vr.end; base += 32) {
      const long v = base + lane;
      const bool valid = v < vr.end;
      long i = 0;
      int m = -1;
      if (valid) {
        while (j + 1 < L.n && L.pref[j + 1] <= v) ++j;
        m = L.mesh[j];
        i = L.beg[j] + (v - L.pref[j]);
      }
      fn(valid, i, m);
    }
  } else {
    const NodeRange nr = warp_node_range(a.N);
    for (long base = nr.beg; base < nr.end; base += 32) {
      const long i = base + lane;
      const int m = i < nr.end ? a.mesh_of_node[i] : -1;
      fn(i < nr.end && mask[m], i, m);
    }
  }
}

// Running per-mesh sums of a warp (mesh ids are non-decreasing along nodes).
template <int NV, int Stride = kBatchSlots>
struct SegSum {
  int cur;  // uniform across the warp; -1: none yet
  DF acc[NV];
  __device__ __forceinline__ void start(int mesh) {
    cur = mesh;
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = DF{0.f, 0.f};
  }
  __device__ __forceinline__ void flush(double* acc_half) {
    DF x;
    const int k = warp_totals<DF, NV>(acc, x);
    if (k >= 0 && cur >= 0) atomicAdd(&acc_half[Stride * cur + k], AccOps<DF>::to_double(x));
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = DF{0.f, 0.f};
  }
  // adds each valid lane's values to the sums of its mesh m (m >= cur)
  __device__ __forceinline__ void add(bool valid, int m, const float (&v)[NV], double* acc_half) {
    if (valid && m == cur) {
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = df_add(acc[k], DF{v[k], 0.f});
    }
    unsigned rest = __ballot_sync(0xffffffffu, valid && m != cur);
    while (rest) {
      flush(acc_half);
      cur = __shfl_sync(0xffffffffu, m, __ffs(rest) - 1);
      if (valid && m == cur) {
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = df_add(acc[k], DF{v[k], 0.f});
      }
      rest = __ballot_sync(0xffffffffu, valid && m > cur);
    }
  }
};

// Grid barrier whose last CTA runs fin(a, mesh, totals[kBatchSlots], counts) for
// every mesh (totals: this round's accumulators, which it clears afterwards)
// and publishes the first two of the 4 integer counts the finisher
// accumulates (e.g. meshes still active, each at most 65,535 here) in the
// word that releases the round, so that the other CTAs read them with the
// release instead of after it.
template <typename Fin>
__device__ bool batch_reduce(const MixedArgs& a, unsigned& round, Fin fin, int (&counts)[4]) {
  __shared__ int s_flag;
  __shared__ int s_cnt[4];
  ++round;
  const int half = int(round & 1u);
  __syncthreads();
  if (threadIdx.x == 0) {
    // 2: last CTA, 1: wait for the release (0 once the wait failed); an
    // error recorded earlier ends the wait or the next synchronisation
    s_flag = arrive(a.sync, round) ? 2 : 1;
  }
  if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  if (s_flag == 2) {
    double* acc = a.bacc + size_t(half) * a.num_meshes * kBatchSlots;
    for (int m = threadIdx.x; m < a.num_meshes; m += blockDim.x) {
      double t[kBatchSlots];
#pragma unroll
      for (int k = 0; k < kBatchSlots; ++k) t[k] = __ldcg(acc + kBatchSlots * m + k);
      fin(a, m, t, s_cnt);
#pragma unroll
      for (int k = 0; k < kBatchSlots; ++k) acc[kBatchSlots * m + k] = 0.0;  // for round r + 2
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      clear_stale_acc(a.sync, round);
      const unsigned long long packed =
          (unsigned long long)min(s_cnt[0], 0xFFFF) | ((unsigned long long)min(s_cnt[1], 0xFFFF) << 16);
      const unsigned long long word = (unsigned long long)round | (packed << 32);
      asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(&a.sync->gen), "l"(word) : "memory");
    }
  } else if (threadIdx.x == 0 && s_flag == 1) {
    // wait for the release of this round; the counts come with it
    const long long start = clock64();
    unsigned polls = 0;
    int ok = 1;
    for (;;) {
      unsigned long long w;
      asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(&a.sync->gen) : "memory");
      if (int(unsigned(w) - round) >= 0) {
        s_cnt[0] = int((w >> 32) & 0xFFFFull);
        s_cnt[1] = int((w >> 48) & 0xFFFFull);
        break;
      }
      if ((++polls & 63u) == 0u && ld_status(&a.sync->status) != 0) {
        ok = 0;
        break;
      }
      if (clock64() - start > a.spin_limit) {
        atomicCAS(&a.sync->status, 0, OTFEM_ERR_TIMEOUT);
        ok = 0;
        break;
      }
    }
    s_flag = ok;
  }
  __syncthreads();
  const bool good = s_flag != 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) counts[k] = s_cnt[k];
  __syncthreads();
  return good;
}

// totals: |b|^2 of the free rows
struct FinBatchInit {
  __device__ void operator()(const MixedArgs& a, int m, const double* t, int* cnt) const {
    BatchMesh& b = a.bm[m];
    b.bnorm2 = t[0];
    b.thresh = float(a.rtol * a.rtol * t[0]);
  }
};

// projected / learned start: each mesh's Gram system (a.wbacc), solved per mesh
struct FinBatchGram {
  __device__ void operator()(const MixedArgs& a, int m, const double* t, int* cnt) const {
    warm_solve(a.wbacc + size_t(m) * kMaxWarmSums, a.nwarm, a.bm[m].wgam);
  }
};

// totals: |r0|^2 of the initial guess
struct FinBatchStart {
  __device__ void operator()(const MixedArgs& a, int m, const double* t, int* cnt) const {
    BatchMesh& b = a.bm[m];
    b.rho = b.rho0 = b.best_true = t[0];
    b.est = float(t[0]);
    b.prev_est = -1.f;
    b.restart = b.stalls = b.iterations = 0;
    b.best_buf = 0;
    b.stalled = 0;
    b.applies = 1 + a.nwarm;
    b.status = isfinite(t[0]) && isfinite(b.bnorm2) ? 0 : OTFEM_ERR_NONFINITE;
    b.converged = b.status == 0 && t[0] <= b.thresh;
    b.active = b.status == 0 && !b.converged && a.max_it > 0;
    unsigned char* mk = a.bmask;
    mk[kMaskApply * a.num_meshes + m] = b.active;
    mk[kMaskUpdate * a.num_meshes + m] = 0;
    mk[kMaskRefresh * a.num_meshes + m] = 0;
    if (b.active) atomicAdd(&cnt[0], 1);
  }
};

// totals: those of FinPcgF for the meshes in the sweep
struct FinBatchIter {
  __device__ void operator()(const MixedArgs& a, int m, const double* t, int* cnt) const {
    BatchMesh& b = a.bm[m];
    unsigned char* mk = a.bmask;
    const int M = a.num_meshes;
    mk[kMaskUpdate * M + m] = 0;
    mk[kMaskRefresh * M + m] = 0;
    if (!mk[kMaskApply * M + m]) return;
    // the scalar step of k_cg_mixed (FinPcgF), on the totals as (hi, lo) pairs
    DF td[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) td[k] = df_of(t[k]);
    float o[5];
    FinPcgF{b.prev_est, b.restart != 0}(td, o);
    if (o[3] != 0.f) {
      // 1: NaN/Inf in this mesh's system (an error); 2: finite breakdown
      if (o[3] == 1.f) b.status = OTFEM_ERR_NONFINITE;
      b.active = 0;
      mk[kMaskApply * M + m] = 0;
      return;
    }
    b.alpha = o[0];
    b.beta = o[1];
    b.est = o[2];
    b.rho = dfbits::widen(o[2]);
    b.prev_est = o[4];
    b.restart = 0;
    ++b.iterations;
    ++b.applies;
    mk[kMaskUpdate * M + m] = 1;
    // a mesh whose estimate reached the tolerance refreshes at the next
    // multiple of 4 iterations, so the meshes share refresh sweeps
    const bool refresh = (a.refresh > 0 && b.iterations % a.refresh == 0) || (o[2] <= b.thresh && b.iterations % 4 == 0);
    if (refresh) {
      mk[kMaskRefresh * M + m] = 1;
      ++b.applies;
      atomicAdd(&cnt[1], 1);
    } else if (b.iterations >= a.max_it) {
      b.active = 0;  // the update of this iteration is its last
      mk[kMaskApply * M + m] = 0;
    }
    if (b.active) atomicAdd(&cnt[0], 1);
  }
};

// totals: the true |b - A v|^2 of the refreshed meshes
struct FinBatchRefresh {
  __device__ void operator()(const MixedArgs& a, int m, const double* t, int* cnt) const {
    BatchMesh& b = a.bm[m];
    unsigned char* mk = a.bmask;
    const int M = a.num_meshes;
    if (mk[kMaskRefresh * M + m]) {
      b.restart = t[0] > 4.0 * b.est;
      b.prev_est = -1.f;
      b.rho = t[0];
      const bool periodic = a.refresh <= 0 || b.iterations % a.refresh == 0;
      if (t[0] < b.best_true) {
        b.best_true = t[0];
        b.best_buf ^= 1;
        b.stalls = 0;
      } else if (periodic && ++b.stalls >= 3) {
        b.active = 0;  // at the precision floor: no progress over three periods
        b.stalled = 1;
        b.rho = b.best_true;
      }
      if (t[0] <= b.thresh) {
        b.converged = 1;
        b.active = 0;
      }
      if (b.iterations >= a.max_it) b.active = 0;
      mk[kMaskApply * M + m] = b.active;
    }
    if (b.active) atomicAdd(&cnt[0], 1);
  }
};

// Batches of at most kLocalMeshes meshes: every CTA runs each iteration's
// scalar step (FinBatchIter's) itself, thread m for mesh m, on a shared-memory
// copy of the meshes' iteration state and masks, right after the grid barrier
// that completes the iteration's sums.  No CTA waits for a finisher to
// release the round or reads the scalars and masks back from global memory.
// All CTAs read the same totals and run the same FP32 code, so their copies
// stay identical; CTA 0 writes its copy back to the BatchMesh records and the
// global masks after the next grid barrier (when every CTA has read the
// totals), for the finisher-style reductions (refresh, the end of the step)
// that read them there.  Those reductions' results are loaded back into
// every CTA's copy.
constexpr int kLocalMeshes = 512;
struct LocalMeshes {
  unsigned char mask[3][kLocalMeshes];  // kMaskApply, kMaskUpdate, kMaskRefresh
  unsigned char restart[kLocalMeshes];
  float alpha[kLocalMeshes], beta[kLocalMeshes];
  float prev_est[kLocalMeshes], thresh[kLocalMeshes], est[kLocalMeshes];
  int iterations[kLocalMeshes], applies[kLocalMeshes];
};

// Every CTA: the copy of the meshes' state from the BatchMesh records and the
// global masks (after a finisher-style reduction changed them).
__device__ void local_load(const MixedArgs& a, LocalMeshes& L) {
  const int m = threadIdx.x, M = a.num_meshes;
  if (m < M) {
    const BatchMesh& b = a.bm[m];
    L.prev_est[m] = __ldcg(&b.prev_est);
    L.thresh[m] = __ldcg(&b.thresh);
    L.est[m] = __ldcg(&b.est);
    L.iterations[m] = __ldcg(&b.iterations);
    L.applies[m] = __ldcg(&b.applies);
    L.restart[m] = __ldcg(&b.restart) != 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) L.mask[k][m] = __ldcg(a.bmask + k * M + m);
  }
  __syncthreads();
}

// The iteration's reduction without a finisher: a grid barrier, then every
// CTA's scalar step for the meshes in the sweep (FinBatchIter on the copy).
// counts[0]: meshes still iterating; counts[1]: meshes due for a refresh.
__device__ bool batch_iter_local(const MixedArgs& a, unsigned& round, LocalMeshes& L, int (&counts)[4]) {
  if (!grid_barrier(a.sync, a.spin_limit, round)) return false;
  const int m = threadIdx.x, M = a.num_meshes;
  bool active = false, refresh = false;
  if (m < M) {
    L.mask[kMaskUpdate][m] = 0;
    L.mask[kMaskRefresh][m] = 0;
    if (L.mask[kMaskApply][m]) {
      const double* t = a.bacc + (size_t(round & 1u) * M + m) * kBatchSlots;
      DF td[7];
#pragma unroll
      for (int k = 0; k < 7; ++k) td[k] = df_of(__ldcg(t + k));
      float o[5];
      FinPcgF{L.prev_est[m], L.restart[m] != 0}(td, o);
      if (o[3] != 0.f) {
        // 1: NaN/Inf in this mesh's system (an error, recorded by CTA 0 now:
        // nothing reads the status during the solve); 2: finite breakdown
        if (o[3] == 1.f && blockIdx.x == 0) a.bm[m].status = OTFEM_ERR_NONFINITE;
        L.mask[kMaskApply][m] = 0;
      } else {
        L.alpha[m] = o[0];
        L.beta[m] = o[1];
        L.est[m] = o[2];
        L.prev_est[m] = o[4];
        L.restart[m] = 0;
        const int its = ++L.iterations[m];
        ++L.applies[m];
        L.mask[kMaskUpdate][m] = 1;
        // as FinBatchIter: refreshes at the next multiple of 4 iterations
        // once the estimate reached the tolerance
        refresh = (a.refresh > 0 && its % a.refresh == 0) || (o[2] <= L.thresh[m] && its % 4 == 0);
        if (refresh) {
          L.mask[kMaskRefresh][m] = 1;
          ++L.applies[m];
        } else if (its >= a.max_it) {
          L.mask[kMaskApply][m] = 0;  // the update of this iteration is its last
        }
      }
      active = L.mask[kMaskApply][m] != 0;
    }
  }
  counts[0] = __syncthreads_count(active);
  counts[1] = __syncthreads_count(refresh);
  counts[2] = counts[3] = 0;
  return true;
}

// CTA 0, after the grid barrier that follows the iteration of reduction
// round `iter_round`: the copy into the BatchMesh records and the global
// masks, and that round's totals cleared for round iter_round + 2.
__device__ void local_store(const MixedArgs& a, const LocalMeshes& L, unsigned iter_round) {
  const int m = threadIdx.x, M = a.num_meshes;
  if (m >= M) return;
  BatchMesh& b = a.bm[m];
  if (L.mask[kMaskUpdate][m]) {
    b.alpha = L.alpha[m];
    b.beta = L.beta[m];
    b.est = L.est[m];
    b.rho = dfbits::widen(L.est[m]);
    b.prev_est = L.prev_est[m];
    b.restart = 0;
    b.iterations = L.iterations[m];
    b.applies = L.applies[m];
  }
  if (b.active && !L.mask[kMaskApply][m]) b.active = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) a.bmask[k * M + m] = L.mask[k][m];
  double* t = a.bacc + (size_t(iter_round & 1u) * M + m) * kBatchSlots;
#pragma unroll
  for (int k = 0; k < kBatchSlots; ++k) t[k] = 0.0;
}

__global__ void __launch_bounds__(kBlock, 1) k_cg_batch(MixedArgs a) {
  const int N = a.N, M = a.num_meshes;
  const float scale = float(a.dt * a.dt);
  const DF dt_pair = df_of(a.dt);
  const DF damp_pair = df_add(DF{1.f, 0.f}, df_mul2(dt_pair, df_of(a.alpha)));  // 1 + dt alpha
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  unsigned round = 0;
  extern __shared__ __align__(16) unsigned char smem[];
  const NodeRange nr = warp_node_range(N);
  const int lane = threadIdx.x & 31;
  const int first_mesh = nr.beg < nr.end ? a.mesh_of_node[nr.beg] : -1;
  const unsigned char* mask_apply = a.bmask + kMaskApply * M;
  const unsigned char* mask_update = a.bmask + kMaskUpdate * M;
  const unsigned char* mask_refresh = a.bmask + kMaskRefresh * M;
  int counts[4];
  int sweeps = 0;
  auto acc_half = [&](unsigned next_round) { return a.bacc + size_t(next_round & 1u) * M * kBatchSlots; };
  const bool tracer = is_tracer();
  const long long t_start = tracer ? cycles_now() : 0ll;
  if (tracer) clear_phase_stamps(a);

  // The extrapolated start in a batch: a mesh whose previous solve took at
  // least half the batch's largest iteration count (the meshes the lock-step
  // waits for) starts from its projected start instead; the others
  // extrapolate, and their tets skip the search directions in the start
  // sweep.  Batches of at most kLocalMeshes meshes; larger ones project every
  // mesh.  proj: null when every mesh projects.
  __shared__ unsigned char s_proj[kLocalMeshes];
  __shared__ int s_maxits;
  const bool hybrid = a.extrap_k > 0 && a.nwarm > 0 && a.nwarm == a.hist_k && M <= kLocalMeshes &&
                      blockDim.x == kBlock;
  if (hybrid) {
    if (threadIdx.x == 0) s_maxits = 0;
    __syncthreads();
    const int its = threadIdx.x < M ? __ldcg(&a.bm[threadIdx.x].iterations) : 0;
    atomicMax(&s_maxits, its);
    __syncthreads();
    if (threadIdx.x < M) s_proj[threadIdx.x] = 2 * its >= s_maxits ? 1 : 0;
    __syncthreads();
  }
  const unsigned char* proj = hybrid ? s_proj : nullptr;
  // Phase 0 (as k_cg_mixed): b, diagonal, operand v (+ learned guess or
  // extrapolation), q = 0
  const int deg = hybrid ? extrap_degree(a) : 0;
  {
    SegSum<1> ss;
    ss.start(first_mesh);
    for (long base = nr.beg; base < nr.end; base += 32) {
      const long i = base + lane;
      const bool valid = i < nr.end;
      int m = -1;
      float bb[1] = {0.f};
      if (valid) {
        m = a.mesh_of_node[i];
        DF g[3];
        gather_forces(a, i, g);
        // in (hi, lo) pairs: no FP64 instruction
        const bool fx = a.fixed[i] != 0;
        const DF mass = df_of(a.mass[i]);
        const DF vi[3] = {df_of(a.v[3 * i]), df_of(a.v[3 * i + 1]), df_of(a.v[3 * i + 2])};
        float sp = 0.f;
        if (!fx) {
          DF b3[3];
          for (int c = 0; c < 3; ++c) {
            b3[c] = df_add(df_mul2(mass, vi[c]), df_mul2(dt_pair, df_add(df_of(a.fext[3 * i + c]), df_neg(g[c]))));
            a.bvec[3 * i + c] = f64_of(b3[c]);
          }
          a.b_hi[i] = make_float4(b3[0].hi, b3[1].hi, b3[2].hi, 0.f);
          a.b_lo[i] = make_float4(b3[0].lo, b3[1].lo, b3[2].lo, 0.f);
          const float bf[3] = {b3[0].hi + b3[0].lo, b3[1].hi + b3[1].lo, b3[2].hi + b3[2].lo};
          bb[0] = bf[0] * bf[0] + bf[1] * bf[1] + bf[2] * bf[2];
          const DF dg = df_mul2(mass, damp_pair);  // m (1 + dt alpha)
          a.diag[i] = f64_of(dg);
          a.diag_f[i] = dg.hi;
          a.diag_lo[i] = dg.lo;
          sp = a.precond ? 1.f / (dg.hi + scale * dfbits::trunc_f32(a.node_k[i])) : 1.f;
        } else {
          a.diag[i] = 0.0;
          a.diag_f[i] = 0.f;
          a.diag_lo[i] = 0.f;
        }
        a.r_f[i] = make_float4(0.f, 0.f, 0.f, sp);  // r.w: the node's preconditioner scalar
        DF v0[3] = {vi[0], vi[1], vi[2]};
        if (deg > 0 && !fx && !proj[m]) extrapolate(a, i, deg, v0);  // extrapolated start (as k_cg_mixed)
        a.v_f[i] = make_float4(v0[0].hi, v0[1].hi, v0[2].hi, fx ? 0.f : 1.f);
        a.v_lo[i] = make_float4(v0[0].lo, v0[1].lo, v0[2].lo, 0.f);
        a.q_f[i] = zero4;
        if (a.nwarm) {
          // learned start: the network's correction is the last search direction
          if (a.nwarm > a.hist_k) {
            const float4 d = fx ? zero4 : a.dv_last[i], w = fx ? zero4 : a.warm_dv[i];
            a.wprod[size_t(kMaxWarmDirs) * N + i] = make_float4(w.x - d.x, w.y - d.y, w.z - d.z, fx ? 0.f : 1.f);
          }
          for (int j = 0; j < a.nwarm; ++j) a.wprod[size_t(j) * N + i] = zero4;
        }
      }
      ss.add(valid, m, bb, acc_half(round + 1));
    }
    ss.flush(acc_half(round + 1));
  }
  if (!batch_reduce(a, round, FinBatchInit(), counts)) return;
  if (tracer) phase_stamp(a, 0, t_start);

  // initial residual r = b - A v (FP64), p = S r, for every mesh; with the
  // projected or learned start also A W_j and each mesh's start (k_cg_mixed)
  if (a.nwarm) {
    if (!apply_start_operands<true>(a, scale, smem, round, proj)) return;
    sweeps += 1 + a.nwarm;
  } else {
    apply_sweep<float>(a, a.v_f, a.v_lo, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem);
    ++sweeps;
  }
  if (!grid_barrier(a.sync, a.spin_limit, round)) return;
  if (tracer) phase_stamp(a, 1, t_start);
  if (a.nwarm) {
    const int nw = a.nwarm;
    // r = b - A v; A W_j += diag W_j (the mass term)
    for (long i = nr.beg + lane; i < nr.end; i += 32) {
      if (a.fixed[i]) continue;
      const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
      float rf[3];
      node_residual(a, i, vh, vl, q4, rf);
      a.r_f[i] = make_float4(rf[0], rf[1], rf[2], a.r_f[i].w);
      add_mass_term(a, i, a.diag_f[i]);
    }
    // per-mesh Gram systems, in chunks of 8 sums: W_i.A W_j (i <= j), then W_i.r
    __shared__ signed char s_pi[kMaxWarmSums], s_pj[kMaxWarmSums];
    if (threadIdx.x == 0) {
      int m = 0;
      for (int i = 0; i < nw; ++i)
        for (int j = i; j < nw; ++j, ++m) s_pi[m] = (signed char)i, s_pj[m] = (signed char)j;
      for (int i = 0; i < nw; ++i, ++m) s_pi[m] = (signed char)i, s_pj[m] = -1;
    }
    __syncthreads();
    const int nv = nw * (nw + 1) / 2 + nw;
    for (int c0 = 0; c0 < nv; c0 += 8) {
      SegSum<8, kMaxWarmSums> ss;
      ss.start(first_mesh);
      for (long base = nr.beg; base < nr.end; base += 32) {
        const long i = base + lane;
        const bool valid = i < nr.end;
        int m = -1;
        float v8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (valid) {
          m = a.mesh_of_node[i];
          if (!a.fixed[i] && (!proj || proj[m])) {  // extrapolating meshes: no Gram system (no move)
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              if (c0 + k >= nv) break;
              const float4 w = warm_dir(a, s_pi[c0 + k])[i];
              const float4 q = s_pj[c0 + k] >= 0 ? a.wprod[size_t(s_pj[c0 + k]) * N + i] : a.r_f[i];
              v8[k] = w.x * q.x + w.y * q.y + w.z * q.z;
            }
          }
        }
        ss.add(valid, m, v8, a.wbacc + c0);
      }
      ss.flush(a.wbacc + c0);
    }
    if (!batch_reduce(a, round, FinBatchGram(), counts)) return;
  }
  {
    SegSum<1> ss;
    ss.start(first_mesh);
    for (long base = nr.beg; base < nr.end; base += 32) {
      const long i = base + lane;
      const bool valid = i < nr.end;
      int m = -1;
      float rr[1] = {0.f};
      if (valid) {
        m = a.mesh_of_node[i];
        if (a.fixed[i]) {
          a.p_f[i] = zero4;
          a.r_f[i] = zero4;
        } else {
          const float sp = a.r_f[i].w;
          float rf[3];
          if (a.nwarm) {
            // v += sum_j g_j W_j (the mesh's coefficients); r -= sum_j g_j A W_j
            const float4 r4 = a.r_f[i];
            float4 vh = a.v_f[i], vl = a.v_lo[i];
            rf[0] = r4.x;
            rf[1] = r4.y;
            rf[2] = r4.z;
            move_to_start(a, i, a.bm[m].wgam, vh, vl, rf);
            a.v_f[i] = vh;
            a.v_lo[i] = vl;
          } else {
            const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
            node_residual(a, i, vh, vl, q4, rf);
          }
          a.r_f[i] = make_float4(rf[0], rf[1], rf[2], sp);
          a.p_f[i] = make_float4(sp * rf[0], sp * rf[1], sp * rf[2], 1.f);  // p = z = S r
          a.q_f[i] = zero4;
          a.v_keep[i] = a.v_f[i];  // the start is the first kept iterate
          a.v_keep[N + i] = a.v_lo[i];
          rr[0] = rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2];
        }
      }
      ss.add(valid, m, rr, acc_half(round + 1));
    }
    ss.flush(acc_half(round + 1));
  }
  if (!batch_reduce(a, round, FinBatchStart(), counts)) return;
  // batches of at most kLocalMeshes meshes: the iterations' scalar steps in
  // every CTA, and the sweeps' masks from shared memory
  const bool local = M <= kLocalMeshes && blockDim.x == kBlock;
  __shared__ LocalMeshes s_local;
  if (local) {
    local_load(a, s_local);
    mask_apply = s_local.mask[kMaskApply];
    mask_update = s_local.mask[kMaskUpdate];
    mask_refresh = s_local.mask[kMaskRefresh];
  }
  if (tracer) phase_stamp(a, 2, t_start);
  int n_active = counts[0];
  __shared__ double stamp[6];  // trace stamps, written by the tracer thread only

  for (int it = 0; n_active > 0 && it < a.max_it; ++it) {
    const int active_before = n_active;
    // q += dt^2 K' p for the meshes still iterating
    apply_sweep<float>(a, a.p_f, nullptr, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem, mask_apply);
    ++sweeps;
    if (tracer) stamp[0] = double(cycles_now() - t_start);
    if (!grid_barrier(a.sync, a.spin_limit, round)) return;
    if (tracer) stamp[1] = double(cycles_now() - t_start);
    // q = diag p + q; the totals of FinPcgF per mesh, over the meshes in the sweep
    {
      SegSum<7> ss;
      ss.start(-1);
      masked_node_walk(a, mask_apply, [&](bool valid, long i, int m) {
        float s7[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (valid) {
          if (!a.fixed[i]) {
            const float4 q4 = load_acc(a.q_f + i), p4 = a.p_f[i], r4 = a.r_f[i];
            const float d = a.diag_f[i];
            const float qx = d * p4.x + q4.x, qy = d * p4.y + q4.y, qz = d * p4.z + q4.z;
            s7[0] = p4.x * qx + p4.y * qy + p4.z * qz;
            s7[4] = r4.x * qx + r4.y * qy + r4.z * qz;
            s7[5] = qx * qx + qy * qy + qz * qz;
            s7[6] = r4.x * r4.x + r4.y * r4.y + r4.z * r4.z;
            s7[1] = r4.w * s7[4];
            s7[2] = r4.w * s7[5];
            s7[3] = r4.w * s7[6];
          }
        }
        ss.add(valid, m, s7, acc_half(round + 1));
      });
      ss.flush(acc_half(round + 1));
    }
    if (tracer) stamp[2] = double(cycles_now() - t_start);
    if (local) {
      if (!batch_iter_local(a, round, s_local, counts)) return;
    } else if (!batch_reduce(a, round, FinBatchIter(), counts)) {
      return;
    }
    const unsigned iter_round = round;
    if (tracer) stamp[3] = double(cycles_now() - t_start);
    n_active = counts[0];
    const bool any_refresh = counts[1] > 0;
    // v += alpha p, r -= alpha q, p = r + beta p with each mesh's scalars
    masked_node_walk(a, mask_update, [&](bool valid, long i, int m) {
      if (!valid || a.fixed[i]) return;
      const float alpha = local ? s_local.alpha[m] : a.bm[m].alpha, beta = local ? s_local.beta[m] : a.bm[m].beta;
      float4 q4 = load_acc(a.q_f + i), p4 = a.p_f[i], r4 = a.r_f[i];
      float4 vh = a.v_f[i], vl = a.v_lo[i];
      const float d = a.diag_f[i];
      const float qx = d * p4.x + q4.x, qy = d * p4.y + q4.y, qz = d * p4.z + q4.z;
      df_inc(vh.x, vl.x, alpha * p4.x);
      df_inc(vh.y, vl.y, alpha * p4.y);
      df_inc(vh.z, vl.z, alpha * p4.z);
      const float rx = r4.x - alpha * qx, ry = r4.y - alpha * qy, rz = r4.z - alpha * qz;
      const float sp = r4.w;
      a.v_f[i] = vh;
      a.v_lo[i] = vl;
      a.r_f[i] = make_float4(rx, ry, rz, sp);
      a.p_f[i] = make_float4(sp * rx + beta * p4.x, sp * ry + beta * p4.y, sp * rz + beta * p4.z, 1.f);
      a.q_f[i] = zero4;
    });
    if (tracer) stamp[4] = double(cycles_now() - t_start);
    if (!grid_barrier(a.sync, a.spin_limit, round)) return;
    if (local && blockIdx.x == 0) local_store(a, s_local, iter_round);
    // trace row: the meshes iterating, whether a refresh sweep follows
    if (tracer) trace_row(a, it, double(active_before), 0.0, any_refresh ? 1.0 : 0.0, 0.0, stamp, t_start);
    if (any_refresh) {
      // r = b - A v (residual replacement, FP64) for the meshes due
      apply_sweep<float>(a, a.v_f, a.v_lo, a.q_f, a.re_f, a.b_f, a.c_f, scale, smem, mask_refresh);
      ++sweeps;
      if (!grid_barrier(a.sync, a.spin_limit, round)) return;
      SegSum<1> ss;
      ss.start(-1);
      masked_node_walk(a, mask_refresh, [&](bool valid, long i, int m) {
        float tr[1] = {0.f};
        if (valid) {
          if (!a.fixed[i]) {
            const float4 q4 = load_acc(a.q_f + i), vh = a.v_f[i], vl = a.v_lo[i];
            float rr3[3];
            node_residual(a, i, vh, vl, q4, rr3);
            const float rx = rr3[0], ry = rr3[1], rz = rr3[2];
            a.r_f[i] = make_float4(rx, ry, rz, a.r_f[i].w);
            a.q_f[i] = zero4;
            const long cand = 2L * (a.bm[m].best_buf ^ 1) * N;  // the kept copy that is not the best
            a.v_keep[cand + i] = vh;
            a.v_keep[cand + N + i] = vl;
            tr[0] = rx * rx + ry * ry + rz * rz;
          }
        }
        ss.add(valid, m, tr, acc_half(round + 1));
      });
      ss.flush(acc_half(round + 1));
      if (!batch_reduce(a, round, FinBatchRefresh(), counts)) return;
      if (local) local_load(a, s_local);
      n_active = counts[0];
    }
  }

  if (tracer) phase_stamp(a, 3, t_start);
  // v back to FP64 (a mesh stopped at the floor takes its kept best
  // iterate); position update; velocity change (all meshes)
  for (long i = nr.beg + lane; i < nr.end; i += 32) {
    if (a.fixed[i]) continue;
    const BatchMesh& bmi = a.bm[a.mesh_of_node[i]];
    const long kb = 2L * bmi.best_buf * N;
    const float4 vh = bmi.stalled ? a.v_keep[kb + i] : a.v_f[i], vl = bmi.stalled ? a.v_keep[kb + N + i] : a.v_lo[i];
    // in pairs, with one FP64 addition per coordinate (x keeps its 53 bits)
    const DF v3[3] = {{vh.x, vl.x}, {vh.y, vl.y}, {vh.z, vl.z}};
    DF dv[3];
    for (int c = 0; c < 3; ++c) {
      dv[c] = df_add(v3[c], df_neg(df_of(a.v[3 * i + c])));
      a.v[3 * i + c] = f64_of(v3[c]);
      a.x[3 * i + c] += f64_of(df_mul2(v3[c], dt_pair));
    }
    a.dv_last[i] = make_float4(dv[0].hi, dv[1].hi, dv[2].hi, 0.f);
    if (a.hist) record_velocity_change(a, i, dv);
  }
  if (tracer) phase_stamp(a, 4, t_start);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // batch summary: the largest iteration count and relative residual, the
    // worst status
    int its = 0, st = ld_status(&a.sync->status), warn = 0;
    double rel = 0.0, rel0 = 0.0;
    for (int m = 0; m < M; ++m) {
      BatchMesh& b = a.bm[m];
      if (b.status == 0 && !b.converged) b.status = OTFEM_WARN_NOT_CONVERGED;
      if (b.status < 0 && st == 0) st = b.status;
      if (b.status > 0) warn = 1;
      its = its > b.iterations ? its : b.iterations;
      const double bb = b.bnorm2 > 0.0 ? b.bnorm2 : 1.0;
      rel = fmax(rel, b.rho / bb);
      rel0 = fmax(rel0, b.rho0 / bb);
    }
    a.stats->iterations = its;
    a.stats->applies = sweeps;
    a.stats->status = st != 0 ? st : (warn ? OTFEM_WARN_NOT_CONVERGED : 0);
    a.stats->rr = rel;
    a.stats->rr0 = rel0;
    a.stats->bb = 1.0;
    advance_fill(a);
  }
}

// K1, mixed: FP32 orientation and elastic forces.  The rows of E^-1 are
// -b_k (fem_compute_b.h), so F = -sum_k e'_k (x) b_k, which Gram-Schmidt
// orthonormalises exactly as the reference's F (a positive multiple of it)
// would be.
//
// The deformation d_k = Re^T (x_k - x_0) - (x0_k - x0_0) is the small
// difference of two edge-sized vectors, so it is formed in (hi, lo) pair
// arithmetic and only then rounded to FP32: the current edges as exact pairs
// from the split FP64 positions (two-sums of the high parts, plus the
// differences of the low parts), the rest edges as pairs from k_rest_edges'
// table, and Re as a pair orthonormal to ~1e-14: the FP32 rotation R plus
// the correction -R (R^T R - I) / 2 of one Newton-Schulz step, with R^T R
// from exact products.  In FP32 both edges carry rounding errors of ~6e-8 of
// an edge, and a rotation orthonormal only to FP32 adds a symmetric part of
// that size to Re^T e; either one is a spurious strain of ~1e-7, which on a
// stiff body that deforms little (strains of 1e-5) is a force error of 1e-2
// per element.  With the pair arithmetic the strain keeps FP32 relative
// precision, and the rest of the element force (stress, rotation back,
// node forces) is FP32 with ~1e-7 relative error.
__global__ void k_orient_rhs_f32(int T, int warp, const int4* __restrict__ tets, const double* __restrict__ x,
                                 const float* __restrict__ e0_f, const float* __restrict__ b_f,
                                 const float* __restrict__ c_f, float* re_f, float4* g_f, float* tile_f,
                                 int tile_tets) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int4 n = tets[t];
  const int nn[4] = {n.x, n.y, n.z, n.w};
  // current edges x_k - x_0 as pairs from the positions' (hi, lo) split
  // (integer instructions), rounded (ep) for the orientation; rest edges as
  // pairs from the table (hi: 9 x T words, then lo: 9 x T words)
  float ep[3][3];
  DF epp[3][3], e0p[3][3];
  {
    DF p0[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) p0[c] = df_of(x[3 * nn[0] + c]);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const DF pk = df_of(x[3 * nn[k + 1] + c]);
        float s, e;
        two_sum(pk.hi, -p0[c].hi, s, e);
        e += pk.lo - p0[c].lo;
        const float h = s + e;
        epp[k][c] = DF{h, e - (h - s)};
        ep[k][c] = h;
        e0p[k][c] = DF{e0_f[long(3 * k + c) * T + t], e0_f[long(9 + 3 * k + c) * T + t]};
      }
  }
  float b[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) b[q] = b_f[(long)q * T + t];
  float R[9];
  if (warp) {
    float F[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) F[3 * a + c] = -(ep[0][a] * b[c] + ep[1][a] * b[3 + c] + ep[2][a] * b[6 + c]);
    // row Gram-Schmidt (math_matrix3x3.h:536-558)
    float r0[3] = {F[0], F[1], F[2]}, r1[3] = {F[3], F[4], F[5]};
    float l0 = sqrtf(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
    if (l0 != 0.f) r0[0] /= l0, r0[1] /= l0, r0[2] /= l0;
    float d = r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2];
    r1[0] -= r0[0] * d, r1[1] -= r0[1] * d, r1[2] -= r0[2] * d;
    float l1 = sqrtf(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
    if (l1 != 0.f) r1[0] /= l1, r1[1] /= l1, r1[2] /= l1;
    R[0] = r0[0], R[1] = r0[1], R[2] = r0[2];
    R[3] = r1[0], R[4] = r1[1], R[5] = r1[2];
    R[6] = r0[1] * r1[2] - r1[1] * r0[2];
    R[7] = r1[0] * r0[2] - r0[0] * r1[2];
    R[8] = r0[0] * r1[1] - r1[0] * r0[1];
  } else {
#pragma unroll
    for (int q = 0; q < 9; ++q) R[q] = (q == 0 || q == 4 || q == 8) ? 1.f : 0.f;
  }
  // The rotation every FP32 apply variant uses is the one the staged apply
  // rebuilds from its quaternion, so forces and operator agree.
  const float4 quat = rotation_to_quaternion(R);
  quaternion_to_rotation(quat, R);
  tile_f[tile_word(tile_tets, t, 4)] = quat.x;
  tile_f[tile_word(tile_tets, t, 5)] = quat.y;
  tile_f[tile_word(tile_tets, t, 6)] = quat.z;
  tile_f[tile_word(tile_tets, t, 7)] = quat.w;
#pragma unroll
  for (int q = 0; q < 9; ++q) re_f[(long)q * T + t] = R[q];
  // Re as a pair: R + R_lo, R_lo = -R (R^T R - I) / 2 (one Newton-Schulz
  // step; the entries of R^T R - I from exact products and two-sums)
  float Rl[9];
  {
    float E[3][3];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = b; c < 3; ++c) {
        DF acc = {0.f, 0.f};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float p = R[3 * a + b] * R[3 * a + c];
          acc = df_add(acc, DF{p, fmaf(R[3 * a + b], R[3 * a + c], -p)});
        }
        if (b == c) acc = df_add(acc, DF{-1.f, 0.f});
        E[b][c] = E[c][b] = acc.hi + acc.lo;
      }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        Rl[3 * a + c] = -0.5f * (R[3 * a] * E[0][c] + R[3 * a + 1] * E[1][c] + R[3 * a + 2] * E[2][c]);
  }
  // rest-frame displacements d_k = Re^T (x_k - x_0) - (x0_k - x0_0) in pairs
  float dk[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      DF acc = df_neg(e0p[k][a]);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc = df_add(acc, df_mul2(DF{R[3 * c + a], Rl[3 * c + a]}, epp[k][c]));
      dk[k][a] = acc.hi + acc.lo;
    }
  float H[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) H[a][c] = dk[0][a] * b[c] + dk[1][a] * b[3 + c] + dk[2][a] * b[6 + c];
  const float c0 = c_f[t], c1 = c_f[T + t], c2 = c_f[2L * T + t];
  float tr = c1 * (H[0][0] + H[1][1] + H[2][2]);
  float s[3][3];
  s[0][0] = c0 * H[0][0] + tr;
  s[1][1] = c0 * H[1][1] + tr;
  s[2][2] = c0 * H[2][2] + tr;
  s[0][1] = s[1][0] = c2 * (H[0][1] + H[1][0]);
  s[0][2] = s[2][0] = c2 * (H[0][2] + H[2][0]);
  s[1][2] = s[2][1] = c2 * (H[1][2] + H[2][1]);
  float S[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) S[a][c] = R[3 * a] * s[0][c] + R[3 * a + 1] * s[1][c] + R[3 * a + 2] * s[2][c];
  float f[4][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int a = 0; a < 3; ++a) f[k + 1][a] = S[a][0] * b[3 * k] + S[a][1] * b[3 * k + 1] + S[a][2] * b[3 * k + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) f[0][a] = -(f[1][a] + f[2][a] + f[3][a]);
  // w of the four entries: the tet's quaternion (x, y, z, w), read by the
  // network inputs (one 64-byte line per tet instead of four tile words)
  const float qv[4] = {quat.x, quat.y, quat.z, quat.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) g_f[4L * t + k] = make_float4(f[k][0], f[k][1], f[k][2], qv[k]);
}

// The rotation words of the tiles from the FP32 orientations (re_f), after
// the tiles were laid out anew.
__global__ void k_tile_quats_from_re(int T, const float* __restrict__ re_f, float* tile_f, int tile_tets) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  float R[9];
  for (int q = 0; q < 9; ++q) R[q] = re_f[(long)q * T + t];
  const float4 quat = rotation_to_quaternion(R);
  tile_f[tile_word(tile_tets, t, 4)] = quat.x;
  tile_f[tile_word(tile_tets, t, 5)] = quat.y;
  tile_f[tile_word(tile_tets, t, 6)] = quat.z;
  tile_f[tile_word(tile_tets, t, 7)] = quat.w;
}

__global__ void k_identity_f32(int T, float* re_f, float* tile_f, int tile_tets) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  for (int q = 0; q < 9; ++q) re_f[(long)q * T + t] = (q == 0 || q == 4 || q == 8) ? 1.f : 0.f;
  for (int q = 0; q < 4; ++q) tile_f[tile_word(tile_tets, t, 4 + q)] = q == 3 ? 1.f : 0.f;
}

// m_Re of every tet (FP64, row-major) from the FP32 structure-of-arrays copy.
__global__ void k_re_from_f32(int T, const float* __restrict__ re_f, double* Re) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  for (int q = 0; q < 9; ++q) Re[9L * t + q] = double(re_f[(long)q * T + t]);
}

// K1: orientation (FP64, reference Gram-Schmidt) and the elastic forces
// g_k = Re Ke (Re^T x - x0) of the tet's nodes, via displacements relative to
// node 0: d_k = Re^T (x_k - x_0) - (x0_k - x0_0).
__global__ void k_orient_rhs(int T, int warp, const int4* __restrict__ tets, const double* __restrict__ x,
                             const double* __restrict__ x0, const double* __restrict__ E,
                             const double* __restrict__ V, const double* __restrict__ Bv,
                             const double* __restrict__ D, double* Re, float* re_f, double* re_d,
                             double* tet_force, float* tile_f, int tile_tets) {
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
  float Rf[9];
  for (int q = 0; q < 9; ++q) {
    Re[9 * t + q] = R[q];
    re_f[(long)q * T + t] = Rf[q] = float(R[q]);
    re_d[(long)q * T + t] = R[q];
  }
  const float4 quat = rotation_to_quaternion(Rf);
  tile_f[tile_word(tile_tets, t, 4)] = quat.x;
  tile_f[tile_word(tile_tets, t, 5)] = quat.y;
  tile_f[tile_word(tile_tets, t, 6)] = quat.z;
  tile_f[tile_word(tile_tets, t, 7)] = quat.w;
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
__global__ void k_prepare(int T, const int4* __restrict__ tets, const double* __restrict__ Bv,
                          const double* __restrict__ D, const double* __restrict__ V, float* b_f, float* c_f,
                          double* b_d, double* c_d, float* tile_f, int tile_tets) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  for (int q = 0; q < 9; ++q) {
    double val = Bv[12 * t + 3 + q];
    b_f[(long)q * T + t] = float(val);
    b_d[(long)q * T + t] = val;
    tile_f[tile_word(tile_tets, t, 8 + q)] = float(val);
  }
  double vol = V[t];
  double c[3] = {vol * (D[3 * t] - D[3 * t + 1]), vol * D[3 * t + 1], vol * D[3 * t + 2]};
  for (int q = 0; q < 3; ++q) {
    c_f[(long)q * T + t] = float(c[q]);
    c_d[(long)q * T + t] = c[q];
    tile_f[tile_word(tile_tets, t, 17 + q)] = float(c[q]);
  }
  const int4 n = tets[t];
  tile_f[tile_word(tile_tets, t, 0)] = __int_as_float(n.x);
  tile_f[tile_word(tile_tets, t, 1)] = __int_as_float(n.y);
  tile_f[tile_word(tile_tets, t, 2)] = __int_as_float(n.z);
  tile_f[tile_word(tile_tets, t, 3)] = __int_as_float(n.w);
  tile_f[tile_word(tile_tets, t, 4)] = 0.f;  // identity until the first orientation
  tile_f[tile_word(tile_tets, t, 5)] = 0.f;
  tile_f[tile_word(tile_tets, t, 6)] = 0.f;
  tile_f[tile_word(tile_tets, t, 7)] = 1.f;
}

// The timeout path of the grid barrier: one CTA arrives at a round that two
// arrivals complete, so the wait runs until its limit, records
// OTFEM_ERR_TIMEOUT and returns; the kernel then reports the status.
__global__ void k_wait_timeout(DeviceSync* sync, long long limit, int* status_out) {
  if (threadIdx.x != 0) return;
  const bool ok = sync_round(sync, 2u, limit);  // gridDim.x == 1: two arrivals never come
  *status_out = ok ? 0 : ld_status(&sync->status);
}

// Rest-frame edges x0_k - x0_0 of every tet (k = 1..3) as (hi, lo) float
// pairs of the FP64 differences (SoA: 9 x T high parts, then 9 x T low
// parts): the orientation kernel's rest term, recomputed whenever the model
// coordinates change.
__global__ void k_rest_edges(int T, const int4* __restrict__ tets, const double* __restrict__ x0, float* e0_f) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int4 n = tets[t];
  const int nn[4] = {n.x, n.y, n.z, n.w};
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) {
      const double d = x0[3 * nn[k + 1] + c] - x0[3 * nn[0] + c];
      const float hi = float(d);
      e0_f[long(3 * k + c) * T + t] = hi;
      e0_f[long(9 + 3 * k + c) * T + t] = float(d - double(hi));
    }
}

// Node stiffness scale of the Jacobi preconditioner: k_i = sum over the
// node's tets of tr(Ke_ii) / 3.  For the node's B-vector b the element apply
// gives, in the tet frame, Ke_ii[a][a] = (c0 + c1) b_a^2 + c2 (|b|^2 - b_a^2),
// so tr(Ke_ii) = (c0 + c1 + 2 c2) |b|^2; the rotation Re Ke_ii Re^T keeps the
// trace, so k does not change from step to step.  Sums in ascending tet order.
__global__ void k_node_stiffness(int N, int T, const int* __restrict__ inc_ptr, const int* __restrict__ inc_ent,
                                 const double* __restrict__ Bv, const double* __restrict__ c_d, double* node_k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double k = 0.0;
  for (int q = inc_ptr[i]; q < inc_ptr[i + 1]; ++q) {
    const int e = inc_ent[q], t = e >> 2, slot = e & 3;
    const double* b = Bv + 12L * t + 3 * slot;
    const double c = c_d[t] + c_d[(long)T + t] + 2.0 * c_d[2L * T + t];
    k += c * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  }
  node_k[i] = k / 3.0;
}

// Standalone y = A x (diagnostics and the apply-only measurement): pack, one
// element-apply sweep, finalize.
template <typename V4>
__global__ void k_pack_operand(int N, const unsigned char* __restrict__ fixed, const double* __restrict__ x,
                               V4* u, V4* ulo, V4* q) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  store_operand(u, ulo, i, x[3 * i], x[3 * i + 1], x[3 * i + 2], fixed[i] ? 0.0 : 1.0);
  q[i] = make_v4<V4, double>(0.0, 0.0, 0.0, 0.0);
}

template <typename R>
__global__ void __launch_bounds__(kBlock, 1) k_apply_sweep(MixedArgs a, const typename ApplyOps<R>::V4* u,
                                                           const typename ApplyOps<R>::V4* ulo,
                                                           typename ApplyOps<R>::V4* q) {
  const R* re = sizeof(R) == 4 ? (const R*)a.re_f : (const R*)a.re_d;
  const R* bb = sizeof(R) == 4 ? (const R*)a.b_f : (const R*)a.b_d;
  const R* cc = sizeof(R) == 4 ? (const R*)a.c_f : (const R*)a.c_d;
  extern __shared__ __align__(16) unsigned char smem[];
  apply_sweep<R>(a, u, ulo, q, re, bb, cc, R(a.dt * a.dt), smem, a.sweep_mask);
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

void set_patch_args(MixedArgs& a, const Context& c) {
  a.num_patches = c.num_patches;
  a.patch_max_nodes_padded = (c.patch_max_nodes + 3) / 4 * 4;
  a.patch_node_ptr = c.patch_node_ptr;
  a.patch_nodes = c.patch_nodes;
  a.lconn = c.lconn;
  a.patch_inc_ptr = c.patch_inc_ptr;
  a.patch_inc = c.patch_inc;
  a.apply_variant = c.apply_variant;
  a.stream_tiles = c.stream_tiles ? 1 : 0;
}

template <typename R>
const void* cg_kernel() {
  return std::is_same<R, float>::value ? reinterpret_cast<const void*>(&k_cg_mixed)
                                       : reinterpret_cast<const void*>(&k_cg_fp64);
}

}  // namespace

// Patches of kPatchTets consecutive tets (in mesh order, which the block
// generator and most mesh files lay out with spatial locality).  For each
// patch: its nodes in ascending order (bit 31 set if another patch touches
// the node), and every tet's nodes as indices into that list.
cudaError_t build_patches(Context& c, const int32_t* tets) {
  const int T = c.T, N = c.N;
  const int P = (T + kPatchTets - 1) / kPatchTets;
  std::vector<int> npatch(size_t(N), 0), stamp(size_t(N), -1), local(size_t(N), 0);
  for (int p = 0; p < P; ++p)
    for (int t = p * kPatchTets; t < std::min(T, (p + 1) * kPatchTets); ++t)
      for (int k = 0; k < 4; ++k) {
        int n = tets[4L * t + k];
        if (stamp[n] != p) {
          stamp[n] = p;
          ++npatch[n];
        }
      }
  std::vector<int> ptr(size_t(P) + 1, 0), nodes;
  std::vector<ushort4> lconn(size_t(T > 0 ? T : 1));
  std::fill(stamp.begin(), stamp.end(), -1);
  int maxn = 0;
  std::vector<int> list, inc_ptr;
  std::vector<unsigned short> inc;
  for (int p = 0; p < P; ++p) {
    list.clear();
    const int t0 = p * kPatchTets, t1 = std::min(T, (p + 1) * kPatchTets);
    for (int t = t0; t < t1; ++t)
      for (int k = 0; k < 4; ++k) {
        int n = tets[4L * t + k];
        if (stamp[n] != p) {
          stamp[n] = p;
          list.push_back(n);
        }
      }
    std::sort(list.begin(), list.end());
    for (size_t j = 0; j < list.size(); ++j) {
      local[list[j]] = int(j);
      nodes.push_back(list[j] | (npatch[list[j]] > 1 ? int(0x80000000u) : 0));
    }
    for (int t = t0; t < t1; ++t) {
      const int32_t* n = tets + 4L * t;
      lconn[t] = make_ushort4((unsigned short)local[n[0]], (unsigned short)local[n[1]],
                              (unsigned short)local[n[2]], (unsigned short)local[n[3]]);
    }
    // per patch node, its (local tet, slot) entries in ascending tet order
    std::vector<int> cnt(list.size() + 1, 0);
    for (int t = t0; t < t1; ++t)
      for (int k = 0; k < 4; ++k) ++cnt[local[tets[4L * t + k]] + 1];
    for (size_t j = 0; j < list.size(); ++j) cnt[j + 1] += cnt[j];
    const int base = int(inc.size());
    inc.resize(inc.size() + size_t(4 * (t1 - t0)));
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int t = t0; t < t1; ++t)
      for (int k = 0; k < 4; ++k)
        inc[base + fill[local[tets[4L * t + k]]]++] = (unsigned short)(((t - t0) << 2) | k);
    for (size_t j = 0; j < list.size(); ++j) inc_ptr.push_back(base + cnt[j]);
    ptr[p + 1] = ptr[p] + int(list.size());
    maxn = std::max(maxn, int(list.size()));
  }
  inc_ptr.push_back(int(inc.size()));
  c.num_patches = P;
  c.patch_max_nodes = maxn;
  const int cap = (maxn + 3) / 4 * 4;
  // the patch variants' staging: atomics (operand + accumulators) and gather
  // (operand + 12 forces per tet); the kernels accept the largest staging of
  // all variants, and each launch asks for its variant's (launch_smem)
  c.patch_smem[0] = size_t(cap) * std::max(SmemOperand<float>::bytes, SmemOperand<double>::bytes);
  c.patch_smem[1] = size_t(cap) * sizeof(double4) + size_t(kPatchTets) * 12 * sizeof(double);
  c.apply_smem = std::max(std::max(c.patch_smem[0], c.patch_smem[1]), kStagedSmem);
  cudaError_t e;
  if ((e = cudaMalloc(&c.patch_node_ptr, sizeof(int) * ptr.size())) != cudaSuccess) return e;
  if ((e = cudaMalloc(&c.patch_nodes, sizeof(int) * std::max<size_t>(nodes.size(), 1))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&c.lconn, sizeof(ushort4) * lconn.size())) != cudaSuccess) return e;
  if ((e = cudaMemcpy(c.patch_node_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if (!nodes.empty() &&
      (e = cudaMemcpy(c.patch_nodes, nodes.data(), sizeof(int) * nodes.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpy(c.lconn, lconn.data(), sizeof(ushort4) * lconn.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if ((e = cudaMalloc(&c.patch_inc_ptr, sizeof(int) * inc_ptr.size())) != cudaSuccess) return e;
  if ((e = cudaMalloc(&c.patch_inc, sizeof(unsigned short) * std::max<size_t>(inc.size(), 1))) != cudaSuccess)
    return e;
  if ((e = cudaMemcpy(c.patch_inc_ptr, inc_ptr.data(), sizeof(int) * inc_ptr.size(), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return e;
  if (!inc.empty() && (e = cudaMemcpy(c.patch_inc, inc.data(), sizeof(unsigned short) * inc.size(),
                                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  // kernels that stage patches may need more than the default 48 KB
  const void* fns[] = {cg_kernel<float>(), cg_kernel<double>(), reinterpret_cast<const void*>(&k_apply_sweep<float>),
                       reinterpret_cast<const void*>(&k_apply_sweep<double>),
                       reinterpret_cast<const void*>(&k_cg_batch)};
  for (const void* f : fns)
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(c.apply_smem))) != cudaSuccess)
      return e;
  return cudaSuccess;
}

void staged_tiles(Context& c) {
  const long T = c.T;
  const long G = c.mf_grid > 0 ? c.mf_grid : 1;
  // rounds of tiles per CTA at the largest tile, then the smallest tile that
  // still covers the tets in that many rounds, rounded up to a multiple of 16
  // tets (each word array of a tile then starts on a 64-byte boundary)
  const long rounds = std::max(1L, (T + G * kTileMaxTets - 1) / (G * kTileMaxTets));
  long tt = (T + G * rounds - 1) / (G * rounds);
  tt = std::min<long>(kTileMaxTets, std::max(16L, (tt + 15) / 16 * 16));
  c.tile_tets = int(tt);
  c.tile_balanced = int(tt);
  c.tile_magic = tile_magic_of(c.tile_tets);
  c.num_tiles = int((T + tt - 1) / tt);
}

// Dynamic shared memory of a launch with the mesh's apply variant: the
// tiled-tets variant needs none, so L1 keeps the rest of the SM's 256 KB.
size_t launch_smem(const Context& c) {
  switch (c.apply_variant) {
    case kApplyAtomics: return c.patch_smem[0];
    case kApplyGather: return c.patch_smem[1];
    case kApplyStaged: return kStagedSmem;
    default: return 0;
  }
}

int mixed_grid_shape(Context& c, int* grid, int* block) {
  int occ32 = 0, occ64 = 0, occb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, k_cg_mixed, kBlock, c.apply_smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, k_cg_fp64, kBlock, c.apply_smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occb, k_cg_batch, kBlock, c.apply_smem);
  int occ = std::min(occ32, std::min(occ64, occb));
  if (occ < 1) occ = 1;
  if (occ > 2) occ = 2;
  *grid = c.num_sms * occ;
  if (*grid > kMaxGrid) *grid = kMaxGrid;
  *block = kBlock;
  return occ;
}

cudaError_t mixed_prepare(Context& c) {
  int nb = (c.T + 255) / 256;
  if (nb < 1) nb = 1;
  // padding tets of the last tile: node 0, no stiffness (never computed)
  cudaError_t e = cudaMemsetAsync(c.tile_f, 0, sizeof(float) * kTileWords * size_t(c.tile_tets) * c.num_tiles,
                                  c.stream);
  if (e != cudaSuccess) return e;
  k_prepare<<<nb, 256, 0, c.stream>>>(c.T, c.tets, c.Bv, c.D, c.V, c.b_f, c.c_f, c.b_d, c.c_d, c.tile_f,
                                      c.tile_tets);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = mixed_rest_edges(c)) != cudaSuccess) return e;
  const int nn = c.N > 0 ? (c.N + 255) / 256 : 1;
  k_node_stiffness<<<nn, 256, 0, c.stream>>>(c.N, c.T, c.inc_ptr, c.inc_ent, c.Bv, c.c_d, c.node_k);
  return cudaGetLastError();
}

cudaError_t check_wait_timeout(Context& c, long long cycles, int* status) {
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(c.sync, 0, sizeof(DeviceSync), c.stream);
  if (e == cudaSuccess) {
    k_wait_timeout<<<1, 32, 0, c.stream>>>(c.sync, cycles, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(status, d, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c.sync, 0, sizeof(DeviceSync), c.stream);
  if (d) cudaFree(d);
  return e;
}

cudaError_t mixed_rest_edges(Context& c) {
  if (c.T == 0) return cudaSuccess;
  k_rest_edges<<<(c.T + 255) / 256, 256, 0, c.stream>>>(c.T, c.tets, c.x0, c.e0_f);
  return cudaGetLastError();
}

cudaError_t launch_mixed_orient(Context& c, double dt, bool warp, int solver) {
  int nb = (c.T + 255) / 256;
  if (nb < 1) nb = 1;
  cudaError_t e;
  if (solver == OTFEM_SOLVER_FP64) {
    k_orient_rhs<<<nb, 256, 0, c.stream>>>(c.T, warp ? 1 : 0, c.tets, c.x, c.x0, c.E, c.V, c.Bv, c.D, c.Re,
                                           c.re_f, c.re_d, c.elastic_force, c.tile_f, c.tile_tets);
    c.re_f32_pending = false;
    c.quat_in_g_f = false;
  } else {
    k_orient_rhs_f32<<<nb, 256, 0, c.stream>>>(c.T, warp ? 1 : 0, c.tets, c.x, c.e0_f, c.b_f, c.c_f, c.re_f,
                                               c.g_f, c.tile_f, c.tile_tets);
    c.re_f32_pending = true;
    c.quat_in_g_f = true;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // add_plasticity_force (fem_simulate.h:102) runs between the assembly and
  // the right-hand side, as in the reference; it only changes f_ext when
  // creep and max are both positive, which the host records at init.  It
  // reads the FP64 orientations.
  if (c.plastic_active) {
    if (c.re_f32_pending && (e = sync_orientations(c)) != cudaSuccess) return e;
    if ((e = launch_plasticity(c, dt)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int tile_candidates(const Context& c, int* out, size_t* floats) {
  const int fixed_sizes[4] = {128, 256, 512, 1024};
  int n = 0;
  out[n++] = c.tile_balanced;  // staged_tiles
  for (int s : fixed_sizes) {
    if (s > kTileMaxTets) continue;
    bool seen = false;
    for (int k = 0; k < n; ++k) seen = seen || out[k] == s;
    if (!seen) out[n++] = s;
  }
  size_t most = 0;
  for (int k = 0; k < n; ++k) {
    const size_t tiles = (size_t(c.T) + out[k] - 1) / out[k];
    most = std::max(most, tiles * kTileWords * size_t(out[k]));
  }
  if (floats) *floats = std::max<size_t>(most, 1);
  return n;
}

cudaError_t set_tile_layout(Context& c, int tile_tets) {
  const size_t tiles = (size_t(c.T) + tile_tets - 1) / tile_tets;
  if (tiles * kTileWords * size_t(tile_tets) > c.tile_capacity) return cudaErrorInvalidValue;
  c.tile_tets = tile_tets;
  c.tile_magic = tile_magic_of(tile_tets);
  c.num_tiles = int(tiles);
  // tiles that do not fit in L2 stream from HBM in every sweep
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) == cudaSuccess)
    c.stream_tiles = tiles * kTileWords * size_t(tile_tets) * sizeof(float) > size_t(l2);
  if (c.T == 0) return cudaSuccess;
  const int nb = (c.T + 255) / 256;
  // padding tets of the last tile: node 0, no stiffness (never computed)
  cudaError_t e = cudaMemsetAsync(c.tile_f, 0, sizeof(float) * kTileWords * tiles * size_t(tile_tets), c.stream);
  if (e != cudaSuccess) return e;
  k_prepare<<<nb, 256, 0, c.stream>>>(c.T, c.tets, c.Bv, c.D, c.V, c.b_f, c.c_f, c.b_d, c.c_d, c.tile_f,
                                      c.tile_tets);
  k_tile_quats_from_re<<<nb, 256, 0, c.stream>>>(c.T, c.re_f, c.tile_f, c.tile_tets);
  return cudaGetLastError();
}

// The search: the patch variants (single meshes; they do not read the
// tiles) once, the tiled variants (tets, staged) at every candidate tile
// size, each as the best of 3 timings of 4 back-to-back sweeps after one
// warm-up sweep; the fastest combination wins.  Representative operands:
// identity orientations and the node positions.  Batches time masked
// sweeps (every fourth mesh, as late in a step) of the variants that take
// masks.
cudaError_t autotune_apply(Context& c) {
  if (c.T == 0) return cudaSuccess;
  int nb = (c.T + 255) / 256, nbn = (c.N + 255) / 256 > 0 ? (c.N + 255) / 256 : 1;
  k_identity_f32<<<nb, 256, 0, c.stream>>>(c.T, c.re_f, c.tile_f, c.tile_tets);
  k_pack_operand<float4><<<nbn, 256, 0, c.stream>>>(c.N, c.fixed, c.x, c.p_f, c.p_lo, c.q_f);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  if (c.num_meshes > 1) {
    std::vector<unsigned char> mask(size_t(3) * c.num_meshes, 0);
    for (int m = 0; m < c.num_meshes; m += 4) mask[size_t(m)] = 1;
    e = cudaMemcpy(c.bmask, mask.data(), mask.size(), cudaMemcpyHostToDevice);
  }
  auto time_sweep = [&](float* best_ms) -> cudaError_t {
    *best_ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaError_t r = launch_apply_sweeps(c, OTFEM_SOLVER_MIXED, 0.01, 1, true);
      if (r != cudaSuccess) return r;
      cudaEventRecord(e0, c.stream);
      if ((r = launch_apply_sweeps(c, OTFEM_SOLVER_MIXED, 0.01, 4, true)) != cudaSuccess) return r;
      cudaEventRecord(e1, c.stream);
      if ((r = cudaEventSynchronize(e1)) != cudaSuccess) return r;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      *best_ms = std::min(*best_ms, ms / 4.f);
    }
    return cudaSuccess;
  };
  c.tune_rows = 0;
  for (int v = 0; v < kApplyVariants; ++v) c.apply_ms[v] = 0.0;
  int cand[5];
  const int nc = tile_candidates(c, cand, nullptr);
  const int balanced = cand[0];
  int best_v = -1, best_tt = balanced;
  float best = 1e30f;
  auto record = [&](int v, int tt, float ms) {
    if (c.tune_rows < Context::kMaxTuneRows) {
      c.tune_variant[c.tune_rows] = v;
      c.tune_tile[c.tune_rows] = tt;
      c.tune_ms[c.tune_rows] = ms;
      ++c.tune_rows;
    }
    if (c.apply_ms[v] <= 0.0 || ms < c.apply_ms[v]) c.apply_ms[v] = ms;
    if (ms < best) best = ms, best_v = v, best_tt = tt;
  };
  if (c.num_meshes == 1)
    for (int v = kApplyAtomics; v <= kApplyGather && e == cudaSuccess; ++v) {
      c.apply_variant = v;
      float ms;
      if ((e = time_sweep(&ms)) == cudaSuccess) record(v, 0, ms);
    }
  for (int k = 0; k < nc && e == cudaSuccess; ++k) {
    if ((e = set_tile_layout(c, cand[k])) != cudaSuccess) break;
    for (int v = kApplyTets; v <= kApplyStaged && e == cudaSuccess; ++v) {
      c.apply_variant = v;
      float ms;
      if ((e = time_sweep(&ms)) == cudaSuccess) record(v, cand[k], ms);
    }
  }
  if (e == cudaSuccess) {
    c.apply_variant = best_v >= 0 ? best_v : kApplyTets;
    // the patch variants keep the balanced layout (the tiles still serve the
    // batch masks and the diagnostics)
    const int tt = best_v >= kApplyTets ? best_tt : balanced;
    if (tt != c.tile_tets) e = set_tile_layout(c, tt);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t sync_orientations(Context& c) {
  if (!c.re_f32_pending) return cudaSuccess;
  int nb = (c.T + 255) / 256;
  if (nb < 1) nb = 1;
  k_re_from_f32<<<nb, 256, 0, c.stream>>>(c.T, c.re_f, c.Re);
  c.re_f32_pending = false;
  return cudaGetLastError();
}

static void fill_args(MixedArgs& a, Context& c, double dt, const otfem_solver_params& prm) {
  a = MixedArgs();
  a.N = c.N;
  a.T = c.T;
  a.tets = c.tets;
  a.fixed = c.fixed;
  a.inc_ptr = c.inc_ptr;
  a.inc_ent = c.inc_ent;
  a.tet_force = c.elastic_force;
  a.g_f = c.g_f;
  a.mass = c.mass;
  a.fext = c.fext;
  a.x = c.x;
  a.v = c.v;
  a.bvec = c.bvec;
  a.r = c.r;
  a.p = c.p;
  a.diag = c.diag;
  a.diag_f = c.diag_f;
  a.diag_lo = c.diag_lo;
  a.b_hi = c.b_hi;
  a.b_lo = c.b_lo;
  a.node_k = c.node_k;
  a.precond = prm.preconditioner == OTFEM_PRECONDITIONER_JACOBI ? 1 : 0;
  a.re_f = c.re_f;
  a.b_f = c.b_f;
  a.c_f = c.c_f;
  a.p_f = c.p_f;
  a.v_f = c.v_f;
  a.q_f = c.q_f;
  a.p_lo = c.p_lo;
  a.v_lo = c.v_lo;
  a.r_f = c.r_f;
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
  set_patch_args(a, c);
  a.tile_f = c.tile_f;
  a.tile_tets = c.tile_tets;
  a.num_tiles = c.num_tiles;
  a.tile_magic = c.tile_magic;
  a.ordered_sums = prm.sequential_dots ? 1 : 0;
  const bool learned = prm.warm_start == OTFEM_WARM_START_LEARNED && c.warm_hist != nullptr;
  a.warm_dv = learned ? c.warm_dv : nullptr;
  a.dv_last = c.dv_last;
  a.v_keep = c.v_keep;
  a.hist = c.warm_hist;
  a.wprod = c.warm_prod;
  a.wpart = c.warm_part;
  a.wbacc = c.warm_bacc;
  a.hist_k = 0;
  if (a.hist && prm.warm_start == OTFEM_WARM_START_PROJECTED) a.hist_k = prm.warm_history;
  if (a.hist && learned) a.hist_k = std::max(prm.warm_history, 1);
  // batches: the extrapolated start projects the meshes that iterate longest
  // (k_cg_batch), so their search directions are set up as for the projected start
  if (a.hist && prm.warm_start == OTFEM_WARM_START_EXTRAPOLATED && c.num_meshes > 1) a.hist_k = prm.warm_history;
  a.nwarm = a.hist_k + (learned ? 1 : 0);
  a.extrap_k = a.hist && prm.warm_start == OTFEM_WARM_START_EXTRAPOLATED ? prm.warm_history : 0;
  a.hist_fill = c.hist_fill;
  // a step records the levels it searches or sums (all of them when it uses none)
  a.hist_rec = a.hist ? (a.hist_k > 0 ? a.hist_k : (a.extrap_k > 0 ? a.extrap_k : kMaxHistory)) : 0;
  a.num_meshes = c.num_meshes;
  a.mesh_of_node = c.mesh_of_node;
  a.mesh_of_tet = c.mesh_of_tet;
  a.mesh_tet_start = c.mesh_tet_start;
  a.mesh_node_start = c.mesh_node_start;
  a.bm = c.bmesh;
  a.bacc = c.bacc;
  a.bmask = c.bmask;
  a.sweep_mask = nullptr;
  a.spin_limit = 4000000000LL;  // clock cycles, about two seconds
}

// After a persistent solve: an error the grid recorded (a timed-out wait, a
// non-finite scalar) reaches the step statistics even when the kernel left
// before writing them.
__global__ void k_merge_status(const DeviceSync* sync, DeviceStats* stats) {
  const int st = sync->status;
  if (st < 0) stats->status = st;
}

static cudaError_t merge_status(Context& c) {
  k_merge_status<<<1, 1, 0, c.stream>>>(c.sync, c.stats);
  return cudaGetLastError();
}

cudaError_t launch_mixed_solve(Context& c, double dt, const otfem_solver_params& prm) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(c.sync, 0, sizeof(DeviceSync), c.stream)) != cudaSuccess) return e;
  MixedArgs a;
  fill_args(a, c, dt, prm);
  void* args[] = {&a};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.mf_grid);
  cfg.blockDim = dim3(c.mf_block);
  cfg.dynamicSmemBytes = launch_smem(c);
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const void* fn = prm.solver == OTFEM_SOLVER_FP64 ? cg_kernel<double>() : cg_kernel<float>();
  if ((e = cudaLaunchKernelExC(&cfg, fn, args)) != cudaSuccess) return e;
  return merge_status(c);
}

// Standalone element-apply launches start the staged apply's tile tickets
// at zero, as a solver launch does.
static cudaError_t reset_tile_tickets(Context& c) {
  return cudaMemsetAsync(&c.sync->tile_ticket, 0, sizeof(unsigned), c.stream);
}

cudaError_t launch_batch_solve(Context& c, double dt, const otfem_solver_params& prm) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(c.sync, 0, sizeof(DeviceSync), c.stream)) != cudaSuccess) return e;
  if (c.warm_bacc &&
      (e = cudaMemsetAsync(c.warm_bacc, 0, sizeof(double) * (kMaxWarmSums * size_t(c.num_meshes) + 8), c.stream)) !=
          cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(c.bacc, 0, sizeof(double) * 2 * kBatchSlots * size_t(c.num_meshes), c.stream)) != cudaSuccess)
    return e;
  MixedArgs a;
  fill_args(a, c, dt, prm);
  void* args[] = {&a};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.mf_grid);
  cfg.blockDim = dim3(c.mf_block);
  cfg.dynamicSmemBytes = launch_smem(c);
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if ((e = cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(&k_cg_batch), args)) != cudaSuccess) return e;
  return merge_status(c);
}

cudaError_t launch_apply_sweeps(Context& c, int solver, double dt, int sweeps, bool masked) {
  MixedArgs a;
  otfem_solver_params prm;
  otfem_default_params(&prm);
  fill_args(a, c, dt, prm);
  if (masked && c.num_meshes > 1) a.sweep_mask = c.bmask;
  // tile tickets matter to the staged variant only (the measured launches
  // are then the sweeps alone)
  if (c.apply_variant == kApplyStaged)
    if (cudaError_t e = reset_tile_tickets(c)) return e;
  for (int k = 0; k < sweeps; ++k) {
    if (solver == OTFEM_SOLVER_FP64)
      k_apply_sweep<double><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, c.p_d4, nullptr, c.q_d);
    else
      k_apply_sweep<float><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, c.p_f, nullptr, c.q_f);
  }
  return cudaGetLastError();
}

cudaError_t launch_apply_operator(Context& c, int solver, double dt, double mass_damping, const double* x,
                                  double* y) {
  MixedArgs a;
  otfem_solver_params prm;
  otfem_default_params(&prm);
  fill_args(a, c, dt, prm);
  if (cudaError_t e = reset_tile_tickets(c)) return e;
  int nb = (c.N + 255) / 256 > 0 ? (c.N + 255) / 256 : 1;
  if (solver == OTFEM_SOLVER_FP64) {
    k_pack_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, c.v_d4, nullptr, c.q_d);
    k_apply_sweep<double><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, c.v_d4, nullptr, c.q_d);
    k_finalize_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, c.q_d, y);
  } else {
    k_pack_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, c.v_f, c.v_lo, c.q_f);
    k_apply_sweep<float><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, c.v_f, c.v_lo, c.q_f);
    k_finalize_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, c.q_f, y);
  }
  return cudaGetLastError();
}

cudaError_t launch_apply_operator_scratch(Context& c, int solver, double dt, double mass_damping,
                                          const double* x, double* y, void* scratch) {
  MixedArgs a;
  otfem_solver_params prm;
  otfem_default_params(&prm);
  fill_args(a, c, dt, prm);
  if (cudaError_t e = reset_tile_tickets(c)) return e;
  int nb = (c.N + 255) / 256 > 0 ? (c.N + 255) / 256 : 1;
  if (solver == OTFEM_SOLVER_FP64) {
    double4* u = static_cast<double4*>(scratch);
    double4* q = u + c.N;
    k_pack_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, u, nullptr, q);
    k_apply_sweep<double><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, u, nullptr, q);
    k_finalize_operand<double4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, q, y);
  } else {
    float4* u = static_cast<float4*>(scratch);
    float4* ulo = u + c.N;
    float4* q = ulo + c.N;
    k_pack_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, x, u, ulo, q);
    k_apply_sweep<float><<<c.mf_grid, kBlock, launch_smem(c), c.stream>>>(a, u, ulo, q);
    k_finalize_operand<float4><<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.mass, dt, mass_damping, x, q, y);
  }
  return cudaGetLastError();
}

}  // namespace otfem
