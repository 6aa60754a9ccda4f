// otfem_internal.h -- device-resident state of one FEM mesh and the host-side
// launch wrappers shared by the translation units of libotfem_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/otfem_gpu.h"

namespace otfem {

// Per-CTA partial sums written before a grid barrier (one slot per scalar).
constexpr int kMaxPartials = 16;
// Doubles between consecutive grid-sum accumulators (one 128-byte line each).
constexpr int kAccStride = 16;
// Projected start: velocity changes kept, and the grid sums of its Gram
// system (pairs of up to kMaxHistory + 1 directions, and their right-hand
// sides).
constexpr int kMaxHistory = OTFEM_MAX_WARM_HISTORY;
constexpr int kMaxWarmDirs = kMaxHistory + 1;
constexpr int kMaxWarmSums = kMaxWarmDirs * (kMaxWarmDirs + 1) / 2 + kMaxWarmDirs;
// Rows of the per-iteration CG trace kept per step.  Each row holds
// kTraceCols doubles: rho, p.q, alpha, beta, then SM-clock stamps (cycles
// since the kernel started, taken on CTA 0) after the apply sweep, after its
// barrier, after the reduction phase, after its grid sum, after the update
// phase and after its grid sum.
constexpr int kTraceRows = 256;
constexpr int kTraceCols = 10;

// Counters for the bounded grid barrier and the device status word.  Each
// word sits on its own 128-byte line: arrivals (atomics on `count`) do not
// contend with the CTAs polling `gen`.
struct DeviceSync {
  unsigned int count;        // monotonic arrival counter
  int status;                // 0 = OK, else an OTFEM_ERR_* / OTFEM_WARN_* code; next to the
                             // counter, so that one 8-byte load polls both
  unsigned int pad0[30];
  unsigned int gen;          // number of completed barriers (written by the last arrival)
  unsigned int pad1[31];
  double result[2][8];       // grid-sum results, double-buffered by barrier parity
  double pad3[16];
  double acc[3][8][kAccStride];  // grid-sum accumulators (FP64 reductions): three rotating
                                 // sets of 8 values, each value on its own 128-byte line
  unsigned tile_ticket;      // staged apply: monotonic tile tickets
  unsigned pad5[31];
  double wacc[kMaxWarmSums][kAccStride];  // projected start: Gram system totals (FP64
                                          // reductions), each on its own 128-byte line
};

// Per-mesh state of a batched solve (device memory, one per mesh).
struct BatchMesh {
  double bnorm2, rho, rho0, best_true;
  // the iteration's scalars, FP32 (FP64 instructions are slow on GB300)
  float thresh, est, prev_est, alpha, beta;
  float wgam[kMaxWarmDirs];   // projected / learned start: the mesh's coefficients
  int active, restart, stalls, iterations, applies, status, converged, pad;
  int best_buf;  // which kept iterate (v_keep) has the smallest true residual
  int stalled;   // stopped at the precision floor: the kept iterate is the result
};

// Statistics written by the step kernels (device memory).
struct DeviceStats {
  int iterations;
  int status;
  int applies;     // element-apply sweeps (initial residual, iterations, refreshes)
  int pad;
  double rr;       // squared residual norm at exit (free rows)
  double rr0;      // squared residual of the initial guess
  double bb;       // squared norm of b (free rows)
};

// Everything a mesh keeps on the device.  Node vectors are packed xyz
// doubles; per-tet matrices row-major.  Arrays named *_f are FP32 copies used
// by the matrix-free apply, stored structure-of-arrays (component c of tet t
// at [c*T + t]) so that a warp's loads are coalesced.
struct Context;
// Accessors for the allocation-free entry point (otfem_noalloc.cu): the
// handle's context, and setting the message otfem_last_error returns.
Context* context_of(otfem_handle h);
int record_error(int code, const std::string& msg);

struct Context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;            // stream created by otfem_create
  // otfem_simulate_host: a second stream for the copies that overlap the
  // orientation phase and each other, the events that fork and join it, and
  // the step graph of page-locked host arrays (created by the first call)
  cudaStream_t io_stream = nullptr;
  cudaEvent_t io_fork = nullptr, io_join = nullptr;
  cudaGraphExec_t host_graph = nullptr;
  std::string host_graph_key;
  int N = 0, T = 0;
  bool initialized = false;
  bool k_assembled = false;
  bool plastic_active = false;

  // mesh and node fields (fem_node_traits.h:37-52)
  int4* tets = nullptr;
  double *x = nullptr, *x0 = nullptr, *v = nullptr, *fext = nullptr, *mass = nullptr;
  double *f0 = nullptr, *b = nullptr;
  unsigned char* fixed = nullptr;
  // reference-solver CG vectors (persist between steps like the node members)
  double *prev = nullptr, *update = nullptr, *residual = nullptr;
  double* node_dots = nullptr;  // 2*N per-node dot products for the reductions
  double* scal = nullptr;       // device scalars of the reference CG

  // tet fields (fem_tetrahedron_traits.h:18-49)
  double *Ke = nullptr, *Re = nullptr, *V = nullptr, *E = nullptr /*e10,e20,e30*/;
  double *Bv = nullptr, *D = nullptr, *plastic = nullptr;
  double *young = nullptr, *poisson = nullptr, *density = nullptr;
  double *yield = nullptr, *creep = nullptr, *cmax = nullptr;
  double* tet_force = nullptr;      // 12*T scratch: per-tet plastic node forces
  double* elastic_force = nullptr;  // 12*T: per-tet elastic node forces (matrix-free rhs)

  // node -> incident (tet, slot) lists, ascending tet index
  int* inc_ptr = nullptr;  // N+1
  int* inc_ent = nullptr;  // 4T entries tet*4+slot
  // K_row pattern (ascending columns) and per-block contribution lists
  int64_t nnz = 0;
  int* row_ptr = nullptr;
  int* cols = nullptr;
  int* bc_ptr = nullptr;  // nnz+1
  int* bc_ent = nullptr;  // 16T entries tet*16 + li*4 + lj, ascending tet
  double *K = nullptr, *A = nullptr;

  // matrix-free data
  float *re_f = nullptr, *b_f = nullptr, *c_f = nullptr;  // 9T, 9T, 3T
  float* e0_f = nullptr;                                  // 18T: rest edges x0_k - x0_0 as (hi, lo) pairs (k_rest_edges)
  double *re_d = nullptr, *b_d = nullptr, *c_d = nullptr;  // 9T, 9T, 3T (FP64 apply)
  double* diag = nullptr;                                 // N: m(1+dt*alpha)
  float* diag_f = nullptr;                                // N: the same as (hi, lo) FP32 pairs
  float* diag_lo = nullptr;                               // N
  float4* b_hi = nullptr;                                 // N: b as (hi, lo) FP32 pairs
  float4* b_lo = nullptr;                                 // N
  double* node_k = nullptr;  // N: tr(sum_e Ke_ii) / 3 over the node's tets (Jacobi preconditioner), from init
  double *r = nullptr, *p = nullptr, *bvec = nullptr;    // 3N
  float4 *p_f = nullptr, *v_f = nullptr, *q_f = nullptr;  // N (p_f/v_f: high part, w = free flag)
  float4 *p_lo = nullptr, *v_lo = nullptr;                // N: low parts, x - double(float(x))
  float4* r_f = nullptr;                                   // N: mixed-solver residual
  float4* g_f = nullptr;                                   // 4T: mixed elastic node forces
  bool re_f32_pending = false;  // the FP64 m_Re copy lags the FP32 orientations
  bool quat_in_g_f = false;     // g_f[4t + k].w holds quaternion component k of tet t (mixed orientation)
  double4* q_d = nullptr;                                  // N (FP64 apply accumulator)
  double4 *p_d4 = nullptr, *v_d4 = nullptr;               // N (FP64 apply operands)
  double* partials = nullptr;                              // kMaxPartials * max grid
  // patches: contiguous ranges of kPatchTets tets, each with its sorted set of
  // nodes (bit 31 set when another patch touches the node too) and the tets'
  // connectivity as patch-local 16-bit indices
  int num_patches = 0, patch_max_nodes = 0;
  int* patch_node_ptr = nullptr;  // num_patches + 1
  int* patch_nodes = nullptr;
  ushort4* lconn = nullptr;       // T
  int* patch_inc_ptr = nullptr;   // per patch node (+1): offsets into patch_inc
  unsigned short* patch_inc = nullptr;  // 4T entries (patch-local tet << 2) | slot
  // staged apply: tiles of tile_tets consecutive tets, each stored as 20
  // word arrays of tile_tets entries (node ids, rotation quaternion, b_1..b_3,
  // c0..c2), copied to shared memory whole by the bulk-copy engine
  float* tile_f = nullptr;
  int num_tiles = 0, tile_tets = 0;
  int tile_balanced = 0;  // the tile size that splits the tets evenly over the persistent grid (staged_tiles)
  unsigned long long tile_magic = 0;  // tile_magic_of(tile_tets)
  // learned warm start: the velocity change of the last matrix-free step,
  // the network's initial guess for the next, the per-node network inputs
  // of the last step (kept when collecting training samples) and the
  // attached network
  float4* dv_last = nullptr;      // N (w unused)
  float4* warm_dv = nullptr;      // N
  float4* warm_tmp = nullptr;     // N, allocated with smoothing passes
  // projected and learned starts of one mesh (allocated by the first step
  // that uses them): the velocity-change history as a difference basis
  // (D_0 = the last change, D_j = its j-th backward difference; (hi, lo)
  // float pairs, hi.w = 1 on free nodes), the products of the search
  // directions with A, the network's correction as a direction, and per-CTA
  // partial sums of the Gram system
  float4* warm_hist = nullptr;    // 2 kMaxHistory x N: hi parts, then lo parts
  // the number of history levels that hold backward differences of the last
  // steps' velocity changes (device; the extrapolated start's degree limit)
  int* hist_fill = nullptr;
  float4* warm_prod = nullptr;    // (kMaxWarmDirs + 1) x N: products, then the correction
  double* warm_part = nullptr;    // kMaxWarmSums x max grid
  double* warm_bacc = nullptr;    // batch: num_meshes x kMaxWarmSums (+ 8) per-mesh Gram totals
  // two kept copies of the CG iterate (hi, lo) from the true-residual
  // refreshes: a solve stopped at the precision floor returns the best one
  float4* v_keep = nullptr;       // 4N
  int warm_smoothing = 0;         // 1-ring mean passes over the network's correction
  float* features = nullptr;      // N x kFeatureStride, allocated when collecting
  int collect = 0;
  bool features_valid = false;    // c.features hold the inputs of the last step
  struct otfem_mlp_s* mlp = nullptr;
  // batch of independent meshes (otfem_batch_create): mesh m owns nodes
  // [mesh_node_off[m], mesh_node_off[m+1]) and tets [mesh_tet_off[m], ...)
  int num_meshes = 1;
  std::vector<int> mesh_node_off, mesh_tet_off;  // host, num_meshes + 1
  int* mesh_of_node = nullptr;                    // N
  int* mesh_of_tet = nullptr;                     // T
  int* mesh_tet_start = nullptr;                  // num_meshes + 1: mesh_tet_off on the device
  int* mesh_node_start = nullptr;                 // num_meshes + 1: mesh_node_off on the device
  BatchMesh* bmesh = nullptr;                     // num_meshes
  BatchMesh* bmesh_host = nullptr;                // num_meshes, pinned
  double* bacc = nullptr;                         // 2 x num_meshes x 8 accumulators
  unsigned char* bmask = nullptr;                 // 3 x num_meshes: apply, update, refresh
  size_t apply_smem = 0;          // dynamic shared memory of the apply (bytes): the most any variant needs
  size_t patch_smem[2] = {0, 0};  // that of the patch variants (atomics, gather); see launch_smem
  int apply_variant = 0;          // element-apply variant chosen by the autotuner
  bool stream_tiles = false;      // the tiles exceed L2: tiled sweeps read them past L1 (set_tile_layout)
  double apply_ms[OTFEM_NUM_APPLY_VARIANTS] = {};  // measured time of one sweep per variant (best tile size)
  // the autotuner's search (autotune_apply): every measured (variant, tile
  // size; 0 for the patch variants, which do not read tiles) and its time
  static constexpr int kMaxTuneRows = 16;
  int tune_rows = 0;
  int tune_variant[kMaxTuneRows] = {}, tune_tile[kMaxTuneRows] = {};
  double tune_ms[kMaxTuneRows] = {};
  size_t tile_capacity = 0;       // floats allocated at tile_f: the largest candidate layout
  DeviceSync* sync = nullptr;
  double* trace = nullptr;                                 // kTraceRows x kTraceCols
  DeviceStats* stats = nullptr;
  DeviceStats* stats_host = nullptr;  // pinned
  int mf_grid = 0, mf_block = 0;      // persistent CG launch shape
  int last_solver = -1;
  int64_t launches = 0;               // kernels enqueued by this handle

  // cached step graph
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
  int last_status = 0;
};

// Drops the cached step graphs (the kernels' arguments changed).
inline void drop_step_graphs(Context& c) {
  if (c.graph) cudaGraphExecDestroy(c.graph);
  if (c.host_graph) cudaGraphExecDestroy(c.host_graph);
  c.graph = nullptr;
  c.host_graph = nullptr;
  c.graph_key.clear();
  c.host_graph_key.clear();
}

// ---- pattern / incidence (otfem_pattern.cu) ------------------------------
cudaError_t build_incidence(Context& c);
// Exclusive prefix sum of n counts into out[0..n], out[n] = total.
cudaError_t prefix_sum_counts(Context& c, long n, const int* in, int* out);
cudaError_t build_pattern(Context& c);

// ---- reference-order FP64 kernels (otfem_exact.cu) ------------------------
cudaError_t launch_init_elements(Context& c, double young, double poisson, double density, double c_yield,
                                 double c_creep, double c_max, const double* young_t = nullptr,
                                 const double* poisson_t = nullptr, const double* density_t = nullptr);
cudaError_t launch_orientation(Context& c, bool warp);
cudaError_t launch_assembly(Context& c);
cudaError_t launch_plasticity(Context& c, double dt);
cudaError_t launch_dynamics_assembly(Context& c, double mass_damping, double dt);
cudaError_t launch_reference_cg(Context& c, int min_it, int max_it, bool sequential);
cudaError_t launch_position_update(Context& c, double dt);
cudaError_t launch_export_k(Context& c, int* row_ptr_out, int* cols_out, double* vals_out);
cudaError_t launch_export_k_counts(Context& c, int* row_cnt);

// ---- matrix-free solver (otfem_mixed.cu) ----------------------------------
cudaError_t mixed_prepare(Context& c);  // FP32/FP64 per-tet operands from init data
cudaError_t mixed_rest_edges(Context& c);  // the FP32 rest edges from the model coordinates
cudaError_t check_wait_timeout(Context& c, long long cycles, int* status);  // the barrier's timeout path
// Tile size of the staged apply for the persistent grid (sets tile_tets and
// num_tiles): tiles of at most kTileMaxTets tets, as even a share of the
// tets per CTA as a multiple of 16 allows.
void staged_tiles(Context& c);
// Candidate tile sizes of the autotuner's search: the balanced size of
// staged_tiles first, then 128, 256, 512 and 1024 tets (each at most once).
// Returns how many (at most 5) and, in *floats, the tile_f size the largest
// layout needs.
int tile_candidates(const Context& c, int* out, size_t* floats);
// Lays the tiles out with tile_tets tets each (tile words from the init data,
// identity rotations until the next orientation phase).
cudaError_t set_tile_layout(Context& c, int tile_tets);
// Builds the apply patches from the host connectivity (once per mesh).
cudaError_t build_patches(Context& c, const int32_t* tets_host);
cudaError_t launch_mixed_orient(Context& c, double dt, bool warp, int solver);
// Times one element-apply sweep of every variant on this mesh, the tiled
// variants at every candidate tile size, and keeps the fastest combination
// in c.apply_variant and the tile layout (synchronises the stream).
cudaError_t autotune_apply(Context& c);
constexpr int kNumApplyVariants = OTFEM_NUM_APPLY_VARIANTS;
static_assert(sizeof(Context::apply_ms) == sizeof(double) * kNumApplyVariants, "one time per apply variant");
// Learned warm start: per-node inputs (v, previous dv, f_ext, 1-ring mean
// of the 9 entries of Re) stored with this stride (floats).
constexpr int kFeatures = 18;
constexpr int kFeatureStride = 20;
// Computes the network inputs of every node for the coming solve (into
// c.features when collecting) and, with predict, the initial guess c.warm_dv
// from the attached network.  After the orientation phase.
cudaError_t launch_node_features(Context& c, bool predict);
// Staged-apply tiles: at most kTileMaxTets tets of kTileWords 32-bit words.
constexpr int kTileMaxTets = 1024;
constexpr int kTileWords = 20;

// Rotation of a unit quaternion (x, y, z, w), row-major.
__device__ __forceinline__ void quaternion_to_rotation(float4 q, float* R) {
  const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
  const float xw = q.x * q.w, yw = q.y * q.w, zw = q.z * q.w;
  R[0] = 1.f - 2.f * (yy + zz), R[1] = 2.f * (xy - zw), R[2] = 2.f * (xz + yw);
  R[3] = 2.f * (xy + zw), R[4] = 1.f - 2.f * (xx + zz), R[5] = 2.f * (yz - xw);
  R[6] = 2.f * (xz - yw), R[7] = 2.f * (yz + xw), R[8] = 1.f - 2.f * (xx + yy);
}

// t / tile_tets for 0 <= t < 2^32 and 2 <= tile_tets: the high half of
// t * magic with magic = floor((2^64 - 1) / tile_tets) + 1 (= ceil(2^64 /
// tile_tets)), exact because t * (magic - 2^64 / tile_tets) / 2^64 < 2^-32 is
// below the distance 1 / tile_tets from t / tile_tets to the next integer
// (division by invariant integers by multiplication, Granlund and
// Montgomery 1994).
__device__ __forceinline__ int tile_of(int t, unsigned long long magic) {
  return int(__umul64hi(static_cast<unsigned long long>(t), magic));
}
inline unsigned long long tile_magic_of(int tile_tets) { return ~0ull / static_cast<unsigned>(tile_tets) + 1ull; }

// Word w of tet t in the staged-apply tiles (Context::tile_f).
__device__ __forceinline__ long tile_word(int tile_tets, int t, int w) {
  const int tile = t / tile_tets;
  return (long(tile) * kTileWords + w) * tile_tets + (t - tile * tile_tets);
}

// The rotation quaternion (tile words 4..7) of tet t in tile `tile`.
__device__ __forceinline__ float4 tile_quaternion(const float* tile_f, int tile_tets, int tile, int t) {
  const float* w = tile_f + (long(tile) * kTileWords + 4) * tile_tets + (t - tile * tile_tets);
  return make_float4(w[0], w[tile_tets], w[2 * tile_tets], w[3 * tile_tets]);
}

// Writes m_Re (FP64) from the FP32 orientations of the last mixed step.
cudaError_t sync_orientations(Context& c);
cudaError_t launch_mixed_solve(Context& c, double dt, const otfem_solver_params& p);
// Batched matrix-free solve: every mesh of the batch runs its own CG (own
// scalars, convergence and iteration count) in one persistent launch.
cudaError_t launch_batch_solve(Context& c, double dt, const otfem_solver_params& prm);
// y = A x with the matrix-free apply of the given precision and the current
// orientations (x, y: device, 3 doubles per node; rows of fixed nodes = 0).
cudaError_t launch_apply_operator(Context& c, int solver, double dt, double mass_damping, const double* x, double* y);
// The same y = A x with the operand and accumulator in caller-provided
// device scratch (48 B per node FP32, 64 B per node FP64); no allocation.
cudaError_t launch_apply_operator_scratch(Context& c, int solver, double dt, double mass_damping, const double* x,
                                          double* y, void* scratch);
// `sweeps` element-apply sweeps on the resident operand (no host transfer):
// the apply kernel alone, for timing.
cudaError_t launch_apply_sweeps(Context& c, int solver, double dt, int sweeps, bool masked = false);
int mixed_grid_shape(Context& c, int* grid, int* block);

}  // namespace otfem
