// otfem_api.cu -- the C ABI of libotfem_gpu.so (include/otfem_gpu.h): context
// lifetime, host<->device transfers, and the step orchestration, replayed
// from a CUDA graph per (solver, dt, warp, parameters) key.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "otfem_internal.h"

using otfem::Context;

struct otfem_context {
  Context c;
};

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace otfem {
Context* context_of(otfem_handle h) { return h ? &h->c : nullptr; }
int record_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
}  // namespace otfem

namespace {

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(OTFEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define OT_CUDA(call)                                                  \
  do {                                                                 \
    cudaError_t e_ = (call);                                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);                \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count > 0 ? count : 1));
}

void free_all(Context& c) {
  void* ptrs[] = {c.tets, c.x, c.x0, c.v, c.fext, c.mass, c.f0, c.b, c.fixed, c.prev, c.update,
                  c.residual, c.node_dots, c.scal, c.Ke, c.Re, c.V, c.E, c.Bv, c.D, c.plastic,
                  c.young, c.poisson, c.density, c.yield, c.creep, c.cmax, c.tet_force, c.elastic_force, c.inc_ptr,
                  c.inc_ent, c.row_ptr, c.cols, c.bc_ptr, c.bc_ent, c.K, c.A, c.re_f, c.b_f, c.c_f, c.tile_f,
                  c.re_d, c.b_d, c.c_d, c.e0_f, c.diag, c.diag_f, c.diag_lo, c.b_hi, c.b_lo, c.node_k, c.r, c.p, c.bvec, c.p_f, c.v_f, c.q_f, c.p_lo, c.v_lo, c.r_f, c.g_f, c.dv_last, c.warm_dv, c.warm_tmp, c.v_keep, c.features, c.q_d,
                  c.p_d4, c.v_d4, c.partials, c.sync, c.trace, c.stats, c.patch_node_ptr, c.patch_nodes, c.lconn,
                  c.patch_inc_ptr, c.patch_inc};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c.stats_host) cudaFreeHost(c.stats_host);
  if (c.bmesh_host) cudaFreeHost(c.bmesh_host);
  void* batch[] = {c.mesh_of_node, c.mesh_of_tet, c.mesh_tet_start, c.mesh_node_start, c.bmesh, c.bacc, c.bmask,
                   c.warm_hist, c.warm_prod, c.warm_part, c.warm_bacc, c.hist_fill};
  for (void* p : batch)
    if (p) cudaFree(p);
  if (c.graph) cudaGraphExecDestroy(c.graph);
  if (c.own_stream && c.stream) cudaStreamDestroy(c.stream);
  if (c.host_graph) cudaGraphExecDestroy(c.host_graph);
  if (c.io_stream) cudaStreamDestroy(c.io_stream);
  if (c.io_fork) cudaEventDestroy(c.io_fork);
  if (c.io_join) cudaEventDestroy(c.io_join);
}

double* node_field(Context& c, int field) {
  switch (field) {
    case OTFEM_COORD: return c.x;
    case OTFEM_MODEL_COORD: return c.x0;
    case OTFEM_VELOCITY: return c.v;
    case OTFEM_F_EXTERNAL: return c.fext;
    case OTFEM_MASS: return c.mass;
    case OTFEM_F0: return c.f0;
    case OTFEM_B: return c.last_solver == OTFEM_SOLVER_REFERENCE ? c.b : c.bvec;
    case OTFEM_NODE_STIFFNESS: return c.node_k;
    default: return nullptr;
  }
}

int64_t field_count(Context& c, int field) {
  return field == OTFEM_MASS || field == OTFEM_NODE_STIFFNESS ? int64_t(c.N) : 3 * int64_t(c.N);
}

int check_params(const Context& c, const otfem_solver_params& p) {
  if (p.solver < OTFEM_SOLVER_REFERENCE || p.solver > OTFEM_SOLVER_FP64)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown solver");
  if (p.max_iterations < 0 || p.min_iterations < 0)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "iteration counts must be non-negative");
  if (p.solver != OTFEM_SOLVER_REFERENCE && !(p.rtol >= 0.0))
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "rtol must be non-negative");
  if (p.warm_start != OTFEM_WARM_START_PREVIOUS && p.warm_start != OTFEM_WARM_START_LEARNED &&
      p.warm_start != OTFEM_WARM_START_PROJECTED && p.warm_start != OTFEM_WARM_START_EXTRAPOLATED)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown warm start");
  if (p.warm_history < 0 || p.warm_history > OTFEM_MAX_WARM_HISTORY)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "warm_history out of range");
  if (p.preconditioner != OTFEM_PRECONDITIONER_NONE && p.preconditioner != OTFEM_PRECONDITIONER_JACOBI)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown preconditioner");
  if (c.num_meshes > 1 && p.solver != OTFEM_SOLVER_MIXED)
    return fail(OTFEM_ERR_UNSUPPORTED, "a batch of meshes steps with OTFEM_SOLVER_MIXED (one CG per mesh)");
  if (p.warm_start == OTFEM_WARM_START_LEARNED && p.solver != OTFEM_SOLVER_MIXED)
    return fail(OTFEM_ERR_UNSUPPORTED, "the learned warm start runs with OTFEM_SOLVER_MIXED");
  if (p.warm_start == OTFEM_WARM_START_PROJECTED && p.solver != OTFEM_SOLVER_MIXED)
    return fail(OTFEM_ERR_UNSUPPORTED, "the projected start runs with OTFEM_SOLVER_MIXED");
  if (p.warm_start == OTFEM_WARM_START_PROJECTED && p.warm_history < 1)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "the projected start needs warm_history >= 1");
  if (p.warm_start == OTFEM_WARM_START_EXTRAPOLATED && p.solver != OTFEM_SOLVER_MIXED)
    return fail(OTFEM_ERR_UNSUPPORTED, "the extrapolated start runs with OTFEM_SOLVER_MIXED");
  if (p.warm_start == OTFEM_WARM_START_EXTRAPOLATED && p.warm_history < 1)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "the extrapolated start needs warm_history >= 1");
  if (p.warm_start == OTFEM_WARM_START_LEARNED && !c.mlp)
    return fail(OTFEM_ERR_NOT_INITIALIZED, "learned warm start without a network (otfem_set_mlp)");
  return OTFEM_OK;
}

// The projected and learned starts search previous velocity changes and
// the extrapolated start sums them: their history, the products and sums are
// allocated (the history and its fill count zeroed) by the first step that
// needs them; from then on every mixed step of the mesh records its velocity
// change.
cudaError_t ensure_history(Context& c, const otfem_solver_params& p) {
  const bool needs = p.solver == OTFEM_SOLVER_MIXED &&
                     (p.warm_start == OTFEM_WARM_START_PROJECTED || p.warm_start == OTFEM_WARM_START_LEARNED ||
                      p.warm_start == OTFEM_WARM_START_EXTRAPOLATED);
  if (!needs || c.warm_hist) return cudaSuccess;
  const size_t n = size_t(c.N > 0 ? c.N : 1);
  cudaError_t e;
  if ((e = cudaMalloc(&c.warm_hist, sizeof(float4) * 2 * otfem::kMaxHistory * n)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&c.warm_prod, sizeof(float4) * (otfem::kMaxWarmDirs + 1) * n)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&c.warm_part, sizeof(double) * otfem::kMaxWarmSums * size_t(c.mf_grid))) != cudaSuccess)
    return e;
  if (c.num_meshes > 1 &&
      (e = cudaMalloc(&c.warm_bacc, sizeof(double) * (otfem::kMaxWarmSums * size_t(c.num_meshes) + 8))) !=
          cudaSuccess)
    return e;
  if ((e = cudaMalloc(&c.hist_fill, sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(c.hist_fill, 0, sizeof(int), c.stream)) != cudaSuccess) return e;
  return cudaMemsetAsync(c.warm_hist, 0, sizeof(float4) * 2 * otfem::kMaxHistory * n, c.stream);
}

// A step that records no velocity change (the reference and FP64 solvers,
// the reference's stages) leaves the history without the newest change:
// the extrapolated start starts over.
cudaError_t history_gap(Context& c) {
  return c.hist_fill ? cudaMemsetAsync(c.hist_fill, 0, sizeof(int), c.stream) : cudaSuccess;
}

// After the orientation phase of a matrix-free step: the network inputs of
// the nodes (when collecting training samples) and the learned initial guess.
cudaError_t launch_warm_start(Context& c, const otfem_solver_params& p) {
  const bool predict = p.warm_start == OTFEM_WARM_START_LEARNED;
  c.features_valid = c.collect != 0;
  if (!predict && !c.collect) return cudaSuccess;
  return otfem::launch_node_features(c, predict);
}

// Enqueues one step on c.stream (no host synchronisation).
// The matrix-free step's orientation phase (orientation, element forces,
// plasticity, the learned start's inputs) and its solve (K2), which
// enqueue_step runs back to back.
cudaError_t enqueue_orient(Context& c, double dt, bool warp, const otfem_solver_params& p) {
  cudaError_t e = otfem::launch_mixed_orient(c, dt, warp, p.solver);
  return e != cudaSuccess ? e : launch_warm_start(c, p);
}
cudaError_t enqueue_solve(Context& c, double dt, const otfem_solver_params& p) {
  if (p.solver == OTFEM_SOLVER_FP64) {
    cudaError_t e = history_gap(c);
    if (e != cudaSuccess) return e;
  }
  return c.num_meshes > 1 ? otfem::launch_batch_solve(c, dt, p) : otfem::launch_mixed_solve(c, dt, p);
}

cudaError_t enqueue_step(Context& c, double dt, bool warp, const otfem_solver_params& p) {
  cudaError_t e;
  if (p.solver == OTFEM_SOLVER_REFERENCE) {
    // fem_simulate.h:94-112
    if ((e = otfem::launch_orientation(c, warp)) != cudaSuccess) return e;
    if ((e = otfem::launch_assembly(c)) != cudaSuccess) return e;
    if ((e = otfem::launch_plasticity(c, dt)) != cudaSuccess) return e;
    if ((e = otfem::launch_dynamics_assembly(c, p.mass_damping, dt)) != cudaSuccess) return e;
    if ((e = otfem::launch_reference_cg(c, p.min_iterations, p.max_iterations, p.sequential_dots != 0)) !=
        cudaSuccess)
      return e;
    if ((e = otfem::launch_position_update(c, dt)) != cudaSuccess) return e;
    if ((e = history_gap(c)) != cudaSuccess) return e;
  } else {
    if ((e = enqueue_orient(c, dt, warp, p)) != cudaSuccess) return e;
    if ((e = enqueue_solve(c, dt, p)) != cudaSuccess) return e;
  }
  return cudaMemcpyAsync(c.stats_host, c.stats, sizeof(otfem::DeviceStats), cudaMemcpyDeviceToHost, c.stream);
}

struct HostArrays {
  double* coord;
  double* velocity;
  const double* f_external;
};

// Page-locked (or registered) host memory: its copies are asynchronous and
// can be captured into a graph.
bool page_locked(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// One step on host arrays: the positions are copied in first, half on each
// stream (the orientation phase reads only them), the velocity and the
// external forces on the second stream while the orientation phase runs, and
// the solve waits for them; the new positions and velocities go back on the
// two streams at once.  Where plasticity or the learned start's inputs read the velocity or
// the forces in the orientation phase, and for the reference solver, they are
// copied before it.
cudaError_t enqueue_host_step(Context& c, double dt, bool warp, const otfem_solver_params& p, const HostArrays& io) {
  const size_t bytes = sizeof(double) * 3 * size_t(c.N);
  if (!bytes) return enqueue_step(c, dt, warp, p);
  const bool late_inputs = p.solver != OTFEM_SOLVER_REFERENCE && !c.plastic_active &&
                           p.warm_start != OTFEM_WARM_START_LEARNED && !c.collect;
  cudaError_t e;
  if (late_inputs) {
    // the positions in two halves, one per stream (two copy engines), the
    // orientation phase after both; then the velocity and forces
    const size_t half = sizeof(double) * 3 * size_t(c.N / 2);
    if ((e = cudaEventRecord(c.io_fork, c.stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(c.io_stream, c.io_fork, 0)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.x, io.coord, half, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(reinterpret_cast<char*>(c.x) + half, reinterpret_cast<const char*>(io.coord) + half,
                             bytes - half, cudaMemcpyHostToDevice, c.io_stream)) != cudaSuccess)
      return e;
    if ((e = cudaEventRecord(c.io_join, c.io_stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(c.stream, c.io_join, 0)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.v, io.velocity, bytes, cudaMemcpyHostToDevice, c.io_stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.fext, io.f_external, bytes, cudaMemcpyHostToDevice, c.io_stream)) != cudaSuccess)
      return e;
    if ((e = cudaEventRecord(c.io_join, c.io_stream)) != cudaSuccess) return e;
    if ((e = enqueue_orient(c, dt, warp, p)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(c.stream, c.io_join, 0)) != cudaSuccess) return e;
    if ((e = enqueue_solve(c, dt, p)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.stats_host, c.stats, sizeof(otfem::DeviceStats), cudaMemcpyDeviceToHost, c.stream)) !=
        cudaSuccess)
      return e;
  } else {
    if ((e = cudaMemcpyAsync(c.x, io.coord, bytes, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.v, io.velocity, bytes, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.fext, io.f_external, bytes, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return e;
    if ((e = enqueue_step(c, dt, warp, p)) != cudaSuccess) return e;
  }
  if ((e = cudaEventRecord(c.io_fork, c.stream)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(c.io_stream, c.io_fork, 0)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(io.velocity, c.v, bytes, cudaMemcpyDeviceToHost, c.io_stream)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(io.coord, c.x, bytes, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(c.io_join, c.io_stream)) != cudaSuccess) return e;
  return cudaStreamWaitEvent(c.stream, c.io_join, 0);
}

std::string step_key(const Context& c, double dt, bool warp, const otfem_solver_params& p) {
  char buf[320];
  snprintf(buf, sizeof(buf), "%d|%a|%d|%a|%d|%d|%a|%d|%d|%d|%d|%d|%p|%p|%d|%d", p.solver, dt, int(warp),
           p.mass_damping, p.min_iterations, p.max_iterations, p.rtol, p.refresh_period, p.sequential_dots,
           p.warm_start, p.preconditioner, p.warm_history, static_cast<void*>(c.mlp),
           static_cast<void*>(c.warm_hist), c.collect, c.warm_smoothing);
  return buf;
}

int kernels_per_step(const Context& c, const otfem_solver_params& p) {
  if (p.solver == OTFEM_SOLVER_REFERENCE) return 1 + 2 + 2 + 1 + (1 + 5 * p.max_iterations + 1) + 1;
  const bool learned = p.warm_start == OTFEM_WARM_START_LEARNED;
  const bool features = learned || c.collect;
  // orientation, persistent solve, status merge; plasticity; network inputs
  // and the smoothing passes of the learned start
  return 3 + (c.plastic_active ? 2 : 0) + (features ? 1 : 0) + (learned ? c.warm_smoothing : 0);
}

}  // namespace

extern "C" {

void otfem_default_params(otfem_solver_params* p) {
  if (!p) return;
  p->solver = OTFEM_SOLVER_REFERENCE;
  p->mass_damping = 2.0;
  p->min_iterations = 20;
  p->max_iterations = 20;
  p->rtol = 1e-6;
  p->refresh_period = 16;
  p->sequential_dots = 0;
  p->warm_start = OTFEM_WARM_START_PREVIOUS;
  p->graph = 1;
  p->preconditioner = OTFEM_PRECONDITIONER_JACOBI;
  p->warm_history = 4;
}

const char* otfem_last_error(void) { return g_last_error.c_str(); }
int otfem_abi_version(void) { return OTFEM_ABI_VERSION; }

int otfem_create(const otfem_mesh_desc* d, void* stream, otfem_handle* out) {
  if (!d || !out) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (d->num_nodes < 0 || d->num_tets < 0) return fail(OTFEM_ERR_INVALID_ARGUMENT, "negative size");
  if ((d->num_tets > 0 && !d->tets) || (d->num_nodes > 0 && !d->coord))
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "missing tets or coord");
  if (int64_t(d->num_tets) * 16 > 0x7fffffffLL) return fail(OTFEM_ERR_INVALID_ARGUMENT, "too many tets");
  // t4mesh_t4mesh.h:139-144 and :232 (verify_nodes): indices in range and distinct
  for (int64_t t = 0; t < d->num_tets; ++t) {
    const int32_t* n = d->tets + 4 * t;
    for (int a = 0; a < 4; ++a) {
      if (n[a] < 0 || n[a] >= d->num_nodes)
        return fail(OTFEM_ERR_BAD_MESH, "tet " + std::to_string(t) + " has a node index out of range");
      for (int b = 0; b < a; ++b)
        if (n[a] == n[b]) return fail(OTFEM_ERR_BAD_MESH, "tet " + std::to_string(t) + " repeats a node");
    }
  }
  otfem_context* h = new (std::nothrow) otfem_context;
  if (!h) return fail(OTFEM_ERR_OUT_OF_MEMORY, "host allocation failed");
  Context& c = h->c;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  c.N = d->num_nodes;
  c.T = d->num_tets;
  const size_t N = size_t(c.N), T = size_t(c.T);
  int rc = OTFEM_OK;
  auto bail = [&](cudaError_t e, const char* what) {
    rc = cuda_fail(e, what);
    free_all(c);
    delete h;
    return rc;
  };
  cudaError_t e;
#define OT_ALLOC(ptr, n) \
  if ((e = dalloc(&(ptr), (n))) != cudaSuccess) return bail(e, "cudaMalloc " #ptr);
  if ((e = cudaGetDevice(&c.device)) != cudaSuccess) return bail(e, "cudaGetDevice");
  if (!c.stream) {
    // A stream of our own: the legacy default stream cannot be captured into
    // the step graph.  It synchronises with the legacy default stream.
    if ((e = cudaStreamCreate(&c.stream)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    c.own_stream = true;
  }
  if ((e = cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, c.device)) != cudaSuccess)
    return bail(e, "cudaDeviceGetAttribute");
  OT_ALLOC(c.tets, T);
  OT_ALLOC(c.x, 3 * N);
  OT_ALLOC(c.x0, 3 * N);
  OT_ALLOC(c.v, 3 * N);
  OT_ALLOC(c.fext, 3 * N);
  OT_ALLOC(c.mass, N);
  OT_ALLOC(c.f0, 3 * N);
  OT_ALLOC(c.b, 3 * N);
  OT_ALLOC(c.fixed, N);
  OT_ALLOC(c.prev, 3 * N);
  OT_ALLOC(c.update, 3 * N);
  OT_ALLOC(c.residual, 3 * N);
  OT_ALLOC(c.node_dots, 2 * N);
  OT_ALLOC(c.scal, 8);
  OT_ALLOC(c.Ke, 144 * T);
  OT_ALLOC(c.Re, 9 * T);
  OT_ALLOC(c.V, T);
  OT_ALLOC(c.E, 9 * T);
  OT_ALLOC(c.Bv, 12 * T);
  OT_ALLOC(c.D, 3 * T);
  OT_ALLOC(c.plastic, 6 * T);
  OT_ALLOC(c.young, T);
  OT_ALLOC(c.poisson, T);
  OT_ALLOC(c.density, T);
  OT_ALLOC(c.yield, T);
  OT_ALLOC(c.creep, T);
  OT_ALLOC(c.cmax, T);
  OT_ALLOC(c.tet_force, 12 * T);
  OT_ALLOC(c.elastic_force, 12 * T);
  OT_ALLOC(c.re_f, 9 * T);
  OT_ALLOC(c.b_f, 9 * T);
  OT_ALLOC(c.c_f, 3 * T);
  OT_ALLOC(c.e0_f, 18 * T);
  OT_ALLOC(c.re_d, 9 * T);
  OT_ALLOC(c.b_d, 9 * T);
  OT_ALLOC(c.c_d, 3 * T);
  OT_ALLOC(c.diag, N);
  OT_ALLOC(c.diag_f, N);
  OT_ALLOC(c.diag_lo, N);
  OT_ALLOC(c.b_hi, N);
  OT_ALLOC(c.b_lo, N);
  OT_ALLOC(c.node_k, N);
  OT_ALLOC(c.r, 3 * N);
  OT_ALLOC(c.p, 3 * N);
  OT_ALLOC(c.bvec, 3 * N);
  OT_ALLOC(c.p_f, N);
  OT_ALLOC(c.v_f, N);
  OT_ALLOC(c.q_f, N);
  OT_ALLOC(c.p_lo, N);
  OT_ALLOC(c.v_lo, N);
  OT_ALLOC(c.r_f, N);
  OT_ALLOC(c.dv_last, N);
  OT_ALLOC(c.v_keep, 4 * size_t(N));
  OT_ALLOC(c.warm_dv, N);
  OT_ALLOC(c.g_f, 4 * T);
  OT_ALLOC(c.q_d, N);
  OT_ALLOC(c.p_d4, N);
  OT_ALLOC(c.v_d4, N);
  OT_ALLOC(c.sync, 1);
  OT_ALLOC(c.trace, size_t(otfem::kTraceCols) * (otfem::kTraceRows + 1));  // + the phase stamps
  cudaMemsetAsync(c.trace, 0, sizeof(double) * otfem::kTraceCols * (otfem::kTraceRows + 1), c.stream);
  OT_ALLOC(c.stats, 1);
  if ((e = cudaMallocHost(reinterpret_cast<void**>(&c.stats_host), sizeof(otfem::DeviceStats))) != cudaSuccess)
    return bail(e, "cudaMallocHost");
  memset(c.stats_host, 0, sizeof(otfem::DeviceStats));
  if ((e = otfem::build_patches(c, d->tets)) != cudaSuccess) return bail(e, "build_patches");
  otfem::mixed_grid_shape(c, &c.mf_grid, &c.mf_block);
  otfem::staged_tiles(c);
  {
    int cand[5];
    otfem::tile_candidates(c, cand, &c.tile_capacity);
  }
  OT_ALLOC(c.tile_f, c.tile_capacity);
  OT_ALLOC(c.partials, size_t(otfem::kMaxPartials) * c.mf_grid);

  // zero-initialised node members (math_vector3.h:63-66) and uploads
  const size_t bytes3 = sizeof(double) * 3 * N;
  if ((e = cudaMemsetAsync(c.v, 0, bytes3, c.stream)) != cudaSuccess) return bail(e, "memset");
  cudaMemsetAsync(c.fext, 0, bytes3, c.stream);
  cudaMemsetAsync(c.f0, 0, bytes3, c.stream);
  cudaMemsetAsync(c.b, 0, bytes3, c.stream);
  cudaMemsetAsync(c.prev, 0, bytes3, c.stream);
  cudaMemsetAsync(c.update, 0, bytes3, c.stream);
  cudaMemsetAsync(c.residual, 0, bytes3, c.stream);
  cudaMemsetAsync(c.mass, 0, sizeof(double) * N, c.stream);
  cudaMemsetAsync(c.fixed, 0, N > 0 ? N : 1, c.stream);
  cudaMemsetAsync(c.plastic, 0, sizeof(double) * 6 * T, c.stream);
  cudaMemsetAsync(c.sync, 0, sizeof(otfem::DeviceSync), c.stream);
  cudaMemsetAsync(c.stats, 0, sizeof(otfem::DeviceStats), c.stream);
  if (T && (e = cudaMemcpyAsync(c.tets, d->tets, sizeof(int4) * T, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
    return bail(e, "upload tets");
  if (N) {
    if ((e = cudaMemcpyAsync(c.x, d->coord, bytes3, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return bail(e, "upload coord");
    const double* mc = d->model_coord ? d->model_coord : d->coord;
    if ((e = cudaMemcpyAsync(c.x0, mc, bytes3, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return bail(e, "upload model coord");
    if (d->fixed && (e = cudaMemcpyAsync(c.fixed, d->fixed, N, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return bail(e, "upload fixed");
  }
  if ((e = otfem::build_incidence(c)) != cudaSuccess) return bail(e, "build_incidence");
  if ((e = otfem::build_pattern(c)) != cudaSuccess) return bail(e, "build_pattern");
  OT_ALLOC(c.K, 9 * size_t(c.nnz));
  OT_ALLOC(c.A, 9 * size_t(c.nnz));
  cudaMemsetAsync(c.K, 0, sizeof(double) * 9 * size_t(c.nnz), c.stream);
  cudaMemsetAsync(c.A, 0, sizeof(double) * 9 * size_t(c.nnz), c.stream);
  if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return bail(e, "create sync");
#undef OT_ALLOC
  *out = h;
  return OTFEM_OK;
}

int otfem_destroy(otfem_handle h) {
  if (!h) return OTFEM_OK;
  cudaStreamSynchronize(h->c.stream);
  free_all(h->c);
  delete h;
  return OTFEM_OK;
}

int otfem_num_nodes(otfem_handle h, int32_t* n) {
  if (!h || !n) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *n = h->c.N;
  return OTFEM_OK;
}

int otfem_num_tets(otfem_handle h, int32_t* t) {
  if (!h || !t) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *t = h->c.T;
  return OTFEM_OK;
}

// fem_uniform_young.h:32, fem_uniform_poisson.h:33-34, fem_uniform_density.h:27,
// fem_initialize_plastic.h:42-44 (debug asserts in the reference)
static bool material_ok(double young, double poisson, double density) {
  return young >= 0.0 && poisson >= 0.0 && poisson <= 0.5 && density > 0.0;
}

// fem::init with uniform materials, or per tet (device arrays) when given.
static int init_impl(Context& c, double young, double poisson, double density, double c_yield, double c_creep,
                     double c_max, const double* young_t, const double* poisson_t, const double* density_t) {
  if (!(c_yield >= 0.0) || !(c_creep >= 0.0) || !(c_max >= 0.0))
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "material parameter out of range");
  cudaError_t e;
  if ((e = otfem::launch_init_elements(c, young, poisson, density, c_yield, c_creep, c_max, young_t, poisson_t,
                                       density_t)) != cudaSuccess)
    return cuda_fail(e, "init elements");
  if ((e = otfem::mixed_prepare(c)) != cudaSuccess) return cuda_fail(e, "prepare");
  // clear_stiffness_assembly (fem_init.h:60)
  OT_CUDA(cudaMemsetAsync(c.f0, 0, sizeof(double) * 3 * size_t(c.N), c.stream));
  if (c.k_assembled) OT_CUDA(cudaMemsetAsync(c.K, 0, sizeof(double) * 9 * size_t(c.nnz), c.stream));
  // no velocity history yet (learned warm start)
  OT_CUDA(cudaMemsetAsync(c.dv_last, 0, sizeof(float4) * size_t(c.N), c.stream));
  OT_CUDA(cudaMemsetAsync(c.warm_dv, 0, sizeof(float4) * size_t(c.N), c.stream));
  if (c.warm_hist)
    OT_CUDA(cudaMemsetAsync(c.warm_hist, 0, sizeof(float4) * 2 * otfem::kMaxHistory * size_t(c.N), c.stream));
  if (c.hist_fill) OT_CUDA(cudaMemsetAsync(c.hist_fill, 0, sizeof(int), c.stream));
  // choose the element-apply variant for this mesh
  if ((e = otfem::autotune_apply(c)) != cudaSuccess) return cuda_fail(e, "autotune");
  std::vector<double> vol(size_t(c.T));
  if (c.T) OT_CUDA(cudaMemcpyAsync(vol.data(), c.V, sizeof(double) * c.T, cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  c.plastic_active = c_creep > 0.0 && c_max > 0.0;
  c.initialized = true;
  drop_step_graphs(c);
  // fem_initialize_stiffness_elements.h:48
  for (int t = 0; t < c.T; ++t)
    if (!(vol[t] > 0.0))
      return fail(OTFEM_ERR_BAD_MESH, "tet " + std::to_string(t) + " has non-positive volume");
  return OTFEM_OK;
}

int otfem_init(otfem_handle h, double young, double poisson, double density, double c_yield,
               double c_creep, double c_max) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  if (!material_ok(young, poisson, density)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "material parameter out of range");
  return init_impl(h->c, young, poisson, density, c_yield, c_creep, c_max, nullptr, nullptr, nullptr);
}

int otfem_batch_create(const otfem_mesh_desc* meshes, int32_t count, void* stream, otfem_handle* out) {
  if (!meshes || count < 1 || !out) return fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  *out = nullptr;
  int64_t N = 0, T = 0;
  for (int m = 0; m < count; ++m) {
    const otfem_mesh_desc& d = meshes[m];
    if (d.num_nodes < 0 || d.num_tets < 0 || (d.num_tets > 0 && !d.tets) || (d.num_nodes > 0 && !d.coord))
      return fail(OTFEM_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(m) + ": bad descriptor");
    N += d.num_nodes;
    T += d.num_tets;
  }
  if (N > INT32_MAX || T > INT32_MAX) return fail(OTFEM_ERR_INVALID_ARGUMENT, "batch too large");
  std::vector<int32_t> tets(size_t(4) * T);
  std::vector<double> coord(size_t(3) * N), model(size_t(3) * N);
  std::vector<uint8_t> fixed(size_t(N), 0);
  std::vector<int> noff(size_t(count) + 1, 0), toff(size_t(count) + 1, 0);
  for (int m = 0; m < count; ++m) {
    const otfem_mesh_desc& d = meshes[m];
    const int n0 = noff[m], t0 = toff[m];
    for (int64_t k = 0; k < 4LL * d.num_tets; ++k) {
      if (d.tets[k] < 0 || d.tets[k] >= d.num_nodes)
        return fail(OTFEM_ERR_BAD_MESH, "mesh " + std::to_string(m) + ": node index out of range");
      tets[size_t(4) * t0 + k] = d.tets[k] + n0;
    }
    const double* mc = d.model_coord ? d.model_coord : d.coord;
    std::copy(d.coord, d.coord + 3 * d.num_nodes, coord.begin() + 3 * size_t(n0));
    std::copy(mc, mc + 3 * d.num_nodes, model.begin() + 3 * size_t(n0));
    if (d.fixed) std::copy(d.fixed, d.fixed + d.num_nodes, fixed.begin() + n0);
    noff[m + 1] = n0 + d.num_nodes;
    toff[m + 1] = t0 + d.num_tets;
  }
  otfem_mesh_desc all = {int32_t(N), int32_t(T), tets.data(), coord.data(), model.data(), fixed.data()};
  int rc = otfem_create(&all, stream, out);
  if (rc != OTFEM_OK) return rc;
  Context& c = (*out)->c;
  c.num_meshes = count;
  c.mesh_node_off = noff;
  c.mesh_tet_off = toff;
  std::vector<int> mon(size_t(std::max<int64_t>(N, 1))), mot(size_t(std::max<int64_t>(T, 1)));
  for (int m = 0; m < count; ++m) {
    for (int i = noff[m]; i < noff[m + 1]; ++i) mon[size_t(i)] = m;
    for (int t = toff[m]; t < toff[m + 1]; ++t) mot[size_t(t)] = m;
  }
  cudaError_t e = cudaMalloc(&c.mesh_of_node, sizeof(int) * mon.size());
  if (e == cudaSuccess) e = cudaMalloc(&c.mesh_of_tet, sizeof(int) * mot.size());
  if (e == cudaSuccess) e = cudaMalloc(&c.mesh_tet_start, sizeof(int) * toff.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(c.mesh_tet_start, toff.data(), sizeof(int) * toff.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c.mesh_node_start, sizeof(int) * noff.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(c.mesh_node_start, noff.data(), sizeof(int) * noff.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c.bmesh, sizeof(otfem::BatchMesh) * size_t(count));
  if (e == cudaSuccess) e = cudaMallocHost(&c.bmesh_host, sizeof(otfem::BatchMesh) * size_t(count));
  if (e == cudaSuccess) e = cudaMalloc(&c.bacc, sizeof(double) * 16 * size_t(count));
  if (e == cudaSuccess) e = cudaMalloc(&c.bmask, 3 * size_t(count));
  if (e == cudaSuccess) e = cudaMemcpy(c.mesh_of_node, mon.data(), sizeof(int) * mon.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c.mesh_of_tet, mot.data(), sizeof(int) * mot.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(c.bmesh, 0, sizeof(otfem::BatchMesh) * size_t(count));
  if (e != cudaSuccess) {
    otfem_destroy(*out);
    *out = nullptr;
    return cuda_fail(e, "batch arrays");
  }
  return OTFEM_OK;
}

int otfem_batch_init(otfem_handle h, const double* young, const double* poisson, const double* density,
                     double c_yield, double c_creep, double c_max) {
  if (!h || !young || !poisson || !density) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  const int M = c.num_meshes;
  for (int m = 0; m < M; ++m)
    if (!material_ok(young[m], poisson[m], density[m]))
      return fail(OTFEM_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(m) + ": material parameter out of range");
  std::vector<double> e_t(size_t(std::max(c.T, 1))), nu_t(e_t.size()), rho_t(e_t.size());
  for (int m = 0; m < M; ++m) {
    const int t0 = M > 1 ? c.mesh_tet_off[m] : 0, t1 = M > 1 ? c.mesh_tet_off[m + 1] : c.T;
    for (int t = t0; t < t1; ++t) e_t[size_t(t)] = young[m], nu_t[size_t(t)] = poisson[m], rho_t[size_t(t)] = density[m];
  }
  double* d = nullptr;
  const size_t n = e_t.size();
  OT_CUDA(cudaMalloc(&d, sizeof(double) * 3 * n));
  cudaError_t e = cudaMemcpy(d, e_t.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, nu_t.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + 2 * n, rho_t.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  int rc = e == cudaSuccess ? init_impl(c, 0.0, 0.0, 1.0, c_yield, c_creep, c_max, d, d + n, d + 2 * n)
                            : cuda_fail(e, "batch materials");
  cudaStreamSynchronize(c.stream);
  cudaFree(d);
  return rc;
}

int otfem_batch_layout(otfem_handle h, int32_t* count, int32_t* node_offsets, int32_t* tet_offsets) {
  if (!h || !count) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  const Context& c = h->c;
  *count = c.num_meshes;
  for (int m = 0; m <= c.num_meshes; ++m) {
    const bool single = c.num_meshes == 1;
    if (node_offsets) node_offsets[m] = single ? (m ? c.N : 0) : c.mesh_node_off[m];
    if (tet_offsets) tet_offsets[m] = single ? (m ? c.T : 0) : c.mesh_tet_off[m];
  }
  return OTFEM_OK;
}

int otfem_batch_stats(otfem_handle h, int32_t* iterations, int32_t* status, double* rel_residual,
                      double* initial_rel_residual) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (c.num_meshes < 2 || !c.bmesh) return fail(OTFEM_ERR_INVALID_ARGUMENT, "not a batch of meshes");
  const int M = c.num_meshes;
  OT_CUDA(cudaMemcpyAsync(c.bmesh_host, c.bmesh, sizeof(otfem::BatchMesh) * M, cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  for (int m = 0; m < M; ++m) {
    const otfem::BatchMesh& b = c.bmesh_host[m];
    const double bb = b.bnorm2 > 0.0 ? b.bnorm2 : 1.0;
    if (iterations) iterations[m] = b.iterations;
    if (status) status[m] = b.status;
    if (rel_residual) rel_residual[m] = std::sqrt(b.rho / bb);
    if (initial_rel_residual) initial_rel_residual[m] = std::sqrt(b.rho0 / bb);
  }
  return OTFEM_OK;
}

static int transfer(otfem_handle h, int field, double* ptr, int64_t count, bool to_device, cudaMemcpyKind kind) {
  if (!h || (!ptr && count)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  double* d = node_field(c, field);
  if (!d) return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown field");
  if (to_device && field > OTFEM_F_EXTERNAL) return fail(OTFEM_ERR_INVALID_ARGUMENT, "field is read-only");
  if (count != field_count(c, field)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "count does not match the field size");
  if (!count) return OTFEM_OK;
  size_t bytes = sizeof(double) * size_t(count);
  if (to_device) {
    OT_CUDA(cudaMemcpyAsync(d, ptr, bytes, kind, c.stream));
    // the mixed solver's rest edges follow the model coordinates
    if (field == OTFEM_MODEL_COORD) OT_CUDA(otfem::mixed_rest_edges(c));
  } else {
    OT_CUDA(cudaMemcpyAsync(ptr, d, bytes, kind, c.stream));
    if (kind == cudaMemcpyDeviceToHost) OT_CUDA(cudaStreamSynchronize(c.stream));
  }
  return OTFEM_OK;
}

int otfem_set_nodes(otfem_handle h, int field, const double* src, int64_t count) {
  return transfer(h, field, const_cast<double*>(src), count, true, cudaMemcpyHostToDevice);
}
int otfem_get_nodes(otfem_handle h, int field, double* dst, int64_t count) {
  return transfer(h, field, dst, count, false, cudaMemcpyDeviceToHost);
}
int otfem_set_nodes_device(otfem_handle h, int field, const double* src, int64_t count) {
  return transfer(h, field, const_cast<double*>(src), count, true, cudaMemcpyDeviceToDevice);
}
int otfem_get_nodes_device(otfem_handle h, int field, double* dst, int64_t count) {
  return transfer(h, field, dst, count, false, cudaMemcpyDeviceToDevice);
}
int otfem_get_nodes_async(otfem_handle h, int field, double* dst, int64_t count) {
  // cudaMemcpyDefault: the copy direction follows from the pointers; transfer()
  // waits only for cudaMemcpyDeviceToHost
  return transfer(h, field, dst, count, false, cudaMemcpyDefault);
}

int otfem_set_fixed(otfem_handle h, const uint8_t* fixed, int64_t count) {
  if (!h || (!fixed && count)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  if (count != h->c.N) return fail(OTFEM_ERR_INVALID_ARGUMENT, "count does not match the node count");
  if (count) OT_CUDA(cudaMemcpyAsync(h->c.fixed, fixed, size_t(count), cudaMemcpyHostToDevice, h->c.stream));
  return OTFEM_OK;
}

int otfem_simulate_ex(otfem_handle h, double dt, int warp, const otfem_solver_params* params,
                      otfem_step_stats* stats) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (!(dt > 0.0)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "time step must be positive");
  otfem_solver_params p;
  if (params) p = *params;
  else otfem_default_params(&p);
  int rc = check_params(c, p);
  if (rc != OTFEM_OK) return rc;
  cudaError_t e0 = ensure_history(c, p);
  if (e0 != cudaSuccess) return cuda_fail(e0, "warm-start history");
  bool use_warp = warp != 0;
  cudaError_t e;
  if (p.graph) {
    std::string key = step_key(c, dt, use_warp, p);
    if (!c.graph || key != c.graph_key) {
      if (c.graph) {
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      OT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t ee = enqueue_step(c, dt, use_warp, p);
      cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
      if (ee != cudaSuccess) return cuda_fail(ee, "capture step");
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&c.graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      c.graph_key = key;
    }
    OT_CUDA(cudaGraphLaunch(c.graph, c.stream));
  } else {
    if ((e = enqueue_step(c, dt, use_warp, p)) != cudaSuccess) return cuda_fail(e, "enqueue step");
  }
  if (p.solver == OTFEM_SOLVER_REFERENCE) c.k_assembled = true;
  c.last_solver = p.solver;
  c.launches += kernels_per_step(c, p);
  if (stats) return otfem_last_stats(h, stats);
  return OTFEM_OK;
}

int otfem_simulate(otfem_handle h, double dt, int warp) { return otfem_simulate_ex(h, dt, warp, nullptr, nullptr); }

int otfem_simulate_host(otfem_handle h, double dt, int warp, const otfem_solver_params* params,
                        otfem_step_stats* stats, double* coord, double* velocity, const double* f_external) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (!(dt > 0.0)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "time step must be positive");
  const int64_t n3 = 3 * int64_t(c.N);
  if (n3 && (!coord || !velocity || !f_external)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  otfem_solver_params p;
  if (params) p = *params;
  else otfem_default_params(&p);
  int rc = check_params(c, p);
  if (rc != OTFEM_OK) return rc;
  cudaError_t e0 = ensure_history(c, p);
  if (e0 != cudaSuccess) return cuda_fail(e0, "warm-start history");
  if (!c.io_stream) {
    OT_CUDA(cudaStreamCreateWithFlags(&c.io_stream, cudaStreamNonBlocking));
    OT_CUDA(cudaEventCreateWithFlags(&c.io_fork, cudaEventDisableTiming));
    OT_CUDA(cudaEventCreateWithFlags(&c.io_join, cudaEventDisableTiming));
  }
  const HostArrays io{coord, velocity, f_external};
  const bool use_warp = warp != 0;
  cudaError_t e;
  // one graph for page-locked arrays (pageable copies cannot be captured)
  if (p.graph && n3 && page_locked(coord) && page_locked(velocity) && page_locked(f_external)) {
    char ptrs[80];
    snprintf(ptrs, sizeof(ptrs), "|%p|%p|%p", static_cast<void*>(coord), static_cast<void*>(velocity),
             static_cast<const void*>(f_external));
    const std::string key = step_key(c, dt, use_warp, p) + ptrs;
    if (!c.host_graph || key != c.host_graph_key) {
      if (c.host_graph) {
        cudaGraphExecDestroy(c.host_graph);
        c.host_graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      OT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t ee = enqueue_host_step(c, dt, use_warp, p, io);
      cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
      if (ee != cudaSuccess) return cuda_fail(ee, "capture step");
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&c.host_graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      c.host_graph_key = key;
    }
    OT_CUDA(cudaGraphLaunch(c.host_graph, c.stream));
  } else if ((e = enqueue_host_step(c, dt, use_warp, p, io)) != cudaSuccess) {
    return cuda_fail(e, "enqueue step");
  }
  if (p.solver == OTFEM_SOLVER_REFERENCE) c.k_assembled = true;
  c.last_solver = p.solver;
  c.launches += kernels_per_step(c, p);
  otfem_step_stats local;
  return otfem_last_stats(h, stats ? stats : &local);
}

int otfem_simulate_phase(otfem_handle h, double dt, int warp, const otfem_solver_params* params, int phase) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (!(dt > 0.0)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "time step must be positive");
  otfem_solver_params p;
  if (params) p = *params;
  else otfem_default_params(&p);
  int rc = check_params(c, p);
  if (rc != OTFEM_OK) return rc;
  if (p.solver == OTFEM_SOLVER_REFERENCE) return fail(OTFEM_ERR_UNSUPPORTED, "phases exist for the matrix-free solvers");
  cudaError_t e0 = ensure_history(c, p);
  if (e0 != cudaSuccess) return cuda_fail(e0, "warm-start history");
  cudaError_t e;
  if (phase == OTFEM_PHASE_ORIENT) {
    if ((e = otfem::launch_mixed_orient(c, dt, warp != 0, p.solver)) != cudaSuccess) return cuda_fail(e, "orient phase");
    c.launches += 1 + (c.plastic_active ? 2 : 0);
    if ((e = launch_warm_start(c, p)) != cudaSuccess) return cuda_fail(e, "warm start");
    if (p.warm_start == OTFEM_WARM_START_LEARNED || c.collect) c.launches += 1;
    if (p.warm_start == OTFEM_WARM_START_LEARNED) c.launches += c.warm_smoothing;
  } else if (phase == OTFEM_PHASE_SOLVE) {
    e = enqueue_solve(c, dt, p);
    if (e != cudaSuccess) return cuda_fail(e, "solve phase");
    OT_CUDA(cudaMemcpyAsync(c.stats_host, c.stats, sizeof(otfem::DeviceStats), cudaMemcpyDeviceToHost, c.stream));
    c.launches += 2;
    c.last_solver = p.solver;
  } else {
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown phase");
  }
  return OTFEM_OK;
}

int otfem_last_stats(otfem_handle h, otfem_step_stats* s) {
  if (!h || !s) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  OT_CUDA(cudaStreamSynchronize(c.stream));
  const otfem::DeviceStats& d = *c.stats_host;
  s->iterations = d.iterations;
  s->applies = d.applies;
  s->status = d.status;
  s->bnorm = d.bb > 0 ? sqrt(d.bb) : 0.0;
  double ref = d.bb > 0 ? d.bb : 1.0;
  s->rel_residual = sqrt(d.rr / ref);
  s->initial_rel_residual = sqrt(d.rr0 / ref);
  if (d.status < 0) {
    const char* what = d.status == OTFEM_ERR_TIMEOUT ? "a device-side wait timed out"
                       : d.status == OTFEM_ERR_NONFINITE ? "non-finite or non-positive CG scalar"
                                                          : "device error";
    return fail(d.status, what);
  }
  if (d.status > 0) g_last_error = "CG reached max_iterations before rtol";
  return d.status;
}

int otfem_synchronize(otfem_handle h) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  OT_CUDA(cudaStreamSynchronize(h->c.stream));
  return OTFEM_OK;
}

int otfem_update_original_coord(otfem_handle h) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (c.N) OT_CUDA(cudaMemcpyAsync(c.x0, c.x, sizeof(double) * 3 * size_t(c.N), cudaMemcpyDeviceToDevice, c.stream));
  OT_CUDA(otfem::mixed_rest_edges(c));
  return OTFEM_OK;
}

int otfem_export_k_csr(otfem_handle h, int64_t* nnz_blocks, int32_t* row_ptr, int32_t* col_idx, double* values) {
  if (!h || !nnz_blocks) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  int* cnt = nullptr;
  OT_CUDA(dalloc(&cnt, size_t(c.N) + 1));
  cudaError_t e = otfem::launch_export_k_counts(c, cnt);
  std::vector<int> hc(size_t(c.N) + 1, 0), hp(size_t(c.N) + 1, 0);
  if (e == cudaSuccess && c.N) e = cudaMemcpyAsync(hc.data(), cnt, sizeof(int) * c.N, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    cudaFree(cnt);
    return cuda_fail(e, "export counts");
  }
  for (int i = 0; i < c.N; ++i) hp[i + 1] = hp[i] + hc[i];
  *nnz_blocks = hp[c.N];
  if (!row_ptr || !col_idx || !values) {
    cudaFree(cnt);
    return OTFEM_OK;
  }
  int* dcols = nullptr;
  double* dvals = nullptr;
  e = dalloc(&dcols, size_t(hp[c.N]));
  if (e == cudaSuccess) e = dalloc(&dvals, 9 * size_t(hp[c.N]));
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, hp.data(), sizeof(int) * (c.N + 1), cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = otfem::launch_export_k(c, cnt, dcols, dvals);
  if (e == cudaSuccess && hp[c.N])
    e = cudaMemcpyAsync(col_idx, dcols, sizeof(int) * hp[c.N], cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && hp[c.N])
    e = cudaMemcpyAsync(values, dvals, sizeof(double) * 9 * size_t(hp[c.N]), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  cudaFree(cnt);
  if (dcols) cudaFree(dcols);
  if (dvals) cudaFree(dvals);
  if (e != cudaSuccess) return cuda_fail(e, "export fill");
  memcpy(row_ptr, hp.data(), sizeof(int) * (size_t(c.N) + 1));
  return OTFEM_OK;
}

int otfem_k_pattern(otfem_handle h, int64_t* nnz_blocks, int32_t* row_ptr, int32_t* col_idx) {
  if (!h || !nnz_blocks) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  *nnz_blocks = c.nnz;
  if (!row_ptr || !col_idx) return OTFEM_OK;
  OT_CUDA(cudaMemcpyAsync(row_ptr, c.row_ptr, sizeof(int) * (size_t(c.N) + 1), cudaMemcpyDeviceToHost, c.stream));
  if (c.nnz) OT_CUDA(cudaMemcpyAsync(col_idx, c.cols, sizeof(int) * size_t(c.nnz), cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  return OTFEM_OK;
}

int otfem_k_values(otfem_handle h, double* vals) {
  if (!h || (!vals && h->c.nnz)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  if (c.nnz) OT_CUDA(cudaMemcpyAsync(vals, c.K, sizeof(double) * 9 * size_t(c.nnz), cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  return OTFEM_OK;
}

int otfem_a_values(otfem_handle h, double* vals) {
  if (!h || (!vals && h->c.nnz)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  if (c.nnz) OT_CUDA(cudaMemcpyAsync(vals, c.A, sizeof(double) * 9 * size_t(c.nnz), cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  return OTFEM_OK;
}

// One step of fem::simulate (fem_simulate.h:94-111) on its own, with the
// reference solver's kernels and arithmetic order.
int otfem_reference_stage(otfem_handle h, int stage, double dt, double mass_damping, int32_t min_iterations,
                          int32_t max_iterations) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (c.num_meshes > 1) return fail(OTFEM_ERR_UNSUPPORTED, "the reference's steps run on single meshes");
  const bool needs_dt = stage == OTFEM_STAGE_ADD_PLASTICITY_FORCE || stage == OTFEM_STAGE_DYNAMICS_ASSEMBLY ||
                        stage == OTFEM_STAGE_POSITION_UPDATE;
  if (needs_dt && !(dt > 0.0)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "time step must be positive");
  // a cached matrix-free step graph stays valid: the stages write the same
  // node arrays a step reads at its start
  cudaError_t e = cudaSuccess;
  switch (stage) {
    case OTFEM_STAGE_CLEAR_STIFFNESS_ASSEMBLY:
      e = cudaMemsetAsync(c.f0, 0, sizeof(double) * 3 * size_t(c.N), c.stream);
      if (e == cudaSuccess && c.nnz) e = cudaMemsetAsync(c.K, 0, sizeof(double) * 9 * size_t(c.nnz), c.stream);
      break;
    case OTFEM_STAGE_UPDATE_ORIENTATION:
    case OTFEM_STAGE_RESET_ORIENTATION:
      e = otfem::launch_orientation(c, stage == OTFEM_STAGE_UPDATE_ORIENTATION);
      c.re_f32_pending = false;
      c.launches += 1;
      break;
    case OTFEM_STAGE_STIFFNESS_ASSEMBLY:
      e = otfem::launch_assembly(c);
      c.k_assembled = true;
      c.launches += 2;
      break;
    case OTFEM_STAGE_ADD_PLASTICITY_FORCE:
      e = otfem::launch_plasticity(c, dt);
      c.launches += 2;
      break;
    case OTFEM_STAGE_DYNAMICS_ASSEMBLY:
      e = otfem::launch_dynamics_assembly(c, mass_damping, dt);
      c.launches += 1;
      break;
    case OTFEM_STAGE_CONJUGATE_GRADIENTS:
      if (min_iterations < 0 || max_iterations < 0)
        return fail(OTFEM_ERR_INVALID_ARGUMENT, "iteration counts must not be negative");
      e = otfem::launch_reference_cg(c, min_iterations, max_iterations, true);
      c.launches += 1;
      break;
    case OTFEM_STAGE_POSITION_UPDATE:
      e = otfem::launch_position_update(c, dt);
      c.launches += 1;
      break;
    default:
      return fail(OTFEM_ERR_INVALID_ARGUMENT, "unknown stage");
  }
  if (e == cudaSuccess) e = history_gap(c);  // the reference's steps record no velocity change
  if (e != cudaSuccess) return cuda_fail(e, "reference stage");
  OT_CUDA(cudaStreamSynchronize(c.stream));
  return OTFEM_OK;
}

static int get_tet_array(otfem_handle h, const double* src, size_t per, double* dst) {
  if (!h || (!dst && h->c.T)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  if (c.T) OT_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * per * size_t(c.T), cudaMemcpyDeviceToHost, c.stream));
  OT_CUDA(cudaStreamSynchronize(c.stream));
  return OTFEM_OK;
}

int otfem_get_orientations(otfem_handle h, double* re) {
  if (h) {
    cudaError_t e = otfem::sync_orientations(h->c);
    if (e != cudaSuccess) return cuda_fail(e, "orientations");
  }
  return get_tet_array(h, h ? h->c.Re : nullptr, 9, re);
}
int otfem_get_plastic(otfem_handle h, double* pl) { return get_tet_array(h, h ? h->c.plastic : nullptr, 6, pl); }
int otfem_get_volumes(otfem_handle h, double* vol) { return get_tet_array(h, h ? h->c.V : nullptr, 1, vol); }

int otfem_apply_operator(otfem_handle h, int solver, double dt, double mass_damping, const double* x,
                         double* y) {
  if (!h || !x || !y) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (solver != OTFEM_SOLVER_MIXED && solver != OTFEM_SOLVER_FP64)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "solver must be OTFEM_SOLVER_MIXED or OTFEM_SOLVER_FP64");
  size_t bytes = sizeof(double) * 3 * size_t(c.N);
  double *dx = nullptr, *dy = nullptr;
  OT_CUDA(dalloc(&dx, 3 * size_t(c.N)));
  cudaError_t e = dalloc(&dy, 3 * size_t(c.N));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = otfem::launch_apply_operator(c, solver, dt, mass_damping, dx, dy);
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  cudaFree(dx);
  if (dy) cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(e, "apply operator");
  c.launches += 3;
  return OTFEM_OK;
}

int otfem_apply_sweeps(otfem_handle h, int solver, double dt, int32_t sweeps) {
  if (!h || sweeps < 0) return fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  if (solver != OTFEM_SOLVER_MIXED && solver != OTFEM_SOLVER_FP64)
    return fail(OTFEM_ERR_INVALID_ARGUMENT, "solver must be OTFEM_SOLVER_MIXED or OTFEM_SOLVER_FP64");
  cudaError_t e = otfem::launch_apply_sweeps(c, solver, dt, sweeps);
  if (e != cudaSuccess) return cuda_fail(e, "apply sweeps");
  c.launches += sweeps;
  return OTFEM_OK;
}

int otfem_check_wait_timeout(otfem_handle h, int64_t cycles, int32_t* status) {
  if (!h || !status || cycles <= 0) return fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  int st = 0;
  cudaError_t e = otfem::check_wait_timeout(h->c, static_cast<long long>(cycles), &st);
  if (e != cudaSuccess) return cuda_fail(e, "wait timeout check");
  *status = st;
  return OTFEM_OK;
}

int otfem_solver_trace(otfem_handle h, double* out, int32_t max_rows, int32_t* rows) {
  if (!h || !rows || (!out && max_rows > 0)) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  OT_CUDA(cudaStreamSynchronize(c.stream));
  int n = c.stats_host->iterations;
  if (n > otfem::kTraceRows) n = otfem::kTraceRows;
  if (n > max_rows) n = max_rows;
  if (n > 0)
    OT_CUDA(cudaMemcpy(out, c.trace, sizeof(double) * otfem::kTraceCols * size_t(n), cudaMemcpyDeviceToHost));
  *rows = n;
  return OTFEM_OK;
}

int otfem_solver_phases(otfem_handle h, double* out) {
  if (!h || !out) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  Context& c = h->c;
  OT_CUDA(cudaStreamSynchronize(c.stream));
  OT_CUDA(cudaMemcpy(out, c.trace + size_t(otfem::kTraceCols) * otfem::kTraceRows, sizeof(double) * 8,
                     cudaMemcpyDeviceToHost));
  return OTFEM_OK;
}

int otfem_tuning(otfem_handle h, int32_t* variant, double* ms_per_variant) {
  if (!h || !variant) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *variant = h->c.apply_variant;
  if (ms_per_variant)
    for (int v = 0; v < otfem::kNumApplyVariants; ++v) ms_per_variant[v] = h->c.apply_ms[v];
  return OTFEM_OK;
}

int otfem_tuning_search(otfem_handle h, int32_t max_rows, int32_t* rows, int32_t* variant, int32_t* tile_tets,
                        double* ms, int32_t* chosen_tile_tets) {
  if (!h || !rows) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  const Context& c = h->c;
  *rows = c.tune_rows;
  for (int k = 0; k < c.tune_rows && k < max_rows; ++k) {
    if (variant) variant[k] = c.tune_variant[k];
    if (tile_tets) tile_tets[k] = c.tune_tile[k];
    if (ms) ms[k] = c.tune_ms[k];
  }
  if (chosen_tile_tets) *chosen_tile_tets = c.tile_tets;
  return OTFEM_OK;
}

int otfem_set_apply_shape(otfem_handle h, int32_t variant, int32_t tile_tets) {
  if (!h) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  Context& c = h->c;
  if (!c.initialized) return fail(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  int cand[5];
  size_t floats = 0;
  const int nc = otfem::tile_candidates(c, cand, &floats);
  bool ok = tile_tets == 0;
  for (int k = 0; k < nc; ++k) ok = ok || cand[k] == tile_tets;
  if (!ok) return fail(OTFEM_ERR_INVALID_ARGUMENT, "tile size is not one of the autotuner's candidates");
  int rc = otfem_set_apply_variant(h, variant);
  if (rc != OTFEM_OK) return rc;
  if (tile_tets != 0 && tile_tets != c.tile_tets) {
    cudaError_t e;
    if ((e = otfem::set_tile_layout(c, tile_tets)) != cudaSuccess) return cuda_fail(e, "tile layout");
  }
  return OTFEM_OK;
}

int otfem_set_apply_variant(otfem_handle h, int32_t variant) {
  if (!h || variant < 0 || variant >= otfem::kNumApplyVariants) return fail(OTFEM_ERR_INVALID_ARGUMENT, "bad variant");
  Context& c = h->c;
  if (c.num_meshes > 1 && variant < 2)
    return fail(OTFEM_ERR_UNSUPPORTED, "a batch of meshes uses apply variant 2 or 3");
  c.apply_variant = variant;
  drop_step_graphs(c);
  return OTFEM_OK;
}

int otfem_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *ptr = nullptr;
  cudaError_t e = cudaMallocHost(ptr, bytes > 0 ? bytes : 1);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
  return OTFEM_OK;
}

int otfem_host_free(void* ptr) {
  if (ptr) OT_CUDA(cudaFreeHost(ptr));
  return OTFEM_OK;
}

int otfem_launch_count(otfem_handle h, int64_t* n) {
  if (!h || !n) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *n = h->c.launches;
  return OTFEM_OK;
}

int otfem_solver_shape(otfem_handle h, int32_t* grid, int32_t* block) {
  if (!h || !grid || !block) return fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  *grid = h->c.mf_grid;
  *block = h->c.mf_block;
  return OTFEM_OK;
}

}  // extern "C"
