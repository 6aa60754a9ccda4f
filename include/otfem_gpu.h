/*
 * otfem_gpu.h -- C ABI of libotfem_gpu.so, the GB300 (sm_103a) implementation
 * of OpenTissue's stiffness-warped tetrahedral FEM time step.
 *
 * Every function returns an int status: 0 = OK, > 0 = warning (the step ran;
 * e.g. the CG hit its iteration cap), < 0 = error.  otfem_last_error() gives
 * a thread-local message for the last non-zero status.  A handle is bound to
 * one CUDA stream and one device; calls on one handle are not thread-safe,
 * distinct handles are independent.  Pointers marked "host" are host memory,
 * pointers marked "device" are device memory on the handle's device.  Node
 * vectors are packed xyz doubles (3 per node); 3x3 matrices are row-major.
 *
 * Reference citations are relative to the OpenTissue source tree.
 */
#ifndef OTFEM_GPU_H
#define OTFEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OTFEM_ABI_VERSION 8

#if defined(__GNUC__)
#define OTFEM_API __attribute__((visibility("default")))
#else
#define OTFEM_API
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  OTFEM_OK = 0,
  OTFEM_WARN_NOT_CONVERGED = 1,  /* relative-residual CG stopped at max_iterations */
  OTFEM_ERR_INVALID_ARGUMENT = -1,
  OTFEM_ERR_BAD_MESH = -2,       /* index out of range, repeated node, non-positive volume */
  OTFEM_ERR_NOT_INITIALIZED = -3,/* otfem_init not called yet */
  OTFEM_ERR_CUDA = -4,           /* a CUDA runtime call failed */
  OTFEM_ERR_NONFINITE = -5,      /* NaN/Inf in a CG scalar */
  OTFEM_ERR_TIMEOUT = -6,        /* a bounded device-side wait gave up */
  OTFEM_ERR_OUT_OF_MEMORY = -7,
  OTFEM_ERR_UNSUPPORTED = -8
};

/* ---- node fields for otfem_set_nodes / otfem_get_nodes ------------------ */
enum {
  OTFEM_COORD = 0,       /* m_coord        (fem_node_traits.h:44) set/get */
  OTFEM_MODEL_COORD = 1, /* m_model_coord  (fem_node_traits.h:43) set/get */
  OTFEM_VELOCITY = 2,    /* m_velocity     (fem_node_traits.h:46) set/get */
  OTFEM_F_EXTERNAL = 3,  /* m_f_external   (fem_node_traits.h:48) set/get */
  OTFEM_MASS = 4,        /* m_mass, 1 double per node (fem_node_traits.h:47) get */
  OTFEM_F0 = 5,          /* m_f0           (fem_node_traits.h:39) get */
  OTFEM_B = 6,           /* m_b            (fem_node_traits.h:40) get */
  OTFEM_NODE_STIFFNESS = 7 /* 1 double per node, get: tr(sum_e Ke_ii) / 3 over the node's tets,
                              the rotation-invariant scale of its stiffness diagonal block
                              (sets the Jacobi preconditioner of the matrix-free solvers) */
};

/* ---- solver selection --------------------------------------------------- */
enum {
  /* The reference's own step (fem_simulate.h:94-112): FP64 assembled K and A
   * rows, reference operation order, CG with min/max iterations, the absolute
   * clamps tiny = 1e-10 and the d1 < 0.001 break (fem_conjugate_gradients.h). */
  OTFEM_SOLVER_REFERENCE = 0,
  /* Matrix-free step: FP32 orientation and stiffness apply (the element
   * deformations formed in (hi, lo) float pairs), FP64 positions, the
   * velocity and the right-hand side as (hi, lo) float pairs, dot products
   * and alpha/beta in float-pair arithmetic (~48-bit), residual replaced by
   * b - A v every refresh_period iterations, stop at ||r|| <= rtol*||b||.
   * One persistent CG kernel per step, replayed from a CUDA graph. */
  OTFEM_SOLVER_MIXED = 1,
  /* Matrix-free step with the FP64 stiffness apply (accuracy reference for the
   * mixed solver; FP64 throughput on GB300 is far below FP32). */
  OTFEM_SOLVER_FP64 = 2
};

enum {
  OTFEM_WARM_START_PREVIOUS = 0, /* CG starts from the previous velocity (reference) */
  /* CG starts from the point of least energy x.A.x/2 - b.x on v + span{the
   * network's correction, the last max(warm_history, 1) velocity changes};
   * the network predicts v + dv (otfem_set_mlp) */
  OTFEM_WARM_START_LEARNED = 1,
  /* CG starts from the point of least energy on v + span{the last
   * warm_history velocity changes} (projection onto previous solutions);
   * one extra element-apply per vector and step */
  OTFEM_WARM_START_PROJECTED = 2,
  /* CG starts from v + the velocity change extrapolated by the polynomial of
   * degree warm_history through the last warm_history + 1 velocities (the sum
   * of the newest change's backward differences up to order warm_history - 1;
   * the degree is lowered while fewer steps are recorded since otfem_init or
   * since a step that recorded none).  No extra element-apply.  A smooth
   * trajectory's next velocity is predicted well; after an abrupt change of
   * the motion (a velocity set by hand, a jump of the load) the start can be
   * poor for a few steps, and CG still stops at the same residual.  In a
   * batch of at most 512 meshes, a mesh whose previous solve took at least
   * half the batch's largest iteration count starts from its projected start
   * instead (larger batches: every mesh). */
  OTFEM_WARM_START_EXTRAPOLATED = 3
};

/* Velocity changes kept for the projected, learned and extrapolated starts. */
#define OTFEM_MAX_WARM_HISTORY 8

enum {
  OTFEM_PRECONDITIONER_NONE = 0,   /* plain CG (the reference's method) */
  /* CG preconditioned by the node-wise scalar 1 / (m (1 + dt alpha) + dt^2 k),
   * k = tr(sum_e Ke_ii) / 3 (OTFEM_NODE_STIFFNESS): the trace of the node's
   * diagonal block of A over 3, which rotations leave unchanged, so it is
   * computed once at init.  Same stop (||r|| <= rtol ||b||), fewer iterations
   * on stiffness-dominated steps.  Matrix-free solvers only (default). */
  OTFEM_PRECONDITIONER_JACOBI = 1
};

typedef struct otfem_solver_params {
  int solver;               /* OTFEM_SOLVER_* */
  double mass_damping;      /* Rayleigh mass coefficient; reference 2.0 (fem_simulate.h:104) */
  int min_iterations;       /* reference solver: 20 (fem_simulate.h:108) */
  int max_iterations;       /* reference: 20 (fem_simulate.h:109); matrix-free: cap */
  double rtol;              /* matrix-free: stop at ||r|| <= rtol*||b|| (free rows) */
  int refresh_period;       /* matrix-free: recompute r = b - A v every N iterations (16) */
  int sequential_dots;      /* reference solver: 1 = sum dot products in node order on one
                               thread (bit-identical to the reference), 0 = parallel tree.
                               matrix-free: the mixed solver's CG sums always add the CTA
                               totals in CTA order; 1 also orders the
                               projected start's Gram sums, the FP64 solver's and the
                               batches' sums, 0 = FP64 atomic accumulation of those */
  int warm_start;           /* OTFEM_WARM_START_* (PROJECTED, LEARNED, EXTRAPOLATED: OTFEM_SOLVER_MIXED,
                               single meshes and batches; a batch solves each mesh's own
                               search space) */
  int graph;                /* 1 = replay the step from a CUDA graph (default) */
  int preconditioner;       /* matrix-free: OTFEM_PRECONDITIONER_* (default JACOBI);
                               the reference solver ignores it */
  int warm_history;         /* projected and learned starts: previous velocity changes in the
                               search space; extrapolated start: the polynomial degree;
                               0..OTFEM_MAX_WARM_HISTORY (default 4) */
} otfem_solver_params;

typedef struct otfem_step_stats {
  int iterations;           /* CG iterations taken this step */
  int status;               /* same code the call returned */
  double rel_residual;      /* ||b - A v|| / ||b|| over free rows at exit (matrix-free) */
  double initial_rel_residual; /* same for the initial guess */
  double bnorm;             /* ||b|| over free rows */
  int applies;              /* element-apply sweeps of the step (initial residual,
                               one per iteration, one per residual refresh) */
} otfem_step_stats;

typedef struct otfem_mesh_desc {
  int32_t num_nodes;
  int32_t num_tets;
  const int32_t* tets;         /* host, 4*num_tets node indices i,j,k,m (t4mesh_t4tetrahedron.h:39) */
  const double* coord;         /* host, 3*num_nodes, m_coord */
  const double* model_coord;   /* host, 3*num_nodes, m_model_coord (NULL: = coord) */
  const uint8_t* fixed;        /* host, num_nodes, m_fixed (NULL: none fixed) */
} otfem_mesh_desc;

typedef struct otfem_context* otfem_handle;

/* Defaults: reference solver, mass damping 2, 20/20 iterations, rtol 1e-6,
 * refresh 16, parallel dots, previous-velocity warm start, graph on. */
OTFEM_API void otfem_default_params(otfem_solver_params* p);

OTFEM_API const char* otfem_last_error(void);
OTFEM_API int otfem_abi_version(void);

/* Creates the device-resident mesh (replaces building fem::Mesh, fem_mesh.h:21-34,
 * over t4mesh::T4Mesh, t4mesh.h:48-55).  stream: a cudaStream_t (NULL = the
 * library creates and owns a stream).  Builds the node->tet incidence and the K_row
 * sparsity pattern on the GPU.  The fixed flags must be final before otfem_init
 * (compute_mass reads them, fem_compute_mass.h:154-160). */
OTFEM_API int otfem_create(const otfem_mesh_desc* desc, void* stream, otfem_handle* out);
OTFEM_API int otfem_destroy(otfem_handle h);
OTFEM_API int otfem_num_nodes(otfem_handle h, int32_t* n);
OTFEM_API int otfem_num_tets(otfem_handle h, int32_t* t);

/* fem::init (fem_init.h:45-65): uniform material, element stiffness, lumped
 * mass, plasticity state. */
OTFEM_API int otfem_init(otfem_handle h, double young, double poisson, double density, double c_yield,
               double c_creep, double c_max);

/* Node field transfer (direct member access on the reference's nodes). */
OTFEM_API int otfem_set_nodes(otfem_handle h, int field, const double* host_src, int64_t count);
OTFEM_API int otfem_get_nodes(otfem_handle h, int field, double* host_dst, int64_t count);
OTFEM_API int otfem_set_nodes_device(otfem_handle h, int field, const double* device_src, int64_t count);
OTFEM_API int otfem_get_nodes_device(otfem_handle h, int field, double* device_dst, int64_t count);
/* As otfem_get_nodes without waiting: the copy is queued on the handle's
 * stream behind the work already there, and host_dst holds the values once
 * the stream has reached it (otfem_synchronize, or a later blocking call).
 * With page-locked host memory several fields download back to back with one
 * wait; with pageable memory the copy completes before the call returns. */
OTFEM_API int otfem_get_nodes_async(otfem_handle h, int field, double* host_dst, int64_t count);
OTFEM_API int otfem_set_fixed(otfem_handle h, const uint8_t* host_fixed, int64_t count);

/* fem::simulate (fem_simulate.h:49-113) with the reference's fixed solver
 * settings.  Asynchronous on the handle's stream. */
OTFEM_API int otfem_simulate(otfem_handle h, double time_step, int use_stiffness_warping);
/* The same step with explicit solver parameters; stats (optional, host) are
 * filled after a stream synchronisation. */
OTFEM_API int otfem_simulate_ex(otfem_handle h, double time_step, int use_stiffness_warping,
                      const otfem_solver_params* params, otfem_step_stats* stats);
/* fem::simulate on host arrays (fem_simulate.h:49-113 with the node fields
 * read from and written back to the reference's nodes, which the drop-in
 * headers do around each step): the same result as
 *   otfem_set_nodes(COORD, coord), otfem_set_nodes(VELOCITY, velocity),
 *   otfem_set_nodes(F_EXTERNAL, f_external), otfem_simulate_ex,
 *   otfem_get_nodes(COORD, coord), otfem_get_nodes(VELOCITY, velocity)
 * (3 * node count doubles each; returns once coord and velocity hold the new
 * state, with stats (optional) filled).  The positions are copied first; the
 * velocity and the external forces are copied on a second stream while the
 * orientation phase runs (it reads only the positions), and the two
 * downloads run at once.  With page-locked host arrays the whole step,
 * copies included, is one CUDA graph, kept per set of array addresses: keep
 * the same arrays from step to step.  With plasticity or the learned start
 * (whose orientation phase reads the velocity and forces) and with the
 * reference solver the inputs are copied before the step.  No counterpart in
 * the reference's interface: the reference's step works in the host arrays
 * themselves. */
OTFEM_API int otfem_simulate_host(otfem_handle h, double time_step, int use_stiffness_warping,
                                  const otfem_solver_params* params, otfem_step_stats* stats, double* coord,
                                  double* velocity, const double* f_external);
/* The two kernels of a matrix-free step enqueued separately (same result as
 * otfem_simulate_ex when ORIENT is followed by SOLVE), so a caller can time
 * them or insert work between them.  ORIENT: orientation, element forces and
 * plasticity; SOLVE: right-hand side, CG and position update. */
enum { OTFEM_PHASE_ORIENT = 1, OTFEM_PHASE_SOLVE = 2 };
OTFEM_API int otfem_simulate_phase(otfem_handle h, double time_step, int use_stiffness_warping,
                                   const otfem_solver_params* params, int phase);
/* Reads the statistics of the last step (synchronises the stream). */
OTFEM_API int otfem_last_stats(otfem_handle h, otfem_step_stats* stats);
OTFEM_API int otfem_synchronize(otfem_handle h);

/* fem::update_original_coord (fem_update_original_coord.h:28-33). */
OTFEM_API int otfem_update_original_coord(otfem_handle h);

/* fem::export_K (fem_export_k.h:23-68) as CSR of 3x3 blocks.  Rows of fixed
 * nodes hold one identity block; columns of fixed nodes are omitted.  Before
 * the first reference-solver step no K is assembled (empty free rows), as in
 * the reference.  Call with NULL arrays to get the block count. */
OTFEM_API int otfem_export_k_csr(otfem_handle h, int64_t* nnz_blocks, int32_t* row_ptr, int32_t* col_idx,
                       double* values);
/* The K_row key sets of all nodes (fem_node_traits.h:30-36), built on the GPU
 * at otfem_create: CSR with ascending columns.  NULL arrays: count only. */
OTFEM_API int otfem_k_pattern(otfem_handle h, int64_t* nnz_blocks, int32_t* row_ptr, int32_t* col_idx);
/* The assembled K_row values (9 doubles per pattern block) of the last
 * reference-solver step. */
OTFEM_API int otfem_k_values(otfem_handle h, double* host_values);

/* The assembled A_row values (9 doubles per pattern block, the K_row
 * pattern of otfem_k_pattern) of the last reference dynamics assembly
 * (fem_dynamics_assembly.h:79-86). */
OTFEM_API int otfem_a_values(otfem_handle h, double* host_values);

/* The steps of fem::simulate (fem_simulate.h:94-111) one at a time, for host
 * code that calls OpenTissue's fem::detail functions itself: the reference
 * solver's kernels and FP64 operation order on the device-resident mesh
 * (the CG sums its dot products in node order, bit-identical to the
 * reference).  Synchronous.  stage: */
enum {
  OTFEM_STAGE_CLEAR_STIFFNESS_ASSEMBLY = 1, /* detail::clear_stiffness_assembly (fem_clear_stiffness_assembly.h:23-33):
                                               K and f0 set to zero */
  OTFEM_STAGE_UPDATE_ORIENTATION = 2,       /* detail::update_orientation (fem_update_orientation.h:22-215) */
  OTFEM_STAGE_RESET_ORIENTATION = 3,        /* detail::reset_orientation (fem_reset_orientation.h:22-27) */
  OTFEM_STAGE_STIFFNESS_ASSEMBLY = 4,       /* detail::stiffness_assembly (fem_stiffness_assembly.h:171-209);
                                               writes K and f0 (the sums of the step, not added to
                                               values left by an assembly without a clear) */
  OTFEM_STAGE_ADD_PLASTICITY_FORCE = 5,     /* detail::add_plasticity_force (fem_add_plasticity_force.h:26-204), dt */
  OTFEM_STAGE_DYNAMICS_ASSEMBLY = 6,        /* detail::dynamics_assembly (fem_dynamics_assembly.h:47-93),
                                               mass_damping, dt: A and b */
  OTFEM_STAGE_CONJUGATE_GRADIENTS = 7,      /* detail::conjugate_gradients (fem_conjugate_gradients.h:25-133),
                                               min_iterations, max_iterations */
  OTFEM_STAGE_POSITION_UPDATE = 8           /* detail::position_update (fem_position_update.h:25-39), dt */
};
OTFEM_API int otfem_reference_stage(otfem_handle h, int stage, double dt, double mass_damping,
                                    int32_t min_iterations, int32_t max_iterations);

/* Per-tet state: m_Re (9 doubles, row-major), m_plastic (6), m_V (1). */
OTFEM_API int otfem_get_orientations(otfem_handle h, double* host_re);
OTFEM_API int otfem_get_plastic(otfem_handle h, double* host_plastic);
OTFEM_API int otfem_get_volumes(otfem_handle h, double* host_volume);

/* ---- batches of meshes (no counterpart in the reference) -----------------
 * One handle over `count` independent meshes (uneven sizes allowed), stepped
 * together by one persistent launch per step in which every mesh runs its
 * own CG (own alpha, beta, residuals and convergence; OTFEM_SOLVER_MIXED).
 * Node fields of the handle are the meshes' fields one after another
 * (otfem_batch_layout gives the offsets); otfem_last_stats reports the
 * largest iteration count and relative residual and the worst status. */
OTFEM_API int otfem_batch_create(const otfem_mesh_desc* meshes, int32_t count, void* stream, otfem_handle* out);
/* fem::init with one material per mesh (arrays of `count`). */
OTFEM_API int otfem_batch_init(otfem_handle h, const double* young, const double* poisson, const double* density,
                               double c_yield, double c_creep, double c_max);
/* Number of meshes and the first node / tet of each (count + 1 entries). */
OTFEM_API int otfem_batch_layout(otfem_handle h, int32_t* count, int32_t* node_offsets, int32_t* tet_offsets);
/* Per-mesh results of the last step (arrays of `count`, each may be NULL). */
OTFEM_API int otfem_batch_stats(otfem_handle h, int32_t* iterations, int32_t* status, double* rel_residual,
                                double* initial_rel_residual);

/* ---- learned warm start (no counterpart in the reference) ----------------
 * fem_conjugate_gradients.h:44-46 starts CG from the previous velocity.  With
 * OTFEM_WARM_START_LEARNED (OTFEM_SOLVER_MIXED only) CG starts instead from
 * v + dv_prev + net(inputs), where dv_prev is the node's velocity change of
 * the previous step and net is a node-wise MLP (inputs: v, dv_prev, f_ext
 * and the mean of the 9 entries of Re over the node's tets; 3 hidden layers
 * of 64 with GELU; BF16 tensor cores, FP32 accumulation) trained on the GPU
 * on (inputs, dv - dv_prev) pairs of converged steps.  CG runs to the same
 * relative residual either way.
 *
 * Network state (OTFEM_MLP_STATE_SIZE floats): W1[64][18], b1[64],
 * W2[64][64], b2[64], W3[64][64], b3[64], W4[3][64], b4[3] (each W as
 * weight[out][in]), then input mean[18], input std[18], target mean[3],
 * target std[3].  Outputs and targets are normalised by the target mean/std. */
#define OTFEM_MLP_STATE_SIZE 9773
typedef struct otfem_mlp_s* otfem_mlp;
/* A network with seeded random weights, identity normalisation and room for
 * `capacity` training samples on the current device. */
OTFEM_API int otfem_mlp_create(int64_t capacity, uint64_t seed, otfem_mlp* out);
OTFEM_API int otfem_mlp_destroy(otfem_mlp m);
/* Save / load the network state (weights and normalisation); loading resets
 * the optimiser state. */
OTFEM_API int otfem_mlp_get_state(otfem_mlp m, float* state, int64_t n);
OTFEM_API int otfem_mlp_set_state(otfem_mlp m, const float* state, int64_t n);
/* Training set: otfem_set_collect(h, 1) makes every matrix-free step of h
 * keep the network inputs of its nodes; otfem_mlp_add_samples then appends
 * the free nodes of h's last step (each kept with probability `fraction`,
 * by a hash of the node index and `seed`) with targets dv - dv_prev. */
OTFEM_API int otfem_set_collect(otfem_handle h, int32_t enable);
/* The network inputs of every node in the last step (out[num_nodes][18]). */
OTFEM_API int otfem_get_features(otfem_handle h, float* out, int64_t n);
OTFEM_API int otfem_mlp_add_samples(otfem_mlp m, otfem_handle h, double fraction, uint64_t seed, int64_t* total);
OTFEM_API int otfem_mlp_num_samples(otfem_mlp m, int64_t* count);
OTFEM_API int otfem_mlp_clear_samples(otfem_mlp m);
/* Sets the input and target normalisation to the training set's column means
 * and standard deviations. */
OTFEM_API int otfem_mlp_fit_normalization(otfem_mlp m);
/* Adam (beta 0.9, 0.999, eps 1e-8) on the mean squared normalised error over
 * shuffled minibatches of `batch` samples; returns the mean loss of the last
 * epoch. */
OTFEM_API int otfem_mlp_train(otfem_mlp m, int32_t epochs, int32_t batch, double learning_rate, uint64_t seed,
                              double* last_epoch_loss);
/* Mean squared normalised error over the training set. */
OTFEM_API int otfem_mlp_evaluate(otfem_mlp m, double* loss);
/* Diagnostics: loss and its gradient w.r.t. the OTFEM_MLP_STATE_SIZE - 42
 * weights over n host samples (inputs x[n][18], targets y[n][3]); and the
 * de-normalised predictions y[n][3] of n host inputs. */
OTFEM_API int otfem_mlp_gradient(otfem_mlp m, const float* x, const float* y, int64_t n, double* loss, float* grad);
OTFEM_API int otfem_mlp_predict(otfem_mlp m, const float* x, int64_t n, float* y);
/* Attaches a network to a mesh for OTFEM_WARM_START_LEARNED (NULL detaches).
 * The network must outlive its use and must not be trained while steps
 * that use it are in flight. */
OTFEM_API int otfem_set_mlp(otfem_handle h, otfem_mlp m);
/* Passes (0..64, default 0) of 1-ring mean aggregation over the network's
 * correction net(inputs) before it enters the initial guess: each pass
 * replaces a node's correction by the mean over its tets of the tet's node
 * mean.  (Smoothing lowers the initial residual of the network's guess on
 * its own; inside the projected search space it changes nothing measurable
 * and costs one node pass each.) */
OTFEM_API int otfem_set_warm_start_smoothing(otfem_handle h, int32_t passes);

/* ---- host staging (no counterpart in the reference) ---------------------- */
/* Page-locked host memory for fast transfers (used by the drop-in headers). */
OTFEM_API int otfem_host_alloc(size_t bytes, void** ptr);
OTFEM_API int otfem_host_free(void* ptr);

/* ---- diagnostics (no counterpart in the reference) ---------------------- */
/* y = A x for the matrix-free operator A = M(1 + dt*mass_damping) + dt^2 K'
 * (solver OTFEM_SOLVER_MIXED: FP32 element apply, OTFEM_SOLVER_FP64: FP64),
 * using the orientations of the last matrix-free step or ORIENT phase.
 * x, y: host, 3 doubles per node; rows of fixed nodes are returned as 0. */
OTFEM_API int otfem_apply_operator(otfem_handle h, int solver, double dt, double mass_damping, const double* x,
                                   double* y);
/* The same y = A x without allocating (no counterpart in the reference),
 * for callers that may not allocate device memory at the call: fixed-rate
 * loops, where cudaMalloc/cudaFree stall the device and take unbounded time,
 * and hosts whose device memory is owned by another allocator with a cap or
 * pool of its own.  x_device, y_device: device (or managed) arrays of 3
 * doubles per node on the handle's device, written on the handle's stream
 * and not synchronized; other pointers return OTFEM_ERR_INVALID_ARGUMENT.
 * The operand and accumulator live in one 16 MiB static device array that
 * every GPU loading the library holds until exit, so meshes are limited to
 * 262,144 nodes (larger ones return OTFEM_ERR_INVALID_ARGUMENT).  All calls
 * share that array: calls that may overlap on the GPU (other handles, other
 * streams) race; order them.  The first call on a device looks up the
 * array's device address (with that device current, which must be the
 * handle's device) and keeps it; make it before any stream capture.  A call
 * with x_device = y_device = NULL does only that set-up and returns OTFEM_OK.
 * The kept address does not survive cudaDeviceReset (which invalidates every
 * handle of the device as well). */
OTFEM_API int otfem_apply_operator_noalloc(otfem_handle h, int solver, double dt, double mass_damping,
                                           const double* x_device, double* y_device);
/* Enqueues `sweeps` element-apply sweeps q += dt^2 K' p on the resident
 * search direction of the last matrix-free step, asynchronously on the
 * handle's stream: the stiffness apply alone, for timing.  Leaves the solver
 * state unspecified until the next step. */
OTFEM_API int otfem_apply_sweeps(otfem_handle h, int solver, double dt, int32_t sweeps);
/* Runs the grid barrier's bounded wait once with nothing to release it (one
 * CTA waits for a second arrival that never comes) and a limit of `cycles` SM
 * clock cycles, and reports the status the wait recorded: OTFEM_ERR_TIMEOUT.
 * A diagnostic of the timeout path every device-side wait takes; the handle
 * stays usable.  Not during a captured step. */
OTFEM_API int otfem_check_wait_timeout(otfem_handle h, int64_t cycles, int32_t* status);
/* Convergence history of the last matrix-free step, one row of 10 doubles per
 * CG iteration (at most 256 rows): the squared residual norm (its estimate)
 * before the iteration, p.Ap (0 where the solver does not form it), alpha,
 * beta, then six stamps in SM clock cycles since the kernel started (taken by
 * the middle CTA of the grid): apply sweep done, its barrier passed,
 * reduction phase done, reduction complete, update phase done, update
 * synchronised.  For a batch, one row per iteration of its persistent launch
 * with the number of meshes still iterating in column 0 and 1 in column 2
 * where a residual-refresh sweep follows (columns 1 and 3 are 0), then the
 * same six stamps. */
OTFEM_API int otfem_solver_trace(otfem_handle h, double* out, int32_t max_rows, int32_t* rows);
/* Phases of the last OTFEM_SOLVER_MIXED solve of one mesh: 8 stamps in SM
 * clock cycles since the kernel started (middle CTA): b done, the
 * initial residual's element sweeps (and the search directions') done, the
 * start ready (projection solved), CG loop done, position update done; then,
 * for the projected and learned starts (else 0), the Gram sums begun, the
 * Gram totals in, the coefficients solved.  A batch records the first five
 * stamps for its persistent launch.  out holds 8 doubles. */
OTFEM_API int otfem_solver_phases(otfem_handle h, double* out);
/* The element-apply variant the autotuner chose for this mesh at otfem_init
 * (0: patches with shared-memory atomics, 1: patches with a deterministic
 * per-node gather, 2: one tet per thread with global reductions, 3: as 2 with
 * each tile of tets staged in shared memory by bulk copies) and the measured
 * time of one sweep of each (ms, OTFEM_NUM_APPLY_VARIANTS doubles; may be
 * NULL).  The FP64 solver runs variant 3 as 2. */
#define OTFEM_NUM_APPLY_VARIANTS 4
OTFEM_API int otfem_tuning(otfem_handle h, int32_t* variant, double* ms_per_variant);
/* Forces an element-apply variant (0..OTFEM_NUM_APPLY_VARIANTS-1) for the
 * following steps. */
OTFEM_API int otfem_set_apply_variant(otfem_handle h, int32_t variant);
/* The autotuner's search at otfem_init (no counterpart in the reference):
 * the patch variants 0 and 1 once (single meshes; tile_tets reported as 0),
 * the tiled variants 2 and 3 at every candidate tile size (the size that
 * splits the tets evenly over the persistent grid, then 128, 256, 512 and
 * 1024 tets per tile), each timed as the best of 3 x 4 sweeps; the fastest
 * combination is kept.  rows: the number of measured combinations (at most
 * 16); the first max_rows are written to variant, tile_tets and ms (each may
 * be NULL); chosen_tile_tets (may be NULL): the tile size in use. */
OTFEM_API int otfem_tuning_search(otfem_handle h, int32_t max_rows, int32_t* rows, int32_t* variant,
                                  int32_t* tile_tets, double* ms, int32_t* chosen_tile_tets);
/* Forces an element-apply variant and a tile size (one of the autotuner's
 * candidates; 0 keeps the current one) for the following steps; the tiles'
 * rotations are rebuilt from the last orientations. */
OTFEM_API int otfem_set_apply_shape(otfem_handle h, int32_t variant, int32_t tile_tets);
/* Number of kernels this handle has enqueued so far (graph replays included). */
OTFEM_API int otfem_launch_count(otfem_handle h, int64_t* count);
/* Launch shape of the persistent CG kernel (grid CTAs, threads per CTA). */
OTFEM_API int otfem_solver_shape(otfem_handle h, int32_t* grid, int32_t* block);

/* ---- mesh coupling (t4mesh::mesh_coupling, t4mesh_mesh_coupling.h) ------
 * A point set (the vertices of a render surface, say) bound to the tets of a
 * mesh and moved with them.  The surface refers to its mesh's handle, which
 * must outlive it; calls run on the mesh's stream. */
typedef struct otfem_surface_s* otfem_surface;
/* bind_surface (t4mesh_mesh_coupling.h:129-236): binds each of `count`
 * points (host, 3 doubles each) to a tet that embeds it in the mesh's current
 * coordinates, all four barycentric weights in (-1e-4, 1 + 1e-4)
 * (collision_policy::report, :84-111; weights as geometry_barycentric.h:
 * 343-385); where several tets embed a point, the lowest tet index.  Points
 * no tet embeds stay unbound, as in the reference (they keep their given
 * position in updates).  bound (may be NULL): number of bound points. */
OTFEM_API int otfem_surface_bind(otfem_handle h, const double* points, int64_t count, otfem_surface* out,
                                 int64_t* bound);
/* update_surface (:238-275): every bound point at w0 x_i + w1 x_j + w2 x_k +
 * w3 x_m of its tet's current node coordinates; host_out: 3 doubles per
 * point (synchronises); the _device form writes a device array on the mesh's
 * stream without synchronising. */
OTFEM_API int otfem_surface_update(otfem_surface s, double* host_out, int64_t count);
OTFEM_API int otfem_surface_update_device(otfem_surface s, double* device_out, int64_t count);
/* The binding as bind_surface stores it: tet index per point (-1: unbound)
 * and its `barycentric` (w1, w2, w3), the weights of the tet's nodes j, k, m
 * (node i takes 1 - w1 - w2 - w3).  Either output may be NULL. */
OTFEM_API int otfem_surface_binding(otfem_surface s, int32_t* tet, double* barycentric, int64_t count);
OTFEM_API int otfem_surface_destroy(otfem_surface s);

#ifdef __cplusplus
}
#endif
#endif
