#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_GPU_STATE_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_GPU_STATE_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem: the device state a
// fem::Mesh owns.  Not part of the reference interface.
//
// Each fem::Mesh holds one otfem handle (device-resident mesh, libotfem_gpu.so)
// and page-locked staging buffers.  fem::init creates it; fem::simulate moves
// the host-writable node fields (m_coord, m_model_coord, m_velocity,
// m_f_external, m_fixed) to the device, runs the step, and moves m_coord and
// m_velocity (and m_f_external, which plasticity accumulates into) back.
// Copies of a mesh do not share device state: call fem::init on a copy.
//
#include <cstddef>
#include <stdexcept>
#include <string>

#include "otfem_gpu.h"

namespace OpenTissue {
namespace fem {

// Solver settings for the simulate() overload.  reference_solver() is what
// simulate(mesh, dt, warp) uses: the reference's 20-iteration CG with its
// clamps and mass damping 2.0 (fem_simulate.h:104-109).
typedef otfem_solver_params SolverParams;
typedef otfem_step_stats StepStats;

inline SolverParams reference_solver() {
  SolverParams p;
  otfem_default_params(&p);
  return p;
}

// Matrix-free solver: FP32 element apply, Jacobi-preconditioned CG with the
// velocity, dot products and scalars in (hi, lo) float pairs (~48-bit), stop
// at ||r|| <= rtol ||b||.
inline SolverParams mixed_solver(double rtol = 1e-6, int max_iterations = 10000) {
  SolverParams p = reference_solver();
  p.solver = OTFEM_SOLVER_MIXED;
  p.rtol = rtol;
  p.max_iterations = max_iterations;
  return p;
}

// The matrix-free solver starting from the least-energy point on the span of
// the last `history` velocity changes (the same stopping rule).
inline SolverParams projected_solver(double rtol = 1e-6, int history = 4, int max_iterations = 10000) {
  SolverParams p = mixed_solver(rtol, max_iterations);
  p.warm_start = OTFEM_WARM_START_PROJECTED;
  p.warm_history = history;
  return p;
}

// The matrix-free solver starting from the velocity extrapolated by the
// polynomial of degree `degree` through the last degree + 1 velocities (the
// same stopping rule; no extra element-apply).
inline SolverParams extrapolated_solver(double rtol = 1e-6, int degree = 4, int max_iterations = 10000) {
  SolverParams p = mixed_solver(rtol, max_iterations);
  p.warm_start = OTFEM_WARM_START_EXTRAPOLATED;
  p.warm_history = degree;
  return p;
}

namespace gpu {

inline void check(int rc, char const* where) {
  if (rc < 0) throw std::runtime_error(std::string(where) + ": " + otfem_last_error());
}

class State {
 public:
  State() {}
  State(State const&) {}  // a copied mesh starts without device state
  State& operator=(State const&) {
    release();
    return *this;
  }
  ~State() { release(); }

  bool ready() const { return m_handle != 0; }
  otfem_handle handle() const { return m_handle; }
  SolverParams& params() { return m_params; }
  StepStats const& last_stats() const { return m_stats; }
  StepStats& stats() { return m_stats; }

  void create(otfem_mesh_desc const& desc) {
    release();
    check(otfem_create(&desc, 0, &m_handle), "fem::init");
    m_nodes = size_t(desc.num_nodes);
    void* p = 0;
    check(otfem_host_alloc(sizeof(double) * 3 * m_nodes * 4 + m_nodes, &p), "fem::init");
    m_stage = static_cast<double*>(p);
    m_params = reference_solver();
  }

  double* x() { return m_stage; }
  double* x0() { return m_stage + 3 * m_nodes; }
  double* v() { return m_stage + 6 * m_nodes; }
  double* f() { return m_stage + 9 * m_nodes; }
  unsigned char* fixed() { return reinterpret_cast<unsigned char*>(m_stage + 12 * m_nodes); }

  void release() {
    if (m_stage) otfem_host_free(m_stage);
    if (m_handle) otfem_destroy(m_handle);
    m_stage = 0;
    m_handle = 0;
    m_nodes = 0;
  }

 private:
  otfem_handle m_handle = 0;
  double* m_stage = 0;
  size_t m_nodes = 0;
  SolverParams m_params = SolverParams();
  StepStats m_stats = StepStats();
};

}  // namespace gpu
}  // namespace fem
}  // namespace OpenTissue

#endif
