#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_SIMULATE_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_SIMULATE_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// fem::simulate (reference: fem_simulate.h:49-113), same signature: one
// implicit stiffness-warped time step
//   (M + dt C + dt^2 K) v' = M v - dt (K x + f0 - f_ext),  x' = x + dt v'.
// The host-writable node fields are sent to the device, the step runs there
// (libotfem_gpu.so), and m_coord, m_velocity and m_f_external come back.
// External forces must be set before the call, as in the reference.
//
// simulate(mesh, dt, warp) reproduces the reference's solver settings
// (20-iteration CG, mass damping 2.0); the overload taking SolverParams
// selects e.g. mixed_solver(1e-6), the matrix-free relative-residual solver,
// and returns the step's statistics.  Errors throw std::runtime_error.
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/dynamics/fem/fem_mesh.h>

#include <stdexcept>

namespace OpenTissue {
namespace fem {

template <typename fem_mesh, typename real_type>
inline StepStats simulate(fem_mesh& mesh, real_type const& time_step, bool use_stiffness_warping,
                          SolverParams const& params) {
  gpu::State& g = mesh.gpu_state();
  if (!g.ready()) throw std::logic_error("fem::simulate(): fem::init has not been called on this mesh");
  std::size_t const N = mesh.size_nodes();
  double *x = g.x(), *x0 = g.x0(), *v = g.v(), *f = g.f();
  unsigned char* fx = g.fixed();
  for (std::size_t i = 0; i < N; ++i) {
    typename fem_mesh::node_type& n = mesh.node_at(i);
    for (int c = 0; c < 3; ++c) {
      x[3 * i + c] = double(n.m_coord(c));
      x0[3 * i + c] = double(n.m_model_coord(c));
      v[3 * i + c] = double(n.m_velocity(c));
      f[3 * i + c] = double(n.m_f_external(c));
    }
    fx[i] = n.m_fixed ? 1 : 0;
  }
  otfem_handle h = g.handle();
  int64_t const n3 = int64_t(3 * N);
  gpu::check(otfem_set_fixed(h, fx, int64_t(N)), "fem::simulate");
  gpu::check(otfem_set_nodes(h, OTFEM_MODEL_COORD, x0, n3), "fem::simulate");
  // positions, velocities and external forces in and out of the page-locked
  // staging buffers around the step (one graph, copies overlapped)
  gpu::check(otfem_simulate_host(h, double(time_step), use_stiffness_warping ? 1 : 0, &params, &g.stats(), x, v, f),
             "fem::simulate");
  // the external forces as the step left them (plasticity adds to them)
  gpu::check(otfem_get_nodes(h, OTFEM_F_EXTERNAL, f, n3), "fem::simulate");
  for (std::size_t i = 0; i < N; ++i) {
    typename fem_mesh::node_type& n = mesh.node_at(i);
    for (int c = 0; c < 3; ++c) {
      n.m_coord(c) = real_type(x[3 * i + c]);
      n.m_velocity(c) = real_type(v[3 * i + c]);
      n.m_f_external(c) = real_type(f[3 * i + c]);
    }
  }
  return g.last_stats();
}

template <typename fem_mesh, typename real_type>
inline void simulate(fem_mesh& mesh, real_type const& time_step, bool use_stiffness_warping) {
  simulate(mesh, time_step, use_stiffness_warping, reference_solver());
}

namespace gpu {

// Copies m_Re and m_plastic of every tetrahedron back from the device.
template <typename fem_mesh>
inline void download_tetrahedra(fem_mesh& mesh) {
  std::size_t const T = mesh.size_tetrahedra();
  std::vector<double> re(9 * T), pl(6 * T);
  check(otfem_get_orientations(mesh.gpu_state().handle(), re.data()), "fem::gpu::download_tetrahedra");
  check(otfem_get_plastic(mesh.gpu_state().handle(), pl.data()), "fem::gpu::download_tetrahedra");
  for (std::size_t t = 0; t < T; ++t) {
    typename fem_mesh::tetrahedron_type& e = mesh.tetrahedron_at(t);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) e.m_Re(r, c) = re[9 * t + 3 * r + c];
    for (int q = 0; q < 6; ++q) e.m_plastic[q] = pl[6 * t + q];
  }
}

// Fills every node's m_K_row map from the device (the values of the last
// reference-solver step), keys as the reference creates them.
template <typename fem_mesh>
inline void download_stiffness_rows(fem_mesh& mesh) {
  otfem_handle h = mesh.gpu_state().handle();
  int64_t nnz = 0;
  check(otfem_k_pattern(h, &nnz, 0, 0), "fem::gpu::download_stiffness_rows");
  std::vector<int32_t> rp(mesh.size_nodes() + 1), cols(std::size_t(nnz) + 1);
  std::vector<double> vals(9 * std::size_t(nnz) + 1);
  check(otfem_k_pattern(h, &nnz, rp.data(), cols.data()), "fem::gpu::download_stiffness_rows");
  check(otfem_k_values(h, vals.data()), "fem::gpu::download_stiffness_rows");
  for (std::size_t i = 0; i < mesh.size_nodes(); ++i) {
    typename fem_mesh::node_type& n = mesh.node_at(i);
    n.m_K_row.clear();
    for (int32_t q = rp[i]; q < rp[i + 1]; ++q) {
      typename fem_mesh::matrix3x3_type& K = n.K(cols[q]);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) K(r, c) = vals[9 * std::size_t(q) + 3 * r + c];
    }
  }
}

}  // namespace gpu
}  // namespace fem
}  // namespace OpenTissue

#endif
