#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_INIT_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_INIT_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// fem::init (reference: fem_init.h:45-65), same signature and effect: uniform
// material, element stiffness, lumped mass (fixed nodes get the largest
// real), plasticity state.  The element data is computed on the device by
// otfem_init; m_mass, m_V and the per-tet material fields are written back to
// the host container.  Fixed flags must be set before this call, as in the
// reference (compute_mass reads them).  Throws std::runtime_error on a bad
// mesh or a device error.
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/dynamics/fem/fem_mesh.h>

#include <cstdint>
#include <vector>

namespace OpenTissue {
namespace fem {

template <typename fem_mesh, typename real_type>
inline void init(fem_mesh& mesh, real_type const& young, real_type const& poisson, real_type const& density,
                 real_type const& c_yield, real_type const& c_creep, real_type const& c_max) {
  std::size_t const N = mesh.size_nodes(), T = mesh.size_tetrahedra();
  std::vector<int32_t> tets(4 * T);
  std::vector<double> x(3 * N), x0(3 * N);
  std::vector<uint8_t> fixed(N);
  for (std::size_t t = 0; t < T; ++t)
    for (int k = 0; k < 4; ++k) tets[4 * t + k] = int32_t(mesh.tetrahedron_at(t).node_idx(k));
  for (std::size_t i = 0; i < N; ++i) {
    typename fem_mesh::node_type& n = mesh.node_at(i);
    for (int c = 0; c < 3; ++c) {
      x[3 * i + c] = double(n.m_coord(c));
      x0[3 * i + c] = double(n.m_model_coord(c));
    }
    fixed[i] = n.m_fixed ? 1 : 0;
  }
  otfem_mesh_desc d;
  d.num_nodes = int32_t(N);
  d.num_tets = int32_t(T);
  d.tets = tets.data();
  d.coord = x.data();
  d.model_coord = x0.data();
  d.fixed = fixed.data();
  gpu::State& g = mesh.gpu_state();
  g.create(d);
  gpu::check(otfem_init(g.handle(), double(young), double(poisson), double(density), double(c_yield),
                        double(c_creep), double(c_max)),
             "fem::init");
  std::vector<double> mass(N), vol(T);
  gpu::check(otfem_get_nodes(g.handle(), OTFEM_MASS, mass.data(), int64_t(N)), "fem::init");
  gpu::check(otfem_get_volumes(g.handle(), vol.data()), "fem::init");
  for (std::size_t i = 0; i < N; ++i) {
    mesh.node_at(i).m_mass = real_type(mass[i]);
    mesh.node_at(i).m_gpu_mesh = &mesh;
  }
  for (std::size_t t = 0; t < T; ++t) {
    typename fem_mesh::tetrahedron_type& e = mesh.tetrahedron_at(t);
    e.m_gpu_mesh = &mesh;
    e.m_young = young;
    e.m_poisson = poisson;
    e.m_density = density;
    e.m_yield = c_yield;
    e.m_creep = c_creep;
    e.m_max = c_max;
    e.m_V = real_type(vol[t]);
    for (int q = 0; q < 6; ++q) e.m_plastic[q] = real_type(0);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) e.m_Re(r, c) = real_type(r == c ? 1 : 0);
  }
}

}  // namespace fem
}  // namespace OpenTissue

#endif
