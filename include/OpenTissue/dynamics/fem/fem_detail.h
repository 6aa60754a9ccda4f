#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_DETAIL_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_DETAIL_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// The steps fem::simulate is made of (reference: fem_simulate.h:94-111), as
// the fem::detail functions host code can call one by one, same names and
// signatures:
//
//   clear_stiffness_assembly(node_begin, node_end)      fem_clear_stiffness_assembly.h:23-33
//   update_orientation(tet_begin, tet_end)              fem_update_orientation.h:22-215
//   reset_orientation(tet_begin, tet_end)               fem_reset_orientation.h:22-27
//   stiffness_assembly(tet_begin, tet_end)              fem_stiffness_assembly.h:171-209
//   add_plasticity_force(tet_begin, tet_end, dt)        fem_add_plasticity_force.h:26-204
//   dynamics_assembly(mesh, mass_damping, dt)           fem_dynamics_assembly.h:47-93
//   conjugate_gradients(mesh, min_it, max_it)           fem_conjugate_gradients.h:25-133
//   position_update(mesh, dt)                           fem_position_update.h:25-39
//
// Each runs on the device with the reference solver's kernels (FP64,
// reference operation order; the CG sums its dot products in node order, so
// a step made of these calls is bit-identical to the reference's), after
// sending the host node fields the step reads (m_coord, m_model_coord,
// m_velocity, m_f_external, m_fixed), and writes back the fields the
// reference step writes: m_Re, the m_K_row maps and m_f0, m_plastic and
// m_f_external, the m_A_row maps and m_b, m_velocity, m_coord.  The device
// keeps its own K, A and Re: host edits of m_K_row, m_A_row or m_Re between
// the calls are not seen by the next one.
//
// The ranges must cover the whole mesh of a fem::init'ed fem::Mesh (the
// device runs every step over every element); a partial range throws
// std::invalid_argument, a mesh without fem::init std::logic_error.  Unlike
// the reference, stiffness_assembly writes this step's sums instead of adding
// to what a previous assembly left (the reference adds; simulate always
// clears first, so the two agree within a step).
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/dynamics/fem/fem_mesh.h>
#include <OpenTissue/dynamics/fem/fem_simulate.h>

#include <cstddef>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

namespace OpenTissue {
namespace fem {
namespace detail {
namespace gpu_stage {

// The fem::Mesh owning the elements of [begin, end), which must be all of
// its `count(mesh)` elements.
template <typename mesh_type, typename iterator, typename counter>
inline mesh_type& whole_mesh(iterator begin, iterator end, counter count, char const* where) {
  if (begin == end) throw std::invalid_argument(std::string(where) + ": empty range");
  void* owner = begin->m_gpu_mesh;
  if (!owner) throw std::logic_error(std::string(where) + ": fem::init has not been called on this mesh");
  mesh_type& mesh = *static_cast<mesh_type*>(owner);
  if (!mesh.gpu_state().ready())
    throw std::logic_error(std::string(where) + ": fem::init has not been called on this mesh");
  std::size_t n = 0;
  for (iterator it = begin; it != end; ++it) ++n;
  if (n != count(mesh))
    throw std::invalid_argument(std::string(where) + ": the GPU runs each step on a whole mesh (partial range)");
  return mesh;
}

template <typename mesh_type>
struct NodeCount {
  std::size_t operator()(mesh_type& m) const { return m.size_nodes(); }
};
template <typename mesh_type>
struct TetCount {
  std::size_t operator()(mesh_type& m) const { return m.size_tetrahedra(); }
};

// Host node field -> device.  The copy is queued asynchronously from the
// field's own page-locked staging buffer; every stage ends with a stream
// synchronisation, so a buffer is rewritten only after its last copy ran.
template <typename mesh_type>
inline void upload(mesh_type& mesh, int field, char const* where) {
  gpu::State& g = mesh.gpu_state();
  std::size_t const N = mesh.size_nodes();
  double* buf = field == OTFEM_COORD ? g.x() : field == OTFEM_MODEL_COORD ? g.x0() : field == OTFEM_VELOCITY ? g.v()
                                                                                                         : g.f();
  for (std::size_t i = 0; i < N; ++i) {
    typename mesh_type::node_type& n = mesh.node_at(i);
    typename mesh_type::vector3_type const& v = field == OTFEM_COORD         ? n.m_coord
                                                : field == OTFEM_MODEL_COORD ? n.m_model_coord
                                                : field == OTFEM_VELOCITY    ? n.m_velocity
                                                                             : n.m_f_external;
    for (int c = 0; c < 3; ++c) buf[3 * i + c] = double(v(c));
  }
  gpu::check(otfem_set_nodes(g.handle(), field, buf, int64_t(3 * N)), where);
}

template <typename mesh_type>
inline void upload_fixed(mesh_type& mesh, char const* where) {
  gpu::State& g = mesh.gpu_state();
  std::size_t const N = mesh.size_nodes();
  unsigned char* fx = g.fixed();
  for (std::size_t i = 0; i < N; ++i) fx[i] = mesh.node_at(i).m_fixed ? 1 : 0;
  gpu::check(otfem_set_fixed(g.handle(), fx, int64_t(N)), where);
}

// Device node field -> host (synchronous; after the stage's synchronisation,
// so the staging buffer it uses has no copy in flight).
template <typename mesh_type>
inline void download(mesh_type& mesh, int field, char const* where) {
  typedef typename mesh_type::real_type real_type;
  gpu::State& g = mesh.gpu_state();
  std::size_t const N = mesh.size_nodes();
  double* buf = g.x();
  gpu::check(otfem_get_nodes(g.handle(), field, buf, int64_t(3 * N)), where);
  for (std::size_t i = 0; i < N; ++i) {
    typename mesh_type::node_type& n = mesh.node_at(i);
    typename mesh_type::vector3_type& v = field == OTFEM_COORD      ? n.m_coord
                                          : field == OTFEM_VELOCITY ? n.m_velocity
                                          : field == OTFEM_F0       ? n.m_f0
                                          : field == OTFEM_B        ? n.m_b
                                                                    : n.m_f_external;
    for (int c = 0; c < 3; ++c) v(c) = real_type(buf[3 * i + c]);
  }
}

// The m_A_row maps from the device (keys: the K_row pattern).
template <typename mesh_type>
inline void download_dynamics_rows(mesh_type& mesh, char const* where) {
  otfem_handle h = mesh.gpu_state().handle();
  int64_t nnz = 0;
  gpu::check(otfem_k_pattern(h, &nnz, 0, 0), where);
  std::vector<int32_t> rp(mesh.size_nodes() + 1), cols(std::size_t(nnz) + 1);
  std::vector<double> vals(9 * std::size_t(nnz) + 1);
  gpu::check(otfem_k_pattern(h, &nnz, rp.data(), cols.data()), where);
  gpu::check(otfem_a_values(h, vals.data()), where);
  for (std::size_t i = 0; i < mesh.size_nodes(); ++i) {
    typename mesh_type::node_type& n = mesh.node_at(i);
    n.m_A_row.clear();
    for (int32_t q = rp[i]; q < rp[i + 1]; ++q) {
      typename mesh_type::matrix3x3_type& A = n.A(cols[q]);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A(r, c) = vals[9 * std::size_t(q) + 3 * r + c];
    }
  }
}

inline void run(otfem_handle h, int stage, double dt, double mass_damping, int min_it, int max_it,
                char const* where) {
  gpu::check(otfem_reference_stage(h, stage, dt, mass_damping, int32_t(min_it), int32_t(max_it)), where);
}

}  // namespace gpu_stage

template <typename node_iterator>
inline void clear_stiffness_assembly(node_iterator begin, node_iterator end) {
  typedef typename node_iterator::value_type node_type;
  typedef Mesh<typename node_type::fem_math_types> mesh_type;
  char const* where = "fem::detail::clear_stiffness_assembly";
  mesh_type& mesh = gpu_stage::whole_mesh<mesh_type>(begin, end, gpu_stage::NodeCount<mesh_type>(), where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_CLEAR_STIFFNESS_ASSEMBLY, 0.0, 0.0, 0, 0, where);
  for (node_iterator n = begin; n != end; ++n) {
    n->m_f0.clear();
    for (typename node_type::matrix_iterator K = n->Kbegin(); K != n->Kend(); ++K) K->second.clear();
  }
}

template <typename tetrahedron_iterator>
inline void update_orientation(tetrahedron_iterator const& begin, tetrahedron_iterator const& end) {
  typedef typename tetrahedron_iterator::value_type tetrahedron_type;
  typedef Mesh<typename tetrahedron_type::fem_math_types> mesh_type;
  char const* where = "fem::detail::update_orientation";
  mesh_type& mesh = gpu_stage::whole_mesh<mesh_type>(begin, end, gpu_stage::TetCount<mesh_type>(), where);
  gpu_stage::upload(mesh, OTFEM_COORD, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_UPDATE_ORIENTATION, 0.0, 0.0, 0, 0, where);
  gpu::download_tetrahedra(mesh);
}

template <typename tetrahedron_iterator>
inline void reset_orientation(tetrahedron_iterator const& begin, tetrahedron_iterator const& end) {
  typedef typename tetrahedron_iterator::value_type tetrahedron_type;
  typedef Mesh<typename tetrahedron_type::fem_math_types> mesh_type;
  char const* where = "fem::detail::reset_orientation";
  mesh_type& mesh = gpu_stage::whole_mesh<mesh_type>(begin, end, gpu_stage::TetCount<mesh_type>(), where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_RESET_ORIENTATION, 0.0, 0.0, 0, 0, where);
  for (tetrahedron_iterator T = begin; T != end; ++T)
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) T->m_Re(r, c) = r == c ? 1 : 0;
}

template <typename tetrahedron_iterator>
inline void stiffness_assembly(tetrahedron_iterator const& begin, tetrahedron_iterator const& end) {
  typedef typename tetrahedron_iterator::value_type tetrahedron_type;
  typedef Mesh<typename tetrahedron_type::fem_math_types> mesh_type;
  char const* where = "fem::detail::stiffness_assembly";
  mesh_type& mesh = gpu_stage::whole_mesh<mesh_type>(begin, end, gpu_stage::TetCount<mesh_type>(), where);
  gpu_stage::upload(mesh, OTFEM_MODEL_COORD, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_STIFFNESS_ASSEMBLY, 0.0, 0.0, 0, 0, where);
  gpu::download_stiffness_rows(mesh);
  gpu_stage::download(mesh, OTFEM_F0, where);
}

template <typename tetrahedron_iterator, typename real_type>
inline void add_plasticity_force(tetrahedron_iterator begin, tetrahedron_iterator end, real_type const& dt) {
  typedef typename tetrahedron_iterator::value_type tetrahedron_type;
  typedef Mesh<typename tetrahedron_type::fem_math_types> mesh_type;
  char const* where = "fem::detail::add_plasticity_force";
  mesh_type& mesh = gpu_stage::whole_mesh<mesh_type>(begin, end, gpu_stage::TetCount<mesh_type>(), where);
  gpu_stage::upload(mesh, OTFEM_COORD, where);
  gpu_stage::upload(mesh, OTFEM_MODEL_COORD, where);
  gpu_stage::upload(mesh, OTFEM_F_EXTERNAL, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_ADD_PLASTICITY_FORCE, double(dt), 0.0, 0, 0, where);
  gpu::download_tetrahedra(mesh);
  gpu_stage::download(mesh, OTFEM_F_EXTERNAL, where);
}

template <typename fem_mesh, typename real_type>
inline void dynamics_assembly(fem_mesh& mesh, real_type const& mass_damping, real_type const& dt) {
  char const* where = "fem::detail::dynamics_assembly";
  if (!mesh.gpu_state().ready()) throw std::logic_error(std::string(where) + ": fem::init has not been called");
  gpu_stage::upload(mesh, OTFEM_COORD, where);
  gpu_stage::upload(mesh, OTFEM_VELOCITY, where);
  gpu_stage::upload(mesh, OTFEM_F_EXTERNAL, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_DYNAMICS_ASSEMBLY, double(dt), double(mass_damping), 0, 0,
                 where);
  gpu_stage::download_dynamics_rows(mesh, where);
  gpu_stage::download(mesh, OTFEM_B, where);
}

template <typename fem_mesh>
inline void conjugate_gradients(fem_mesh& mesh, unsigned int min_iterations, unsigned int max_iterations) {
  char const* where = "fem::detail::conjugate_gradients";
  if (!mesh.gpu_state().ready()) throw std::logic_error(std::string(where) + ": fem::init has not been called");
  gpu_stage::upload_fixed(mesh, where);
  gpu_stage::upload(mesh, OTFEM_VELOCITY, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_CONJUGATE_GRADIENTS, 0.0, 0.0, int(min_iterations),
                 int(max_iterations), where);
  gpu_stage::download(mesh, OTFEM_VELOCITY, where);
}

template <typename fem_mesh, typename real_type>
inline void position_update(fem_mesh& mesh, real_type const& dt) {
  char const* where = "fem::detail::position_update";
  if (!mesh.gpu_state().ready()) throw std::logic_error(std::string(where) + ": fem::init has not been called");
  gpu_stage::upload_fixed(mesh, where);
  gpu_stage::upload(mesh, OTFEM_COORD, where);
  gpu_stage::upload(mesh, OTFEM_VELOCITY, where);
  gpu_stage::run(mesh.gpu_state().handle(), OTFEM_STAGE_POSITION_UPDATE, double(dt), 0.0, 0, 0, where);
  gpu_stage::download(mesh, OTFEM_COORD, where);
}

}  // namespace detail
}  // namespace fem
}  // namespace OpenTissue

#endif
