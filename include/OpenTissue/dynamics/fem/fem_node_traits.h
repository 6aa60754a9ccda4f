#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_NODE_TRAITS_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_NODE_TRAITS_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// Node fields of fem::Mesh (reference: fem_node_traits.h:21-70), same names.
//
// m_K_row / m_A_row stay empty: K and A live on the device.  fem::export_K
// reads K from there; fem::gpu::download_stiffness_rows(mesh) fills m_K_row
// on request.  m_f0, m_b, m_update, m_prev and m_residual are device-only.
//
#include <OpenTissue/configuration.h>

#include <map>

namespace OpenTissue {
namespace fem {
namespace detail {

template <typename math_types>
class NodeTraits {
 public:
  typedef math_types fem_math_types;  // (drop-in) names the owning fem::Mesh<fem_math_types>
  typedef typename math_types::real_type real_type;
  typedef typename math_types::vector3_type vector3_type;
  typedef typename math_types::matrix3x3_type matrix3x3_type;
  typedef typename std::map<int, matrix3x3_type> matrix_container;
  typedef typename matrix_container::iterator matrix_iterator;

 public:
  matrix_container m_K_row;
  matrix_container m_A_row;
  vector3_type m_f0;
  vector3_type m_b;
  bool m_fixed;
  vector3_type m_model_coord;
  vector3_type m_coord;
  vector3_type m_velocity;
  real_type m_mass;
  vector3_type m_f_external;
  vector3_type m_update;
  vector3_type m_prev;
  vector3_type m_residual;
  // (drop-in, no counterpart in the reference) the fem::Mesh that owns the
  // node, set by fem::init: how the fem::detail functions, which take
  // iterators, reach the mesh's device state
  void* m_gpu_mesh;

 public:
  matrix_iterator Kbegin() { return m_K_row.begin(); }
  matrix_iterator Kend() { return m_K_row.end(); }
  matrix_iterator Abegin() { return m_A_row.begin(); }
  matrix_iterator Aend() { return m_A_row.end(); }
  matrix3x3_type& K(int const& column_idx) { return m_K_row[column_idx]; }
  matrix3x3_type& A(int const& column_idx) { return m_A_row[column_idx]; }

  NodeTraits() : m_fixed(false), m_mass(0), m_gpu_mesh(0) {}
};

}  // namespace detail
}  // namespace fem
}  // namespace OpenTissue

#endif
