#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_MESH_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_MESH_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// fem::Mesh (reference: fem_mesh.h:21-34): the same t4mesh container with the
// fem node and tetrahedron traits, plus the device state of the mesh.
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/core/containers/t4mesh/t4mesh.h>
#include <OpenTissue/dynamics/fem/fem_gpu_state.h>
#include <OpenTissue/dynamics/fem/fem_node_traits.h>
#include <OpenTissue/dynamics/fem/fem_tetrahedron_traits.h>

#include <cstddef>

namespace OpenTissue {
namespace fem {

template <typename math_types>
class Mesh : public OpenTissue::t4mesh::T4Mesh<math_types, OpenTissue::fem::detail::NodeTraits<math_types>,
                                               OpenTissue::fem::detail::TetrahedronTraits<math_types> > {
 public:
  typedef typename math_types::real_type real_type;
  typedef typename math_types::vector3_type vector3_type;
  typedef typename math_types::matrix3x3_type matrix3x3_type;
  typedef OpenTissue::t4mesh::T4Mesh<math_types, OpenTissue::fem::detail::NodeTraits<math_types>,
                                     OpenTissue::fem::detail::TetrahedronTraits<math_types> >
      base_type;
  typedef typename base_type::node_type node_type;
  typedef typename base_type::tetrahedron_type tetrahedron_type;

  // Device state (no counterpart in the reference).
  gpu::State& gpu_state() { return m_gpu; }
  // Contiguous access to the container's storage, used to stage transfers
  // without going through the bounds-checked iterators.
  node_type& node_at(std::size_t i) { return this->m_nodes[i]; }
  tetrahedron_type& tetrahedron_at(std::size_t t) { return this->m_tetrahedra[t]; }

 private:
  gpu::State m_gpu;
};

}  // namespace fem
}  // namespace OpenTissue

#endif
