#ifndef OPENTISSUE_DYNAMICS_DEFORMATION_FEM_STIFFNESSWARPING_H
#define OPENTISSUE_DYNAMICS_DEFORMATION_FEM_STIFFNESSWARPING_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// Tetrahedron fields of fem::Mesh (reference: fem_tetrahedron_traits.h:18-49),
// same names.  fem::init sets the material fields and m_V on the host; m_Ke,
// m_B, m_D live on the device; fem::gpu::download_tetrahedra(mesh) copies
// m_Re and m_plastic back on request.
//
#include <OpenTissue/configuration.h>

namespace OpenTissue {
namespace fem {
namespace detail {

template <typename math_types>
class TetrahedronTraits {
 public:
  typedef math_types fem_math_types;  // (drop-in) names the owning fem::Mesh<fem_math_types>
  typedef typename math_types::real_type real_type;
  typedef typename math_types::vector3_type vector3_type;
  typedef typename math_types::matrix3x3_type matrix3x3_type;

 public:
  real_type m_young;
  real_type m_poisson;
  real_type m_density;
  matrix3x3_type m_Ke[4][4];
  matrix3x3_type m_Re;
  real_type m_V;
  vector3_type m_e10;
  vector3_type m_e20;
  vector3_type m_e30;
  vector3_type m_B[4];
  vector3_type m_D;
  real_type m_plastic[6];
  real_type m_yield;
  real_type m_creep;
  real_type m_max;
  // (drop-in, no counterpart in the reference) the fem::Mesh that owns the
  // tetrahedron, set by fem::init (see fem_detail.h)
  void* m_gpu_mesh;

  TetrahedronTraits() : m_gpu_mesh(0) {}
};

}  // namespace detail
}  // namespace fem
}  // namespace OpenTissue

#endif
