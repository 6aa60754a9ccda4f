// ref_coupling.cpp -- t4mesh::mesh_coupling (core/containers/t4mesh/util/
// t4mesh_mesh_coupling.h) from the UNMODIFIED reference headers, behind two C
// functions of the oracle interface: bind_surface (:129-236, with its
// spatial-hashing point query and collision_policy::report, :84-111) and
// update_surface (:238-275), on the reference's FEM mesh type.
//
// TEST INFRASTRUCTURE ONLY.  Built with ref_capi.cpp by oracle/ref/
// build_ref.sh into oracle/_ref/libotfem_ref.so from the reference sources
// where they lie; the reference headers are never copied into this repository.
//
// The surface mesh is a small stand-in with what the two templates use:
// vertices with m_coord, m_tag and get_handle().get_idx(), size_vertices(),
// vertex_begin()/vertex_end(), and mesh::clear_vertex_tags.
#include <OpenTissue/configuration.h>
#include <OpenTissue/core/math/math_basic_types.h>
#include <OpenTissue/dynamics/fem/fem.h>

#include <cstddef>
#include <vector>

#include "../otfem_oracle.h"

namespace {

typedef OpenTissue::math::BasicMathTypes<double, size_t> math_types;
typedef OpenTissue::fem::Mesh<math_types> volume_mesh;
typedef math_types::vector3_type vector3_type;

struct SurfaceVertex {
  struct Handle {
    size_t idx;
    size_t get_idx() const { return idx; }
  };
  vector3_type m_coord;
  int m_tag;
  size_t m_idx;
  Handle get_handle() const { return Handle{m_idx}; }
};

struct SurfaceMesh {
  typedef SurfaceVertex vertex_type;
  typedef std::vector<SurfaceVertex>::iterator vertex_iterator;
  std::vector<SurfaceVertex> v;
  size_t size_vertices() const { return v.size(); }
  vertex_iterator vertex_begin() { return v.begin(); }
  vertex_iterator vertex_end() { return v.end(); }
};

// bind_surface resizes its outputs to the number of bound points but indexes
// them by point index; these containers never shrink below the point count,
// so a point set with unbound points stays in bounds (unbound entries keep
// their initial values).
template <typename T>
struct FixedVector {
  std::vector<T> v;
  void resize(size_t n) {
    if (n > v.size()) v.resize(n);
  }
  T& operator[](size_t i) { return v[i]; }
  const T& operator[](size_t i) const { return v[i]; }
};

void build_volume(volume_mesh& V, int n_nodes, int n_tets, const int* tets, const double* coord) {
  for (int i = 0; i < n_nodes; ++i) {
    volume_mesh::node_iterator nd = V.insert();
    for (int c = 0; c < 3; ++c) nd->m_coord(c) = coord[3 * i + c];
  }
  for (int t = 0; t < n_tets; ++t)
    V.insert(size_t(tets[4 * t]), size_t(tets[4 * t + 1]), size_t(tets[4 * t + 2]), size_t(tets[4 * t + 3]));
}

void build_surface(SurfaceMesh& M, int n_points, const double* points) {
  M.v.resize(size_t(n_points));
  for (int i = 0; i < n_points; ++i) {
    for (int c = 0; c < 3; ++c) M.v[size_t(i)].m_coord(c) = points ? points[3 * i + c] : 0.0;
    M.v[size_t(i)].m_tag = 0;
    M.v[size_t(i)].m_idx = size_t(i);
  }
}

}  // namespace

namespace OpenTissue {
namespace mesh {
inline void clear_vertex_tags(SurfaceMesh& M) {
  for (size_t i = 0; i < M.v.size(); ++i) M.v[i].m_tag = 0;
}
}  // namespace mesh
}  // namespace OpenTissue

// t4mesh_mesh_coupling.h calls geometry::barycentric_algebraic without
// including its header (core/geometry/geometry_barycentric.h)
#include <OpenTissue/core/geometry/geometry_barycentric.h>
#include <OpenTissue/core/containers/t4mesh/util/t4mesh_mesh_coupling.h>

extern "C" {

int orc_coupling_bind(int n_nodes, int n_tets, const int* tets, const double* coord, int n_points,
                      const double* points, int* tet_out, double* bary_out) {
  volume_mesh V;
  build_volume(V, n_nodes, n_tets, tets, coord);
  SurfaceMesh M;
  build_surface(M, n_points, points);
  FixedVector<vector3_type> bary;
  FixedVector<long> index;
  bary.v.assign(size_t(n_points), vector3_type(0.0, 0.0, 0.0));
  index.v.assign(size_t(n_points), -1L);
  OpenTissue::t4mesh::mesh_coupling::bind_surface(M, V, bary, index);
  int bound = 0;
  for (int i = 0; i < n_points; ++i) {
    const bool b = M.v[size_t(i)].m_tag == 1;
    bound += b ? 1 : 0;
    tet_out[i] = b ? int(index[size_t(i)]) : -1;
    for (int c = 0; c < 3; ++c) bary_out[3 * i + c] = b ? bary[size_t(i)](c) : 0.0;
  }
  return bound;
}

int orc_coupling_update(int n_nodes, int n_tets, const int* tets, const double* coord, int n_points,
                        const int* tet, const double* bary, double* out) {
  volume_mesh V;
  build_volume(V, n_nodes, n_tets, tets, coord);
  SurfaceMesh M;
  build_surface(M, n_points, 0);
  std::vector<vector3_type> b(static_cast<size_t>(n_points));
  std::vector<size_t> index(static_cast<size_t>(n_points));
  for (int i = 0; i < n_points; ++i) {
    if (tet[i] < 0) return -1;  // update_surface indexes a tet for every point
    index[size_t(i)] = size_t(tet[i]);
    b[size_t(i)] = vector3_type(bary[3 * i], bary[3 * i + 1], bary[3 * i + 2]);
  }
  OpenTissue::t4mesh::mesh_coupling::update_surface(M, V, b, index);
  for (int i = 0; i < n_points; ++i)
    for (int c = 0; c < 3; ++c) out[3 * i + c] = M.v[size_t(i)].m_coord(c);
  return 0;
}

}  // extern "C"
