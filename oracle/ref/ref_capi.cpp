// ref_capi.cpp -- exports the oracle C interface (oracle/otfem_oracle.h) on top
// of the UNMODIFIED OpenTissue FEM headers, so the C restatement in
// oracle/otfem_oracle.c can be checked bit for bit against the reference.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/build_ref.sh into
// oracle/_ref/libotfem_ref.so from the reference sources where they lie; the
// reference headers are never copied into this repository.
#include <OpenTissue/configuration.h>
#include <OpenTissue/core/math/math_basic_types.h>
#include <OpenTissue/dynamics/fem/fem.h>
#include <OpenTissue/core/containers/t4mesh/util/t4mesh_block_generator.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../otfem_oracle.h"

typedef OpenTissue::math::BasicMathTypes<double, size_t> math_types;
typedef OpenTissue::fem::Mesh<math_types> mesh_type;
typedef mesh_type::node_iterator node_iterator;
typedef mesh_type::tetrahedron_iterator tetrahedron_iterator;
typedef math_types::vector3_type vector3_type;
typedef math_types::matrix3x3_type matrix3x3_type;

struct orc_mesh {
  mesh_type mesh;
};

namespace {

// Minimal uBLAS-style sink for fem::export_K: resize(), clear(), push_back().
struct TripletSink {
  std::vector<int> rows, cols;
  std::vector<double> vals;
  void resize(size_t, size_t, bool) {}
  void clear() { rows.clear(); cols.clear(); vals.clear(); }
  void push_back(size_t r, size_t c, double v) {
    rows.push_back(int(r));
    cols.push_back(int(c));
    vals.push_back(v);
  }
};

// Relative-residual CG with the fixed-row / fixed-column semantics of
// fem_conjugate_gradients.h:48-131, written against the reference node fields.
// Same arithmetic order as conjugate_gradients_converged in otfem_oracle.c.
void cg_converged(mesh_type& mesh, double rtol, int max_it, int* iters, double* rel_res) {
  typedef mesh_type::node_type::matrix_iterator matrix_iterator;
  node_iterator begin = mesh.node_begin(), end = mesh.node_end();
  double bb = 0.0, rr = 0.0;
  for (node_iterator n = begin; n != end; ++n) {
    if (n->m_fixed) continue;
    n->m_residual = n->m_b;
    for (matrix_iterator A = n->Abegin(); A != n->Aend(); ++A)
      n->m_residual -= A->second * mesh.node(A->first)->m_velocity;
    n->m_prev = n->m_residual;
    bb += n->m_b * n->m_b;
    rr += n->m_residual * n->m_residual;
  }
  double thresh = rtol * rtol * bb;
  int it = 0;
  while (it < max_it && rr > thresh) {
    double pq = 0.0;
    for (node_iterator n = begin; n != end; ++n) {
      if (n->m_fixed) continue;
      n->m_update.clear();
      for (matrix_iterator A = n->Abegin(); A != n->Aend(); ++A)
        n->m_update += A->second * mesh.node(A->first)->m_prev;
      pq += n->m_prev * n->m_update;
    }
    double alpha = rr / pq, rr_new = 0.0;
    for (node_iterator n = begin; n != end; ++n) {
      if (n->m_fixed) continue;
      n->m_velocity += n->m_prev * alpha;
      n->m_residual -= n->m_update * alpha;
      rr_new += n->m_residual * n->m_residual;
    }
    double beta = rr_new / rr;
    rr = rr_new;
    for (node_iterator n = begin; n != end; ++n) {
      if (n->m_fixed) continue;
      n->m_prev = n->m_residual + n->m_prev * beta;
    }
    ++it;
  }
  double tr = 0.0;
  for (node_iterator n = begin; n != end; ++n) {
    if (n->m_fixed) continue;
    vector3_type r = n->m_b;
    for (matrix_iterator A = n->Abegin(); A != n->Aend(); ++A)
      r -= A->second * mesh.node(A->first)->m_velocity;
    tr += r * r;
  }
  if (iters) *iters = it;
  if (rel_res) *rel_res = bb > 0.0 ? std::sqrt(tr / bb) : std::sqrt(tr);
}

}  // namespace

extern "C" {

void orc_generate_blocks(int I, int J, int K, double w, double h, double d, int* tets, double* coord) {
  mesh_type mesh;
  OpenTissue::t4mesh::generate_blocks(unsigned(I), unsigned(J), unsigned(K), w, h, d, mesh);
  size_t n = 0;
  for (node_iterator nd = mesh.node_begin(); nd != mesh.node_end(); ++nd, ++n)
    for (int c = 0; c < 3; ++c) coord[3 * n + c] = nd->m_coord(c);
  size_t t = 0;
  for (tetrahedron_iterator T = mesh.tetrahedron_begin(); T != mesh.tetrahedron_end(); ++T, ++t)
    for (int a = 0; a < 4; ++a) tets[4 * t + a] = int(T->node_idx(a));
}

orc_mesh* orc_create(int n_nodes, int n_tets, const int* tets, const double* coord,
                     const double* model_coord, const unsigned char* fixed) {
  orc_mesh* m = new orc_mesh;
  for (int i = 0; i < n_nodes; ++i) {
    node_iterator nd = m->mesh.insert();
    for (int c = 0; c < 3; ++c) {
      if (coord) nd->m_coord(c) = coord[3 * i + c];
      if (model_coord) nd->m_model_coord(c) = model_coord[3 * i + c];
    }
    nd->m_fixed = fixed ? (fixed[i] != 0) : false;
  }
  for (int t = 0; t < n_tets; ++t)
    m->mesh.insert(size_t(tets[4 * t]), size_t(tets[4 * t + 1]), size_t(tets[4 * t + 2]), size_t(tets[4 * t + 3]));
  return m;
}

void orc_destroy(orc_mesh* m) { delete m; }

void orc_set_fixed(orc_mesh* m, const unsigned char* fixed) {
  size_t i = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd, ++i) nd->m_fixed = fixed[i] != 0;
}

static vector3_type* field(node_iterator nd, int f) {
  switch (f) {
    case ORC_COORD: return &nd->m_coord;
    case ORC_MODEL_COORD: return &nd->m_model_coord;
    case ORC_VELOCITY: return &nd->m_velocity;
    case ORC_F_EXTERNAL: return &nd->m_f_external;
    case ORC_F0: return &nd->m_f0;
    case ORC_B: return &nd->m_b;
    default: return 0;
  }
}

void orc_set_field(orc_mesh* m, int f, const double* src) {
  size_t i = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd, ++i) {
    vector3_type* v = field(nd, f);
    if (!v || f > ORC_F_EXTERNAL) return;
    for (int c = 0; c < 3; ++c) (*v)(c) = src[3 * i + c];
  }
}

void orc_get_field(orc_mesh* m, int f, double* dst) {
  size_t i = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd, ++i) {
    if (f == ORC_MASS) {
      dst[i] = nd->m_mass;
      continue;
    }
    vector3_type* v = field(nd, f);
    if (!v) return;
    for (int c = 0; c < 3; ++c) dst[3 * i + c] = (*v)(c);
  }
}

void orc_init(orc_mesh* m, double young, double poisson, double density, double c_yield, double c_creep,
              double c_max) {
  OpenTissue::fem::init(m->mesh, young, poisson, density, c_yield, c_creep, c_max);
}

void orc_simulate(orc_mesh* m, double dt, int use_warping) {
  OpenTissue::fem::simulate(m->mesh, dt, use_warping != 0);
}

void orc_simulate_converged(orc_mesh* m, double dt, int use_warping, double mass_damping, double rtol,
                            int max_iterations, int* iterations, double* rel_residual) {
  namespace d = OpenTissue::fem::detail;
  mesh_type& mesh = m->mesh;
  d::clear_stiffness_assembly(mesh.node_begin(), mesh.node_end());
  if (use_warping)
    d::update_orientation(mesh.tetrahedron_begin(), mesh.tetrahedron_end());
  else
    d::reset_orientation(mesh.tetrahedron_begin(), mesh.tetrahedron_end());
  d::stiffness_assembly(mesh.tetrahedron_begin(), mesh.tetrahedron_end());
  d::add_plasticity_force(mesh.tetrahedron_begin(), mesh.tetrahedron_end(), dt);
  d::dynamics_assembly(mesh, mass_damping, dt);
  cg_converged(mesh, rtol, max_iterations, iterations, rel_residual);
  d::position_update(mesh, dt);
}

void orc_update_original_coord(orc_mesh* m) {
  OpenTissue::fem::update_original_coord(m->mesh.node_begin(), m->mesh.node_end());
}

long orc_export_k_count(orc_mesh* m) {
  TripletSink s;
  OpenTissue::fem::export_K(m->mesh, s);
  return long(s.vals.size());
}

void orc_export_k(orc_mesh* m, int* rows, int* cols, double* vals) {
  TripletSink s;
  OpenTissue::fem::export_K(m->mesh, s);
  for (size_t q = 0; q < s.vals.size(); ++q) {
    rows[q] = s.rows[q];
    cols[q] = s.cols[q];
    vals[q] = s.vals[q];
  }
}

long orc_k_nnz(orc_mesh* m) {
  long n = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd) n += long(nd->m_K_row.size());
  return n;
}

void orc_k_pattern(orc_mesh* m, int* row_ptr, int* cols) {
  long n = 0;
  size_t i = 0;
  row_ptr[0] = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd, ++i) {
    for (auto& kv : nd->m_K_row) cols[n++] = kv.first;
    row_ptr[i + 1] = int(n);
  }
}

void orc_k_values(orc_mesh* m, double* vals) {
  long n = 0;
  for (node_iterator nd = m->mesh.node_begin(); nd != m->mesh.node_end(); ++nd)
    for (auto& kv : nd->m_K_row) {
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) vals[9 * n + 3 * r + c] = kv.second(r, c);
      ++n;
    }
}

void orc_get_re(orc_mesh* m, double* re) {
  size_t t = 0;
  for (tetrahedron_iterator T = m->mesh.tetrahedron_begin(); T != m->mesh.tetrahedron_end(); ++T, ++t)
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) re[9 * t + 3 * r + c] = T->m_Re(r, c);
}

void orc_get_plastic(orc_mesh* m, double* pl) {
  size_t t = 0;
  for (tetrahedron_iterator T = m->mesh.tetrahedron_begin(); T != m->mesh.tetrahedron_end(); ++T, ++t)
    for (int q = 0; q < 6; ++q) pl[6 * t + q] = T->m_plastic[q];
}

void orc_get_volume(orc_mesh* m, double* vol) {
  size_t t = 0;
  for (tetrahedron_iterator T = m->mesh.tetrahedron_begin(); T != m->mesh.tetrahedron_end(); ++T, ++t)
    vol[t] = T->m_V;
}

}  // extern "C"
