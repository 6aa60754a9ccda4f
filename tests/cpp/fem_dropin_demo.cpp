// Host program written against OpenTissue's fem interface, as reference user
// code is: build a block beam with t4mesh::generate_blocks, fix the x = 0
// face, fem::init, then per step set m_f_external = m g and call
// fem::simulate.  Compiled against the drop-in headers (include/) and linked
// with libotfem_gpu.so; used by tests/test_dropin_cpp.py.
//
// usage: fem_dropin_demo I J K steps solver out.bin [export.bin]
//   solver: reference | sequential | mixed | projected | detail
//     (detail: each step is the reference's own sequence of fem::detail
//     calls, fem_simulate.h:94-111, instead of fem::simulate)
//   out.bin: per step the N x 3 positions then the N x 3 velocities (doubles)
//   export.bin: fem::export_K triplets after step 1 (int row, int col, double);
//     in detail mode the host m_K_row maps after step 1 instead (int row, int
//     col, 9 doubles per entry, rows and keys in order)
#include <OpenTissue/configuration.h>
#include <OpenTissue/core/math/math_basic_types.h>
#include <OpenTissue/core/containers/t4mesh/util/t4mesh_block_generator.h>
#include <OpenTissue/dynamics/fem/fem.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <vector>

typedef OpenTissue::math::BasicMathTypes<double, size_t> math_types;
typedef OpenTissue::fem::Mesh<math_types> mesh_type;

struct TripletSink {  // uBLAS-style: resize, clear, push_back
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

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: %s I J K steps solver out.bin [export.bin]\n", argv[0]);
    return 2;
  }
  unsigned I = unsigned(std::atoi(argv[1])), J = unsigned(std::atoi(argv[2])), K = unsigned(std::atoi(argv[3]));
  int steps = std::atoi(argv[4]);
  const char* solver = argv[5];
  try {
    mesh_type mesh;
    OpenTissue::t4mesh::generate_blocks(I, J, K, 0.1, 0.1, 0.1, mesh);
    for (mesh_type::node_iterator n = mesh.node_begin(); n != mesh.node_end(); ++n) {
      n->m_model_coord = n->m_coord;
      n->m_fixed = n->idx() < (J + 1) * (K + 1);
    }
    OpenTissue::fem::init(mesh, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0);
    OpenTissue::fem::SolverParams params = OpenTissue::fem::reference_solver();
    if (std::strcmp(solver, "sequential") == 0) params.sequential_dots = 1;
    if (std::strcmp(solver, "mixed") == 0) params = OpenTissue::fem::mixed_solver(1e-6);
    if (std::strcmp(solver, "projected") == 0) params = OpenTissue::fem::projected_solver(1e-6, 4);
    if (std::strcmp(solver, "extrapolated") == 0) params = OpenTissue::fem::extrapolated_solver(1e-6, 4);
    FILE* out = std::fopen(argv[6], "wb");
    if (!out) return 3;
    std::vector<double> buf(3 * mesh.size_nodes());
    for (int s = 1; s <= steps; ++s) {
      for (mesh_type::node_iterator n = mesh.node_begin(); n != mesh.node_end(); ++n) {
        n->m_f_external.clear();
        if (!n->m_fixed) n->m_f_external(1) = -9.81 * n->m_mass;
      }
      if (std::strcmp(solver, "detail") == 0) {
        namespace fd = OpenTissue::fem::detail;
        fd::clear_stiffness_assembly(mesh.node_begin(), mesh.node_end());
        fd::update_orientation(mesh.tetrahedron_begin(), mesh.tetrahedron_end());
        fd::stiffness_assembly(mesh.tetrahedron_begin(), mesh.tetrahedron_end());
        fd::add_plasticity_force(mesh.tetrahedron_begin(), mesh.tetrahedron_end(), 0.01);
        fd::dynamics_assembly(mesh, 2.0, 0.01);
        fd::conjugate_gradients(mesh, 20u, 20u);
        fd::position_update(mesh, 0.01);
      } else if (std::strcmp(solver, "reference") == 0) {
        OpenTissue::fem::simulate(mesh, 0.01, true);
      } else {
        OpenTissue::fem::simulate(mesh, 0.01, true, params);
      }
      size_t i = 0;
      for (mesh_type::node_iterator n = mesh.node_begin(); n != mesh.node_end(); ++n, ++i)
        for (int c = 0; c < 3; ++c) buf[3 * i + c] = n->m_coord(c);
      std::fwrite(buf.data(), sizeof(double), buf.size(), out);
      i = 0;
      for (mesh_type::node_iterator n = mesh.node_begin(); n != mesh.node_end(); ++n, ++i)
        for (int c = 0; c < 3; ++c) buf[3 * i + c] = n->m_velocity(c);
      std::fwrite(buf.data(), sizeof(double), buf.size(), out);
      if (s == 1 && argc > 7 && std::strcmp(solver, "detail") == 0) {
        FILE* ex = std::fopen(argv[7], "wb");
        if (!ex) return 3;
        for (mesh_type::node_iterator n = mesh.node_begin(); n != mesh.node_end(); ++n)
          for (mesh_type::node_type::matrix_iterator K = n->Kbegin(); K != n->Kend(); ++K) {
            int rc[2] = {int(n->idx()), K->first};
            std::fwrite(rc, sizeof(int), 2, ex);
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c) {
                double v = K->second(r, c);
                std::fwrite(&v, sizeof(double), 1, ex);
              }
          }
        std::fclose(ex);
      } else if (s == 1 && argc > 7) {
        TripletSink sink;
        OpenTissue::fem::export_K(mesh, sink);
        FILE* ex = std::fopen(argv[7], "wb");
        if (!ex) return 3;
        for (size_t q = 0; q < sink.vals.size(); ++q) {
          std::fwrite(&sink.rows[q], sizeof(int), 1, ex);
          std::fwrite(&sink.cols[q], sizeof(int), 1, ex);
          std::fwrite(&sink.vals[q], sizeof(double), 1, ex);
        }
        std::fclose(ex);
      }
    }
    std::fclose(out);
    // a mesh that was never initialised throws like the reference's misuse
    mesh_type fresh;
    OpenTissue::t4mesh::generate_blocks(1u, 1u, 1u, 0.1, 0.1, 0.1, fresh);
    try {
      OpenTissue::fem::simulate(fresh, 0.01, true);
      std::fprintf(stderr, "expected std::logic_error\n");
      return 4;
    } catch (std::logic_error const&) {
    }
    try {
      OpenTissue::fem::detail::update_orientation(fresh.tetrahedron_begin(), fresh.tetrahedron_end());
      std::fprintf(stderr, "expected std::logic_error from fem::detail\n");
      return 4;
    } catch (std::logic_error const&) {
    }
    if (std::strcmp(solver, "detail") == 0) {
      // the device runs a step on whole meshes: a partial range throws
      mesh_type::tetrahedron_iterator last = mesh.tetrahedron_begin();
      ++last;
      try {
        OpenTissue::fem::detail::update_orientation(mesh.tetrahedron_begin(), last);
        std::fprintf(stderr, "expected std::invalid_argument\n");
        return 4;
      } catch (std::invalid_argument const&) {
      }
    }
  } catch (std::exception const& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
