#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_EXPORT_K_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_EXPORT_K_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// fem::export_K (reference: fem_export_k.h:23-68), same signature and output:
// bigK is resized to 3N x 3N and cleared, then filled row by row with
// push_back(row, col, value): a fixed node's rows get 1.0 on the diagonal, a
// free node's rows get the entries of its K_row blocks whose column node is
// not fixed, in ascending column order.  K comes from the device (the last
// reference-solver step), exported as block CSR by otfem_export_k_csr.
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/dynamics/fem/fem_mesh.h>

#include <vector>

namespace OpenTissue {
namespace fem {

template <typename fem_mesh, typename matrix_type>
inline void export_K(fem_mesh& mesh, matrix_type& bigK) {
  unsigned int const N = static_cast<unsigned int>(mesh.size_nodes());
  bigK.resize(N * 3, N * 3, false);
  bigK.clear();
  otfem_handle h = mesh.gpu_state().handle();
  if (!h) throw std::logic_error("fem::export_K(): fem::init has not been called on this mesh");
  int64_t nnz = 0;
  gpu::check(otfem_export_k_csr(h, &nnz, 0, 0, 0), "fem::export_K");
  std::vector<int32_t> rp(N + 1), cols(std::size_t(nnz) + 1);
  std::vector<double> vals(9 * std::size_t(nnz) + 1);
  gpu::check(otfem_export_k_csr(h, &nnz, rp.data(), cols.data(), vals.data()), "fem::export_K");
  unsigned int row = 0;
  for (unsigned int i = 0; i < N; ++i) {
    bool fixed = mesh.node_at(i).m_fixed;
    for (unsigned int r = 0; r < 3; ++r, ++row) {
      if (fixed) {
        bigK.push_back(row, row, 1.0);
        continue;
      }
      for (int32_t q = rp[i]; q < rp[i + 1]; ++q) {
        unsigned int column = unsigned(cols[q]) * 3;
        for (unsigned int c = 0; c < 3; ++c) bigK.push_back(row, column + c, vals[9 * std::size_t(q) + 3 * r + c]);
      }
    }
  }
}

}  // namespace fem
}  // namespace OpenTissue

#endif
