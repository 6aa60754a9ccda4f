// Test stand-in for t4mesh::generate_blocks (t4mesh_block_generator.h:32-110):
// (I+1)(J+1)(K+1) nodes at (w x, h z, d y) in x-major, z-minor order and five
// tets per block, split by the parity of i+j+k.  Written for the drop-in tests.
#ifndef OTFEM_TEST_T4MESH_BLOCK_GENERATOR_H
#define OTFEM_TEST_T4MESH_BLOCK_GENERATOR_H
namespace OpenTissue {
namespace t4mesh {

template <typename real_type, typename t4mesh_type>
void generate_blocks(unsigned int const& I, unsigned int const& J, unsigned int const& K,
                     real_type const& w, real_type const& h, real_type const& d, t4mesh_type& mesh) {
  mesh.clear();
  for (unsigned int x = 0; x <= I; ++x)
    for (unsigned int y = 0; y <= J; ++y)
      for (unsigned int z = 0; z <= K; ++z) {
        typename t4mesh_type::node_iterator n = mesh.insert();
        n->m_coord(0) = w * x;
        n->m_coord(2) = d * y;
        n->m_coord(1) = h * z;
      }
  for (unsigned int i = 0; i < I; ++i)
    for (unsigned int j = 0; j < J; ++j)
      for (unsigned int k = 0; k < K; ++k) {
        unsigned int c0 = (i * (J + 1) + j) * (K + 1) + k, c1 = c0 + 1;
        unsigned int c3 = ((i + 1) * (J + 1) + j) * (K + 1) + k, c2 = c3 + 1;
        unsigned int c7 = ((i + 1) * (J + 1) + (j + 1)) * (K + 1) + k, c6 = c7 + 1;
        unsigned int c4 = (i * (J + 1) + (j + 1)) * (K + 1) + k, c5 = c4 + 1;
        if ((i + j + k) % 2 == 1) {
          mesh.insert(c1, c2, c6, c3);
          mesh.insert(c3, c6, c4, c7);
          mesh.insert(c1, c4, c6, c5);
          mesh.insert(c1, c3, c4, c0);
          mesh.insert(c1, c6, c4, c3);
        } else {
          mesh.insert(c2, c0, c5, c1);
          mesh.insert(c2, c7, c0, c3);
          mesh.insert(c2, c5, c7, c6);
          mesh.insert(c0, c7, c5, c4);
          mesh.insert(c2, c0, c7, c5);
        }
      }
}

}  // namespace t4mesh
}  // namespace OpenTissue
#endif
