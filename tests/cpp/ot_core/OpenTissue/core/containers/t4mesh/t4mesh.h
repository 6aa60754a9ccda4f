// Test stand-in for OpenTissue's t4mesh container (core/containers/t4mesh):
// the subset of its interface that the fem path and its host code use --
// index-based node/tet storage in std::vectors named m_nodes / m_tetrahedra,
// bounds-checked node(idx) that throws std::out_of_range, index iterators,
// insert(), idx(), node_idx(), i()/j()/k()/m().  Written for the drop-in
// tests only.
#ifndef OTFEM_TEST_T4MESH_H
#define OTFEM_TEST_T4MESH_H
#include <array>
#include <cstddef>
#include <stdexcept>
#include <vector>

namespace OpenTissue {
namespace t4mesh {
namespace detail {

template <typename container_type>
class IndexIterator {
 public:
  typedef typename container_type::value_type value_type;
  IndexIterator() : m_c(0), m_i(0) {}
  IndexIterator(container_type const& c, std::size_t i) : m_c(const_cast<container_type*>(&c)), m_i(i) {}
  value_type& operator*() const {
    if (m_i >= m_c->size()) throw std::out_of_range("IndexIterator: past the end");
    return (*m_c)[m_i];
  }
  value_type* operator->() const { return &**this; }
  IndexIterator& operator++() {
    if (m_i >= m_c->size()) throw std::out_of_range("IndexIterator: increment past the end");
    ++m_i;
    return *this;
  }
  bool operator==(IndexIterator const& o) const { return m_c == o.m_c && m_i == o.m_i; }
  bool operator!=(IndexIterator const& o) const { return !(*this == o); }

 private:
  container_type* m_c;
  std::size_t m_i;
};

template <typename M, typename N, typename T>
class T4Mesh;

template <typename mesh_type>
class T4Node : public mesh_type::node_traits {
 public:
  typedef typename mesh_type::index_type index_type;
  index_type idx() const { return m_idx; }
  index_type m_idx;
  mesh_type* m_owner;
};

template <typename mesh_type>
class T4Tetrahedron : public mesh_type::tetrahedron_traits {
 public:
  typedef typename mesh_type::index_type index_type;
  typedef typename mesh_type::node_iterator node_iterator;
  index_type idx() const { return m_idx; }
  index_type node_idx(index_type k) const { return m_nodes[k]; }
  node_iterator i() { return m_owner->node(m_nodes[0]); }
  node_iterator j() { return m_owner->node(m_nodes[1]); }
  node_iterator k() { return m_owner->node(m_nodes[2]); }
  node_iterator m() { return m_owner->node(m_nodes[3]); }
  node_iterator node(int local) { return m_owner->node(m_nodes[local]); }
  index_type m_idx;
  mesh_type* m_owner;
  std::array<index_type, 4> m_nodes;
};

template <typename M, typename N, typename T>
class T4Mesh {
 public:
  typedef M math_types;
  typedef N node_traits;
  typedef T tetrahedron_traits;
  typedef T4Mesh<M, N, T> mesh_type;
  typedef T4Node<mesh_type> node_type;
  typedef T4Tetrahedron<mesh_type> tetrahedron_type;
  typedef std::size_t index_type;

 protected:
  typedef std::vector<node_type> node_container;
  typedef std::vector<tetrahedron_type> tetrahedra_container;
  node_container m_nodes;
  tetrahedra_container m_tetrahedra;

 public:
  typedef IndexIterator<node_container> node_iterator;
  typedef IndexIterator<tetrahedra_container> tetrahedron_iterator;

  node_iterator node_begin() { return node_iterator(m_nodes, 0); }
  node_iterator node_end() { return node_iterator(m_nodes, m_nodes.size()); }
  tetrahedron_iterator tetrahedron_begin() { return tetrahedron_iterator(m_tetrahedra, 0); }
  tetrahedron_iterator tetrahedron_end() { return tetrahedron_iterator(m_tetrahedra, m_tetrahedra.size()); }
  std::size_t size_nodes() const { return m_nodes.size(); }
  std::size_t size_tetrahedra() const { return m_tetrahedra.size(); }
  void clear() {
    m_nodes.clear();
    m_tetrahedra.clear();
  }
  node_iterator node(index_type idx) {
    if (idx >= m_nodes.size()) throw std::out_of_range("T4Mesh::node(idx): idx out of range");
    return node_iterator(m_nodes, idx);
  }
  node_iterator insert() {
    m_nodes.push_back(node_type());
    m_nodes.back().m_idx = m_nodes.size() - 1;
    m_nodes.back().m_owner = this;
    return node_iterator(m_nodes, m_nodes.size() - 1);
  }
  tetrahedron_iterator insert(index_type i, index_type j, index_type k, index_type m) {
    if (i >= m_nodes.size() || j >= m_nodes.size() || k >= m_nodes.size() || m >= m_nodes.size())
      throw std::out_of_range("T4Mesh::insert(): node index out of range");
    m_tetrahedra.push_back(tetrahedron_type());
    tetrahedron_type& t = m_tetrahedra.back();
    t.m_idx = m_tetrahedra.size() - 1;
    t.m_owner = this;
    t.m_nodes = {{i, j, k, m}};
    return tetrahedron_iterator(m_tetrahedra, t.m_idx);
  }
};

}  // namespace detail

template <typename M, typename N, typename T>
class T4Mesh : public detail::T4Mesh<M, N, T> {};

}  // namespace t4mesh
}  // namespace OpenTissue
#endif
