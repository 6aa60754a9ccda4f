// Minimal stand-in for boost::indirect_iterator (boost/iterator/
// indirect_iterator.hpp), written against the standard library for the
// reference build of the oracle: an iterator over pointers that dereferences
// twice.  Only what OpenTissue's spatial hashing grid uses
// (collision/spatial_hashing/spatial_hashing_grid.h): construction from the
// pointer iterator, *, ->, ++, == and !=.
#ifndef OTFEM_SHIM_BOOST_INDIRECT_ITERATOR_HPP
#define OTFEM_SHIM_BOOST_INDIRECT_ITERATOR_HPP

#include <cstddef>
#include <iterator>

namespace boost {

template <class Iterator, class Value>
class indirect_iterator {
 public:
  typedef Value value_type;
  typedef Value& reference;
  typedef Value* pointer;
  typedef std::ptrdiff_t difference_type;
  typedef std::forward_iterator_tag iterator_category;

  indirect_iterator() {}
  explicit indirect_iterator(Iterator it) : it_(it) {}

  reference operator*() const { return **it_; }
  pointer operator->() const { return &**it_; }
  indirect_iterator& operator++() {
    ++it_;
    return *this;
  }
  indirect_iterator operator++(int) {
    indirect_iterator old(*this);
    ++it_;
    return old;
  }
  bool operator==(const indirect_iterator& o) const { return it_ == o.it_; }
  bool operator!=(const indirect_iterator& o) const { return it_ != o.it_; }

 private:
  Iterator it_;
};

}  // namespace boost

#endif
