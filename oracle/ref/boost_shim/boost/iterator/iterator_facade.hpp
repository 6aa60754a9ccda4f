// Minimal stand-in for boost/iterator/iterator_facade.hpp (oracle build only).
// Supports the forward-traversal subset that OpenTissue's IndexIterator uses:
// the derived class supplies dereference(), increment() and equal(), and
// iterator_core_access forwards to them.
#ifndef OTFEM_SHIM_BOOST_ITERATOR_FACADE_HPP
#define OTFEM_SHIM_BOOST_ITERATOR_FACADE_HPP
#include <cstddef>
#include <iterator>
#include <boost/detail/workaround.hpp>
#include <boost/utility/enable_if.hpp>
#include <boost/type_traits/is_convertible.hpp>
namespace boost {

struct forward_traversal_tag : std::forward_iterator_tag {};

class iterator_core_access {
 public:
  template <class F>
  static typename F::reference dereference(F const& f) { return f.dereference(); }
  template <class F>
  static void increment(F& f) { f.increment(); }
  template <class F1, class F2>
  static bool equal(F1 const& a, F2 const& b) { return a.equal(b); }
};

template <class Derived, class Value, class Traversal, class Reference = Value&,
          class Difference = std::ptrdiff_t>
class iterator_facade {
 public:
  typedef Value value_type;
  typedef Reference reference;
  typedef Value* pointer;
  typedef Difference difference_type;
  typedef std::forward_iterator_tag iterator_category;

  reference operator*() const { return iterator_core_access::dereference(derived()); }
  pointer operator->() const { return &iterator_core_access::dereference(derived()); }
  Derived& operator++() {
    iterator_core_access::increment(derived());
    return derived();
  }
  Derived operator++(int) {
    Derived tmp(derived());
    ++*this;
    return tmp;
  }

 private:
  Derived& derived() { return *static_cast<Derived*>(this); }
  Derived const& derived() const { return *static_cast<Derived const*>(this); }
};

template <class D1, class V1, class T1, class R1, class F1, class D2, class V2, class T2, class R2, class F2>
inline bool operator==(iterator_facade<D1, V1, T1, R1, F1> const& a, iterator_facade<D2, V2, T2, R2, F2> const& b) {
  return iterator_core_access::equal(static_cast<D1 const&>(a), static_cast<D2 const&>(b));
}
template <class D1, class V1, class T1, class R1, class F1, class D2, class V2, class T2, class R2, class F2>
inline bool operator!=(iterator_facade<D1, V1, T1, R1, F1> const& a, iterator_facade<D2, V2, T2, R2, F2> const& b) {
  return !iterator_core_access::equal(static_cast<D1 const&>(a), static_cast<D2 const&>(b));
}

}  // namespace boost
#endif
