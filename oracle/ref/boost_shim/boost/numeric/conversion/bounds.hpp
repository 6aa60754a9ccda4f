// Minimal stand-in for boost/numeric/conversion/bounds.hpp (oracle build only).
#ifndef OTFEM_SHIM_BOOST_BOUNDS_HPP
#define OTFEM_SHIM_BOOST_BOUNDS_HPP
#include <limits>
namespace boost { namespace numeric {
template <class T>
struct bounds {
  static T highest() { return std::numeric_limits<T>::max(); }
  static T lowest() { return std::numeric_limits<T>::lowest(); }
  static T smallest() {
    return std::numeric_limits<T>::is_integer ? T(1) : std::numeric_limits<T>::min();
  }
};
}}  // namespace boost::numeric
#endif
