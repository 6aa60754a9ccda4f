// Minimal stand-in for boost/type_traits.hpp (oracle build only).
#ifndef OTFEM_SHIM_BOOST_TYPE_TRAITS_HPP
#define OTFEM_SHIM_BOOST_TYPE_TRAITS_HPP
#include <type_traits>
#include <boost/type_traits/is_convertible.hpp>
namespace boost {
using std::remove_cv;
using std::is_same;
template <class T>
struct has_trivial_assign : std::integral_constant<bool, std::is_trivially_copy_assignable<T>::value> {};
}  // namespace boost
#endif
