// Minimal stand-in for boost/utility/enable_if.hpp (oracle build only).
#ifndef OTFEM_SHIM_BOOST_ENABLE_IF_HPP
#define OTFEM_SHIM_BOOST_ENABLE_IF_HPP
#include <type_traits>
namespace boost {
template <class Cond, class T = void>
struct enable_if : std::enable_if<Cond::value, T> {};
template <bool B, class T = void>
struct enable_if_c : std::enable_if<B, T> {};
}  // namespace boost
#endif
