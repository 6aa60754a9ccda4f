// Minimal stand-in for boost/type_traits/is_convertible.hpp (oracle build only).
#ifndef OTFEM_SHIM_BOOST_IS_CONVERTIBLE_HPP
#define OTFEM_SHIM_BOOST_IS_CONVERTIBLE_HPP
#include <type_traits>
namespace boost { using std::is_convertible; }
#endif
