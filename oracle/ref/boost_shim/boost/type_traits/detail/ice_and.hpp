// Minimal stand-in for boost/type_traits/detail/ice_and.hpp (oracle build only).
#ifndef OTFEM_SHIM_BOOST_ICE_AND_HPP
#define OTFEM_SHIM_BOOST_ICE_AND_HPP
namespace boost { namespace type_traits {
template <bool b1, bool b2, bool b3 = true, bool b4 = true, bool b5 = true, bool b6 = true, bool b7 = true>
struct ice_and { static const bool value = b1 && b2 && b3 && b4 && b5 && b6 && b7; };
}}  // namespace boost::type_traits
#endif
