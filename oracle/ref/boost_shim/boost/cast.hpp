// Minimal stand-in for boost/cast.hpp, written for the oracle build only.
// The reference FEM path uses numeric_cast between identical floating types,
// so a static_cast preserves every value bit for bit.
#ifndef OTFEM_SHIM_BOOST_CAST_HPP
#define OTFEM_SHIM_BOOST_CAST_HPP
namespace boost {
template <class Target, class Source>
inline Target numeric_cast(Source const& s) { return static_cast<Target>(s); }
}  // namespace boost
#endif
