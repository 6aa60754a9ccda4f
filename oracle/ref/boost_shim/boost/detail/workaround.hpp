// Minimal stand-in for boost/detail/workaround.hpp (oracle build only):
// no compiler workaround is active.
#ifndef OTFEM_SHIM_BOOST_WORKAROUND_HPP
#define OTFEM_SHIM_BOOST_WORKAROUND_HPP
#define BOOST_WORKAROUND(symbol, test) 0
#endif
