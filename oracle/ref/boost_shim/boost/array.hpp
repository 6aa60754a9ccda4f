// Minimal stand-in for boost/array.hpp (oracle build only): std::array plus
// boost::array's assign(value), which fills every element.
#ifndef OTFEM_SHIM_BOOST_ARRAY_HPP
#define OTFEM_SHIM_BOOST_ARRAY_HPP
#include <array>
#include <cstddef>
namespace boost {
template <class T, std::size_t N>
struct array : std::array<T, N> {
  void assign(T const& value) { this->fill(value); }
};
}  // namespace boost
#endif
