// Test stand-in for the parts of OpenTissue's core/math that the fem path
// and its host code use: Vector3, Matrix3x3 (zero-initialised, element
// access by operator()), BasicMathTypes.  Written for the drop-in tests only.
#ifndef OTFEM_TEST_MATH_BASIC_TYPES_H
#define OTFEM_TEST_MATH_BASIC_TYPES_H
#include <cstddef>

namespace OpenTissue {
namespace math {

template <typename T>
class Vector3 {
 public:
  typedef T value_type;
  Vector3() : x(0), y(0), z(0) {}
  Vector3(T a, T b, T c) : x(a), y(b), z(c) {}
  T& operator()(std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
  T const& operator()(std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
  T& operator[](std::size_t i) { return (*this)(i); }
  T const& operator[](std::size_t i) const { return (*this)(i); }
  void clear() { x = y = z = 0; }
  T x, y, z;
};

template <typename T>
class Matrix3x3 {
 public:
  typedef T value_type;
  Matrix3x3() {
    for (int i = 0; i < 9; ++i) m[i] = 0;
  }
  T& operator()(std::size_t r, std::size_t c) { return m[3 * r + c]; }
  T const& operator()(std::size_t r, std::size_t c) const { return m[3 * r + c]; }
  void clear() {
    for (int i = 0; i < 9; ++i) m[i] = 0;
  }

 private:
  T m[9];
};

template <typename real_type_, typename index_type_>
class BasicMathTypes {
 public:
  typedef real_type_ real_type;
  typedef index_type_ index_type;
  typedef Vector3<real_type> vector3_type;
  typedef Matrix3x3<real_type> matrix3x3_type;
};

}  // namespace math
}  // namespace OpenTissue
#endif
