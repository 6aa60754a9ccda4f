// otfem_refmath.cuh -- FP64 3x3 helpers that keep the association order of
// OpenTissue's Vector3 / Matrix3x3 operators (core/math/math_vector3.h,
// core/math/math_matrix3x3.h).  Included only by translation units compiled
// with -fmad=false, where each expression below is exactly the IEEE operation
// sequence of the reference.
#pragma once

#include <cuda_runtime.h>

namespace otfem {
namespace ref {

// Matrix3x3 * Vector3: each row dotted as x*v0 + y*v1 + z*v2
// (math_matrix3x3.h:151, math_vector3.h:194).
__host__ __device__ inline void mv(const double* M, const double* v, double* out) {
  double a = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
  double b = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
  double c = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
  out[0] = a;
  out[1] = b;
  out[2] = c;
}

// Matrix3x3 * Matrix3x3: C(r,c) = 0, then += A(r,i)*B(i,c) for i = 0..2
// (math_matrix3x3.h:254-266).
__host__ __device__ inline void mm(const double* A, const double* B, double* C) {
  double t[9];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i) s += A[r * 3 + i] * B[i * 3 + c];
      t[r * 3 + c] = s;
    }
#pragma unroll
  for (int q = 0; q < 9; ++q) C[q] = t[q];
}

__host__ __device__ inline void transpose(const double* M, double* Mt) {
  double t[9] = {M[0], M[3], M[6], M[1], M[4], M[7], M[2], M[5], M[8]};
#pragma unroll
  for (int q = 0; q < 9; ++q) Mt[q] = t[q];
}

__host__ __device__ inline double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// ortonormalize (math_matrix3x3.h:536-558): row Gram-Schmidt with true
// divisions by the row lengths and row2 = cross(row0, row1)
// (math_vector3.h:375-378).
__host__ __device__ inline void ortonormalize(double* A) {
  double r0[3] = {A[0], A[1], A[2]}, r1[3] = {A[3], A[4], A[5]};
  double l0 = sqrt(dot3(r0, r0));
  if (l0 != 0.0) {
    r0[0] /= l0;
    r0[1] /= l0;
    r0[2] /= l0;
  }
  double d = dot3(r0, r1);
  r1[0] -= r0[0] * d;
  r1[1] -= r0[1] * d;
  r1[2] -= r0[2] * d;
  double l1 = sqrt(dot3(r1, r1));
  if (l1 != 0.0) {
    r1[0] /= l1;
    r1[1] /= l1;
    r1[2] /= l1;
  }
  A[0] = r0[0]; A[1] = r0[1]; A[2] = r0[2];
  A[3] = r1[0]; A[4] = r1[1]; A[5] = r1[2];
  A[6] = r0[1] * r1[2] - r1[1] * r0[2];
  A[7] = -r0[0] * r1[2] + r1[0] * r0[2];
  A[8] = r0[0] * r1[1] - r1[0] * r0[1];
}

// The orientation of one tet (fem_update_orientation.h:31,173-208):
// Re = ortonormalize([q1-q0, q2-q0, q3-q0] * [n1; n2; n3]) with the n-vectors
// from the rest edges scaled by div6V = (1/V)*6.
__host__ __device__ inline void orientation(const double* e /*e10,e20,e30*/, double V,
                                            const double* p0, const double* p1,
                                            const double* p2, const double* p3, double* R) {
  double div6V = 1.0 / V * 6.0;
  double e1x = e[0], e1y = e[1], e1z = e[2];
  double e2x = e[3], e2y = e[4], e2z = e[5];
  double e3x = e[6], e3y = e[7], e3z = e[8];
  double n1x = (e2y * e3z - e3y * e2z) * div6V;
  double n1y = (e3x * e2z - e2x * e3z) * div6V;
  double n1z = (e2x * e3y - e3x * e2y) * div6V;
  double n2x = (e1z * e3y - e1y * e3z) * div6V;
  double n2y = (e1x * e3z - e1z * e3x) * div6V;
  double n2z = (e1y * e3x - e1x * e3y) * div6V;
  double n3x = (e1y * e2z - e1z * e2y) * div6V;
  double n3y = (e1z * e2x - e1x * e2z) * div6V;
  double n3z = (e1x * e2y - e1y * e2x) * div6V;
  e1x = p1[0] - p0[0]; e1y = p1[1] - p0[1]; e1z = p1[2] - p0[2];
  e2x = p2[0] - p0[0]; e2y = p2[1] - p0[1]; e2z = p2[2] - p0[2];
  e3x = p3[0] - p0[0]; e3y = p3[1] - p0[1]; e3z = p3[2] - p0[2];
  R[0] = e1x * n1x + e2x * n2x + e3x * n3x;
  R[1] = e1x * n1y + e2x * n2y + e3x * n3y;
  R[2] = e1x * n1z + e2x * n2z + e3x * n3z;
  R[3] = e1y * n1x + e2y * n2x + e3y * n3x;
  R[4] = e1y * n1y + e2y * n2y + e3y * n3y;
  R[5] = e1y * n1z + e2y * n2z + e3y * n3z;
  R[6] = e1z * n1x + e2z * n2x + e3z * n3x;
  R[7] = e1z * n1y + e2z * n2y + e3z * n3y;
  R[8] = e1z * n1z + e2z * n2z + e3z * n3z;
  ortonormalize(R);
}

}  // namespace ref
}  // namespace otfem
