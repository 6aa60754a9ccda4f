// FP64 <-> (hi, lo) FP32 pair conversions by bit manipulation.
//
// On GB300 every FP64 instruction, conversions included, holds the issuing SM
// sub-partition for ~64 cycles, so the mixed solver converts its FP64 node
// data (masses, velocities, positions, forces) to (hi, lo) float pairs and
// back with integer instructions only, and does its arithmetic on the pairs.
// The functions are host and device code so that the CPU tests can check them
// bit for bit.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define OTFEM_HD __host__ __device__ __forceinline__
#else
#define OTFEM_HD inline
#endif

namespace otfem {
namespace dfbits {

OTFEM_HD uint64_t bits64(double d) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(d));
#else
  uint64_t u;
  std::memcpy(&u, &d, sizeof u);
  return u;
#endif
}
OTFEM_HD double from_bits64(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double d;
  std::memcpy(&d, &u, sizeof d);
  return d;
#endif
}
OTFEM_HD uint32_t bits32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, sizeof u);
  return u;
#endif
}
OTFEM_HD float from_bits32(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
#endif
}
// Position of the highest set bit of x != 0 (0..63).
OTFEM_HD int top_bit(uint64_t x) {
#ifdef __CUDA_ARCH__
  return 63 - __clzll(static_cast<long long>(x));
#else
  return 63 - __builtin_clzll(x);
#endif
}

constexpr uint64_t kMant52 = (uint64_t(1) << 52) - 1;

// x = hi + lo + e with |e| < 2^-47 |x| for |x| >= 2^-74: hi is x truncated to
// 24 significant bits, lo the remaining 29 bits truncated to 24.  hi and lo
// carry x's sign.  Magnitudes below the FP32 normal range give 0 (hi, or lo
// alone when the remainder is that small, so |e| < 2^-23 |x| below 2^-74),
// above it infinity; NaN gives NaN.
OTFEM_HD void split(double x, float& hi, float& lo) {
  const uint64_t u = bits64(x);
  const uint32_t sign = uint32_t(u >> 32) & 0x80000000u;
  const int e = int((u >> 52) & 0x7ffu);
  const uint64_t m = u & kMant52;
  lo = from_bits32(sign);
  if (e == 0x7ff) {
    hi = from_bits32(m != 0 ? 0x7fc00000u : (sign | 0x7f800000u));
    return;
  }
  const int E = e - 1023;
  if (E < -126) {
    hi = from_bits32(sign);
    return;
  }
  if (E > 127) {
    hi = from_bits32(sign | 0x7f800000u);
    return;
  }
  hi = from_bits32(sign | (uint32_t(E + 127) << 23) | uint32_t(m >> 29));
  const uint64_t r = m & ((uint64_t(1) << 29) - 1);  // the rest: r * 2^(E - 52)
  if (r == 0) return;
  const int p = top_bit(r);  // 0..28
  const int El = E - 52 + p;
  if (El < -126) return;
  const uint32_t ml = uint32_t(p >= 23 ? (r >> (p - 23)) : (r << (23 - p))) & 0x7fffffu;
  lo = from_bits32(sign | (uint32_t(El + 127) << 23) | ml);
}

// x truncated to 24 significant bits (the hi part of split).
OTFEM_HD float trunc_f32(double x) {
  float hi, lo;
  split(x, hi, lo);
  return hi;
}

// The FP64 value of an FP32 number (exact); FP32 subnormals give 0.
OTFEM_HD double widen(float f) {
  const uint32_t u = bits32(f);
  const uint64_t sign = uint64_t(u & 0x80000000u) << 32;
  const int e = int((u >> 23) & 0xffu);
  const uint64_t m = uint64_t(u & 0x7fffffu) << 29;
  if (e == 0) return from_bits64(sign);
  if (e == 0xff) return from_bits64(sign | (uint64_t(0x7ff) << 52) | m);
  return from_bits64(sign | (uint64_t(e - 127 + 1023) << 52) | m);
}

// hi + lo in FP64 for a pair with |lo| <= 2^-22 |hi| (or hi == 0): exact while
// lo's bits lie within the 53 bits below hi's leading bit, else truncated
// (error below 2^-51 |hi|).
OTFEM_HD double join(float hi, float lo) {
  uint32_t uh = bits32(hi), ul = bits32(lo);
  int eh = int((uh >> 23) & 0xffu), el = int((ul >> 23) & 0xffu);
  if (el > eh) {  // outside the contract: take the larger part as the leading one
    const uint32_t tu = uh;
    uh = ul;
    ul = tu;
    const int te = eh;
    eh = el;
    el = te;
  }
  if (eh == 0) return widen(from_bits32(ul));
  if (el == 0 || eh == 0xff) return widen(from_bits32(uh));
  const uint64_t sign = uint64_t(uh & 0x80000000u) << 32;
  int E = eh - 127;
  // significands as 53-bit integers (the implicit bit at position 52)
  const uint64_t H = (uint64_t(1) << 52) | (uint64_t(uh & 0x7fffffu) << 29);
  const uint64_t L = (uint64_t(1) << 52) | (uint64_t(ul & 0x7fffffu) << 29);
  const int shift = eh - el;
  const uint64_t La = shift >= 64 ? 0 : (L >> shift);
  uint64_t S = ((uh ^ ul) & 0x80000000u) ? H - La : H + La;
  if (S >> 53) {
    S >>= 1;
    ++E;
  } else {
    while (S != 0 && !(S >> 52)) {
      S <<= 1;
      --E;
    }
    if (S == 0) return from_bits64(sign);
  }
  if (E + 1023 <= 0) return from_bits64(sign);
  if (E + 1023 >= 0x7ff) return from_bits64(sign | (uint64_t(0x7ff) << 52));
  return from_bits64(sign | (uint64_t(E + 1023) << 52) | (S & kMant52));
}

}  // namespace dfbits
}  // namespace otfem
