// Bit-level FP64 <-> (hi, lo) conversions of otfem_df.h against long double
// arithmetic and the C library's rounding modes.  Prints "ok" or the first
// failure and exits nonzero.
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <random>

#include "otfem_df.h"

using otfem::dfbits::join;
using otfem::dfbits::split;
using otfem::dfbits::trunc_f32;
using otfem::dfbits::widen;

static int fail(const char* what, double x) {
  std::printf("FAIL %s at %.17g\n", what, x);
  return 1;
}

static float toward_zero(double x) {
  std::fesetround(FE_TOWARDZERO);
  volatile double vx = x;
  volatile float f = static_cast<float>(vx);
  std::fesetround(FE_TONEAREST);
  return f;
}

int main() {
  std::mt19937_64 rng(20261203);
  std::uniform_real_distribution<double> expo(-120.0, 120.0), mant(1.0, 2.0);
  for (int n = 0; n < 200000; ++n) {
    const double x = (n & 1 ? -1.0 : 1.0) * mant(rng) * std::pow(2.0, expo(rng));
    float hi, lo;
    split(x, hi, lo);
    if (hi != toward_zero(x)) return fail("hi is x truncated to FP32", x);
    if (lo != 0.f && std::signbit(lo) != std::signbit(x)) return fail("lo carries x's sign", x);
    // full precision while the remainder stays in the FP32 normal range
    // (|x| >= 2^-74), else the truncation of hi alone
    const long double err = std::fabs(static_cast<long double>(x) - (static_cast<long double>(hi) + lo));
    const int bits = std::fabs(x) >= std::ldexp(1.0, -74) ? 47 : 23;
    if (err > std::ldexp(std::fabs(static_cast<long double>(x)), -bits)) return fail("split error", x);
    // the pair of a split is 48 bits wide: join rebuilds it exactly
    const double j = join(hi, lo);
    if (static_cast<long double>(j) != static_cast<long double>(hi) + lo) return fail("join of a split", x);
    if (trunc_f32(x) != hi) return fail("trunc_f32", x);
    if (widen(hi) != static_cast<double>(hi)) return fail("widen", x);
    // pairs from (hi, lo) arithmetic: lo of either sign, |lo| <= ulp(hi)
    const float h2 = static_cast<float>(x);
    const float l2 = static_cast<float>((mant(rng) - 1.5) * std::ldexp(std::fabs(static_cast<double>(h2)), -23 - int(n % 40)));
    if (std::fabs(h2) < 1e-30f || std::fabs(l2) < 1e-37f) continue;
    const long double exact = static_cast<long double>(h2) + l2;
    const double j2 = join(h2, l2);
    const long double e2 = std::fabs(static_cast<long double>(j2) - exact);
    if (e2 > std::ldexp(std::fabs(exact), -51)) return fail("join error", x);
    int eh, el;
    std::frexp(h2, &eh);
    std::frexp(l2, &el);
    if (eh - el <= 29 && static_cast<long double>(j2) != exact) return fail("join exact within 29 bits", x);
  }
  // special values
  float hi, lo;
  split(0.0, hi, lo);
  if (hi != 0.f || lo != 0.f || std::signbit(hi)) return fail("+0", 0.0);
  split(-0.0, hi, lo);
  if (hi != 0.f || !std::signbit(hi)) return fail("-0", -0.0);
  split(INFINITY, hi, lo);
  if (!std::isinf(hi) || hi < 0 || lo != 0.f) return fail("inf", INFINITY);
  split(-INFINITY, hi, lo);
  if (!std::isinf(hi) || hi > 0) return fail("-inf", -INFINITY);
  split(NAN, hi, lo);
  if (!std::isnan(hi)) return fail("nan", NAN);
  split(1e-40, hi, lo);
  if (hi != 0.f || lo != 0.f) return fail("below FP32 range", 1e-40);
  split(1e39, hi, lo);
  if (!std::isinf(hi)) return fail("above FP32 range", 1e39);
  split(1.0 + std::ldexp(1.0, -40), hi, lo);
  if (hi != 1.f || lo != std::ldexp(1.0f, -40)) return fail("small remainder", 1.0);
  if (join(0.f, 3.f) != 3.0 || join(2.f, 0.f) != 2.0) return fail("join with a zero part", 0.0);
  if (join(1.f, -std::ldexp(1.0f, -30)) != 1.0 - std::ldexp(1.0, -30)) return fail("join borrow", 1.0);
  if (widen(1e-42f) != 0.0) return fail("widen subnormal", 1e-42);
  std::printf("ok\n");
  return 0;
}
