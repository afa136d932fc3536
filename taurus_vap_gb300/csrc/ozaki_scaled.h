// Exact conversion of the two integer accumulators of the emulated
// products to a double: (h 2^28 + l) 2^s rounded to nearest (ties to even),
// negated when neg, from the 128-bit integer with integer instructions only.
// It equals fma(double(h), 2^28, double(l)) * (+-2^s) -- both round once
// when |h|, |l| < 2^53 -- at a fraction of the cost on a part whose FP64
// pipe retires two operations per SM and cycle.  Returns false when the
// result would be subnormal or infinite (the caller then takes the
// floating-point formula, which rounds the same way there).  Plain C++ as
// well, so that host code can check it.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define TVAP_HD __host__ __device__ __forceinline__
#else
#define TVAP_HD inline
#endif

namespace tvap {
namespace oztc {

TVAP_HD int clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(x));
#else
  return __builtin_clzll(x);
#endif
}

TVAP_HD double bits_to_double(unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(b));
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

TVAP_HD bool scaled(long long h, long long l, int s, bool neg, double& out) {
  unsigned long long lo = static_cast<unsigned long long>(h) << 28;
  long long hi = h >> 36;
  const unsigned long long sum = lo + static_cast<unsigned long long>(l);
  hi += (l >> 63) + (sum < lo ? 1 : 0);
  lo = sum;
  bool sign = neg;
  if (hi < 0) {
    sign = !sign;
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  const unsigned long long uh = static_cast<unsigned long long>(hi);
  if ((uh | lo) == 0) {
    out = neg ? -0.0 : 0.0;
    return true;
  }
  int msb = uh ? 127 - clz64(uh) : 63 - clz64(lo);
  unsigned long long mant;
  if (msb <= 52) {
    mant = lo << (52 - msb);
  } else {
    const int sh = msb - 52;
    if (sh > 63) return false;
    unsigned long long top = (lo >> sh) | (uh << (64 - sh));
    const unsigned long long rem = lo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (top & 1ull))) {
      ++top;
      if (top >> 53) {
        top >>= 1;
        ++msb;
      }
    }
    mant = top;
  }
  const int e = msb + s + 1023;
  if (e <= 0 || e >= 2047) return false;
  out = bits_to_double((sign ? 1ull << 63 : 0ull) | (static_cast<unsigned long long>(e) << 52) |
                       (mant & ((1ull << 52) - 1ull)));
  return true;
}

}  // namespace oztc
}  // namespace tvap
