// Host check of the integer conversion of the emulated products' accumulators
// (ozaki_scaled.h): bit-identical to fma(double(h), 2^28, double(l)) * (+-2^s)
// on random, tie, carry and range-end cases; outside the normal range it
// must decline.  Built and run by test_ozaki_scaled.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "ozaki_scaled.h"
int main() {
  std::mt19937_64 rng(7);
  long long bad = 0, fell = 0, n = 0;
  auto bitsof = [](double d) { unsigned long long b; std::memcpy(&b, &d, 8); return b; };
  auto check = [&](long long h, long long l, int s, bool neg) {
    ++n;
    const double ref = std::fma(double(h), 0x1p28, double(l)) * (neg ? -std::ldexp(1.0, s) : std::ldexp(1.0, s));
    double got;
    if (tvap::oztc::scaled(h, l, s, neg, got)) {
      if (bitsof(got) != bitsof(ref)) {
        if (++bad < 10) printf("mismatch h=%lld l=%lld s=%d neg=%d got=%a ref=%a\n", h, l, s, neg, got, ref);
      }
    } else {
      ++fell;
      const double a = std::fabs(ref);
      if (!(a == 0.0 || a < 0x1p-1022 || std::isinf(a) || a >= 0x1p1023)) {
        if (++bad < 10) printf("fallback outside range h=%lld l=%lld s=%d ref=%a\n", h, l, s, ref);
      }
    }
  };
  for (int it = 0; it < 3000000; ++it) {
    const int bh = int(rng() % 50), bl = int(rng() % 50);
    long long h = (long long)(rng() >> (64 - bh)) * ((rng() & 1) ? -1 : 1);
    long long l = (long long)(rng() >> (64 - bl)) * ((rng() & 1) ? -1 : 1);
    if (bh == 0) h = 0;
    if (bl == 0) l = 0;
    const int s = int(rng() % 400) - 200;
    check(h, l, s, rng() & 1);
  }
  // ties and carries: l chosen so that the dropped bits are exactly half
  for (int it = 0; it < 200000; ++it) {
    long long h = (long long)(rng() >> 16) | (1LL << 47);
    const int sh = int(rng() % 24) + 1;
    long long l = ((long long)1 << (sh - 1)) + ((rng() & 1) ? ((long long)1 << sh) : 0);
    if (rng() & 1) h = -h;
    check(h, l, int(rng() % 100) - 50, rng() & 1);
    check(h, -l, int(rng() % 100) - 50, rng() & 1);
    check((1LL << 25) - 1, (1LL << 28) - 1, 0, false);
  }
  // range ends
  for (int s = -1140; s <= -1000; ++s) check(12345, 678, s, false);
  for (int s = 930; s <= 1023; ++s) check(1LL << 47, 99, s, true);
  check(0, 0, 5, false);
  check(0, 0, 5, true);
  printf("cases %lld fallback %lld bad %lld\n", n, fell, bad);
  return bad != 0;
}
