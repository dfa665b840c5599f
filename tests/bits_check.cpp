// Host check of mantaray_gb300/csrc/bits.h: the integer-pipe conversions
// against the compiler's IEEE conversions, on edge cases and pseudo-random
// bit patterns.  Prints the number of mismatches (0 expected).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>

#include "../mantaray_gb300/csrc/bits.h"

static uint64_t state = 0x12345678abcdefull;
static uint64_t next() {  // SplitMix64
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static bool same_f(float a, float b) {
  uint32_t x, y;
  memcpy(&x, &a, 4);
  memcpy(&y, &b, 4);
  return x == y || (std::isnan(a) && std::isnan(b));
}
static bool same_d(double a, double b) {
  uint64_t x, y;
  memcpy(&x, &a, 8);
  memcpy(&y, &b, 8);
  return x == y || (std::isnan(a) && std::isnan(b));
}

int main() {
  long bad = 0, n = 0;
  auto check_d = [&](double d) {
    ++n;
    if (!same_f(mr::d2f(d), static_cast<float>(d))) {
      if (bad < 5) printf("d2f mismatch %a\n", d);
      ++bad;
    }
    if (mr::nan_bits(d) != std::isnan(d)) ++bad;
  };
  auto check_f = [&](float f) {
    ++n;
    if (!same_d(mr::f2d(f), static_cast<double>(f))) {
      if (bad < 5) printf("f2d mismatch %a\n", static_cast<double>(f));
      ++bad;
    }
  };
  const double specials[] = {0.0, -0.0, 1.0, -1.0, 0.1, 1e-40, -1e-45, 1e-38, 1.1754943508222875e-38,
                             1.1754942106924411e-38, 3.4028234663852886e38, 3.4028235677973366e38,
                             3.4028236e38, 1e39, -1e300, 1e-300, INFINITY, -INFINITY, NAN,
                             std::numeric_limits<double>::denorm_min(), 5e4, 123456.789};
  for (double d : specials) { check_d(d); check_d(std::nextafter(d, 1e308)); check_d(std::nextafter(d, -1e308)); }
  for (int i = 0; i < 3000000; ++i) {
    uint64_t b = next();
    double d;
    memcpy(&d, &b, 8);
    check_d(d);
    // exponents near the float range, and exact halfway cases (29 dropped bits = 2^28)
    const uint64_t e = 860 + (next() % 320);
    uint64_t c = (b & 0x800fffffffffffffull) | (e << 52);
    memcpy(&d, &c, 8);
    check_d(d);
    c = (c & ~0x1fffffffull) | 0x10000000ull;
    memcpy(&d, &c, 8);
    check_d(d);
    uint32_t u = static_cast<uint32_t>(next());
    float f;
    memcpy(&f, &u, 4);
    check_f(f);
  }
  const float fspecials[] = {0.0f, -0.0f, 1e-45f, -1e-40f, 1.17549435e-38f, 3.40282347e38f,
                             INFINITY, -INFINITY, NAN};
  for (float f : fspecials) check_f(f);
  printf("%ld %ld\n", bad, n);
  return bad != 0;
}
