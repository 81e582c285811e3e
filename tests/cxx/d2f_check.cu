// Host check of the integer-pipe double-to-float conversions (d2f_rn,
// d2f_split in psph_common.cuh) against the compiler's own conversion: the
// same bits for hi = (float)x and lo = (float)(x - (double)hi), over random
// bit patterns of every exponent, exact ties, carries into the next binade and
// the range edges. Prints the mismatch count and exits non-zero on any.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "psph_common.cuh"

static unsigned fb(float f) {
  unsigned u;
  memcpy(&u, &f, sizeof u);
  return u;
}
static double from_bits(unsigned long long b) {
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
}

static long long bad = 0, checked = 0;

static void check(double x) {
  float lo = 0.f;
  const float hi = psph::d2f_split(x, &lo);
  const float rh = (float)x;
  const float rl = (float)(x - (double)rh);
  ++checked;
  const bool nan = std::isnan(rh);
  const bool ok = nan ? (std::isnan(hi)) : (fb(hi) == fb(rh) && (std::isnan(rl) ? std::isnan(lo) : fb(lo) == fb(rl)));
  if (!ok || (!nan && fb(psph::d2f_rn(x)) != fb(rh))) {
    if (bad < 10)
      printf("mismatch x=%.17g hi=%08x ref=%08x lo=%08x ref=%08x\n", x, fb(hi), fb(rh), fb(lo), fb(rl));
    ++bad;
  }
}

int main() {
  std::mt19937_64 rng(12345);
  for (int k = 0; k < 4000000; ++k) check(from_bits(rng()));  // every exponent, both signs
  for (int k = 0; k < 4000000; ++k) {  // FP32's range, where the integer path runs
    const unsigned long long e = 890 + rng() % 270;
    const unsigned long long m = rng() & 0xfffffffffffffull;
    check(from_bits((rng() & 1ull) << 63 | e << 52 | m));
  }
  for (unsigned long long e = 890; e < 1160; ++e)  // ties, carries, the dropped bits' extremes
    for (unsigned long long keep : {0ull, 1ull, 2ull, 0x3ffffeull, 0x7fffffull})
      for (unsigned long long rem : {0ull, 1ull, 0xfffffffull, 0x10000000ull, 0x10000001ull, 0x1fffffffull})
        for (unsigned long long s : {0ull, 1ull})
          check(from_bits(s << 63 | e << 52 | keep << 29 | rem));
  for (double x : {0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 1e300, std::numeric_limits<double>::infinity(),
                   -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                   (double)std::numeric_limits<float>::max(), (double)std::numeric_limits<float>::min(),
                   (double)std::numeric_limits<float>::denorm_min(), 3.4028235677973366e38, 5e-324})
    check(x);
  printf("checked %lld mismatches %lld\n", checked, bad);
  return bad ? 1 : 0;
}
