// Host check of the double-float bit routines of simpeg_gb300/csrc/dc_dfbits.h
// (compiled and run by tests/test_host.py): split_df_bits gives hi = v
// truncated to 24 significant bits, |lo| < ulp(hi) and hi + lo = v to 2^-48;
// widen_bits equals the fp32 -> fp64 conversion bit for bit.  Exit status 0 on
// success.
#include "../simpeg_gb300/csrc/dc_dfbits.h"

#include <cmath>
#include <cstdio>
#include <random>

using namespace dc;

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  long bad = 0, covered = 0;
  auto check = [&](double v) {
    float h, l;
    if (!split_df_bits(v, h, l)) return;
    ++covered;
    if (v == 0.0) {
      if (h != 0.0f || l != 0.0f || std::signbit(h) != std::signbit(v)) ++bad;
      return;
    }
    const double trunc = from_bits64(bits64(v) & ~0x1FFFFFFFull);
    if ((double)h != trunc) ++bad;
    if (std::fabs(((double)h + (double)l) - v) > std::ldexp(std::fabs(v), -48)) ++bad;
    if (std::fabs(l) >= std::fabs((double)std::nextafter(h, INFINITY) - (double)h)) ++bad;
  };
  for (int i = 0; i < 2000000; ++i) {
    double v = std::ldexp(1.0 + U(rng), (int)std::floor(-90.0 + 240.0 * U(rng)));
    check(U(rng) < 0.5 ? -v : v);
  }
  for (double v : {0.0, -0.0, 1.0, -1.0 / 3.0, std::ldexp(1.0, -74), std::ldexp(1.9999, 127)}) check(v);
  float h, l;
  const bool outside = !split_df_bits(std::ldexp(1.0, -75), h, l) && !split_df_bits(std::ldexp(1.0, 128), h, l) &&
                       !split_df_bits(INFINITY, h, l) && !split_df_bits(NAN, h, l) && !split_df_bits(5e-324, h, l);
  long wbad = 0, wcov = 0;
  std::mt19937 r32(9);
  for (long i = 0; i < 5000000; ++i) {
    const float f = from_bits32((uint32_t)r32());
    double d;
    if (!widen_bits(f, d)) continue;
    ++wcov;
    if (bits64(d) != bits64((double)f)) ++wbad;
  }
  for (float f : {0.0f, -0.0f, 1.0f, -2.5f, 1.2e-38f, 3.4e38f}) {
    double d;
    if (!widen_bits(f, d) || bits64(d) != bits64((double)f)) ++wbad;
  }
  double d;
  if (widen_bits(1e-40f, d) || widen_bits(INFINITY, d) || widen_bits(NAN, d)) ++wbad;  // denormal, inf, nan
  std::printf("split covered %ld bad %ld outside-range rejected %d; widen covered %ld bad %ld\n", covered, bad,
              (int)outside, wcov, wbad);
  return (bad || wbad || !outside || covered < 1000000 || wcov < 1000000) ? 1 : 0;
}
