// Host check of the double-float bit routines of simpeg_gb300/csrc/dc_dfbits.h
// (compiled and run by tests/test_host.py): split_df_bits gives hi = v
// truncated to 24 significant bits, |lo| < ulp(hi) and hi + lo = v to 2^-48;
// widen_bits equals the fp32 -> fp64 conversion bit for bit; df_sum_bits
// equals the fp64 addition of the widened pair bit for bit (random pairs over
// every exponent gap, exact ties at every shift, power-of-two hi, zeros).
// Exit status 0 on success.
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
  // df_sum_bits against the fp64 addition
  long sbad = 0, scov = 0, snorm = 0, snorm_cov = 0;
  std::mt19937_64 rs(11);
  auto sum_check = [&](float hi, float lo) {
    double v;
    const bool normalised = std::isnormal(hi) && (lo == 0.0f || (std::isnormal(lo) && std::ilogb(hi) - std::ilogb(lo) >= 24));
    const bool pow2_minus = std::isnormal(lo) && (bits32(hi) & 0x7FFFFFu) == 0 && std::signbit(hi) != std::signbit(lo) &&
                            std::ilogb(hi) - std::ilogb(lo) >= 30;
    if (normalised && !pow2_minus) ++snorm;
    if (!df_sum_bits(hi, lo, v)) return;
    ++scov;
    if (normalised && !pow2_minus) ++snorm_cov;
    if (bits64(v) != bits64((double)hi + (double)lo)) ++sbad;
  };
  auto mk = [](uint32_t sign, int e, uint32_t frac) { return from_bits32((sign << 31) | ((uint32_t)e << 23) | (frac & 0x7FFFFFu)); };
  for (long i = 0; i < 4000000; ++i) {
    const uint64_t u = rs();
    const int eh = 1 + (int)(u % 254);
    const float hi = mk((uint32_t)(u >> 8) & 1, eh, (i % 7 == 0) ? 0u : (uint32_t)(u >> 20));
    const int g = (int)((u >> 44) % 64);
    float lo = 0.0f;
    if ((u >> 50) % 10 != 0 && eh - g >= 1) {
      uint32_t frac = (uint32_t)(rs());
      const int sh = g - 29;
      if (sh >= 1 && sh <= 24 && (u >> 54) % 3 == 0) {  // an exact tie at this shift
        const uint32_t ml = ((frac | 0x800000u) & ~((1u << sh) - 1)) | (1u << (sh - 1));
        frac = ml & 0x7FFFFFu;
      }
      lo = mk((uint32_t)(u >> 60) & 1, eh - g, frac);
    }
    sum_check(hi, lo);
  }
  for (float hi : {1.0f, -1.0f, 2.0f, 3.4e38f, 1.2e-38f})
    for (int g = 24; g < 60; ++g)
      for (float sgn : {1.0f, -1.0f}) {
        const int el = std::ilogb(hi) - g;
        if (el < -126) continue;
        sum_check(hi, sgn * std::ldexp(1.0f, el));
        sum_check(hi, sgn * std::ldexp(1.5f, el));
        sum_check(hi, sgn * std::nextafter(std::ldexp(2.0f, el), 0.0f));
      }
  for (float a : {0.0f, -0.0f})
    for (float b : {0.0f, -0.0f}) sum_check(a, b);
  std::printf("split covered %ld bad %ld outside-range rejected %d; widen covered %ld bad %ld; "
              "sum covered %ld (normalised pairs %ld of %ld) bad %ld\n",
              covered, bad, (int)outside, wcov, wbad, scov, snorm_cov, snorm, sbad);
  return (bad || wbad || !outside || covered < 1000000 || wcov < 1000000 || sbad || scov < 1000000 ||
          snorm_cov != snorm)
             ? 1
             : 0;
}
