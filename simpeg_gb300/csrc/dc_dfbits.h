// Conversions between fp64 and double-float (hi + lo fp32 pairs) by integer
// operations.  GB300 issues fp64 arithmetic and the fp64 <-> fp32 conversion
// instructions at 1/64 of the fp32 rate, so the split of the right-hand sides
// and the widening of the solution, once per element of a multi-RHS solve,
// use the IEEE-754 bit layouts instead (integer and fp32 instructions only);
// values outside the range these cover take the fp64 instructions.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define DC_HD __host__ __device__ __forceinline__
#else
#define DC_HD inline
#endif

namespace dc {

DC_HD uint64_t bits64(double v) {
  uint64_t u;
  memcpy(&u, &v, sizeof u);
  return u;
}
DC_HD double from_bits64(uint64_t u) {
  double v;
  memcpy(&v, &u, sizeof v);
  return v;
}
DC_HD uint32_t bits32(float v) {
  uint32_t u;
  memcpy(&u, &v, sizeof u);
  return u;
}
DC_HD float from_bits32(uint32_t u) {
  float v;
  memcpy(&v, &u, sizeof v);
  return v;
}

// v = hi + lo: hi = v truncated to 24 significant bits (the fp32 with v's sign,
// exponent and leading 23 fraction bits), lo = the remaining 29 fraction bits
// rounded to fp32, so hi + lo equals v to 2^-48 relatively and |lo| < ulp(hi).
// Exact zero for a zero v.  Returns false when hi or lo would leave the normal
// fp32 range (|v| >= 2^128 or 0 < |v| < 2^-74, denormals, inf, nan).
DC_HD bool split_df_bits(double v, float &hi, float &lo) {
  const uint64_t u = bits64(v);
  const uint32_t sign = (uint32_t)(u >> 63);
  if ((u << 1) == 0) {  // +-0
    hi = from_bits32(sign << 31);
    lo = hi;
    return true;
  }
  const int e = (int)((u >> 52) & 0x7ff);  // biased fp64 exponent
  if (e < 949 || e > 1150) return false;
  const uint64_t m = u & 0xFFFFFFFFFFFFFull;                                             // 52 fraction bits
  hi = from_bits32((sign << 31) | ((uint32_t)(e - 896) << 23) | (uint32_t)(m >> 29));  // fp32 exponent e - 1023 + 127
  const uint32_t r = (uint32_t)(m & 0x1FFFFFFFu);                                      // v - hi = r * 2^(e - 1075)
  const float l = (float)r * from_bits32((uint32_t)(e - 948) << 23);                    // 2^(e - 1075): a normal fp32
  lo = sign ? -l : l;
  return true;
}

// (double)f for zero and normal f by bit widening; false for denormals, inf, nan.
DC_HD bool widen_bits(float f, double &d) {
  const uint32_t b = bits32(f);
  const uint64_t sign = (uint64_t)(b >> 31) << 63;
  if ((b << 1) == 0) {
    d = from_bits64(sign);
    return true;
  }
  const uint32_t fe = (b >> 23) & 0xff;
  if (fe == 0 || fe == 255) return false;
  d = from_bits64(sign | ((uint64_t)(fe + 896) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29));
  return true;
}

// d = (double)hi + (double)lo rounded to nearest even, as the fp64 addition
// rounds it, by integer operations, for a normalised double-float pair: hi
// normal and lo zero, or lo normal at least 24 binades below hi (exponent gap
// g >= 24, which |lo| <= ulp(hi) / 2 implies).  In units of 2^-52 of hi's
// binade hi is the 53-bit integer m = (hi's significand) << 29 and lo is
// (lo's significand) * 2^(29 - g): an integer for g <= 29, added exactly
// (below 2^53); for g >= 30 its integer part is added and the shifted-out
// bits round the sum.  False for what is left to the fp64 addition: hi zero
// (unless lo is zero too), denormal, inf or nan; lo denormal, inf or nan;
// g < 24; hi a power of two with lo of the opposite sign and g >= 30 (the sum
// falls into the binade below, where the rounding point moves).
DC_HD bool df_sum_bits(float hi, float lo, double &d) {
  const uint32_t bh = bits32(hi), bl = bits32(lo);
  const uint32_t eh = (bh >> 23) & 0xff;
  if ((bh << 1) == 0 && (bl << 1) == 0) {  // +-0 + +-0: -0 only when both are -0
    d = from_bits64((uint64_t)(bh & bl & 0x80000000u) << 32);
    return true;
  }
  if (eh == 0 || eh == 255) return false;
  uint64_t m = (uint64_t)((bh & 0x7FFFFFu) | 0x800000u) << 29;
  uint32_t ed = eh + 896;  // fp64 biased exponent of hi
  if ((bl << 1) != 0) {
    const uint32_t el = (bl >> 23) & 0xff;
    if (el == 0 || el == 255) return false;
    const int g = (int)eh - (int)el;
    if (g < 24) return false;
    const uint64_t ml = (bl & 0x7FFFFFu) | 0x800000u;
    const bool same = (bh >> 31) == (bl >> 31);
    if (g <= 29) {
      const uint64_t t = ml << (29 - g);
      m = same ? m + t : m - t;  // exact: below 2^53, and above 2^51 after a subtraction
      if (m < (1ull << 52)) {    // hi a power of two, lo subtracted: one binade down, exactly
        m <<= 1;
        --ed;
      }
    } else {
      if (!same && m == (1ull << 52)) return false;
      const int sh = g - 29;
      if (sh <= 24) {  // for larger gaps |lo| is below half a unit: the sum rounds to hi
        const uint64_t q = ml >> sh, rem = ml & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (same) {
          m += q;
          if (rem > half || (rem == half && (m & 1))) ++m;
        } else {
          m -= q;
          if (rem) {  // m - q - rem / 2^sh = (m - q - 1) + (2^sh - rem) / 2^sh
            const uint64_t f = (1ull << sh) - rem;
            --m;
            if (f > half || (f == half && (m & 1))) ++m;
          }
        }
      }
    }
  }
  d = from_bits64(((uint64_t)(bh >> 31) << 63) | ((uint64_t)ed << 52) | (m & 0xFFFFFFFFFFFFFull));
  return true;
}

}  // namespace dc
