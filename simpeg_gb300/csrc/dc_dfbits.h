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

}  // namespace dc
