// Floating-point conversions on bit patterns, usable from host and device
// code (the host side lets the CPU tests check them bit for bit against the
// host's IEEE conversion).
#pragma once

namespace gb {

// IEEE-754 binary64 -> binary32 conversion, round to nearest even, on the
// bit pattern with integer operations only (GB300's FP64 units are few; a
// pass that converts every element of a matrix is otherwise bound by them).
// Overflow gives infinity, results below the binary32 range round through
// the subnormals to zero, NaN gives the quiet NaN 0x7FFFFFFF.
#if defined(__CUDACC__)
#define GB_HD __host__ __device__
#else
#define GB_HD
#endif
GB_HD inline unsigned f64_bits_to_f32_bits_rn(unsigned long long b) {
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long ab = b & 0x7FFFFFFFFFFFFFFFull;
  if (ab >= 0x7FF0000000000000ull) return ab == 0x7FF0000000000000ull ? (sign | 0x7F800000u) : 0x7FFFFFFFu;
  const int be = (int)(ab >> 52);                       // biased exponent, 0 for zero / subnormal
  if (be == 0) return sign;                             // |x| < 2^-1022 rounds to zero
  const int e = be - 1023;
  const unsigned long long m = (ab & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;   // 53-bit significand
  if (e >= -126) {
    // normal result: keep 24 bits
    unsigned long long r = m >> 29;
    const unsigned long long rem = m & 0x1FFFFFFFull;
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (r & 1ull))) ++r;
    int ee = e;
    if (r == (1ull << 24)) { r >>= 1; ++ee; }
    if (ee > 127) return sign | 0x7F800000u;
    return sign | ((unsigned)(ee + 127) << 23) | ((unsigned)r & 0x7FFFFFu);
  }
  // subnormal result (or zero): keep 24 - (-126 - e) bits
  const int shift = 29 + (-126 - e);
  if (shift > 54) return sign;                          // below half the smallest subnormal
  const unsigned long long r0 = m >> shift;
  const unsigned long long rem = m & ((1ull << shift) - 1ull);
  const unsigned long long half = 1ull << (shift - 1);
  const unsigned long long r = (rem > half || (rem == half && (r0 & 1ull))) ? r0 + 1ull : r0;
  return sign | (unsigned)r;                            // r == 2^23 is the smallest normal
}

}  // namespace gb
