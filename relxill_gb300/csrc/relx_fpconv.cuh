// relx_fpconv.cuh -- double <-> float conversions and comparisons of positive doubles with integer
// operations.  Device code includes it through relx_device.cuh; tests/test_fpconv.py compiles it for
// the host (with the bit-cast intrinsics defined there) and checks it against the compiler's
// conversions bit for bit.
#pragma once

#ifndef RELX_FPCONV_FN
#define RELX_FPCONV_FN __device__ __forceinline__
#endif

namespace relx {

// ---- FP64 values handled on the integer pipes ------------------------------
// On this part the FP64 pipe issues 2 lanes per clock per SM, and the double <-> float conversion
// instructions run on it as well.  Conversions are done here with integer operations, and
// comparisons of positive doubles as comparisons of their bit patterns (which order like the
// values for non-negative finite doubles).
// (float) d, rounded to nearest even, every case on the integer pipes (a conversion instruction
// on the rare path would be if-converted into every call)
RELX_FPCONV_FN float d2f(double d) {
  const unsigned long long b = (unsigned long long) __double_as_longlong(d);
  const unsigned int sgn = (unsigned int) (b >> 32) & 0x80000000u;
  const int eb = (int) (b >> 52) & 0x7ff;
  const unsigned long long frac = b & 0xfffffffffffffull;
  const int E = eb - 1023 + 127;  // biased float exponent
  unsigned int f;
  if (eb == 0x7ff) {
    f = frac ? 0x7fc00000u : 0x7f800000u;  // NaN, infinity
  } else if (E >= 255) {
    f = 0x7f800000u;  // overflow
  } else if (E > 0) {
    const unsigned int m = (unsigned int) (frac >> 29);           // leading 23 fraction bits
    const unsigned int rem = (unsigned int) frac & 0x1fffffffu;   // the 29 bits dropped
    f = ((unsigned int) E << 23) | m;
    f += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;  // a carry moves the exponent
  } else if (eb == 0 || E < -24) {
    f = 0u;  // below half the smallest float denormal
  } else {  // float denormal: the 53-bit significand shifted by 30 - E, rounded
    const unsigned long long m = (1ull << 52) | frac;
    const int sh = 30 - E;  // 30 .. 54
    const unsigned long long q = m >> sh, rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    f = (unsigned int) q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u);
  }
  return __uint_as_float(f | sgn);
}
// (double) f, exact, every case on the integer pipes
RELX_FPCONV_FN double f2d(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xffu, frac = u & 0x7fffffu;
  unsigned long long b = (unsigned long long) (u & 0x80000000u) << 32;
  if (e == 255u) {
    b |= (0x7ffull << 52) | ((unsigned long long) frac << 29);  // infinity, NaN
  } else if (e != 0u) {
    b |= ((unsigned long long) (e + 896u) << 52) | ((unsigned long long) frac << 29);
  } else if (frac != 0u) {  // float denormal: frac * 2^-149 with its leading bit at p
    const int p = 31 - __clz(frac);
    b |= ((unsigned long long) (p - 149 + 1023) << 52) | (((unsigned long long) frac << (52 - p)) & 0xfffffffffffffull);
  }
  return __longlong_as_double((long long) b);
}
// a > b and a >= b where b > 0 and a is not NaN (a may be negative)
RELX_FPCONV_FN bool dgt(double a, double b) { return __double_as_longlong(a) > __double_as_longlong(b); }
RELX_FPCONV_FN bool dge(double a, double b) { return __double_as_longlong(a) >= __double_as_longlong(b); }
}  // namespace relx
