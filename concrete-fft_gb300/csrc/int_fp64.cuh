// int_fp64.cuh -- IEEE binary64 addition on the integer pipe.
//
// GB300 issues FP64 instructions at 1/64 of its FP32/INT32 rate, and every FFT
// kernel of this library is bound by that FP64 pipe.  dadd_int computes the
// correctly rounded (round-to-nearest-even) double sum with 32-bit integer
// instructions only, so a kernel can route part of its additions through the
// integer pipe while the FP64 pipe works on the rest.  The result is the
// IEEE-754 sum, bit for bit: it is a different instruction sequence for the
// same value, so the transforms stay bit-identical to the reference.
//
// Operands or results outside the normal range (zero, subnormal, inf, nan,
// overflow, gradual underflow) take the native __dadd_rn path.
//
// Method (textbook significand addition with guard bits and a sticky bit):
// order the operands by magnitude, place both 53-bit significands at bits
// 61..9 of a 64-bit word (9 guard bits), shift the smaller one right by the
// exponent difference OR-ing every lost bit into bit 0, add or subtract,
// renormalise the leading one to bit 61, and round to nearest even on bit 9.
// With at least two guard bits above the sticky bit, the OR-ed sticky value
// and the exact value lie strictly on the same side of every rounding
// boundary, so the rounding decision is exact.
#pragma once
#include <cstdint>

namespace cfft {

__device__ __forceinline__ double dadd_int(double x, double y) {
  const uint64_t kAbs = 0x7fffffffffffffffull;
  const uint64_t kMant = 0x000fffffffffffffull;
  const uint64_t kHid = 0x0010000000000000ull;
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const uint64_t uy = (uint64_t)__double_as_longlong(y);
  const uint64_t ax = ux & kAbs, ay = uy & kAbs;
  const bool sw = ax < ay;
  const uint64_t big = sw ? uy : ux;
  const uint64_t abig = sw ? ay : ax;
  const uint64_t asml = sw ? ax : ay;
  const int eb = (int)(abig >> 52);
  const int es = (int)(asml >> 52);
  if (eb == 0x7ff || es == 0) return __dadd_rn(x, y);
  const uint64_t mb = ((abig & kMant) | kHid) << 9;
  const uint64_t ms = ((asml & kMant) | kHid) << 9;
  const int d = eb - es;
  uint64_t msa;
  if (d == 0) msa = ms;
  else if (d >= 63) msa = 1;
  else msa = (ms >> d) | (uint64_t)((ms << (64 - d)) != 0);
  const bool sub = ((ux ^ uy) >> 63) != 0;
  uint64_t m = sub ? mb - msa : mb + msa;
  if (m == 0) return 0.0;  // exact cancellation: +0 under round-to-nearest
  int e = eb;
  const int lz = __clzll((long long)m);
  if (lz == 1) {
    m = (m >> 1) | (m & 1);
    e += 1;
  } else if (lz > 2) {
    m <<= (lz - 2);
    e -= (lz - 2);
  }
  if (e <= 0 || e >= 0x7ff) return __dadd_rn(x, y);
  uint64_t mant = m >> 9;  // 53 bits, hidden bit at 52
  const uint32_t rem = (uint32_t)m & 0x1ffu;
  mant += (rem > 0x100u || (rem == 0x100u && (mant & 1))) ? 1 : 0;
  // the hidden bit adds one to the exponent field; a rounding carry to 2^53
  // adds one more and leaves a zero fraction, as IEEE requires
  return __longlong_as_double((long long)((big & ~kAbs) | ((((uint64_t)(e - 1)) << 52) + mant)));
}

__device__ __forceinline__ double dsub_int(double x, double y) { return dadd_int(x, -y); }

}  // namespace cfft
