// Digit arithmetic of the emulated-FP64 GEMM (Ozaki splitting), shared by the
// large-product engine (ozaki.cu) and the grouped small-problem kernel
// (batched.cu):
//   * the scale exponent of a row (column) from the bits of its largest |x|:
//     every |x| on the row is below 2^e;
//   * the truncated fixed-point magnitude trunc(|x| 2^(t - e)) (< 2^t, t <= 64)
//     taken straight from the IEEE bits; with t = 8S its base-256 digits (most
//     significant first) are the S slices of x;
//   * one element of C from an exact integer (a level sum
//     acc = sum_L P_L 2^(8(S+1-L)), or the CRT value of the modular scheme),
//     rounded once to FP64 and scaled by alpha and a power of two.
// Integer work only where it can be: FP64 is the scarcest unit on this part.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

namespace gb {
namespace ozd {

constexpr int DIGIT_BITS = 8;  // bits of one slice digit, |digit| <= 255
constexpr unsigned long long DIGIT_MASK = (1ull << DIGIT_BITS) - 1;
constexpr int NONFINITE = -100000;  // exponent marker of a row/column with Inf/NaN

// e with |x| < 2^e for every x of a row whose largest |x| has the bit
// pattern `b` (0 for an all-zero row, NONFINITE when it holds Inf/NaN).
__device__ __forceinline__ int exponent_of_max(unsigned long long b) {
  int e = 0;
  const int E = (int)((b >> 52) & 0x7ff);
  if (E == 0x7ff) {
    e = NONFINITE;
  } else if (E > 0) {
    e = E - 1022;  // max = 1.f * 2^(E-1023) < 2^(E-1022)
  } else if (b != 0) {
    frexp(__longlong_as_double((long long)b), &e);  // subnormal maximum
  }
  return e;
}

// trunc(|x| 2^(t - e)) (truncation toward zero, < 2^t for |x| < 2^e, t <= 64)
// and the sign of x; 0 for a row marked NONFINITE.
__device__ __forceinline__ unsigned long long fixed_magnitude(double x, int e, int t, bool &neg) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  neg = (bits >> 63) != 0;
  const int E = (int)((bits >> 52) & 0x7ff);
  unsigned long long M = bits & 0xFFFFFFFFFFFFFull;
  int sh;  // |x| = M * 2^(sh0) with sh0 = E - 1075 (normal) or -1074 (subnormal)
  if (E == 0) {
    sh = -1074;
  } else {
    M |= 1ull << 52;
    sh = E - 1075;
  }
  sh += t - e;
  if (e == NONFINITE || M == 0) return 0;
  if (sh >= 0) return M << sh;        // |x| < 2^e keeps the result below 2^t
  if (sh > -64) return M >> (-sh);    // truncation toward zero
  return 0;
}

// The S-digit fixed-point value trunc(|x| 2^(8S - e)) whose base-256 digits
// are the slices of x.
__device__ __forceinline__ unsigned long long digit_magnitude(double x, int e, int S, bool &neg) {
  return fixed_magnitude(x, e, DIGIT_BITS * S, neg);
}

// y * alpha * 2^x when alpha * 2^x is not a normal number (or alpha is
// subnormal, zero, Inf or NaN).  The product can still be a normal number
// (y is up to 2^64), so y is scaled by alpha's significand first and by the
// whole power of two once: a subnormal or underflowed alpha * 2^x would lose
// it.  Rarely taken, so kept out of line, away from the callers' registers.
static __device__ __noinline__ double scale_out_of_range(double y, double alpha, int x) {
  int e_sig;
  const double m_alpha = frexp(alpha, &e_sig);
  return ldexp(y * m_alpha, x + e_sig);
}

// alpha * 2^x0 * acc, acc rounded once to FP64 (sticky bit).
__device__ __forceinline__ double scaled_value(__int128 acc, int x0, double alpha) {
  if (acc == 0) return 0.0;
  const bool neg = acc < 0;
  unsigned __int128 u = neg ? (unsigned __int128)(-acc) : (unsigned __int128)acc;
  const unsigned long long hi = (unsigned long long)(u >> 64);
  const int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)(unsigned long long)u);
  const int sh = msb > 63 ? msb - 63 : 0;
  unsigned long long top = (unsigned long long)(u >> sh);
  if (sh && (u & (((unsigned __int128)1 << sh) - 1)) != 0) top |= 1ull;  // sticky bit
  const double t = __ull2double_rn(top);
  const int x = sh + x0;
  const long long ab = __double_as_longlong(alpha);
  const int e_alpha = (int)((ab >> 52) & 0x7ff);
  if (e_alpha > 0 && e_alpha < 0x7ff && e_alpha + x > 0 && e_alpha + x < 0x7ff)
    return (neg ? -t : t) * __longlong_as_double(ab + ((long long)x << 52));
  return scale_out_of_range(neg ? -t : t, alpha, x);
}

// Leading zeros and bit casts on both sides, so the rounding below also
// compiles as host code (tested against exact integer rounding on the CPU).
__host__ __device__ __forceinline__ int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}
__host__ __device__ __forceinline__ double bits_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// v * 2^x0 for the two's-complement 128-bit integer v = hi:lo, rounded to
// nearest (ties to even) with integer operations only, when the result is a
// normal number (ok = true; FP64 arithmetic is the scarcest unit on this
// part).  The magnitude is normalised to its leading 64 bits; the 11 bits
// below the 53-bit significand and a sticky bit for everything under them
// decide the rounding.
__host__ __device__ __forceinline__ double i128_scaled(unsigned long long hi, unsigned long long lo,
                                                       int x0, bool &ok) {
  ok = true;
  const bool neg = (long long)hi < 0;
  if (neg) {  // |v|
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
  }
  if ((hi | lo) == 0) return 0.0;
  int msb;
  unsigned long long top;
  bool sticky;
  if (hi != 0) {
    const int lz = clz64(hi);
    msb = 127 - lz;
    top = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    sticky = (lz ? lo << lz : lo) != 0;
  } else {
    const int lz = clz64(lo);
    msb = 63 - lz;
    top = lo << lz;
    sticky = false;
  }
  unsigned long long mant = top >> 11;  // 53 bits, the leading one at bit 52
  const unsigned rem = (unsigned)(top & 0x7FFu), half = 0x400u;
  if (rem > half || (rem == half && (sticky || (mant & 1ull)))) {
    if (++mant >> 53) {  // rounded up to the next power of two
      mant >>= 1;
      ++msb;
    }
  }
  const int E = msb + x0 + 1023;  // biased exponent of mant * 2^(msb - 52 + x0)
  if (E <= 0 || E >= 0x7ff) {
    ok = false;
    return 0.0;
  }
  return bits_double(((unsigned long long)neg << 63) | ((unsigned long long)E << 52) |
                     (mant & 0xFFFFFFFFFFFFFull));
}

// alpha * 2^(ei + fj - 8(S+1)) * acc: one element of C from its level sum.
__device__ __forceinline__ double level_value(__int128 acc, int S, int ei, int fj, double alpha) {
  return scaled_value(acc, ei + fj - DIGIT_BITS * (S + 1), alpha);
}

}  // namespace ozd
}  // namespace gb
