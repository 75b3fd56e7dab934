// Exact fixed-point moments for the moving-window kernels.
//
// A finite double is m * 2^(e - 1075) with an integer mantissa m < 2^53 and a biased
// exponent e (e = 1 for subnormals).  Given a scale exponent E (the largest biased
// exponent in a tile), values, squares and cross products become 128-bit integers:
//     x      -> m << (e - E + 40)               LSB 2^(E - 1115)
//     x^2    -> m^2 << (2(e - E) - 13)          LSB 2^(2E - 2137)
//     x * y  -> mx*my << ((ex-Ex)+(ey-Ey) - 13) LSB 2^(Ex + Ey - 2137)
// The largest value occupies bits 40..93, leaving 34 bits of headroom: sums of up to
// 2^34 terms cannot overflow.  Bits more than 2^40 (values) or 2^93 (squares) below
// the tile's largest term are truncated, a relative error below 2^-80 of that term.
// Integer addition is exact and associative, so a window sum accumulated this way does
// not drift with the position in the row, and any tiling gives identical bits.
#pragma once

#include "nbg_common.cuh"

namespace nbg {
namespace fx {

typedef __int128 i128;
typedef unsigned __int128 u128;

constexpr int kValueShift = 40;
constexpr int kSquareShift = -13;

NBG_DEVICE int biased_exponent(double x) {
  const int e = static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(x)) >> 52) & 0x7ff);
  return e ? e : 1;
}
NBG_DEVICE bool is_inf(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull) == 0x7ff0000000000000ull;
}
NBG_DEVICE unsigned long long mantissa(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long m = b & 0x000fffffffffffffull;
  return ((b >> 52) & 0x7ff) ? (m | 0x0010000000000000ull) : m;
}
NBG_DEVICE bool negative(double x) { return __double_as_longlong(x) < 0; }

// (u128)m shifted left by sh (sh may be negative: truncating right shift)
NBG_DEVICE u128 shift_u(u128 m, int sh) {
  if (sh >= 0) return sh >= 128 ? 0 : (m << sh);
  return -sh >= 128 ? 0 : (m >> (-sh));
}

NBG_DEVICE i128 fix_value(double x, int E) {
  const u128 v = shift_u(static_cast<u128>(mantissa(x)), biased_exponent(x) - E + kValueShift);
  return negative(x) ? -static_cast<i128>(v) : static_cast<i128>(v);
}
NBG_DEVICE i128 fix_square(double x, int E) {
  const unsigned long long m = mantissa(x);
  const u128 sq = static_cast<u128>(m) * m;
  return static_cast<i128>(shift_u(sq, 2 * (biased_exponent(x) - E) + kSquareShift));
}
NBG_DEVICE i128 fix_product(double x, double y, int Ex, int Ey) {
  const u128 p = static_cast<u128>(mantissa(x)) * mantissa(y);
  const u128 v = shift_u(p, (biased_exponent(x) - Ex) + (biased_exponent(y) - Ey) + kSquareShift);
  return (negative(x) != negative(y)) ? -static_cast<i128>(v) : static_cast<i128>(v);
}

// LSB exponents of the three kinds of moment
NBG_HOST_DEVICE int lsb_value(int E) { return E - 1075 - kValueShift; }
NBG_HOST_DEVICE int lsb_product(int Ex, int Ey) { return (Ex - 1075) + (Ey - 1075) - kSquareShift; }

// arithmetic right shift by d >= 0
NBG_DEVICE i128 shr(i128 v, int d) {
  if (d <= 0) return v;
  if (d >= 127) return v < 0 ? static_cast<i128>(-1) : static_cast<i128>(0);
  return v >> d;
}

NBG_DEVICE int clz128(u128 a) {
  const unsigned long long hi = static_cast<unsigned long long>(a >> 64);
  const unsigned long long lo = static_cast<unsigned long long>(a);
  return hi ? __clzll(static_cast<long long>(hi)) : (lo ? 64 + __clzll(static_cast<long long>(lo)) : 128);
}

// v * 2^L rounded to the nearest double (ties to even).
NBG_DEVICE double to_double(i128 v, int L) {
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const u128 a = neg ? static_cast<u128>(-v) : static_cast<u128>(v);
  const int lz = clz128(a);
  const u128 n = a << lz;
  unsigned long long t = static_cast<unsigned long long>(n >> 64);
  if (static_cast<unsigned long long>(n) != 0ull) t |= 1ull;  // sticky bit below the round bit
  double d = __ull2double_rn(t);                               // t in [2^63, 2^64): exponent 63 or 64
  const int k = 64 - lz + L;                                    // value = t * 2^k
  const long long bits = __double_as_longlong(d);
  const int e = static_cast<int>((bits >> 52) & 0x7ff) + k;
  if (e >= 1 && e <= 2046) {
    d = __longlong_as_double((bits & ~(0x7ffll << 52)) | (static_cast<long long>(e) << 52));
  } else {
    d = scalbn(d, k);  // overflow to inf or a subnormal result
  }
  return neg ? -d : d;
}

// v * 2^L rounded to the nearest float64 (ties to even), with integer instructions;
// results outside the normal range go through the general conversion.
NBG_DEVICE double to_f64(i128 v, int L) {
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const u128 a = neg ? static_cast<u128>(-v) : static_cast<u128>(v);
  const int lz = clz128(a);
  const u128 nrm = a << lz;  // leading one at bit 127
  unsigned long long mant = static_cast<unsigned long long>(nrm >> 75);  // 53 bits
  const u128 rest = nrm & ((static_cast<u128>(1) << 75) - 1);
  const u128 half = static_cast<u128>(1) << 74;
  int e = 127 - lz + L + 1023;  // biased exponent of the leading one
  if (rest > half || (rest == half && (mant & 1))) {
    if (++mant == (1ull << 53)) {
      mant >>= 1;
      ++e;
    }
  }
  if (e < 1 || e > 2046) return to_double(v, L);
  const unsigned long long bits = (static_cast<unsigned long long>(neg) << 63) |
                                  (static_cast<unsigned long long>(e) << 52) | (mant & 0x000fffffffffffffull);
  return __longlong_as_double(static_cast<long long>(bits));
}

}  // namespace fx
}  // namespace nbg
