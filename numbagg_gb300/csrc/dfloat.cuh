// Double-float arithmetic on the FP32 pipes, for the FP32-compensated ("fp32c") forms.
//
// A df is hi + lo with |lo| <= ulp(hi) / 2: about 48 significant bits from two
// float32 words, computed with the error-free transformations
//   TwoSum     (Knuth, The Art of Computer Programming vol. 2, 4.2.2),
//   FastTwoSum (Dekker, Numer. Math. 18, 1971),
//   TwoProduct with a fused multiply-add (Ogita, Rump and Oishi, SIAM J. Sci. Comput.
//   26(6), 2005),
// and the double-float add, multiply, divide and square root of Hida, Li and Bailey's
// QD library paper (ARITH-15, 2001; square root by Karp's method).  Every operation is
// an explicitly rounded float32 intrinsic, so the compiler cannot contract it.
//
// An sdf ("scaled df") keeps the exponent apart: value = m * 2^e with m a df in
// [1, 2) (or zero), so results never leave float32's exponent range; finalisations
// built from exact integer sums go integer -> sdf -> float64 without touching the
// FP64 pipe, which on this GPU accepts one warp instruction per 16 cycles.
#pragma once

#include "fixed128.cuh"

namespace nbg {
namespace dfl {

struct df {
  float hi, lo;
};

NBG_DEVICE df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}
NBG_DEVICE df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
NBG_DEVICE df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df{p, __fmaf_rn(a, b, -p)};
}
NBG_DEVICE df df_add(df x, df y) {  // the accurate ("IEEE") double-float sum
  df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  float e = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, e);
  e = __fadd_rn(t.lo, s.lo);
  return fast_two_sum(s.hi, e);
}
NBG_DEVICE df df_neg(df x) { return df{-x.hi, -x.lo}; }
// the cheaper ("sloppy") sum: error about 2^-44 of |x| + |y| (the accurate one above is
// within a few ulps of the result even when x + y cancels)
NBG_DEVICE df df_add_fast(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, x.lo), y.lo));
}
NBG_DEVICE df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
NBG_DEVICE df df_mul(df x, df y) {
  const df p = two_prod(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  return fast_two_sum(p.hi, e);
}
NBG_DEVICE df df_mul_f(df x, float y) {
  const df p = two_prod(x.hi, y);
  return fast_two_sum(p.hi, __fmaf_rn(x.lo, y, p.lo));
}
NBG_DEVICE df df_div(df x, df y) {  // three-quotient long division
  const float q1 = __fdiv_rn(x.hi, y.hi);
  df r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fdiv_rn(r.hi, y.hi);
  r = df_sub(r, df_mul_f(y, q2));
  const float q3 = __fdiv_rn(r.hi, y.hi);
  return df_add(fast_two_sum(q1, q2), df{q3, 0.0f});
}
NBG_DEVICE df df_sqrt(df a) {  // a > 0; Karp: sqrt(a) ~ a*x + (a - (a*x)^2) * x / 2, x = 1/sqrt(a)
  const float x = __frsqrt_rn(a.hi);
  const float ax = __fmul_rn(a.hi, x);
  const df d = df_sub(a, two_prod(ax, ax));
  return fast_two_sum(ax, __fmul_rn(d.hi, __fmul_rn(x, 0.5f)));
}

// ---- scaled double-float ------------------------------------------------------------
struct sdf {
  df m;       // in [1, 2) or zero, sign in m
  int e;      // value = m * 2^e
  bool zero;
};

NBG_DEVICE float pow2f(int k) {  // 2^k for -126 <= k <= 127
  return __int_as_float((k + 127) << 23);
}

// renormalise m into [1, 2) (m nonzero and finite)
NBG_DEVICE sdf sdf_norm(df m, int e) {
  const int k = ((__float_as_int(m.hi) >> 23) & 0xff) - 127;  // exponent of hi
  const float s = pow2f(-k);
  sdf r;
  r.m = df{__fmul_rn(m.hi, s), __fmul_rn(m.lo, s)};
  r.e = e + k;
  r.zero = false;
  return r;
}

// |u| (a nonzero 128-bit magnitude) * 2^L as an sdf, sign given
NBG_DEVICE sdf sdf_from_u128(fx::u128 a, int L, bool neg) {
  sdf r;
  if (a == 0) {
    r.m = df{0.0f, 0.0f};
    r.e = 0;
    r.zero = true;
    return r;
  }
  const int lz = fx::clz128(a);
  const fx::u128 n = a << lz;  // leading one at bit 127
  // hi: bits 127..104 (24 bits), lo: the next 24 bits, both truncated (48-bit value)
  const unsigned hm = static_cast<unsigned>(n >> 104);
  const unsigned lm = static_cast<unsigned>(n >> 80) & 0xffffffu;
  const float hi = __uint2float_rn(hm) * pow2f(-23);            // in [1, 2)
  const float lo = __uint2float_rn(lm) * pow2f(-47);            // exact: 24 bits
  df m = fast_two_sum(hi, lo);  // may round up to exactly 2
  if (neg) m = df_neg(m);
  return sdf_norm(m, (127 - lz) + L);
}

NBG_DEVICE sdf sdf_div(const sdf& x, const sdf& y) {  // y nonzero
  if (x.zero) return x;
  return sdf_norm(df_div(x.m, y.m), x.e - y.e);
}
NBG_DEVICE sdf sdf_mul(const sdf& x, const sdf& y) {
  if (x.zero) return x;
  if (y.zero) return y;
  return sdf_norm(df_mul(x.m, y.m), x.e + y.e);
}
NBG_DEVICE sdf sdf_sqrt(const sdf& x) {  // x >= 0
  if (x.zero) return x;
  df m = x.m;
  int e = x.e;
  if (e & 1) {  // make the exponent even: m in [2, 4)
    m = df{__fmul_rn(m.hi, 2.0f), __fmul_rn(m.lo, 2.0f)};
    e -= 1;
  }
  return sdf_norm(df_sqrt(m), e / 2);
}
// an integer count as an sdf (exact below 2^48)
NBG_DEVICE sdf sdf_from_count(long long c) {
  return sdf_from_u128(static_cast<fx::u128>(c), 0, false);
}

// float64 nearest to x (hi + lo exactly combined, then rounded once), integer only
NBG_DEVICE double sdf_to_f64(const sdf& x) {
  if (x.zero) return 0.0;
  // both words as signed 64-bit integers scaled by 2^62 relative to 2^e, summed exactly
  const unsigned hb = static_cast<unsigned>(__float_as_int(x.m.hi));
  const unsigned lb = static_cast<unsigned>(__float_as_int(x.m.lo));
  const bool neg = (hb >> 31) != 0;
  const int eh = static_cast<int>((hb >> 23) & 0xff) - 127;  // 0 after normalisation
  long long vh = static_cast<long long>((hb & 0x7fffffu) | 0x800000u) << (62 - 23 + eh);
  long long vl = 0;
  if ((lb & 0x7fffffffu) != 0) {
    const int el = static_cast<int>((lb >> 23) & 0xff) - 127;
    const long long ml = static_cast<long long>((lb & 0x7fffffu) | 0x800000u);
    const int sh = 62 - 23 + el;
    vl = sh >= 0 ? (ml << sh) : (sh > -64 ? (ml >> -sh) : 0);
    if ((lb >> 31) != (hb >> 31)) vl = -vl;
  }
  const long long v = vh + vl;  // |v| < 2^63, sign of hi
  return fx::to_f64(static_cast<fx::i128>(neg ? -v : v), x.e - 62);
}

// ---- 256-bit integers for exact moment numerators ------------------------------------
struct u256 {
  unsigned long long w[4];  // little-endian words
};

NBG_DEVICE u256 mul128(fx::u128 a, fx::u128 b) {
  const unsigned long long a0 = static_cast<unsigned long long>(a), a1 = static_cast<unsigned long long>(a >> 64);
  const unsigned long long b0 = static_cast<unsigned long long>(b), b1 = static_cast<unsigned long long>(b >> 64);
  const fx::u128 p00 = static_cast<fx::u128>(a0) * b0;
  const fx::u128 p01 = static_cast<fx::u128>(a0) * b1;
  const fx::u128 p10 = static_cast<fx::u128>(a1) * b0;
  const fx::u128 p11 = static_cast<fx::u128>(a1) * b1;
  u256 r;
  r.w[0] = static_cast<unsigned long long>(p00);
  fx::u128 mid = (p00 >> 64) + static_cast<unsigned long long>(p01) + static_cast<unsigned long long>(p10);
  r.w[1] = static_cast<unsigned long long>(mid);
  fx::u128 hi = (mid >> 64) + (p01 >> 64) + (p10 >> 64) + p11;
  r.w[2] = static_cast<unsigned long long>(hi);
  r.w[3] = static_cast<unsigned long long>(hi >> 64);
  return r;
}
NBG_DEVICE u256 shl256(u256 x, int s) {  // 0 <= s < 64
  if (s == 0) return x;
  u256 r;
  r.w[3] = (x.w[3] << s) | (x.w[2] >> (64 - s));
  r.w[2] = (x.w[2] << s) | (x.w[1] >> (64 - s));
  r.w[1] = (x.w[1] << s) | (x.w[0] >> (64 - s));
  r.w[0] = x.w[0] << s;
  return r;
}
NBG_DEVICE u256 shl256_words(u256 x, int words) {
  u256 r = {{0, 0, 0, 0}};
  for (int i = 3; i >= words; --i) r.w[i] = x.w[i - words];
  return r;
}
NBG_DEVICE bool ge256(const u256& a, const u256& b) {
  for (int i = 3; i >= 0; --i)
    if (a.w[i] != b.w[i]) return a.w[i] > b.w[i];
  return true;
}
NBG_DEVICE u256 sub256(const u256& a, const u256& b) {  // a >= b
  u256 r;
  unsigned long long borrow = 0;
  for (int i = 0; i < 4; ++i) {
    const unsigned long long t = a.w[i] - b.w[i];
    const unsigned long long b1 = a.w[i] < b.w[i];
    r.w[i] = t - borrow;
    borrow = b1 | (t < borrow);
  }
  return r;
}

// |x| * 2^L as an sdf (48 leading bits, truncated below)
NBG_DEVICE sdf sdf_from_u256(const u256& x, int L, bool neg) {
  int top = 3;
  while (top > 0 && x.w[top] == 0) --top;
  if (x.w[top] == 0) return sdf_from_u128(0, 0, false);
  // take the two words ending at `top` as a 128-bit window
  const fx::u128 win = (static_cast<fx::u128>(x.w[top]) << 64) | (top > 0 ? x.w[top - 1] : 0ull);
  return sdf_from_u128(win, L + 64 * (top - 1), neg);
}

// s * v for a signed 128-bit s and a magnitude v: sign and 256-bit magnitude
struct s256 {
  u256 mag;
  bool neg;
};
NBG_DEVICE s256 smul(fx::i128 a, fx::i128 b) {
  const bool na = a < 0, nb = b < 0;
  const fx::u128 ua = na ? static_cast<fx::u128>(-a) : static_cast<fx::u128>(a);
  const fx::u128 ub = nb ? static_cast<fx::u128>(-b) : static_cast<fx::u128>(b);
  return s256{mul128(ua, ub), na != nb};
}
// x - y for signed 256-bit values
NBG_DEVICE s256 ssub(const s256& x, const s256& y) {
  if (x.neg != y.neg) {  // magnitudes add
    u256 r;
    unsigned long long carry = 0;
    for (int i = 0; i < 4; ++i) {
      const unsigned long long t = x.mag.w[i] + y.mag.w[i];
      const unsigned long long c1 = t < x.mag.w[i];
      r.w[i] = t + carry;
      carry = c1 | (r.w[i] < t);
    }
    return s256{r, x.neg};
  }
  if (ge256(x.mag, y.mag)) return s256{sub256(x.mag, y.mag), x.neg};
  return s256{sub256(y.mag, x.mag), !x.neg};
}

}  // namespace dfl

// a float64 as a double-float with integer instructions (the FP64 pipe converts slowly
// on this GPU): the top 24 bits of the mantissa as hi, the next 29 rounded into lo
// (about 48 bits in all); infinities and NaN keep their class, values beyond float32's
// range overflow to infinity and values below its normal range round through float32.
NBG_DEVICE dfl::df df_from_f64(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  const unsigned long long m = b & 0x000fffffffffffffull;
  if (e == 0x7ff) return dfl::df{__int_as_float(static_cast<int>(sign | 0x7f800000u | (m ? 0x400000u : 0u))), 0.0f};
  const int E = e - 1023;
  if (e == 0 || E < -126) {  // below float32's normal range: a float32 rounding of it
    const float h = __double2float_rn(x);
    return dfl::df{h, __double2float_rn(x - static_cast<double>(h))};
  }
  if (E > 127) return dfl::df{__int_as_float(static_cast<int>(sign | 0x7f800000u)), 0.0f};
  const unsigned long long M = m | 0x0010000000000000ull;
  const float hi = __int_as_float(static_cast<int>(sign | (static_cast<unsigned>(E + 127) << 23) |
                                                  static_cast<unsigned>((M >> 29) & 0x7fffffu)));
  const unsigned rem = static_cast<unsigned>(M & ((1ull << 29) - 1));
  float lo = 0.0f;
  if (rem && E - 52 >= -126) {
    lo = __fmul_rn(__uint2float_rn(rem), dfl::pow2f(E - 52));
    if (sign) lo = -lo;
  }
  return dfl::fast_two_sum(hi, lo);
}

// a float32 widened to float64 from its bit pattern (the FP64 pipe executes the
// conversion instruction, slowly on this GPU); zeros keep their sign, subnormals,
// infinities and NaN take the conversion instruction
NBG_DEVICE double widen_f32(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned ef = (b >> 23) & 0xffu;
  if ((b << 1) == 0u) return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(b >> 31) << 63));
  if (ef == 0u || ef == 0xffu) return static_cast<double>(x);
  const unsigned long long sign = static_cast<unsigned long long>(b >> 31) << 63;
  const unsigned long long e = static_cast<unsigned long long>(ef - 127u + 1023u);
  return __longlong_as_double(static_cast<long long>(sign | (e << 52) | (static_cast<unsigned long long>(b & 0x7fffffu) << 29)));
}
// hi + lo rounded to float64: two exact widenings and one float64 add
NBG_DEVICE double df_to_double(dfl::df x) { return widen_f32(x.hi) + widen_f32(x.lo); }
// a nonnegative count below 2^31 as a double-float, exactly
NBG_DEVICE dfl::df df_of_int(long long c) {
  if (c < (1ll << 24)) return dfl::df{f32_of_count(c), 0.0f};
  const int ci = static_cast<int>(c);
  const float hi = __int2float_rn(ci);
  return dfl::df{hi, __int2float_rn(ci - __float2int_rz(hi))};
}

// The pivot as a signed integer mantissa and biased exponent, and x - p from the two
// integer mantissas aligned at the larger exponent (9 guard bits, so the difference is
// exact whenever the exponents are within 9 and within 2^-53 of |x - p| otherwise),
// normalised into a double-float (48 bits) with integer instructions: no float64
// subtraction on the FP64 pipe.
struct Piv {
  long long m;
  int e;
  double d;  // the pivot itself
};
NBG_DEVICE Piv piv_of(double p) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(p));
  const int e0 = static_cast<int>((b >> 52) & 0x7ff);
  long long m = static_cast<long long>((b & 0x000fffffffffffffull) | (e0 ? 0x0010000000000000ull : 0ull));
  if (b >> 63) m = -m;
  return Piv{m, e0 ? e0 : 1, p};
}
NBG_DEVICE dfl::df sub_pivot(unsigned long long xb, Piv p) {
  const int e0 = static_cast<int>((xb >> 52) & 0x7ff);
  const int ex = e0 ? e0 : 1;
  long long mx = static_cast<long long>((xb & 0x000fffffffffffffull) | (e0 ? 0x0010000000000000ull : 0ull));
  if (xb >> 63) mx = -mx;
  const int E = ex > p.e ? ex : p.e;
  const int sx = E - ex, sp = E - p.e;
  const long long X = sx > 61 ? (mx < 0 ? -1ll : 0ll) : (mx * 512) >> sx;  // |mx * 512| < 2^62
  const long long P = sp > 61 ? (p.m < 0 ? -1ll : 0ll) : (p.m * 512) >> sp;
  const long long D = X - P;  // |D| < 2^63
  if (D == 0) return dfl::df{0.0f, 0.0f};
  const unsigned sign = D < 0 ? 0x80000000u : 0u;
  const unsigned long long U = static_cast<unsigned long long>(D < 0 ? -D : D);
  const int lz = __clzll(static_cast<long long>(U));
  const unsigned long long N = U << lz;  // leading one at bit 63
  const int fe = E - 894 - lz;           // float32 exponent field of the leading one
  if (fe < 1 + 48 || fe > 254)  // outside float32's comfortable range: the general path
    return df_from_f64(__longlong_as_double(static_cast<long long>(xb)) - p.d);
  const float hi = __uint_as_float(sign | (static_cast<unsigned>(fe) << 23) | static_cast<unsigned>((N >> 40) & 0x7fffffu));
  const unsigned L = static_cast<unsigned>((N >> 16) & 0xffffffu);  // the next 24 bits (the rest truncated)
  float l = __fmul_rn(__uint2float_rn(L), __uint_as_float(static_cast<unsigned>(fe - 47) << 23));
  if (sign) l = -l;
  return dfl::df{hi, l};
}

}  // namespace nbg
