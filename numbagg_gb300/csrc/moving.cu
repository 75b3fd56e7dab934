// Moving-window family: move_sum / move_mean / move_var / move_std / move_cov /
// move_corr (numbagg/moving.py:12-275), float64 and float32 arrays.
//
// The reference keeps running sums, adding the value that enters the window and
// removing the one that leaves (numbagg/moving.py:30-55).  The window state at i is
// therefore the prefix sum of the per-position difference
//     d_i = contrib(x_i) - contrib(x_{i-w})          (second term only when i >= w)
// where contrib() is the count and the moments the statistic needs (x; x, x^2; the
// pairwise-complete a, b, ab, a^2, b^2); a NaN contributes nothing.
//
// Exact sums.  The moments are accumulated as 128-bit fixed-point integers
// (fixed128.cuh) at the scale of the largest exponent in the tile, so every window
// sum is exact (to 2^-80 of its largest term) whatever the position in the row: the
// reference's own add/subtract drift is the only difference left between the two.
// Integer addition is associative, so results do not depend on how a row is cut into
// chunks and tiles, and are the same run to run, as long as no valid value in a row is
// more than 2^40 times smaller than the largest one met before it in its chunk (those
// would lose bits below the fixed-point LSB).  The exact sums are rounded once to
// float64 with integer instructions only and finalised with the reference's formulas.
// The division of the mean and of the squared sum by the count is correctly rounded
// (a table of reciprocals 1/c and Markstein's correction: q0 = s*r; e = fma(-q0, c, s);
// q = fma(e, r, q0); P. Markstein, IBM J. Res. Dev. 34(1), 1990), so exact zero
// variances stay zero; the final division by count - 1 multiplies by 1/(c - 1)
// (within one ulp of the quotient).  This GPU's FP64 pipe takes 16 cycles per warp
// instruction, so the finalisation is what bounds these kernels.
//
// Infinities follow the reference: an infinity in the running sum makes every later
// sum NaN once it leaves the window (inf - inf), or while infinities of both signs
// are inside; for the variance-like statistics any infinity (or |x| >= 2^512, whose
// square overflows) turns the rest of the row NaN.  These are tracked as counts.
//
// Parallel structure: a row is cut into chunks of at least 8 windows; a CTA seeds its
// chunk with the exact sums of the window before it (the w values preceding the chunk)
// and walks the chunk in sub-tiles of 2048 positions: coalesced loads of the entering
// and leaving values through a padded shared stage, 8 consecutive positions per
// thread, a block scan of the thread totals and a carry into the next sub-tile.  The
// scale only grows along the chunk (the carry is shifted when it does).  No state
// crosses chunks, except that the reference never recovers from an infinity: once one
// has left the window (sum, mean) or entered it (variance-like statistics) every later
// output of the row is NaN; the kernels record each row's first such position and a
// second kernel writes the NaNs after it.  Accumulation is exact for float32 arrays
// too (numba keeps float64 accumulators there, numbagg/moving.py:16); the result is
// rounded to float32.
#include "dfloat.cuh"
#include "fixed128.cuh"

#include <algorithm>
#include <climits>

namespace nbg {
namespace moving {

using fx::i128;

enum Op : int { kSum = 0, kMean = 1, kVar = 2, kStd = 3, kCov = 4, kCorr = 5 };

template <int OP>
struct Traits;
template <>
struct Traits<kSum> { static constexpr int NS = 1; static constexpr bool TWO = false; static constexpr bool VARLIKE = false; };
template <>
struct Traits<kMean> { static constexpr int NS = 1; static constexpr bool TWO = false; static constexpr bool VARLIKE = false; };
template <>
struct Traits<kVar> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kStd> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kCov> { static constexpr int NS = 3; static constexpr bool TWO = true; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kCorr> { static constexpr int NS = 5; static constexpr bool TWO = true; static constexpr bool VARLIKE = true; };

// moment j is a^order_a * b^order_b:  mean: a   var: a, a^2   cov: a, b, ab
// corr: a, b, ab, a^2, b^2
template <int OP>
NBG_HOST_DEVICE int order_a(int j) {
  if (OP == kSum || OP == kMean) return 1;
  if (OP == kVar || OP == kStd) return j == 0 ? 1 : 2;
  return j == 0 ? 1 : (j == 1 ? 0 : (j == 2 ? 1 : (j == 3 ? 2 : 0)));
}
template <int OP>
NBG_HOST_DEVICE int order_b(int j) {
  if (!Traits<OP>::TWO) return 0;
  return j == 0 ? 0 : (j == 1 ? 1 : (j == 2 ? 1 : (j == 3 ? 0 : 2)));
}

template <int NS>
struct Sums {  // tile-local moments (one scale for the whole tile)
  i128 s[NS];
  long long cnt;
  int inf_pos, inf_neg, inf_left;  // infinities entered (+, -) and left the window
  int pad;
};


template <int NS>
NBG_DEVICE Sums<NS> zero_sums() {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = 0;
  r.cnt = 0;
  r.inf_pos = r.inf_neg = r.inf_left = 0;
  r.pad = 0;
  return r;
}

template <int NS>
NBG_DEVICE Sums<NS> add(const Sums<NS>& a, const Sums<NS>& b) {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = a.s[j] + b.s[j];
  r.cnt = a.cnt + b.cnt;
  r.inf_pos = a.inf_pos + b.inf_pos;
  r.inf_neg = a.inf_neg + b.inf_neg;
  r.inf_left = a.inf_left + b.inf_left;
  r.pad = 0;
  return r;
}

// shift a tile's sums from scale (ea, eb) to (ea2, eb2) >= it
template <int OP>
NBG_DEVICE Sums<Traits<OP>::NS> rescale(const Sums<Traits<OP>::NS>& v, int ea, int eb, int ea2, int eb2) {
  Sums<Traits<OP>::NS> r = v;
  if (ea2 == ea && eb2 == eb) return r;
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j)
    r.s[j] = fx::shr(v.s[j], order_a<OP>(j) * (ea2 - ea) + order_b<OP>(j) * (eb2 - eb));
  return r;
}

NBG_DEVICE i128 shfl_i128(i128 v, int src_or_delta, bool up) {
  const unsigned long long lo = static_cast<unsigned long long>(v);
  const unsigned long long hi = static_cast<unsigned long long>(v >> 64);
  const unsigned long long rlo = up ? __shfl_up_sync(0xffffffffu, lo, src_or_delta) : __shfl_xor_sync(0xffffffffu, lo, src_or_delta);
  const unsigned long long rhi = up ? __shfl_up_sync(0xffffffffu, hi, src_or_delta) : __shfl_xor_sync(0xffffffffu, hi, src_or_delta);
  return static_cast<i128>((static_cast<fx::u128>(rhi) << 64) | rlo);
}

template <int NS>
NBG_DEVICE Sums<NS> shfl_sums(const Sums<NS>& v, int d, bool up) {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = shfl_i128(v.s[j], d, up);
  r.cnt = up ? __shfl_up_sync(0xffffffffu, v.cnt, d) : __shfl_xor_sync(0xffffffffu, v.cnt, d);
  r.inf_pos = up ? __shfl_up_sync(0xffffffffu, v.inf_pos, d) : __shfl_xor_sync(0xffffffffu, v.inf_pos, d);
  r.inf_neg = up ? __shfl_up_sync(0xffffffffu, v.inf_neg, d) : __shfl_xor_sync(0xffffffffu, v.inf_neg, d);
  r.inf_left = up ? __shfl_up_sync(0xffffffffu, v.inf_left, d) : __shfl_xor_sync(0xffffffffu, v.inf_left, d);
  r.pad = 0;
  return r;
}

// ---------------------------------------------------------------------------------
// values from their bits (integer instructions only)
// ---------------------------------------------------------------------------------
struct Val {
  unsigned long long m;  // integer mantissa: value = m * 2^(e - 1075)
  int e;                 // biased float64 exponent, 1 for zeros and subnormals
  bool neg, nan, inf;
};
NBG_DEVICE Val val_of(unsigned long long b) {  // float64 bits
  const int eb = static_cast<int>((b >> 52) & 0x7ff);
  Val v;
  const unsigned long long f = b & 0x000fffffffffffffull;
  v.m = f | (eb ? 0x0010000000000000ull : 0ull);
  v.e = eb ? eb : 1;
  v.neg = (b >> 63) != 0;
  v.nan = eb == 0x7ff && f != 0;
  v.inf = eb == 0x7ff && f == 0;
  return v;
}
NBG_DEVICE Val val_of(unsigned b) {  // float32 bits, restated exactly in the float64 format
  const int eb = static_cast<int>((b >> 23) & 0xff);
  const unsigned f = b & 0x7fffffu;
  Val v;
  v.m = static_cast<unsigned long long>(f | (eb ? 0x800000u : 0u)) << 29;
  v.e = eb ? eb + 896 : 897;
  v.neg = (b >> 31) != 0;
  v.nan = eb == 0xff && f != 0;
  v.inf = eb == 0xff && f == 0;
  return v;
}

NBG_DEVICE i128 fix_v(const Val& x, int E) {
  const fx::u128 v = fx::shift_u(static_cast<fx::u128>(x.m), x.e - E + fx::kValueShift);
  return x.neg ? -static_cast<i128>(v) : static_cast<i128>(v);
}
NBG_DEVICE i128 fix_sq(const Val& x, int E) {
  return static_cast<i128>(fx::shift_u(static_cast<fx::u128>(x.m) * x.m, 2 * (x.e - E) + fx::kSquareShift));
}
NBG_DEVICE i128 fix_pr(const Val& x, const Val& y, int Ex, int Ey) {
  const fx::u128 v = fx::shift_u(static_cast<fx::u128>(x.m) * y.m, (x.e - Ex) + (y.e - Ey) + fx::kSquareShift);
  return (x.neg != y.neg) ? -static_cast<i128>(v) : static_cast<i128>(v);
}

// the reference's x * x overflows to inf: |x| >= 2^512
NBG_DEVICE bool sq_overflow(const Val& x) { return x.e >= 1023 + 512; }

// A position: valid (pairwise complete), "bad" (an infinity, or for the variance-like
// statistics a value whose square overflows), and its exponents for the scale.
template <int OP>
struct Pos {
  Val a, b;
  bool valid, bad;
};
template <int OP, typename B>
NBG_DEVICE Pos<OP> pos_of(B ab, B bb) {
  constexpr bool TWO = Traits<OP>::TWO, VL = Traits<OP>::VARLIKE;
  Pos<OP> p;
  p.a = val_of(ab);
  p.b = TWO ? val_of(bb) : p.a;
  p.valid = !p.a.nan && !(TWO && p.b.nan);
  p.bad = p.valid && (p.a.inf || (TWO && p.b.inf) || (VL && (sq_overflow(p.a) || (TWO && sq_overflow(p.b)))));
  return p;
}

// Add (sign = +1, the entering value) or remove (sign = -1, the leaving value) one
// position's contribution at the scale (Ea, Eb).
template <int OP>
NBG_DEVICE void accumulate(Sums<Traits<OP>::NS>& acc, const Pos<OP>& p, int sign, int Ea, int Eb) {
  constexpr bool TWO = Traits<OP>::TWO;
  if (!p.valid) return;
  acc.cnt += sign;
  if (p.bad) {
    if (sign > 0) {
      if (TWO || Traits<OP>::VARLIKE || !p.a.neg) acc.inf_pos += 1; else acc.inf_neg += 1;
    } else {
      acc.inf_left += 1;
    }
    return;
  }
  i128 m[5];
  if (OP == kSum || OP == kMean) {
    m[0] = fix_v(p.a, Ea);
  } else if (OP == kVar || OP == kStd) {
    m[0] = fix_v(p.a, Ea);
    m[1] = fix_sq(p.a, Ea);
  } else {
    m[0] = fix_v(p.a, Ea);
    m[1] = fix_v(p.b, Eb);
    m[2] = fix_pr(p.a, p.b, Ea, Eb);
    if (OP == kCorr) {
      m[3] = fix_sq(p.a, Ea);
      m[4] = fix_sq(p.b, Eb);
    }
  }
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) acc.s[j] = sign > 0 ? acc.s[j] + m[j] : acc.s[j] - m[j];
}

NBG_DEVICE bool finite_bits(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// 1/c from the table (correctly rounded), beyond it a division
NBG_DEVICE double rcp_of(long long c, const double* __restrict__ rcp, long long rcp_n) {
  return c <= rcp_n ? __ldg(rcp + c) : 1.0 / static_cast<double>(c);
}
// s / c correctly rounded (Markstein's correction of s * (1/c)); non-finite s divides
NBG_DEVICE double div_count(double s, long long c, double r) {
  if (!finite_bits(s)) return s / static_cast<double>(c);
  const double q0 = s * r;
  const double e = fma(-q0, f64_of_count(c), s);
  return fma(e, r, q0);
}

template <int OP>
NBG_DEVICE double finalize(const Sums<Traits<OP>::NS>& st, int ea, int eb, long long min_count,
                           const double* __restrict__ rcp, long long rcp_n) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long c = st.cnt;
  if (OP == kSum || OP == kMean) {
    const long long mc = OP == kMean ? (min_count > 1 ? min_count : 1) : min_count;
    if (c < mc) return nan;
    if (st.inf_left > 0 || (st.inf_pos > 0 && st.inf_neg > 0)) return nan;
    double s;
    if (st.inf_pos > 0) s = __longlong_as_double(0x7ff0000000000000ll);
    else if (st.inf_neg > 0) s = __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
    else s = fx::to_f64(st.s[0], fx::lsb_value(ea));
    return OP == kSum ? s : div_count(s, c, rcp_of(c, rcp, rcp_n));
  }
  if (OP == kVar || OP == kStd) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc || st.inf_pos > 0) return nan;
    const double s1 = fx::to_f64(st.s[0], fx::lsb_value(ea));
    const double s2 = fx::to_f64(st.s[1], fx::lsb_product(ea, ea));
    // (asum_sq - asum**2 / count) / (count - 1)    numbagg/moving.py:147-148
    const double v = (s2 - div_count(s1 * s1, c, rcp_of(c, rcp, rcp_n))) * rcp_of(c - 1, rcp, rcp_n);
    return OP == kStd ? sqrt(v) : v;
  }
  if (OP == kCov) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc || st.inf_pos > 0) return nan;
    const double sa = fx::to_f64(st.s[0], fx::lsb_value(ea));
    const double sb = fx::to_f64(st.s[1], fx::lsb_value(eb));
    const double sab = fx::to_f64(st.s[2], fx::lsb_product(ea, eb));
    // (prodsum - asum * bsum / count) / (count - 1)   numbagg/moving.py:217-218
    return (sab - div_count(sa * sb, c, rcp_of(c, rcp, rcp_n))) * rcp_of(c - 1, rcp, rcp_n);
  }
  // kCorr, numbagg/moving.py:263-273
  const long long mc = min_count > 1 ? min_count : 1;
  if (c < mc || st.inf_pos > 0) return nan;
  const double sa = fx::to_f64(st.s[0], fx::lsb_value(ea));
  const double sb = fx::to_f64(st.s[1], fx::lsb_value(eb));
  const double sab = fx::to_f64(st.s[2], fx::lsb_product(ea, eb));
  const double saa = fx::to_f64(st.s[3], fx::lsb_product(ea, ea));
  const double sbb = fx::to_f64(st.s[4], fx::lsb_product(eb, eb));
  const double rc = rcp_of(c, rcp, rcp_n);
  const double avg_a = sa * rc;
  const double avg_b = sb * rc;
  const double var_a = saa * rc - avg_a * avg_a;
  const double var_b = sbb * rc - avg_b * avg_b;
  const double cov_ab = sab * rc - avg_a * avg_b;
  const double vv = var_a * var_b;
  return vv > 0 ? cov_ab / sqrt(vv) : nan;
}

// The FP32-compensated ("fp32c") finalisation: no floating-point rounding until the
// last step.  The second moments are exact integer numerators
//     N_xy = c * S_xy * 2^93 - S_x * S_y        (256-bit, units of 2^(Lx + Ly))
// so var = N_xx / (c (c - 1)), cov = N_xy / (c (c - 1)), corr = N_ab / sqrt(N_aa N_bb)
// (the reference's formulas with the common factors cancelled), evaluated in scaled
// double-float on the FP32 pipes and rounded once to float64.  About 2^-46 relative
// error, and no cancellation: the result is that of the exact window sums.
NBG_DEVICE dfl::s256 numerator(i128 sxy, i128 sx, i128 sy, long long c) {
  dfl::s256 a = dfl::smul(sxy, static_cast<i128>(c));
  a.mag = dfl::shl256(dfl::shl256_words(a.mag, 1), 29);  // * 2^93
  return dfl::ssub(a, dfl::smul(sx, sy));
}

template <int OP>
NBG_DEVICE double finalize_c(const Sums<Traits<OP>::NS>& st, int ea, int eb, long long min_count) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long c = st.cnt;
  if (OP == kSum || OP == kMean) {
    const long long mc = OP == kMean ? (min_count > 1 ? min_count : 1) : min_count;
    if (c < mc) return nan;
    if (st.inf_left > 0 || (st.inf_pos > 0 && st.inf_neg > 0)) return nan;
    if (st.inf_pos > 0) return __longlong_as_double(0x7ff0000000000000ll);
    if (st.inf_neg > 0) return __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
    if (OP == kSum) return fx::to_f64(st.s[0], fx::lsb_value(ea));
    const i128 s1 = st.s[0];
    const dfl::sdf m = dfl::sdf_from_u128(s1 < 0 ? static_cast<fx::u128>(-s1) : static_cast<fx::u128>(s1),
                                          fx::lsb_value(ea), s1 < 0);
    return dfl::sdf_to_f64(dfl::sdf_div(m, dfl::sdf_from_count(c)));
  }
  if (OP == kVar || OP == kStd || OP == kCov) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc || st.inf_pos > 0) return nan;
    const dfl::s256 nm = OP == kCov ? numerator(st.s[2], st.s[0], st.s[1], c) : numerator(st.s[1], st.s[0], st.s[0], c);
    const int L = fx::lsb_value(ea) + fx::lsb_value(OP == kCov ? eb : ea);
    const dfl::sdf v = dfl::sdf_div(dfl::sdf_from_u256(nm.mag, L, nm.neg), dfl::sdf_from_count(c * (c - 1)));
    if (OP == kStd) return nm.neg ? nan : dfl::sdf_to_f64(dfl::sdf_sqrt(v));
    return dfl::sdf_to_f64(v);
  }
  // kCorr
  const long long mc = min_count > 1 ? min_count : 1;
  if (c < mc || st.inf_pos > 0) return nan;
  const dfl::s256 nab = numerator(st.s[2], st.s[0], st.s[1], c);
  const dfl::s256 naa = numerator(st.s[3], st.s[0], st.s[0], c);
  const dfl::s256 nbb = numerator(st.s[4], st.s[1], st.s[1], c);
  const int la = fx::lsb_value(ea), lb = fx::lsb_value(eb);
  const dfl::sdf vaa = dfl::sdf_from_u256(naa.mag, 2 * la, naa.neg);
  const dfl::sdf vbb = dfl::sdf_from_u256(nbb.mag, 2 * lb, nbb.neg);
  if (vaa.zero || vbb.zero || naa.neg != nbb.neg) return nan;  // var_a * var_b > 0
  const dfl::sdf den = dfl::sdf_sqrt(dfl::sdf_mul(vaa, vbb));
  const dfl::sdf cov = dfl::sdf_from_u256(nab.mag, la + lb, nab.neg);
  return dfl::sdf_to_f64(dfl::sdf_div(cov, den));
}

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------
constexpr int NT = 256;
constexpr int KT = 8;              // consecutive positions per thread
constexpr int SUB = NT * KT;       // positions per sub-tile
constexpr int SPAD = SUB + SUB / KT;
constexpr long long kRcpEntries = 65536;

// padded stage index: one spare word after every thread's run of KT, so the 32
// threads of a warp reading word k of their runs hit distinct banks
NBG_DEVICE int spad(int p) { return p + p / KT; }

template <int NS>
NBG_DEVICE Sums<NS> block_sum(Sums<NS> v, Sums<NS>* warp_buf) {  // result valid in every thread
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = add(v, shfl_sums(v, o, false));
  __syncthreads();
  if (lane == 0) warp_buf[warp] = v;
  __syncthreads();
  Sums<NS> r = warp_buf[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) r = add(r, warp_buf[w]);
  return r;
}

NBG_DEVICE int block_max(int v, int* buf) {  // result valid in every thread; buf[NT/32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(v)));
  __syncthreads();
  if (lane == 0) buf[warp] = v;
  __syncthreads();
  int r = buf[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) r = max(r, buf[w]);
  return r;
}

// CTAs per SM the kernels are compiled for: three for the single-input statistics, two
// for covariance / correlation (five 128-bit sums)
template <int OP>
struct MoveOcc {
  static constexpr int value = Traits<OP>::TWO ? 2 : 3;
};

template <int OP, typename T, bool C>
__global__ void __launch_bounds__(NT, MoveOcc<OP>::value) move_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                     T* __restrict__ out, Layout lay, long long window,
                                                     long long min_count, long long chunk_len,
                                                     const double* __restrict__ rcp, long long rcp_n,
                                                     long long* __restrict__ first_bad,
                                                     const unsigned* __restrict__ only_rows) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool TWO = Traits<OP>::TWO;
  typedef typename BitsOf<T>::type B;
  using S = Sums<NS>;
  // stage (dynamic shared memory): entering a, leaving a[, entering b, leaving b]
  extern __shared__ __align__(16) unsigned char stage_raw[];
  B(*stage)[SPAD] = reinterpret_cast<B(*)[SPAD]>(stage_raw);
  __shared__ S warp_buf[NT / 32];
  __shared__ S carry_s;
  __shared__ int red[2][NT / 32];
  const B nanb = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned long long last_use = l2_evict_first();
  const long long items = layout_items(lay);
  // a persistent grid walks the chunks (of rows, or of ragged series)
  for (long long id = blockIdx.x; id < items; id += gridDim.x) {
  const Item it = layout_item(lay, id);
  const long long row = it.row, n = it.len;
  // only_rows: recompute just the rows the double-float scan flagged (the whole CTA
  // takes the same branch, before any barrier)
  if (only_rows && only_rows[row] == 0u) continue;
  const long long c0 = it.index * chunk_len, c1 = min(n, c0 + chunk_len);
  const B* ar = as_bits(a) + it.base;
  const B* br = TWO ? as_bits(b) + it.base : ar;
  T* orow = out + it.base;

  // ---- the state entering the chunk: the window [c0 - w, c0) ----
  const long long h0 = c0 > window ? c0 - window : 0;
  int ea = 0, eb = 0;
  for (long long i = h0 + tid; i < c0; i += NT) {
    const Pos<OP> p = pos_of<OP>(ar[i], TWO ? br[i] : ar[i]);
    if (p.valid && !p.bad) {
      ea = max(ea, p.a.e);
      eb = max(eb, p.b.e);
    }
  }
  int Ea = max(1, block_max(ea, red[0]));
  int Eb = TWO ? max(1, block_max(eb, red[1])) : 1;
  S seed = zero_sums<NS>();
  for (long long i = h0 + tid; i < c0; i += NT)
    accumulate<OP>(seed, pos_of<OP>(ar[i], TWO ? br[i] : ar[i]), +1, Ea, Eb);
  seed = block_sum(seed, warp_buf);
  if (tid == 0) carry_s = seed;

  long long bad_pos = LLONG_MAX;
  for (long long s0 = c0; s0 < c1; s0 += SUB) {
    // ---- stage the entering and leaving values; the sub-tile's exponents ----
    int ma = 0, mb = 0;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      const long long i = s0 + p;
      const bool in = i < c1, old = in && i >= window;
      const B xa = in ? ar[i] : nanb;
      const B xo = old ? ld_hint(ar + (i - window), last_use) : nanb;
      const B ya = (TWO && in) ? br[i] : nanb;
      const B yo = (TWO && old) ? ld_hint(br + (i - window), last_use) : nanb;
      stage[0][spad(p)] = xa;
      stage[1][spad(p)] = xo;
      if (TWO) {
        stage[2][spad(p)] = ya;
        stage[3][spad(p)] = yo;
      }
      const Pos<OP> pe = pos_of<OP>(xa, ya), po = pos_of<OP>(xo, yo);
      if (pe.valid && !pe.bad) {
        ma = max(ma, pe.a.e);
        mb = max(mb, pe.b.e);
      }
      if (po.valid && !po.bad) {
        ma = max(ma, po.a.e);
        mb = max(mb, po.b.e);
      }
      if (pe.bad) bad_pos = min(bad_pos, i);
    }
    const int Ean = max(Ea, block_max(ma, red[0]));  // the syncs also publish the stage
    const int Ebn = TWO ? max(Eb, block_max(mb, red[1])) : Eb;
    S carry = rescale<OP>(carry_s, Ea, Eb, Ean, Ebn);
    Ea = Ean;
    Eb = Ebn;

    // ---- thread totals over KT consecutive positions, block scan ----
    const int q0 = tid * KT;
    S tot = zero_sums<NS>();
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      const int sp = spad(q0 + k);
      accumulate<OP>(tot, pos_of<OP>(stage[0][sp], TWO ? stage[2][sp] : stage[0][sp]), +1, Ea, Eb);
      accumulate<OP>(tot, pos_of<OP>(stage[1][sp], TWO ? stage[3][sp] : stage[1][sp]), -1, Ea, Eb);
    }
    S incl = tot;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const S up = shfl_sums(incl, d, true);
      if (lane >= d) incl = add(up, incl);
    }
    if (lane == 31) warp_buf[warp] = incl;
    __syncthreads();
    S st = carry;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w)
      if (w < warp) st = add(st, warp_buf[w]);
    S lane_excl = shfl_sums(incl, 1, true);
    if (lane > 0) st = add(st, lane_excl);

    // ---- outputs, written back over the thread's own entering slots ----
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      const int sp = spad(q0 + k);
      accumulate<OP>(st, pos_of<OP>(stage[0][sp], TWO ? stage[2][sp] : stage[0][sp]), +1, Ea, Eb);
      accumulate<OP>(st, pos_of<OP>(stage[1][sp], TWO ? stage[3][sp] : stage[1][sp]), -1, Ea, Eb);
      const T r = static_cast<T>(C ? finalize_c<OP>(st, Ea, Eb, min_count) : finalize<OP>(st, Ea, Eb, min_count, rcp, rcp_n));
      if (sizeof(T) == 8) stage[0][sp] = static_cast<B>(__double_as_longlong(static_cast<double>(r)));
      else stage[0][sp] = static_cast<B>(__float_as_uint(static_cast<float>(r)));
    }
    if (tid == NT - 1) carry_s = st;  // everyone read carry_s before the scan's barrier
    __syncthreads();
    B* ob = as_bits(orow);
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      if (s0 + p < c1) ob[s0 + p] = stage[0][spad(p)];
    }
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) bad_pos = min(bad_pos, __shfl_xor_sync(0xffffffffu, bad_pos, o));
  if (lane == 0 && bad_pos != LLONG_MAX) atomicMin(reinterpret_cast<unsigned long long*>(first_bad + row),
                                                   static_cast<unsigned long long>(bad_pos));
  __syncthreads();  // the shared state is reused by the next chunk
  }
}

// reciprocal table and per-row first infinity, once per call
__global__ void move_setup_kernel(double* __restrict__ rcp, long long rcp_n, long long* __restrict__ first_bad,
                                  long long rows, unsigned* __restrict__ flags) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const long long t0 = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (long long c = t0; c <= rcp_n; c += stride) rcp[c] = c ? 1.0 / static_cast<double>(c) : 0.0;
  for (long long r = t0; r < rows; r += stride) {
    first_bad[r] = LLONG_MAX;
    if (flags) flags[r] = 0u;
  }
}

// The reference never recovers from an infinity (inf - inf = NaN in its running sums):
// NaN from the first position where one has left the window (sum, mean) or entered it.
template <typename T, bool VARLIKE>
__global__ void move_poison_kernel(T* __restrict__ out, Layout lay, long long window,
                                   const long long* __restrict__ first_bad) {
  for (long long r = blockIdx.x; r < lay.rows; r += gridDim.x) {
    const long long f = first_bad[r];
    if (f == LLONG_MAX) continue;
    const long long n = layout_row_len(lay, r), base = layout_row_base(lay, r);
    const long long from = VARLIKE ? f : (f > LLONG_MAX - window ? LLONG_MAX : f + window);
    const T nan = quiet_nan(T(0));
    for (long long i = (from < n ? from : n) + threadIdx.x; i < n; i += blockDim.x) out[base + i] = nan;
  }
}

// ---------------------------------------------------------------------------------
// FP32-compensated form, one pass: double-float window sums
// ---------------------------------------------------------------------------------
// The window state at i (the count and the sums: x; or y = x - p, y^2; ya, yb, ya yb,
// ya^2, yb^2, with p the row's pivot, its first finite value) is the prefix sum of the
// differences d_i = c(x_i) - c(x_{i-w}).  Rows are cut into tiles of 1024 positions,
// claimed row-interleaved.  A tile stages its entering and leaving values; each thread
// folds the differences of 8 consecutive positions in double-float (about 48 bits, on
// the FP32 pipes); a warp scan and a fold over the warps give the tile's total; lane 0
// chains it to the inclusive prefix that the row's previous tile published (a bounded
// wait) and publishes its own, so the result does not depend on timing; each thread
// then replays its positions from the state entering them and finalises.  Every value
// is read once as entering and once as leaving (from L2 while the window is short).
// Rows holding an infinity or a value outside the range these sums keep to the
// stated bound (|x| or |y| of 2^50 and more, or a nonzero |y| below 2^-60; |x| outside
// [2^-100, 2^100] for sums and means) are flagged and recomputed by move_kernel's exact
// sums, which also carry the reference's infinity semantics.
namespace dsc {
constexpr int NT = 128;
constexpr int KT = 8;
constexpr int TILE = NT * KT;
constexpr int SPAD = TILE + TILE / KT;
NBG_DEVICE int spad(int p) { return p + p / KT; }

template <int NS>
struct St {
  dfl::df s[NS];
  int cnt;
  int pad;
};
template <int NS>
NBG_DEVICE St<NS> st_zero() {
  St<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = dfl::df{0.0f, 0.0f};
  r.cnt = 0;
  r.pad = 0;
  return r;
}
template <int NS>
NBG_DEVICE St<NS> st_add(const St<NS>& a, const St<NS>& b) {
  St<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = dfl::df_add(a.s[j], b.s[j]);
  r.cnt = a.cnt + b.cnt;
  r.pad = 0;
  return r;
}
template <int NS>
NBG_DEVICE St<NS> st_shfl_up(const St<NS>& v, int d) {
  St<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j)
    r.s[j] = dfl::df{__shfl_up_sync(0xffffffffu, v.s[j].hi, d), __shfl_up_sync(0xffffffffu, v.s[j].lo, d)};
  r.cnt = __shfl_up_sync(0xffffffffu, v.cnt, d);
  r.pad = 0;
  return r;
}

// |x| within [2^-100, 2^100] or zero (sums, means); |x| below 2^50 (the rest)
template <bool VL>
NBG_DEVICE bool raw_ok(unsigned long long b) {
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  if (VL) return e < 1023 + 50;
  return (b << 1) == 0 || (e >= 1023 - 100 && e <= 1023 + 100);
}
// a pivoted value zero or at least 2^-60 in magnitude
NBG_DEVICE bool piv_ok(dfl::df y) {
  const unsigned b = __float_as_uint(y.hi);
  return (b << 1) == 0u || static_cast<int>((b >> 23) & 0xff) >= 127 - 60;
}

// One position's contributions (the value pair is valid): x for sums and means; the
// pivoted y = x - p (sub_pivot), y^2
// (variance); ya, yb, ya yb (covariance); + ya^2, yb^2 (correlation).  `ok` turns
// false when a value is outside the range above.
template <int OP>
NBG_DEVICE void contrib(unsigned long long xb, unsigned long long yb, Piv px, Piv py, dfl::df* c, bool& ok) {
  constexpr bool VL = Traits<OP>::VARLIKE, TWO = Traits<OP>::TWO;
  using namespace dfl;
  ok = ok && raw_ok<VL>(xb) && (!TWO || raw_ok<VL>(yb));
  if (!VL) {
    c[0] = df_from_f64(__longlong_as_double(static_cast<long long>(xb)));
    return;
  }
  // one input: the float64 subtraction (its pipe has room here); two inputs: the
  // integer one (measured faster for each)
  const df x = TWO ? sub_pivot(xb, px) : df_from_f64(__longlong_as_double(static_cast<long long>(xb)) - px.d);
  ok = ok && piv_ok(x);
  if (OP == kVar || OP == kStd) {
    c[0] = x;
    c[1] = df_mul(x, x);
    return;
  }
  const df y = sub_pivot(yb, py);
  ok = ok && piv_ok(y);
  c[0] = x;
  c[1] = y;
  c[2] = df_mul(x, y);
  if (OP == kCorr) {
    c[3] = df_mul(x, x);
    c[4] = df_mul(y, y);
  }
}

// s / c for a count c >= 1 (exact in float32 below 2^24)
NBG_DEVICE dfl::df df_div_count(dfl::df s, long long c) {
  using namespace dfl;
  const float cf = f32_of_count(c);
  if (c < (1ll << 24)) {  // a reciprocal, a quotient and one corrected quotient (~2^-44)
    const float rc = __frcp_rn(cf);
    const float q1 = __fmul_rn(s.hi, rc);
    const df r = df_sub(s, two_prod(q1, cf));
    return fast_two_sum(q1, __fmul_rn(r.hi, rc));
  }
  const double cd = static_cast<double>(c);
  return df_div(s, df_from_f64(cd));
}
NBG_DEVICE dfl::df df_of_count(long long c) {
  return c < (1ll << 31) ? df_of_int(c) : df_from_f64(static_cast<double>(c));
}
NBG_DEVICE double df_out(dfl::df x) {
  if (!isfinite(x.hi)) return static_cast<double>(x.hi);
  return df_to_double(x);
}

// the reference's statistics from the window sums (numbagg/moving.py:12-275), with the
// common factors cancelled: var = (c S_yy - S_y^2) / (c (c - 1)), the same for the
// covariance, corr = N_ab / sqrt(N_aa N_bb)
template <int OP>
NBG_DEVICE double finalize_d(const St<Traits<OP>::NS>& st, long long min_count) {
  using namespace dfl;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long c = st.cnt;
  // an empty window sums to exactly zero (the double-float prefix differences would
  // leave the rounding residue of the values that came and went)
  if (OP == kSum) return c >= min_count ? (c == 0 ? 0.0 : df_out(st.s[0])) : nan;
  if (OP == kMean) return c >= (min_count > 1 ? min_count : 1) ? df_out(df_div_count(st.s[0], c)) : nan;
  const df cd = df_of_count(c);
  if (OP == kVar || OP == kStd || OP == kCov) {
    if (c < (min_count > 2 ? min_count : 2)) return nan;
    const df num = OP == kCov ? df_sub(df_mul(cd, st.s[2]), df_mul(st.s[0], st.s[1]))
                              : df_sub(df_mul(cd, st.s[1]), df_mul(st.s[0], st.s[0]));
    const long long cc = c * (c - 1);
    const df v = cc < (1ll << 24) ? df_div_count(num, cc) : df_div_count(df_div_count(num, c), c - 1);
    if (OP != kStd) return df_out(v);
    if (v.hi < 0.0f) return nan;
    return v.hi == 0.0f ? 0.0 : df_out(df_sqrt(v));
  }
  if (c < (min_count > 1 ? min_count : 1)) return nan;
  const df naa = df_sub(df_mul(cd, st.s[3]), df_mul(st.s[0], st.s[0]));
  const df nbb = df_sub(df_mul(cd, st.s[4]), df_mul(st.s[1], st.s[1]));
  const df nab = df_sub(df_mul(cd, st.s[2]), df_mul(st.s[0], st.s[1]));
  const df vv = df_mul(naa, nbb);
  if (!(vv.hi > 0.0f || (vv.hi == 0.0f && vv.lo > 0.0f))) return nan;
  return df_out(df_div(nab, df_sqrt(vv)));
}

// the row's (or ragged series') pivot: its first finite value (0 when it has none)
template <typename T>
__global__ void dsc_pivot_kernel(const T* __restrict__ a, const T* __restrict__ b, long long rows, long long n,
                                 const long long* __restrict__ offsets, double* __restrict__ pivots) {
  const int lane = threadIdx.x & 31;
  const long long row = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (row >= rows) return;
  if (offsets) n = offsets[row + 1] - offsets[row];
  const long long base = offsets ? offsets[row] : row * n;
  for (int w = 0; w < (b ? 2 : 1); ++w) {
    const T* r = (w ? b : a) + base;
    double pv = 0.0;
    for (long long base = 0; base < n; base += 32) {
      const long long i = base + lane;
      const double v = i < n ? static_cast<double>(r[i]) : 0.0;
      const bool fin = i < n && ((static_cast<unsigned long long>(__double_as_longlong(v)) >> 52 & 0x7ff) != 0x7ff);
      const unsigned m = __ballot_sync(0xffffffffu, fin);
      if (m) {
        pv = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
        break;
      }
    }
    if (lane == 0) pivots[2 * row + w] = pv;
  }
}

template <int OP, typename T>
__global__ void __launch_bounds__(NT) move_dscan_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                        T* __restrict__ out, long long rows, long long n,
                                                        long long window, long long min_count,
                                                        long long tiles_per_row, void* ws_base, size_t ws_bytes,
                                                        const double* __restrict__ pivots,
                                                        unsigned* __restrict__ row_flags) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool TWO = Traits<OP>::TWO;
  constexpr bool VL = Traits<OP>::VARLIKE;
  typedef typename BitsOf<T>::type B;
  using S = St<NS>;
  using dfl::df;
  // single-input statistics keep each position's difference for the replay
  constexpr bool CACHE = !TWO;
  __shared__ B sx[SPAD], so[SPAD];
  __shared__ B sy[TWO ? SPAD : 1], syo[TWO ? SPAD : 1];
  __shared__ df sdl[CACHE ? NS : 1][CACHE ? SPAD : 1];
  __shared__ signed char sdc[CACHE ? SPAD : 1];
  __shared__ S wtot[NT / 32];
  __shared__ S carry_smem;
  __shared__ long long tile_smem;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const B nanb = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);
  const long long total_tiles = rows * tiles_per_row;
  const unsigned long long last_use = l2_evict_first();

  for (;;) {
    if (tid == 0) tile_smem = claim_tile(ws.hdr);
    __syncthreads();
    const long long tile = tile_smem;
    if (tile >= total_tiles) break;
    const TileCoord tc = tile_coord(tile, rows);
    const long long row = tc.row, chunk = tc.chunk;
    const long long t0 = chunk * TILE;
    const B* ar = as_bits(a) + row * n;
    const B* br = TWO ? as_bits(b) + row * n : nullptr;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      const long long i = t0 + p;
      const bool in = i < n, old = in && i >= window;
      sx[spad(p)] = in ? ar[i] : nanb;
      so[spad(p)] = old ? ld_hint(ar + (i - window), last_use) : nanb;
      if (TWO) {
        sy[spad(p)] = in ? br[i] : nanb;
        syo[spad(p)] = old ? ld_hint(br + (i - window), last_use) : nanb;
      }
    }
    __syncthreads();
    const Piv px = piv_of(VL ? pivots[2 * row] : 0.0);
    const Piv py = piv_of((VL && TWO) ? pivots[2 * row + 1] : 0.0);
    const int q0 = tid * KT;
    bool ok = true;
    // position k's difference: the entering contributions minus the leaving ones
    auto delta = [&](int k, df* d, int& dc) {
      const int sp = spad(q0 + k);
      const B xi = sx[sp], xo = so[sp];
      const B yi = TWO ? sy[sp] : xi, yo = TWO ? syo[sp] : xo;
      df c[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) d[j] = df{0.0f, 0.0f};
      dc = 0;
      if (!nan_bits(xi) && !(TWO && nan_bits(yi))) {
        contrib<OP>(xi, yi, px, py, c, ok);
#pragma unroll
        for (int j = 0; j < NS; ++j) d[j] = c[j];
        dc = 1;
      }
      if (!nan_bits(xo) && !(TWO && nan_bits(yo))) {
        contrib<OP>(xo, yo, px, py, c, ok);
#pragma unroll
        for (int j = 0; j < NS; ++j) d[j] = dfl::df_add_fast(d[j], dfl::df_neg(c[j]));
        --dc;
      }
    };
    // ---- this thread's run of differences, then the warp scan ----
    S run = st_zero<NS>();
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      df d[NS];
      int dc;
      delta(k, d, dc);
#pragma unroll
      for (int j = 0; j < NS; ++j) run.s[j] = dfl::df_add_fast(run.s[j], d[j]);
      run.cnt += dc;
      if (CACHE) {
        const int sp = spad(q0 + k);
#pragma unroll
        for (int j = 0; j < NS; ++j) sdl[j][sp] = d[j];
        sdc[sp] = static_cast<signed char>(dc);
      }
    }
    S incl = run;
#pragma unroll
    for (int dl = 1; dl < 32; dl <<= 1) {
      const S up = st_shfl_up(incl, dl);
      if (lane >= dl) incl = st_add(up, incl);
    }
    S e = st_shfl_up(incl, 1);
    if (lane == 0) e = st_zero<NS>();
    if (lane == 31) wtot[warp] = incl;
    __syncthreads();
    {
      S w = st_zero<NS>();
      for (int u = 0; u < warp; ++u) w = st_add(w, wtot[u]);
      e = st_add(w, e);
    }
    // ---- the tile's total, the chained look-back, the carry ----
    if (tid == 0) {
      S agg = wtot[0];
      for (int u = 1; u < NT / 32; ++u) agg = st_add(agg, wtot[u]);
      S excl = st_zero<NS>();
      if (chunk > 0) {
        const long long pred = tile - rows;
        if (wait_status(ws, pred, epoch) == kStatePrefix) excl = read_payload<S>(ws, pred, kStatePrefix);
        else record_error(ws.hdr, kLookbackTimeout, static_cast<unsigned>(tile));
      }
      if (chunk + 1 < tiles_per_row) publish(ws, tile, epoch, kStatePrefix, st_add(excl, agg));
      carry_smem = excl;
    }
    __syncthreads();
    // ---- replay from the state entering this thread's run ----
    S st = st_add(carry_smem, e);
    T res[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      df d[NS];
      int dc;
      if (CACHE) {
        const int sp = spad(q0 + k);
#pragma unroll
        for (int j = 0; j < NS; ++j) d[j] = sdl[j][sp];
        dc = sdc[sp];
      } else {
        delta(k, d, dc);
      }
#pragma unroll
      for (int j = 0; j < NS; ++j) st.s[j] = dfl::df_add_fast(st.s[j], d[j]);
      st.cnt += dc;
      res[k] = static_cast<T>(finalize_d<OP>(st, min_count));
    }
    const int bad = __syncthreads_or(ok ? 0 : 1);  // every thread has also read its run
#pragma unroll
    for (int k = 0; k < KT; ++k)
      sx[spad(q0 + k)] = sizeof(T) == 8 ? static_cast<B>(__double_as_longlong(static_cast<double>(res[k])))
                                        : static_cast<B>(__float_as_uint(static_cast<float>(res[k])));
    __syncthreads();
    B* ob = as_bits(out) + row * n;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      if (t0 + p < n) ob[t0 + p] = sx[spad(p)];
    }
    if (bad && tid == 0) atomicOr(row_flags + row, 1u);
    __syncthreads();  // the stage is reused by the next tile
  }
  if (tid == 0) finish_cta(ws.hdr);
}

// Ragged series (single-input statistics): three phases, since a chained scan would
// serialise the tiles of a long series.  Phase 0 folds each tile's differences into its
// total (aggs[tile]); dsc_carry_kernel scans every series' totals in order; phase 2
// replays each tile from carries[tile].  Tiles beyond the workspace's capacity flag their
// series for the exact kernel.
template <int OP, typename T, int PHASE>
__global__ void __launch_bounds__(NT) move_dtile_kernel(const T* __restrict__ a, T* __restrict__ out, Layout lay,
                                                        long long window, long long min_count,
                                                        St<Traits<OP>::NS>* __restrict__ aggs,
                                                        const St<Traits<OP>::NS>* __restrict__ carries,
                                                        long long capacity, const double* __restrict__ pivots,
                                                        unsigned* __restrict__ row_flags) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool VL = Traits<OP>::VARLIKE;
  static_assert(!Traits<OP>::TWO, "single-input statistics");
  typedef typename BitsOf<T>::type B;
  using S = St<NS>;
  using dfl::df;
  __shared__ B sx[SPAD], so[SPAD];
  __shared__ df sdl[NS][SPAD];
  __shared__ signed char sdc[SPAD];
  __shared__ S wtot[NT / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const B nanb = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  const long long items = layout_items(lay);
  const unsigned long long last_use = l2_evict_first();
  for (long long id = blockIdx.x; id < items; id += gridDim.x) {
    const Item it = layout_item(lay, id);
    const long long row = it.row, n = it.len;
    if (id >= capacity) {  // beyond the workspace: the exact kernel takes the series
      if (PHASE == 0 && tid == 0) atomicOr(row_flags + row, 1u);
      continue;
    }
    const long long t0 = it.index * TILE;
    const B* ar = as_bits(a) + it.base;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      const long long i = t0 + p;
      const bool in = i < n, old = in && i >= window;
      sx[spad(p)] = in ? ar[i] : nanb;
      so[spad(p)] = old ? ld_hint(ar + (i - window), last_use) : nanb;
    }
    __syncthreads();
    const Piv px = piv_of(VL ? pivots[2 * row] : 0.0);
    const int q0 = tid * KT;
    bool ok = true;
    S run = st_zero<NS>();
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      const int sp = spad(q0 + k);
      const B xi = sx[sp], xo = so[sp];
      df c[NS], d[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) d[j] = df{0.0f, 0.0f};
      int dc = 0;
      if (!nan_bits(xi)) {
        contrib<OP>(xi, xi, px, px, c, ok);
#pragma unroll
        for (int j = 0; j < NS; ++j) d[j] = c[j];
        dc = 1;
      }
      if (!nan_bits(xo)) {
        contrib<OP>(xo, xo, px, px, c, ok);
#pragma unroll
        for (int j = 0; j < NS; ++j) d[j] = dfl::df_add_fast(d[j], dfl::df_neg(c[j]));
        --dc;
      }
#pragma unroll
      for (int j = 0; j < NS; ++j) run.s[j] = dfl::df_add_fast(run.s[j], d[j]);
      run.cnt += dc;
      if (PHASE == 2) {
#pragma unroll
        for (int j = 0; j < NS; ++j) sdl[j][sp] = d[j];
        sdc[sp] = static_cast<signed char>(dc);
      }
    }
    S incl = run;
#pragma unroll
    for (int dl = 1; dl < 32; dl <<= 1) {
      const S up = st_shfl_up(incl, dl);
      if (lane >= dl) incl = st_add(up, incl);
    }
    S e = st_shfl_up(incl, 1);
    if (lane == 0) e = st_zero<NS>();
    if (lane == 31) wtot[warp] = incl;
    const int bad = __syncthreads_or(ok ? 0 : 1);
    if (PHASE == 0) {
      if (tid == 0) {
        S agg = wtot[0];
        for (int u = 1; u < NT / 32; ++u) agg = st_add(agg, wtot[u]);
        aggs[id] = agg;
        if (bad) atomicOr(row_flags + row, 1u);
      }
      __syncthreads();  // the stage is reused by the next tile
      continue;
    }
    {
      S w = carries[id];
      for (int u = 0; u < warp; ++u) w = st_add(w, wtot[u]);
      e = st_add(w, e);
    }
    S st = e;
    T res[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      const int sp = spad(q0 + k);
#pragma unroll
      for (int j = 0; j < NS; ++j) st.s[j] = dfl::df_add_fast(st.s[j], sdl[j][sp]);
      st.cnt += sdc[sp];
      res[k] = static_cast<T>(finalize_d<OP>(st, min_count));
    }
    __syncthreads();  // every thread has read its run
#pragma unroll
    for (int k = 0; k < KT; ++k)
      sx[spad(q0 + k)] = static_cast<B>(__double_as_longlong(static_cast<double>(res[k])));
    __syncthreads();
    B* ob = as_bits(out) + it.base;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      if (t0 + p < n) ob[t0 + p] = sx[spad(p)];
    }
    __syncthreads();
  }
}

// per series, the state entering each tile: its earlier tiles' totals added in order
template <int NS>
__global__ void dsc_carry_kernel(const St<NS>* __restrict__ aggs, St<NS>* __restrict__ carries,
                                 const long long* __restrict__ item_start, long long nseries, long long capacity) {
  const long long srs = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (srs >= nseries) return;
  const long long first = item_start[srs];
  const long long last = item_start[srs + 1] < capacity ? item_start[srs + 1] : capacity;
  St<NS> run = st_zero<NS>();
  for (long long t = first; t < last; ++t) {
    carries[t] = run;
    run = st_add(run, aggs[t]);
  }
}
}  // namespace dsc

// ---------------------------------------------------------------------------------
// Along a non-last axis: one thread per column
// ---------------------------------------------------------------------------------
// A C-contiguous array scanned along axis k is `outer` blocks of n x `inner` values:
// position p of column i of block o sits at (o n + p) inner + i.  Each thread owns one
// column and runs numbagg's loop down it with its float64 running sums, operation for
// operation (rounded multiplies, adds and divisions, never contracted into a multiply-
// add; float32 values widened to float64 as numba's float64 locals take them), so the
// results are the reference's bit for bit, infinities included.  Consecutive threads
// read consecutive addresses at every step, and nothing is copied or transposed.
NBG_DEVICE double ld_col(const double* p) { return __ldg(p); }
NBG_DEVICE double ld_col(const float* p) { return static_cast<double>(__ldg(p)); }
NBG_DEVICE bool isnan_d(double x) { return nan_bits(static_cast<unsigned long long>(__double_as_longlong(x))); }

template <int OP, typename T>
__global__ void __launch_bounds__(256) move_cols_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                        T* __restrict__ out, long long outer, long long n,
                                                        long long inner, long long window, long long min_count) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long col = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (col >= outer * inner) return;
  const long long o = col / inner, c = col - o * inner;
  const long long base = o * n * inner + c;
  const T* ac = a + base;
  const T* bc = Traits<OP>::TWO ? b + base : nullptr;
  T* oc = out + base;
  if (OP == kSum || OP == kMean) {  // numbagg/moving.py:12-55, :58-99
    const long long mc = OP == kMean ? (min_count > 1 ? min_count : 1) : min_count;
    double asum = 0.0;
    long long count = 0;
    const long long w0 = window < n ? window : n;
    for (long long p = 0; p < w0; ++p) {
      if (p + kColPrefetch < n) prefetch_l2(ac + (p + kColPrefetch) * inner);
      const double ai = ld_col(ac + p * inner);
      if (!isnan_d(ai)) {
        asum = __dadd_rn(asum, ai);
        ++count;
      }
      oc[p * inner] = static_cast<T>(count >= mc ? (OP == kMean ? __ddiv_rn(asum, static_cast<double>(count)) : asum) : nan);
    }
    for (long long p = window; p < n; ++p) {
      if (p + kColPrefetch < n) prefetch_l2(ac + (p + kColPrefetch) * inner);
      const double ai = ld_col(ac + p * inner);
      const double aold = ld_col(ac + (p - window) * inner);
      if (OP == kMean) {  // removes the old value first
        if (!isnan_d(aold)) {
          asum = __dsub_rn(asum, aold);
          --count;
        }
        if (!isnan_d(ai)) {
          asum = __dadd_rn(asum, ai);
          ++count;
        }
      } else {  // adds the new value first
        if (!isnan_d(ai)) {
          asum = __dadd_rn(asum, ai);
          ++count;
        }
        if (!isnan_d(aold)) {
          asum = __dsub_rn(asum, aold);
          --count;
        }
      }
      oc[p * inner] = static_cast<T>(count >= mc ? (OP == kMean ? __ddiv_rn(asum, static_cast<double>(count)) : asum) : nan);
    }
    return;
  }
  if (OP == kVar || OP == kStd) {  // numbagg/moving.py:123-181
    const long long mc = min_count > 2 ? min_count : 2;
    double asum = 0.0, asum_sq = 0.0;
    long long count = 0;
    for (long long p = 0; p < n; ++p) {
      if (p + kColPrefetch < n) prefetch_l2(ac + (p + kColPrefetch) * inner);
      const double ai = ld_col(ac + p * inner);
      if (p >= window) {
        const double aold = ld_col(ac + (p - window) * inner);
        if (!isnan_d(aold)) {
          asum = __dsub_rn(asum, aold);
          asum_sq = __dsub_rn(asum_sq, __dmul_rn(aold, aold));
          --count;
        }
      }
      if (!isnan_d(ai)) {
        asum = __dadd_rn(asum, ai);
        asum_sq = __dadd_rn(asum_sq, __dmul_rn(ai, ai));
        ++count;
      }
      double r = nan;
      if (count >= mc) {
        const double v = __ddiv_rn(__dsub_rn(asum_sq, __ddiv_rn(__dmul_rn(asum, asum), static_cast<double>(count))),
                                   static_cast<double>(count - 1));
        r = OP == kStd ? __dsqrt_rn(v) : v;
      }
      oc[p * inner] = static_cast<T>(r);
    }
    return;
  }
  // kCov / kCorr, numbagg/moving.py:184-275
  const long long mc = OP == kCov ? (min_count > 2 ? min_count : 2) : (min_count > 1 ? min_count : 1);
  double asum = 0.0, bsum = 0.0, prodsum = 0.0, asum_sq = 0.0, bsum_sq = 0.0;
  long long count = 0;
  for (long long p = 0; p < n; ++p) {
    if (p + kColPrefetch < n) {
      prefetch_l2(ac + (p + kColPrefetch) * inner);
      prefetch_l2(bc + (p + kColPrefetch) * inner);
    }
    const double ai = ld_col(ac + p * inner), bi = ld_col(bc + p * inner);
    if (p >= window) {
      const double aold = ld_col(ac + (p - window) * inner), bold = ld_col(bc + (p - window) * inner);
      if (!(isnan_d(aold) || isnan_d(bold))) {
        asum = __dsub_rn(asum, aold);
        bsum = __dsub_rn(bsum, bold);
        prodsum = __dsub_rn(prodsum, __dmul_rn(aold, bold));
        if (OP == kCorr) {
          asum_sq = __dsub_rn(asum_sq, __dmul_rn(aold, aold));
          bsum_sq = __dsub_rn(bsum_sq, __dmul_rn(bold, bold));
        }
        --count;
      }
    }
    if (!(isnan_d(ai) || isnan_d(bi))) {
      asum = __dadd_rn(asum, ai);
      bsum = __dadd_rn(bsum, bi);
      prodsum = __dadd_rn(prodsum, __dmul_rn(ai, bi));
      if (OP == kCorr) {
        asum_sq = __dadd_rn(asum_sq, __dmul_rn(ai, ai));
        bsum_sq = __dadd_rn(bsum_sq, __dmul_rn(bi, bi));
      }
      ++count;
    }
    double r = nan;
    if (count >= mc) {
      if (OP == kCov) {
        r = __ddiv_rn(__dsub_rn(prodsum, __ddiv_rn(__dmul_rn(asum, bsum), static_cast<double>(count))),
                      static_cast<double>(count - 1));
      } else {
        const double cr = __ddiv_rn(1.0, static_cast<double>(count));
        const double avg_a = __dmul_rn(asum, cr), avg_b = __dmul_rn(bsum, cr);
        const double var_a = __dsub_rn(__dmul_rn(asum_sq, cr), __dmul_rn(avg_a, avg_a));
        const double var_b = __dsub_rn(__dmul_rn(bsum_sq, cr), __dmul_rn(avg_b, avg_b));
        const double cov_ab = __dsub_rn(__dmul_rn(prodsum, cr), __dmul_rn(avg_a, avg_b));
        const double vv = __dmul_rn(var_a, var_b);
        if (vv > 0) r = __ddiv_rn(cov_ab, __dsqrt_rn(vv));
      }
    }
    oc[p * inner] = static_cast<T>(r);
  }
}

}  // namespace moving
}  // namespace nbg

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
using namespace nbg;
using namespace nbg::moving;

namespace {

long long dsc_tiles_per_row(long long n) { return n <= 0 ? 0 : (n + dsc::TILE - 1) / dsc::TILE; }

// the exact kernels' tables, then (rows x n calls) the double-float scan's look-back
// workspace, pivots and row flags
size_t move_scratch_bytes(long long rows, long long n) {
  size_t b = 256 + static_cast<size_t>(kRcpEntries + 1) * 8 + 256 + static_cast<size_t>(rows) * 8 + 256 +
             static_cast<size_t>(rows + 1) * 8;
  if (n > 0) b += 256 + workspace_bytes(rows * dsc_tiles_per_row(n)) + 256 + static_cast<size_t>(rows) * 16 + 256 +
                  static_cast<size_t>(rows) * 4;
  return b;
}

struct MoveScratch {
  double* rcp;
  long long* first_bad;
  long long* item_start;
  void* lb;  // look-back workspace of the double-float scan
  size_t lb_bytes;
  double* pivots;
  unsigned* flags;
};
MoveScratch carve_move(void* ws, long long rows, long long n = 0) {
  auto up = [](size_t p) { return (p + 255) & ~static_cast<size_t>(255); };
  MoveScratch m;
  size_t p = up(reinterpret_cast<size_t>(ws));
  m.rcp = reinterpret_cast<double*>(p);
  p = up(p + static_cast<size_t>(kRcpEntries + 1) * 8);
  m.first_bad = reinterpret_cast<long long*>(p);
  p = up(p + static_cast<size_t>(rows) * 8);
  m.item_start = reinterpret_cast<long long*>(p);
  p = up(p + static_cast<size_t>(rows + 1) * 8);
  m.lb = reinterpret_cast<void*>(p);
  m.lb_bytes = n > 0 ? workspace_bytes(rows * dsc_tiles_per_row(n)) : 0;
  p = up(p + m.lb_bytes);
  m.pivots = reinterpret_cast<double*>(p);
  p = up(p + static_cast<size_t>(rows) * 16);
  m.flags = reinterpret_cast<unsigned*>(p);
  return m;
}

// Chunks of at least 8 windows (the seed re-reads one window per chunk), 16 sub-tiles
// at least; smaller when the rows would not give four waves of two CTAs per SM.
long long default_chunk_len(long long window) {
  const long long w8 = (window > (LLONG_MAX / 16) ? LLONG_MAX / 16 : window) * 8;
  return std::max<long long>(16LL * SUB, ((w8 + SUB - 1) / SUB) * SUB);
}
long long chunk_len_for(long long rows, long long n, long long window) {
  long long len = default_chunk_len(window);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = 4LL * 2 * sms;
  while (len > SUB && rows * ((n + len - 1) / len) < want)
    len = std::max<long long>(SUB, ((len / 2 + SUB - 1) / SUB) * SUB);
  return len;
}

// Ragged series: the exact kernels' scratch, then pivots, flags, the tile plan and the
// double-float tile totals and carries (single-input statistics: at most two sums).
constexpr size_t kDscRaggedTileBytes = 2 * sizeof(dsc::St<2>);
size_t dsc_ragged_fixed_bytes(long long nseries) {
  return move_scratch_bytes(nseries, 0) + 256 + static_cast<size_t>(nseries) * 16 + 256 +
         static_cast<size_t>(nseries) * 4 + 256 + static_cast<size_t>(nseries + 1) * 8 + 256;
}
size_t move_ragged_scratch_bytes(long long nseries, long long total) {
  const long long tiles = total / dsc::TILE + nseries;
  return dsc_ragged_fixed_bytes(nseries) + static_cast<size_t>(tiles) * kDscRaggedTileBytes;
}

template <int OP, typename T>
int launch_dtile(const T* a, T* out, const long long* offsets, long long nseries, long long window,
                 long long min_count, const MoveScratch& sc, void* ws, size_t ws_bytes, cudaStream_t stream) {
  using S = dsc::St<Traits<OP>::NS>;
  auto up = [](size_t p) { return (p + 255) & ~static_cast<size_t>(255); };
  size_t p = up(reinterpret_cast<size_t>(sc.flags) + static_cast<size_t>(nseries) * 4);
  long long* tile_start = reinterpret_cast<long long*>(p);
  p = up(p + static_cast<size_t>(nseries + 1) * 8);
  const size_t end = reinterpret_cast<size_t>(ws) + ws_bytes;
  const long long capacity = end > p ? static_cast<long long>((end - p) / (2 * sizeof(S))) : 0;
  S* aggs = reinterpret_cast<S*>(p);
  S* carries = aggs + capacity;
  ragged_plan_kernel<<<1, 1024, 0, stream>>>(offsets, nseries, dsc::TILE, tile_start);
  if (Traits<OP>::VARLIKE)
    dsc::dsc_pivot_kernel<T><<<static_cast<int>((nseries * 32 + 255) / 256), 256, 0, stream>>>(a, nullptr, nseries, 0,
                                                                                             offsets, sc.pivots);
  Layout lay{offsets, tile_start, nseries, 0, 0};
  static int per_sm = 0;
  if (per_sm == 0) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, dsc::move_dtile_kernel<OP, T, 2>, dsc::NT, 0);
    per_sm = nb > 0 ? nb : 1;
  }
  const int grid = layout_grid(LLONG_MAX, per_sm);
  dsc::move_dtile_kernel<OP, T, 0><<<grid, dsc::NT, 0, stream>>>(a, out, lay, window, min_count, aggs, carries,
                                                                  capacity, sc.pivots, sc.flags);
  dsc::dsc_carry_kernel<Traits<OP>::NS><<<static_cast<int>((nseries + 255) / 256), 256, 0, stream>>>(
      aggs, carries, tile_start, nseries, capacity);
  dsc::move_dtile_kernel<OP, T, 2><<<grid, dsc::NT, 0, stream>>>(a, out, lay, window, min_count, aggs, carries,
                                                                  capacity, sc.pivots, sc.flags);
  return (Traits<OP>::VARLIKE ? 5 : 4);
}

// the double-float scan over rows x n (pivots first for the variance-like statistics)
template <int OP, typename T>
int launch_dscan(const T* a, const T* b, T* out, long long rows, long long n, long long window, long long min_count,
                 const MoveScratch& sc, cudaStream_t stream) {
  const long long tpr = dsc_tiles_per_row(n);
  const long long tiles = rows * tpr;
  if (cudaMemsetAsync(sc.lb, 0, 256 + static_cast<size_t>(tiles) * 8, stream) != cudaSuccess) return kLaunchError;
  if (Traits<OP>::VARLIKE)
    dsc::dsc_pivot_kernel<T><<<static_cast<int>((rows * 32 + 255) / 256), 256, 0, stream>>>(
        a, Traits<OP>::TWO ? b : nullptr, rows, n, nullptr, sc.pivots);
  static int per_sm = 0;  // resident CTAs per SM, from the occupancy calculator
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm == 0) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, dsc::move_dscan_kernel<OP, T>, dsc::NT, 0);
    per_sm = nb > 0 ? nb : 1;
  }
  const long long cap = static_cast<long long>(sms) * per_sm;
  const int grid = static_cast<int>(tiles < cap ? tiles : cap);
  dsc::move_dscan_kernel<OP, T><<<grid, dsc::NT, 0, stream>>>(a, b, out, rows, n, window, min_count, tpr, sc.lb,
                                                              sc.lb_bytes, sc.pivots, sc.flags);
  return kOk;
}

// offsets == nullptr: rows x n; else ragged series (n unused), chunk_len 0 = default
template <int OP, typename T, bool C>
int launch_move(const T* a, const T* b, T* out, const long long* offsets, long long rows, long long n,
                long long window, long long min_count, long long chunk_len, void* ws, size_t ws_bytes,
                cudaStream_t stream) {
  if (rows < 0 || n < 0 || window <= 0 || min_count < 0 || chunk_len < 0) return kInvalidArgument;
  if (rows == 0 || (!offsets && n == 0)) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b)) return kInvalidArgument;
  // the compensated form over rows runs the double-float scan first (float64 arrays)
  constexpr bool kDsc = C && sizeof(T) == 8;
  // ragged single-input series take the three-phase double-float scan when the scratch
  // holds its tile plan (nbg_move_ragged_workspace_bytes), else the exact kernel alone
  // (windows below 2^24 keep the double-float window sums inside float32's range for the
  // value ranges the scan accepts; longer ones take the exact kernel)
  const bool dtile = kDsc && offsets && !Traits<OP>::TWO && window < (1ll << 24) &&
                     ws_bytes >= dsc_ragged_fixed_bytes(rows) + kDscRaggedTileBytes;
  const bool dsc = (kDsc && !offsets && window < (1ll << 24)) || dtile;
  if (!ws || ws_bytes < move_scratch_bytes(rows, (kDsc && !offsets) ? n : 0)) return kWorkspaceTooSmall;
  const MoveScratch sc = carve_move(ws, rows, (kDsc && !offsets) ? n : 0);
  const long long rcp_n = std::min<long long>(window, kRcpEntries);
  Layout lay{offsets, sc.item_start, rows, n, 0};
  long long len;
  int launches = 3;
  long long grid_items;
  if (!offsets) {
    len = chunk_len ? ((chunk_len + SUB - 1) / SUB) * SUB : chunk_len_for(rows, n, window);
    lay.items_per_row = (n + len - 1) / len;
    grid_items = rows * lay.items_per_row;
  } else {
    len = chunk_len ? ((chunk_len + SUB - 1) / SUB) * SUB : default_chunk_len(window);
    ragged_plan_kernel<<<1, 1024, 0, stream>>>(offsets, rows, len, sc.item_start);
    ++launches;
    grid_items = LLONG_MAX;
  }
  const long long setup_items = std::max(rcp_n + 1, rows);
  move_setup_kernel<<<static_cast<int>(std::min<long long>((setup_items + 255) / 256, 1024)), 256, 0, stream>>>(
      sc.rcp, rcp_n, sc.first_bad, rows, dsc ? sc.flags : nullptr);
  if constexpr (kDsc) {
    if (dsc && !offsets) {  // rows x n
      const int r = launch_dscan<OP, T>(a, b, out, rows, n, window, min_count, sc, stream);
      if (r != kOk) return r;
      launches += Traits<OP>::VARLIKE ? 2 : 1;
    } else if (dtile) {
      if constexpr (!Traits<OP>::TWO) launches += launch_dtile<OP, T>(a, out, offsets, rows, window, min_count, sc, ws,
                                                                      ws_bytes, stream);
    }
  }
  const size_t smem = static_cast<size_t>(Traits<OP>::TWO ? 4 : 2) * SPAD * sizeof(typename BitsOf<T>::type);
  auto kern = move_kernel<OP, T, C>;
  // the shared-memory opt-in is per device, so it is set on every call
  if (smem > 32 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  // the persistent grid: as many CTAs as can be resident at once (a CTA beyond that
  // would wait for a slot and run as a tail)
  static const int per_sm = [&] {
    int r = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, NT, smem) != cudaSuccess || r < 1) r = 2;
    return r;
  }();
  // after the double-float scan this recomputes only the rows it flagged
  kern<<<layout_grid(grid_items, per_sm), NT, smem, stream>>>(a, b, out, lay, window, min_count, len, sc.rcp, rcp_n,
                                                              sc.first_bad, dsc ? sc.flags : nullptr);
  move_poison_kernel<T, Traits<OP>::VARLIKE><<<static_cast<int>(std::min<long long>(rows, 4096)), 256, 0, stream>>>(
      out, lay, window, sc.first_bad);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

template <int OP, typename T>
int launch_move_cols(const T* a, const T* b, T* out, long long outer, long long n, long long inner, long long window,
                     long long min_count, cudaStream_t s) {
  if (outer < 0 || n < 0 || inner < 0 || window <= 0 || min_count < 0) return kInvalidArgument;
  if (outer == 0 || n == 0 || inner == 0) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b)) return kInvalidArgument;
  const long long blocks = (outer * inner + 255) / 256;
  if (blocks > 0x7fffffffLL) return kUnsupported;
  move_cols_kernel<OP, T><<<static_cast<int>(blocks), 256, 0, s>>>(a, b, out, outer, n, inner, window, min_count);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_move_workspace_bytes(long long rows, long long n) { return move_scratch_bytes(rows, n); }
size_t nbg_move_ragged_workspace_bytes(long long nseries, long long total) {
  return nseries < 0 || total < 0 ? 0 : move_ragged_scratch_bytes(nseries, total);
}

#define NBG_MOVE1(NAME, OPC, T, SFX, C)                                                        \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long n, long long window,  \
                         long long min_count, void* ws, size_t ws_bytes, void* stream) {     \
    return launch_move<OPC, T, C>(a, nullptr, out, nullptr, rows, n, window, min_count, 0, ws, ws_bytes, \
                               static_cast<cudaStream_t>(stream));                          \
  }
#define NBG_MOVE2(NAME, OPC, T, SFX, C)                                                        \
  int nbg_##NAME##_##SFX(const T* a, const T* b, T* out, long long rows, long long n,        \
                         long long window, long long min_count, void* ws, size_t ws_bytes,   \
                         void* stream) {                                                    \
    return launch_move<OPC, T, C>(a, b, out, nullptr, rows, n, window, min_count, 0, ws, ws_bytes, \
                               static_cast<cudaStream_t>(stream));                          \
  }

NBG_MOVE1(move_sum, kSum, double, f64, false)
NBG_MOVE1(move_sum, kSum, float, f32, false)
NBG_MOVE1(move_mean, kMean, double, f64, false)
NBG_MOVE1(move_mean, kMean, float, f32, false)
NBG_MOVE1(move_var, kVar, double, f64, false)
NBG_MOVE1(move_var, kVar, float, f32, false)
NBG_MOVE1(move_std, kStd, double, f64, false)
NBG_MOVE1(move_std, kStd, float, f32, false)
NBG_MOVE2(move_cov, kCov, double, f64, false)
NBG_MOVE2(move_cov, kCov, float, f32, false)
NBG_MOVE2(move_corr, kCorr, double, f64, false)
NBG_MOVE2(move_corr, kCorr, float, f32, false)
// FP32-compensated forms (float64 arrays): the same exact window sums, finalised in
// scaled double-float (no reference counterpart; numbagg computes in float64 only)
NBG_MOVE1(move_sum, kSum, double, f64_fp32c, true)
NBG_MOVE1(move_mean, kMean, double, f64_fp32c, true)
NBG_MOVE1(move_var, kVar, double, f64_fp32c, true)
NBG_MOVE1(move_std, kStd, double, f64_fp32c, true)
NBG_MOVE2(move_cov, kCov, double, f64_fp32c, true)
NBG_MOVE2(move_corr, kCorr, double, f64_fp32c, true)

// Along a non-last axis of a C-contiguous array: `outer` blocks of n x `inner` values,
// scanned along n, one thread per column running numbagg's loop (move_cols_kernel).
#define NBG_MOVE1_COLS(NAME, OPC, T, SFX)                                                         \
  int nbg_##NAME##_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner,   \
                              long long window, long long min_count, void* stream) {               \
    return launch_move_cols<OPC, T>(a, nullptr, out, outer, n, inner, window, min_count,            \
                                    static_cast<cudaStream_t>(stream));                             \
  }
#define NBG_MOVE2_COLS(NAME, OPC, T, SFX)                                                         \
  int nbg_##NAME##_cols_##SFX(const T* a, const T* b, T* out, long long outer, long long n,        \
                              long long inner, long long window, long long min_count, void* stream) { \
    return launch_move_cols<OPC, T>(a, b, out, outer, n, inner, window, min_count,                  \
                                    static_cast<cudaStream_t>(stream));                             \
  }
NBG_MOVE1_COLS(move_sum, kSum, double, f64)
NBG_MOVE1_COLS(move_sum, kSum, float, f32)
NBG_MOVE1_COLS(move_mean, kMean, double, f64)
NBG_MOVE1_COLS(move_mean, kMean, float, f32)
NBG_MOVE1_COLS(move_var, kVar, double, f64)
NBG_MOVE1_COLS(move_var, kVar, float, f32)
NBG_MOVE1_COLS(move_std, kStd, double, f64)
NBG_MOVE1_COLS(move_std, kStd, float, f32)
NBG_MOVE2_COLS(move_cov, kCov, double, f64)
NBG_MOVE2_COLS(move_cov, kCov, float, f32)
NBG_MOVE2_COLS(move_corr, kCorr, double, f64)
NBG_MOVE2_COLS(move_corr, kCorr, float, f32)

// Ragged series: series s is values[offsets[s] : offsets[s + 1]] (nseries + 1 offsets,
// on the device), out has the same layout; chunk_len 0 picks the default.
#define NBG_MOVE_RAGGED(NAME, OPC, SFX, C)                                                      \
  int nbg_##NAME##_ragged_##SFX(const double* values, const long long* offsets, long long nseries, \
                                double* out, long long window, long long min_count,             \
                                long long chunk_len, void* ws, size_t ws_bytes, void* stream) {  \
    return launch_move<OPC, double, C>(values, nullptr, out, offsets, nseries, 0, window, min_count, \
                                       chunk_len, ws, ws_bytes, static_cast<cudaStream_t>(stream)); \
  }
NBG_MOVE_RAGGED(move_sum, kSum, f64, false)
NBG_MOVE_RAGGED(move_mean, kMean, f64, false)
NBG_MOVE_RAGGED(move_var, kVar, f64, false)
NBG_MOVE_RAGGED(move_std, kStd, f64, false)
NBG_MOVE_RAGGED(move_sum, kSum, f64_fp32c, true)
NBG_MOVE_RAGGED(move_mean, kMean, f64_fp32c, true)
NBG_MOVE_RAGGED(move_var, kVar, f64_fp32c, true)
NBG_MOVE_RAGGED(move_std, kStd, f64_fp32c, true)

}  // extern "C"
