// Exponentially weighted family move_exp_nan{count,mean,sum,var,std,cov,corr}
// (numbagg/moving_exp.py:12-335), float64 and float32 arrays, plus FP32-compensated
// ("fp32c") forms of the float64 entry points.
//
// Each reference state variable follows s_i = decay_i * s_{i-1} + b_i, where
// decay_i = 1 - alpha_i and b_i is the contribution of position i (zero when the
// value is NaN); sum_weight_2 decays by decay_i**2.  A position is therefore an
// affine map s -> A*s + B, and maps compose associatively:
//     (A2, B2) o (A1, B1) = (A2*A1, A2*B1 + B2).
// A row is cut into tiles of 1024 positions.  Phase 0 composes each tile's map
// (thread-serial over 8 consecutive positions, then a fixed-structure warp-shuffle
// scan); phase 1 scans the tile maps of each row in a fixed order to get the state
// entering every tile; phase 2 replays each position with the reference's update (a
// rounded multiply followed by a rounded add, no FMA) from that state, and finalises
// with the reference's formulas.  The composition order never depends on timing, so
// results are bit-identical run to run and a prefix of a row gives the same bits as
// the whole row.  Values, alphas and outputs pass through a padded shared stage so
// that every global access of a warp is one contiguous run.
//
// The arithmetic is a policy: F64 is the reference's float64 (bound by this GPU's
// FP64 pipe, one warp instruction per 16 cycles); DF is double-float on the FP32
// pipes (dfloat.cuh, about 48 bits).  The DF forms of the shift-invariant statistics
// (variance, standard deviation, covariance, correlation) first subtract a per-row
// pivot, the row's first finite value, from every value, so data such as 1e6 + N(0,1)
// keeps its significant digits; the mean and the sums need no pivot.
//
// alpha: a scalar, a 1-D array along the scanned axis shared by every row, or one
// value per element (numbagg/decorators.py:398-409).
#include "dfloat.cuh"

#include <algorithm>
#include <climits>

namespace nbg {
namespace mexp {

enum Op : int {
  kCount = 0, kMean, kSum, kVar, kStd, kCov, kCorr,
  // The one-pass scan (a scalar alpha): the reference's `weight` state, the sum of
  // alpha * decay^k over the valid positions, is then alpha times the sum of the
  // weights decay^k that the statistic scans anyway, so it is not scanned.  Same
  // statistics, one state fewer (move_exp_nansum keeps its two states).
  kCountW, kMeanW, kVarW, kStdW, kCovW, kCorrW
};

template <int OP>
struct Traits;
// state order and decay kind per op; W2 marks the sum_weight_2 state (decay**2)
template <>
struct Traits<kCount> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr int W2 = -1; static constexpr bool PIVOT = false; };
template <>
struct Traits<kMean> { static constexpr int NS = 3; static constexpr bool TWO = false; static constexpr int W2 = -1; static constexpr bool PIVOT = false; };
template <>
struct Traits<kSum> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr int W2 = -1; static constexpr bool PIVOT = false; };
template <>
struct Traits<kVar> { static constexpr int NS = 5; static constexpr bool TWO = false; static constexpr int W2 = 3; static constexpr bool PIVOT = true; };
template <>
struct Traits<kStd> { static constexpr int NS = 5; static constexpr bool TWO = false; static constexpr int W2 = 3; static constexpr bool PIVOT = true; };
template <>
struct Traits<kCov> { static constexpr int NS = 6; static constexpr bool TWO = true; static constexpr int W2 = 4; static constexpr bool PIVOT = true; };
template <>
struct Traits<kCorr> { static constexpr int NS = 8; static constexpr bool TWO = true; static constexpr int W2 = 4; static constexpr bool PIVOT = true; };
template <>
struct Traits<kCountW> { static constexpr int NS = 1; static constexpr bool TWO = false; static constexpr int W2 = -1; static constexpr bool PIVOT = false; };
template <>
struct Traits<kMeanW> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr int W2 = -1; static constexpr bool PIVOT = false; };
template <>
struct Traits<kVarW> { static constexpr int NS = 4; static constexpr bool TWO = false; static constexpr int W2 = 3; static constexpr bool PIVOT = true; };
template <>
struct Traits<kStdW> { static constexpr int NS = 4; static constexpr bool TWO = false; static constexpr int W2 = 3; static constexpr bool PIVOT = true; };
template <>
struct Traits<kCovW> { static constexpr int NS = 5; static constexpr bool TWO = true; static constexpr int W2 = 4; static constexpr bool PIVOT = true; };
template <>
struct Traits<kCorrW> { static constexpr int NS = 7; static constexpr bool TWO = true; static constexpr int W2 = 4; static constexpr bool PIVOT = true; };

// the statistic an op computes, and the op the one-pass scan runs for it
NBG_HOST_DEVICE constexpr int base_op(int op) {
  return op == kCountW ? kCount : op == kMeanW ? kMean : op == kVarW ? kVar : op == kStdW ? kStd
       : op == kCovW ? kCov : op == kCorrW ? kCorr : op;
}
NBG_HOST_DEVICE constexpr int scan_op(int op) {
  return op == kCount ? kCountW : op == kMean ? kMeanW : op == kVar ? kVarW : op == kStd ? kStdW
       : op == kCov ? kCovW : op == kCorr ? kCorrW : op;
}

// ---------------------------------------------------------------------------------
// arithmetic policies
// ---------------------------------------------------------------------------------
struct F64 {
  typedef double T;
  static constexpr bool kDF = false;
  static NBG_DEVICE T zero() { return 0.0; }
  static NBG_DEVICE T one() { return 1.0; }
  static NBG_DEVICE T mul(T a, T b) { return __dmul_rn(a, b); }
  static NBG_DEVICE T add(T a, T b) { return __dadd_rn(a, b); }
  static NBG_DEVICE T sub(T a, T b) { return __dsub_rn(a, b); }
  static NBG_DEVICE T fma(T a, T b, T c) { return ::fma(a, b, c); }
};


NBG_DEVICE double df_to_f64(dfl::df x) {
  const unsigned hb = static_cast<unsigned>(__float_as_int(x.hi));
  if (((hb >> 23) & 0xff) == 0xff) {  // inf or NaN
    const unsigned long long s = static_cast<unsigned long long>(hb >> 31) << 63;
    return __longlong_as_double(static_cast<long long>(s | 0x7ff0000000000000ull | ((hb & 0x7fffffu) ? (1ull << 51) : 0ull)));
  }
  if ((hb & 0x7fffffffu) == 0) return x.lo == 0.0f ? __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(hb >> 31) << 63)) : static_cast<double>(x.lo);
  return dfl::sdf_to_f64(dfl::sdf_norm(x, 0));
}

struct DF {
  typedef dfl::df T;
  static constexpr bool kDF = true;
  static NBG_DEVICE T zero() { return dfl::df{0.0f, 0.0f}; }
  static NBG_DEVICE T one() { return dfl::df{1.0f, 0.0f}; }
  static NBG_DEVICE T mul(T a, T b) { return dfl::df_mul(a, b); }
  static NBG_DEVICE T add(T a, T b) { return dfl::df_add(a, b); }
  static NBG_DEVICE T sub(T a, T b) { return dfl::df_sub(a, b); }
  // the decayed recurrences' multiply-add: the product plus the cheaper sum (about
  // 2^-44 of the terms' magnitudes, far inside the compensated form's bound)
  static NBG_DEVICE T fma(T a, T b, T c) { return dfl::df_add_fast(dfl::df_mul(a, b), c); }
};

// a value of the array as the policy's number (float64 policy: exact widening)
NBG_DEVICE double value_as(F64, unsigned long long bits) { return __longlong_as_double(static_cast<long long>(bits)); }
NBG_DEVICE double value_as(F64, unsigned bits) { return static_cast<double>(__int_as_float(static_cast<int>(bits))); }
NBG_DEVICE dfl::df value_as(DF, unsigned long long bits) { return df_from_f64(__longlong_as_double(static_cast<long long>(bits))); }
NBG_DEVICE dfl::df value_as(DF, unsigned bits) { return dfl::df{__int_as_float(static_cast<int>(bits)), 0.0f}; }
NBG_DEVICE double as_f64(double x) { return x; }
NBG_DEVICE double as_f64(dfl::df x) { return df_to_f64(x); }
NBG_DEVICE dfl::df as_num(DF, double x) { return df_from_f64(x); }
NBG_DEVICE double as_num(F64, double x) { return x; }

template <int NS, typename N>
struct Map {
  typename N::T A1, A2;  // product of decays, product of squared decays
  typename N::T B[NS];
  int seen;  // any valid value (move_exp_nansum's zero_count flag)
  int pad;
};

template <int OP, typename N>
NBG_DEVICE Map<Traits<OP>::NS, N> identity_map() {
  Map<Traits<OP>::NS, N> m;
  m.A1 = N::one();
  m.A2 = N::one();
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) m.B[j] = N::zero();
  m.seen = 0;
  m.pad = 0;
  return m;
}

// later o earlier
template <int OP, typename N>
NBG_DEVICE Map<Traits<OP>::NS, N> compose(const Map<Traits<OP>::NS, N>& earlier, const Map<Traits<OP>::NS, N>& later) {
  Map<Traits<OP>::NS, N> r;
  r.A1 = N::mul(later.A1, earlier.A1);
  r.A2 = N::mul(later.A2, earlier.A2);
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) {
    const typename N::T a = (j == Traits<OP>::W2) ? later.A2 : later.A1;
    r.B[j] = N::fma(a, earlier.B[j], later.B[j]);
  }
  r.seen = earlier.seen | later.seen;
  r.pad = 0;
  return r;
}

NBG_DEVICE double shfl_up_num(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
NBG_DEVICE dfl::df shfl_up_num(dfl::df v, int d) {
  return dfl::df{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}

template <int OP, typename N>
NBG_DEVICE Map<Traits<OP>::NS, N> shfl_up_map(const Map<Traits<OP>::NS, N>& v, int d) {
  Map<Traits<OP>::NS, N> r;
  r.A1 = shfl_up_num(v.A1, d);
  r.A2 = shfl_up_num(v.A2, d);
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) r.B[j] = shfl_up_num(v.B[j], d);
  r.seen = __shfl_up_sync(0xffffffffu, v.seen, d);
  r.pad = 0;
  return r;
}

// contributions b_j of one position, in the reference's state order
template <int OP, typename N>
NBG_DEVICE void contributions(typename N::T x, typename N::T y, typename N::T alpha, typename N::T* b) {
  const typename N::T one = N::one();
  if (OP == kCount) {  // count, weight
    b[0] = one; b[1] = alpha;
  } else if (OP == kMean) {  // numer, denom, weight
    b[0] = x; b[1] = one; b[2] = alpha;
  } else if (OP == kSum) {  // numer, weight
    b[0] = x; b[1] = alpha;
  } else if (OP == kVar || OP == kStd) {  // sum_x_2, sum_x, sum_weight, sum_weight_2, weight
    b[0] = N::mul(x, x); b[1] = x; b[2] = one; b[3] = one; b[4] = alpha;
  } else if (OP == kCov) {  // sum_x1, sum_x2, sum_x1x2, sum_weight, sum_weight_2, weight
    b[0] = x; b[1] = y; b[2] = N::mul(x, y); b[3] = one; b[4] = one; b[5] = alpha;
  } else if (OP == kCorr) {  // + sum_x1_2, sum_x2_2
    b[0] = x; b[1] = y; b[2] = N::mul(x, y); b[3] = one; b[4] = one; b[5] = alpha;
    b[6] = N::mul(x, x); b[7] = N::mul(y, y);
  } else if (OP == kCountW) {  // the same without the weight
    b[0] = one;
  } else if (OP == kMeanW) {
    b[0] = x; b[1] = one;
  } else if (OP == kVarW || OP == kStdW) {
    b[0] = N::mul(x, x); b[1] = x; b[2] = one; b[3] = one;
  } else if (OP == kCovW) {
    b[0] = x; b[1] = y; b[2] = N::mul(x, y); b[3] = one; b[4] = one;
  } else {  // kCorrW
    b[0] = x; b[1] = y; b[2] = N::mul(x, y); b[3] = one; b[4] = one;
    b[5] = N::mul(x, x); b[6] = N::mul(y, y);
  }
}

// The reference's full state from a weightless one: weight = alpha * sum_weight
// (the count for move_exp_nancount, the denominator for the mean).
template <int OP, typename N>
NBG_DEVICE void with_weight(const typename N::T* s, typename N::T alpha, typename N::T* f) {
  if (OP == kCountW) {
    f[0] = s[0]; f[1] = N::mul(alpha, s[0]);
  } else if (OP == kMeanW) {
    f[0] = s[0]; f[1] = s[1]; f[2] = N::mul(alpha, s[1]);
  } else if (OP == kVarW || OP == kStdW) {
    f[0] = s[0]; f[1] = s[1]; f[2] = s[2]; f[3] = s[3]; f[4] = N::mul(alpha, s[2]);
  } else if (OP == kCovW) {
#pragma unroll
    for (int j = 0; j < 5; ++j) f[j] = s[j];
    f[5] = N::mul(alpha, s[3]);
  } else if (OP == kCorrW) {
#pragma unroll
    for (int j = 0; j < 5; ++j) f[j] = s[j];
    f[5] = N::mul(alpha, s[3]);
    f[6] = s[5]; f[7] = s[6];
  } else {
#pragma unroll
    for (int j = 0; j < Traits<OP>::NS; ++j) f[j] = s[j];
  }
}

template <int OP>
NBG_DEVICE double finalize(F64, const double* s, int seen, double min_weight) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (OP == kCount) return s[1] >= min_weight ? s[0] : nan;
  if (OP == kMean) return s[2] >= min_weight ? __ddiv_rn(s[0], s[1]) : nan;
  if (OP == kSum) return (s[1] >= min_weight && seen) ? s[0] : nan;
  if (OP == kVar || OP == kStd) {
    // numbagg/moving_exp.py:142-156
    const double m = __ddiv_rn(s[1], s[2]);
    const double var_biased = __dadd_rn(__ddiv_rn(s[0], s[2]), -__dmul_rn(m, m));
    const double bias = __dadd_rn(1.0, -__ddiv_rn(s[3], __dmul_rn(s[2], s[2])));
    if (s[4] >= min_weight && bias > 0) {
      const double v = __ddiv_rn(var_biased, bias);
      return OP == kStd ? __dsqrt_rn(v) : v;
    }
    return nan;
  }
  if (OP == kCov) {
    // numbagg/moving_exp.py:265-273
    const double cov_biased =
        __ddiv_rn(__dadd_rn(s[2], -__ddiv_rn(__dmul_rn(s[0], s[1]), s[3])), s[3]);
    const double bias = __dadd_rn(1.0, -__ddiv_rn(s[4], __dmul_rn(s[3], s[3])));
    return (s[5] >= min_weight && bias > 0) ? __ddiv_rn(cov_biased, bias) : nan;
  }
  // kCorr, numbagg/moving_exp.py:318-335
  const double cov = __dadd_rn(s[2], -__ddiv_rn(__dmul_rn(s[0], s[1]), s[3]));
  const double var1 = __dadd_rn(s[6], -__ddiv_rn(__dmul_rn(s[0], s[0]), s[3]));
  const double var2 = __dadd_rn(s[7], -__ddiv_rn(__dmul_rn(s[1], s[1]), s[3]));
  const double bias = __dadd_rn(1.0, -__ddiv_rn(s[4], __dmul_rn(s[3], s[3])));
  if (s[5] >= min_weight && bias > 0) {
    const double den = __dsqrt_rn(__dmul_rn(var1, var2));
    return den > 0 ? __ddiv_rn(cov, den) : nan;
  }
  return nan;
}

// double-float comparisons
NBG_DEVICE bool df_pos(dfl::df x) { return x.hi > 0.0f || (x.hi == 0.0f && x.lo > 0.0f); }
NBG_DEVICE bool df_ge(dfl::df x, double y) {  // x >= y (y a float64 constant of the call)
  const dfl::df d = dfl::df_sub(x, df_from_f64(y));
  return d.hi > 0.0f || (d.hi == 0.0f && d.lo >= 0.0f);
}
NBG_DEVICE dfl::df df_div0(dfl::df x, dfl::df y) {  // x / y with IEEE zeros, infinities and NaN
  if (y.hi == 0.0f || !isfinite(y.hi) || !isfinite(x.hi)) return dfl::df{__fdiv_rn(x.hi, y.hi), 0.0f};
  if (x.hi == 0.0f) return dfl::df{0.0f, 0.0f};
  return dfl::df_div(x, y);
}

// The reference's formulas in double-float (the statistics that see pivoted values are
// invariant under the shift).
template <int OP>
NBG_DEVICE double finalize(DF, const dfl::df* s, int seen, double min_weight) {
  using namespace dfl;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const df one{1.0f, 0.0f};
  if (OP == kCount) return df_ge(s[1], min_weight) ? df_to_f64(s[0]) : nan;
  if (OP == kMean) return df_ge(s[2], min_weight) ? df_to_f64(df_div0(s[0], s[1])) : nan;
  if (OP == kSum) return (df_ge(s[1], min_weight) && seen) ? df_to_f64(s[0]) : nan;
  if (OP == kVar || OP == kStd) {
    const df m = df_div0(s[1], s[2]);
    const df var_biased = df_sub(df_div0(s[0], s[2]), df_mul(m, m));
    const df bias = df_sub(one, df_div0(s[3], df_mul(s[2], s[2])));
    if (df_ge(s[4], min_weight) && df_pos(bias)) {
      const df v = df_div0(var_biased, bias);
      if (OP == kVar) return df_to_f64(v);
      if (v.hi < 0.0f) return nan;
      return v.hi == 0.0f ? 0.0 : df_to_f64(df_sqrt(v));
    }
    return nan;
  }
  if (OP == kCov) {
    const df cov_biased = df_div0(df_sub(s[2], df_div0(df_mul(s[0], s[1]), s[3])), s[3]);
    const df bias = df_sub(one, df_div0(s[4], df_mul(s[3], s[3])));
    return (df_ge(s[5], min_weight) && df_pos(bias)) ? df_to_f64(df_div0(cov_biased, bias)) : nan;
  }
  const df cov = df_sub(s[2], df_div0(df_mul(s[0], s[1]), s[3]));
  const df var1 = df_sub(s[6], df_div0(df_mul(s[0], s[0]), s[3]));
  const df var2 = df_sub(s[7], df_div0(df_mul(s[1], s[1]), s[3]));
  const df bias = df_sub(one, df_div0(s[4], df_mul(s[3], s[3])));
  if (df_ge(s[5], min_weight) && df_pos(bias)) {
    const df vv = df_mul(var1, var2);
    if (!df_pos(vv)) return nan;
    return df_to_f64(df_div0(cov, df_sqrt(vv)));
  }
  return nan;
}

constexpr int NT = 128;
constexpr int KT = 8;
constexpr int TILE = NT * KT;
constexpr int SPAD = TILE + TILE / KT;
NBG_DEVICE int spad(int p) { return p + p / KT; }

template <int OP>
NBG_DEVICE double finalize_dfast(const dfl::df* s, int seen, dfl::df mw);

// Phase 0 (PHASE == 0): the map of each tile, composed in position order, to maps[].
// Phase 2 (PHASE == 2): outputs, starting from the state carries[tile] before the tile.
// One CTA per tile; tiles do not wait on each other.
template <int OP, typename T, typename N, int PHASE>
__global__ void __launch_bounds__(NT) exp_tile_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                      const T* __restrict__ alpha_arr, double alpha_scalar,
                                                      int alpha_mode, double min_weight,
                                                      T* __restrict__ out, Layout lay,
                                                      Map<Traits<OP>::NS, N>* maps,
                                                      const Map<Traits<OP>::NS, N>* carries,
                                                      const double* __restrict__ pivots) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool TWO = Traits<OP>::TWO;
  constexpr bool SHIFT = Traits<OP>::PIVOT && N::kDF;
  typedef typename BitsOf<T>::type B;
  typedef typename N::T V;
  using M = Map<NS, N>;
  __shared__ M warp_tot[NT / 32];
  __shared__ B sx[SPAD];
  __shared__ B sy[TWO ? SPAD : 1];
  __shared__ B sa[SPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const B nanb = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  const long long items = layout_items(lay);
  // a persistent grid walks the tiles (of rows, or of ragged series)
  for (long long tile = blockIdx.x; tile < items; tile += gridDim.x) {
  const Item it = layout_item(lay, tile);
  const long long row = it.row, n = it.len;
  const long long t0 = it.index * TILE;
  const B* ar = as_bits(a) + it.base;
  const B* br = TWO ? as_bits(b) + it.base : nullptr;
  const B* alr = alpha_mode == 2 ? as_bits(alpha_arr) + it.base : as_bits(alpha_arr);

  // ---- stage the tile (coalesced), then each thread takes 8 consecutive positions ----
#pragma unroll
  for (int j = 0; j < KT; ++j) {
    const int p = j * NT + tid;
    const long long i = t0 + p;
    const bool in = i < n;
    sx[spad(p)] = in ? ar[i] : nanb;
    if (TWO) sy[spad(p)] = in ? br[i] : nanb;
    if (alpha_mode != 0) sa[spad(p)] = in ? alr[i] : B(0);
  }
  __syncthreads();
  V px = N::zero(), py = N::zero();
  if (SHIFT) {
    px = as_num(N(), pivots[2 * row]);
    if (TWO) py = as_num(N(), pivots[2 * row + 1]);
  }
  const V al_s = as_num(N(), alpha_scalar);
  const V d_s = N::sub(N::one(), al_s);
  const V dd_s = N::mul(d_s, d_s);
  const dfl::df mw_df = df_from_f64(min_weight);
  const int q0 = tid * KT;

  auto position = [&](int k, V& x, V& y, V& al, V& d, V& dd, bool& valid, bool& in) {
    const int sp = spad(q0 + k);
    in = t0 + q0 + k < n;
    const B xb = sx[sp];
    const B yb = TWO ? sy[sp] : xb;
    valid = in && !nan_bits(xb) && !(TWO && nan_bits(yb));
    x = value_as(N(), xb);
    y = TWO ? value_as(N(), yb) : x;
    if (SHIFT) {
      x = N::sub(x, px);
      if (TWO) y = N::sub(y, py);
    }
    if (alpha_mode == 0) {
      al = al_s;
      d = d_s;
      dd = dd_s;
    } else {
      al = value_as(N(), sa[sp]);
      d = N::sub(N::one(), al);
      dd = N::mul(d, d);
    }
  };

  // ---- this thread's maps composed in order ----
  M agg = identity_map<OP, N>();
#pragma unroll
  for (int k = 0; k < KT; ++k) {
    V x, y, al, d, dd;
    bool valid, in;
    position(k, x, y, al, d, dd, valid, in);
    if (!in) break;
    V bj[NS];
    contributions<OP, N>(x, y, al, bj);
    agg.A1 = N::mul(agg.A1, d);
    agg.A2 = N::mul(agg.A2, dd);
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const V f = (j == Traits<OP>::W2) ? dd : d;
      agg.B[j] = valid ? N::fma(agg.B[j], f, bj[j]) : N::mul(agg.B[j], f);
    }
    agg.seen |= valid ? 1 : 0;
  }
  // ---- block scan (fixed structure, so the result does not depend on timing) ----
  M incl = agg;
#pragma unroll
  for (int dlt = 1; dlt < 32; dlt <<= 1) {
    const M up = shfl_up_map<OP, N>(incl, dlt);
    if (lane >= dlt) incl = compose<OP, N>(up, incl);
  }
  M excl = shfl_up_map<OP, N>(incl, 1);
  if (lane == 0) excl = identity_map<OP, N>();
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (tid == 0) {
    M run = warp_tot[0];
    for (int w = 1; w < NT / 32; ++w) {
      run = compose<OP, N>(run, warp_tot[w]);
      warp_tot[w] = run;
    }
  }
  __syncthreads();
  if (PHASE == 0) {
    if (tid == 0) maps[tile] = warp_tot[NT / 32 - 1];
    __syncthreads();  // the stage and warp_tot are reused by the next tile
    continue;
  }
  if (warp > 0) excl = compose<OP, N>(warp_tot[warp - 1], excl);
  // state entering this thread = (excl o carry) applied to the zero state
  const M start = compose<OP, N>(carries[tile], excl);
  V s[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) s[j] = start.B[j];
  int seen = start.seen;

  // ---- the reference's update, position by position; outputs back into the stage ----
#pragma unroll
  for (int k = 0; k < KT; ++k) {
    V x, y, al, d, dd;
    bool valid, in;
    position(k, x, y, al, d, dd, valid, in);
    if (!in) break;
#pragma unroll
    for (int j = 0; j < NS; ++j) s[j] = N::mul(s[j], (j == Traits<OP>::W2) ? dd : d);
    if (valid) {
      V bj[NS];
      contributions<OP, N>(x, y, al, bj);
#pragma unroll
      for (int j = 0; j < NS; ++j) s[j] = N::add(s[j], bj[j]);
      seen = 1;
    }
    // the double-float form finalises like the one-pass scan (divisions cleared)
    double r;
    if constexpr (N::kDF) r = finalize_dfast<OP>(s, seen, mw_df);
    else r = finalize<OP>(N(), s, seen, min_weight);
    const T rt = static_cast<T>(r);
    sx[spad(q0 + k)] = sizeof(T) == 8 ? static_cast<B>(__double_as_longlong(static_cast<double>(rt)))
                                      : static_cast<B>(__float_as_uint(static_cast<float>(rt)));
  }
  __syncthreads();
  B* ob = as_bits(out) + it.base;
#pragma unroll
  for (int j = 0; j < KT; ++j) {
    const int p = j * NT + tid;
    if (t0 + p < n) ob[t0 + p] = sx[spad(p)];
  }
  __syncthreads();  // the stage and warp_tot are reused by the next tile
  (void)row;
  }
}

// Phase 1: per row, the state before each tile, composing the tile maps in a fixed
// order (a block-wide scan over chunks of NT tiles), so the carries are reproducible.
template <int OP, typename N>
__global__ void __launch_bounds__(NT) exp_carry_kernel(const Map<Traits<OP>::NS, N>* __restrict__ maps,
                                                       Map<Traits<OP>::NS, N>* __restrict__ carries, Layout lay) {
  using M = Map<Traits<OP>::NS, N>;
  __shared__ M warp_tot[NT / 32];
  __shared__ M running_smem;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long row = blockIdx.x; row < lay.rows; row += gridDim.x) {
  const long long first = lay.offsets ? lay.item_start[row] : row * lay.items_per_row;
  const long long tiles_per_row = lay.offsets ? lay.item_start[row + 1] - first : lay.items_per_row;
  const M* mr = maps + first;
  M* cr = carries + first;
  __syncthreads();
  if (threadIdx.x == 0) running_smem = identity_map<OP, N>();
  __syncthreads();
  for (long long base = 0; base < tiles_per_row; base += NT) {
    const long long t = base + threadIdx.x;
    M v = t < tiles_per_row ? mr[t] : identity_map<OP, N>();
    M incl = v;
#pragma unroll
    for (int dlt = 1; dlt < 32; dlt <<= 1) {
      const M up = shfl_up_map<OP, N>(incl, dlt);
      if (lane >= dlt) incl = compose<OP, N>(up, incl);
    }
    M excl = shfl_up_map<OP, N>(incl, 1);
    if (lane == 0) excl = identity_map<OP, N>();
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      M run = warp_tot[0];
      for (int w = 1; w < NT / 32; ++w) {
        run = compose<OP, N>(run, warp_tot[w]);
        warp_tot[w] = run;
      }
    }
    __syncthreads();
    if (warp > 0) excl = compose<OP, N>(warp_tot[warp - 1], excl);
    const M running = running_smem;
    if (t < tiles_per_row) {
      M c = compose<OP, N>(running, excl);
      c.A1 = N::zero();  // only the state (B) is used downstream
      c.A2 = N::zero();
      cr[t] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) running_smem = compose<OP, N>(running, warp_tot[NT / 32 - 1]);
    __syncthreads();
  }
  }
}

// The pivot of each row (and of b): its first finite value, 0 if none.  One warp per row.
template <typename T>
__global__ void exp_pivot_kernel(const T* __restrict__ a, const T* __restrict__ b, Layout lay,
                                 double* __restrict__ pivots) {
  typedef typename BitsOf<T>::type B;
  const int lane = threadIdx.x & 31;
  const long long row = static_cast<long long>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (row >= lay.rows) return;
  const long long n = layout_row_len(lay, row);
  for (int which = 0; which < (b ? 2 : 1); ++which) {
    const B* r = as_bits(which ? b : a) + layout_row_base(lay, row);
    double p = 0.0;
    for (long long base = 0; base < n; base += 32) {
      const long long i = base + lane;
      const B v = i < n ? r[i] : B(0);
      const bool ok = i < n && !nan_bits(v) && ((sizeof(B) == 8) ? ((static_cast<unsigned long long>(v) >> 52 & 0x7ff) != 0x7ff)
                                                                 : ((static_cast<unsigned>(v) >> 23 & 0xff) != 0xff));
      const unsigned m = __ballot_sync(0xffffffffu, ok);
      if (m) {
        const B f = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
        p = sizeof(B) == 8 ? __longlong_as_double(static_cast<long long>(f)) : static_cast<double>(__int_as_float(static_cast<int>(f)));
        break;
      }
    }
    if (lane == 0) pivots[2 * row + which] = p;
  }
}

// ---------------------------------------------------------------------------------
// Scalar alpha over rows: one pass with decoupled look-back
// ---------------------------------------------------------------------------------
// With one alpha every position decays every state by the same d (d^2 for
// sum_weight_2), so a run of k positions maps s -> d^k s + B.  A tile of 1024
// positions: each thread folds its 8 positions from zero (one multiply-add per state
// and position); a warp scan with the multipliers d^(8 * 2^i) and a fold over the
// four warps give every thread the tile-relative state before its run and the tile's
// aggregate (d^1024, B); the state entering the tile is the inclusive prefix that the
// row's previous tile published (tiles are claimed row-interleaved, so with many rows
// it is usually there already), and the tile publishes its own; each thread then
// starts from (carry * d^(8 t) + its prefix) and replays its positions with the
// reference's update, finalising each.  The input is read once, and the divisions of the finalisation
// are float32 reciprocals corrected by one float64 step (about 2^-46 relative) in
// the float64 arithmetic.  Deterministic: every fold has a fixed order.

// float64 <-> float32 conversions for the seeds of the divisions below, built from the
// bit patterns on the integer pipes (the FP64 pipe, which bounds these kernels, would
// otherwise execute the conversions).  Valid for exponents within 120 of 0 (callers
// check): the float32 keeps the top 23 fraction bits (truncated), the float64 is exact.
NBG_DEVICE float f32_of(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
  const unsigned e = static_cast<unsigned>((b >> 52) & 0x7ff) - 1023u + 127u;
  return __uint_as_float(sign | (e << 23) | static_cast<unsigned>((b >> 29) & 0x7fffffu));
}
NBG_DEVICE double f64_of(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned long long sign = static_cast<unsigned long long>(b >> 31) << 63;
  const unsigned long long e = static_cast<unsigned long long>(((b >> 23) & 0xff) - 127u + 1023u);
  return __longlong_as_double(static_cast<long long>(sign | (e << 52) | (static_cast<unsigned long long>(b & 0x7fffffu) << 29)));
}
// about 1 / b to float32 precision (2^-22 or so), b's exponent within 120 of 0
NBG_DEVICE double rcp_seed(double b) { return f64_of(__frcp_rn(f32_of(b))); }

// a / b within about 2^-46: a float32 reciprocal of b seeds one float64 correction;
// exponents far from 1, zeros, infinities and NaN take the IEEE division
NBG_DEVICE double fdiv(double a, double b) {
  const unsigned eb = static_cast<unsigned>(static_cast<unsigned long long>(__double_as_longlong(b)) >> 52) & 0x7ffu;
  const unsigned ea = static_cast<unsigned>(static_cast<unsigned long long>(__double_as_longlong(a)) >> 52) & 0x7ffu;
  if (eb < 1023 - 120 || eb > 1023 + 120 || ea == 0x7ffu) return a / b;
  const double r = rcp_seed(b);
  const double q0 = a * r;
  return fma(fma(-q0, b, a), r, q0);
}

// x >= y for float64 values on the integer pipes (false if either is NaN): the
// comparisons of the finalisation, which the FP64 pipe would otherwise execute
NBG_DEVICE bool ge_f64(double x, double y) {
  const unsigned long long bx = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long by = static_cast<unsigned long long>(__double_as_longlong(y));
  if (nan_bits(bx) || nan_bits(by)) return false;
  return order_key_ieee(x) >= order_key_ieee(y);
}
NBG_DEVICE bool gt0_f64(double x) {  // x > 0 (false for NaN and both zeros)
  const long long b = __double_as_longlong(x);
  return b > 0 && !nan_bits(static_cast<unsigned long long>(b));
}

NBG_DEVICE bool gt_f64(double x, double y) {  // x > y on the integer pipes (false for NaN)
  const unsigned long long bx = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long by = static_cast<unsigned long long>(__double_as_longlong(y));
  if (nan_bits(bx) || nan_bits(by)) return false;
  return order_key_ieee(x) > order_key_ieee(y);
}
NBG_DEVICE unsigned exp_bits(double x) {
  return static_cast<unsigned>(static_cast<unsigned long long>(__double_as_longlong(x)) >> 52) & 0x7ffu;
}

// The reference's test bias > 0, bias = 1 - fl(sw2 / S2) with S2 = fl(sw^2)
// (numbagg/moving_exp.py:150-152), decided without the division: fl(q) < 1 exactly
// when q < 1 - 2^-54 (the midpoint below 1 rounds to 1, the even neighbour), that is
// when S2 - sw2 > S2 2^-54.  For S2 in the normal range that difference is exact
// whenever it decides (sw2 within a factor 2 of S2, Sterbenz) and S2 2^-54 is an
// exponent shift.  `d` returns S2 - sw2, which is S2 times the reference's bias up to
// the rounding of that bias.  Other exponents take the reference's expression.
NBG_DEVICE bool bias_positive(double S2, double sw2, double& d) {
  d = S2 - sw2;
  const unsigned e = exp_bits(S2);
  if (e < 64 || e == 0x7ffu) return gt0_f64(1.0 - sw2 / S2);
  const double tiny = __longlong_as_double(__double_as_longlong(S2) - (54ll << 52));
  return gt_f64(d, tiny);
}

// 1 / b to about an ulp: a float32 reciprocal refined twice (Newton), b's exponent
// within 120 of 0 (the caller checks)
NBG_DEVICE double rcp2(double b) {
  double r = rcp_seed(b);
  r = fma(fma(-b, r, 1.0), r, r);
  return fma(fma(-b, r, 1.0), r, r);
}

// The reference's statistics (numbagg/moving_exp.py:142-156, :265-273, :318-335) with
// the divisions cleared: var = (sw sum_x2 - sum_x^2) / (sw^2 - sw2) is var_biased / bias
// multiplied through by sw^2, cov the same, and the correlation's three centred sums
// take one reciprocal of sw.  Every cancellation keeps the reference's conditioning
// (the same differences of the same products) and happens before the one quotient,
// which is therefore not amplified and is taken to about 2^-46 (fdiv); the NaN
// decisions are the reference's (bias_positive,
// weight >= min_weight, the denominator > 0).  Exponents outside the ranges those forms
// assume take the reference's expressions with IEEE divisions.
template <int OP>
NBG_DEVICE double finalize_ref(const double* s, double min_weight) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (OP == kVar || OP == kStd) {
    const double m = s[1] / s[2];
    const double vb = s[0] / s[2] - m * m;
    const double bias = 1.0 - s[3] / (s[2] * s[2]);
    if (!(s[4] >= min_weight && bias > 0)) return nan;
    const double v = vb / bias;
    return OP == kStd ? sqrt(v) : v;
  }
  if (OP == kCov) {
    const double cb = (s[2] - s[0] * s[1] / s[3]) / s[3];
    const double bias = 1.0 - s[4] / (s[3] * s[3]);
    return (s[5] >= min_weight && bias > 0) ? cb / bias : nan;
  }
  const double cov = s[2] - s[0] * s[1] / s[3];
  const double v1 = s[6] - s[0] * s[0] / s[3];
  const double v2 = s[7] - s[1] * s[1] / s[3];
  const double bias = 1.0 - s[4] / (s[3] * s[3]);
  if (!(s[5] >= min_weight && bias > 0)) return nan;
  const double den = sqrt(v1 * v2);
  return den > 0 ? cov / den : nan;
}

template <int OP>
NBG_DEVICE double finalize_fast(const double* s, int seen, double min_weight) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (OP == kCount) return ge_f64(s[1], min_weight) ? s[0] : nan;
  if (OP == kMean) return ge_f64(s[2], min_weight) ? fdiv(s[0], s[1]) : nan;
  if (OP == kSum) return (ge_f64(s[1], min_weight) && seen) ? s[0] : nan;
  constexpr int W = (OP == kVar || OP == kStd) ? 2 : 3;  // sum_weight; W + 1 sum_weight_2, W + 2 weight
  const unsigned ew = exp_bits(s[W]);
  if (ew < 1023 - 100 || ew > 1023 + 100) return finalize_ref<OP>(s, min_weight);
  double d;
  if (!(ge_f64(s[W + 2], min_weight) && bias_positive(s[W] * s[W], s[W + 1], d))) return nan;
  if (OP == kVar || OP == kStd) {
    const double num = fma(s[0], s[2], -(s[1] * s[1]));
    const unsigned en = exp_bits(num);
    if (en == 0x7ffu || en > 1023 + 900) return finalize_ref<OP>(s, min_weight);
    const double v = fdiv(num, d);
    return OP == kStd ? sqrt(v) : v;
  }
  if (OP == kCov) {
    const double num = fma(s[2], s[3], -(s[0] * s[1]));
    const unsigned en = exp_bits(num);
    if (en == 0x7ffu || en > 1023 + 900) return finalize_ref<OP>(s, min_weight);
    return fdiv(num, d);
  }
  // kCorr
  const double r = rcp2(s[3]);
  const double cov = fma(-(s[0] * s[1]), r, s[2]);
  const double v1 = fma(-(s[0] * s[0]), r, s[6]);
  const double v2 = fma(-(s[1] * s[1]), r, s[7]);
  const double den = sqrt(v1 * v2);
  return gt0_f64(den) ? fdiv(cov, den) : nan;
}

// Double-float finalisation of the one-pass scan: min_weight converted once per
// kernel, comparisons on the (hi, lo) pair, and divisions as one float32 quotient plus
// one correction (about 2^-44 relative, far inside the compensated form's bound).
NBG_DEVICE bool df_ge_df(dfl::df x, dfl::df y) {  // x >= y for normalised pairs
  return x.hi > y.hi || (x.hi == y.hi && x.lo >= y.lo);
}
NBG_DEVICE dfl::df df_div_fast(dfl::df x, dfl::df y) {
  using namespace dfl;
  if (y.hi == 0.0f || !isfinite(y.hi) || !isfinite(x.hi)) return df{__fdiv_rn(x.hi, y.hi), 0.0f};
  const float r = __frcp_rn(y.hi);
  const float q1 = __fmul_rn(x.hi, r);
  const df e = df_sub(x, df_mul_f(y, q1));
  return fast_two_sum(q1, __fmul_rn(e.hi, r));
}
// hi + lo in float64 (two conversions and an add on the FP64 pipe, which this form
// leaves mostly idle; widening the bit patterns on the integer pipes measured slower
// here, where instruction issue is the bound)
NBG_DEVICE double df_out(dfl::df x) {
  if (!isfinite(x.hi)) return static_cast<double>(x.hi);
  return static_cast<double>(x.hi) + static_cast<double>(x.lo);
}
template <int OP>
NBG_DEVICE double finalize_dfast(const dfl::df* s, int seen, dfl::df mw) {
  using namespace dfl;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (OP == kCount) return df_ge_df(s[1], mw) ? df_out(s[0]) : nan;
  if (OP == kMean) return df_ge_df(s[2], mw) ? df_out(df_div_fast(s[0], s[1])) : nan;
  if (OP == kSum) return (df_ge_df(s[1], mw) && seen) ? df_out(s[0]) : nan;
  // the variance family with the divisions cleared as in finalize_fast: var =
  // (sw sum_x2 - sum_x^2) / (sw^2 - sw2), the bias test sw^2 > sw2, and the correlation
  // from the centred sums multiplied through by sw (on pivoted values, so the products
  // stay far inside float32's range)
  if (OP == kVar || OP == kStd) {
    const df den = df_sub(df_mul(s[2], s[2]), s[3]);
    if (!(df_ge_df(s[4], mw) && df_pos(den))) return nan;
    const df v = df_div_fast(df_sub(df_mul(s[0], s[2]), df_mul(s[1], s[1])), den);
    if (OP == kVar) return df_out(v);
    if (v.hi < 0.0f) return nan;
    return v.hi == 0.0f ? 0.0 : df_out(df_sqrt(v));
  }
  const df den = df_sub(df_mul(s[3], s[3]), s[4]);
  if (!(df_ge_df(s[5], mw) && df_pos(den))) return nan;
  if (OP == kCov) return df_out(df_div_fast(df_sub(df_mul(s[2], s[3]), df_mul(s[0], s[1])), den));
  const df cov = df_sub(df_mul(s[2], s[3]), df_mul(s[0], s[1]));
  const df var1 = df_sub(df_mul(s[6], s[3]), df_mul(s[0], s[0]));
  const df var2 = df_sub(df_mul(s[7], s[3]), df_mul(s[1], s[1]));
  const df vv = df_mul(var1, var2);
  if (!df_pos(vv)) return nan;
  return df_out(df_div_fast(cov, df_sqrt(vv)));
}

template <int OP>
NBG_DEVICE double finalize_scan(F64, const double* s, int seen, double min_weight, double, double alpha) {
  double f[Traits<base_op(OP)>::NS];
  with_weight<OP, F64>(s, alpha, f);
  return finalize_fast<base_op(OP)>(f, seen, min_weight);
}
template <int OP>
NBG_DEVICE double finalize_scan(DF, const dfl::df* s, int seen, double, dfl::df mw, dfl::df alpha) {
  dfl::df f[Traits<base_op(OP)>::NS];
  with_weight<OP, DF>(s, alpha, f);
  return finalize_dfast<base_op(OP)>(f, seen, mw);
}

template <typename N>
NBG_DEVICE typename N::T pow_n(typename N::T x, int e) {  // x^e for e >= 0, by squaring
  typename N::T r = N::one();
  while (e) {
    if (e & 1) r = N::mul(r, x);
    x = N::mul(x, x);
    e >>= 1;
  }
  return r;
}

template <int OP, typename T, typename N>
__global__ void __launch_bounds__(NT) exp_scan_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                      double alpha_scalar, double min_weight, T* __restrict__ out,
                                                      long long rows, long long n, long long tiles_per_row,
                                                      void* ws_base, size_t ws_bytes,
                                                      const double* __restrict__ pivots) {
  constexpr int NS = Traits<OP>::NS;
  constexpr int W2 = Traits<OP>::W2;
  constexpr bool TWO = Traits<OP>::TWO;
  constexpr bool SHIFT = Traits<OP>::PIVOT && N::kDF;
  typedef typename BitsOf<T>::type B;
  typedef typename N::T V;
  using M = Map<NS, N>;
  __shared__ B sx[SPAD];
  __shared__ B sy[TWO ? SPAD : 1];
  __shared__ V wtot[NT / 32][NS];
  __shared__ int wseen[NT / 32];
  __shared__ M carry_smem;
  __shared__ long long tile_smem;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const B nanb = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);
  const long long total_tiles = rows * tiles_per_row;

  const V mw_n = as_num(N(), min_weight);  // min_weight in the policy's numbers, once
  // decay powers shared by every tile: d^k and (d^2)^k for the runs of this thread
  const V al = as_num(N(), alpha_scalar);
  const V d = N::sub(N::one(), al);
  const V dd = N::mul(d, d);
  const V d8 = pow_n<N>(d, KT), dd8 = pow_n<N>(dd, KT);
  const V d_lane = pow_n<N>(d8, lane), dd_lane = pow_n<N>(dd8, lane);          // over this lane's predecessors
  const V d_warp = pow_n<N>(pow_n<N>(d8, 32), warp), dd_warp = pow_n<N>(pow_n<N>(dd8, 32), warp);
  const V d_start = N::mul(d_warp, d_lane), dd_start = N::mul(dd_warp, dd_lane);  // d^(8 tid)
  const V d_tile = pow_n<N>(d8, NT), dd_tile = pow_n<N>(dd8, NT);
  // the warp scan's factors (d^8)^(2^k), k = 0..5, once per CTA (float64: a multiply
  // per level and tile saved on the FP64 pipe; double-float squares them per tile, as
  // the registers for a table would spill there)
  V pw1[6], pw2[6];
  pw1[0] = d8;
  pw2[0] = dd8;
#pragma unroll
  for (int k = 1; k < 6; ++k) {
    pw1[k] = N::mul(pw1[k - 1], pw1[k - 1]);
    pw2[k] = N::mul(pw2[k - 1], pw2[k - 1]);
  }

  for (;;) {
    if (tid == 0) tile_smem = claim_tile(ws.hdr);
    __syncthreads();
    const long long tile = tile_smem;
    if (tile >= total_tiles) break;
    const TileCoord tc = tile_coord(tile, rows);  // claimed row-interleaved
    const long long row = tc.row, chunk = tc.chunk;
    const long long t0 = chunk * TILE;
    const B* ar = as_bits(a) + row * n;
    const B* br = TWO ? as_bits(b) + row * n : nullptr;
#pragma unroll
    for (int j = 0; j < KT; ++j) {
      const int p = j * NT + tid;
      const long long i = t0 + p;
      const bool in = i < n;
      sx[spad(p)] = in ? ar[i] : nanb;
      if (TWO) sy[spad(p)] = in ? br[i] : nanb;
    }
    __syncthreads();
    V px = N::zero(), py = N::zero();
    if (SHIFT) {
      px = as_num(N(), pivots[2 * row]);
      if (TWO) py = as_num(N(), pivots[2 * row + 1]);
    }
    const int q0 = tid * KT;
    auto load = [&](int k, V& x, V& y, bool& valid) {
      const int sp = spad(q0 + k);
      const B xb = sx[sp];
      const B yb = TWO ? sy[sp] : xb;
      valid = !nan_bits(xb) && !(TWO && nan_bits(yb));  // positions past n hold NaN
      x = value_as(N(), xb);
      y = TWO ? value_as(N(), yb) : x;
      if (SHIFT) {
        x = N::sub(x, px);
        if (TWO) y = N::sub(y, py);
      }
    };
    // ---- this thread's run folded from zero ----
    V s[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) s[j] = N::zero();
    int seen = 0;
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      V x, y;
      bool valid;
      load(k, x, y, valid);
      V bj[NS];
      contributions<OP, N>(x, y, al, bj);
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        // a missing value contributes zero: one multiply-add either way (s * f + 0
        // rounds like the product alone)
        if (!valid) bj[j] = N::zero();
        s[j] = N::fma(s[j], (j == W2) ? dd : d, bj[j]);
      }
      seen |= valid ? 1 : 0;
    }
    // ---- warp scan: S_lane = sum over lanes l' <= lane of (d^8)^(lane - l') s_l' ----
    V f1 = d8, f2 = dd8;
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
      const int dl = 1 << lvl;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        const V up = shfl_up_num(s[j], dl);
        if (lane >= dl) s[j] = N::fma(up, (j == W2) ? f2 : f1, s[j]);
      }
      const int us = __shfl_up_sync(0xffffffffu, seen, dl);
      if (lane >= dl) seen |= us;
      if constexpr (N::kDF) {
        f1 = N::mul(f1, f1);
        f2 = N::mul(f2, f2);
      } else {
        f1 = pw1[lvl + 1];
        f2 = pw2[lvl + 1];
      }
    }
    // exclusive prefix within the warp
    V e[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      e[j] = shfl_up_num(s[j], 1);
      if (lane == 0) e[j] = N::zero();
    }
    int eseen = __shfl_up_sync(0xffffffffu, seen, 1);
    if (lane == 0) eseen = 0;
    if (lane == 31) {
#pragma unroll
      for (int j = 0; j < NS; ++j) wtot[warp][j] = s[j];
      wseen[warp] = seen;
    }
    __syncthreads();
    // the warps before this one, folded in order (f1 = d^256 after the scan)
    {
      V w[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) w[j] = N::zero();
      int ws_seen = 0;
      for (int u = 0; u < warp; ++u) {
#pragma unroll
        for (int j = 0; j < NS; ++j) w[j] = N::fma(w[j], (j == W2) ? f2 : f1, wtot[u][j]);
        ws_seen |= wseen[u];
      }
      // state before this thread's run, relative to the tile start
#pragma unroll
      for (int j = 0; j < NS; ++j) e[j] = N::fma(w[j], (j == W2) ? dd_lane : d_lane, e[j]);
      eseen |= ws_seen;
    }
    // ---- the tile's aggregate, the look-back, the carry ----
    if (warp == 0) {
      M agg;
      agg.A1 = d_tile;
      agg.A2 = dd_tile;
      agg.pad = 0;
      agg.seen = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) agg.B[j] = N::zero();
      if (lane == 0) {
        for (int u = 0; u < NT / 32; ++u) {
#pragma unroll
          for (int j = 0; j < NS; ++j) agg.B[j] = N::fma(agg.B[j], (j == W2) ? f2 : f1, wtot[u][j]);
          agg.seen |= wseen[u];
        }
      }
      // chained look-back: wait for the inclusive prefix of the row's previous tile
      // (claimed `rows` claims earlier, so usually finished) and publish this tile's;
      // composing in that fixed order keeps the result independent of timing
      M excl = identity_map<OP, N>();
      if (lane == 0) {
        if (chunk > 0) {
          const long long pred = tile - rows;
          if (wait_status(ws, pred, epoch) == kStatePrefix) excl = read_payload<M>(ws, pred, kStatePrefix);
          else record_error(ws.hdr, kLookbackTimeout, static_cast<unsigned>(tile));
        }
        if (chunk + 1 < tiles_per_row) publish(ws, tile, epoch, kStatePrefix, compose<OP, N>(excl, agg));
        carry_smem = excl;
      }
    }
    __syncthreads();
    // ---- replay from the state entering this thread's run ----
    const M carry = carry_smem;
#pragma unroll
    for (int j = 0; j < NS; ++j) s[j] = N::fma(carry.B[j], (j == W2) ? dd_start : d_start, e[j]);
    seen = eseen | carry.seen;
    T res[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      V x, y;
      bool valid;
      load(k, x, y, valid);
      V bj[NS];
      contributions<OP, N>(x, y, al, bj);
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        if (!valid) bj[j] = N::zero();
        s[j] = N::fma(s[j], (j == W2) ? dd : d, bj[j]);
      }
      seen |= valid ? 1 : 0;
      res[k] = static_cast<T>(finalize_scan<OP>(N(), s, seen, min_weight, mw_n, al));
    }
    __syncthreads();  // every thread has read its run: the stage takes the outputs
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
    __syncthreads();  // the stage is reused by the next tile
  }
  if (tid == 0) finish_cta(ws.hdr);
}

// ---------------------------------------------------------------------------------
// Along a non-last axis: one thread per column
// ---------------------------------------------------------------------------------
// A C-contiguous array scanned along axis k is a batch of `outer` blocks of n x `inner`
// values: position p of column i of block o sits at (o n + p) inner + i.  Each thread
// owns one column and runs the reference's loop down it (a rounded multiply, then a
// rounded add, and the reference's finalisation), so consecutive threads read
// consecutive addresses and nothing is copied or transposed.  With the float64
// arithmetic this is numbagg's own sequence of operations.  alpha_mode 0: scalar;
// 1: n values along the axis; 2: one per element, laid out like `a`.
template <int OP, typename T, typename N>
__global__ void __launch_bounds__(256) exp_cols_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                       const T* __restrict__ alpha_arr, double alpha_scalar,
                                                       int alpha_mode, double min_weight, T* __restrict__ out,
                                                       long long outer, long long n, long long inner) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool TWO = Traits<OP>::TWO;
  constexpr bool SHIFT = Traits<OP>::PIVOT && N::kDF;
  typedef typename BitsOf<T>::type B;
  typedef typename N::T V;
  const long long col = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (col >= outer * inner) return;
  const long long o = col / inner, i = col - o * inner;
  const long long base = o * n * inner + i;
  const B* ab = as_bits(a) + base;
  const B* bb = TWO ? as_bits(b) + base : nullptr;
  const B* alb = alpha_mode == 2 ? as_bits(alpha_arr) + base : as_bits(alpha_arr);
  const long long astep = alpha_mode == 2 ? inner : 1;
  // the pivot of the shift-invariant statistics (double-float only): the column's first
  // finite value, as the row kernels take each row's
  V px = N::zero(), py = N::zero();
  if (SHIFT) {
    for (int w = 0; w < (TWO ? 2 : 1); ++w) {
      const B* r = w ? bb : ab;
      for (long long p = 0; p < n; ++p) {
        const B v = r[p * inner];
        const bool fin = sizeof(B) == 8 ? ((static_cast<unsigned long long>(v) >> 52 & 0x7ff) != 0x7ff)
                                        : ((static_cast<unsigned>(v) >> 23 & 0xff) != 0xff);
        if (fin) {
          (w ? py : px) = value_as(N(), v);
          break;
        }
      }
    }
  }
  const V al_s = as_num(N(), alpha_scalar);
  V s[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) s[j] = N::zero();
  int seen = 0;
  for (long long p = 0; p < n; ++p) {
    const B xb = ab[p * inner];
    const B yb = TWO ? bb[p * inner] : xb;
    const bool valid = !nan_bits(xb) && !(TWO && nan_bits(yb));
    const V al = alpha_mode == 0 ? al_s : value_as(N(), alb[p * astep]);
    const V d = N::sub(N::one(), al);
    const V dd = N::mul(d, d);
#pragma unroll
    for (int j = 0; j < NS; ++j) s[j] = N::mul(s[j], (j == Traits<OP>::W2) ? dd : d);
    if (valid) {
      V x = value_as(N(), xb), y = TWO ? value_as(N(), yb) : x;
      if (SHIFT) {
        x = N::sub(x, px);
        if (TWO) y = N::sub(y, py);
      }
      V bj[NS];
      contributions<OP, N>(x, y, al, bj);
#pragma unroll
      for (int j = 0; j < NS; ++j) s[j] = N::add(s[j], bj[j]);
      seen = 1;
    }
    const T r = static_cast<T>(finalize<OP>(N(), s, seen, min_weight));
    as_bits(out)[base + p * inner] = sizeof(T) == 8 ? static_cast<B>(__double_as_longlong(static_cast<double>(r)))
                                                   : static_cast<B>(__float_as_uint(static_cast<float>(r)));
  }
}

}  // namespace mexp
}  // namespace nbg

using namespace nbg;
using namespace nbg::mexp;

namespace {

long long exp_tiles_per_row(long long n) { return n <= 0 ? 0 : (n + TILE - 1) / TILE; }
constexpr long long kScanMinRows = 32;

// maps and carries for `tiles` tiles (or the look-back workspace of the one-pass scan,
// whichever is larger), pivots and the ragged plan for `rows` series
size_t exp_scratch_for(long long rows, long long tiles) {
  const size_t maps = 2 * static_cast<size_t>(tiles) * sizeof(Map<Traits<kCorr>::NS, F64>);
  const size_t lookback = workspace_bytes(tiles);
  return (maps > lookback ? maps : lookback) + 1024 + static_cast<size_t>(rows) * 16 + static_cast<size_t>(rows + 1) * 8;
}

// One pass with decoupled look-back (scalar alpha, rows x n).  The look-back state
// (header and one status word per tile) is cleared at the start of the call.
template <int OP, typename T, typename N>
int launch_exp_scan(const T* a, const T* b, double alpha_scalar, double min_weight, T* out, long long rows,
                    long long n, void* ws, cudaStream_t s) {
  const long long tpr = exp_tiles_per_row(n);
  const long long tiles = rows * tpr;
  const size_t lb = workspace_bytes(tiles);
  double* pivots = reinterpret_cast<double*>((reinterpret_cast<size_t>(ws) + lb + 255) & ~static_cast<size_t>(255));
  if (cudaMemsetAsync(ws, 0, 256 + static_cast<size_t>(tiles) * 8, s) != cudaSuccess) return kLaunchError;
  int launches = 1;
  constexpr bool SHIFT = Traits<OP>::PIVOT && N::kDF;
  if (SHIFT) {
    Layout lay{nullptr, nullptr, rows, n, tpr};
    exp_pivot_kernel<T><<<static_cast<int>((rows + 7) / 8), 256, 0, s>>>(a, Traits<OP>::TWO ? b : nullptr, lay, pivots);
    ++launches;
  }
  static int per_sm = 0;  // resident CTAs per SM, from the occupancy calculator
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm == 0) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, exp_scan_kernel<scan_op(OP), T, N>, NT, 0);
    per_sm = nb > 0 ? nb : 1;
  }
  const long long cap = static_cast<long long>(sms) * per_sm;
  const int grid = static_cast<int>(tiles < cap ? tiles : cap);
  exp_scan_kernel<scan_op(OP), T, N><<<grid, NT, 0, s>>>(a, b, alpha_scalar, min_weight, out, rows, n, tpr, ws, lb,
                                                          pivots);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

// offsets == nullptr: rows x n; else ragged series with `total` values in all
template <int OP, typename T, typename N>
int launch_exp(const T* a, const T* b, const T* alpha, double alpha_scalar, int alpha_mode,
               double min_weight, T* out, const long long* offsets, long long rows, long long n, long long total,
               void* ws, size_t ws_bytes, cudaStream_t s) {
  if (rows < 0 || n < 0 || total < 0 || alpha_mode < 0 || alpha_mode > 2) return kInvalidArgument;
  if (offsets && alpha_mode == 1) return kInvalidArgument;  // one alpha per position needs equal lengths
  if (rows == 0 || (!offsets && n == 0)) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b) || (alpha_mode > 0 && !alpha)) return kInvalidArgument;
  // an upper bound on the tiles: each series adds at most one partial tile
  const long long tiles = offsets ? total / TILE + rows : rows * exp_tiles_per_row(n);
  if (!ws || ws_bytes < exp_scratch_for(rows, tiles)) return kWorkspaceTooSmall;
  // the one-pass scan chains tiles row by row: with few rows the chain would serialise,
  // so those keep the three-phase scan
  if (alpha_mode == 0 && !offsets && rows >= kScanMinRows)
    return launch_exp_scan<OP, T, N>(a, b, alpha_scalar, min_weight, out, rows, n, ws, s);
  using M = Map<Traits<OP>::NS, N>;
  static_assert(sizeof(M) <= sizeof(Map<Traits<kCorr>::NS, F64>), "8-byte numbers");
  auto up = [](size_t p) { return (p + 255) & ~static_cast<size_t>(255); };
  M* maps = reinterpret_cast<M*>(up(reinterpret_cast<size_t>(ws)));
  M* carries = maps + tiles;
  double* pivots = reinterpret_cast<double*>(up(reinterpret_cast<size_t>(carries + tiles)));
  long long* item_start = reinterpret_cast<long long*>(up(reinterpret_cast<size_t>(pivots + 2 * rows)));
  Layout lay{offsets, item_start, rows, n, offsets ? 0 : exp_tiles_per_row(n)};
  int launches = 3;
  if (offsets) {
    ragged_plan_kernel<<<1, 1024, 0, s>>>(offsets, rows, TILE, item_start);
    ++launches;
  }
  constexpr bool SHIFT = Traits<OP>::PIVOT && N::kDF;
  if (SHIFT) {
    exp_pivot_kernel<T><<<static_cast<int>((rows + 7) / 8), 256, 0, s>>>(a, Traits<OP>::TWO ? b : nullptr, lay, pivots);
    ++launches;
  }
  // rows: one CTA per tile; ragged series: a persistent grid over the planned tiles
  const int grid = offsets ? layout_grid(LLONG_MAX, 16) : static_cast<int>(std::min<long long>(tiles, 0x7fffffffLL));
  exp_tile_kernel<OP, T, N, 0><<<grid, NT, 0, s>>>(a, b, alpha, alpha_scalar, alpha_mode, min_weight, out, lay, maps,
                                                   carries, pivots);
  exp_carry_kernel<OP, N><<<static_cast<int>(std::min<long long>(rows, 65535)), NT, 0, s>>>(maps, carries, lay);
  exp_tile_kernel<OP, T, N, 2><<<grid, NT, 0, s>>>(a, b, alpha, alpha_scalar, alpha_mode, min_weight, out, lay, maps,
                                                   carries, pivots);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
template <int OP, typename T, typename N>
int launch_exp_cols(const T* a, const T* b, const T* alpha, double alpha_scalar, int alpha_mode, double min_weight,
                    T* out, long long outer, long long n, long long inner, cudaStream_t s) {
  if (outer < 0 || n < 0 || inner < 0 || alpha_mode < 0 || alpha_mode > 2) return kInvalidArgument;
  if (outer == 0 || n == 0 || inner == 0) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b) || (alpha_mode > 0 && !alpha)) return kInvalidArgument;
  const long long cols = outer * inner;
  const long long blocks = (cols + 255) / 256;
  if (blocks > 0x7fffffffLL) return kUnsupported;
  exp_cols_kernel<OP, T, N><<<static_cast<int>(blocks), 256, 0, s>>>(a, b, alpha, alpha_scalar, alpha_mode,
                                                                      min_weight, out, outer, n, inner);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

// the largest state (move_exp_nancorr) bounds every function's scratch
size_t nbg_move_exp_workspace_bytes(long long rows, long long n) {
  return exp_scratch_for(rows, rows * exp_tiles_per_row(n));
}
// ragged series holding `total` values in all
size_t nbg_move_exp_ragged_workspace_bytes(long long nseries, long long total) {
  return exp_scratch_for(nseries, total / TILE + nseries);
}

// alpha_mode: 0 = scalar `alpha_scalar`, 1 = `alpha` has n values shared by all rows,
// 2 = `alpha` has rows*n values laid out like `a`.
#define NBG_EXP1(NAME, OPC, T, SFX, N)                                                           \
  int nbg_##NAME##_##SFX(const T* a, const T* alpha, double alpha_scalar, int alpha_mode,         \
                         double min_weight, T* out, long long rows, long long n, void* ws,        \
                         size_t ws_bytes, void* stream) {                                         \
    return launch_exp<OPC, T, N>(a, nullptr, alpha, alpha_scalar, alpha_mode, min_weight, out,   \
                                 nullptr, rows, n, 0, ws, ws_bytes, static_cast<cudaStream_t>(stream)); \
  }
#define NBG_EXP2(NAME, OPC, T, SFX, N)                                                           \
  int nbg_##NAME##_##SFX(const T* a, const T* b, const T* alpha, double alpha_scalar,             \
                         int alpha_mode, double min_weight, T* out, long long rows, long long n,   \
                         void* ws, size_t ws_bytes, void* stream) {                               \
    return launch_exp<OPC, T, N>(a, b, alpha, alpha_scalar, alpha_mode, min_weight, out, nullptr, rows, \
                                 n, 0, ws, ws_bytes, static_cast<cudaStream_t>(stream));          \
  }

NBG_EXP1(move_exp_nancount, kCount, double, f64, F64)
NBG_EXP1(move_exp_nancount, kCount, float, f32, F64)
NBG_EXP1(move_exp_nanmean, kMean, double, f64, F64)
NBG_EXP1(move_exp_nanmean, kMean, float, f32, F64)
NBG_EXP1(move_exp_nansum, kSum, double, f64, F64)
NBG_EXP1(move_exp_nansum, kSum, float, f32, F64)
NBG_EXP1(move_exp_nanvar, kVar, double, f64, F64)
NBG_EXP1(move_exp_nanvar, kVar, float, f32, F64)
NBG_EXP1(move_exp_nanstd, kStd, double, f64, F64)
NBG_EXP1(move_exp_nanstd, kStd, float, f32, F64)
NBG_EXP2(move_exp_nancov, kCov, double, f64, F64)
NBG_EXP2(move_exp_nancov, kCov, float, f32, F64)
NBG_EXP2(move_exp_nancorr, kCorr, double, f64, F64)
NBG_EXP2(move_exp_nancorr, kCorr, float, f32, F64)
// FP32-compensated forms of the float64 entry points (double-float on the FP32 pipes)
NBG_EXP1(move_exp_nancount, kCount, double, f64_fp32c, DF)
NBG_EXP1(move_exp_nanmean, kMean, double, f64_fp32c, DF)
NBG_EXP1(move_exp_nansum, kSum, double, f64_fp32c, DF)
NBG_EXP1(move_exp_nanvar, kVar, double, f64_fp32c, DF)
NBG_EXP1(move_exp_nanstd, kStd, double, f64_fp32c, DF)
NBG_EXP2(move_exp_nancov, kCov, double, f64_fp32c, DF)
NBG_EXP2(move_exp_nancorr, kCorr, double, f64_fp32c, DF)

// Along a non-last axis of a C-contiguous array: `outer` blocks of n x `inner` values,
// scanned along n, one thread per column (exp_cols_kernel).
#define NBG_EXP1_COLS(NAME, OPC, T, SFX, N)                                                          \
  int nbg_##NAME##_cols_##SFX(const T* a, const T* alpha, double alpha_scalar, int alpha_mode,        \
                              double min_weight, T* out, long long outer, long long n, long long inner, \
                              void* stream) {                                                        \
    return launch_exp_cols<OPC, T, N>(a, nullptr, alpha, alpha_scalar, alpha_mode, min_weight, out,  \
                                      outer, n, inner, static_cast<cudaStream_t>(stream));           \
  }
#define NBG_EXP2_COLS(NAME, OPC, T, SFX, N)                                                          \
  int nbg_##NAME##_cols_##SFX(const T* a, const T* b, const T* alpha, double alpha_scalar,            \
                              int alpha_mode, double min_weight, T* out, long long outer, long long n, \
                              long long inner, void* stream) {                                       \
    return launch_exp_cols<OPC, T, N>(a, b, alpha, alpha_scalar, alpha_mode, min_weight, out, outer, n, \
                                      inner, static_cast<cudaStream_t>(stream));                     \
  }
#define NBG_EXP_COLS_ALL(T, SFX, NP)                                  \
  NBG_EXP1_COLS(move_exp_nancount, kCount, T, SFX, NP)               \
  NBG_EXP1_COLS(move_exp_nanmean, kMean, T, SFX, NP)                 \
  NBG_EXP1_COLS(move_exp_nansum, kSum, T, SFX, NP)                   \
  NBG_EXP1_COLS(move_exp_nanvar, kVar, T, SFX, NP)                   \
  NBG_EXP1_COLS(move_exp_nanstd, kStd, T, SFX, NP)                   \
  NBG_EXP2_COLS(move_exp_nancov, kCov, T, SFX, NP)                   \
  NBG_EXP2_COLS(move_exp_nancorr, kCorr, T, SFX, NP)
NBG_EXP_COLS_ALL(double, f64, F64)
NBG_EXP_COLS_ALL(float, f32, F64)
NBG_EXP_COLS_ALL(double, f64_fp32c, DF)

// Ragged series: series s is values[offsets[s] : offsets[s + 1]] (nseries + 1 offsets on
// the device, `total` = offsets[nseries]); a scalar alpha (alpha_mode 0) or one per
// value (alpha_mode 2).
#define NBG_EXP_RAGGED(NAME, OPC, SFX, N)                                                          \
  int nbg_##NAME##_ragged_##SFX(const double* values, const long long* offsets, long long nseries,   \
                                long long total, const double* alpha, double alpha_scalar,          \
                                int alpha_mode, double min_weight, double* out, void* ws,           \
                                size_t ws_bytes, void* stream) {                                    \
    return launch_exp<OPC, double, N>(values, nullptr, alpha, alpha_scalar, alpha_mode, min_weight, \
                                      out, offsets, nseries, 0, total, ws, ws_bytes,                \
                                      static_cast<cudaStream_t>(stream));                           \
  }
NBG_EXP_RAGGED(move_exp_nanmean, kMean, f64, F64)
NBG_EXP_RAGGED(move_exp_nanvar, kVar, f64, F64)
NBG_EXP_RAGGED(move_exp_nanstd, kStd, f64, F64)
NBG_EXP_RAGGED(move_exp_nanmean, kMean, f64_fp32c, DF)
NBG_EXP_RAGGED(move_exp_nanvar, kVar, f64_fp32c, DF)
NBG_EXP_RAGGED(move_exp_nanstd, kStd, f64_fp32c, DF)

}  // extern "C"
