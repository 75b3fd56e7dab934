// Exponentially weighted family move_exp_nan{count,mean,sum,var,std,cov,corr}
// (numbagg/moving_exp.py:12-335), float64 and float32 arrays.
//
// Each reference state variable follows s_i = decay_i * s_{i-1} + b_i, where
// decay_i = 1 - alpha_i and b_i is the contribution of position i (zero when the
// value is NaN); sum_weight_2 decays by decay_i**2.  A position is therefore an
// affine map s -> A*s + B, and maps compose associatively:
//     (A2, B2) o (A1, B1) = (A2*A1, A2*B1 + B2).
// A row is cut into tiles.  Phase 0 composes each tile's map (thread-serial over K
// positions, then a fixed-structure warp-shuffle scan); phase 1 scans the tile maps
// of each row in a fixed order to get the state entering every tile; phase 2 replays
// each position with the reference's own update, a rounded multiply followed by a
// rounded add (no FMA), starting from that state, and finalises with the reference's
// formulas.  The composition order never depends on timing, so results are
// bit-identical run to run and a prefix of a row gives the same bits as the whole
// row.  Phase 0 and 2 both read the input; the plain float64 form is bound by the
// FP64 pipe (about 1.6 adds per clock per SM on GB300), not by that extra read.
//
// alpha: a scalar, a 1-D array along the scanned axis shared by every row, or one
// value per element (numbagg/decorators.py:398-409).
#include "nbg_common.cuh"

namespace nbg {
namespace mexp {

enum Op : int { kCount = 0, kMean, kSum, kVar, kStd, kCov, kCorr };

template <int OP>
struct Traits;
// state order and decay kind per op; kW2 marks the sum_weight_2 state (decay**2)
template <>
struct Traits<kCount> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr int W2 = -1; };
template <>
struct Traits<kMean> { static constexpr int NS = 3; static constexpr bool TWO = false; static constexpr int W2 = -1; };
template <>
struct Traits<kSum> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr int W2 = -1; };
template <>
struct Traits<kVar> { static constexpr int NS = 5; static constexpr bool TWO = false; static constexpr int W2 = 3; };
template <>
struct Traits<kStd> { static constexpr int NS = 5; static constexpr bool TWO = false; static constexpr int W2 = 3; };
template <>
struct Traits<kCov> { static constexpr int NS = 6; static constexpr bool TWO = true; static constexpr int W2 = 4; };
template <>
struct Traits<kCorr> { static constexpr int NS = 8; static constexpr bool TWO = true; static constexpr int W2 = 4; };

template <int NS>
struct Map {
  double A1, A2;  // product of decays, product of squared decays
  double B[NS];
  int seen;       // any valid value (move_exp_nansum's zero_count flag)
  int pad;
};

template <int OP>
NBG_DEVICE Map<Traits<OP>::NS> identity_map() {
  Map<Traits<OP>::NS> m;
  m.A1 = 1.0;
  m.A2 = 1.0;
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) m.B[j] = 0.0;
  m.seen = 0;
  m.pad = 0;
  return m;
}

// later o earlier
template <int OP>
NBG_DEVICE Map<Traits<OP>::NS> compose(const Map<Traits<OP>::NS>& earlier, const Map<Traits<OP>::NS>& later) {
  Map<Traits<OP>::NS> r;
  r.A1 = later.A1 * earlier.A1;
  r.A2 = later.A2 * earlier.A2;
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) {
    const double a = (j == Traits<OP>::W2) ? later.A2 : later.A1;
    r.B[j] = fma(a, earlier.B[j], later.B[j]);
  }
  r.seen = earlier.seen | later.seen;
  r.pad = 0;
  return r;
}

template <int OP>
struct ComposeOp {
  NBG_DEVICE Map<Traits<OP>::NS> identity() const { return identity_map<OP>(); }
  NBG_DEVICE Map<Traits<OP>::NS> combine(const Map<Traits<OP>::NS>& e, const Map<Traits<OP>::NS>& l) const {
    return compose<OP>(e, l);
  }
};

template <int OP>
NBG_DEVICE Map<Traits<OP>::NS> shfl_up_map(const Map<Traits<OP>::NS>& v, int d) {
  Map<Traits<OP>::NS> r;
  r.A1 = __shfl_up_sync(0xffffffffu, v.A1, d);
  r.A2 = __shfl_up_sync(0xffffffffu, v.A2, d);
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) r.B[j] = __shfl_up_sync(0xffffffffu, v.B[j], d);
  r.seen = __shfl_up_sync(0xffffffffu, v.seen, d);
  r.pad = 0;
  return r;
}

// contributions b_j of one position, in the reference's state order
template <int OP>
NBG_DEVICE void contributions(double x, double y, double alpha, double* b) {
  if (OP == kCount) {  // count, weight
    b[0] = 1.0; b[1] = alpha;
  } else if (OP == kMean) {  // numer, denom, weight
    b[0] = x; b[1] = 1.0; b[2] = alpha;
  } else if (OP == kSum) {  // numer, weight
    b[0] = x; b[1] = alpha;
  } else if (OP == kVar || OP == kStd) {  // sum_x_2, sum_x, sum_weight, sum_weight_2, weight
    b[0] = __dmul_rn(x, x); b[1] = x; b[2] = 1.0; b[3] = 1.0; b[4] = alpha;
  } else if (OP == kCov) {  // sum_x1, sum_x2, sum_x1x2, sum_weight, sum_weight_2, weight
    b[0] = x; b[1] = y; b[2] = __dmul_rn(x, y); b[3] = 1.0; b[4] = 1.0; b[5] = alpha;
  } else {  // kCorr: + sum_x1_2, sum_x2_2
    b[0] = x; b[1] = y; b[2] = __dmul_rn(x, y); b[3] = 1.0; b[4] = 1.0; b[5] = alpha;
    b[6] = __dmul_rn(x, x); b[7] = __dmul_rn(y, y);
  }
}

template <int OP>
NBG_DEVICE double finalize(const double* s, int seen, double min_weight) {
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

constexpr int NT = 128;

// Phase 0 (PHASE == 0): the map of each tile, composed in position order, to maps[].
// Phase 2 (PHASE == 2): outputs, starting from the state carries[tile] before the tile.
// One CTA per tile; tiles do not wait on each other.
template <int OP, typename T, int K, int PHASE>
__global__ void __launch_bounds__(NT) exp_tile_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                      const T* __restrict__ alpha_arr, double alpha_scalar,
                                                      int alpha_mode, double min_weight,
                                                      T* __restrict__ out, long long rows, long long n,
                                                      long long tiles_per_row, Map<Traits<OP>::NS>* maps,
                                                      const Map<Traits<OP>::NS>* carries) {
  constexpr int NS = Traits<OP>::NS;
  constexpr long long TILE = static_cast<long long>(NT) * K;
  using M = Map<NS>;
  __shared__ M warp_tot[NT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long tile = blockIdx.x;
  const long long row = tile / tiles_per_row;
  const long long chunk = tile - row * tiles_per_row;
  const long long p0 = chunk * TILE + static_cast<long long>(threadIdx.x) * K;
  const T* ar = a + row * n;
  const T* br = Traits<OP>::TWO ? b + row * n : nullptr;
  const T* alr = alpha_mode == 2 ? alpha_arr + row * n : alpha_arr;

  T xv[K], yv[K];
  double al[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const long long i = p0 + k;
    const bool in = i < n;
    xv[k] = in ? ar[i] : T(0);
    yv[k] = (Traits<OP>::TWO && in) ? br[i] : T(0);
    al[k] = alpha_mode == 0 ? alpha_scalar : (in ? static_cast<double>(alr[i]) : 0.0);
  }
  // ---- this thread's maps composed in order ----
  M agg = identity_map<OP>();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const long long i = p0 + k;
    if (i >= n) break;
    const double d = __dadd_rn(1.0, -al[k]);
    const double dd = __dmul_rn(d, d);
    bool valid = !is_nan(xv[k]);
    if (Traits<OP>::TWO) valid = valid && !is_nan(yv[k]);
    double bj[NS];
    contributions<OP>(static_cast<double>(xv[k]), static_cast<double>(yv[k]), al[k], bj);
    agg.A1 = agg.A1 * d;
    agg.A2 = agg.A2 * dd;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const double f = (j == Traits<OP>::W2) ? dd : d;
      agg.B[j] = valid ? fma(agg.B[j], f, bj[j]) : agg.B[j] * f;
    }
    agg.seen |= valid ? 1 : 0;
  }
  // ---- block scan (fixed structure, so the result does not depend on timing) ----
  M incl = agg;
#pragma unroll
  for (int dlt = 1; dlt < 32; dlt <<= 1) {
    const M up = shfl_up_map<OP>(incl, dlt);
    if (lane >= dlt) incl = compose<OP>(up, incl);
  }
  M excl = shfl_up_map<OP>(incl, 1);
  if (lane == 0) excl = identity_map<OP>();
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    M run = warp_tot[0];
    for (int w = 1; w < NT / 32; ++w) {
      run = compose<OP>(run, warp_tot[w]);
      warp_tot[w] = run;
    }
  }
  __syncthreads();
  if (PHASE == 0) {
    if (threadIdx.x == 0) maps[tile] = warp_tot[NT / 32 - 1];
    return;
  }
  if (warp > 0) excl = compose<OP>(warp_tot[warp - 1], excl);
  // state entering this thread = (excl o carry) applied to the zero state
  const M start = compose<OP>(carries[tile], excl);
  double s[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) s[j] = start.B[j];
  int seen = start.seen;

  // ---- the reference's update, position by position ----
  T* orow = out + row * n;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const long long i = p0 + k;
    if (i >= n) break;
    const double d = __dadd_rn(1.0, -al[k]);
    const double dd = __dmul_rn(d, d);
#pragma unroll
    for (int j = 0; j < NS; ++j) s[j] = __dmul_rn(s[j], (j == Traits<OP>::W2) ? dd : d);
    bool valid = !is_nan(xv[k]);
    if (Traits<OP>::TWO) valid = valid && !is_nan(yv[k]);
    if (valid) {
      double bj[NS];
      contributions<OP>(static_cast<double>(xv[k]), static_cast<double>(yv[k]), al[k], bj);
#pragma unroll
      for (int j = 0; j < NS; ++j) s[j] = __dadd_rn(s[j], bj[j]);
      seen = 1;
    }
    orow[i] = static_cast<T>(finalize<OP>(s, seen, min_weight));
  }
}

// Phase 1: per row, the state before each tile, composing the tile maps in a fixed
// order (a block-wide scan over chunks of NT tiles), so the carries are reproducible.
template <int OP>
__global__ void __launch_bounds__(NT) exp_carry_kernel(const Map<Traits<OP>::NS>* __restrict__ maps,
                                                       Map<Traits<OP>::NS>* __restrict__ carries,
                                                       long long tiles_per_row) {
  using M = Map<Traits<OP>::NS>;
  __shared__ M warp_tot[NT / 32];
  __shared__ M running_smem;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long row = blockIdx.x;
  const M* mr = maps + row * tiles_per_row;
  M* cr = carries + row * tiles_per_row;
  if (threadIdx.x == 0) running_smem = identity_map<OP>();
  __syncthreads();
  for (long long base = 0; base < tiles_per_row; base += NT) {
    const long long t = base + threadIdx.x;
    M v = t < tiles_per_row ? mr[t] : identity_map<OP>();
    M incl = v;
#pragma unroll
    for (int dlt = 1; dlt < 32; dlt <<= 1) {
      const M up = shfl_up_map<OP>(incl, dlt);
      if (lane >= dlt) incl = compose<OP>(up, incl);
    }
    M excl = shfl_up_map<OP>(incl, 1);
    if (lane == 0) excl = identity_map<OP>();
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      M run = warp_tot[0];
      for (int w = 1; w < NT / 32; ++w) {
        run = compose<OP>(run, warp_tot[w]);
        warp_tot[w] = run;
      }
    }
    __syncthreads();
    if (warp > 0) excl = compose<OP>(warp_tot[warp - 1], excl);
    const M running = running_smem;
    if (t < tiles_per_row) {
      M c = compose<OP>(running, excl);
      c.A1 = 0.0;  // only the state (B) is used downstream
      c.A2 = 0.0;
      cr[t] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) running_smem = compose<OP>(running, warp_tot[NT / 32 - 1]);
    __syncthreads();
  }
}

}  // namespace mexp
}  // namespace nbg

using namespace nbg;
using namespace nbg::mexp;

namespace {
constexpr int kExpK = 8;

long long exp_tiles_per_row(long long n) {
  const long long tile = static_cast<long long>(NT) * kExpK;
  return n <= 0 ? 0 : (n + tile - 1) / tile;
}

template <int OP>
size_t exp_scratch_bytes(long long rows, long long n) {
  return 2 * static_cast<size_t>(rows * exp_tiles_per_row(n)) * sizeof(Map<Traits<OP>::NS>) + 256;
}

template <int OP, typename T>
int launch_exp(const T* a, const T* b, const T* alpha, double alpha_scalar, int alpha_mode,
               double min_weight, T* out, long long rows, long long n, void* ws, size_t ws_bytes,
               cudaStream_t s) {
  if (rows < 0 || n < 0 || alpha_mode < 0 || alpha_mode > 2) return kInvalidArgument;
  if (rows == 0 || n == 0) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b) || (alpha_mode > 0 && !alpha)) return kInvalidArgument;
  const long long tpr = exp_tiles_per_row(n);
  const long long total = rows * tpr;
  if (total > 0x7fffffffll) return kUnsupported;
  if (!ws || ws_bytes < exp_scratch_bytes<OP>(rows, n)) return kWorkspaceTooSmall;
  using M = Map<Traits<OP>::NS>;
  M* maps = reinterpret_cast<M*>((reinterpret_cast<size_t>(ws) + 127) & ~static_cast<size_t>(127));
  M* carries = maps + total;
  const int grid = static_cast<int>(total);
  exp_tile_kernel<OP, T, kExpK, 0><<<grid, NT, 0, s>>>(a, b, alpha, alpha_scalar, alpha_mode, min_weight,
                                                       out, rows, n, tpr, maps, carries);
  exp_carry_kernel<OP><<<static_cast<int>(rows), NT, 0, s>>>(maps, carries, tpr);
  exp_tile_kernel<OP, T, kExpK, 2><<<grid, NT, 0, s>>>(a, b, alpha, alpha_scalar, alpha_mode, min_weight,
                                                       out, rows, n, tpr, maps, carries);
  note_launches(3);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

// the largest state (move_exp_nancorr) bounds every function's scratch
size_t nbg_move_exp_workspace_bytes(long long rows, long long n) {
  return exp_scratch_bytes<kCorr>(rows, n);
}

// alpha_mode: 0 = scalar `alpha_scalar`, 1 = `alpha` has n values shared by all rows,
// 2 = `alpha` has rows*n values laid out like `a`.
#define NBG_EXP1(NAME, OPC, T, SFX)                                                            \
  int nbg_##NAME##_##SFX(const T* a, const T* alpha, double alpha_scalar, int alpha_mode,       \
                         double min_weight, T* out, long long rows, long long n, void* ws,      \
                         size_t ws_bytes, void* stream) {                                       \
    return launch_exp<OPC, T>(a, nullptr, alpha, alpha_scalar, alpha_mode, min_weight, out, rows, \
                              n, ws, ws_bytes, static_cast<cudaStream_t>(stream));             \
  }
#define NBG_EXP2(NAME, OPC, T, SFX)                                                            \
  int nbg_##NAME##_##SFX(const T* a, const T* b, const T* alpha, double alpha_scalar,           \
                         int alpha_mode, double min_weight, T* out, long long rows, long long n, \
                         void* ws, size_t ws_bytes, void* stream) {                             \
    return launch_exp<OPC, T>(a, b, alpha, alpha_scalar, alpha_mode, min_weight, out, rows, n,   \
                              ws, ws_bytes, static_cast<cudaStream_t>(stream));                \
  }

NBG_EXP1(move_exp_nancount, kCount, double, f64)
NBG_EXP1(move_exp_nancount, kCount, float, f32)
NBG_EXP1(move_exp_nanmean, kMean, double, f64)
NBG_EXP1(move_exp_nanmean, kMean, float, f32)
NBG_EXP1(move_exp_nansum, kSum, double, f64)
NBG_EXP1(move_exp_nansum, kSum, float, f32)
NBG_EXP1(move_exp_nanvar, kVar, double, f64)
NBG_EXP1(move_exp_nanvar, kVar, float, f32)
NBG_EXP1(move_exp_nanstd, kStd, double, f64)
NBG_EXP1(move_exp_nanstd, kStd, float, f32)
NBG_EXP2(move_exp_nancov, kCov, double, f64)
NBG_EXP2(move_exp_nancov, kCov, float, f32)
NBG_EXP2(move_exp_nancorr, kCorr, double, f64)
NBG_EXP2(move_exp_nancorr, kCorr, float, f32)

}  // extern "C"
