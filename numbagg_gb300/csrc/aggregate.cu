// Static aggregations over the last axis of a (rows, m) view: allnan, anynan, nancount,
// nansum, nanmean, nanvar, nanstd (numbagg/funcs.py:23-159, the ndaggregate family)
// and nanargmax, nanargmin, nanmax, nanmin (numbagg/funcs.py:162-242, ndreduce).  The
// caller moves the reduced axes last and flattens them, as numbagg's move_axes does
// (numbagg/utils.py:20-32).
//
// A CTA reduces one chunk of one row to a partial (float sum, wrapping integer sum,
// count, and the best order key with its first column); a second kernel folds each
// row's partials in chunk order.  nanvar / nanstd are two passes like the reference
// (numbagg/funcs.py:106-159): the row means first, then the sum of squared deviations
// from them.  Float sums take half their elements in an exact 128-bit fixed-point sum
// and half in float64 (numba accumulates in float64, or in float32 for the float32
// nansum); every reduction order is fixed, so results are the same run to run.
#include "dfloat.cuh"

#include <climits>

namespace nbg {
namespace agg {

enum Fn : int { kAllNan = 0, kAnyNan, kCount, kSum, kMean, kVar, kStd, kMax, kMin, kArgMax, kArgMin };
constexpr int AT = 256;
constexpr long long kNone = LLONG_MAX;  // no column selected yet

struct Part {
  fx::i128 fx;             // float sums, half the elements: exact fixed-point sum
  double s;                // the other half, summed in float64 (and the variance's
                           // squared deviations outside the double-float range)
  dfl::df q;               // the variance's squared deviations, in double-float
  long long i;             // integer sum, wrapping like the reference's integer loops
  long long cnt;           // elements that are not NaN
  unsigned long long key;  // selection: order key of the best element
  long long idx;           // and its column (kNone: none)
  int sc;                  // fx's scale: the largest biased exponent met
  int pinf, ninf;          // +inf / -inf terms of a float sum
};

NBG_DEVICE Part none_part() {
  Part p;
  p.fx = 0;
  p.s = 0.0;
  p.q = dfl::df{0.0f, 0.0f};
  p.i = 0;
  p.cnt = 0;
  p.key = 0ull;
  p.idx = kNone;
  p.sc = 0;
  p.pinf = p.ninf = 0;
  return p;
}

// a before b in the fixed reduction order; the selection keeps the larger key and,
// among equal keys, the smaller column (numbagg/funcs.py:171-176: the first maximum).
// Fixed-point sums are aligned to the larger scale and added: exact and associative.
NBG_DEVICE Part combine(const Part& a, const Part& b) {
  Part r;
  r.sc = a.sc > b.sc ? a.sc : b.sc;
  r.fx = fx::shr(a.fx, r.sc - a.sc) + fx::shr(b.fx, r.sc - b.sc);
  r.s = a.s + b.s;
  r.q = dfl::df_add(a.q, b.q);
  r.i = static_cast<long long>(static_cast<unsigned long long>(a.i) + static_cast<unsigned long long>(b.i));
  r.cnt = a.cnt + b.cnt;
  const bool take_b = b.idx != kNone && (a.idx == kNone || b.key > a.key || (b.key == a.key && b.idx < a.idx));
  r.key = take_b ? b.key : a.key;
  r.idx = take_b ? b.idx : a.idx;
  r.pinf = a.pinf + b.pinf;
  r.ninf = a.ninf + b.ninf;
  return r;
}

NBG_DEVICE Part shfl_part(const Part& v, int o) {
  Part r;
  const unsigned long long lo = static_cast<unsigned long long>(v.fx);
  const unsigned long long hi = static_cast<unsigned long long>(v.fx >> 64);
  r.fx = static_cast<fx::i128>((static_cast<fx::u128>(__shfl_xor_sync(0xffffffffu, hi, o)) << 64) |
                               __shfl_xor_sync(0xffffffffu, lo, o));
  r.s = __shfl_xor_sync(0xffffffffu, v.s, o);
  r.q = dfl::df{__shfl_xor_sync(0xffffffffu, v.q.hi, o), __shfl_xor_sync(0xffffffffu, v.q.lo, o)};
  r.i = __shfl_xor_sync(0xffffffffu, v.i, o);
  r.cnt = __shfl_xor_sync(0xffffffffu, v.cnt, o);
  r.key = __shfl_xor_sync(0xffffffffu, v.key, o);
  r.idx = __shfl_xor_sync(0xffffffffu, v.idx, o);
  r.sc = __shfl_xor_sync(0xffffffffu, v.sc, o);
  r.pinf = __shfl_xor_sync(0xffffffffu, v.pinf, o);
  r.ninf = __shfl_xor_sync(0xffffffffu, v.ninf, o);
  return r;
}

// The float sum a partial holds: the fixed-point half rounded once to float64 plus the
// float64 half; the reference's float64 running sum gives inf with +inf terms, -inf
// with -inf terms and NaN with both (inf - inf).
NBG_DEVICE double part_sum(const Part& r) {
  if (r.pinf > 0 && r.ninf > 0) return quiet_nan(0.0);
  if (r.pinf > 0) return __longlong_as_double(0x7ff0000000000000ll);
  if (r.ninf > 0) return __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
  return fx::to_f64(r.fx, fx::lsb_value(r.sc)) + r.s;
}
// the squared deviations: the double-float sum and the float64 one
NBG_DEVICE double part_ssq(const Part& r) {
  return (static_cast<double>(r.q.hi) + static_cast<double>(r.q.lo)) + r.s;
}

// order keys: x < y  <=>  key(x) < key(y) for non-NaN values, -0.0 == +0.0
NBG_DEVICE unsigned long long sel_key(double x) { return order_key_ieee(x); }
NBG_DEVICE unsigned long long sel_key(float x) {
  unsigned b = static_cast<unsigned>(__float_as_int(x));
  if ((b << 1) == 0) b = 0;  // +-0 -> +0
  return static_cast<unsigned long long>((b >> 31) ? ~b : (b | 0x80000000u));
}
NBG_DEVICE unsigned long long sel_key(int x) {
  return static_cast<unsigned long long>(static_cast<unsigned>(x) ^ 0x80000000u);
}
NBG_DEVICE unsigned long long sel_key(long long x) {
  return static_cast<unsigned long long>(x) ^ 0x8000000000000000ull;
}

template <typename T>
struct IsFloat {
  static constexpr bool value = false;
};
template <>
struct IsFloat<double> {
  static constexpr bool value = true;
};
template <>
struct IsFloat<float> {
  static constexpr bool value = true;
};

// One element x at column c into a thread's partial.  DEV: the variance's second pass
// (squared deviations from the mean mu).  A thread meets its columns in increasing
// order, so the first extreme wins among equal keys.  Float sums split a thread's
// elements between two accumulators that run on different pipes: FIX (every other
// element) shifts the value's integer mantissa into a 128-bit fixed-point sum at the
// scale of the largest exponent met so far (fixed128.cuh, shifted right when a larger
// one arrives; exact) with integer instructions, the others take one float64 add.
// Either alone binds the kernel to its pipe at about twice the time of the pair.
template <int F, typename T, bool DEV, bool FIX>
NBG_DEVICE void absorb(Part& p, T x, long long c, double mu) {
  constexpr bool SEL = F == kMax || F == kMin || F == kArgMax || F == kArgMin;
  constexpr bool MINIMUM = F == kMin || F == kArgMin;
  if (is_nan(x)) return;
  ++p.cnt;
  if (DEV) {
    // (x - mean)^2 summed (numbagg/funcs.py:120-126): the deviation rounded in float64
    // as the reference's, its square and the sum in double-float on the FP32 pipes
    // (about 2^-46 relative, and the squares are all positive, so nothing cancels);
    // deviations beyond 2^(+-40) (whose squares, summed, could leave float32's range),
    // zeros, infinities and NaN take float64
    const double d = static_cast<double>(x) - mu;
    const int ed = static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(d)) >> 52) & 0x7ff);
    if (ed >= 1023 - 40 && ed <= 1023 + 40) {
      const dfl::df dd = df_from_f64(d);
      p.q = dfl::df_add_fast(p.q, dfl::df_mul(dd, dd));
    } else {
      p.s = fma(d, d, p.s);
    }
  } else if (F == kSum || F == kMean || F == kVar || F == kStd) {
    if (IsFloat<T>::value) {
      const double xd = static_cast<double>(x);
      if (fx::is_inf(xd)) {
        if (xd > 0) ++p.pinf;
        else ++p.ninf;
        return;
      }
      if (!FIX) {
        p.s += xd;
        return;
      }
      const int e = fx::biased_exponent(xd);
      if (e > p.sc) {
        p.fx = fx::shr(p.fx, e - p.sc);
        p.sc = e;
      }
      p.fx += fx::fix_value(xd, p.sc);
    } else {
      p.i = static_cast<long long>(static_cast<unsigned long long>(p.i) + static_cast<unsigned long long>(x));
    }
  } else if (SEL) {
    const unsigned long long k = MINIMUM ? ~sel_key(x) : sel_key(x);
    if (p.idx == kNone || k > p.key) {
      p.key = k;
      p.idx = c;
    }
  }
}

// One CTA per (row, chunk).
template <int F, typename T, bool DEV>
__global__ void __launch_bounds__(AT) agg_part_kernel(const T* __restrict__ a, long long rows, long long m,
                                                      long long chunk_len, long long chunks,
                                                      const double* __restrict__ mean, Part* __restrict__ parts) {
  __shared__ Part warp_parts[AT / 32];
  const long long row = blockIdx.x / chunks, chunk = blockIdx.x - row * chunks;
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  const T* ar = a + row * m;
  const double mu = DEV ? mean[row] : 0.0;
  Part p = none_part();
  // float sums: four loads in flight per thread before any of them is consumed (a
  // loop-carried sum would otherwise leave one load per thread outstanding, too few to
  // cover DRAM latency); the other statistics keep the plain loop, which measured faster
  constexpr bool SUM = (F == kSum || F == kMean || F == kVar || F == kStd) && IsFloat<T>::value;
  long long c = c0 + threadIdx.x;
  if (!SUM) {
    for (; c < c1; c += AT) absorb<F, T, DEV, false>(p, ar[c], c, mu);
  }
  for (; c + 3 * AT < c1; c += 4 * AT) {
    const T x0 = ar[c], x1 = ar[c + AT], x2 = ar[c + 2 * AT], x3 = ar[c + 3 * AT];
    absorb<F, T, DEV, false>(p, x0, c, mu);
    absorb<F, T, DEV, true>(p, x1, c + AT, mu);
    absorb<F, T, DEV, false>(p, x2, c + 2 * AT, mu);
    absorb<F, T, DEV, true>(p, x3, c + 3 * AT, mu);
  }
  for (int k = 0; c < c1; c += AT, ++k) {
    if (k & 1) absorb<F, T, DEV, true>(p, ar[c], c, mu);
    else absorb<F, T, DEV, false>(p, ar[c], c, mu);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const Part q = shfl_part(p, o);
    p = (lane & o) ? combine(q, p) : combine(p, q);  // lower lanes first
  }
  if (lane == 0) warp_parts[warp] = p;
  __syncthreads();
  if (threadIdx.x == 0) {
    Part r = warp_parts[0];
    for (int w = 1; w < AT / 32; ++w) r = combine(r, warp_parts[w]);
    parts[row * chunks + chunk] = r;
  }
}

// The reduced axes in the middle of a C-contiguous array, viewed as (outer, m, inner):
// output (o, i) reduces a[(o m + r) inner + i] over r, in place (no copy).  A CTA takes
// 32 consecutive outputs, one per lane, and a chunk of r; warp w takes r = c0 + w,
// c0 + w + 8, ..., so every warp load is 32 consecutive values.  The warps' partials
// are combined in warp order and the (output, chunk) partials folded like the rows'.
template <int F, typename T, bool DEV>
__global__ void __launch_bounds__(AT) agg_cols_part_kernel(const T* __restrict__ a, long long outer, long long m,
                                                           long long inner, long long chunk_len, long long chunks,
                                                           const double* __restrict__ mean, Part* __restrict__ parts) {
  __shared__ Part warp_parts[AT / 32][32];
  const long long cols = outer * inner;
  const long long tile = blockIdx.x / chunks, chunk = blockIdx.x - tile * chunks;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long col = tile * 32 + lane;
  const bool live = col < cols;
  Part p = none_part();
  if (live) {
    const long long o = col / inner, i = col - o * inner;
    const T* ac = a + o * m * inner + i;
    const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
    const double mu = DEV ? mean[col] : 0.0;
    constexpr int W = AT / 32;
    constexpr bool SUM = (F == kSum || F == kMean || F == kVar || F == kStd) && IsFloat<T>::value;
    long long r = c0 + warp;
    if (!SUM) {
#pragma unroll 4
      for (; r < c1; r += W) absorb<F, T, DEV, false>(p, ac[r * inner], r, mu);
    }
    for (; r + 3 * W < c1; r += 4 * W) {
      const T x0 = ac[r * inner], x1 = ac[(r + W) * inner], x2 = ac[(r + 2 * W) * inner], x3 = ac[(r + 3 * W) * inner];
      absorb<F, T, DEV, false>(p, x0, r, mu);
      absorb<F, T, DEV, true>(p, x1, r + W, mu);
      absorb<F, T, DEV, false>(p, x2, r + 2 * W, mu);
      absorb<F, T, DEV, true>(p, x3, r + 3 * W, mu);
    }
    for (int k = 0; r < c1; r += W, ++k) {
      if (k & 1) absorb<F, T, DEV, true>(p, ac[r * inner], r, mu);
      else absorb<F, T, DEV, false>(p, ac[r * inner], r, mu);
    }
  }
  warp_parts[warp][lane] = p;
  __syncthreads();
  if (warp == 0 && live) {
    Part q = warp_parts[0][lane];
#pragma unroll
    for (int w = 1; w < AT / 32; ++w) q = combine(q, warp_parts[w][lane]);
    parts[col * chunks + chunk] = q;
  }
}

// a row's partials in chunk order
NBG_DEVICE Part fold_row(const Part* __restrict__ parts, long long row, long long chunks) {
  Part r = parts[row * chunks];
  for (long long c = 1; c < chunks; ++c) r = combine(r, parts[row * chunks + c]);
  return r;
}

// the variance's first pass -> row means (NaN where nothing is valid)
__global__ void agg_mean_kernel(const Part* __restrict__ parts, long long rows, long long chunks,
                                double* __restrict__ mean) {
  for (long long row = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; row < rows;
       row += static_cast<long long>(gridDim.x) * blockDim.x) {
    const Part r = fold_row(parts, row, chunks);
    mean[row] = r.cnt > 0 ? part_sum(r) / static_cast<double>(r.cnt) : quiet_nan(0.0);
  }
}

template <int F, typename T, typename O>
__global__ void agg_finish_kernel(const T* __restrict__ a, const Part* __restrict__ parts, long long rows,
                                  long long m, long long inner, long long chunks, long long ddof,
                                  O* __restrict__ out) {
  for (long long row = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; row < rows;
       row += static_cast<long long>(gridDim.x) * blockDim.x) {
    const Part r = fold_row(parts, row, chunks);
    O res;
    if (F == kAllNan) {
      res = static_cast<O>(r.cnt == 0);  // numbagg/funcs.py:31-36
    } else if (F == kAnyNan) {
      res = static_cast<O>(r.cnt < m);  // numbagg/funcs.py:47-52
    } else if (F == kCount) {
      res = static_cast<O>(r.cnt);
    } else if (F == kSum) {
      if (IsFloat<T>::value) res = static_cast<O>(part_sum(r));
      else res = static_cast<O>(static_cast<T>(r.i));  // wraps to the input's width
    } else if (F == kMean) {
      res = static_cast<O>(r.cnt > 0 ? part_sum(r) / static_cast<double>(r.cnt) : quiet_nan(0.0));  // :93-103
    } else if (F == kVar || F == kStd) {
      // :113-133 / :143-159: sum of squared deviations / (count - ddof), NaN unless count > ddof
      double v = quiet_nan(0.0);
      if (r.cnt > ddof && r.cnt > 0) v = part_ssq(r) / static_cast<double>(r.cnt - ddof);
      if (F == kStd) v = sqrt(v);
      res = static_cast<O>(v);
    } else if (F == kMax || F == kMin) {
      // :207-221 / :229-242: NaN where every element is NaN
      if (r.idx == kNone) res = static_cast<O>(quiet_nan(0.0));
      else res = static_cast<O>(a[((row / inner) * m + r.idx) * inner + row % inner]);
    } else {
      // :167-199: the first extreme column; -1 marks an all-NaN row (the caller raises)
      res = static_cast<O>(r.idx == kNone ? -1ll : r.idx);
    }
    out[row] = res;
  }
}

struct Plan {
  long long chunk_len, chunks;
};

inline Plan plan(long long rows, long long m) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long target = static_cast<long long>(sms) * 8;  // CTAs per call
  const long long min_len = static_cast<long long>(AT) * 8;
  long long per_row = (target + rows - 1) / (rows > 0 ? rows : 1);
  const long long cap = (m + min_len - 1) / min_len;
  if (per_row > cap) per_row = cap;
  if (per_row < 1) per_row = 1;
  Plan p;
  p.chunk_len = m > 0 ? (m + per_row - 1) / per_row : 1;
  p.chunks = m > 0 ? (m + p.chunk_len - 1) / p.chunk_len : 1;
  return p;
}

inline size_t workspace_bytes(long long rows, long long m) {
  const Plan p = plan(rows, m);
  return static_cast<size_t>(rows) * static_cast<size_t>(p.chunks) * sizeof(Part) + 256 +
         static_cast<size_t>(rows) * 8 + 256;
}

inline int fin_grid(long long rows) {
  const long long b = (rows + 255) / 256;
  return static_cast<int>(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

template <int F, typename T, typename O>
int launch(const T* a, O* out, long long rows, long long m, long long ddof, void* ws, size_t ws_bytes,
           cudaStream_t s) {
  if (rows < 0 || m < 0) return kInvalidArgument;
  if (rows == 0) return kOk;
  if (!out || (m > 0 && !a)) return kInvalidArgument;
  constexpr bool SEL = F == kMax || F == kMin || F == kArgMax || F == kArgMin;
  if (SEL && m == 0) return kInvalidArgument;  // numbagg raises on an empty reduction
  if (!ws || ws_bytes < workspace_bytes(rows, m)) return kWorkspaceTooSmall;
  const Plan p = plan(rows, m);
  if (rows * p.chunks > 0x7fffffffll) return kUnsupported;
  const size_t up = (reinterpret_cast<size_t>(ws) + 255) & ~static_cast<size_t>(255);
  Part* parts = reinterpret_cast<Part*>(up);
  double* mean = reinterpret_cast<double*>((up + static_cast<size_t>(rows * p.chunks) * sizeof(Part) + 255) &
                                           ~static_cast<size_t>(255));
  const int grid = static_cast<int>(rows * p.chunks);
  int launches = 2;
  agg_part_kernel<F, T, false><<<grid, AT, 0, s>>>(a, rows, m, p.chunk_len, p.chunks, nullptr, parts);
  if (F == kVar || F == kStd) {
    agg_mean_kernel<<<fin_grid(rows), 256, 0, s>>>(parts, rows, p.chunks, mean);
    agg_part_kernel<F, T, true><<<grid, AT, 0, s>>>(a, rows, m, p.chunk_len, p.chunks, mean, parts);
    launches += 2;
  }
  agg_finish_kernel<F, T, O><<<fin_grid(rows), 256, 0, s>>>(a, parts, rows, m, 1, p.chunks, ddof, out);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

// the column layout: tiles of 32 outputs, each split into chunks of r
inline Plan plan_cols(long long cols, long long m) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (cols + 31) / 32;
  const long long target = static_cast<long long>(sms) * 8;
  long long per_tile = (target + tiles - 1) / (tiles > 0 ? tiles : 1);
  const long long cap = (m + 63) / 64;  // at least 8 values per warp and chunk
  if (per_tile > cap) per_tile = cap;
  if (per_tile < 1) per_tile = 1;
  Plan p;
  p.chunk_len = m > 0 ? (m + per_tile - 1) / per_tile : 1;
  p.chunks = m > 0 ? (m + p.chunk_len - 1) / p.chunk_len : 1;
  return p;
}

inline size_t cols_workspace_bytes(long long outer, long long m, long long inner) {
  const long long cols = outer * inner;
  const Plan p = plan_cols(cols, m);
  return static_cast<size_t>(cols) * static_cast<size_t>(p.chunks) * sizeof(Part) + 256 +
         static_cast<size_t>(cols) * 8 + 256;
}

template <int F, typename T, typename O>
int launch_cols(const T* a, O* out, long long outer, long long m, long long inner, long long ddof, void* ws,
                size_t ws_bytes, cudaStream_t s) {
  if (outer < 0 || m < 0 || inner < 0) return kInvalidArgument;
  const long long cols = outer * inner;
  if (cols == 0) return kOk;
  if (!out || (m > 0 && !a)) return kInvalidArgument;
  constexpr bool SEL = F == kMax || F == kMin || F == kArgMax || F == kArgMin;
  if (SEL && m == 0) return kInvalidArgument;
  if (!ws || ws_bytes < cols_workspace_bytes(outer, m, inner)) return kWorkspaceTooSmall;
  const Plan p = plan_cols(cols, m);
  const long long tiles = (cols + 31) / 32;
  if (tiles * p.chunks > 0x7fffffffll) return kUnsupported;
  const size_t up = (reinterpret_cast<size_t>(ws) + 255) & ~static_cast<size_t>(255);
  Part* parts = reinterpret_cast<Part*>(up);
  double* mean = reinterpret_cast<double*>((up + static_cast<size_t>(cols * p.chunks) * sizeof(Part) + 255) &
                                           ~static_cast<size_t>(255));
  const int grid = static_cast<int>(tiles * p.chunks);
  int launches = 2;
  agg_cols_part_kernel<F, T, false><<<grid, AT, 0, s>>>(a, outer, m, inner, p.chunk_len, p.chunks, nullptr, parts);
  if (F == kVar || F == kStd) {
    agg_mean_kernel<<<fin_grid(cols), 256, 0, s>>>(parts, cols, p.chunks, mean);
    agg_cols_part_kernel<F, T, true><<<grid, AT, 0, s>>>(a, outer, m, inner, p.chunk_len, p.chunks, mean, parts);
    launches += 2;
  }
  agg_finish_kernel<F, T, O><<<fin_grid(cols), 256, 0, s>>>(a, parts, cols, m, inner, p.chunks, ddof, out);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

}  // namespace agg
}  // namespace nbg

using namespace nbg;
using namespace nbg::agg;

extern "C" {

size_t nbg_aggregate_workspace_bytes(long long rows, long long m) { return workspace_bytes(rows, m); }
size_t nbg_aggregate_cols_workspace_bytes(long long outer, long long m, long long inner) {
  return outer < 0 || m < 0 || inner < 0 ? 0 : cols_workspace_bytes(outer, m, inner);
}

// each function over the last axis of (rows, m), and (_cols) over the middle axis of a
// C-contiguous (outer, m, inner) array
#define NBG_AGG(NAME, FN, T, O, SFX)                                                                   \
  int nbg_##NAME##_##SFX(const T* a, O* out, long long rows, long long m, void* ws, size_t ws_bytes,   \
                         void* stream) {                                                             \
    return launch<FN, T, O>(a, out, rows, m, 0, ws, ws_bytes, static_cast<cudaStream_t>(stream));     \
  }                                                                                                  \
  int nbg_##NAME##_cols_##SFX(const T* a, O* out, long long outer, long long m, long long inner,       \
                              void* ws, size_t ws_bytes, void* stream) {                             \
    return launch_cols<FN, T, O>(a, out, outer, m, inner, 0, ws, ws_bytes, static_cast<cudaStream_t>(stream)); \
  }
#define NBG_AGG_DDOF(NAME, FN, T, SFX)                                                                 \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long m, long long ddof, void* ws,     \
                         size_t ws_bytes, void* stream) {                                            \
    return launch<FN, T, T>(a, out, rows, m, ddof, ws, ws_bytes, static_cast<cudaStream_t>(stream));  \
  }                                                                                                  \
  int nbg_##NAME##_cols_##SFX(const T* a, T* out, long long outer, long long m, long long inner,       \
                              long long ddof, void* ws, size_t ws_bytes, void* stream) {             \
    return launch_cols<FN, T, T>(a, out, outer, m, inner, ddof, ws, ws_bytes, static_cast<cudaStream_t>(stream)); \
  }
#define NBG_AGG_ALL(NAME, FN, O)            \
  NBG_AGG(NAME, FN, double, O, f64)         \
  NBG_AGG(NAME, FN, float, O, f32)          \
  NBG_AGG(NAME, FN, int, O, i32)            \
  NBG_AGG(NAME, FN, long long, O, i64)
#define NBG_AGG_SAME(NAME, FN)              \
  NBG_AGG(NAME, FN, double, double, f64)    \
  NBG_AGG(NAME, FN, float, float, f32)      \
  NBG_AGG(NAME, FN, int, int, i32)          \
  NBG_AGG(NAME, FN, long long, long long, i64)

NBG_AGG_ALL(allnan, kAllNan, unsigned char)
NBG_AGG_ALL(anynan, kAnyNan, unsigned char)
NBG_AGG_ALL(nancount, kCount, long long)
NBG_AGG_SAME(nansum, kSum)
NBG_AGG(nanmean, kMean, double, double, f64)
NBG_AGG(nanmean, kMean, float, float, f32)
NBG_AGG_DDOF(nanvar, kVar, double, f64)
NBG_AGG_DDOF(nanvar, kVar, float, f32)
NBG_AGG_DDOF(nanstd, kStd, double, f64)
NBG_AGG_DDOF(nanstd, kStd, float, f32)
NBG_AGG_SAME(nanmax, kMax)
NBG_AGG_SAME(nanmin, kMin)
NBG_AGG_ALL(nanargmax, kArgMax, long long)
NBG_AGG_ALL(nanargmin, kArgMin, long long)

}  // extern "C"
