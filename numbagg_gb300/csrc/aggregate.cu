// Static aggregations over the last axis of a (rows, m) view: allnan, anynan, nancount,
// nansum, nanmean, nanvar, nanstd (numbagg/funcs.py:23-159, the ndaggregate family)
// and nanargmax, nanargmin, nanmax, nanmin (numbagg/funcs.py:162-242, ndreduce).  The
// caller moves the reduced axes last and flattens them, as numbagg's move_axes does
// (numbagg/utils.py:20-32).
//
// A CTA reduces one chunk of one row to a partial (float sum, wrapping integer sum,
// count, and the best order key with its first column); a second kernel folds each
// row's partials in chunk order.  Every reduction order is fixed, so results are the
// same run to run.  nanvar / nanstd are two passes like the reference
// (numbagg/funcs.py:106-159): the row means first, then the sum of squared deviations
// from them.  Float sums accumulate in float64, as numba's loops do for every float
// statistic except the float32 nansum (float32 accumulator there; the float64 one
// is the more accurate of the two, rounded once to float32).
#include "nbg_common.cuh"

#include <climits>

namespace nbg {
namespace agg {

enum Fn : int { kAllNan = 0, kAnyNan, kCount, kSum, kMean, kVar, kStd, kMax, kMin, kArgMax, kArgMin };
constexpr int AT = 256;
constexpr long long kNone = LLONG_MAX;  // no column selected yet

struct Part {
  double s;                // float sum (sum, mean, first pass of the variance) or squared deviations
  long long i;             // integer sum, wrapping like the reference's integer loops
  long long cnt;           // elements that are not NaN
  unsigned long long key;  // selection: order key of the best element
  long long idx;           // and its column (kNone: none)
};

NBG_DEVICE Part none_part() { return Part{0.0, 0, 0, 0ull, kNone}; }

// a before b in the fixed reduction order; the selection keeps the larger key and,
// among equal keys, the smaller column (numbagg/funcs.py:171-176: the first maximum)
NBG_DEVICE Part combine(const Part& a, const Part& b) {
  Part r;
  r.s = a.s + b.s;
  r.i = static_cast<long long>(static_cast<unsigned long long>(a.i) + static_cast<unsigned long long>(b.i));
  r.cnt = a.cnt + b.cnt;
  const bool take_b = b.idx != kNone && (a.idx == kNone || b.key > a.key || (b.key == a.key && b.idx < a.idx));
  r.key = take_b ? b.key : a.key;
  r.idx = take_b ? b.idx : a.idx;
  return r;
}

NBG_DEVICE Part shfl_part(const Part& v, int o) {
  Part r;
  r.s = __shfl_xor_sync(0xffffffffu, v.s, o);
  r.i = __shfl_xor_sync(0xffffffffu, v.i, o);
  r.cnt = __shfl_xor_sync(0xffffffffu, v.cnt, o);
  r.key = __shfl_xor_sync(0xffffffffu, v.key, o);
  r.idx = __shfl_xor_sync(0xffffffffu, v.idx, o);
  return r;
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

// One CTA per (row, chunk).  DEV: the variance's second pass (squared deviations from
// mean[row]).
template <int F, typename T, bool DEV>
__global__ void __launch_bounds__(AT) agg_part_kernel(const T* __restrict__ a, long long rows, long long m,
                                                      long long chunk_len, long long chunks,
                                                      const double* __restrict__ mean, Part* __restrict__ parts) {
  __shared__ Part warp_parts[AT / 32];
  const long long row = blockIdx.x / chunks, chunk = blockIdx.x - row * chunks;
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  const T* ar = a + row * m;
  const double mu = DEV ? mean[row] : 0.0;
  constexpr bool SEL = F == kMax || F == kMin || F == kArgMax || F == kArgMin;
  constexpr bool MINIMUM = F == kMin || F == kArgMin;
  Part p = none_part();
  for (long long c = c0 + threadIdx.x; c < c1; c += AT) {
    const T x = ar[c];
    if (is_nan(x)) continue;
    ++p.cnt;
    if (DEV) {
      const double d = static_cast<double>(x) - mu;
      p.s = fma(d, d, p.s);
    } else if (F == kSum || F == kMean || F == kVar || F == kStd) {
      if (IsFloat<T>::value) p.s += static_cast<double>(x);
      else p.i = static_cast<long long>(static_cast<unsigned long long>(p.i) + static_cast<unsigned long long>(x));
    } else if (SEL) {
      const unsigned long long k = MINIMUM ? ~sel_key(x) : sel_key(x);
      if (p.idx == kNone || k > p.key) {  // columns arrive in increasing order per thread
        p.key = k;
        p.idx = c;
      }
    }
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
    mean[row] = r.cnt > 0 ? r.s / static_cast<double>(r.cnt) : quiet_nan(0.0);
  }
}

template <int F, typename T, typename O>
__global__ void agg_finish_kernel(const T* __restrict__ a, const Part* __restrict__ parts, long long rows,
                                  long long m, long long chunks, long long ddof, O* __restrict__ out) {
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
      if (IsFloat<T>::value) res = static_cast<O>(r.s);
      else res = static_cast<O>(static_cast<T>(r.i));  // wraps to the input's width
    } else if (F == kMean) {
      res = static_cast<O>(r.cnt > 0 ? r.s / static_cast<double>(r.cnt) : quiet_nan(0.0));  // :93-103
    } else if (F == kVar || F == kStd) {
      // :113-133 / :143-159: sum of squared deviations / (count - ddof), NaN unless count > ddof
      double v = quiet_nan(0.0);
      if (r.cnt > ddof && r.cnt > 0) v = r.s / static_cast<double>(r.cnt - ddof);
      if (F == kStd) v = sqrt(v);
      res = static_cast<O>(v);
    } else if (F == kMax || F == kMin) {
      // :207-221 / :229-242: NaN where every element is NaN
      if (r.idx == kNone) res = static_cast<O>(quiet_nan(0.0));
      else res = static_cast<O>(a[row * m + r.idx]);
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
  agg_finish_kernel<F, T, O><<<fin_grid(rows), 256, 0, s>>>(a, parts, rows, m, p.chunks, ddof, out);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

}  // namespace agg
}  // namespace nbg

using namespace nbg;
using namespace nbg::agg;

extern "C" {

size_t nbg_aggregate_workspace_bytes(long long rows, long long m) { return workspace_bytes(rows, m); }

#define NBG_AGG(NAME, FN, T, O, SFX)                                                                   \
  int nbg_##NAME##_##SFX(const T* a, O* out, long long rows, long long m, void* ws, size_t ws_bytes,   \
                         void* stream) {                                                             \
    return launch<FN, T, O>(a, out, rows, m, 0, ws, ws_bytes, static_cast<cudaStream_t>(stream));     \
  }
#define NBG_AGG_DDOF(NAME, FN, T, SFX)                                                                 \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long m, long long ddof, void* ws,     \
                         size_t ws_bytes, void* stream) {                                            \
    return launch<FN, T, T>(a, out, rows, m, ddof, ws, ws_bytes, static_cast<cudaStream_t>(stream));  \
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
