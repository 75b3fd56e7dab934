// Labelled reductions group_nan* (numbagg/grouped.py:7-270) along non-last axes, in
// place, for every function and values dtype (float64, float32, int32, int64).
//
// When the reduced axes are consecutive and not last, a C-contiguous array is `outer`
// blocks of m x `inner` values: position r of column i of block o sits at
// (o m + r) inner + i, and the labels run over r.  numbagg's gufunc walks each column's
// positions in order (np.ndindex over the core axes), so one thread per column runs
// that loop, with its per-label state in shared memory (slot k * NT + thread, so a
// warp's updates touch consecutive words) and the reference's arithmetic in the values'
// dtype: float sums rounded per addition, integer sums wrapping like numba's int64
// arithmetic stored into the narrow type, extremes compared as float64 with the first
// index kept on ties.  Consecutive threads read consecutive addresses at every step,
// nothing is copied, and the results are the reference's bit for bit.  The result for
// column (o, i) and label k lands at out[(o inner + i) K + k], the shape numbagg
// returns (the unreduced axes, then num_labels).  Labels < 0 or >= K are skipped.
#include "grouped_common.cuh"

#include <climits>

namespace nbg {
namespace gcols {

// function numbering shared with the row kernels (grouped_common.cuh)
using grouped::kAll;
using grouped::kAny;
using grouped::kArgMax;
using grouped::kArgMin;
using grouped::kCount;
using grouped::kFirst;
using grouped::kLast;
using grouped::kMax;
using grouped::kMean;
using grouped::kMin;
using grouped::kProd;
using grouped::kStd;
using grouped::kSum;
using grouped::kSumSq;
using grouped::kVar;
constexpr int NT = 128;

template <typename V>
struct Ar;  // the reference's arithmetic in the values dtype
template <>
struct Ar<double> {
  static NBG_DEVICE double add(double a, double b) { return __dadd_rn(a, b); }
  static NBG_DEVICE double mul(double a, double b) { return __dmul_rn(a, b); }
  static NBG_DEVICE bool isnan_(double v) { return is_nan(v); }
  static NBG_DEVICE double nan_out() { return __longlong_as_double(0x7ff8000000000000ll); }
};
template <>
struct Ar<float> {
  static NBG_DEVICE float add(float a, float b) { return __fadd_rn(a, b); }
  static NBG_DEVICE float mul(float a, float b) { return __fmul_rn(a, b); }
  static NBG_DEVICE bool isnan_(float v) { return is_nan(v); }
  static NBG_DEVICE float nan_out() { return __int_as_float(0x7fc00000); }
};
template <>
struct Ar<int> {
  static NBG_DEVICE int add(int a, int b) {
    return static_cast<int>(static_cast<unsigned>(static_cast<unsigned long long>(static_cast<long long>(a)) +
                                                  static_cast<unsigned long long>(static_cast<long long>(b))));
  }
  static NBG_DEVICE int mul(int a, int b) {
    return static_cast<int>(static_cast<unsigned>(static_cast<unsigned long long>(static_cast<long long>(a)) *
                                                  static_cast<unsigned long long>(static_cast<long long>(b))));
  }
  static NBG_DEVICE bool isnan_(int) { return false; }
  static NBG_DEVICE int nan_out() { return INT_MIN; }  // numba's NaN -> int conversion
};
template <>
struct Ar<long long> {
  static NBG_DEVICE long long add(long long a, long long b) {
    return static_cast<long long>(static_cast<unsigned long long>(a) + static_cast<unsigned long long>(b));
  }
  static NBG_DEVICE long long mul(long long a, long long b) {
    return static_cast<long long>(static_cast<unsigned long long>(a) * static_cast<unsigned long long>(b));
  }
  static NBG_DEVICE bool isnan_(long long) { return false; }
  static NBG_DEVICE long long nan_out() { return LLONG_MIN; }
};
template <typename V>
struct IsFloatV {
  static constexpr bool value = false;
};
template <>
struct IsFloatV<double> {
  static constexpr bool value = true;
};
template <>
struct IsFloatV<float> {
  static constexpr bool value = true;
};

// Up to three 8-byte words of state per (label, column) slot, each an array [K][NT]:
//   a: the running value in V (sums, products, counts, mean's and var's sums, first /
//      last values, any / all flags, the index of an extreme)
//   b: var's sum of squares in V, or an extreme's value as float64 (NaN: none yet)
//   c: the count of mean / var, or first's seen flag
template <int F>
struct Words {
  static constexpr bool B = F == kVar || F == kStd || F == kArgMax || F == kArgMin || F == kMax || F == kMin;
  static constexpr bool C = F == kMean || F == kVar || F == kStd || F == kFirst;
  static constexpr int n = 1 + (B ? 1 : 0) + (C ? 1 : 0);
};

template <int F, typename V, typename L>
__global__ void __launch_bounds__(NT) group_cols_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                        V* __restrict__ out, long long outer, long long m,
                                                        long long inner, int K, long long ddof) {
  using A = Ar<V>;
  using W = Words<F>;
  constexpr bool EXT = F == kArgMax || F == kArgMin || F == kMax || F == kMin;
  constexpr bool MAXI = F == kArgMax || F == kMax;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const size_t plane = static_cast<size_t>(K) * NT * 8;
  V* sa = reinterpret_cast<V*>(smem_raw);  // one V per 8-byte word
  double* sb = reinterpret_cast<double*>(smem_raw + plane);
  long long* sc = reinterpret_cast<long long*>(smem_raw + plane * (W::B ? 2 : 1));
  constexpr int SA = 8 / static_cast<int>(sizeof(V));
  const int tid = threadIdx.x;
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  for (int k = 0; k < K; ++k) {
    const int slot = k * NT + tid;
    V init = V(0);
    if (F == kProd || F == kAll) init = V(1);
    if (F == kLast) init = A::nan_out();
    sa[slot * SA] = init;
    if (W::B) sb[slot] = EXT ? qnan : 0.0;
    if (W::C) sc[slot] = 0;
  }
  const long long col = static_cast<long long>(blockIdx.x) * NT + tid;
  if (col >= outer * inner) return;
  const long long o = col / inner, i = col - o * inner;
  const V* vc = values + o * m * inner + i;
  // a ring of the next D positions' values and labels, so D loads are in flight while
  // one position is reduced (a thread's walk is serial: the ring is its parallelism)
  constexpr int D = 8;
  V ring[D];
  int lring[D];  // the label, or -1 where it is skipped
  auto label_at = [&](long long r) {
    const long long l = static_cast<long long>(__ldg(labels + r));
    return (l < 0 || l >= K) ? -1 : static_cast<int>(l);
  };
#pragma unroll
  for (int d = 0; d < D; ++d) {
    ring[d] = d < m ? __ldg(vc + d * inner) : V(0);
    lring[d] = d < m ? label_at(d) : -1;
  }
  for (long long r0 = 0; r0 < m; r0 += D) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const long long r = r0 + d;
      if (r >= m) break;
      const V x = ring[d];
      const int lab = lring[d];
      if (r + D < m) {
        ring[d] = __ldg(vc + (r + D) * inner);
        lring[d] = label_at(r + D);
      }
      if (lab < 0) continue;
      if (A::isnan_(x)) continue;
      const int slot = lab * NT + tid;
      V& a = sa[slot * SA];
      if (F == kSum) a = A::add(a, x);
      if (F == kSumSq) a = A::add(a, A::mul(x, x));
      if (F == kProd) a = A::mul(a, x);
      if (F == kCount) a = A::add(a, V(1));
      if (F == kMean || F == kVar || F == kStd) {
        a = A::add(a, x);
        sc[slot] += 1;
        if (F != kMean) {  // var's sum of squares in V, kept in the float64 word
          V* q = reinterpret_cast<V*>(sb + slot);
          *q = A::add(*q, A::mul(x, x));
        }
      }
      if (EXT) {  // numbagg/grouped.py:54-92, :211-244: float64 comparison, first index on ties
        const double xd = static_cast<double>(x);
        const double e = sb[slot];
        if (is_nan(e) || (MAXI ? xd > e : xd < e)) {
          sb[slot] = xd;
          if (F == kArgMax || F == kArgMin) a = static_cast<V>(r);
        }
      }
      if (F == kFirst && sc[slot] == 0) {
        sc[slot] = 1;
        a = x;
      }
      if (F == kLast) a = x;
      if (F == kAny && x != V(0)) a = V(1);
      if (F == kAll && x == V(0)) a = V(0);
    }
  }
  V* oc = out + col * K;
  for (int k = 0; k < K; ++k) {
    const int slot = k * NT + tid;
    const V a = sa[slot * SA];
    V res = a;
    if (F == kMean) {  // numbagg/grouped.py:22-27: the float64 quotient, stored in V
      const long long c = sc[slot];
      res = c == 0 ? A::nan_out() : static_cast<V>(static_cast<double>(a) / static_cast<double>(c));
    }
    if (F == kVar || F == kStd) {  // numbagg/grouped.py:170-176, :199-208
      const long long c = sc[slot];
      const long long denom = c - ddof;
      res = A::nan_out();
      if (denom > 0) {
        const V s2 = A::mul(a, a);
        const V sq = *reinterpret_cast<const V*>(sb + slot);
        double v = __ddiv_rn(__dsub_rn(static_cast<double>(sq), __ddiv_rn(static_cast<double>(s2), static_cast<double>(c))),
                             static_cast<double>(denom));
        if (F == kStd) v = __dsqrt_rn(v);
        res = static_cast<V>(v);
      }
    }
    if (EXT) {
      const double e = sb[slot];
      if (is_nan(e)) res = A::nan_out();
      else if (F == kMax || F == kMin) res = static_cast<V>(e);
    }
    if (F == kFirst && sc[slot] == 0) res = IsFloatV<V>::value ? A::nan_out() : V(0);
    oc[k] = res;
  }
}

// shared memory for K labels (bytes)
inline size_t cols_smem(int F, long long K) {
  int words = 1;
  switch (F) {
    case kMean: words = Words<kMean>::n; break;
    case kVar: words = Words<kVar>::n; break;
    case kStd: words = Words<kStd>::n; break;
    case kArgMax: case kArgMin: case kMax: case kMin: words = Words<kMax>::n; break;
    case kFirst: words = Words<kFirst>::n; break;
    default: break;
  }
  return static_cast<size_t>(K) * NT * 8 * words;
}

}  // namespace gcols
}  // namespace nbg

using namespace nbg;
using namespace nbg::gcols;

namespace {
constexpr size_t kColsSmemMax = 96 * 1024;

template <int F, typename V, typename L>
int launch_group_cols(const V* values, const L* labels, V* out, long long outer, long long m, long long inner,
                      long long K, long long ddof, cudaStream_t s) {
  if (outer < 0 || m < 0 || inner < 0 || K < 0) return kInvalidArgument;
  if (outer == 0 || inner == 0 || K == 0) return kOk;
  if (!out || (m > 0 && (!values || !labels))) return kInvalidArgument;
  const size_t smem = cols_smem(F, K);
  if (smem > kColsSmemMax) return kUnsupported;  // the caller moves the axes last instead
  const long long blocks = (outer * inner + NT - 1) / NT;
  if (blocks > 0x7fffffffLL) return kUnsupported;
  auto kern = group_cols_kernel<F, V, L>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  kern<<<static_cast<int>(blocks), NT, smem, s>>>(values, labels, out, outer, m, inner, static_cast<int>(K), ddof);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_group_cols_max_labels(int func) {
  if (func < 0 || func >= grouped::kNumFuncs) return 0;
  return kColsSmemMax / cols_smem(func, 1);
}

#define NBG_GROUP_COLS1(NAME, FN, V, VS, L, LS)                                                      \
  int nbg_group_##NAME##_cols_##VS##_##LS(const V* values, const L* labels, V* out, long long outer,  \
                                          long long m, long long inner, long long K, long long ddof,  \
                                          void* stream) {                                            \
    return launch_group_cols<FN, V, L>(values, labels, out, outer, m, inner, K, ddof,                \
                                       static_cast<cudaStream_t>(stream));                           \
  }
#define NBG_GROUP_COLS_L(NAME, FN, V, VS) NBG_GROUP_COLS1(NAME, FN, V, VS, int, i32) NBG_GROUP_COLS1(NAME, FN, V, VS, long long, i64)
#define NBG_GROUP_COLS_FLOAT(NAME, FN) NBG_GROUP_COLS_L(NAME, FN, double, f64) NBG_GROUP_COLS_L(NAME, FN, float, f32)
#define NBG_GROUP_COLS_ALL(NAME, FN) \
  NBG_GROUP_COLS_FLOAT(NAME, FN) NBG_GROUP_COLS_L(NAME, FN, int, i32) NBG_GROUP_COLS_L(NAME, FN, long long, i64)
NBG_GROUP_COLS_ALL(nansum, kSum)
NBG_GROUP_COLS_ALL(nancount, kCount)
NBG_GROUP_COLS_FLOAT(nanmean, kMean)
NBG_GROUP_COLS_FLOAT(nanvar, kVar)
NBG_GROUP_COLS_FLOAT(nanstd, kStd)
NBG_GROUP_COLS_ALL(nansum_of_squares, kSumSq)
NBG_GROUP_COLS_ALL(nanprod, kProd)
NBG_GROUP_COLS_ALL(nanargmax, kArgMax)
NBG_GROUP_COLS_ALL(nanargmin, kArgMin)
NBG_GROUP_COLS_ALL(nanmax, kMax)
NBG_GROUP_COLS_ALL(nanmin, kMin)
NBG_GROUP_COLS_ALL(nanfirst, kFirst)
NBG_GROUP_COLS_ALL(nanlast, kLast)
NBG_GROUP_COLS_ALL(nanany, kAny)
NBG_GROUP_COLS_ALL(nanall, kAll)

}  // extern "C"
