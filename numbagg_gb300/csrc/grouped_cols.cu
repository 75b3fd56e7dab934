// Labelled reductions along a non-last axis, in place: group_nansum, group_nanmean,
// group_nancount, group_nanvar, group_nanstd (numbagg/grouped.py:7-51, :148-208) of
// float64 values whose reduced axes are consecutive and not last.
//
// A C-contiguous array is then `outer` blocks of m x `inner` values: position r of
// column i of block o sits at (o m + r) inner + i, and the labels run over r.  numbagg's
// gufunc walks each column's positions in order (np.ndindex over the core axes), so one
// thread per column runs that loop: its per-label sums, sums of squares and counts sit
// in shared memory (slot k * NT + thread, so a warp's updates touch consecutive words),
// consecutive threads read consecutive addresses at every step, and every sum is taken
// in the reference's order with its float64 operations: the results are numbagg's bit
// for bit.  The result for column (o, i) and label k lands at out[(o inner + i) K + k],
// the shape numbagg returns (the unreduced axes, then num_labels).
#include "nbg_common.cuh"

namespace nbg {
namespace gcols {

enum Fn : int { kSum = 0, kMean, kCount, kVar, kStd };
constexpr int NT = 128;

template <int F, typename L>
__global__ void __launch_bounds__(NT) group_cols_kernel(const double* __restrict__ values, const L* __restrict__ labels,
                                                        double* __restrict__ out, long long outer, long long m,
                                                        long long inner, int K, long long ddof) {
  constexpr bool S2 = F == kVar || F == kStd;
  constexpr bool CNT = F != kSum;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s1 = reinterpret_cast<double*>(smem_raw);                                  // [K][NT]
  double* s2 = reinterpret_cast<double*>(smem_raw + static_cast<size_t>(K) * NT * 8);  // [K][NT] (var)
  long long* cn = reinterpret_cast<long long*>(smem_raw + static_cast<size_t>(K) * NT * (S2 ? 16 : 8));
  const int tid = threadIdx.x;
  for (int k = 0; k < K; ++k) {
    s1[k * NT + tid] = 0.0;
    if (S2) s2[k * NT + tid] = 0.0;
    if (CNT) cn[k * NT + tid] = 0;
  }
  const long long col = static_cast<long long>(blockIdx.x) * NT + tid;
  const bool live = col < outer * inner;
  if (live) {
    const long long o = col / inner, i = col - o * inner;
    const double* vc = values + o * m * inner + i;
    for (long long r = 0; r < m; ++r) {
      const long long lab = static_cast<long long>(__ldg(labels + r));
      if (lab < 0 || lab >= K) continue;
      const double x = __ldg(vc + r * inner);
      if (is_nan(x)) continue;
      const int slot = static_cast<int>(lab) * NT + tid;
      if (F == kCount) {
        cn[slot] += 1;
        continue;
      }
      s1[slot] = __dadd_rn(s1[slot], x);
      if (CNT) cn[slot] += 1;
      if (S2) s2[slot] = __dadd_rn(s2[slot], __dmul_rn(x, x));
    }
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    double* oc = out + col * K;
    for (int k = 0; k < K; ++k) {
      const int slot = k * NT + tid;
      double r;
      if (F == kSum) {
        r = s1[slot];
      } else if (F == kCount) {
        r = static_cast<double>(cn[slot]);
      } else if (F == kMean) {  // numbagg/grouped.py:22-27
        const long long c = cn[slot];
        r = c == 0 ? nan : __ddiv_rn(s1[slot], static_cast<double>(c));
      } else {  // numbagg/grouped.py:170-176, :199-208
        const long long c = cn[slot];
        const long long denom = c - ddof;
        r = nan;
        if (denom > 0) {
          const double s = s1[slot];
          r = __ddiv_rn(__dsub_rn(s2[slot], __ddiv_rn(__dmul_rn(s, s), static_cast<double>(c))),
                        static_cast<double>(denom));
          if (F == kStd) r = __dsqrt_rn(r);
        }
      }
      oc[k] = r;
    }
  }
}

// shared memory for K labels (bytes), the launch refuses more than the opt-in limit
inline size_t cols_smem(int F, long long K) {
  const size_t per = (F == kVar || F == kStd) ? 24 : (F == kSum ? 8 : 16);
  return static_cast<size_t>(K) * NT * per;
}

}  // namespace gcols
}  // namespace nbg

using namespace nbg;
using namespace nbg::gcols;

namespace {
constexpr size_t kColsSmemMax = 96 * 1024;

template <int F, typename L>
int launch_group_cols(const double* values, const L* labels, double* out, long long outer, long long m,
                      long long inner, long long K, long long ddof, cudaStream_t s) {
  if (outer < 0 || m < 0 || inner < 0 || K < 0) return kInvalidArgument;
  if (outer == 0 || inner == 0 || K == 0) return kOk;
  if (!out || (m > 0 && (!values || !labels))) return kInvalidArgument;
  const size_t smem = cols_smem(F, K);
  if (smem > kColsSmemMax) return kUnsupported;  // the caller moves the axes last instead
  const long long blocks = (outer * inner + NT - 1) / NT;
  if (blocks > 0x7fffffffLL) return kUnsupported;
  auto kern = group_cols_kernel<F, L>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  kern<<<static_cast<int>(blocks), NT, smem, s>>>(values, labels, out, outer, m, inner, static_cast<int>(K), ddof);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_group_cols_max_labels(int func) {
  if (func < 0 || func > kStd) return 0;
  return kColsSmemMax / cols_smem(func, 1);
}

#define NBG_GROUP_COLS(NAME, FN)                                                                     \
  int nbg_group_##NAME##_cols_f64_i32(const double* values, const int* labels, double* out, long long outer, \
                                      long long m, long long inner, long long K, long long ddof, void* stream) { \
    return launch_group_cols<FN, int>(values, labels, out, outer, m, inner, K, ddof,                 \
                                      static_cast<cudaStream_t>(stream));                            \
  }                                                                                                  \
  int nbg_group_##NAME##_cols_f64_i64(const double* values, const long long* labels, double* out,      \
                                      long long outer, long long m, long long inner, long long K,     \
                                      long long ddof, void* stream) {                                 \
    return launch_group_cols<FN, long long>(values, labels, out, outer, m, inner, K, ddof,           \
                                            static_cast<cudaStream_t>(stream));                      \
  }
NBG_GROUP_COLS(nansum, kSum)
NBG_GROUP_COLS(nanmean, kMean)
NBG_GROUP_COLS(nancount, kCount)
NBG_GROUP_COLS(nanvar, kVar)
NBG_GROUP_COLS(nanstd, kStd)

}  // extern "C"
