// group_nan{argmax,argmin,max,min,first,last} on int32 values, the ragged
// grouped entry points and the fast paths' workspace query (the kernels are in
// grouped_fast.cuh).
#include "grouped_fast.cuh"

namespace nbg {
namespace grouped {
size_t fast_bytes_query(int f, long long rows, long long m, long long K) {
  if (!(is_moments(f) || is_select(f) || f == kFirst || f == kLast)) return 0;
  return fast_bytes(f, rows, m, K);
}
}  // namespace grouped
}  // namespace nbg

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nanargmax, kArgMax, int, i32, int)
NBG_GFAST_LABELS(nanargmin, kArgMin, int, i32, int)
NBG_GFAST_LABELS(nanmax, kMax, int, i32, int)
NBG_GFAST_LABELS(nanmin, kMin, int, i32, int)
NBG_GFAST_LABELS(nanfirst, kFirst, int, i32, int)
NBG_GFAST_LABELS(nanlast, kLast, int, i32, int)

// Ragged series with their own labels: values, labels: `total` values in series
// s = [offsets[s], offsets[s + 1]); out: nseries x num_labels (float64).
size_t nbg_group_ragged_workspace_bytes(long long nseries, long long total, long long num_labels) {
  return ragged_group_bytes(nseries < 0 ? 0 : nseries, total < 0 ? 0 : total, num_labels < 0 ? 0 : num_labels);
}
#define NBG_GRAGGED(NAME, FC, L, LS)                                                                 \
  int nbg_group_##NAME##_ragged_f64_##LS(const double* values, const L* labels, const long long* offsets, \
                                         long long nseries, long long total, long long num_labels,       \
                                         double* out, void* ws, size_t ws_bytes, void* stream) {         \
    return launch_ragged_group<FC, L>(values, labels, offsets, nseries, total, num_labels, out, ws,      \
                                      ws_bytes, static_cast<cudaStream_t>(stream));                      \
  }
NBG_GRAGGED(nansum, kSum, int, i32)
NBG_GRAGGED(nansum, kSum, long long, i64)
NBG_GRAGGED(nanmean, kMean, int, i32)
NBG_GRAGGED(nanmean, kMean, long long, i64)
NBG_GRAGGED(nancount, kCount, int, i32)
NBG_GRAGGED(nancount, kCount, long long, i64)
}  // extern "C"
