// group_nan{argmax,argmin,max,min,first,last} on int64 values (the kernels are in
// grouped_fast.cuh).
#include "grouped_fast.cuh"

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nanargmax, kArgMax, long long, i64, long long)
NBG_GFAST_LABELS(nanargmin, kArgMin, long long, i64, long long)
NBG_GFAST_LABELS(nanmax, kMax, long long, i64, long long)
NBG_GFAST_LABELS(nanmin, kMin, long long, i64, long long)
NBG_GFAST_LABELS(nanfirst, kFirst, long long, i64, long long)
NBG_GFAST_LABELS(nanlast, kLast, long long, i64, long long)
}  // extern "C"
