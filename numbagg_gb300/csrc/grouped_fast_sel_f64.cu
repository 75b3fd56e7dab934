// group_nan{argmax,argmin,max,min,first,last} on float64 values (the kernels are in
// grouped_fast.cuh).
#include "grouped_fast.cuh"

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nanargmax, kArgMax, double, f64, double)
NBG_GFAST_LABELS(nanargmin, kArgMin, double, f64, double)
NBG_GFAST_LABELS(nanmax, kMax, double, f64, double)
NBG_GFAST_LABELS(nanmin, kMin, double, f64, double)
NBG_GFAST_LABELS(nanfirst, kFirst, double, f64, double)
NBG_GFAST_LABELS(nanlast, kLast, double, f64, double)
}  // extern "C"
