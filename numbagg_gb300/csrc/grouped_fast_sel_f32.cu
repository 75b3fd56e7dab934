// group_nan{argmax,argmin,max,min,first,last} on float32 values (the kernels are in
// grouped_fast.cuh).
#include "grouped_fast.cuh"

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nanargmax, kArgMax, float, f32, float)
NBG_GFAST_LABELS(nanargmin, kArgMin, float, f32, float)
NBG_GFAST_LABELS(nanmax, kMax, float, f32, float)
NBG_GFAST_LABELS(nanmin, kMin, float, f32, float)
NBG_GFAST_LABELS(nanfirst, kFirst, float, f32, float)
NBG_GFAST_LABELS(nanlast, kLast, float, f32, float)
}  // extern "C"
