// group_nan{sum,count,mean,var,std,sum_of_squares} on float32 values (the kernels
// are in grouped_fast.cuh).
#include "grouped_fast.cuh"

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nansum, kSum, float, f32, float)
NBG_GFAST_LABELS(nancount, kCount, float, f32, float)
NBG_GFAST_LABELS(nanmean, kMean, float, f32, float)
NBG_GFAST_LABELS(nanvar, kVar, float, f32, float)
NBG_GFAST_LABELS(nanstd, kStd, float, f32, float)
NBG_GFAST_LABELS(nansum_of_squares, kSumSq, float, f32, float)
}  // extern "C"
