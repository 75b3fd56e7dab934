// group_nan{sum,count,mean,var,std,sum_of_squares} on float64 values (the kernels
// are in grouped_fast.cuh).
#include "grouped_fast.cuh"

using namespace nbg::grouped;

extern "C" {
NBG_GFAST_LABELS(nansum, kSum, double, f64, double)
NBG_GFAST_LABELS(nancount, kCount, double, f64, double)
NBG_GFAST_LABELS(nanmean, kMean, double, f64, double)
NBG_GFAST_LABELS(nanvar, kVar, double, f64, double)
NBG_GFAST_LABELS(nanstd, kStd, double, f64, double)
NBG_GFAST_LABELS(nansum_of_squares, kSumSq, double, f64, double)
}  // extern "C"
