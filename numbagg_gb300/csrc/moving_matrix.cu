// move_covmatrix / move_corrmatrix (numbagg/moving_matrix.py:16-201).
//
// Input (batch, T, V), output (batch, T, V, V).  For every pair (i, j) the reference
// keeps pairwise-complete rolling sums over the rows where both a[t, i] and a[t, j]
// are valid: sums_i, sums_j, prods (+ sums_sq_i / sums_sq_j for the correlation) and
// an int64 pair count, adding the entering row and removing the leaving one.
//
// The accumulators are in the input dtype, as the reference's (numbagg/moving_matrix.py:
// 149-152): float32 arrays accumulate in float32, so the float32 kernel runs on the
// FP32 pipes and is bound by its output write (T x V x V values), not by the FP64 pipe.
#include "nbg_common.cuh"

namespace nbg {
namespace mmatrix {

constexpr int NT = 256;   // columns j of one CTA
constexpr int IB = 8;     // rows i of one CTA: an input row loaded once serves IB outputs
constexpr int kRcp = 1024;

NBG_DEVICE double div_count(double s, long long c, const double* rcp) {
  if (c < kRcp && isfinite(s)) {
    const double r = rcp[c];
    const double q0 = s * r;
    const double e = fma(-q0, static_cast<double>(c), s);
    return fma(e, r, q0);
  }
  return s / static_cast<double>(c);
}

// the reference's products and sums in the input dtype, each rounded on its own
NBG_DEVICE double mul_t(double x, double y) { return __dmul_rn(x, y); }
NBG_DEVICE float mul_t(float x, float y) { return __fmul_rn(x, y); }
NBG_DEVICE double add_t(double x, double y) { return __dadd_rn(x, y); }
NBG_DEVICE float add_t(float x, float y) { return __fadd_rn(x, y); }
NBG_DEVICE double sub_t(double x, double y) { return __dsub_rn(x, y); }
NBG_DEVICE float sub_t(float x, float y) { return __fsub_rn(x, y); }

// Finalisation, numbagg/moving_matrix.py:189-201 (cov) and :92-114 (corr).  float64
// arrays: the reference's float64 formulas, divisions correctly rounded.  float32
// arrays: the accumulators are float32 as in the reference, and the finalisation runs
// in float32 with reciprocals from a table (the reference finalises in float64 from
// the same float32 accumulators; the two differ by a few float32 rounding steps,
// far below the accumulators' own error).
template <bool CORR>
NBG_DEVICE double finish(double si, double sj, double pr, double qi, double qj, long long nn, long long mc,
                         const double* rcp) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (!CORR) {
    if (!(nn >= mc && nn > 1)) return nan;
    const double mi = div_count(si, nn, rcp), mj = div_count(sj, nn, rcp);
    return div_count((div_count(pr, nn, rcp) - mi * mj) * static_cast<double>(nn), nn - 1, rcp);
  }
  if (nn < (mc > 2 ? mc : 2)) return nan;
  const double mi = div_count(si, nn, rcp), mj = div_count(sj, nn, rcp);
  const double vi = div_count(qi, nn, rcp) - mi * mi;
  const double vj = div_count(qj, nn, rcp) - mj * mj;
  const double cv = div_count(pr, nn, rcp) - mi * mj;
  return (vi > 0 && vj > 0) ? cv / sqrt(vi * vj) : nan;
}
template <bool CORR>
NBG_DEVICE float finish(float si, float sj, float pr, float qi, float qj, long long nn, long long mc,
                        const float* rcp) {
  const float nan = __int_as_float(0x7fc00000);
  if (!CORR) {
    if (!(nn >= mc && nn > 1)) return nan;
    const float rn = nn < kRcp ? rcp[nn] : 1.0f / static_cast<float>(nn);
    const float rm = nn - 1 < kRcp ? rcp[nn - 1] : 1.0f / static_cast<float>(nn - 1);
    const float mi = si * rn, mj = sj * rn;
    const float p = __fmul_rn(mi, mj);  // subtracted exactly, as in the correlation below
    const float c = __fsub_rn(__fmaf_rn(pr, rn, -p), __fmaf_rn(mi, mj, -p));
    return c * (static_cast<float>(nn) * rm);
  }
  if (nn < (mc > 2 ? mc : 2)) return nan;
  const float rn = nn < kRcp ? rcp[nn] : 1.0f / static_cast<float>(nn);
  const float mi = si * rn, mj = sj * rn;
  // q * rn - m * m with the product subtracted exactly (its rounding error recovered by
  // an FMA), so the cancellation at small counts costs no extra digits
  auto diff = [](float q, float r, float x, float y) {
    const float p = __fmul_rn(x, y);
    const float e = __fmaf_rn(x, y, -p);
    return __fsub_rn(__fmaf_rn(q, r, -p), e);
  };
  const float vi = diff(qi, rn, mi, mi);
  const float vj = diff(qj, rn, mj, mj);
  const float cv = diff(pr, rn, mi, mj);
  return (vi > 0.0f && vj > 0.0f) ? cv * rsqrtf(vi * vj) : nan;
}

template <typename T>
NBG_DEVICE T rcp_entry(int c);
template <>
NBG_DEVICE double rcp_entry<double>(int c) { return c ? 1.0 / static_cast<double>(c) : 0.0; }
template <>
NBG_DEVICE float rcp_entry<float>(int c) { return c ? 1.0f / static_cast<float>(c) : 0.0f; }

// A CTA owns rows i0..i0+IB-1 of the matrix, NT columns j and one time segment.  It
// seeds the window state at the segment start by direct summation of the `window`
// rows before it (so rounding drift does not cross segments), then rolls forward
// through the segment: per step, the leaving row is removed and the entering row
// added to the IB x NT pair states (each thread holds IB of them), and IB output rows
// out[t, i, j0:j0+NT] are written with coalesced streaming stores.
template <typename T, bool CORR>
__global__ void __launch_bounds__(NT) matrix_kernel(const T* __restrict__ a, T* __restrict__ out,
                                                    long long n_obs, long long n_vars,
                                                    long long window, long long min_count,
                                                    long long seg_len, long long n_seg,
                                                    long long jblocks, long long iblocks) {
  __shared__ T rcp[kRcp];
  for (int c = threadIdx.x; c < kRcp; c += NT) rcp[c] = rcp_entry<T>(c);
  __syncthreads();
  long long bid = blockIdx.x;
  const long long jb = bid % jblocks;
  bid /= jblocks;
  const long long ib = bid % iblocks;
  bid /= iblocks;
  const long long seg = bid % n_seg;
  const long long batch = blockIdx.y;
  const long long j = jb * NT + threadIdx.x;
  const bool active = j < n_vars;
  const long long jj = active ? j : 0;
  const long long i0 = ib * IB;
  const T* ab = a + batch * n_obs * n_vars;
  T* ob = out + batch * n_obs * n_vars * n_vars;
  const long long t0 = seg * seg_len;
  const long long t1 = t0 + seg_len < n_obs ? t0 + seg_len : n_obs;
  const long long mc = min_count > 1 ? min_count : 1;

  T si[IB], sj[IB], pr[IB], qi[IB], qj[IB];
  int cnt[IB];
#pragma unroll
  for (int r = 0; r < IB; ++r) {
    si[r] = sj[r] = pr[r] = qi[r] = qj[r] = T(0);
    cnt[r] = 0;
  }
  const bool whole = i0 + IB <= n_vars;  // every row of the block exists (uniform)
  auto update = [&](long long t, bool add) {
    const T* row = ab + t * n_vars;
    const T vj = row[jj];
    if (is_nan(vj)) return;
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      if (!whole && i0 + r >= n_vars) break;
      const T vi = __ldg(row + i0 + r);
      if (is_nan(vi)) continue;
      if (add) {
        si[r] = add_t(si[r], vi);
        sj[r] = add_t(sj[r], vj);
        pr[r] = add_t(pr[r], mul_t(vi, vj));
        if (CORR) {
          qi[r] = add_t(qi[r], mul_t(vi, vi));
          qj[r] = add_t(qj[r], mul_t(vj, vj));
        }
        ++cnt[r];
      } else {
        si[r] = sub_t(si[r], vi);
        sj[r] = sub_t(sj[r], vj);
        pr[r] = sub_t(pr[r], mul_t(vi, vj));
        if (CORR) {
          qi[r] = sub_t(qi[r], mul_t(vi, vi));
          qj[r] = sub_t(qj[r], mul_t(vj, vj));
        }
        --cnt[r];
      }
    }
  };
  // seed: the window at t0 - 1 holds rows [t0 - window, t0 - 1]
  for (long long t = (t0 > window ? t0 - window : 0); t < t0; ++t) update(t, true);
  for (long long t = t0; t < t1; ++t) {
    if (t >= window) update(t - window, false);
    update(t, true);
    T* o = ob + (t * n_vars + i0) * n_vars + j;
#pragma unroll
    for (int r = 0; r < IB; ++r, o += n_vars) {
      if (!whole && i0 + r >= n_vars) break;
      const T res = finish<CORR>(si[r], sj[r], pr[r], qi[r], qj[r], cnt[r], mc, rcp);
      if (active) __stcs(o, res);
    }
  }
}

}  // namespace mmatrix
}  // namespace nbg

using namespace nbg;
using namespace nbg::mmatrix;

namespace {
template <typename T, bool CORR>
int launch_matrix(const T* a, T* out, long long batch, long long n_obs, long long n_vars,
                  long long window, long long min_count, cudaStream_t s) {
  if (batch < 0 || n_obs < 0 || n_vars < 0 || window <= 0 || min_count < 0) return kInvalidArgument;
  if (batch == 0 || n_obs == 0 || n_vars == 0) return kOk;
  if (!a || !out || batch > 65535 || window > 0x7fffffffll) return kInvalidArgument;
  const long long jblocks = (n_vars + NT - 1) / NT;
  const long long iblocks = (n_vars + IB - 1) / IB;
  // segments of at least 8 windows (each re-reads one window to seed), fewer when the
  // grid would not cover the GPU twice
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long seg_len = window * 8 > 256 ? window * 8 : 256;
  while (seg_len > 256 && batch * iblocks * jblocks * ((n_obs + seg_len - 1) / seg_len) < 4LL * sms) seg_len /= 2;
  const long long n_seg = (n_obs + seg_len - 1) / seg_len;
  const long long gx = n_seg * iblocks * jblocks;
  if (gx > 0x7fffffffll) return kUnsupported;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(batch));
  matrix_kernel<T, CORR><<<grid, NT, 0, s>>>(a, out, n_obs, n_vars, window, min_count, seg_len, n_seg, jblocks,
                                             iblocks);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {
#define NBG_MATRIX(NAME, CORR, T, SFX)                                                          \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long batch, long long n_obs, long long n_vars,  \
                         long long window, long long min_count, void* stream) {                  \
    return launch_matrix<T, CORR>(a, out, batch, n_obs, n_vars, window, min_count,               \
                                  static_cast<cudaStream_t>(stream));                           \
  }
NBG_MATRIX(move_covmatrix, false, double, f64)
NBG_MATRIX(move_covmatrix, false, float, f32)
NBG_MATRIX(move_corrmatrix, true, double, f64)
NBG_MATRIX(move_corrmatrix, true, float, f32)
}
