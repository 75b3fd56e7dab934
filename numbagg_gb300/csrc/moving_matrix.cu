// move_covmatrix / move_corrmatrix (numbagg/moving_matrix.py:16-201).
//
// Input (batch, T, V), output (batch, T, V, V).  For every pair (i, j) the reference
// keeps pairwise-complete rolling sums over the rows where both a[t, i] and a[t, j]
// are valid: sums_i, sums_j, prods (+ sums_sq_i / sums_sq_j for the correlation) and
// an int64 pair count, adding the entering row and removing the leaving one.
//
// Here a CTA owns one matrix row i, 256 columns j and one time segment.  It seeds the
// window state at the segment start by direct summation of the `window` rows before
// it (so rounding cannot drift across segments), then rolls forward through the
// segment writing one output row per step: out[t, i, j0:j0+256] is a coalesced store.
// The input rows are re-read by the V CTAs of a segment from L2.  Accumulation is in
// float64; the finalisation follows the reference's formulas with divisions by the
// count done through a reciprocal table and Markstein's correction.
#include "nbg_common.cuh"

namespace nbg {
namespace mmatrix {

constexpr int NT = 256;
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

template <typename T, bool CORR>
__global__ void __launch_bounds__(NT) matrix_kernel(const T* __restrict__ a, T* __restrict__ out,
                                                    long long n_obs, long long n_vars,
                                                    long long window, long long min_count,
                                                    long long seg_len, long long n_seg,
                                                    long long jblocks) {
  __shared__ double rcp[kRcp];
  for (int c = threadIdx.x; c < kRcp; c += NT) rcp[c] = c ? 1.0 / static_cast<double>(c) : 0.0;
  __syncthreads();
  long long bid = blockIdx.x;
  const long long jb = bid % jblocks;
  bid /= jblocks;
  const long long i = bid % n_vars;
  bid /= n_vars;
  const long long seg = bid % n_seg;
  const long long batch = blockIdx.y;
  const long long j = jb * NT + threadIdx.x;
  const bool active = j < n_vars;
  const long long jj = active ? j : 0;
  const T* ab = a + batch * n_obs * n_vars;
  T* ob = out + batch * n_obs * n_vars * n_vars;
  const long long t0 = seg * seg_len;
  long long t1 = t0 + seg_len;
  if (t1 > n_obs) t1 = n_obs;
  const long long mc = min_count > 1 ? min_count : 1;
  const long long mc2 = mc > 2 ? mc : 2;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);

  double si = 0, sj = 0, pr = 0, qi = 0, qj = 0;
  long long cnt = 0;
  long long ts = t0 - window;
  if (ts < 0) ts = 0;
  // seed: the window at t0 - 1 holds rows [t0 - window, t0 - 1]
  for (long long t = ts; t < t0; ++t) {
    const T vi = ab[t * n_vars + i], vj = ab[t * n_vars + jj];
    if (!is_nan(vi) && !is_nan(vj)) {
      const double x = static_cast<double>(vi), y = static_cast<double>(vj);
      si += x; sj += y; pr += x * y;
      if (CORR) { qi += x * x; qj += y * y; }
      ++cnt;
    }
  }
  for (long long t = t0; t < t1; ++t) {
    if (t >= window) {
      const long long to = t - window;
      const T vi = ab[to * n_vars + i], vj = ab[to * n_vars + jj];
      if (!is_nan(vi) && !is_nan(vj)) {
        const double x = static_cast<double>(vi), y = static_cast<double>(vj);
        si -= x; sj -= y; pr -= x * y;
        if (CORR) { qi -= x * x; qj -= y * y; }
        --cnt;
      }
    }
    {
      const T vi = ab[t * n_vars + i], vj = ab[t * n_vars + jj];
      if (!is_nan(vi) && !is_nan(vj)) {
        const double x = static_cast<double>(vi), y = static_cast<double>(vj);
        si += x; sj += y; pr += x * y;
        if (CORR) { qi += x * x; qj += y * y; }
        ++cnt;
      }
    }
    double r = nan;
    if (!CORR) {
      // numbagg/moving_matrix.py:189-201
      if (cnt >= mc && cnt > 1) {
        const double mi = div_count(si, cnt, rcp), mj = div_count(sj, cnt, rcp);
        const double cov = div_count((div_count(pr, cnt, rcp) - mi * mj) * static_cast<double>(cnt), cnt - 1, rcp);
        r = cov;
      }
    } else {
      // numbagg/moving_matrix.py:92-114
      if (cnt >= mc2) {
        const double mi = div_count(si, cnt, rcp), mj = div_count(sj, cnt, rcp);
        const double vi = div_count(qi, cnt, rcp) - mi * mi;
        const double vj = div_count(qj, cnt, rcp) - mj * mj;
        const double cv = div_count(pr, cnt, rcp) - mi * mj;
        if (vi > 0 && vj > 0) r = cv / sqrt(vi * vj);
      }
    }
    if (active) ob[(t * n_vars + i) * n_vars + j] = static_cast<T>(r);
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
  if (!a || !out || batch > 65535) return kInvalidArgument;
  long long seg_len = window * 4;
  if (seg_len < 256) seg_len = 256;
  const long long n_seg = (n_obs + seg_len - 1) / seg_len;
  const long long jblocks = (n_vars + NT - 1) / NT;
  const long long gx = n_seg * n_vars * jblocks;
  if (gx > 0x7fffffffll) return kUnsupported;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(batch));
  matrix_kernel<T, CORR><<<grid, NT, 0, s>>>(a, out, n_obs, n_vars, window, min_count, seg_len, n_seg, jblocks);
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
