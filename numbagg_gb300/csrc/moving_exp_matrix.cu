// move_exp_nancovmatrix / move_exp_nancorrmatrix (numbagg/moving_matrix.py:204-432).
//
// Input (batch, T, V), alpha (T per batch entry, or shared), output (batch, T, V, V).
// Every pair (i, j) keeps exponentially decayed, pairwise-complete states: sums_i,
// sums_j, prods (+ sums_sq_i, sums_sq_j for the correlation), the alpha weight, the
// decayed count and the count decayed by decay^2.  Each step multiplies every state
// by decay = 1 - alpha_t (decay^2 for the last) and adds the step's row where both
// a[t, i] and a[t, j] are valid.
//
// Every state is an affine recurrence s_t = d_t s_{t-1} + x_t, so time is split into
// segments scanned in parallel:
//   pass 0: each segment is scanned from zero states; its end states (the segment's
//           aggregate) go to the workspace, and the products of its decays (d and d^2)
//           are written once per (batch, segment);
//   pass 1: each segment folds the aggregates of the segments before it, in order,
//           into its carry-in (C = D_m C + S_m), scans again from that carry and
//           writes its outputs.
// The output (T x V x V values) is written once; the input is read twice.
// float64 arrays keep float64 states (the reference's typing); float32 arrays keep
// float32 states, with the decay rounded to float32 (numba multiplies by a float64
// decay and rounds to float32: a difference of at most one float32 rounding per step).
#include "nbg_common.cuh"

namespace nbg {
namespace ematrix {

constexpr int NT = 128;  // columns j of one CTA

// pair rows i per thread: fewer for float64 (twice the registers per state) and for
// the correlation (eight states instead of six)
template <typename T, bool CORR>
struct Rows {
  static constexpr int value = (sizeof(T) == 8 ? 4 : 8) / (CORR ? 2 : 1);
};

template <bool CORR>
struct NStates {
  static constexpr int value = CORR ? 8 : 6;  // si, sj, pr, pw, sw, sw2 [, qi, qj]
};

// The finalisation of numbagg/moving_matrix.py:402-432 (cov) and :308-331 (corr),
// computed in float64 from the states (float64 in the reference for the bias, the
// bias-corrected moments and the correlation).
template <bool CORR, typename T>
NBG_DEVICE T finish(const T (&s)[NStates<CORR>::value], double min_weight) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const double n = static_cast<double>(s[4]);
  const double bias = n > 0 ? 1.0 - static_cast<double>(s[5]) / (n * n) : 0.0;
  if (!(static_cast<double>(s[3]) >= min_weight && bias > 0)) return static_cast<T>(nan);
  const double mi = static_cast<double>(s[0]) / n, mj = static_cast<double>(s[1]) / n;
  const double cb = static_cast<double>(s[2]) / n - mi * mj;
  if (!CORR) return static_cast<T>(cb / bias);
  const double vi = (static_cast<double>(s[6]) / n - mi * mi) / bias;
  const double vj = (static_cast<double>(s[7]) / n - mj * mj) / bias;
  const double cv = cb / bias;
  return static_cast<T>((vi > 0 && vj > 0) ? cv / sqrt(vi * vj) : nan);
}

// One step of the pair states: decay, then add the row where both values are valid.
template <bool CORR, typename T, int IB>
NBG_DEVICE void step(T (&st)[IB][NStates<CORR>::value], T d, T d2, T alpha_t, const T (&vi)[IB], T vj) {
  const bool vj_ok = !is_nan(vj);
#pragma unroll
  for (int r = 0; r < IB; ++r) {
#pragma unroll
    for (int k = 0; k < NStates<CORR>::value; ++k) st[r][k] *= (k == 5 ? d2 : d);
    if (vj_ok && !is_nan(vi[r])) {
      st[r][0] += vi[r];
      st[r][1] += vj;
      st[r][2] += vi[r] * vj;
      st[r][3] += alpha_t;
      st[r][4] += T(1);
      st[r][5] += T(1);
      if (CORR) {
        st[r][6] += vi[r] * vi[r];
        st[r][7] += vj * vj;
      }
    }
  }
}

// grid: x = segment * iblocks * jblocks + ib * jblocks + jb, y = batch entry.
// agg: [batch][seg][state][V][V] aggregates; dec: [batch][seg][2] decay products.
template <typename T, bool CORR, int PASS>
__global__ void __launch_bounds__(NT) exp_matrix_kernel(const T* __restrict__ a, const T* __restrict__ alpha,
                                                        long long alpha_stride, double min_weight,
                                                        T* __restrict__ out, long long n_obs, long long n_vars,
                                                        long long seg_len, long long n_seg, long long jblocks,
                                                        long long iblocks, T* __restrict__ agg, T* __restrict__ dec) {
  constexpr int IB = Rows<T, CORR>::value;
  constexpr int NS = NStates<CORR>::value;
  long long bid = blockIdx.x;
  const long long jb = bid % jblocks;
  bid /= jblocks;
  const long long ib = bid % iblocks;
  const long long seg = bid / iblocks;
  const long long batch = blockIdx.y;
  const long long j = jb * NT + threadIdx.x;
  const bool active = j < n_vars;
  const long long jj = active ? j : 0;
  const long long i0 = ib * IB;
  const long long VV = n_vars * n_vars;
  const T* ab = a + batch * n_obs * n_vars;
  const T* al = alpha + batch * alpha_stride;
  const long long t0 = seg * seg_len;
  const long long t1 = t0 + seg_len < n_obs ? t0 + seg_len : n_obs;
  T* aggb = agg + batch * n_seg * NS * VV;

  T st[IB][NS];
#pragma unroll
  for (int r = 0; r < IB; ++r)
#pragma unroll
    for (int k = 0; k < NS; ++k) st[r][k] = T(0);

  if (PASS == 1) {  // carry-in: the aggregates of the earlier segments, in order
    const T* decb = dec + batch * n_seg * 2;
    for (long long m = 0; m < seg; ++m) {
      const T d = decb[2 * m], d2 = decb[2 * m + 1];
      const T* sm = aggb + m * NS * VV;
#pragma unroll
      for (int r = 0; r < IB; ++r) {
        const long long i = i0 + r < n_vars ? i0 + r : n_vars - 1;
#pragma unroll
        for (int k = 0; k < NS; ++k) st[r][k] = st[r][k] * (k == 5 ? d2 : d) + sm[k * VV + i * n_vars + jj];
      }
    }
  }

  T dprod = T(1), d2prod = T(1);
  for (long long t = t0; t < t1; ++t) {
    const T alpha_t = al[t];
    const T d = T(1) - alpha_t, d2 = d * d;
    const T* row = ab + t * n_vars;
    const T vj = row[jj];
    T vi[IB];
#pragma unroll
    for (int r = 0; r < IB; ++r) vi[r] = i0 + r < n_vars ? __ldg(row + i0 + r) : quiet_nan(T(0));
    step<CORR, T, IB>(st, d, d2, alpha_t, vi, vj);
    if (PASS == 0) {
      dprod *= d;
      d2prod *= d2;
    } else if (active) {
      T* ot = out + (batch * n_obs + t) * VV + j;
#pragma unroll
      for (int r = 0; r < IB; ++r)
        if (i0 + r < n_vars) __stcs(ot + (i0 + r) * n_vars, finish<CORR, T>(st[r], min_weight));
    }
  }
  if (PASS == 0) {
    if (active) {
#pragma unroll
      for (int r = 0; r < IB; ++r) {
        if (i0 + r >= n_vars) break;
#pragma unroll
        for (int k = 0; k < NS; ++k) aggb[(seg * NS + k) * VV + (i0 + r) * n_vars + j] = st[r][k];
      }
    }
    if (ib == 0 && jb == 0 && threadIdx.x == 0) {
      dec[(batch * n_seg + seg) * 2] = dprod;
      dec[(batch * n_seg + seg) * 2 + 1] = d2prod;
    }
  }
}

inline long long segments(long long batch, long long n_obs, long long tiles) {
  // enough segments for about four CTAs per SM, each at least 64 steps long (a
  // segment re-reads the aggregates of all earlier ones, so keep them few)
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long n_seg = 1;
  while (n_seg < 256 && batch * tiles * n_seg < 4LL * sms && n_obs / (2 * n_seg) >= 64) n_seg *= 2;
  return n_seg;
}

}  // namespace ematrix
}  // namespace nbg

using namespace nbg;
using namespace nbg::ematrix;

namespace {
template <typename T, bool CORR>
size_t ws_bytes_for(long long batch, long long n_obs, long long n_vars) {
  const long long tiles = ((n_vars + Rows<T, CORR>::value - 1) / Rows<T, CORR>::value) * ((n_vars + NT - 1) / NT);
  const long long n_seg = segments(batch, n_obs, tiles);
  return static_cast<size_t>(batch * n_seg) * (static_cast<size_t>(NStates<CORR>::value) * n_vars * n_vars + 2) *
             sizeof(T) +
         512;
}

template <typename T, bool CORR>
int launch_exp_matrix(const T* a, const T* alpha, long long alpha_stride, double min_weight, T* out,
                      long long batch, long long n_obs, long long n_vars, void* ws, size_t ws_bytes,
                      cudaStream_t s) {
  if (batch < 0 || n_obs < 0 || n_vars < 0 || alpha_stride < 0) return kInvalidArgument;
  if (batch == 0 || n_obs == 0 || n_vars == 0) return kOk;
  if (!a || !alpha || !out || batch > 65535) return kInvalidArgument;
  constexpr int IB = Rows<T, CORR>::value;
  const long long jblocks = (n_vars + NT - 1) / NT;
  const long long iblocks = (n_vars + IB - 1) / IB;
  const long long n_seg = segments(batch, n_obs, iblocks * jblocks);
  if (!ws || ws_bytes < ws_bytes_for<T, CORR>(batch, n_obs, n_vars)) return kWorkspaceTooSmall;
  const long long seg_len = (n_obs + n_seg - 1) / n_seg;
  const long long gx = n_seg * iblocks * jblocks;
  if (gx > 0x7fffffffll) return kUnsupported;
  T* agg = static_cast<T*>(ws);
  T* dec = agg + batch * n_seg * NStates<CORR>::value * n_vars * n_vars;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(batch));
  int launches = 1;
  if (n_seg > 1) {
    exp_matrix_kernel<T, CORR, 0><<<grid, NT, 0, s>>>(a, alpha, alpha_stride, min_weight, out, n_obs, n_vars,
                                                       seg_len, n_seg, jblocks, iblocks, agg, dec);
    ++launches;
  }
  exp_matrix_kernel<T, CORR, 1><<<grid, NT, 0, s>>>(a, alpha, alpha_stride, min_weight, out, n_obs, n_vars, seg_len,
                                                     n_seg, jblocks, iblocks, agg, dec);
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_move_exp_matrix_workspace_bytes(int corr, int f64, long long batch, long long n_obs, long long n_vars) {
  if (batch <= 0 || n_obs <= 0 || n_vars <= 0) return 0;
  if (f64) return corr ? ws_bytes_for<double, true>(batch, n_obs, n_vars) : ws_bytes_for<double, false>(batch, n_obs, n_vars);
  return corr ? ws_bytes_for<float, true>(batch, n_obs, n_vars) : ws_bytes_for<float, false>(batch, n_obs, n_vars);
}

#define NBG_EXP_MATRIX(NAME, CORR, T, SFX)                                                              \
  int nbg_##NAME##_##SFX(const T* a, const T* alpha, long long alpha_stride, double min_weight, T* out, \
                         long long batch, long long n_obs, long long n_vars, void* ws, size_t ws_bytes,  \
                         void* stream) {                                                                \
    return launch_exp_matrix<T, CORR>(a, alpha, alpha_stride, min_weight, out, batch, n_obs, n_vars, ws, \
                                      ws_bytes, static_cast<cudaStream_t>(stream));                     \
  }
NBG_EXP_MATRIX(move_exp_nancovmatrix, false, double, f64)
NBG_EXP_MATRIX(move_exp_nancovmatrix, false, float, f32)
NBG_EXP_MATRIX(move_exp_nancorrmatrix, true, double, f64)
NBG_EXP_MATRIX(move_exp_nancorrmatrix, true, float, f32)
}
