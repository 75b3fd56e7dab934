// nancovmatrix / nancorrmatrix (numbagg/funcs.py:338-532).
//
// Input (batch, V, n_obs), output (batch, V, V).  For every pair i <= j the reference
// sums, over the observations where both a[i, k] and a[j, k] are valid, a[i, k],
// a[j, k], a[i, k] a[j, k] (+ a[i, k]^2 and a[j, k]^2 for the correlation) in the
// input dtype and counts them in int64; the pairwise-complete covariance or
// correlation is then finalised in float64 and mirrored to (j, i).
//
// This is a masked Gram matrix.  A CTA owns a 32 x 32 tile of pairs (tiles on or above
// the diagonal) and one slice of the observations; it stages 32 observations of its
// 32 row variables and 32 column variables in shared memory at a time (NaN replaced
// by 0 beside a validity flag), and each thread accumulates 2 x 2 pairs with fused
// multiply-adds in the input dtype: sum_i += a_i * valid_j, sum_j += a_j * valid_i,
// prod += a_i * a_j (zero when either is missing).  The slices' partial sums go to the
// workspace and a second kernel folds them in slice order (deterministic) and writes
// both triangles.
#include "nbg_common.cuh"

namespace nbg {
namespace pmatrix {

constexpr int TILE = 32;  // pairs per tile side
constexpr int KO = 32;    // observations per shared-memory stage
constexpr int NT = 256;   // 16 x 16 threads, 2 x 2 pairs each

template <bool CORR>
struct NSums {
  static constexpr int value = CORR ? 5 : 3;  // si, sj, sij [, qi, qj]
};

// partial sums: part[((batch * n_split + split) * NS + k) * V * V + i * V + j],
// counts cnt[(batch * n_split + split) * V * V + i * V + j]
template <typename T, bool CORR>
__global__ void __launch_bounds__(NT) pair_partial_kernel(const T* __restrict__ a, long long n_vars, long long n_obs,
                                                          long long tiles, long long split_len, long long n_split,
                                                          T* __restrict__ part, long long* __restrict__ cnt) {
  constexpr int NS = NSums<CORR>::value;
  __shared__ T si_s[TILE][KO + 1], sj_s[TILE][KO + 1];
  __shared__ unsigned char vi_s[TILE][KO + 1], vj_s[TILE][KO + 1];
  // tile index -> (it, jt) with jt >= it, row by row of the upper triangle
  const long long split = blockIdx.x % n_split;
  long long tile = blockIdx.x / n_split;
  long long it = 0;
  while (tile >= tiles - it) {
    tile -= tiles - it;
    ++it;
  }
  const long long jt = it + tile;
  const long long batch = blockIdx.y;
  const T* ab = a + batch * n_vars * n_obs;
  const long long k0 = split * split_len;
  const long long k1 = k0 + split_len < n_obs ? k0 + split_len : n_obs;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T s[2][2][NS];
  long long c[2][2];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      c[p][q] = 0;
#pragma unroll
      for (int k = 0; k < NS; ++k) s[p][q][k] = T(0);
    }
  for (long long kb = k0; kb < k1; kb += KO) {
    // stage: 32 variables x 32 observations of each side, coalesced along observations
    for (int e = threadIdx.x; e < TILE * KO; e += NT) {
      const int v = e / KO, k = e % KO;
      const long long obs = kb + k;
      const long long gi = it * TILE + v, gj = jt * TILE + v;
      T xi = (obs < k1 && gi < n_vars) ? ab[gi * n_obs + obs] : quiet_nan(T(0));
      T xj = (obs < k1 && gj < n_vars) ? ab[gj * n_obs + obs] : quiet_nan(T(0));
      const bool oi = !is_nan(xi), oj = !is_nan(xj);
      si_s[v][k] = oi ? xi : T(0);
      sj_s[v][k] = oj ? xj : T(0);
      vi_s[v][k] = oi;
      vj_s[v][k] = oj;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < KO; ++k) {
      T xi[2], xj[2];
      bool oi[2], oj[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        xi[p] = si_s[ty * 2 + p][k];
        oi[p] = vi_s[ty * 2 + p][k];
        xj[p] = sj_s[tx * 2 + p][k];
        oj[p] = vj_s[tx * 2 + p][k];
      }
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const T mi = oi[p] ? T(1) : T(0), mj = oj[q] ? T(1) : T(0);
          s[p][q][0] = fma(xi[p], mj, s[p][q][0]);
          s[p][q][1] = fma(xj[q], mi, s[p][q][1]);
          s[p][q][2] = fma(xi[p], xj[q], s[p][q][2]);
          if (CORR) {
            s[p][q][3] = fma(xi[p] * xi[p], mj, s[p][q][3]);
            s[p][q][4] = fma(xj[q] * xj[q], mi, s[p][q][4]);
          }
          c[p][q] += (oi[p] && oj[q]) ? 1 : 0;
        }
    }
    __syncthreads();
  }
  const long long VV = n_vars * n_vars;
  const long long base = batch * n_split + split;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const long long i = it * TILE + ty * 2 + p, j = jt * TILE + tx * 2 + q;
      if (i >= n_vars || j >= n_vars) continue;
#pragma unroll
      for (int k = 0; k < NS; ++k) part[(base * NS + k) * VV + i * n_vars + j] = s[p][q][k];
      cnt[base * VV + i * n_vars + j] = c[p][q];
    }
}

// Fold the slices in order and finalise pairs i <= j (numbagg/funcs.py:433-456 for the
// correlation, :523-532 for the covariance), writing (i, j) and (j, i).
template <typename T, bool CORR>
__global__ void pair_finish_kernel(const T* __restrict__ part, const long long* __restrict__ cnt, T* __restrict__ out,
                                   long long batch, long long n_vars, long long n_split) {
  constexpr int NS = NSums<CORR>::value;
  const long long VV = n_vars * n_vars;
  const long long total = batch * VV;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long b = t / VV, q = t - b * VV;
    const long long i = q / n_vars, j = q - i * n_vars;
    if (j < i) continue;
    T s[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) s[k] = T(0);
    long long c = 0;
    for (long long sp = 0; sp < n_split; ++sp) {
      const long long base = b * n_split + sp;
#pragma unroll
      for (int k = 0; k < NS; ++k) s[k] += part[(base * NS + k) * VV + q];
      c += cnt[base * VV + q];
    }
    double r = nan;
    if (c > 1) {
      const double dc = static_cast<double>(c);
      const double mi = static_cast<double>(s[0]) / dc, mj = static_cast<double>(s[1]) / dc;
      const double cov = static_cast<double>(s[2]) / dc - mi * mj;
      if (!CORR) {
        r = cov * dc / static_cast<double>(c - 1);
      } else {
        const double vi = (static_cast<double>(s[3]) / dc - mi * mi) * dc / static_cast<double>(c - 1);
        const double vj = (static_cast<double>(s[4]) / dc - mj * mj) * dc / static_cast<double>(c - 1);
        const double cu = cov * dc / static_cast<double>(c - 1);
        if (vi > 0 && vj > 0) r = cu / sqrt(vi * vj);
      }
    }
    out[b * VV + i * n_vars + j] = static_cast<T>(r);
    out[b * VV + j * n_vars + i] = static_cast<T>(r);
  }
}

inline long long pair_splits(long long batch, long long n_obs, long long utiles) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long n_split = 1;
  while (n_split < 1024 && batch * utiles * n_split < 2LL * sms && n_obs / (2 * n_split) >= 256) n_split *= 2;
  return n_split;
}

}  // namespace pmatrix
}  // namespace nbg

using namespace nbg;
using namespace nbg::pmatrix;

namespace {
template <typename T, bool CORR>
size_t pair_ws_bytes(long long batch, long long n_vars, long long n_obs) {
  const long long tiles = (n_vars + TILE - 1) / TILE;
  const long long n_split = pair_splits(batch, n_obs, tiles * (tiles + 1) / 2);
  const size_t slots = static_cast<size_t>(batch * n_split) * n_vars * n_vars;
  return slots * (NSums<CORR>::value * sizeof(T) + sizeof(long long)) + 1024;
}

template <typename T, bool CORR>
int launch_pair(const T* a, T* out, long long batch, long long n_vars, long long n_obs, void* ws, size_t ws_bytes,
                cudaStream_t s) {
  if (batch < 0 || n_vars < 0 || n_obs < 0) return kInvalidArgument;
  if (batch == 0 || n_vars == 0) return kOk;
  if (!out || (n_obs > 0 && !a) || batch > 65535) return kInvalidArgument;
  const long long tiles = (n_vars + TILE - 1) / TILE;
  const long long utiles = tiles * (tiles + 1) / 2;
  const long long n_split = pair_splits(batch, n_obs, utiles);
  if (!ws || ws_bytes < pair_ws_bytes<T, CORR>(batch, n_vars, n_obs)) return kWorkspaceTooSmall;
  if (utiles * n_split > 0x7fffffffll) return kUnsupported;
  const long long split_len = n_obs > 0 ? (n_obs + n_split - 1) / n_split : 0;
  const size_t slots = static_cast<size_t>(batch * n_split) * n_vars * n_vars;
  T* part = static_cast<T*>(ws);
  long long* cnt = reinterpret_cast<long long*>(
      (reinterpret_cast<size_t>(part + slots * NSums<CORR>::value) + 255) & ~static_cast<size_t>(255));
  dim3 grid(static_cast<unsigned>(utiles * n_split), static_cast<unsigned>(batch));
  pair_partial_kernel<T, CORR><<<grid, NT, 0, s>>>(a, n_vars, n_obs, tiles, split_len, n_split, part, cnt);
  long long blocks = (batch * n_vars * n_vars + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  pair_finish_kernel<T, CORR><<<static_cast<int>(blocks), 256, 0, s>>>(part, cnt, out, batch, n_vars, n_split);
  note_launches(2);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_pair_matrix_workspace_bytes(int corr, int f64, long long batch, long long n_vars, long long n_obs) {
  if (batch <= 0 || n_vars <= 0 || n_obs < 0) return 0;
  if (f64) return corr ? pair_ws_bytes<double, true>(batch, n_vars, n_obs) : pair_ws_bytes<double, false>(batch, n_vars, n_obs);
  return corr ? pair_ws_bytes<float, true>(batch, n_vars, n_obs) : pair_ws_bytes<float, false>(batch, n_vars, n_obs);
}

#define NBG_PAIR_MATRIX(NAME, CORR, T, SFX)                                                              \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long batch, long long n_vars, long long n_obs, void* ws, \
                         size_t ws_bytes, void* stream) {                                                \
    return launch_pair<T, CORR>(a, out, batch, n_vars, n_obs, ws, ws_bytes, static_cast<cudaStream_t>(stream)); \
  }
NBG_PAIR_MATRIX(nancovmatrix, false, double, f64)
NBG_PAIR_MATRIX(nancovmatrix, false, float, f32)
NBG_PAIR_MATRIX(nancorrmatrix, true, double, f64)
NBG_PAIR_MATRIX(nancorrmatrix, true, float, f32)
}
