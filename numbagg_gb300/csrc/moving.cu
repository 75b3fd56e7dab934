// Moving-window family: move_sum / move_mean / move_var / move_std / move_cov /
// move_corr (numbagg/moving.py:12-275), float64 and float32 arrays.
//
// Algorithm (row-tiled difference scan with decoupled look-back).
//   The reference keeps running sums, adding the entering value and removing the
//   value that leaves the window (numbagg/moving.py:30-55).  The window state at i
//   is therefore the prefix sum of the per-position difference
//       d_i = contrib(x_i) - contrib(x_{i-w})        (the second term only if i >= w)
//   where contrib() is (1, x) for the mean, (1, x, x^2) for the variance and the
//   pairwise-complete moments for cov/corr; a NaN contributes nothing.  A prefix
//   sum is a scan, so a row is cut into tiles of NT*K positions; each thread scans
//   K consecutive positions serially, a warp-shuffle scan combines threads, and the
//   carry between tiles of a row comes from a decoupled look-back.
//
// FP64 economy.  GB300 runs ~1.6 FP64 adds per clock per SM, about one per element
// at the HBM roofline, so: NaN tests are integer tests on the bit pattern, counts are
// integers, and divisions by the count use a per-CTA table of correctly rounded
// reciprocals with Markstein's correction (q0 = s*r; e = fma(-q0, c, s);
// q = fma(e, r, q0); P. Markstein, IBM J. Res. Dev. 34(1), 1990), three FP64 ops in
// place of a full double division.  Results are equal to s / c (checked against the
// hardware division).
//
// Accumulation is in float64 for float32 arrays as well, as numba types the
// reference's accumulators (`asum = 0.0`, numbagg/moving.py:16).
#include "nbg_common.cuh"

namespace nbg {
namespace moving {

enum Op : int { kSum = 0, kMean = 1, kVar = 2, kStd = 3, kCov = 4, kCorr = 5 };

template <int OP>
struct Traits;
template <>
struct Traits<kSum> { static constexpr int NS = 1; static constexpr bool TWO = false; };
template <>
struct Traits<kMean> { static constexpr int NS = 1; static constexpr bool TWO = false; };
template <>
struct Traits<kVar> { static constexpr int NS = 2; static constexpr bool TWO = false; };
template <>
struct Traits<kStd> { static constexpr int NS = 2; static constexpr bool TWO = false; };
template <>
struct Traits<kCov> { static constexpr int NS = 3; static constexpr bool TWO = true; };
template <>
struct Traits<kCorr> { static constexpr int NS = 5; static constexpr bool TWO = true; };

template <int NS>
struct State {
  long long cnt;
  double s[NS];
};

template <int NS>
NBG_DEVICE State<NS> add(const State<NS>& a, const State<NS>& b) {
  State<NS> r;
  r.cnt = a.cnt + b.cnt;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = a.s[j] + b.s[j];
  return r;
}

template <int NS>
NBG_DEVICE State<NS> zero_state() {
  State<NS> r;
  r.cnt = 0;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = 0.0;
  return r;
}

template <int NS>
struct SumOp {
  NBG_DEVICE State<NS> identity() const { return zero_state<NS>(); }
  NBG_DEVICE State<NS> combine(const State<NS>& earlier, const State<NS>& later) const {
    return add(earlier, later);
  }
};

template <int NS>
NBG_DEVICE State<NS> shfl_up_state(const State<NS>& v, int d) {
  State<NS> r;
  r.cnt = __shfl_up_sync(0xffffffffu, v.cnt, d);
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = __shfl_up_sync(0xffffffffu, v.s[j], d);
  return r;
}

// contribution of one position: moments of the value(s) if valid, else zero
template <int OP, typename T>
NBG_DEVICE State<Traits<OP>::NS> contrib(T a, T b, bool use) {
  constexpr int NS = Traits<OP>::NS;
  State<NS> r;
  bool valid = use && !is_nan(a);
  if (Traits<OP>::TWO) valid = valid && !is_nan(b);
  const double x = valid ? static_cast<double>(a) : 0.0;
  r.cnt = valid ? 1 : 0;
  if (OP == kSum || OP == kMean) {
    r.s[0] = x;
  } else if (OP == kVar || OP == kStd) {
    r.s[0] = x;
    r.s[1] = x * x;
  } else {
    const double y = valid ? static_cast<double>(b) : 0.0;
    r.s[0] = x;
    r.s[1] = y;
    r.s[2] = x * y;
    if (OP == kCorr) {
      r.s[3] = x * x;
      r.s[4] = y * y;
    }
  }
  return r;
}

template <int NS>
NBG_DEVICE State<NS> sub(const State<NS>& a, const State<NS>& b) {
  State<NS> r;
  r.cnt = a.cnt - b.cnt;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = a.s[j] - b.s[j];
  return r;
}

constexpr int kRcpTable = 1024;

// s / c for an integer count c >= 1, correctly rounded.
NBG_DEVICE double div_count(double s, long long c, const double* rcp) {
  if (c < kRcpTable) {
    const double r = rcp[c];
    const double dc = static_cast<double>(c);
    const double q0 = s * r;
    const double e = fma(-q0, dc, s);
    return fma(e, r, q0);
  }
  return s / static_cast<double>(c);
}

template <int OP>
NBG_DEVICE double finalize(const State<Traits<OP>::NS>& st, long long min_count, const double* rcp) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long c = st.cnt;
  if (OP == kSum) return c >= min_count ? st.s[0] : nan;
  if (OP == kMean) {
    const long long mc = min_count > 1 ? min_count : 1;
    return c >= mc ? div_count(st.s[0], c, rcp) : nan;
  }
  if (OP == kVar || OP == kStd) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc) return nan;
    // (asum_sq - asum**2 / count) / (count - 1)    numbagg/moving.py:147-148
    const double v = div_count(st.s[1] - div_count(st.s[0] * st.s[0], c, rcp), c - 1, rcp);
    return OP == kStd ? sqrt(v) : v;
  }
  if (OP == kCov) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc) return nan;
    // (prodsum - asum * bsum / count) / (count - 1)   numbagg/moving.py:217-218
    return div_count(st.s[2] - div_count(st.s[0] * st.s[1], c, rcp), c - 1, rcp);
  }
  // kCorr, numbagg/moving.py:263-273
  const long long mc = min_count > 1 ? min_count : 1;
  if (c < mc) return nan;
  const double rc = c < kRcpTable ? rcp[c] : 1.0 / static_cast<double>(c);
  const double avg_a = st.s[0] * rc;
  const double avg_b = st.s[1] * rc;
  const double var_a = st.s[3] * rc - avg_a * avg_a;
  const double var_b = st.s[4] * rc - avg_b * avg_b;
  const double cov_ab = st.s[2] * rc - avg_a * avg_b;
  const double vv = var_a * var_b;
  return vv > 0 ? cov_ab / sqrt(vv) : nan;
}

constexpr int NT = 256;

template <int OP, typename T, int K>
__global__ void __launch_bounds__(NT) move_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                  T* __restrict__ out, long long rows, long long n,
                                                  long long window, long long min_count,
                                                  long long tiles_per_row, void* ws_base,
                                                  size_t ws_bytes) {
  constexpr int NS = Traits<OP>::NS;
  constexpr long long TILE = static_cast<long long>(NT) * K;
  using S = State<NS>;
  __shared__ double rcp[kRcpTable];
  __shared__ S warp_tot[NT / 32];
  __shared__ S carry_smem;
  __shared__ long long tile_smem;

  const long long total_tiles = rows * tiles_per_row;
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);

  for (int c = threadIdx.x; c < kRcpTable; c += NT) rcp[c] = c ? 1.0 / static_cast<double>(c) : 0.0;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) tile_smem = claim_tile(ws.hdr);
    __syncthreads();
    const long long tile = tile_smem;
    if (tile >= total_tiles) break;
    const TileCoord tc = tile_coord(tile, rows);
    const long long row = tc.row, chunk = tc.chunk;
    const long long p0 = chunk * TILE + static_cast<long long>(threadIdx.x) * K;
    const T* ar = a + row * n;
    const T* br = Traits<OP>::TWO ? b + row * n : nullptr;

    // ---- pass 1: per-position differences, thread-serial inclusive scan ----
    T av[K], bv[K], ao[K], bo[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      const bool in = i < n;
      const bool has_old = in && i >= window;
      av[k] = in ? ar[i] : T(0);
      ao[k] = has_old ? ar[i - window] : T(0);
      if (Traits<OP>::TWO) {
        bv[k] = in ? br[i] : T(0);
        bo[k] = has_old ? br[i - window] : T(0);
      } else {
        bv[k] = T(0);
        bo[k] = T(0);
      }
    }
    S run = zero_state<NS>();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      const S dn = contrib<OP, T>(av[k], bv[k], i < n);
      const S dold = contrib<OP, T>(ao[k], bo[k], i < n && i >= window);
      run = add(run, sub(dn, dold));
    }

    // ---- block scan of thread totals ----
    S incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const S up = shfl_up_state(incl, d);
      if (lane >= d) incl = add(up, incl);
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      S wt = lane < NT / 32 ? warp_tot[lane] : zero_state<NS>();
#pragma unroll
      for (int d = 1; d < NT / 32; d <<= 1) {
        const S up = shfl_up_state(wt, d);
        if (lane >= d) wt = add(up, wt);
      }
      if (lane < NT / 32) warp_tot[lane] = wt;  // inclusive warp prefixes
    }
    __syncthreads();
    const S warp_excl = warp ? warp_tot[warp - 1] : zero_state<NS>();
    const S tile_agg = warp_tot[NT / 32 - 1];
    // exclusive prefix inside the warp by shuffle (incl - run would turn inf into NaN)
    S lane_excl = shfl_up_state(incl, 1);
    if (lane == 0) lane_excl = zero_state<NS>();
    const S thread_excl = add(warp_excl, lane_excl);

    // ---- look-back for the carry into this tile (warp 0) ----
    if (warp == 0) {
      if (chunk == 0) {
        if (lane == 0) {
          if (tiles_per_row > 1) publish(ws, tile, epoch, kStatePrefix, tile_agg);
          carry_smem = zero_state<NS>();
        }
      } else {
        if (lane == 0) publish(ws, tile, epoch, kStateAggregate, tile_agg);
        __syncwarp();
        bool ok;
        const S carry = warp_lookback<S>(ws, tile, chunk, rows, epoch, SumOp<NS>(), ok);
        if (lane == 0) {
          publish(ws, tile, epoch, kStatePrefix, add(carry, tile_agg));
          carry_smem = carry;
        }
      }
    }
    __syncthreads();
    S st = add(carry_smem, thread_excl);

    // ---- pass 2: outputs ----
    T* orow = out + row * n;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      const S dn = contrib<OP, T>(av[k], bv[k], i < n);
      const S dold = contrib<OP, T>(ao[k], bo[k], i < n && i >= window);
      st = add(st, sub(dn, dold));
      if (i < n) orow[i] = static_cast<T>(finalize<OP>(st, min_count, rcp));
    }
    __syncthreads();  // warp_tot / carry_smem reuse in the next tile
  }
  if (threadIdx.x == 0) finish_cta(ws.hdr);
}

}  // namespace moving
}  // namespace nbg

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
using namespace nbg;
using namespace nbg::moving;

namespace {
constexpr int kItemsPerThread = 8;

long long tiles_per_row_for(long long n) {
  const long long tile = static_cast<long long>(NT) * kItemsPerThread;
  return n <= 0 ? 0 : (n + tile - 1) / tile;
}

int grid_for(long long total_tiles) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long cap = static_cast<long long>(sms) * 8;
  return static_cast<int>(total_tiles < cap ? total_tiles : cap);
}

template <int OP, typename T>
int launch_move(const T* a, const T* b, T* out, long long rows, long long n, long long window,
                long long min_count, void* ws, size_t ws_bytes, cudaStream_t stream) {
  if (rows < 0 || n < 0 || window <= 0 || min_count < 0) return kInvalidArgument;
  if (rows == 0 || n == 0) return kOk;
  if (!a || !out || (Traits<OP>::TWO && !b)) return kInvalidArgument;
  const long long tpr = tiles_per_row_for(n);
  const long long total = rows * tpr;
  if (!ws || ws_bytes < workspace_bytes(total)) return kWorkspaceTooSmall;
  move_kernel<OP, T, kItemsPerThread><<<grid_for(total), NT, 0, stream>>>(
      a, b, out, rows, n, window, min_count, tpr, ws, ws_bytes);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_move_workspace_bytes(long long rows, long long n) {
  return workspace_bytes(rows * tiles_per_row_for(n));
}

#define NBG_MOVE1(NAME, OPC, T, SFX)                                                        \
  int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long n, long long window,  \
                         long long min_count, void* ws, size_t ws_bytes, void* stream) {     \
    return launch_move<OPC, T>(a, nullptr, out, rows, n, window, min_count, ws, ws_bytes,    \
                               static_cast<cudaStream_t>(stream));                          \
  }
#define NBG_MOVE2(NAME, OPC, T, SFX)                                                        \
  int nbg_##NAME##_##SFX(const T* a, const T* b, T* out, long long rows, long long n,        \
                         long long window, long long min_count, void* ws, size_t ws_bytes,   \
                         void* stream) {                                                    \
    return launch_move<OPC, T>(a, b, out, rows, n, window, min_count, ws, ws_bytes,          \
                               static_cast<cudaStream_t>(stream));                          \
  }

NBG_MOVE1(move_sum, kSum, double, f64)
NBG_MOVE1(move_sum, kSum, float, f32)
NBG_MOVE1(move_mean, kMean, double, f64)
NBG_MOVE1(move_mean, kMean, float, f32)
NBG_MOVE1(move_var, kVar, double, f64)
NBG_MOVE1(move_var, kVar, float, f32)
NBG_MOVE1(move_std, kStd, double, f64)
NBG_MOVE1(move_std, kStd, float, f32)
NBG_MOVE2(move_cov, kCov, double, f64)
NBG_MOVE2(move_cov, kCov, float, f32)
NBG_MOVE2(move_corr, kCorr, double, f64)
NBG_MOVE2(move_corr, kCorr, float, f32)

}  // extern "C"
