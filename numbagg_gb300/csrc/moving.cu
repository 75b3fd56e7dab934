// Moving-window family: move_sum / move_mean / move_var / move_std / move_cov /
// move_corr (numbagg/moving.py:12-275), float64 and float32 arrays.
//
// The reference keeps running sums, adding the value that enters the window and
// removing the one that leaves (numbagg/moving.py:30-55).  The window state at i is
// therefore the prefix sum of the per-position difference
//     d_i = contrib(x_i) - contrib(x_{i-w})          (second term only when i >= w)
// where contrib() is the count and the moments the statistic needs (x; x, x^2; the
// pairwise-complete a, b, ab, a^2, b^2); a NaN contributes nothing.
//
// Exact sums.  The moments are accumulated as 128-bit fixed-point integers
// (fixed128.cuh) at the scale of the largest exponent in the tile, so every window
// sum is exact (to 2^-80 of its largest term) whatever the position in the row: the
// reference's own add/subtract drift is the only difference left between the two.
// Integer addition is associative, so results are bit-identical for any tiling and
// run to run.  The exact sums are rounded once to float64 and finalised with the
// reference's formulas; divisions by the count use a per-CTA table of correctly
// rounded reciprocals and Markstein's correction (q0 = s*r; e = fma(-q0, c, s);
// q = fma(e, r, q0); P. Markstein, IBM J. Res. Dev. 34(1), 1990), which returns s / c.
//
// Infinities follow the reference: an infinity in the running sum makes every later
// sum NaN once it leaves the window (inf - inf), or while infinities of both signs
// are inside; for the variance-like statistics any infinity (or |x| >= 2^512, whose
// square overflows) turns the rest of the row NaN.  These are tracked as counts.
//
// Parallel structure: a row is cut into tiles of NT*K positions; each thread scans K
// consecutive positions serially, warp shuffles combine threads, and the state
// entering a tile comes from a decoupled look-back whose combine step aligns the two
// tiles' scales.  Accumulation is exact for float32 arrays too (numba keeps float64
// accumulators there, numbagg/moving.py:16); the result is rounded to float32.
#include "fixed128.cuh"

namespace nbg {
namespace moving {

using fx::i128;

enum Op : int { kSum = 0, kMean = 1, kVar = 2, kStd = 3, kCov = 4, kCorr = 5 };

template <int OP>
struct Traits;
template <>
struct Traits<kSum> { static constexpr int NS = 1; static constexpr bool TWO = false; static constexpr bool VARLIKE = false; };
template <>
struct Traits<kMean> { static constexpr int NS = 1; static constexpr bool TWO = false; static constexpr bool VARLIKE = false; };
template <>
struct Traits<kVar> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kStd> { static constexpr int NS = 2; static constexpr bool TWO = false; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kCov> { static constexpr int NS = 3; static constexpr bool TWO = true; static constexpr bool VARLIKE = true; };
template <>
struct Traits<kCorr> { static constexpr int NS = 5; static constexpr bool TWO = true; static constexpr bool VARLIKE = true; };

// moment j is a^order_a * b^order_b:  mean: a   var: a, a^2   cov: a, b, ab
// corr: a, b, ab, a^2, b^2
template <int OP>
NBG_HOST_DEVICE int order_a(int j) {
  if (OP == kSum || OP == kMean) return 1;
  if (OP == kVar || OP == kStd) return j == 0 ? 1 : 2;
  return j == 0 ? 1 : (j == 1 ? 0 : (j == 2 ? 1 : (j == 3 ? 2 : 0)));
}
template <int OP>
NBG_HOST_DEVICE int order_b(int j) {
  if (!Traits<OP>::TWO) return 0;
  return j == 0 ? 0 : (j == 1 ? 1 : (j == 2 ? 1 : (j == 3 ? 0 : 2)));
}

template <int NS>
struct Sums {  // tile-local moments (one scale for the whole tile)
  i128 s[NS];
  long long cnt;
  int inf_pos, inf_neg, inf_left;  // infinities entered (+, -) and left the window
  int pad;
};

template <int NS>
struct XState {  // a state that travels between tiles: sums plus their scale
  Sums<NS> m;
  int ea, eb;
  int pad0, pad1;
};

template <int NS>
NBG_DEVICE Sums<NS> zero_sums() {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = 0;
  r.cnt = 0;
  r.inf_pos = r.inf_neg = r.inf_left = 0;
  r.pad = 0;
  return r;
}

template <int NS>
NBG_DEVICE Sums<NS> add(const Sums<NS>& a, const Sums<NS>& b) {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = a.s[j] + b.s[j];
  r.cnt = a.cnt + b.cnt;
  r.inf_pos = a.inf_pos + b.inf_pos;
  r.inf_neg = a.inf_neg + b.inf_neg;
  r.inf_left = a.inf_left + b.inf_left;
  r.pad = 0;
  return r;
}

// shift a tile's sums from scale (ea, eb) to (ea2, eb2) >= it
template <int OP>
NBG_DEVICE Sums<Traits<OP>::NS> rescale(const Sums<Traits<OP>::NS>& v, int ea, int eb, int ea2, int eb2) {
  Sums<Traits<OP>::NS> r = v;
  if (ea2 == ea && eb2 == eb) return r;
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j)
    r.s[j] = fx::shr(v.s[j], order_a<OP>(j) * (ea2 - ea) + order_b<OP>(j) * (eb2 - eb));
  return r;
}

template <int OP>
struct CombineOp {
  using X = XState<Traits<OP>::NS>;
  NBG_DEVICE X identity() const {
    X x;
    x.m = zero_sums<Traits<OP>::NS>();
    x.ea = x.eb = 0;
    x.pad0 = x.pad1 = 0;
    return x;
  }
  NBG_DEVICE X combine(const X& e, const X& l) const {
    X r;
    r.ea = max(e.ea, l.ea);
    r.eb = max(e.eb, l.eb);
    r.m = add(rescale<OP>(e.m, e.ea, e.eb, r.ea, r.eb), rescale<OP>(l.m, l.ea, l.eb, r.ea, r.eb));
    r.pad0 = r.pad1 = 0;
    return r;
  }
};

NBG_DEVICE i128 shfl_up_i128(i128 v, int d) {
  const unsigned long long lo = static_cast<unsigned long long>(v);
  const unsigned long long hi = static_cast<unsigned long long>(v >> 64);
  const unsigned long long rlo = __shfl_up_sync(0xffffffffu, lo, d);
  const unsigned long long rhi = __shfl_up_sync(0xffffffffu, hi, d);
  return static_cast<i128>((static_cast<fx::u128>(rhi) << 64) | rlo);
}

template <int NS>
NBG_DEVICE Sums<NS> shfl_up_sums(const Sums<NS>& v, int d) {
  Sums<NS> r;
#pragma unroll
  for (int j = 0; j < NS; ++j) r.s[j] = shfl_up_i128(v.s[j], d);
  r.cnt = __shfl_up_sync(0xffffffffu, v.cnt, d);
  r.inf_pos = __shfl_up_sync(0xffffffffu, v.inf_pos, d);
  r.inf_neg = __shfl_up_sync(0xffffffffu, v.inf_neg, d);
  r.inf_left = __shfl_up_sync(0xffffffffu, v.inf_left, d);
  r.pad = 0;
  return r;
}

// |x| >= 2^512: the reference's x * x overflows to inf
NBG_DEVICE bool square_overflows(double x) { return fx::biased_exponent(x) >= 1023 + 512; }

// Add (sign = +1, the entering value) or remove (sign = -1, the leaving value) one
// position's contribution at the tile scale (Ea, Eb).
template <int OP, typename T>
NBG_DEVICE void accumulate(Sums<Traits<OP>::NS>& acc, T av, T bv, bool use, int sign, int Ea, int Eb) {
  constexpr bool TWO = Traits<OP>::TWO;
  bool valid = use && !is_nan(av);
  if (TWO) valid = valid && !is_nan(bv);
  if (!valid) return;
  const double a = static_cast<double>(av);
  const double b = TWO ? static_cast<double>(bv) : 0.0;
  acc.cnt += sign;
  bool inf = fx::is_inf(a) || (TWO && fx::is_inf(b));
  if (Traits<OP>::VARLIKE) inf = inf || square_overflows(a) || (TWO && square_overflows(b));
  if (inf) {
    if (sign > 0) {
      if (TWO || Traits<OP>::VARLIKE || a > 0) acc.inf_pos += 1; else acc.inf_neg += 1;
    } else {
      acc.inf_left += 1;
    }
    return;
  }
  i128 m[5];
  if (OP == kSum || OP == kMean) {
    m[0] = fx::fix_value(a, Ea);
  } else if (OP == kVar || OP == kStd) {
    m[0] = fx::fix_value(a, Ea);
    m[1] = fx::fix_square(a, Ea);
  } else {
    m[0] = fx::fix_value(a, Ea);
    m[1] = fx::fix_value(b, Eb);
    m[2] = fx::fix_product(a, b, Ea, Eb);
    if (OP == kCorr) {
      m[3] = fx::fix_square(a, Ea);
      m[4] = fx::fix_square(b, Eb);
    }
  }
#pragma unroll
  for (int j = 0; j < Traits<OP>::NS; ++j) acc.s[j] = sign > 0 ? acc.s[j] + m[j] : acc.s[j] - m[j];
}

constexpr int kRcpTable = 1024;

// s / c for an integer count c >= 1, correctly rounded (non-finite s: plain division,
// the correction step would turn inf into NaN)
NBG_DEVICE double div_count(double s, long long c, const double* rcp) {
  if (c < kRcpTable && isfinite(s)) {
    const double r = rcp[c];
    const double q0 = s * r;
    const double e = fma(-q0, static_cast<double>(c), s);
    return fma(e, r, q0);
  }
  return s / static_cast<double>(c);
}

template <int OP>
NBG_DEVICE double finalize(const Sums<Traits<OP>::NS>& st, int ea, int eb, long long min_count, const double* rcp) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const long long c = st.cnt;
  if (OP == kSum || OP == kMean) {
    const long long mc = OP == kMean ? (min_count > 1 ? min_count : 1) : min_count;
    if (c < mc) return nan;
    if (st.inf_left > 0 || (st.inf_pos > 0 && st.inf_neg > 0)) return nan;
    double s;
    if (st.inf_pos > 0) s = __longlong_as_double(0x7ff0000000000000ll);
    else if (st.inf_neg > 0) s = __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
    else s = fx::to_double(st.s[0], fx::lsb_value(ea));
    return OP == kSum ? s : div_count(s, c, rcp);
  }
  if (OP == kVar || OP == kStd) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc || st.inf_pos > 0) return nan;
    const double s1 = fx::to_double(st.s[0], fx::lsb_value(ea));
    const double s2 = fx::to_double(st.s[1], fx::lsb_product(ea, ea));
    // (asum_sq - asum**2 / count) / (count - 1)    numbagg/moving.py:147-148
    const double v = div_count(s2 - div_count(s1 * s1, c, rcp), c - 1, rcp);
    return OP == kStd ? sqrt(v) : v;
  }
  if (OP == kCov) {
    const long long mc = min_count > 2 ? min_count : 2;
    if (c < mc || st.inf_pos > 0) return nan;
    const double sa = fx::to_double(st.s[0], fx::lsb_value(ea));
    const double sb = fx::to_double(st.s[1], fx::lsb_value(eb));
    const double sab = fx::to_double(st.s[2], fx::lsb_product(ea, eb));
    // (prodsum - asum * bsum / count) / (count - 1)   numbagg/moving.py:217-218
    return div_count(sab - div_count(sa * sb, c, rcp), c - 1, rcp);
  }
  // kCorr, numbagg/moving.py:263-273
  const long long mc = min_count > 1 ? min_count : 1;
  if (c < mc || st.inf_pos > 0) return nan;
  const double sa = fx::to_double(st.s[0], fx::lsb_value(ea));
  const double sb = fx::to_double(st.s[1], fx::lsb_value(eb));
  const double sab = fx::to_double(st.s[2], fx::lsb_product(ea, eb));
  const double saa = fx::to_double(st.s[3], fx::lsb_product(ea, ea));
  const double sbb = fx::to_double(st.s[4], fx::lsb_product(eb, eb));
  const double rc = c < kRcpTable ? rcp[c] : 1.0 / static_cast<double>(c);
  const double avg_a = sa * rc;
  const double avg_b = sb * rc;
  const double var_a = saa * rc - avg_a * avg_a;
  const double var_b = sbb * rc - avg_b * avg_b;
  const double cov_ab = sab * rc - avg_a * avg_b;
  const double vv = var_a * var_b;
  return vv > 0 ? cov_ab / sqrt(vv) : nan;
}

constexpr int NT = 256;

// biased exponent of a finite valid value, 0 otherwise
template <typename T>
NBG_DEVICE int exp_of(T v, bool use) {
  const double x = static_cast<double>(v);
  return (use && !is_nan(v) && !fx::is_inf(x)) ? fx::biased_exponent(x) : 0;
}

template <int OP, typename T, int K>
__global__ void __launch_bounds__(NT) move_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                  T* __restrict__ out, long long rows, long long n,
                                                  long long window, long long min_count,
                                                  long long tiles_per_row, void* ws_base,
                                                  size_t ws_bytes) {
  constexpr int NS = Traits<OP>::NS;
  constexpr bool TWO = Traits<OP>::TWO;
  constexpr long long TILE = static_cast<long long>(NT) * K;
  using S = Sums<NS>;
  using X = XState<NS>;
  __shared__ double rcp[kRcpTable];
  __shared__ S warp_tot[NT / 32];
  __shared__ X carry_smem;
  __shared__ int emax_smem[2][NT / 32];
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
    const T* br = TWO ? b + row * n : nullptr;

    T av[K], bv[K], ao[K], bo[K];
    int ea = 0, eb = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      const bool in = i < n;
      const bool has_old = in && i >= window;
      av[k] = in ? ar[i] : T(0);
      ao[k] = has_old ? ar[i - window] : T(0);
      bv[k] = (TWO && in) ? br[i] : T(0);
      bo[k] = (TWO && has_old) ? br[i - window] : T(0);
      ea = max(ea, max(exp_of(av[k], in), exp_of(ao[k], has_old)));
      if (TWO) eb = max(eb, max(exp_of(bv[k], in), exp_of(bo[k], has_old)));
    }
    // tile scale: block-wide maximum exponent
    ea = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(ea)));
    eb = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(eb)));
    if (lane == 0) {
      emax_smem[0][warp] = ea;
      emax_smem[1][warp] = eb;
    }
    __syncthreads();
    ea = 1;
    eb = 1;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
      ea = max(ea, emax_smem[0][w]);
      eb = max(eb, emax_smem[1][w]);
    }

    // ---- pass 1: thread-serial sum of the differences ----
    S run = zero_sums<NS>();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      accumulate<OP, T>(run, av[k], bv[k], i < n, +1, ea, eb);
      accumulate<OP, T>(run, ao[k], bo[k], i < n && i >= window, -1, ea, eb);
    }
    // ---- block scan of thread totals (exact, one scale) ----
    S incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const S up = shfl_up_sums(incl, d);
      if (lane >= d) incl = add(up, incl);
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      S wt = lane < NT / 32 ? warp_tot[lane] : zero_sums<NS>();
#pragma unroll
      for (int d = 1; d < NT / 32; d <<= 1) {
        const S up = shfl_up_sums(wt, d);
        if (lane >= d) wt = add(up, wt);
      }
      if (lane < NT / 32) warp_tot[lane] = wt;
    }
    __syncthreads();
    S lane_excl = shfl_up_sums(incl, 1);
    if (lane == 0) lane_excl = zero_sums<NS>();
    const S thread_excl = warp ? add(warp_tot[warp - 1], lane_excl) : lane_excl;

    // ---- carry into the tile: decoupled look-back (warp 0) ----
    if (warp == 0) {
      X agg;
      agg.m = warp_tot[NT / 32 - 1];
      agg.ea = ea;
      agg.eb = eb;
      agg.pad0 = agg.pad1 = 0;
      const CombineOp<OP> op;
      if (chunk == 0) {
        if (lane == 0) {
          if (tiles_per_row > 1) publish(ws, tile, epoch, kStatePrefix, agg);
          carry_smem = op.identity();
        }
      } else {
        if (lane == 0) publish(ws, tile, epoch, kStateAggregate, agg);
        __syncwarp();
        bool ok;
        const X carry = warp_lookback<X>(ws, tile, chunk, rows, epoch, op, ok);
        if (lane == 0) {
          publish(ws, tile, epoch, kStatePrefix, op.combine(carry, agg));
          carry_smem = carry;
        }
      }
    }
    __syncthreads();
    // output scale: the larger of the carry's and the tile's
    const X carry = carry_smem;
    const int eo_a = max(carry.ea, ea), eo_b = max(carry.eb, eb);
    S st = add(rescale<OP>(carry.m, carry.ea, carry.eb, eo_a, eo_b), rescale<OP>(thread_excl, ea, eb, eo_a, eo_b));

    // ---- pass 2: outputs ----
    T* orow = out + row * n;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long i = p0 + k;
      S d = zero_sums<NS>();
      accumulate<OP, T>(d, av[k], bv[k], i < n, +1, ea, eb);
      accumulate<OP, T>(d, ao[k], bo[k], i < n && i >= window, -1, ea, eb);
      st = add(st, rescale<OP>(d, ea, eb, eo_a, eo_b));
      if (i < n) orow[i] = static_cast<T>(finalize<OP>(st, eo_a, eo_b, min_count, rcp));
    }
    __syncthreads();  // shared state is reused by the next tile
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
