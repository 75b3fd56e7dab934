// ffill / bfill (numbagg/funcs.py:294-326).
//
// The reference carries `current` and a `lives_remaining` countdown through the row.
// Equivalently, out[i] = a[j] where j is the last valid position <= i (first valid
// position >= i for bfill), provided |i - j| <= limit, else NaN.  "Last valid index"
// is an inclusive max-scan of (valid ? i : -1), so the kernel is a segmented scan:
// each thread scans K consecutive positions, warp shuffles combine threads, and the
// (index, value) of the last valid element before a tile arrives through decoupled
// look-back.  Only selection happens, no arithmetic, so the result is bit-exact.
//
// bfill runs the same scan over the row reversed: tile c of the scan covers the
// c-th chunk counted from the end of the row.
//
// numba types the carried `current` as float64 (unified from `np.nan` and the
// value), so the stored value is (T)(double)a[j].  For float32 and float64 that is
// a[j] itself, so the float kernel moves bit patterns and never touches a float
// register; for integer dtypes, which have no NaN, it makes the fill an element-wise
// copy through double.
#include "nbg_common.cuh"

namespace nbg {
namespace fill {

struct Last {
  long long idx;           // position of the last valid element, -1 if none
  unsigned long long val;  // its bit pattern (a float32 in the low half)
};

struct LastOp {
  NBG_DEVICE Last identity() const { return Last{-1, 0}; }
  NBG_DEVICE Last combine(const Last& earlier, const Last& later) const {
    return later.idx >= 0 ? later : earlier;
  }
};

constexpr int NT = 256;

// One CTA scans tiles of NT * K positions; warp w owns the K * 32 consecutive
// positions starting at w * K * 32, in K groups of 32 (lane l of group j holds
// position j * 32 + l, so every load and store of a warp is one contiguous run).
// Within a group, lane l's last valid position is the highest set bit of the group's
// valid ballot at or below l; a group without one inherits the warp's running
// (position, value).  Positions before the warp's first valid element need the carry
// from earlier warps or tiles and are written after it is known: the warp's carry-in
// is the last valid element of the earlier warps of the tile, else the tile's
// exclusive prefix from decoupled look-back.  A tile holding a valid element already
// knows its inclusive prefix (its own last valid element) and publishes it at once,
// and it looks back only if its first position is NaN.
template <typename T, bool REVERSE, int K>
__global__ void __launch_bounds__(NT, 3) fill_kernel(const T* __restrict__ a, T* __restrict__ out,
                                                  long long rows, long long n, long long limit,
                                                  long long tiles_per_row, void* ws_base,
                                                  size_t ws_bytes) {
  constexpr long long WSPAN = 32LL * K;
  constexpr long long TILE = WSPAN * (NT / 32);
  constexpr int NW = NT / 32;
  __shared__ long long w_idx[NW];
  __shared__ unsigned long long w_val[NW];
  __shared__ int w_first[NW];
  __shared__ long long in_idx[NW];
  __shared__ unsigned long long in_val[NW];
  __shared__ long long tile_smem;
  const long long total_tiles = rows * tiles_per_row;
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lane_le = 0xffffffffu >> (31 - lane);
  typedef typename BitsOf<T>::type B;  // the scan moves bit patterns only
  const B nan = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);

  for (;;) {
    if (threadIdx.x == 0) tile_smem = claim_tile(ws.hdr);
    __syncthreads();
    const long long tile = tile_smem;
    if (tile >= total_tiles) break;
    const TileCoord tc = tile_coord(tile, rows);
    const long long row = tc.row, chunk = tc.chunk;
    // scan-order position q maps to array position i = q (ffill) or n-1-q (bfill)
    const long long wq0 = chunk * TILE + static_cast<long long>(warp) * WSPAN;
    const B* ar = as_bits(a) + row * n;
    B* orow = as_bits(out) + row * n;

    B v[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long q = wq0 + j * 32 + lane;
      v[j] = q < n ? __ldcs(ar + (REVERSE ? n - 1 - q : q)) : B(0);
    }
    long long cidx = -1;  // the warp's running last valid position (uniform)
    B cval = B(0);
    int first = static_cast<int>(WSPAN);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const long long qb = wq0 + j * 32;
      const long long q = qb + lane;
      const bool valid = q < n && !nan_bits(v[j]);
      const unsigned msk = __ballot_sync(0xffffffffu, valid);
      const unsigned mle = msk & lane_le;
      const int src = mle ? 31 - __clz(mle) : lane;
      const B sv = __shfl_sync(0xffffffffu, v[j], src);
      long long ei = cidx;
      B ev = cval;
      if (mle) {
        ei = qb + src;
        ev = sv;
      }
      if (msk) {
        const int top = 31 - __clz(msk);
        cval = __shfl_sync(0xffffffffu, v[j], top);
        cidx = qb + top;
        if (first == static_cast<int>(WSPAN)) first = j * 32 + __ffs(msk) - 1;
      }
      if (q < n && ei >= 0) orow[REVERSE ? n - 1 - q : q] = (q - ei <= limit) ? ev : nan;
    }
    if (lane == 0) {
      w_idx[warp] = cidx;
      w_val[warp] = static_cast<unsigned long long>(cval);
      w_first[warp] = first;
    }
    __syncthreads();
    if (warp == 0) {
      long long li = -1;
      unsigned long long lv = 0;
      if (lane == 0) {
        for (int w = 0; w < NW; ++w) {  // carry-in of every warp from the earlier warps
          in_idx[w] = li;
          in_val[w] = lv;
          if (w_idx[w] >= 0) {
            li = w_idx[w];
            lv = w_val[w];
          }
        }
      }
      li = __shfl_sync(0xffffffffu, li, 0);
      lv = __shfl_sync(0xffffffffu, lv, 0);
      const Last agg{li, lv};
      Last excl{-1, 0};
      if (chunk == 0) {
        if (lane == 0 && tiles_per_row > 1) publish(ws, tile, epoch, kStatePrefix, agg);
      } else if (agg.idx >= 0) {
        if (lane == 0) publish(ws, tile, epoch, kStatePrefix, agg);
        if (w_first[0] != 0) {  // leading NaNs: the carry from earlier tiles is needed
          __syncwarp();
          bool ok;
          excl = warp_lookback<Last>(ws, tile, chunk, rows, epoch, LastOp(), ok);
        }
      } else {  // no valid element: the inclusive prefix is the exclusive one
        if (lane == 0) publish(ws, tile, epoch, kStateAggregate, agg);
        __syncwarp();
        bool ok;
        excl = warp_lookback<Last>(ws, tile, chunk, rows, epoch, LastOp(), ok);
        if (lane == 0) publish(ws, tile, epoch, kStatePrefix, excl);
      }
      if (lane == 0) {
        for (int w = 0; w < NW; ++w) {
          if (in_idx[w] < 0) {
            in_idx[w] = excl.idx;
            in_val[w] = excl.val;
          }
        }
      }
    }
    __syncthreads();
    // the positions before the warp's first valid element
    if (first > 0) {
      const long long ci = in_idx[warp];
      const B cv = static_cast<B>(in_val[warp]);
      const long long qend = min(wq0 + first, n);
      for (long long q = wq0 + lane; q < qend; q += 32)
        orow[REVERSE ? n - 1 - q : q] = (ci >= 0 && q - ci <= limit) ? cv : nan;
    }
  }
  if (threadIdx.x == 0) finish_cta(ws.hdr);
}

// Integer arrays have no NaN: out = (T)(double)a (numba's float64 `current`).
template <typename T>
__global__ void fill_int_kernel(const T* __restrict__ a, T* __restrict__ out, long long total) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += stride)
    out[i] = static_cast<T>(static_cast<double>(a[i]));
}

// Along a non-last axis of a C-contiguous array (`outer` blocks of n x `inner` values,
// position p of column i of block o at (o n + p) inner + i): one thread per column
// carries the last valid position and value down it, so consecutive threads touch
// consecutive addresses and nothing is copied.  Bit patterns only, as above.
template <typename T, bool REVERSE>
__global__ void __launch_bounds__(256) fill_cols_kernel(const T* __restrict__ a, T* __restrict__ out,
                                                        long long outer, long long n, long long inner,
                                                        long long limit) {
  typedef typename BitsOf<T>::type B;
  const B nan = sizeof(B) == 8 ? static_cast<B>(0x7ff8000000000000ull) : static_cast<B>(0x7fc00000u);
  const long long col = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (col >= outer * inner) return;
  const long long o = col / inner, i = col - o * inner;
  const B* src = as_bits(a) + o * n * inner + i;
  B* dst = as_bits(out) + o * n * inner + i;
  long long last = -1;
  B lv = B(0);
  for (long long q = 0; q < n; ++q) {
    const long long p = REVERSE ? n - 1 - q : q;
    const B v = src[p * inner];
    if (!nan_bits(v)) {
      last = q;
      lv = v;
    }
    dst[p * inner] = (last >= 0 && q - last <= limit) ? lv : nan;
  }
}

}  // namespace fill
}  // namespace nbg

using namespace nbg;
using namespace nbg::fill;

namespace {
constexpr int kFillK = 16;

template <typename T>
struct IsFloatT {
  static constexpr bool value = false;
};
template <>
struct IsFloatT<double> {
  static constexpr bool value = true;
};
template <>
struct IsFloatT<float> {
  static constexpr bool value = true;
};

long long fill_tiles_per_row(long long n) {
  const long long tile = static_cast<long long>(NT) * kFillK;
  return n <= 0 ? 0 : (n + tile - 1) / tile;
}

int fill_grid(long long total_tiles) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long cap = static_cast<long long>(sms) * 8;
  return static_cast<int>(total_tiles < cap ? total_tiles : cap);
}

template <typename T, bool REVERSE>
int launch_fill(const T* a, T* out, long long rows, long long n, long long limit, void* ws,
                size_t ws_bytes, cudaStream_t stream) {
  if (rows < 0 || n < 0 || limit < 0) return kInvalidArgument;
  if (rows == 0 || n == 0) return kOk;
  if (!a || !out) return kInvalidArgument;
  const long long tpr = fill_tiles_per_row(n);
  const long long total = rows * tpr;
  if (!ws || ws_bytes < workspace_bytes(total)) return kWorkspaceTooSmall;
  fill_kernel<T, REVERSE, kFillK><<<fill_grid(total), NT, 0, stream>>>(a, out, rows, n, limit,
                                                                       tpr, ws, ws_bytes);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

template <typename T>
int launch_fill_int(const T* a, T* out, long long rows, long long n, long long limit,
                    cudaStream_t stream) {
  if (rows < 0 || n < 0 || limit < 0) return kInvalidArgument;
  const long long total = rows * n;
  if (total == 0) return kOk;
  if (!a || !out) return kInvalidArgument;
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  fill_int_kernel<T><<<static_cast<int>(blocks), 256, 0, stream>>>(a, out, total);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
template <typename T, bool REVERSE>
int launch_fill_cols(const T* a, T* out, long long outer, long long n, long long inner, long long limit,
                     cudaStream_t stream) {
  if (outer < 0 || n < 0 || inner < 0 || limit < 0) return kInvalidArgument;
  const long long cols = outer * inner;
  if (cols == 0 || n == 0) return kOk;
  if (!a || !out) return kInvalidArgument;
  const long long blocks = (cols + 255) / 256;
  if (blocks > 0x7fffffffLL) return kUnsupported;
  if (IsFloatT<T>::value)
    fill_cols_kernel<T, REVERSE><<<static_cast<int>(blocks), 256, 0, stream>>>(a, out, outer, n, inner, limit);
  else
    fill_int_kernel<T><<<static_cast<int>(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, stream>>>(a, out, cols * n);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}
}  // namespace

extern "C" {

size_t nbg_fill_workspace_bytes(long long rows, long long n) {
  return workspace_bytes(rows * fill_tiles_per_row(n));
}

#define NBG_FILL_F(T, SFX)                                                                    \
  int nbg_ffill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,        \
                      void* ws, size_t ws_bytes, void* stream) {                               \
    return launch_fill<T, false>(a, out, rows, n, limit, ws, ws_bytes,                         \
                                 static_cast<cudaStream_t>(stream));                           \
  }                                                                                            \
  int nbg_bfill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,        \
                      void* ws, size_t ws_bytes, void* stream) {                               \
    return launch_fill<T, true>(a, out, rows, n, limit, ws, ws_bytes,                          \
                                static_cast<cudaStream_t>(stream));                            \
  }
#define NBG_FILL_I(T, SFX)                                                                    \
  int nbg_ffill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,        \
                      void* ws, size_t ws_bytes, void* stream) {                               \
    (void)ws; (void)ws_bytes;                                                                  \
    return launch_fill_int<T>(a, out, rows, n, limit, static_cast<cudaStream_t>(stream));      \
  }                                                                                            \
  int nbg_bfill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,        \
                      void* ws, size_t ws_bytes, void* stream) {                               \
    (void)ws; (void)ws_bytes;                                                                  \
    return launch_fill_int<T>(a, out, rows, n, limit, static_cast<cudaStream_t>(stream));      \
  }

NBG_FILL_F(double, f64)
NBG_FILL_F(float, f32)
NBG_FILL_I(int, i32)
NBG_FILL_I(long long, i64)
// Along a non-last axis (fill_cols_kernel).  Integer arrays have no NaN: a copy, as
// above.
#define NBG_FILL_COLS(T, SFX)                                                                      \
  int nbg_ffill_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner,        \
                           long long limit, void* stream) {                                         \
    return launch_fill_cols<T, false>(a, out, outer, n, inner, limit, static_cast<cudaStream_t>(stream)); \
  }                                                                                                 \
  int nbg_bfill_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner,        \
                           long long limit, void* stream) {                                         \
    return launch_fill_cols<T, true>(a, out, outer, n, inner, limit, static_cast<cudaStream_t>(stream)); \
  }
NBG_FILL_COLS(double, f64)
NBG_FILL_COLS(float, f32)
NBG_FILL_COLS(int, i32)
NBG_FILL_COLS(long long, i64)

}  // extern "C"

// ---------------------------------------------------------------------------------
// Allocation-free forward fill
//
// Some callers cannot allocate device memory at all: a host application that owns
// every byte of GPU memory and hands this library only its input and output buffers
// (a database or stream engine running it as a user-defined function under a fixed
// memory budget), or a latency-critical path that must never reach cudaMalloc /
// cudaFree, which can synchronise the whole device.  For them nbg_ffill_f64_noalloc
// keeps the look-back state in a fixed array in device memory that is part of this
// library's image (every GPU that loads the library holds it until the process exits)
// instead of a caller-provided workspace.
// ---------------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = static_cast<size_t>(4) << 20;  // 4 MiB per device
// Zero when the module loads (PTX initialises .global variables without an initialiser
// to zero), which is the state a look-back workspace must start in; every launch
// leaves it that way again (the last CTA resets the counters), so no call clears it.
__device__ __align__(256) unsigned char g_fill_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.  In host code the
// array's name is only a host-side stand-in, never a device address, so every call
// asks the runtime for the address on the device that is current.  The lookup
// allocates nothing; doing it on every call (rather than caching it per device) keeps
// a call after cudaDeviceReset from launching on the address of a module that is gone.
int noalloc_scratch(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_fill_noalloc_scratch) != cudaSuccess || !p) return kLaunchError;
  *out = p;
  return kOk;
}

}  // namespace

extern "C" {

size_t nbg_ffill_noalloc_max_scratch_bytes(void) { return kNoAllocScratchBytes; }

int nbg_ffill_f64_noalloc(const double* a, double* out, long long rows, long long n, long long limit,
                          void* stream) {
  if (rows < 0 || n < 0 || limit < 0) return kInvalidArgument;
  if (rows == 0 || n == 0) return kOk;
  if (!a || !out) return kInvalidArgument;
  const long long tpr = fill_tiles_per_row(n);
  if (workspace_bytes(rows * tpr) > kNoAllocScratchBytes) return kTooLarge;
  void* scratch = nullptr;
  const int st = noalloc_scratch(&scratch);
  if (st != kOk) return st;
  return launch_fill<double, false>(a, out, rows, n, limit, scratch, kNoAllocScratchBytes,
                                    static_cast<cudaStream_t>(stream));
}

// The error word of the fixed scratch: a look-back wait that ran out of its bound
// during an earlier call records NBG_LOOKBACK_TIMEOUT there (and the tile), exactly as
// it does in a caller's workspace, where nbg_workspace_error reads it.  Synchronises
// `stream`, then clears the word.  Plain copies of 8 bytes to and from host memory;
// nothing is allocated.
int nbg_ffill_noalloc_error(int* code, unsigned* tile, void* stream) {
  if (!code || !tile) return kInvalidArgument;
  void* scratch = nullptr;
  const int st = noalloc_scratch(&scratch);
  if (st != kOk) return st;
  return nbg_workspace_error(scratch, code, tile, stream);
}

}  // extern "C"
