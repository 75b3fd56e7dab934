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
// value), so the stored value is (T)(double)a[j]; for integer dtypes, which have no
// NaN, that makes the fill an element-wise copy through double.
#include "nbg_common.cuh"

#include <mutex>

namespace nbg {
namespace fill {

struct Last {
  long long idx;  // position of the last valid element, -1 if none
  double val;     // its value as float64 (numba's `current`)
};

struct LastOp {
  NBG_DEVICE Last identity() const { return Last{-1, 0.0}; }
  NBG_DEVICE Last combine(const Last& earlier, const Last& later) const {
    return later.idx >= 0 ? later : earlier;
  }
};

constexpr int NT = 256;

template <typename T, bool REVERSE, int K>
__global__ void __launch_bounds__(NT) fill_kernel(const T* __restrict__ a, T* __restrict__ out,
                                                  long long rows, long long n, long long limit,
                                                  long long tiles_per_row, void* ws_base,
                                                  size_t ws_bytes) {
  constexpr long long TILE = static_cast<long long>(NT) * K;
  __shared__ long long warp_idx[NT / 32];
  __shared__ double warp_val[NT / 32];
  __shared__ Last carry_smem;
  __shared__ long long tile_smem;
  const long long total_tiles = rows * tiles_per_row;
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);

  for (;;) {
    if (threadIdx.x == 0) tile_smem = claim_tile(ws.hdr);
    __syncthreads();
    const long long tile = tile_smem;
    if (tile >= total_tiles) break;
    const TileCoord tc = tile_coord(tile, rows);
    const long long row = tc.row, chunk = tc.chunk;
    // scan-order position q maps to array position i = q (ffill) or n-1-q (bfill)
    const long long q0 = chunk * TILE + static_cast<long long>(threadIdx.x) * K;
    const T* ar = a + row * n;
    T* orow = out + row * n;

    T v[K];
    long long li = -1;
    double lv = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long q = q0 + k;
      const long long i = REVERSE ? n - 1 - q : q;
      v[k] = q < n ? ar[i] : T(0);
      if (q < n && !is_nan(v[k])) {
        li = q;
        lv = static_cast<double>(v[k]);
      }
    }
    // warp inclusive scan of (li, lv): later valid wins
    long long si = li;
    double sv = lv;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const long long ui = __shfl_up_sync(0xffffffffu, si, d);
      const double uv = __shfl_up_sync(0xffffffffu, sv, d);
      if (lane >= d && si < 0) {
        si = ui;
        sv = uv;
      }
    }
    if (lane == 31) {
      warp_idx[warp] = si;
      warp_val[warp] = sv;
    }
    __syncthreads();
    if (warp == 0) {
      long long wi = lane < NT / 32 ? warp_idx[lane] : -1;
      double wv = lane < NT / 32 ? warp_val[lane] : 0.0;
#pragma unroll
      for (int d = 1; d < NT / 32; d <<= 1) {
        const long long ui = __shfl_up_sync(0xffffffffu, wi, d);
        const double uv = __shfl_up_sync(0xffffffffu, wv, d);
        if (lane >= d && wi < 0) {
          wi = ui;
          wv = uv;
        }
      }
      if (lane < NT / 32) {
        warp_idx[lane] = wi;
        warp_val[lane] = wv;
      }
    }
    __syncthreads();
    // exclusive prefix for this thread: previous lane's inclusive value, else the
    // previous warp's inclusive value
    long long ei = __shfl_up_sync(0xffffffffu, si, 1);
    double ev = __shfl_up_sync(0xffffffffu, sv, 1);
    if (lane == 0) {
      ei = -1;
      ev = 0.0;
    }
    if (ei < 0 && warp > 0) {
      ei = warp_idx[warp - 1];
      ev = warp_val[warp - 1];
    }
    if (warp == 0) {
      const Last agg{warp_idx[NT / 32 - 1], warp_val[NT / 32 - 1]};
      if (chunk == 0) {
        if (lane == 0) {
          if (tiles_per_row > 1) publish(ws, tile, epoch, kStatePrefix, agg);
          carry_smem = Last{-1, 0.0};
        }
      } else {
        if (lane == 0) publish(ws, tile, epoch, kStateAggregate, agg);
        __syncwarp();
        bool ok;
        const Last carry = warp_lookback<Last>(ws, tile, chunk, rows, epoch, LastOp(), ok);
        if (lane == 0) {
          publish(ws, tile, epoch, kStatePrefix, LastOp().combine(carry, agg));
          carry_smem = carry;
        }
      }
    }
    __syncthreads();
    if (ei < 0) {
      ei = carry_smem.idx;
      ev = carry_smem.val;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long q = q0 + k;
      if (q >= n) break;
      const long long i = REVERSE ? n - 1 - q : q;
      if (!is_nan(v[k])) {
        ei = q;
        ev = static_cast<double>(v[k]);
      }
      const double r = (ei >= 0 && q - ei <= limit) ? ev : nan;
      orow[i] = static_cast<T>(r);
    }
    __syncthreads();
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

}  // namespace fill
}  // namespace nbg

using namespace nbg;
using namespace nbg::fill;

namespace {
constexpr int kFillK = 16;

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
__device__ __align__(256) unsigned char g_fill_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The first call on a
// device looks the address up and zero-fills the array on `stream` (the fill kernel
// that follows on the same stream sees it cleared).  In host code the array's name
// is only a host-side stand-in, never a device address.
int noalloc_scratch(cudaStream_t stream, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return kLaunchError;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_fill_noalloc_scratch) != cudaSuccess || !p) return kLaunchError;
    if (cudaMemsetAsync(p, 0, kNoAllocScratchBytes, stream) != cudaSuccess) return kLaunchError;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
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
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  const int st = noalloc_scratch(s, &scratch);
  if (st != kOk) return st;
  return launch_fill<double, false>(a, out, rows, n, limit, scratch, kNoAllocScratchBytes, s);
}

}  // extern "C"
