// Shared device helpers for the numbagg_gb300 kernels (sm_103a).
//
// * NaN tests and order keys work on the IEEE bit pattern with integer
//   instructions: on GB300 the FP64 pipe runs at ~1.6 DADD/clk/SM, so every
//   comparison moved off it is throughput for the arithmetic that needs it.
// * Workspace + decoupled look-back.  Scans along the row carry a state from tile
//   to tile.  Each tile publishes its local aggregate, then walks back over its
//   predecessors (Merrill & Garland, "Single-pass Parallel Prefix Scan with
//   Decoupled Look-back", 2016) until it meets an inclusive prefix.  Tiles are
//   handed out in row-major order through an atomic counter, so every tile a
//   waiter looks at has already been claimed by a running CTA and will publish
//   without waiting on anyone: the look-back cannot deadlock.  Every wait is
//   bounded all the same; when the bound is hit the kernel records an error code
//   in the workspace header, continues with a neutral carry and returns normally.
// * The workspace is zeroed once when it is allocated and then maintains itself:
//   status words carry a launch epoch, and the last CTA of a launch resets the
//   tile counter and advances the epoch, so no per-launch memset is needed.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "numbagg_gb300.h"  // the C ABI every translation unit implements

#ifndef NBG_HOST_DEVICE
#define NBG_HOST_DEVICE __host__ __device__ __forceinline__
#endif
#define NBG_DEVICE __device__ __forceinline__

namespace nbg {

// Host-side count of kernels launched by this library (defined in abi.cu).
void note_launches(int n);
// set through nbg_set_deterministic: only run-to-run reproducible algorithms
bool deterministic_mode();

// ---------------------------------------------------------------------------------
// error codes shared with the host (include/numbagg_gb300.h)
// ---------------------------------------------------------------------------------
enum Status : int {
  kOk = 0,
  kInvalidArgument = 1,
  kLaunchError = 2,
  kWorkspaceTooSmall = 3,
  kLookbackTimeout = 4,
  kUnsupported = 5,
  kTooLarge = 6,
};

// ---------------------------------------------------------------------------------
// bit-level predicates
// ---------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------
// L2 cache policies: inputs streamed once are read with evict-first so that they do
// not displace data that is reused (reduction targets, shared labels), which is
// updated with evict-last.
// ---------------------------------------------------------------------------------
NBG_DEVICE unsigned long long l2_evict_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
NBG_DEVICE unsigned long long l2_evict_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
NBG_DEVICE double ld_hint(const double* a, unsigned long long pol) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE float ld_hint(const float* a, unsigned long long pol) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE int ld_hint(const int* a, unsigned long long pol) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE long long ld_hint(const long long* a, unsigned long long pol) {
  long long v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE void red_add_hint(double* a, double v, unsigned long long pol) {
  asm volatile("red.global.add.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(a), "d"(v), "l"(pol) : "memory");
}
NBG_DEVICE void red_max_hint(unsigned long long* a, unsigned long long v, unsigned long long pol) {
  asm volatile("red.global.max.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(a), "l"(v), "l"(pol) : "memory");
}
NBG_DEVICE void red_min_hint(unsigned long long* a, unsigned long long v, unsigned long long pol) {
  asm volatile("red.global.min.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(a), "l"(v), "l"(pol) : "memory");
}
NBG_DEVICE unsigned long long ld_keep(const unsigned long long* a, unsigned long long pol) {
  unsigned long long v;
  asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE void red_add_hint(unsigned* a, unsigned v, unsigned long long pol) {
  asm volatile("red.global.add.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(a), "r"(v), "l"(pol) : "memory");
}
NBG_DEVICE void red_max_hint(unsigned* a, unsigned v, unsigned long long pol) {
  asm volatile("red.global.max.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(a), "r"(v), "l"(pol) : "memory");
}
NBG_DEVICE unsigned ld_keep(const unsigned* a, unsigned long long pol) {
  unsigned v;
  asm volatile("ld.global.cg.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}

// Ask L2 for a line ahead of its use (no register, no fault on a valid address); the
// column kernels walk a column serially, so this is their memory-level parallelism.
NBG_DEVICE void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
constexpr long long kColPrefetch = 16;  // positions ahead

// Values handled as raw bits.  Loading a float array through its integer twin keeps
// every test on the integer pipes: a NaN test on a float64 register can be compiled
// to a float64 compare, and this GPU's FP64 pipe takes 16 cycles per warp instruction.
template <typename T>
struct BitsOf {
  typedef T type;  // integers are their own bits
};
template <>
struct BitsOf<double> {
  typedef unsigned long long type;
};
template <>
struct BitsOf<float> {
  typedef unsigned type;
};
NBG_DEVICE bool nan_bits(unsigned long long b) { return (b << 1) > 0xffe0000000000000ull; }
NBG_DEVICE bool nan_bits(unsigned b) { return (b << 1) > 0xff000000u; }
NBG_DEVICE bool nan_bits(int) { return false; }
NBG_DEVICE bool nan_bits(long long) { return false; }
template <typename T>
NBG_DEVICE const typename BitsOf<T>::type* as_bits(const T* p) {
  return reinterpret_cast<const typename BitsOf<T>::type*>(p);
}
template <typename T>
NBG_DEVICE typename BitsOf<T>::type* as_bits(T* p) {
  return reinterpret_cast<typename BitsOf<T>::type*>(p);
}
NBG_DEVICE unsigned long long ld_hint(const unsigned long long* a, unsigned long long pol) {
  unsigned long long v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol));
  return v;
}
NBG_DEVICE unsigned ld_hint(const unsigned* a, unsigned long long pol) {
  unsigned v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}

// the quiet NaN numpy writes (np.nan), in the type of the argument
NBG_DEVICE double quiet_nan(double) { return __longlong_as_double(0x7ff8000000000000ll); }
NBG_DEVICE float quiet_nan(float) { return __int_as_float(0x7fc00000); }
// Counts as floating-point values built from their bit patterns: the conversion
// instructions from 64-bit integers execute on this GPU's slow FP64 pipe.
// Exact for 0 <= c < 2^53 (float64) and 0 <= c < 2^24 (float32).
NBG_DEVICE double f64_of_count(long long c) {
  if (c <= 0) return c == 0 ? 0.0 : static_cast<double>(c);
  const int lz = __clzll(c);
  const unsigned long long frac = ((static_cast<unsigned long long>(c) << lz) << 1) >> 12;
  return __longlong_as_double(static_cast<long long>((static_cast<unsigned long long>(1086 - lz) << 52) | frac));
}
NBG_DEVICE float f32_of_count(long long c) {
  if (c <= 0 || c >= (1ll << 24)) return static_cast<float>(c);
  const unsigned u = static_cast<unsigned>(c);
  const int lz = __clz(static_cast<int>(u));
  const unsigned frac = ((u << lz) << 1) >> 9;
  return __uint_as_float((static_cast<unsigned>(158 - lz) << 23) | frac);
}

NBG_DEVICE bool is_nan(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
NBG_DEVICE bool is_nan(float x) {
  return (static_cast<unsigned>(__float_as_int(x)) & 0x7fffffffu) > 0x7f800000u;
}
template <typename T>
NBG_DEVICE bool is_nan(T) { return false; }  // integers

// Monotone unsigned key of a float: a < b  <=>  key(a) < key(b) for non-NaN values.
// -0.0 and +0.0 get different keys (-0 < +0); callers that need IEEE equality of
// zeros compare keys only after mapping -0 to +0 (see order_key_ieee).
NBG_DEVICE unsigned long long order_key(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
// IEEE order: -0.0 == +0.0 share a key.
NBG_DEVICE unsigned long long order_key_ieee(double x) {
  unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  if ((b << 1) == 0) b = 0;  // +-0 -> +0
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

template <typename T>
struct Vec2;
template <>
struct Vec2<double> { using type = double2; };
template <>
struct Vec2<float> { using type = float2; };

// ---------------------------------------------------------------------------------
// workspace layout
// ---------------------------------------------------------------------------------
struct WsHeader {
  unsigned long long tile_counter;  // next tile to claim (dynamic, row-major)
  unsigned long long done_counter;  // CTAs finished this launch
  unsigned int epoch;               // launch epoch tagging the status words
  unsigned int error;               // first error code recorded on the device
  unsigned int error_tile;          // tile that recorded it
  unsigned int pad[57];
};
static_assert(sizeof(WsHeader) == 256, "header must stay 256 bytes");

// Each tile has two payload slots, one for its aggregate and one for its inclusive
// prefix, each written once per launch: a reader that saw "aggregate" must never
// find the slot rewritten under it by the later prefix.
constexpr int kPayloadBytes = 128;  // per slot
constexpr int kSlotsPerTile = 2;
constexpr unsigned kStateNone = 0, kStateAggregate = 1, kStatePrefix = 2;

struct Workspace {
  WsHeader* hdr;
  unsigned long long* status;  // one word per tile: (epoch << 2) | state
  unsigned char* payload;      // kPayloadBytes per tile
};

NBG_HOST_DEVICE size_t workspace_bytes(long long tiles) {
  return 256 + static_cast<size_t>(tiles) * (8 + kSlotsPerTile * kPayloadBytes) + 256;
}

// The layout depends only on the workspace size, so every kernel that shares a
// workspace sees status words only where status words are written.
NBG_HOST_DEVICE Workspace make_workspace(void* base, size_t bytes) {
  Workspace w;
  unsigned char* p = static_cast<unsigned char*>(base);
  const size_t cap = bytes > 512 ? (bytes - 512) / (8 + kSlotsPerTile * kPayloadBytes) : 0;
  w.hdr = reinterpret_cast<WsHeader*>(p);
  w.status = reinterpret_cast<unsigned long long*>(p + 256);
  size_t off = 256 + cap * 8;
  off = (off + 127) & ~static_cast<size_t>(127);
  w.payload = p + off;
  return w;
}

NBG_DEVICE void record_error(WsHeader* h, unsigned code, unsigned tile) {
  if (atomicCAS(&h->error, 0u, code) == 0u) h->error_tile = tile;
}

// Claim the next tile (called by one thread; the caller broadcasts it).
NBG_DEVICE long long claim_tile(WsHeader* h) {
  return static_cast<long long>(atomicAdd(&h->tile_counter, 1ull));
}

// Tiles are claimed row-interleaved: claim t is chunk t / rows of row t % rows, so
// the predecessor of a tile (same row, previous chunk) was claimed `rows` claims
// earlier and is usually finished by the time the tile looks back.
struct TileCoord {
  long long row, chunk;
};
NBG_HOST_DEVICE TileCoord tile_coord(long long t, long long rows) {
  TileCoord c;
  c.chunk = t / rows;
  c.row = t - c.chunk * rows;
  return c;
}

// Called by one thread of every CTA when the CTA has no more tiles.  The last CTA
// resets the counters and advances the epoch for the next launch on this workspace.
NBG_DEVICE void finish_cta(WsHeader* h) {
  __threadfence();
  const unsigned long long done = atomicAdd(&h->done_counter, 1ull) + 1ull;
  if (done == static_cast<unsigned long long>(gridDim.x) * gridDim.y * gridDim.z) {
    h->tile_counter = 0ull;
    h->done_counter = 0ull;
    __threadfence();
    atomicAdd(&h->epoch, 1u);
  }
}

// status word: epoch << 8 | 0xA0 | state  (the tag byte keeps zeroed memory and
// stray words from ever reading as a published state)
NBG_DEVICE unsigned long long status_word(unsigned epoch, unsigned state) {
  return (static_cast<unsigned long long>(epoch) << 8) | 0xA0ull | state;
}

NBG_DEVICE unsigned char* payload_slot(const Workspace& ws, long long tile, unsigned state) {
  return ws.payload + (static_cast<size_t>(tile) * kSlotsPerTile + (state == kStatePrefix ? 1 : 0)) * kPayloadBytes;
}

template <typename P>
NBG_DEVICE void publish(const Workspace& ws, long long tile, unsigned epoch, unsigned state,
                        const P& value) {
  static_assert(sizeof(P) <= kPayloadBytes, "payload too large");
  P* slot = reinterpret_cast<P*>(payload_slot(ws, tile, state));
  *slot = value;
  __threadfence();
  atomicExch(ws.status + tile, status_word(epoch, state));
}

// Spin until `tile` has published for this epoch; returns the state (Aggregate or
// Prefix) or kStateNone after the bound (error recorded by the caller).
constexpr int kDefaultSpinLimit = 1 << 21;  // ~2 s with the back-off below

NBG_DEVICE unsigned wait_status(const Workspace& ws, long long tile, unsigned epoch,
                                int spin_limit = kDefaultSpinLimit) {
  unsigned ns = 32;
  for (int it = 0; it < spin_limit; ++it) {
    const unsigned long long s = atomicAdd(ws.status + tile, 0ull);
    if ((s >> 8) == static_cast<unsigned long long>(epoch) && (s & 0xFCull) == 0xA0ull &&
        (s & 3ull) != 0ull) {
      __threadfence();
      return static_cast<unsigned>(s & 3ull);
    }
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
  }
  return kStateNone;
}

template <typename P>
NBG_DEVICE P read_payload(const Workspace& ws, long long tile, unsigned state) {
  const volatile unsigned* src = reinterpret_cast<const volatile unsigned*>(payload_slot(ws, tile, state));
  P v;
  // copy through volatile words so the compiler cannot hoist the load above the wait
  unsigned* dst = reinterpret_cast<unsigned*>(&v);
#pragma unroll
  for (int i = 0; i < static_cast<int>(sizeof(P) / 4); ++i) dst[i] = src[i];
  return v;
}

template <typename P>
NBG_DEVICE P shfl_down_pod(const P& v, int off) {
  static_assert(sizeof(P) % 4 == 0, "payload must be whole words");
  P r;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < static_cast<int>(sizeof(P) / 4); ++i) d[i] = __shfl_down_sync(0xffffffffu, s[i], off);
  return r;
}

template <typename P>
NBG_DEVICE P shfl_idx_pod(const P& v, int src_lane) {
  P r;
  const unsigned* s = reinterpret_cast<const unsigned*>(&v);
  unsigned* d = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int i = 0; i < static_cast<int>(sizeof(P) / 4); ++i) d[i] = __shfl_sync(0xffffffffu, s[i], src_lane);
  return r;
}

// Exclusive look-back for `tile`, run by all 32 lanes of one warp.  The tile's
// predecessors are tile - stride, tile - 2*stride, ... (`chunk` of them).  Each round
// the 32 lanes wait on 32 predecessors at once (lane 0 the nearest), take the nearest
// inclusive prefix among them if any, and fold the states in time order with an
// ordered warp reduction (`Op::combine(earlier, later)` must be associative; it need
// not commute).  Every lane returns the prefix.
template <typename P, typename Op>
NBG_DEVICE P warp_lookback(const Workspace& ws, long long tile, long long chunk, long long stride,
                           unsigned epoch, const Op& op, bool& ok) {
  const int lane = threadIdx.x & 31;
  P acc = op.identity();
  ok = true;
  for (long long done = 0; done < chunk; done += 32) {
    const long long left = chunk - done;
    const int n = left < 32 ? static_cast<int>(left) : 32;
    P v = op.identity();
    unsigned st = kStatePrefix;
    if (lane < n) {
      const long long p = tile - stride * (done + 1 + lane);
      st = wait_status(ws, p, epoch);
      if (st != kStateNone) v = read_payload<P>(ws, p, st);
    }
    if (__ballot_sync(0xffffffffu, lane < n && st == kStateNone)) {
      if (lane == 0) record_error(ws.hdr, kLookbackTimeout, static_cast<unsigned>(tile));
      ok = false;
      return acc;
    }
    const unsigned pref = __ballot_sync(0xffffffffu, lane < n && st == kStatePrefix);
    const int lim = pref ? (__ffs(static_cast<int>(pref)) - 1) : n - 1;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const P other = shfl_down_pod(v, off);
      if ((lane & (2 * off - 1)) == 0 && lane + off <= lim) v = op.combine(other, v);
    }
    v = shfl_idx_pod(v, 0);
    acc = op.combine(v, acc);
    if (pref) break;
  }
  return acc;
}

// ---------------------------------------------------------------------------------
// block-wide helpers
// ---------------------------------------------------------------------------------
template <typename T>
NBG_DEVICE T shfl_up(T v, int d) {
  return __shfl_up_sync(0xffffffffu, v, d);
}

// Broadcast a value from thread 0 of the block through shared memory.
template <typename T>
NBG_DEVICE T block_broadcast(T v, T* smem_slot) {
  if (threadIdx.x == 0) *smem_slot = v;
  __syncthreads();
  T r = *smem_slot;
  __syncthreads();
  return r;
}

}  // namespace nbg

namespace nbg {

// ---------------------------------------------------------------------------------
// rectangular rows or ragged series
// ---------------------------------------------------------------------------------
// A batch is either `rows` rows of `n` values (offsets == nullptr) or `rows` series of
// uneven length in one flat buffer, series s covering [offsets[s], offsets[s + 1]).
// Kernels walk work items (chunks or tiles of a series); for ragged batches
// `item_start[s]` is the first item of series s and item_start[rows] the total, as
// computed on the device by ragged_plan_kernel, so launches need no host round trip.
struct Layout {
  const long long* offsets;
  const long long* item_start;
  long long rows, n, items_per_row;
};
struct Item {
  long long row, index, base, len;  // series, item within it, first element, series length
};
NBG_DEVICE long long layout_items(const Layout& L) {
  return L.offsets ? L.item_start[L.rows] : L.rows * L.items_per_row;
}
NBG_DEVICE Item layout_item(const Layout& L, long long id) {
  Item it;
  if (!L.offsets) {
    it.row = id / L.items_per_row;
    it.index = id - it.row * L.items_per_row;
    it.base = it.row * L.n;
    it.len = L.n;
    return it;
  }
  long long lo = 0, hi = L.rows - 1;  // last series whose first item is <= id
  while (lo < hi) {
    const long long mid = (lo + hi + 1) >> 1;
    if (L.item_start[mid] <= id) lo = mid;
    else hi = mid - 1;
  }
  it.row = lo;
  it.index = id - L.item_start[lo];
  it.base = L.offsets[lo];
  it.len = L.offsets[lo + 1] - it.base;
  return it;
}
NBG_DEVICE long long layout_row_len(const Layout& L, long long r) {
  return L.offsets ? L.offsets[r + 1] - L.offsets[r] : L.n;
}
NBG_DEVICE long long layout_row_base(const Layout& L, long long r) { return L.offsets ? L.offsets[r] : r * L.n; }

// item_start[s] = sum over earlier series of ceil(len / item_len); one CTA of 1024 threads
__global__ void ragged_plan_kernel(const long long* __restrict__ offsets, long long rows, long long item_len,
                                   long long* __restrict__ item_start);
// persistent grid for a layout: `per_sm` CTAs per SM, fewer when the items are fewer
int layout_grid(long long max_items, int per_sm);

}  // namespace nbg
