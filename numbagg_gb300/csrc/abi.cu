// Library-level entry points: version, status strings, workspace error readout.
#include "nbg_common.cuh"

#include <atomic>

using namespace nbg;

namespace nbg {
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<int> g_deterministic{0};
void note_launches(int n) { g_launches.fetch_add(static_cast<unsigned long long>(n), std::memory_order_relaxed); }
bool deterministic_mode() { return g_deterministic.load(std::memory_order_relaxed) != 0; }
}  // namespace nbg

extern "C" {

unsigned long long nbg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

void nbg_set_deterministic(int on) { g_deterministic.store(on ? 1 : 0, std::memory_order_relaxed); }
int nbg_get_deterministic(void) { return g_deterministic.load(std::memory_order_relaxed); }

int nbg_version(void) { return 10000; }  // 1.0.0

const char* nbg_status_string(int status) {
  switch (status) {
    case kOk: return "ok";
    case kInvalidArgument: return "invalid argument";
    case kLaunchError: return "CUDA launch error";
    case kWorkspaceTooSmall: return "workspace missing or too small";
    case kLookbackTimeout: return "look-back wait exceeded its bound";
    case kUnsupported: return "unsupported shape or dtype";
    case kTooLarge: return "problem larger than the fixed scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

size_t nbg_workspace_header_bytes(void) { return sizeof(WsHeader); }

// Copy the device-side error word of a scan workspace to the host (synchronising
// `stream`), clear it, and report the code and the tile that raised it.
int nbg_workspace_error(void* ws, int* code, unsigned* tile, void* stream) {
  if (!ws || !code || !tile) return kInvalidArgument;
  WsHeader h;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&h, ws, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return kLaunchError;
  if (cudaStreamSynchronize(s) != cudaSuccess) return kLaunchError;
  *code = static_cast<int>(h.error);
  *tile = h.error_tile;
  if (h.error != 0) {
    unsigned zero[2] = {0u, 0u};
    if (cudaMemcpyAsync(reinterpret_cast<unsigned char*>(ws) + offsetof(WsHeader, error), zero,
                        sizeof(zero), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return kLaunchError;
    if (cudaStreamSynchronize(s) != cudaSuccess) return kLaunchError;
  }
  return kOk;
}

// Failure-detection check: a single CTA waits, with a short bound, on a tile status
// that nothing publishes.  The wait gives up, records kLookbackTimeout in the
// workspace header and the kernel returns normally; the host reads the code back
// with nbg_workspace_error.  No fault, trap or unbounded wait is involved.
int nbg_debug_lookback_timeout(void* ws, size_t ws_bytes, int spin_limit, void* stream);

}  // extern "C"

namespace {
__global__ void lookback_timeout_kernel(void* ws_base, size_t ws_bytes, int spin_limit) {
  Workspace ws = make_workspace(ws_base, ws_bytes);
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(&ws.hdr->epoch);
  if (threadIdx.x == 0) {
    // tile 0 of this launch never publishes; tile 1 waits for it
    if (wait_status(ws, 0, epoch + 1000000u, spin_limit) == kStateNone)
      record_error(ws.hdr, kLookbackTimeout, 1u);
  }
}
}  // namespace

extern "C" int nbg_debug_lookback_timeout(void* ws, size_t ws_bytes, int spin_limit, void* stream) {
  if (!ws || ws_bytes < workspace_bytes(2) || spin_limit <= 0 || spin_limit > (1 << 16))
    return kInvalidArgument;
  lookback_timeout_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(ws, ws_bytes, spin_limit);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

namespace nbg {
__global__ void ragged_plan_kernel(const long long* __restrict__ offsets, long long rows, long long item_len,
                                   long long* __restrict__ item_start) {
  __shared__ long long warp_sum[32];
  __shared__ long long carry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (long long base = 0; base < rows; base += blockDim.x) {
    const long long s = base + tid;
    long long v = 0;
    if (s < rows) {
      const long long len = offsets[s + 1] - offsets[s];
      v = len > 0 ? (len + item_len - 1) / item_len : 0;
    }
    long long incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const long long up = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += up;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const int nw = blockDim.x / 32;
      long long w = lane < nw ? warp_sum[lane] : 0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const long long up = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w += up;
      }
      if (lane < nw) warp_sum[lane] = w;
    }
    __syncthreads();
    const long long excl = carry + (warp ? warp_sum[warp - 1] : 0) + incl - v;
    if (s < rows) item_start[s] = excl;
    __syncthreads();
    if (tid == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (tid == 0) item_start[rows] = carry;
}

int layout_grid(long long max_items, int per_sm) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long cap = static_cast<long long>(sms) * per_sm;
  return static_cast<int>(max_items < cap ? (max_items > 0 ? max_items : 1) : cap);
}
}  // namespace nbg
