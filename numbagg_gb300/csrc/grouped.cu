// Labelled reductions group_nan* (numbagg/grouped.py:7-270).
//
// values (rows, m), labels (m,) shared by every row, out (rows, K).  A label < 0 is
// skipped (numbagg/grouped.py:14); a label >= K is skipped as well (numba would write
// out of bounds there, so the reference leaves it undefined).
//
// This file holds the integer sums, counts and sums of squares and every product,
// any and all; float moments and every selection (argmax/argmin/max/min/first/last)
// live in grouped_fast.cuh.  Two strategies, picked on the host from K:
//   * shared-memory bins (K * 24 B fits in shared memory): a CTA owns one column
//     chunk of one row and accumulates into bins in shared memory, replicated per
//     lane (no atomics) for tiny K, per warp for small K, or per CTA; at the end it
//     writes one partial state per bin.  A second kernel folds the partials over the
//     chunks in chunk order and writes the output, so results repeat run to run.
//   * global bins (large K, e.g. 10^6 labels): atomics into an accumulator in the
//     workspace, then the same fold/finalise kernel with one chunk.
//
// Integer sums, products and sums of squares wrap modulo 2^64 and are truncated to
// the output type, which equals numba's int64 arithmetic stored into the narrow
// output; integer results are therefore exact in any order.
#include "grouped_common.cuh"

namespace nbg {
namespace grouped {

constexpr int NT = 256;

// ---- shared-memory strategy -------------------------------------------------------
// grid (chunks, rows).  REP replicas of the K bins: 1 (per CTA), NT/32 (per warp) or
// NT (per thread, plain read-modify-write).
template <int F, typename V, typename L, int REP>
__global__ void __launch_bounds__(NT) accum_smem(const V* __restrict__ values,
                                                 const L* __restrict__ labels, long long m,
                                                 long long K, long long chunk_len,
                                                 Acc* __restrict__ partials) {
  extern __shared__ Acc bins[];
  const long long row = blockIdx.y;
  const long long chunk = blockIdx.x;
  const long long col0 = chunk * chunk_len;
  long long col1 = col0 + chunk_len;
  if (col1 > m) col1 = m;
  const long long nbins = K * REP;
  for (long long j = threadIdx.x; j < nbins; j += NT) bins[j] = acc_init<F, V>();
  __syncthreads();
  const int rep = REP == 1 ? 0 : (REP == NT ? threadIdx.x : (threadIdx.x >> 5));
  Acc* my = bins + static_cast<long long>(rep) * K;
  const V* vr = values + row * m;
  constexpr bool ATOMIC = REP != NT;
  for (long long col = col0 + threadIdx.x; col < col1; col += NT) {
    const long long lab = static_cast<long long>(labels[col]);
    if (lab < 0 || lab >= K) continue;
    const V v = vr[col];
    if (is_nan(v)) continue;
    accumulate<F, V, ATOMIC>(my + lab, v, static_cast<unsigned long long>(col));
  }
  __syncthreads();
  if (is_select(F)) {
    // second sweep: first column holding the bin's extreme key
    for (long long col = col0 + threadIdx.x; col < col1; col += NT) {
      const long long lab = static_cast<long long>(labels[col]);
      if (lab < 0 || lab >= K) continue;
      const V v = vr[col];
      if (is_nan(v)) continue;
      const unsigned long long key = select_key(v, F == kArgMin || F == kMin);
      if (key == my[lab].a) atomicMin(&my[lab].b, static_cast<unsigned long long>(col));
    }
    __syncthreads();
  }
  Acc* out = partials + (row * gridDim.x + chunk) * K;
  for (long long k = threadIdx.x; k < K; k += NT) {
    Acc r = bins[k];
    for (int j = 1; j < REP; ++j) r = fold<F, V>(r, bins[static_cast<long long>(j) * K + k]);
    out[k] = r;
  }
}

// ---- global strategy -----------------------------------------------------------------
template <int F, typename V>
__global__ void init_global(Acc* __restrict__ acc, long long total) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += stride)
    acc[i] = acc_init<F, V>();
}

// grid (chunks, rows); PASS 0 accumulates, PASS 1 is the select tie sweep
template <int F, typename V, typename L, int PASS>
__global__ void __launch_bounds__(NT) accum_global(const V* __restrict__ values,
                                                   const L* __restrict__ labels, long long m,
                                                   long long K, long long chunk_len,
                                                   Acc* __restrict__ acc) {
  const long long row = blockIdx.y;
  const long long col0 = static_cast<long long>(blockIdx.x) * chunk_len;
  long long col1 = col0 + chunk_len;
  if (col1 > m) col1 = m;
  const V* vr = values + row * m;
  Acc* ar = acc + row * K;
  for (long long col = col0 + threadIdx.x; col < col1; col += NT) {
    const long long lab = static_cast<long long>(labels[col]);
    if (lab < 0 || lab >= K) continue;
    const V v = vr[col];
    if (is_nan(v)) continue;
    if (PASS == 0) {
      accumulate<F, V, true>(ar + lab, v, static_cast<unsigned long long>(col));
    } else {
      const unsigned long long key = select_key(v, F == kArgMin || F == kMin);
      if (key == ar[lab].a) atomicMin(&ar[lab].b, static_cast<unsigned long long>(col));
    }
  }
}

// ---- fold partials over chunks and write the output --------------------------------

template <int F, typename V, typename O>
__global__ void finalize(const Acc* __restrict__ partials, const V* __restrict__ values,
                         O* __restrict__ out, long long rows, long long m, long long K,
                         long long chunks, long long ddof) {
  const long long total = rows * K;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long row = t / K, k = t - row * K;
    Acc r = acc_init<F, V>();
    for (long long c = 0; c < chunks; ++c) r = fold<F, V>(r, partials[(row * chunks + c) * K + k]);
    O res;
    if (F == kSum) {
      res = IsFloat<V>::value ? static_cast<O>(as_d(r.a)) : static_cast<O>(static_cast<long long>(r.a));
    } else if (F == kSumSq) {
      res = IsFloat<V>::value ? static_cast<O>(as_d(r.b)) : static_cast<O>(static_cast<long long>(r.b));
    } else if (F == kCount) {
      res = static_cast<O>(r.c);
    } else if (F == kMean) {
      // out[label] /= count   (numbagg/grouped.py:22-27)
      res = r.c == 0 ? nan_of<O>() : static_cast<O>(as_d(r.a) / static_cast<double>(r.c));
    } else if (F == kVar || F == kStd) {
      // (sums_of_squares - sums**2 / count) / (count - ddof)   numbagg/grouped.py:170-176
      const long long cnt = static_cast<long long>(r.c);
      const long long denom = cnt - ddof;
      if (denom <= 0) {
        res = nan_of<O>();
      } else {
        const double s = as_d(r.a);
        double v = (as_d(r.b) - (s * s) / static_cast<double>(cnt)) / static_cast<double>(denom);
        if (F == kStd) v = sqrt(v);
        res = static_cast<O>(v);
      }
    } else if (F == kArgMax || F == kArgMin) {
      res = r.b == kNoIdx ? nan_of<O>() : static_cast<O>(r.b);
    } else if (F == kMax || F == kMin) {
      res = r.b == kNoIdx ? nan_of<O>()
                          : static_cast<O>(static_cast<double>(values[row * m + static_cast<long long>(r.b)]));
    } else if (F == kFirst) {
      if (r.a == kNoIdx)
        res = IsFloat<O>::value ? nan_of<O>() : O(0);
      else
        res = static_cast<O>(values[row * m + static_cast<long long>(r.a)]);
    } else if (F == kLast) {
      res = r.a == 0 ? nan_of<O>() : static_cast<O>(values[row * m + static_cast<long long>(r.a) - 1]);
    } else if (F == kProd) {
      res = IsFloat<V>::value ? static_cast<O>(as_d(r.a)) : static_cast<O>(static_cast<long long>(r.a));
    } else {  // kAny, kAll
      res = static_cast<O>(r.a & 1ull);
    }
    out[t] = res;
  }
}

}  // namespace grouped
}  // namespace nbg

using namespace nbg;
using namespace nbg::grouped;

namespace {

constexpr size_t kSmemBudget = 96 * 1024;

int replicas_for(long long K, int f) {
  // lane-private bins need no atomics; selection needs one replica for the tie sweep
  if (is_select(f)) return 1;
  if (K * static_cast<long long>(sizeof(Acc)) * NT <= static_cast<long long>(kSmemBudget)) return NT;
  if (K * static_cast<long long>(sizeof(Acc)) * (NT / 32) <= static_cast<long long>(kSmemBudget)) return NT / 32;
  return 1;
}

bool use_smem(long long K) { return K * static_cast<long long>(sizeof(Acc)) <= static_cast<long long>(kSmemBudget); }

struct Plan {
  bool smem;
  int rep;
  long long chunks, chunk_len;
};

Plan make_plan(int f, long long rows, long long m, long long K) {
  Plan p;
  p.smem = use_smem(K);
  p.rep = p.smem ? replicas_for(K, f) : 1;
  const long long target_ctas = static_cast<long long>(num_sms()) * 4;
  long long chunks = (target_ctas + rows - 1) / (rows > 0 ? rows : 1);
  // a chunk should be long enough to amortise initialising and flushing its bins
  const long long min_len = p.smem ? (K * 4 > 4096 ? K * 4 : 4096) : 8192;
  const long long max_chunks = (m + min_len - 1) / min_len;
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks < 1) chunks = 1;
  if (chunks > 65535) chunks = 65535;
  p.chunk_len = (m + chunks - 1) / chunks;
  p.chunks = (m + p.chunk_len - 1) / p.chunk_len;
  if (p.chunks < 1) p.chunks = 1;
  return p;
}

size_t plan_bytes(const Plan& p, long long rows, long long K) {
  const long long slots = p.smem ? rows * p.chunks * K : rows * K;
  return static_cast<size_t>(slots) * sizeof(Acc) + 256;
}

template <int F, typename V, typename L, int REP>
cudaError_t run_smem(const V* values, const L* labels, long long rows, long long m, long long K,
                     const Plan& p, Acc* acc, cudaStream_t s) {
  const size_t smem = static_cast<size_t>(K) * REP * sizeof(Acc);
  auto kern = accum_smem<F, V, L, REP>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  dim3 grid(static_cast<unsigned>(p.chunks), static_cast<unsigned>(rows));
  kern<<<grid, NT, smem, s>>>(values, labels, m, K, p.chunk_len, acc);
  note_launches(1);
  return cudaGetLastError();
}

template <int F, typename V, typename L, typename O>
int launch_group(const V* values, const L* labels, O* out, long long rows, long long m, long long K,
                 long long ddof, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (rows < 0 || m < 0 || K < 0) return kInvalidArgument;
  if (rows == 0 || K == 0) return kOk;
  if (rows > 65535) return kUnsupported;
  if (!out || (m > 0 && (!values || !labels))) return kInvalidArgument;
  const Plan p = make_plan(F, rows, m, K);
  if (!ws || ws_bytes < plan_bytes(p, rows, K)) return kWorkspaceTooSmall;
  Acc* acc = static_cast<Acc*>(ws);
  cudaError_t e = cudaSuccess;
  long long fold_chunks = 1;
  if (m == 0) {
    init_global<F, V><<<64, 256, 0, s>>>(acc, rows * K);
    note_launches(1);
  } else if (p.smem) {
    fold_chunks = p.chunks;
    if (p.rep == NT) e = run_smem<F, V, L, NT>(values, labels, rows, m, K, p, acc, s);
    else if (p.rep == NT / 32) e = run_smem<F, V, L, NT / 32>(values, labels, rows, m, K, p, acc, s);
    else e = run_smem<F, V, L, 1>(values, labels, rows, m, K, p, acc, s);
  } else {
    const long long total = rows * K;
    long long blocks = (total + 255) / 256;
    if (blocks > num_sms() * 16) blocks = num_sms() * 16;
    init_global<F, V><<<static_cast<int>(blocks), 256, 0, s>>>(acc, total);
    dim3 grid(static_cast<unsigned>(p.chunks), static_cast<unsigned>(rows));
    accum_global<F, V, L, 0><<<grid, NT, 0, s>>>(values, labels, m, K, p.chunk_len, acc);
    note_launches(2);
    if (is_select(F)) {
      accum_global<F, V, L, 1><<<grid, NT, 0, s>>>(values, labels, m, K, p.chunk_len, acc);
      note_launches(1);
    }
  }
  if (e != cudaSuccess) return kLaunchError;
  const long long total = rows * K;
  long long blocks = (total + 255) / 256;
  if (blocks > num_sms() * 16) blocks = num_sms() * 16;
  finalize<F, V, O><<<static_cast<int>(blocks), 256, 0, s>>>(acc, values, out, rows, m, K, fold_chunks, ddof);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

}  // namespace

extern "C" {

size_t nbg_group_workspace_bytes(int func, long long rows, long long m, long long K) {
  if (func < 0 || func >= kNumFuncs) return 0;
  const size_t generic = plan_bytes(make_plan(func, rows, m, K), rows, K);
  const size_t fast = fast_bytes_query(func, rows, m, K);
  return generic > fast ? generic : fast;
}

// Exported symbol per (function, values dtype, labels dtype); output dtype follows
// numbagg: same as values except mean/var/std on integers, which return float64
// (supports_ints=False, numbagg/decorators.py:614-619).
#define NBG_GROUP_ONE(NAME, FC, V, VS, O, L, LS)                                               \
  int nbg_group_##NAME##_##VS##_##LS(const V* values, const L* labels, O* out, long long rows,  \
                                     long long m, long long num_labels, long long ddof, void* ws, \
                                     size_t ws_bytes, void* stream) {                          \
    return launch_group<FC, V, L, O>(values, labels, out, rows, m, num_labels, ddof, ws, ws_bytes, \
                                     static_cast<cudaStream_t>(stream));                       \
  }
#define NBG_GROUP_LABELS(NAME, FC, V, VS, O)    \
  NBG_GROUP_ONE(NAME, FC, V, VS, O, int, i32) \
  NBG_GROUP_ONE(NAME, FC, V, VS, O, long long, i64)

#define NBG_GROUP_ALLTYPES(NAME, FC)                 \
  NBG_GROUP_LABELS(NAME, FC, double, f64, double)    \
  NBG_GROUP_LABELS(NAME, FC, float, f32, float)      \
  NBG_GROUP_LABELS(NAME, FC, int, i32, int)          \
  NBG_GROUP_LABELS(NAME, FC, long long, i64, long long)
#define NBG_GROUP_FLOATONLY(NAME, FC)                \
  NBG_GROUP_LABELS(NAME, FC, double, f64, double)    \
  NBG_GROUP_LABELS(NAME, FC, float, f32, float)

#define NBG_GROUP_INTONLY(NAME, FC)         \
  NBG_GROUP_LABELS(NAME, FC, int, i32, int) \
  NBG_GROUP_LABELS(NAME, FC, long long, i64, long long)

// float moments and all selections live in grouped_fast.cuh (grouped_fast_*.cu)
NBG_GROUP_INTONLY(nansum, kSum)
NBG_GROUP_INTONLY(nancount, kCount)
NBG_GROUP_INTONLY(nansum_of_squares, kSumSq)
NBG_GROUP_ALLTYPES(nanprod, kProd)
NBG_GROUP_ALLTYPES(nanany, kAny)
NBG_GROUP_ALLTYPES(nanall, kAll)

}  // extern "C"
