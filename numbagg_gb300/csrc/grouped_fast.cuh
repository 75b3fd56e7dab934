// Labelled reductions, fast paths (numbagg/grouped.py:7-244).
//
// values (rows, m), labels (m,) shared by every row, out (rows, K).  Three strategies,
// chosen from K:
//
//  * tiny K (<= 16): every thread owns a private copy of the K bins in shared memory
//    (no atomics).  A warp works through tiles of 32 x 16 columns; within a tile every
//    value is turned into a 64-bit fixed-point integer at the scale of the tile's
//    largest exponent (53 significant bits, exact sums of up to 1024 terms), then the
//    lanes' bins are summed with warp shuffles and added, as float64, to a per-warp
//    accumulator held by lane k for bin k.
//  * medium K (bins fit in shared memory): the bins of a CTA are shared and updated
//    with 64-bit shared-memory atomics on fixed-point integers at a CTA scale that
//    grows with the largest exponent seen; at the end of the chunk (or every 2^15
//    columns when the chunk's label histogram shows a label that frequent) the bins
//    are flushed, as float64, into the CTA's own partial in global memory.
//  * large K (e.g. 10^6): float64 reductions straight into per-row accumulators in
//    global memory.  CTAs are ordered row by row, so only the rows in flight (a few
//    tens of MB of accumulators) are live and they stay in L2.
//
// Counts come from the labels where possible: the number of columns with label k is
// the same for every row, so the valid count is that label histogram (computed once
// per call) minus the NaN count, and only NaN elements pay for a counting atomic.
//
// Selection (argmax / argmin / max / min) keeps the reference's strict comparison on
// float64 values, the first index winning ties (numbagg/grouped.py:62, :86, :221,
// :239): an element is the pair (order key of its float64 value with -0.0 == +0.0,
// column index) and a bin keeps the best pair -- larger key, then smaller index.
// Private bins are updated in column order; shared and global bins with a 128-bit
// compare-and-swap issued only when the element improves on the current pair.
// first / last are a minimum / maximum of the column index.  All of these are exact.
#pragma once

#include "grouped_common.cuh"
#include "fixed128.cuh"

namespace nbg {
namespace grouped {

constexpr int FT = 256;
constexpr int kTinyK = 16;
constexpr int kTileCols = 32 * 16;   // tiny path: chunks are multiples of FT / 32 x kTileCols columns
constexpr int kCtaCols = FT * 8;     // columns of one CTA tile (medium / large paths)

struct MomPart {  // one bin of one chunk: float64 sums, valid count, infinities seen
  double s1, s2;
  long long cnt;
  int pinf, ninf;
};
struct SelPart {
  unsigned long long key, idx;
};

template <int F>
struct Need {
  static constexpr bool s1 = F == kSum || F == kMean || F == kVar || F == kStd;
  static constexpr bool s2 = F == kVar || F == kStd || F == kSumSq;
  static constexpr bool cnt = F == kCount || F == kMean || F == kVar || F == kStd;
  static constexpr bool varlike = F == kVar || F == kStd;
};

NBG_DEVICE int bexp(double x) {
  const int e = static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(x)) >> 52) & 0x7ff);
  return e ? e : 1;
}
NBG_DEVICE unsigned long long mant(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long m = b & 0x000fffffffffffffull;
  return ((b >> 52) & 0x7ff) ? (m | 0x0010000000000000ull) : m;
}
NBG_DEVICE bool is_inf_d(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull) == 0x7ff0000000000000ull;
}
// |x| >= 2^512: the reference's x**2 overflows
NBG_DEVICE bool sq_overflows(double x) { return bexp(x) >= 1023 + 512; }

// mantissa aligned to scale exponent E >= e, then shifted right by `drop` more bits
NBG_DEVICE unsigned long long aligned(double x, int E, int drop) {
  const int sh = E - bexp(x) + drop;
  return sh >= 64 ? 0ull : (mant(x) >> sh);
}
// (a * a) >> s for a < 2^53
NBG_DEVICE unsigned long long square_shift(unsigned long long a, int s) {
  const unsigned long long lo = a * a, hi = __umul64hi(a, a);
  if (s >= 64) return hi >> (s - 64);
  return (hi << (64 - s)) | (lo >> s);
}
NBG_DEVICE long long signed_of(double x, unsigned long long mag) {
  return __double_as_longlong(x) < 0 ? -static_cast<long long>(mag) : static_cast<long long>(mag);
}
// v * 2^L as a double
NBG_DEVICE double fix_to_double(long long v, int L) { return scalbn(__ll2double_rn(v), L); }

// Fixed-point format of the medium path:
//   value = aligned(x, E, 5) * 2^(E - 1070)                (48 bits)
//   square = (a*a) >> 58  * 2^(2(E - 1075) + 58)            a = aligned(x, E, 0)
// with 15 bits of headroom.

NBG_DEVICE bool better(unsigned long long k1, unsigned long long i1, unsigned long long k2, unsigned long long i2) {
  return k1 > k2 || (k1 == k2 && i1 < i2);
}

// 128-bit compare-and-swap of a (key, idx) pair, global or shared (generic address)
NBG_DEVICE void cas128(unsigned long long* addr, unsigned long long& ck, unsigned long long& ci,
                       unsigned long long nk, unsigned long long ni, bool shared) {
  unsigned long long ok, oi;
  if (shared) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(addr));
    asm volatile(
        "{ .reg .b128 c, n, o; mov.b128 c, {%2, %3}; mov.b128 n, {%4, %5};"
        " atom.shared.cas.b128 o, [%6], c, n; mov.b128 {%0, %1}, o; }"
        : "=l"(ok), "=l"(oi)
        : "l"(ck), "l"(ci), "l"(nk), "l"(ni), "r"(a)
        : "memory");
  } else {
    asm volatile(
        "{ .reg .b128 c, n, o; mov.b128 c, {%2, %3}; mov.b128 n, {%4, %5};"
        " atom.global.cas.b128 o, [%6], c, n; mov.b128 {%0, %1}, o; }"
        : "=l"(ok), "=l"(oi)
        : "l"(ck), "l"(ci), "l"(nk), "l"(ni), "l"(addr)
        : "memory");
  }
  ck = ok;
  ci = oi;
}

// keep the better of the pair at addr and (key, idx)
NBG_DEVICE void sel_update(unsigned long long* addr, unsigned long long key, unsigned long long idx, bool shared) {
  unsigned long long ck = shared ? *reinterpret_cast<volatile unsigned long long*>(addr) : __ldcg(addr);
  unsigned long long ci = shared ? *reinterpret_cast<volatile unsigned long long*>(addr + 1) : __ldcg(addr + 1);
  for (int it = 0; it < 1 << 16 && better(key, idx, ck, ci); ++it) {
    const unsigned long long ek = ck, ei = ci;
    cas128(addr, ck, ci, key, idx, shared);
    if (ck == ek && ci == ei) return;  // swapped in
  }
}

// ---------------------------------------------------------------------------------
// values taken apart with integer instructions only.  This GPU's FP64 pipe accepts a
// warp instruction every 16 cycles whatever the number of active lanes, so nothing
// that runs per element (or per bin and tile) may use it.
// ---------------------------------------------------------------------------------
struct Dec {
  unsigned long long m;  // integer mantissa: value = m * 2^(e - 1075)
  int e;                 // biased float64 exponent (1 for zeros and subnormals)
  bool neg;              // sign bit
  bool special;          // infinity or NaN
};
NBG_DEVICE Dec decomp(unsigned long long b) {  // float64 bits
  const int eb = static_cast<int>((b >> 52) & 0x7ff);
  Dec d;
  d.m = (b & 0x000fffffffffffffull) | (eb ? 0x0010000000000000ull : 0ull);
  d.e = eb ? eb : 1;
  d.neg = (b >> 63) != 0;
  d.special = eb == 0x7ff;
  return d;
}
// float32 bits, restated exactly in the float64 format
NBG_DEVICE Dec decomp(unsigned b) {
  const int eb = static_cast<int>((b >> 23) & 0xff);
  Dec d;
  d.m = static_cast<unsigned long long>((b & 0x7fffffu) | (eb ? 0x800000u : 0u)) << 29;
  d.e = eb ? eb + 896 : 897;
  d.neg = (b >> 31) != 0;
  d.special = eb == 0xff;
  return d;
}
// integer values reach the moment kernels only through the generic path; these keep
// the templates well-formed
NBG_DEVICE Dec decomp(int x) {
  return decomp(static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(x))));
}
NBG_DEVICE Dec decomp(long long x) {
  return decomp(static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(x))));
}

// infinity and sign tests on the bits (integers: never infinite)
NBG_DEVICE bool inf_bits(unsigned long long b) { return (b << 1) == 0xffe0000000000000ull; }
NBG_DEVICE bool inf_bits(unsigned b) { return (b << 1) == 0xff000000u; }
NBG_DEVICE bool inf_bits(int) { return false; }
NBG_DEVICE bool inf_bits(long long) { return false; }
NBG_DEVICE bool sign_bit(unsigned long long b) { return (b >> 63) != 0; }
NBG_DEVICE bool sign_bit(unsigned b) { return (b >> 31) != 0; }
NBG_DEVICE bool sign_bit(int v) { return v < 0; }
NBG_DEVICE bool sign_bit(long long v) { return v < 0; }

// the value of a bit pattern as float64
NBG_DEVICE double bits_to_f64(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }
NBG_DEVICE double bits_to_f64(unsigned b) { return static_cast<double>(__int_as_float(static_cast<int>(b))); }
NBG_DEVICE double bits_to_f64(int v) { return static_cast<double>(v); }
NBG_DEVICE double bits_to_f64(long long v) { return static_cast<double>(v); }

// Order key of a value (given as its bits, see BitsOf) for the selection functions:
// a < b (compared as float64, the reference's comparison) <=> key(a) < key(b), -0.0
// and +0.0 equal, and no key is 0 (0 marks an empty bin).
NBG_DEVICE unsigned long long value_key(unsigned long long b) {  // float64 bits
  if ((b << 1) == 0) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
NBG_DEVICE unsigned long long value_key(unsigned b) {  // float32 bits
  if ((b << 1) == 0) b = 0;
  return (b >> 31) ? static_cast<unsigned long long>(~b) : static_cast<unsigned long long>(b | 0x80000000u);
}
NBG_DEVICE unsigned long long value_key(int v) {  // exact as float64; offset binary, plus one
  return static_cast<unsigned long long>(static_cast<unsigned>(v) ^ 0x80000000u) + 1ull;
}
NBG_DEVICE unsigned long long value_key(long long v) { return order_key_ieee(static_cast<double>(v)); }
template <int F, typename V>
NBG_DEVICE unsigned long long sel_key_of(V v) {
  const unsigned long long k = value_key(v);
  return (F == kArgMin || F == kMin) ? ~k : k;
}

// ---------------------------------------------------------------------------------
// tiny K: lane-private bins
// ---------------------------------------------------------------------------------
// A warp keeps a scale exponent E, the largest biased exponent among the finite values
// it has met (it only grows), and every lane keeps its own K bins in shared memory:
//   value  x   -> +-(m >> (E - e + d1))          LSB 2^(E + d1 - 1075)
// d1 comes from the host: with n the number of elements one lane can meet in its chunk
// (< 2^lg), d1 = max(0, lg - 10), so a lane's sums stay below 2^63.  When E grows, each
// lane shifts its own bins down.  Bits below the LSB are truncated: at most
// 2^-(52 - d1) of the largest value the warp met, per term.  At the end of the chunk the
// lanes' bins are summed exactly (128-bit) per warp and rounded once to float64.
// Squares go to float64 lane bins (one fused multiply-add each on the FP64 pipe, which
// the integer work leaves idle; a 64 x 64-bit product and a 128-bit shift per element
// made the variance the slowest of these kernels), reduced in a fixed order per warp:
// each rounding chain is one lane's elements of one chunk, far shorter than the
// reference's sequential sum over the row.
// CTAs per SM the tiny moment kernels are compiled for: sums and means are bound by
// integer issue and gain from a third CTA; the others measured faster with two
template <int F>
struct TinyOcc {
  static constexpr int value = (F == kSum || F == kMean) ? 3 : 2;
};

// SPLIT (sums and means): three of every four elements of a lane's tile go to float64
// lane bins instead of the fixed-point ones (one float64 add on the FP64 pipe, no
// decomposition or shift); the counts of a split mean are 16-bit (the host keeps a
// lane's elements per chunk below 2^16).  The variances do not split: their squares
// already keep the FP64 pipe busy (measured at K = 16: 3.72 ms unsplit, 3.77 ms with
// one element in four split, 3.88 ms with one in two).
// The float64 bins add in a fixed order per lane and are reduced in a fixed order, so
// results stay reproducible, within about 2^-53 times a lane's element count of the
// sum of magnitudes.
template <int F, bool SPLIT>
struct TinyCount {
  typedef int type;
};
template <int F>
struct TinyCount<F, true> {
  typedef unsigned short type;
};

template <int F, typename V, typename L, bool SPLIT>
__global__ void __launch_bounds__(FT, TinyOcc<F>::value) tiny_mom_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                         long long rows, long long m, int K, long long chunk_len,
                                                         long long chunks, int d1,
                                                         MomPart* __restrict__ parts) {
  typedef typename BitsOf<V>::type B;
  typedef typename TinyCount<F, SPLIT>::type C;
  constexpr bool S1 = Need<F>::s1, S2 = Need<F>::s2, CNT = Need<F>::cnt, VL = Need<F>::varlike;
  constexpr bool MOM = S1 || S2;
  static_assert(!SPLIT || (S1 && !S2), "the split is for sums and means");
  constexpr int FMASK = 3;  // elements j of a lane's tile with (j & FMASK) != 0 take the float64 bins
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long* b1 = reinterpret_cast<long long*>(smem_raw);  // [K][FT]
  double* f2 = reinterpret_cast<double*>(smem_raw + (S1 ? K * FT * 8 : 0));  // squares, float64
  double* f1 = reinterpret_cast<double*>(smem_raw + (S1 ? K * FT * 8 : 0) + (S2 ? K * FT * 8 : 0));
  C* bc = reinterpret_cast<C*>(smem_raw + (S1 ? K * FT * 8 : 0) + (S2 ? K * FT * 8 : 0) + (SPLIT ? K * FT * 8 : 0));
  __shared__ double wsum1[FT / 32][kTinyK], wsum2[FT / 32][kTinyK];
  __shared__ int wcnt[FT / 32][kTinyK];
  __shared__ int infs[2][kTinyK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // chunk-major order: the CTAs in flight share the chunks of labels they read
  const long long chunk = blockIdx.x / rows, row = blockIdx.x - chunk * rows;
  const long long c0 = chunk * chunk_len;
  const long long c1 = min(m, c0 + chunk_len);
  for (int k = 0; k < K; ++k) {
    if (S1) b1[k * FT + tid] = 0;
    if (S2) f2[k * FT + tid] = 0.0;
    if (SPLIT) f1[k * FT + tid] = 0.0;
    if (CNT) bc[k * FT + tid] = 0;
  }
  if (tid < 2 * kTinyK) infs[tid / kTinyK][tid % kTinyK] = 0;
  __syncthreads();
  const B* vr = as_bits(values) + row * m;
  int E = 0;  // the warp's scale (uniform across the warp)
  // Warp tiles of 32 x J columns, the next tile's loads issued before the current tile
  // is reduced, so each warp always has a tile in flight.
  constexpr int J = 8;
  constexpr long long TC = 32 * J, STEP = static_cast<long long>(FT / 32) * TC;
  auto load = [&](long long base, B (&v)[J], int (&lab)[J]) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const long long col = base + j * 32 + lane;
      const bool in = col < c1;
      v[j] = in ? __ldcs(vr + col) : B(0);
      const long long l = in ? static_cast<long long>(__ldg(labels + col)) : -1;
      lab[j] = (l >= 0 && l < K) ? static_cast<int>(l) : -1;
    }
  };
  B v[J];
  int lab[J];
  load(c0 + warp * TC, v, lab);
  for (long long base = c0 + warp * TC; base < c1; base += STEP) {
    B vn[J];
    int ln[J];
    load(base + STEP, vn, ln);
    int emax = 0;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      if (nan_bits(v[j])) lab[j] = -1;
      if (S1 && !(SPLIT && (j & FMASK) != 0)) {
        const Dec d = decomp(v[j]);
        if (lab[j] >= 0 && !d.special && !(VL && d.e >= 1023 + 512)) emax = max(emax, d.e);
      }
    }
    if (S1) {
      const int Et = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(emax)));
      if (Et > E) {  // uniform: the warp's scale grows
        if (E > 0) {
          const int dd = Et - E;
          for (int k = 0; k < K; ++k) {
            const int slot = k * FT + tid;
            b1[slot] = dd >= 63 ? (b1[slot] < 0 ? -1ll : 0ll) : (b1[slot] >> dd);
          }
        }
        E = Et;
      }
    }
#pragma unroll
    for (int j = 0; j < J; ++j) {
      if (lab[j] < 0) continue;
      const int slot = lab[j] * FT + tid;
      if (CNT) bc[slot] += 1;
      if (!MOM) continue;
      if (SPLIT && (j & FMASK) != 0) {
        if (inf_bits(v[j])) {
          atomicAdd(&infs[sign_bit(v[j]) ? 1 : 0][lab[j]], 1);
          continue;
        }
        f1[slot] += bits_to_f64(v[j]);
        continue;
      }
      const Dec d = decomp(v[j]);
      if (d.special || (VL && d.e >= 1023 + 512)) {  // infinity, or a square that overflows
        atomicAdd(&infs[d.neg ? 1 : 0][lab[j]], 1);
        continue;
      }
      if (S1) {
        const int sh = E - d.e + d1;
        const unsigned long long a = sh >= 64 ? 0ull : (d.m >> sh);
        b1[slot] += d.neg ? -static_cast<long long>(a) : static_cast<long long>(a);
      }
      if (S2) {
        const double x = bits_to_f64(v[j]);
        f2[slot] = fma(x, x, f2[slot]);
      }
    }
#pragma unroll
    for (int j = 0; j < J; ++j) {
      v[j] = vn[j];
      lab[j] = ln[j];
    }
  }
  // lanes' bins -> exact warp sums -> float64 at the warp's scale
  for (int k = 0; k < K; ++k) {
    const int slot = k * FT + tid;
    if (S1) {
      const long long x = b1[slot];
      unsigned long long lo = static_cast<unsigned long long>(x);
      long long hi = x < 0 ? -1ll : 0ll;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, o);
        const long long ohi = __shfl_xor_sync(0xffffffffu, hi, o);
        const unsigned long long nlo = lo + olo;
        hi = hi + ohi + (nlo < lo ? 1 : 0);
        lo = nlo;
      }
      double fs = 0.0;
      if (SPLIT) {
        fs = f1[slot];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fs += __shfl_xor_sync(0xffffffffu, fs, o);
      }
      if (lane == 0)
        wsum1[warp][k] = fx::to_double((static_cast<fx::i128>(hi) << 64) + static_cast<fx::i128>(lo), E + d1 - 1075) + fs;
    }
    if (S2) {
      double q = f2[slot];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
      if (lane == 0) wsum2[warp][k] = q;
    }
    if (CNT) {
      const int c = static_cast<int>(__reduce_add_sync(0xffffffffu, static_cast<unsigned>(bc[slot])));
      if (lane == 0) wcnt[warp][k] = c;
    }
  }
  __syncthreads();
  if (tid < K) {
    MomPart p;
    p.s1 = 0.0;
    p.s2 = 0.0;
    p.cnt = 0;
    for (int w = 0; w < FT / 32; ++w) {  // fixed order: deterministic
      if (S1) p.s1 += wsum1[w][tid];
      if (S2) p.s2 += wsum2[w][tid];
      if (CNT) p.cnt += wcnt[w][tid];
    }
    p.pinf = infs[0][tid];
    p.ninf = infs[1][tid];
    parts[(row * chunks + chunk) * K + tid] = p;
  }
}

template <int F, typename V, typename L>
__global__ void __launch_bounds__(FT, 2) tiny_sel_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                         long long rows, long long m, int K, long long chunk_len,
                                                         long long chunks, SelPart* __restrict__ parts) {
  typedef typename BitsOf<V>::type B;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* bk = reinterpret_cast<unsigned long long*>(smem_raw);  // [K][FT]
  unsigned long long* bi = bk + K * FT;                                     // [K][FT]
  __shared__ unsigned long long wk[FT / 32][kTinyK], wi[FT / 32][kTinyK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long chunk = blockIdx.x / rows, row = blockIdx.x - chunk * rows;
  const long long c0 = chunk * chunk_len;
  const long long c1 = min(m, c0 + chunk_len);
  constexpr bool is_idx = F == kFirst || F == kLast;
  for (int k = 0; k < K; ++k) {
    bk[k * FT + tid] = (F == kFirst) ? ~0ull : 0ull;
    bi[k * FT + tid] = ~0ull;
  }
  const B* vr = as_bits(values) + row * m;
  // warp tiles of 32 x J columns, the next tile's loads in flight while one is reduced
  constexpr int J = 8;
  constexpr long long TC = 32 * J, STEP = static_cast<long long>(FT / 32) * TC;
  auto load = [&](long long base, B (&v)[J], int (&lab)[J]) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const long long col = base + j * 32 + lane;
      const bool in = col < c1;
      v[j] = in ? __ldcs(vr + col) : B(0);
      const long long l = in ? static_cast<long long>(__ldg(labels + col)) : -1;
      lab[j] = (l >= 0 && l < K) ? static_cast<int>(l) : -1;
    }
  };
  B v[J];
  int lab[J];
  load(c0 + warp * TC, v, lab);
  for (long long base = c0 + warp * TC; base < c1; base += STEP) {
    B vn[J];
    int ln[J];
    load(base + STEP, vn, ln);
    // a lane meets its columns in increasing order
#pragma unroll
    for (int j = 0; j < J; ++j) {
      if (lab[j] < 0 || nan_bits(v[j])) continue;
      const int slot = lab[j] * FT + tid;
      const unsigned long long c = static_cast<unsigned long long>(base + j * 32 + lane);
      if (F == kFirst) {
        if (bk[slot] == ~0ull) bk[slot] = c;
      } else if (F == kLast) {
        bk[slot] = c + 1;
      } else {
        const unsigned long long key = sel_key_of<F>(v[j]);
        if (key > bk[slot]) {  // strict: the earlier column keeps a tie
          bk[slot] = key;
          bi[slot] = c;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < J; ++j) {
      v[j] = vn[j];
      lab[j] = ln[j];
    }
  }
  // reduce lanes, then warps (fixed order)
  for (int k = 0; k < K; ++k) {
    unsigned long long key = bk[k * FT + tid], idx = bi[k * FT + tid];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      const unsigned long long oi = __shfl_xor_sync(0xffffffffu, idx, o);
      if (is_idx) {
        key = (F == kFirst) ? min(key, ok) : max(key, ok);
      } else if (better(ok, oi, key, idx)) {
        key = ok;
        idx = oi;
      }
    }
    if (lane == 0) {
      wk[warp][k] = key;
      wi[warp][k] = idx;
    }
  }
  __syncthreads();
  if (tid < K) {
    unsigned long long key = wk[0][tid], idx = wi[0][tid];
    for (int w = 1; w < FT / 32; ++w) {
      if (is_idx) {
        key = (F == kFirst) ? min(key, wk[w][tid]) : max(key, wk[w][tid]);
      } else if (better(wk[w][tid], wi[w][tid], key, idx)) {
        key = wk[w][tid];
        idx = wi[w][tid];
      }
    }
    parts[(row * chunks + chunk) * K + tid] = SelPart{key, idx};
  }
}

// ---------------------------------------------------------------------------------
// label histograms (shared by all rows)
// ---------------------------------------------------------------------------------
// per chunk (medium path): hist[chunk][k]
template <typename L>
__global__ void __launch_bounds__(FT) chunk_hist_kernel(const L* __restrict__ labels, long long m, int K,
                                                        long long chunk_len, unsigned* __restrict__ hist) {
  extern __shared__ unsigned hsm[];
  const long long chunk = blockIdx.x;
  for (int k = threadIdx.x; k < K; k += FT) hsm[k] = 0;
  __syncthreads();
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  for (long long c = c0 + threadIdx.x; c < c1; c += FT) {
    const long long l = static_cast<long long>(labels[c]);
    if (l >= 0 && l < K) atomicAdd(&hsm[l], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += FT) hist[chunk * K + k] = hsm[k];
}
// whole row (large path): hist[k], and the table rcp[c] = RN(1 / c) for c <= kRcpN.
// Up to kHistSmem labels each CTA counts its share in shared memory first (many
// columns per label: global atomics on few addresses would serialise).
constexpr long long kRcpN = 1 << 16;
constexpr int kHistSmem = 16384;
template <typename L, bool SMEM>
__global__ void __launch_bounds__(FT) row_hist_kernel(const L* __restrict__ labels, long long m, long long K,
                                                      unsigned* __restrict__ hist, double* __restrict__ rcp) {
  extern __shared__ unsigned hsm[];
  const long long stride = static_cast<long long>(gridDim.x) * FT;
  const long long t0 = static_cast<long long>(blockIdx.x) * FT + threadIdx.x;
  for (long long c = t0; c <= kRcpN; c += stride) rcp[c] = c ? 1.0 / static_cast<double>(c) : 0.0;
  if (SMEM) {
    for (int k = threadIdx.x; k < K; k += FT) hsm[k] = 0;
    __syncthreads();
  }
  for (long long c = t0; c < m; c += stride) {
    const long long l = static_cast<long long>(labels[c]);
    if (l >= 0 && l < K) atomicAdd(SMEM ? &hsm[l] : &hist[l], 1u);
  }
  if (SMEM) {
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += FT)
      if (hsm[k]) atomicAdd(&hist[k], hsm[k]);
  }
}

// s / c for a count c >= 1, correctly rounded: Markstein's FMA correction of s * RN(1/c)
// with the reciprocal from the table (three FP64 operations instead of a division);
// beyond the table, and for infinite or NaN s, a division
NBG_DEVICE double div_by_count(double s, long long c, const double* __restrict__ rcp) {
  const bool finite = (static_cast<unsigned long long>(__double_as_longlong(s)) & 0x7ff0000000000000ull) !=
                      0x7ff0000000000000ull;
  if (c > kRcpN || !finite) return s / static_cast<double>(c);
  const double r = __ldg(rcp + c);
  const double q0 = s * r;
  const double e = fma(-q0, f64_of_count(c), s);
  return fma(e, r, q0);
}

// ---------------------------------------------------------------------------------
// medium K: CTA-shared bins
// ---------------------------------------------------------------------------------
template <int F>
NBG_HOST_DEVICE size_t mid_mom_bytes_per_bin() {
  return (Need<F>::s1 ? 8 : 0) + (Need<F>::s2 ? 8 : 0) + (Need<F>::cnt ? 4 : 0) + ((Need<F>::s1 || Need<F>::s2) ? 4 : 0);
}

// A bin may hold at most 2^15 terms in the 48-bit format before it must be flushed.
// The chunk's label histogram (known before the launch) bounds every bin's count, so
// the CTA flushes only when some label is that frequent in the chunk.
constexpr long long kMaxTermsPerFlush = 1ll << 15;

template <int F, typename V, typename L>
__global__ void __launch_bounds__(FT) mid_mom_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                     long long rows, long long m, int K, long long chunk_len,
                                                     long long chunks, const unsigned* __restrict__ hist,
                                                     MomPart* __restrict__ parts) {
  typedef typename BitsOf<V>::type B;
  constexpr bool S1 = Need<F>::s1, S2 = Need<F>::s2, CNT = Need<F>::cnt, VL = Need<F>::varlike;
  constexpr bool MOM = S1 || S2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* cur = smem_raw;
  unsigned long long* b1 = reinterpret_cast<unsigned long long*>(cur);
  if (S1) cur += static_cast<size_t>(K) * 8;
  unsigned long long* b2 = reinterpret_cast<unsigned long long*>(cur);
  if (S2) cur += static_cast<size_t>(K) * 8;
  unsigned* nanc = reinterpret_cast<unsigned*>(cur);
  if (CNT) cur += static_cast<size_t>(K) * 4;
  unsigned* infc = reinterpret_cast<unsigned*>(cur);  // +1 per +inf, +65536 per -inf
  __shared__ unsigned red_w[FT / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // chunk-major order: the CTAs in flight share the chunks of labels they read
  const long long chunk = blockIdx.x / rows, row = blockIdx.x - chunk * rows;
  const long long c0 = chunk * chunk_len;
  const long long c1 = min(m, c0 + chunk_len);
  MomPart* pr = parts + (row * chunks + chunk) * K;
  unsigned hmax = 0;
  for (int k = tid; k < K; k += FT) {
    if (S1) b1[k] = 0;
    if (S2) b2[k] = 0;
    if (CNT) nanc[k] = 0;
    if (MOM) infc[k] = 0;
    pr[k] = MomPart{0.0, 0.0, 0, 0, 0};
    hmax = max(hmax, hist[chunk * K + k]);
  }
  hmax = __reduce_max_sync(0xffffffffu, hmax);
  if (lane == 0) red_w[warp] = hmax;
  __syncthreads();
  hmax = 0;
#pragma unroll
  for (int w = 0; w < FT / 32; ++w) hmax = max(hmax, red_w[w]);
  __syncthreads();
  // also bounds the infinities per counter (2^15 of each fit in the packed word)
  const long long flush_len = (hmax <= kMaxTermsPerFlush) ? chunk_len : kMaxTermsPerFlush;
  const B* vr = as_bits(values) + row * m;
  int E = 0;  // the CTA's scale, the same in every thread
  for (long long sub = c0; sub < c1; sub += flush_len) {
    const long long send = min(c1, sub + flush_len);
    for (long long base = sub; base < send; base += kCtaCols) {
      B v[8];
      int lab[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const long long col = base + j * FT + tid;
        const bool in = col < send;
        v[j] = in ? __ldcs(vr + col) : B(0);
        const long long l = in ? static_cast<long long>(__ldg(labels + col)) : -1;
        lab[j] = (l >= 0 && l < K) ? static_cast<int>(l) : -1;
      }
      int emax = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (lab[j] >= 0 && nan_bits(v[j])) {
          if (CNT) atomicAdd(&nanc[lab[j]], 1u);
          lab[j] = -1;
        }
        if (MOM) {
          const Dec d = decomp(v[j]);
          if (lab[j] >= 0 && !d.special && !(VL && d.e >= 1023 + 512)) emax = max(emax, d.e);
        }
      }
      if (MOM) {
        if (__syncthreads_or(emax > E)) {  // the CTA's scale grows: shift what the bins hold
          const int wm = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(emax)));
          if (lane == 0) red_w[warp] = static_cast<unsigned>(wm);
          __syncthreads();
          int En = E;
#pragma unroll
          for (int w = 0; w < FT / 32; ++w) En = max(En, static_cast<int>(red_w[w]));
          if (E > 0) {
            const int dd = En - E;
            for (int k = tid; k < K; k += FT) {
              if (S1) {
                const long long x = static_cast<long long>(b1[k]);
                b1[k] = static_cast<unsigned long long>(dd >= 63 ? (x < 0 ? -1ll : 0ll) : (x >> dd));
              }
              if (S2) b2[k] = 2 * dd >= 64 ? 0ull : (b2[k] >> (2 * dd));
            }
          }
          E = En;
          __syncthreads();
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (lab[j] < 0) continue;
          const Dec d = decomp(v[j]);
          if (d.special || (VL && d.e >= 1023 + 512)) {  // infinity, or a square that overflows
            atomicAdd(&infc[lab[j]], d.neg ? 65536u : 1u);
            continue;
          }
          if (S1) {
            const int sh = E - d.e + 5;
            const unsigned long long a = sh >= 64 ? 0ull : (d.m >> sh);
            atomicAdd(&b1[lab[j]], d.neg ? (~a + 1ull) : a);
          }
          if (S2) {
            const int sh = 2 * (E - d.e) + 58;
            unsigned long long q = 0ull;
            if (sh < 106) {
              const unsigned long long lo = d.m * d.m, hi = __umul64hi(d.m, d.m);
              q = sh >= 64 ? (hi >> (sh - 64)) : ((hi << (64 - sh)) | (lo >> sh));
            }
            atomicAdd(&b2[lab[j]], q);
          }
        }
      }
    }
    if (MOM) {
      __syncthreads();
      // flush into the CTA's own partial (float64)
      for (int k = tid; k < K; k += FT) {
        MomPart p = pr[k];
        if (S1 && b1[k]) p.s1 += fx::to_double(static_cast<fx::i128>(static_cast<long long>(b1[k])), E + 5 - 1075);
        if (S2 && b2[k]) p.s2 += fx::to_double(static_cast<fx::i128>(b2[k]), 2 * E + 58 - 2150);
        p.pinf += static_cast<int>(infc[k] & 0xffffu);
        p.ninf += static_cast<int>(infc[k] >> 16);
        pr[k] = p;
        if (S1) b1[k] = 0;
        if (S2) b2[k] = 0;
        infc[k] = 0;
      }
      E = 0;
      __syncthreads();
    }
  }
  __syncthreads();
  if (CNT) {
    for (int k = tid; k < K; k += FT) pr[k].cnt = static_cast<long long>(hist[chunk * K + k]) - nanc[k];
  }
}

template <int F, typename V, typename L>
__global__ void __launch_bounds__(FT, 3) mid_sel_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                     long long rows, long long m, int K, long long chunk_len,
                                                     long long chunks, SelPart* __restrict__ parts) {
  typedef typename BitsOf<V>::type B;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* bins = reinterpret_cast<unsigned long long*>(smem_raw);  // [K][2]
  const int tid = threadIdx.x;
  const long long chunk = blockIdx.x / rows, row = blockIdx.x - chunk * rows;
  const long long c0 = chunk * chunk_len;
  const long long c1 = min(m, c0 + chunk_len);
  for (int k = tid; k < K; k += FT) {
    bins[2 * k] = (F == kFirst) ? ~0ull : 0ull;
    bins[2 * k + 1] = ~0ull;
  }
  __syncthreads();
  const B* vr = as_bits(values) + row * m;
  // the next tile's loads are issued before the current tile updates the bins, so a
  // tile is always in flight
  auto load = [&](long long base, B (&v)[8], int (&lab)[8]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const long long col = base + j * FT + tid;
      const bool in = col < c1;
      v[j] = in ? __ldcs(vr + col) : B(0);
      const long long l = in ? static_cast<long long>(__ldg(labels + col)) : -1;
      lab[j] = (l >= 0 && l < K) ? static_cast<int>(l) : -1;
    }
  };
  B v[8];
  int lab[8];
  load(c0, v, lab);
  for (long long base = c0; base < c1; base += kCtaCols) {
    B vn[8];
    int ln[8];
    load(base + kCtaCols, vn, ln);
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (nan_bits(v[j])) lab[j] = -1;
    // Every lane runs the whole update (its loads, then a compare-and-swap loop that
    // rarely iterates): measured several times faster here than first filtering on
    // the bin's key, which makes the warp diverge around the loop.
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (lab[j] < 0) continue;
      const unsigned long long c = static_cast<unsigned long long>(base + j * FT + tid);
      unsigned long long* b = &bins[2 * lab[j]];
      if (F == kFirst) {
        if (c < *reinterpret_cast<volatile unsigned long long*>(b)) atomicMin(b, c);
      } else if (F == kLast) {
        atomicMax(b, c + 1);
      } else {
        sel_update(b, sel_key_of<F>(v[j]), c, true);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      v[j] = vn[j];
      lab[j] = ln[j];
    }
  }
  __syncthreads();
  SelPart* pr = parts + (row * chunks + chunk) * K;
  for (int k = tid; k < K; k += FT) pr[k] = SelPart{bins[2 * k], bins[2 * k + 1]};
}

// ---------------------------------------------------------------------------------
// large K: float64 reductions into L2-resident accumulators, rows in blocks
// ---------------------------------------------------------------------------------
// Rows are taken RB at a time and the accumulators of a row block are laid out label
// by label, acc[k][r] for the block's RB rows, so the RB values of one column (one
// label) land in RB consecutive words.  A warp loads RB rows x 32 columns with the
// lanes along the columns (whole cache lines), passes them through a padded shared
// stage, and reduces with lane l on row l % RB and column group l / RB: the RB lanes
// of a group reduce into one contiguous span, which the L2 serves several times
// faster than RB scattered words.  CTAs run row block after row block and RB is
// chosen so that a block's accumulators fit comfortably in L2.  The order of the
// float64 reductions is not fixed, so sums may differ in the last bits from run to
// run; counts and selections are exact.
constexpr int kBigT = 16;  // loads in flight per lane

NBG_HOST_DEVICE long long big_tile_cols(int rb) { return 32LL * (kBigT / rb) * (FT / 32); }

template <typename V, int RB>
struct BigStage {  // per warp: U sub-tiles of RB rows x 32 columns, rows padded
  static constexpr int U = kBigT / RB;
  static constexpr int P = RB == 1 ? 32 : 32 + 16 / RB;  // conflict-free transposed reads
  V s[FT / 32][U][RB][P];
};

// Loads RB rows x 32U columns of the row block (lanes along the columns) and hands
// f the kBigT elements that lane (r = lane % RB, g = lane / RB) reduces: value of row
// r and label of its column (-1 past c1; labels are below 2^31), with the tile's first
// column (big_col gives each element's column).
template <typename V, typename L, int RB, typename Fn>
NBG_DEVICE void big_tiles(const V* __restrict__ values, const L* __restrict__ labels, long long rows, long long m,
                          long long rb, long long c0, long long c1, BigStage<typename BitsOf<V>::type, RB>& st,
                          Fn&& f) {
  typedef typename BitsOf<V>::type B;
  constexpr int U = BigStage<B, RB>::U, G = 32 / RB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = lane % RB, g = lane / RB;
  const long long row0 = rb * RB;
  const unsigned long long stream = l2_evict_first();
  for (long long cbase = c0 + static_cast<long long>(warp) * 32 * U; cbase < c1;
       cbase += static_cast<long long>(FT / 32) * 32 * U) {
    B x[U][RB];
    long long lab[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long col = cbase + u * 32 + lane;
      const bool in = col < c1;
      lab[u] = in ? static_cast<long long>(ld_hint(labels + col, stream)) : -1;
#pragma unroll
      for (int rr = 0; rr < RB; ++rr)
        x[u][rr] = (in && row0 + rr < rows) ? ld_hint(as_bits(values) + (row0 + rr) * m + col, stream) : B(0);
    }
    B ev[kBigT];
    int el[kBigT];
    if (RB == 1) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        ev[u] = x[u][0];
        el[u] = static_cast<int>(lab[u]);
      }
    } else {
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int rr = 0; rr < RB; ++rr) st.s[warp][u][rr][lane] = x[u][rr];
      __syncwarp();
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int i = 0; i < RB; ++i) {
          const int c = i * G + g;
          ev[u * RB + i] = st.s[warp][u][r][c];
          el[u * RB + i] = static_cast<int>(__shfl_sync(0xffffffffu, lab[u], c));
        }
      }
      __syncwarp();
    }
    f(ev, el, cbase);
  }
}

// column of element e of big_tiles' lane arrays, in the tile starting at cbase
template <int RB>
NBG_DEVICE long long big_col(long long cbase, int e) {
  const int lane = threadIdx.x & 31;
  if (RB == 1) return cbase + e * 32 + lane;
  return cbase + (e / RB) * 32 + (e % RB) * (32 / RB) + lane / RB;
}

template <int F, typename V, typename L, int RB>
__global__ void __launch_bounds__(FT, 2) big_mom_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                     long long rows, long long m, long long K, long long chunk_len,
                                                     long long chunks, double* __restrict__ acc1,
                                                     double* __restrict__ acc2, unsigned* __restrict__ nanc) {
  typedef typename BitsOf<V>::type B;
  __shared__ BigStage<B, RB> st;
  const long long rb = blockIdx.x / chunks, chunk = blockIdx.x - rb * chunks;
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  const int r = (threadIdx.x & 31) % RB;
  const bool live = rb * RB + r < rows;
  const long long off = rb * K * RB + r;  // accumulator of (label l, row r): off + l * RB
  const unsigned long long keep = l2_evict_last();
  big_tiles<V, L, RB>(values, labels, rows, m, rb, c0, c1, st,
                      [&](const B (&ev)[kBigT], const int (&el)[kBigT], long long) {
#pragma unroll
                        for (int e = 0; e < kBigT; ++e) {
                          const long long l = el[e];
                          if (!live || l < 0 || l >= K) continue;
                          const long long a = off + l * RB;
                          if (nan_bits(ev[e])) {
                            if (Need<F>::cnt) red_add_hint(&nanc[a], 1u, keep);
                            continue;
                          }
                          const double x = bits_to_f64(ev[e]);
                          if (Need<F>::s1) red_add_hint(&acc1[a], x, keep);
                          if (Need<F>::s2) red_add_hint(&acc2[a], x * x, keep);
                        }
                      });
}


// Variance / standard deviation with many labels.  Both moments of RB rows of one label
// sit in 2 RB consecutive words, acc[((rb K + k) RB + r) 2 + m] (m = 0: sum, 1: sum of
// squares), and one reduction instruction of a warp covers 32 / (2 RB) columns with
// 2 RB lanes each: lane (r = (lane / 2) % RB, m = lane % 2) adds x or x * x of row r.
// A label's whole span -- 32 bytes for RB = 2 -- is reduced by one instruction instead
// of one per moment, which halves the L2 sector operations that bound this kernel.
template <int F, typename V, typename L, int RB>
__global__ void __launch_bounds__(FT, 2) big_var_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                     long long rows, long long m, long long K, long long chunk_len,
                                                     long long chunks, double* __restrict__ acc,
                                                     unsigned* __restrict__ nanc) {
  typedef typename BitsOf<V>::type B;
  constexpr int U = kBigT / RB;
  constexpr int LPC = 2 * RB;   // lanes per column
  constexpr int CPI = 32 / LPC;  // columns per instruction
  __shared__ BigStage<B, RB> st;
  const long long rb = blockIdx.x / chunks, chunk = blockIdx.x - rb * chunks;
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = (lane >> 1) % RB, mom = lane & 1, q = lane / LPC;
  const long long row0 = rb * RB;
  const bool live = row0 + r < rows;
  const long long off = rb * K * RB + r;  // (label l, row r): off + l * RB
  const unsigned long long stream = l2_evict_first();
  const unsigned long long keep = l2_evict_last();
  for (long long cbase = c0 + static_cast<long long>(warp) * 32 * U; cbase < c1;
       cbase += static_cast<long long>(FT / 32) * 32 * U) {
    B x[U][RB];
    int lab[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long col = cbase + u * 32 + lane;
      const bool in = col < c1;
      lab[u] = in ? static_cast<int>(ld_hint(labels + col, stream)) : -1;
#pragma unroll
      for (int rr = 0; rr < RB; ++rr)
        x[u][rr] = (in && row0 + rr < rows) ? ld_hint(as_bits(values) + (row0 + rr) * m + col, stream) : B(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int rr = 0; rr < RB; ++rr) st.s[warp][u][rr][lane] = x[u][rr];
    __syncwarp();
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int i = 0; i < LPC; ++i) {
        const int c = i * CPI + q;
        const B e = st.s[warp][u][r][c];
        const long long l = __shfl_sync(0xffffffffu, lab[u], c);
        if (!live || l < 0 || l >= K) continue;
        const long long a = off + l * RB;
        if (nan_bits(e)) {
          if (mom == 0) red_add_hint(&nanc[a], 1u, keep);
          continue;
        }
        // both lanes of a pair square the element (the sum lane's square is dropped):
        // with few rows per block the L2 reductions, not the FP64 pipe, bound this
        const double v = bits_to_f64(e);
        red_add_hint(&acc[2 * a + mom], mom ? v * v : v, keep);
      }
    }
    __syncwarp();
  }
}

// Selection with many labels, in two passes of fire-and-forget L2 reductions (no
// compare-and-swap round trips): pass 0 reduces every bin's order key with max
// (first / last: the column with min / max, which finishes the job); pass 1 reads the
// data again and reduces the column with min wherever an element's key equals its
// bin's maximum -- the first column holding the maximum, as the reference's strict
// comparison keeps.  Exact and independent of the order of the reductions.
//
// HL (float64 values, fewer than 2^32 - 1 columns): the L2 serves these reductions and
// loads by 32-byte sectors, so pass 0 reduces only the high 32 bits of each key (eight
// rows' words per sector instead of four) and pass 1 loads those; an element whose high
// half equals its bin's is a candidate and reduces (low 32 bits of its key, 2^32 - 1 -
// column) with max into a 64-bit word.  Every element holding the maximum key is a
// candidate, and among candidates (same high half) the low half orders the keys, so the
// word ends with the maximum key's first column: the same result with half the sector
// operations.
template <int F, typename V, typename L, int RB, int PASS, bool HL>
__global__ void __launch_bounds__(FT, 2) big_sel_kernel(const V* __restrict__ values, const L* __restrict__ labels,
                                                        long long rows, long long m, long long K, long long chunk_len,
                                                        long long chunks, unsigned long long* __restrict__ kmax,
                                                        unsigned long long* __restrict__ imin) {
  typedef typename BitsOf<V>::type B;
  __shared__ BigStage<B, RB> st;
  const long long rb = blockIdx.x / chunks, chunk = blockIdx.x - rb * chunks;
  const long long c0 = chunk * chunk_len, c1 = min(m, c0 + chunk_len);
  const int r = (threadIdx.x & 31) % RB;
  const bool live = rb * RB + r < rows;
  const long long off = rb * K * RB + r;
  const unsigned long long keep = l2_evict_last();
  unsigned* khi = reinterpret_cast<unsigned*>(kmax);  // HL: high halves, 4 bytes a bin
  big_tiles<V, L, RB>(values, labels, rows, m, rb, c0, c1, st,
                      [&](const B (&ev)[kBigT], const int (&el)[kBigT], long long cbase) {
                        if (PASS == 0) {
#pragma unroll
                          for (int e = 0; e < kBigT; ++e) {
                            const int l = el[e];
                            if (!live || l < 0 || l >= K || nan_bits(ev[e])) continue;
                            const long long a = off + static_cast<long long>(l) * RB;
                            const unsigned long long c = static_cast<unsigned long long>(big_col<RB>(cbase, e));
                            if (F == kFirst) red_min_hint(&imin[a], c, keep);
                            else if (F == kLast) red_max_hint(&kmax[a], c + 1, keep);
                            else if (HL) red_max_hint(&khi[a], static_cast<unsigned>(sel_key_of<F>(ev[e]) >> 32), keep);
                            else red_max_hint(&kmax[a], sel_key_of<F>(ev[e]), keep);
                          }
                        } else if (HL) {
                          unsigned best[kBigT];  // independent loads, all in flight
#pragma unroll
                          for (int e = 0; e < kBigT; ++e) {
                            const int l = el[e];
                            best[e] = 0u;
                            if (live && l >= 0 && l < K) best[e] = ld_keep(&khi[off + static_cast<long long>(l) * RB], keep);
                          }
#pragma unroll
                          for (int e = 0; e < kBigT; ++e) {
                            const int l = el[e];
                            if (!live || l < 0 || l >= K || nan_bits(ev[e])) continue;
                            const unsigned long long key = sel_key_of<F>(ev[e]);
                            if (static_cast<unsigned>(key >> 32) != best[e]) continue;
                            const unsigned long long c = static_cast<unsigned long long>(big_col<RB>(cbase, e));
                            red_max_hint(&imin[off + static_cast<long long>(l) * RB], (key << 32) | (0xffffffffull - c),
                                         keep);
                          }
                        } else {
                          unsigned long long best[kBigT];  // independent loads, all in flight
#pragma unroll
                          for (int e = 0; e < kBigT; ++e) {
                            const int l = el[e];
                            best[e] = 0;
                            if (live && l >= 0 && l < K)
                              best[e] = ld_keep(&kmax[off + static_cast<long long>(l) * RB], keep);
                          }
#pragma unroll
                          for (int e = 0; e < kBigT; ++e) {
                            const int l = el[e];
                            if (!live || l < 0 || l >= K || nan_bits(ev[e])) continue;
                            if (sel_key_of<F>(ev[e]) != best[e]) continue;
                            red_min_hint(&imin[off + static_cast<long long>(l) * RB],
                                         static_cast<unsigned long long>(big_col<RB>(cbase, e)), keep);
                          }
                        }
                      });
}

// ---------------------------------------------------------------------------------
// finalisation: fold the partials over chunks (in chunk order) and write the output
// ---------------------------------------------------------------------------------
template <int F, typename O>
NBG_DEVICE O finish_mom(double s1, double s2, long long cnt, int pinf, int ninf, long long ddof) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  if (F == kCount) return static_cast<O>(cnt);
  if (F == kSum || F == kMean) {
    double s = s1;
    if (pinf && ninf) s = nan;
    else if (pinf) s = inf;
    else if (ninf) s = -inf;
    if (F == kSum) return static_cast<O>(s);
    return static_cast<O>(cnt == 0 ? nan : s / static_cast<double>(cnt));  // numbagg/grouped.py:22-27
  }
  if (F == kSumSq) return static_cast<O>((pinf || ninf) ? inf : s2);
  // kVar / kStd, numbagg/grouped.py:170-176
  const long long denom = cnt - ddof;
  if (denom <= 0 || pinf || ninf) return static_cast<O>(nan);
  double v = (s2 - (s1 * s1) / static_cast<double>(cnt)) / static_cast<double>(denom);
  if (F == kStd) v = sqrt(v);
  return static_cast<O>(v);
}

template <int F, typename O>
__global__ void fold_mom_kernel(const MomPart* __restrict__ parts, O* __restrict__ out, long long rows, long long K,
                                long long chunks, long long ddof) {
  const long long total = rows * K;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long row = t / K, k = t - row * K;
    double s1 = 0.0, s2 = 0.0;
    long long cnt = 0;
    int pinf = 0, ninf = 0;
    for (long long c = 0; c < chunks; ++c) {
      const MomPart p = parts[(row * chunks + c) * K + k];
      s1 += p.s1;
      s2 += p.s2;
      cnt += p.cnt;
      pinf += p.pinf;
      ninf += p.ninf;
    }
    out[t] = finish_mom<F, O>(s1, s2, cnt, pinf, ninf, ddof);
  }
}

// ---------------------------------------------------------------------------------
// ragged series with their own labels (values and labels flat, series s covering
// [offsets[s], offsets[s + 1])): chunks of kRagCols values, CTA-shared fixed-point bins
// at the chunk's largest exponent, one partial per chunk and label, folded per series
// in chunk order (deterministic).
// ---------------------------------------------------------------------------------
constexpr int kRagCols = FT * 16;

template <int F, typename L>
__global__ void __launch_bounds__(FT) ragged_mom_kernel(const double* __restrict__ values,
                                                        const L* __restrict__ labels, Layout lay, int K,
                                                        MomPart* __restrict__ parts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* b1 = reinterpret_cast<unsigned long long*>(smem_raw);  // [K]
  unsigned* cnt = reinterpret_cast<unsigned*>(b1 + K);                       // [K]
  unsigned* infc = cnt + K;                                                   // [K]: +1 per +inf, +65536 per -inf
  __shared__ int red[FT / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long items = layout_items(lay);
  for (long long id = blockIdx.x; id < items; id += gridDim.x) {
    const Item it = layout_item(lay, id);
    const long long c0 = it.index * kRagCols, c1 = min(it.len, c0 + kRagCols);
    for (int k = tid; k < K; k += FT) {
      b1[k] = 0;
      cnt[k] = 0;
      infc[k] = 0;
    }
    unsigned long long v[16];
    int lab[16];
    int emax = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const long long col = c0 + j * FT + tid;
      const bool in = col < c1;
      v[j] = in ? __ldcs(reinterpret_cast<const unsigned long long*>(values) + it.base + col) : 0ull;
      const long long l = in ? static_cast<long long>(__ldg(labels + it.base + col)) : -1;
      lab[j] = (l >= 0 && l < K && !nan_bits(v[j])) ? static_cast<int>(l) : -1;
      const Dec d = decomp(v[j]);
      if (lab[j] >= 0 && !d.special) emax = max(emax, d.e);
    }
    emax = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(emax)));
    if (lane == 0) red[warp] = emax;
    __syncthreads();  // also orders the bin reset before the updates
    int E = 1;
#pragma unroll
    for (int w = 0; w < FT / 32; ++w) E = max(E, red[w]);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (lab[j] < 0) continue;
      atomicAdd(&cnt[lab[j]], 1u);
      const Dec d = decomp(v[j]);
      if (d.special) {
        atomicAdd(&infc[lab[j]], d.neg ? 65536u : 1u);
        continue;
      }
      if (Need<F>::s1) {
        const int sh = E - d.e + 4;  // 49-bit terms: 4096 of them fit in 63 bits
        const unsigned long long a = sh >= 64 ? 0ull : (d.m >> sh);
        atomicAdd(&b1[lab[j]], d.neg ? (~a + 1ull) : a);
      }
    }
    __syncthreads();
    for (int k = tid; k < K; k += FT) {
      MomPart p;
      p.s1 = Need<F>::s1 ? fx::to_f64(static_cast<fx::i128>(static_cast<long long>(b1[k])), E + 4 - 1075) : 0.0;
      p.s2 = 0.0;
      p.cnt = cnt[k];
      p.pinf = static_cast<int>(infc[k] & 0xffffu);
      p.ninf = static_cast<int>(infc[k] >> 16);
      parts[id * K + k] = p;
    }
    __syncthreads();
  }
}

template <int F>
__global__ void ragged_fold_kernel(const MomPart* __restrict__ parts, double* __restrict__ out, Layout lay,
                                   long long K) {
  const long long total = lay.rows * K;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long s = t / K, k = t - s * K;
    double s1 = 0.0;
    long long c = 0;
    int pinf = 0, ninf = 0;
    for (long long id = lay.item_start[s]; id < lay.item_start[s + 1]; ++id) {
      const MomPart p = parts[id * K + k];
      s1 += p.s1;
      c += p.cnt;
      pinf += p.pinf;
      ninf += p.ninf;
    }
    out[t] = finish_mom<F, double>(s1, 0.0, c, pinf, ninf, 1);
  }
}

// accumulators acc[t], t = (rb * K + k) * RB + r  ->  out[(rb * RB + r) * K + k]; INTER:
// both moments interleaved in acc1[2 t + m] (big_var_kernel)
template <int F, typename O, int RB, bool INTER>
__global__ void big_mom_finish_kernel(const double* __restrict__ acc1, const double* __restrict__ acc2,
                                      const unsigned* __restrict__ nanc, const unsigned* __restrict__ hist,
                                      const double* __restrict__ rcp, O* __restrict__ out, long long rows,
                                      long long K, long long ddof) {
  const long long total = (rows + RB - 1) / RB * K * RB;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long rb = t / (K * RB), rem = t - rb * K * RB;
    const long long k = rem / RB, row = rb * RB + (rem - k * RB);
    if (row >= rows) continue;
    double s1 = 0.0, s2 = 0.0;
    if (INTER) {
      const double2 p = reinterpret_cast<const double2*>(acc1)[t];
      s1 = p.x;
      s2 = p.y;
    } else {
      s1 = Need<F>::s1 ? acc1[t] : 0.0;
      s2 = Need<F>::s2 ? acc2[t] : 0.0;
    }
    const long long cnt = Need<F>::cnt ? static_cast<long long>(hist[k]) - nanc[t] : 1;
    // infinities are already in the float64 sums (inf + x, inf - inf = NaN)
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    O res;
    if (F == kCount) res = static_cast<O>(cnt);
    else if (F == kSum) res = static_cast<O>(s1);
    else if (F == kSumSq) res = static_cast<O>(s2);
    else if (F == kMean) {
      // s1 / c as the product by the tabled reciprocal (within an ulp of the quotient)
      const bool tab = cnt <= kRcpN && isfinite(s1);
      res = static_cast<O>(cnt == 0 ? nan : (tab ? s1 * __ldg(rcp + cnt) : s1 / static_cast<double>(cnt)));
    } else {
      // (s2 - s1^2 / c) / (c - ddof), numbagg/grouped.py:170-176, with the divisions as
      // products by the tabled reciprocals (within an ulp of each quotient; the
      // subtraction's cancellation is the reference's own)
      const long long denom = cnt - ddof;
      double v = nan;
      if (denom > 0) {
        const bool tab = cnt <= kRcpN && denom <= kRcpN;
        const double rc = tab ? __ldg(rcp + cnt) : 1.0 / static_cast<double>(cnt);
        const double rd = tab ? __ldg(rcp + denom) : 1.0 / static_cast<double>(denom);
        v = (s2 - s1 * (s1 * rc)) * rd;
      }
      if (F == kStd) v = sqrt(v);
      res = static_cast<O>(v);
    }
    out[row * K + k] = res;
  }
}

template <int F, typename V, typename O>
NBG_DEVICE O finish_sel(unsigned long long key, unsigned long long idx, const V* vrow) {
  if (F == kFirst) return key == ~0ull ? (IsFloat<O>::value ? nan_of<O>() : O(0)) : static_cast<O>(vrow[key]);
  if (F == kLast) return key == 0ull ? nan_of<O>() : static_cast<O>(vrow[key - 1]);
  if (idx == ~0ull) return nan_of<O>();
  if (F == kArgMax || F == kArgMin) return static_cast<O>(idx);
  return static_cast<O>(static_cast<double>(vrow[idx]));  // max / min via the float64 running value
}

template <int F, typename V, typename O, int RB, bool HL>
__global__ void big_sel_finish_kernel(const unsigned long long* __restrict__ kmax,
                                      const unsigned long long* __restrict__ imin, const V* __restrict__ values,
                                      O* __restrict__ out, long long rows, long long m, long long K) {
  const long long total = (rows + RB - 1) / RB * K * RB;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long rb = t / (K * RB), rem = t - rb * K * RB;
    const long long k = rem / RB, row = rb * RB + (rem - k * RB);
    if (row >= rows) continue;
    // finish_sel's (key, index) convention: first keeps its column in the key
    unsigned long long key, idx;
    if (HL) {  // (low half of the key, 2^32 - 1 - column); 0: no element
      key = imin[t];
      idx = key ? 0xffffffffull - (key & 0xffffffffull) : ~0ull;
    } else {
      key = F == kFirst ? imin[t] : kmax[t];
      idx = (F == kFirst || F == kLast) ? 0ull : (kmax[t] ? imin[t] : ~0ull);
    }
    out[row * K + k] = finish_sel<F, V, O>(key, idx, values + row * m);
  }
}

template <int F, typename V, typename O>
__global__ void fold_sel_kernel(const SelPart* __restrict__ parts, const V* __restrict__ values, O* __restrict__ out,
                                long long rows, long long m, long long K, long long chunks, int stride_parts) {
  const long long total = rows * K;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const bool is_idx = F == kFirst || F == kLast;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride) {
    const long long row = t / K, k = t - row * K;
    unsigned long long key = (F == kFirst) ? ~0ull : 0ull, idx = ~0ull;
    for (long long c = 0; c < chunks; ++c) {
      const SelPart p = parts[(row * chunks + c) * K + k];
      if (is_idx) {
        key = (F == kFirst) ? min(key, p.key) : max(key, p.key);
      } else if (p.idx != ~0ull && better(p.key, p.idx, key, idx)) {
        key = p.key;
        idx = p.idx;
      }
    }
    out[t] = finish_sel<F, V, O>(key, idx, values + row * m);
  }
}

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
struct FastPlan {
  int strategy;  // 0 tiny, 1 medium, 2 large
  long long chunks, chunk_len;  // large: chunks per row block
  int rb;                       // large: rows per block (1, 2, 4, 8 or 16)
  long long blocks;             // large: row blocks
};

// Rows per block of the large path: as many as 16, as long as the block's
// accumulators (K x RB x the bytes a bin keeps) stay within 64 MB of the L2, and no
// more than the rows rounded up to a power of two.
inline int big_rows_per_block(int f, long long rows, long long K) {
  // selection: the bins that pass 0 reduces (8-byte keys; the float64 argmax / argmin /
  // max / min reduce 4-byte high halves there, so rows per block double for them)
  size_t per = 8;
  if (is_moments(f)) {
    per = 4;  // NaN count (count / mean / var / std; kept for the others too)
    if (f == kSum || f == kMean || f == kVar || f == kStd) per += 8;
    if (f == kVar || f == kStd || f == kSumSq) per += 8;
  }
  int rb = 16;
  const size_t budget = 64ull << 20;
  while (rb > 1 && (rb / 2 >= rows || static_cast<size_t>(K) * rb * per > budget)) rb /= 2;
  return rb;
}

inline size_t mid_smem_bytes(int f, long long K) {
  size_t per = 16;
  switch (f) {
    case kSum: per = mid_mom_bytes_per_bin<kSum>(); break;
    case kCount: per = mid_mom_bytes_per_bin<kCount>(); break;
    case kMean: per = mid_mom_bytes_per_bin<kMean>(); break;
    case kVar: per = mid_mom_bytes_per_bin<kVar>(); break;
    case kStd: per = mid_mom_bytes_per_bin<kStd>(); break;
    case kSumSq: per = mid_mom_bytes_per_bin<kSumSq>(); break;
    default: per = 16; break;
  }
  return static_cast<size_t>(K) * per;
}

inline FastPlan fast_plan(int f, long long rows, long long m, long long K) {
  FastPlan p;
  const long long sms = num_sms();
  if (K <= kTinyK) {
    p.strategy = 0;
  } else if (is_moments(f) && !deterministic_mode()) {
    p.strategy = 2;  // float64 reductions in L2 beat shared-memory 64-bit atomics
  } else if (mid_smem_bytes(f, K) <= 100 * 1024) {
    p.strategy = 1;
  } else {
    p.strategy = 2;
  }
  p.rb = 1;
  p.blocks = rows;
  if (p.strategy == 2) {
    p.rb = big_rows_per_block(f, rows, K);
    p.blocks = (rows + p.rb - 1) / p.rb;
  }
  // large: CTAs per row block (four per SM); tiny / medium: CTAs per call, four
  // waves of two CTAs per SM
  long long target = p.strategy == 2 ? sms * 4 : sms * 8;
  long long chunks = p.strategy == 2 ? target : (target + rows - 1) / max(rows, 1ll);
  const long long unit = p.strategy == 0 ? static_cast<long long>(kTileCols) * (FT / 32)
                                         : (p.strategy == 1 ? kCtaCols : big_tile_cols(p.rb));
  long long min_len = unit;
  if (p.strategy == 1) min_len = max(unit, 4 * K);  // amortise initialising / writing K bins
  long long max_chunks = (m + min_len - 1) / min_len;
  chunks = max(1ll, min(chunks, max_chunks));
  long long len = (m + chunks - 1) / chunks;
  len = ((len + unit - 1) / unit) * unit;
  p.chunk_len = max(len, unit);
  p.chunks = max(1ll, (m + p.chunk_len - 1) / p.chunk_len);
  return p;
}

inline size_t fast_bytes(int f, long long rows, long long m, long long K) {
  const FastPlan p = fast_plan(f, rows, m, K);
  if (p.strategy == 2) {
    const size_t slots = static_cast<size_t>(p.blocks * p.rb * K);
    if (is_moments(f)) return slots * (8 + 8 + 4) + static_cast<size_t>(K) * 4 + (kRcpN + 1) * 8 + 1280;
    return slots * 16 + 1024;
  }
  const size_t part = is_moments(f) ? sizeof(MomPart) : sizeof(SelPart);
  size_t b = static_cast<size_t>(rows * p.chunks * K) * part + 1024;
  if (p.strategy == 1 && is_moments(f)) b += static_cast<size_t>(p.chunks * K) * 4 + 256;
  return b;
}

inline bool fast_path(int f, bool float_values) {
  return (is_moments(f) && float_values) || is_select(f) || f == kFirst || f == kLast;
}

template <typename T>
T* carve(unsigned char*& p, size_t count) {
  p = reinterpret_cast<unsigned char*>((reinterpret_cast<size_t>(p) + 255) & ~static_cast<size_t>(255));
  T* r = reinterpret_cast<T*>(p);
  p += count * sizeof(T);
  return r;
}

inline int fin_grid(long long total) {
  long long blocks = (total + 255) / 256;
  const long long cap = static_cast<long long>(num_sms()) * 16;
  return static_cast<int>(max(1ll, min(blocks, cap)));
}

// The default dynamic limit is 48 KiB minus the kernel's static shared memory (up to a
// few KiB here), so the opt-in is needed from well below 48 KiB of dynamic bytes.
template <typename K>
void set_smem(K kern, size_t bytes) {
  if (bytes > 32 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

template <int F, typename V, typename L, typename O, int RB>
int launch_big_mom(const V* values, const L* labels, O* out, long long rows, long long m, long long K, long long ddof,
                   const FastPlan& p, unsigned char*& cur, cudaStream_t s) {
  const long long slots = p.blocks * RB * K;
  // the variance and standard deviation with few rows per block (many labels, where
  // the L2 reductions bound the kernel) interleave both moments for big_var_kernel
  constexpr bool INTER = Need<F>::varlike && RB <= 4;
  // variance / standard deviation: both moments interleaved in acc1 (big_var_kernel)
  double* acc1 = carve<double>(cur, INTER ? 2 * slots : slots);
  double* acc2 = carve<double>(cur, (Need<F>::s2 && !INTER) ? slots : 1);
  unsigned* nanc = carve<unsigned>(cur, slots);
  unsigned* hist = carve<unsigned>(cur, K);
  double* rcp = carve<double>(cur, kRcpN + 1);
  int launches = 0;
  if (Need<F>::s1) cudaMemsetAsync(acc1, 0, static_cast<size_t>(slots) * (INTER ? 16 : 8), s);
  if (Need<F>::s2 && !INTER) cudaMemsetAsync(acc2, 0, static_cast<size_t>(slots) * 8, s);
  if (Need<F>::cnt) {
    cudaMemsetAsync(nanc, 0, static_cast<size_t>(slots) * 4, s);
    cudaMemsetAsync(hist, 0, static_cast<size_t>(K) * 4, s);
    if (K <= kHistSmem) {
      auto hk = row_hist_kernel<L, true>;
      set_smem(hk, static_cast<size_t>(K) * 4);
      const int grid = static_cast<int>(max(1ll, min(static_cast<long long>(num_sms()) * 2, (m + FT * 64 - 1) / (FT * 64))));
      hk<<<grid, FT, static_cast<size_t>(K) * 4, s>>>(labels, m, K, hist, rcp);
    } else {
      row_hist_kernel<L, false><<<fin_grid(max(m, kRcpN + 1)), FT, 0, s>>>(labels, m, K, hist, rcp);
    }
    ++launches;
  }
  if constexpr (INTER)
    big_var_kernel<F, V, L, RB><<<static_cast<int>(p.blocks * p.chunks), FT, 0, s>>>(values, labels, rows, m, K,
                                                                                     p.chunk_len, p.chunks, acc1, nanc);
  else
    big_mom_kernel<F, V, L, RB><<<static_cast<int>(p.blocks * p.chunks), FT, 0, s>>>(values, labels, rows, m, K,
                                                                                     p.chunk_len, p.chunks, acc1, acc2, nanc);
  big_mom_finish_kernel<F, O, RB, INTER><<<fin_grid(slots), 256, 0, s>>>(acc1, acc2, nanc, hist, rcp, out, rows, K, ddof);
  return launches + 2;
}

template <int F, typename V, typename L, typename O, int RB>
int launch_big_sel(const V* values, const L* labels, O* out, long long rows, long long m, long long K,
                   const FastPlan& p, unsigned char*& cur, cudaStream_t s) {
  const long long slots = p.blocks * RB * K;
  unsigned long long* kmax = carve<unsigned long long>(cur, slots);
  unsigned long long* imin = carve<unsigned long long>(cur, slots);
  const int grid = static_cast<int>(p.blocks * p.chunks);
  constexpr bool kHLType = sizeof(V) == 8 && IsFloat<V>::value && F != kFirst && F != kLast;
  if (kHLType && m < 0xffffffffll) {
    cudaMemsetAsync(kmax, 0, static_cast<size_t>(slots) * 4, s);  // high halves: none yet
    cudaMemsetAsync(imin, 0, static_cast<size_t>(slots) * 8, s);  // no candidate yet
    big_sel_kernel<F, V, L, RB, 0, kHLType><<<grid, FT, 0, s>>>(values, labels, rows, m, K, p.chunk_len, p.chunks,
                                                                 kmax, imin);
    big_sel_kernel<F, V, L, RB, 1, kHLType><<<grid, FT, 0, s>>>(values, labels, rows, m, K, p.chunk_len, p.chunks,
                                                                 kmax, imin);
    big_sel_finish_kernel<F, V, O, RB, kHLType><<<fin_grid(slots), 256, 0, s>>>(kmax, imin, values, out, rows, m, K);
    return 3;
  }
  cudaMemsetAsync(kmax, 0, static_cast<size_t>(slots) * 8, s);     // below every key and column + 1
  cudaMemsetAsync(imin, 0xff, static_cast<size_t>(slots) * 8, s);  // no column yet
  big_sel_kernel<F, V, L, RB, 0, false><<<grid, FT, 0, s>>>(values, labels, rows, m, K, p.chunk_len, p.chunks, kmax,
                                                              imin);
  int launches = 1;
  if (F != kFirst && F != kLast) {
    big_sel_kernel<F, V, L, RB, 1, false><<<grid, FT, 0, s>>>(values, labels, rows, m, K, p.chunk_len, p.chunks, kmax,
                                                                imin);
    ++launches;
  }
  big_sel_finish_kernel<F, V, O, RB, false><<<fin_grid(slots), 256, 0, s>>>(kmax, imin, values, out, rows, m, K);
  return launches + 1;
}

template <int F, typename V, typename L, typename O>
int launch_fast(const V* values, const L* labels, O* out, long long rows, long long m, long long K, long long ddof,
                void* ws, size_t ws_bytes, cudaStream_t s) {
  const FastPlan p = fast_plan(F, rows, m, K);
  if (!ws || ws_bytes < fast_bytes(F, rows, m, K)) return kWorkspaceTooSmall;
  unsigned char* cur = static_cast<unsigned char*>(ws);
  const long long nctas = rows * p.chunks;
  if ((p.strategy < 2 ? nctas : p.blocks * p.chunks) > 0x7fffffffll) return kUnsupported;
  // the float64 reductions of the large path are not reproducible bit for bit
  if (p.strategy == 2 && (Need<F>::s1 || Need<F>::s2) && deterministic_mode()) return kUnsupported;
  int launches = 0;
  if (is_moments(F)) {
    if (p.strategy == 0) {
      MomPart* parts = carve<MomPart>(cur, rows * p.chunks * K);
      // headroom of the lanes' fixed-point sums (see tiny_mom_kernel)
      const long long per_lane = ((p.chunk_len + kTileCols * (FT / 32) - 1) / (kTileCols * (FT / 32))) * 16;
      int lg = 0;
      while ((1ll << lg) < per_lane) ++lg;
      const int d1 = lg > 10 ? lg - 10 : 0;
      constexpr bool can_split = F == kSum || F == kMean;
      const bool split = can_split && per_lane < 65536;
      const size_t smem = static_cast<size_t>(K) * FT *
                          ((Need<F>::s1 ? 8 : 0) + (Need<F>::s2 ? 8 : 0) + (split ? 8 : 0) +
                           (Need<F>::cnt ? (split ? 2 : 4) : 0));
      auto kern = split ? tiny_mom_kernel<F, V, L, can_split> : tiny_mom_kernel<F, V, L, false>;
      set_smem(kern, smem);
      kern<<<static_cast<int>(nctas), FT, smem, s>>>(values, labels, rows, m, static_cast<int>(K), p.chunk_len, p.chunks,
                                                     d1, parts);
      fold_mom_kernel<F, O><<<fin_grid(rows * K), 256, 0, s>>>(parts, out, rows, K, p.chunks, ddof);
      launches += 2;
    } else if (p.strategy == 1) {
      MomPart* parts = carve<MomPart>(cur, rows * p.chunks * K);
      unsigned* hist = carve<unsigned>(cur, p.chunks * K);
      {  // per-chunk label histogram: valid counts, and the flush bound of the bins
        auto hk = chunk_hist_kernel<L>;
        set_smem(hk, static_cast<size_t>(K) * 4);
        hk<<<static_cast<int>(p.chunks), FT, static_cast<size_t>(K) * 4, s>>>(labels, m, static_cast<int>(K), p.chunk_len, hist);
        ++launches;
      }
      const size_t smem = mid_smem_bytes(F, K);
      auto kern = mid_mom_kernel<F, V, L>;
      set_smem(kern, smem);
      kern<<<static_cast<int>(nctas), FT, smem, s>>>(values, labels, rows, m, static_cast<int>(K), p.chunk_len, p.chunks,
                                                     hist, parts);
      fold_mom_kernel<F, O><<<fin_grid(rows * K), 256, 0, s>>>(parts, out, rows, K, p.chunks, ddof);
      launches += 2;
    } else {
      switch (p.rb) {
        case 8: launches += launch_big_mom<F, V, L, O, 8>(values, labels, out, rows, m, K, ddof, p, cur, s); break;
        case 16: launches += launch_big_mom<F, V, L, O, 16>(values, labels, out, rows, m, K, ddof, p, cur, s); break;
        case 4: launches += launch_big_mom<F, V, L, O, 4>(values, labels, out, rows, m, K, ddof, p, cur, s); break;
        case 2: launches += launch_big_mom<F, V, L, O, 2>(values, labels, out, rows, m, K, ddof, p, cur, s); break;
        default: launches += launch_big_mom<F, V, L, O, 1>(values, labels, out, rows, m, K, ddof, p, cur, s); break;
      }
    }
  } else {
    if (p.strategy == 0) {
      SelPart* parts = carve<SelPart>(cur, rows * p.chunks * K);
      const size_t smem = static_cast<size_t>(K) * FT * 16;
      auto kern = tiny_sel_kernel<F, V, L>;
      set_smem(kern, smem);
      kern<<<static_cast<int>(nctas), FT, smem, s>>>(values, labels, rows, m, static_cast<int>(K), p.chunk_len, p.chunks,
                                                     parts);
      fold_sel_kernel<F, V, O><<<fin_grid(rows * K), 256, 0, s>>>(parts, values, out, rows, m, K, p.chunks, 1);
      launches = 2;
    } else if (p.strategy == 1) {
      SelPart* parts = carve<SelPart>(cur, rows * p.chunks * K);
      const size_t smem = static_cast<size_t>(K) * 16;
      auto kern = mid_sel_kernel<F, V, L>;
      set_smem(kern, smem);
      kern<<<static_cast<int>(nctas), FT, smem, s>>>(values, labels, rows, m, static_cast<int>(K), p.chunk_len, p.chunks,
                                                     parts);
      fold_sel_kernel<F, V, O><<<fin_grid(rows * K), 256, 0, s>>>(parts, values, out, rows, m, K, p.chunks, 1);
      launches = 2;
    } else {
      switch (p.rb) {
        case 8: launches = launch_big_sel<F, V, L, O, 8>(values, labels, out, rows, m, K, p, cur, s); break;
        case 16: launches = launch_big_sel<F, V, L, O, 16>(values, labels, out, rows, m, K, p, cur, s); break;
        case 4: launches = launch_big_sel<F, V, L, O, 4>(values, labels, out, rows, m, K, p, cur, s); break;
        case 2: launches = launch_big_sel<F, V, L, O, 2>(values, labels, out, rows, m, K, p, cur, s); break;
        default: launches = launch_big_sel<F, V, L, O, 1>(values, labels, out, rows, m, K, p, cur, s); break;
      }
    }
  }
  note_launches(launches);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

inline size_t ragged_group_bytes(long long nseries, long long total, long long K) {
  return static_cast<size_t>(total / kRagCols + nseries) * static_cast<size_t>(K) * sizeof(MomPart) +
         static_cast<size_t>(nseries + 1) * 8 + 1024;
}

template <int F, typename L>
int launch_ragged_group(const double* values, const L* labels, const long long* offsets, long long nseries,
                        long long total, long long K, double* out, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (nseries < 0 || total < 0 || K < 0) return kInvalidArgument;
  if (nseries == 0 || K == 0) return kOk;
  if (!offsets || !out || (total > 0 && (!values || !labels))) return kInvalidArgument;
  if (K > 8192) return kUnsupported;
  if (!ws || ws_bytes < ragged_group_bytes(nseries, total, K)) return kWorkspaceTooSmall;
  unsigned char* cur = static_cast<unsigned char*>(ws);
  MomPart* parts = carve<MomPart>(cur, (total / kRagCols + nseries) * K);
  long long* item_start = carve<long long>(cur, nseries + 1);
  Layout lay{offsets, item_start, nseries, 0, 0};
  ragged_plan_kernel<<<1, 1024, 0, s>>>(offsets, nseries, kRagCols, item_start);
  const size_t smem = static_cast<size_t>(K) * 16;
  auto kern = ragged_mom_kernel<F, L>;
  set_smem(kern, smem);
  kern<<<layout_grid(LLONG_MAX, 4), FT, smem, s>>>(values, labels, lay, static_cast<int>(K), parts);
  ragged_fold_kernel<F><<<fin_grid(nseries * K), 256, 0, s>>>(parts, out, lay, K);
  note_launches(3);
  return cudaGetLastError() == cudaSuccess ? kOk : kLaunchError;
}

}  // namespace grouped
}  // namespace nbg

// ---------------------------------------------------------------------------------
// exported entry points of the fast paths: the translation units grouped_fast_*.cu
// each instantiate a share of them (they compile in parallel)
// ---------------------------------------------------------------------------------
namespace nbg {
namespace grouped {
template <int F, typename V, typename L, typename O>
int group_fast_entry(const V* values, const L* labels, O* out, long long rows, long long m, long long K,
                     long long ddof, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (rows < 0 || m < 0 || K < 0) return kInvalidArgument;
  if (rows == 0 || K == 0) return kOk;
  if (!out || (m > 0 && (!values || !labels))) return kInvalidArgument;
  if (K > 0x7fffffffll) return kUnsupported;
  // m == 0 still runs: one chunk of no columns writes every output's empty value
  return launch_fast<F, V, L, O>(values, labels, out, rows, m, K, ddof, ws, ws_bytes, s);
}
}  // namespace grouped
}  // namespace nbg

#define NBG_GFAST_ONE(NAME, FC, V, VS, O, L, LS)                                               \
  int nbg_group_##NAME##_##VS##_##LS(const V* values, const L* labels, O* out, long long rows,  \
                                     long long m, long long num_labels, long long ddof, void* ws, \
                                     size_t ws_bytes, void* stream) {                          \
    return nbg::grouped::group_fast_entry<FC, V, L, O>(values, labels, out, rows, m, num_labels, \
                                                       ddof, ws, ws_bytes,                      \
                                                       static_cast<cudaStream_t>(stream));      \
  }
#define NBG_GFAST_LABELS(NAME, FC, V, VS, O) \
  NBG_GFAST_ONE(NAME, FC, V, VS, O, int, i32) NBG_GFAST_ONE(NAME, FC, V, VS, O, long long, i64)
