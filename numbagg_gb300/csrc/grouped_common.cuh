// Shared declarations of the labelled-reduction kernels (grouped.cu, grouped_fast.cuh).
#pragma once

#include "nbg_common.cuh"

#include <climits>
#include <algorithm>

namespace nbg {
namespace grouped {

enum Func : int {
  kSum = 0,
  kCount,
  kMean,
  kVar,
  kStd,
  kSumSq,
  kArgMax,
  kArgMin,
  kMax,
  kMin,
  kFirst,
  kLast,
  kProd,
  kAny,
  kAll,
  kNumFuncs
};

struct Acc {  // one bin: meaning depends on the function family
  unsigned long long a, b, c;
};

constexpr unsigned long long kNoIdx = ~0ull;

NBG_HOST_DEVICE bool is_moments(int f) {
  return f == kSum || f == kCount || f == kMean || f == kVar || f == kStd || f == kSumSq;
}
NBG_HOST_DEVICE bool is_select(int f) { return f == kArgMax || f == kArgMin || f == kMax || f == kMin; }

template <typename V>
struct IsFloat { static constexpr bool value = false; };
template <>
struct IsFloat<double> { static constexpr bool value = true; };
template <>
struct IsFloat<float> { static constexpr bool value = true; };

template <int F>
NBG_DEVICE Acc acc_identity() {
  Acc r{0ull, 0ull, 0ull};
  if (is_select(F) || F == kFirst) r.b = kNoIdx;
  if (F == kFirst) r.a = kNoIdx;
  if (F == kProd) r.a = 0;  // set per value type in init (1 or 1.0)
  if (F == kAll) r.a = 1ull;
  return r;
}

template <int F, typename V>
NBG_DEVICE Acc acc_init() {
  Acc r = acc_identity<F>();
  if (F == kProd) {
    if (IsFloat<V>::value)
      r.a = static_cast<unsigned long long>(__double_as_longlong(1.0));
    else
      r.a = 1ull;
  }
  return r;
}

template <typename V>
NBG_DEVICE unsigned long long select_key(V v, bool minimize) {
  const unsigned long long k = order_key_ieee(static_cast<double>(v));
  return minimize ? ~k : k;
}

NBG_DEVICE double as_d(unsigned long long u) { return __longlong_as_double(static_cast<long long>(u)); }
NBG_DEVICE unsigned long long as_u(double d) { return static_cast<unsigned long long>(__double_as_longlong(d)); }

// Shared-memory double add: compare-and-swap on the bit pattern.
NBG_DEVICE void atomic_add_f64(unsigned long long* p, double v) {
  atomicAdd(reinterpret_cast<double*>(p), v);
}

template <typename V>
NBG_DEVICE void atomic_mul(unsigned long long* p, V v) {
  unsigned long long old = *p, assumed;
  do {
    assumed = old;
    unsigned long long nv;
    if (IsFloat<V>::value)
      nv = as_u(as_d(assumed) * static_cast<double>(v));
    else
      nv = assumed * static_cast<unsigned long long>(static_cast<long long>(v));
    old = atomicCAS(p, assumed, nv);
  } while (old != assumed);
}

// Accumulate one valid element into a bin.  ATOMIC selects atomics vs plain RMW
// (lane-private bins).
template <int F, typename V, bool ATOMIC>
NBG_DEVICE void accumulate(Acc* bin, V v, unsigned long long col) {
  if (is_moments(F)) {
    const bool need_s1 = F == kSum || F == kMean || F == kVar || F == kStd;
    const bool need_s2 = F == kVar || F == kStd || F == kSumSq;
    const bool need_c = F == kCount || F == kMean || F == kVar || F == kStd;
    if (IsFloat<V>::value) {
      const double x = static_cast<double>(v);
      if (ATOMIC) {
        if (need_s1) atomic_add_f64(&bin->a, x);
        if (need_s2) atomic_add_f64(&bin->b, x * x);
        if (need_c) atomicAdd(&bin->c, 1ull);
      } else {
        if (need_s1) bin->a = as_u(as_d(bin->a) + x);
        if (need_s2) bin->b = as_u(as_d(bin->b) + x * x);
        if (need_c) bin->c += 1ull;
      }
    } else {
      const unsigned long long x = static_cast<unsigned long long>(static_cast<long long>(v));
      if (ATOMIC) {
        if (need_s1) atomicAdd(&bin->a, x);
        if (need_s2) atomicAdd(&bin->b, x * x);
        if (need_c) atomicAdd(&bin->c, 1ull);
      } else {
        if (need_s1) bin->a += x;
        if (need_s2) bin->b += x * x;
        if (need_c) bin->c += 1ull;
      }
    }
  } else if (F == kFirst) {
    if (ATOMIC) atomicMin(&bin->a, col); else if (col < bin->a) bin->a = col;
  } else if (F == kLast) {
    if (ATOMIC) atomicMax(&bin->a, col + 1); else if (col + 1 > bin->a) bin->a = col + 1;
  } else if (F == kProd) {
    if (ATOMIC) {
      atomic_mul<V>(&bin->a, v);
    } else {
      if (IsFloat<V>::value)
        bin->a = as_u(as_d(bin->a) * static_cast<double>(v));
      else
        bin->a = bin->a * static_cast<unsigned long long>(static_cast<long long>(v));
    }
  } else if (F == kAny) {
    if (v != V(0)) {
      if (ATOMIC) atomicOr(reinterpret_cast<unsigned*>(&bin->a), 1u); else bin->a = 1ull;
    }
  } else if (F == kAll) {
    if (v == V(0)) {
      if (ATOMIC) atomicAnd(reinterpret_cast<unsigned*>(&bin->a), 0u); else bin->a = 0ull;
    }
  } else if (is_select(F)) {
    const unsigned long long key = select_key(v, F == kArgMin || F == kMin);
    if (ATOMIC) atomicMax(&bin->a, key); else if (key > bin->a) bin->a = key;
  }
}

// Fold bin `src` into `dst` (dst earlier in column order than src).
template <int F, typename V>
NBG_DEVICE Acc fold(Acc dst, const Acc& src) {
  if (is_moments(F)) {
    if (IsFloat<V>::value) {
      dst.a = as_u(as_d(dst.a) + as_d(src.a));
      dst.b = as_u(as_d(dst.b) + as_d(src.b));
    } else {
      dst.a += src.a;
      dst.b += src.b;
    }
    dst.c += src.c;
  } else if (is_select(F)) {
    if (src.a > dst.a || (src.a == dst.a && src.b < dst.b)) dst = src;
  } else if (F == kFirst) {
    if (src.a < dst.a) dst.a = src.a;
  } else if (F == kLast) {
    if (src.a > dst.a) dst.a = src.a;
  } else if (F == kProd) {
    if (IsFloat<V>::value)
      dst.a = as_u(as_d(dst.a) * as_d(src.a));
    else
      dst.a = dst.a * src.a;
  } else if (F == kAny) {
    dst.a |= src.a;
  } else if (F == kAll) {
    dst.a &= src.a;
  }
  return dst;
}

template <typename V>
NBG_DEVICE V load_value(const V* p) { return *p; }


template <typename O>
NBG_DEVICE O nan_of() {
  if (IsFloat<O>::value) return static_cast<O>(__longlong_as_double(0x7ff8000000000000ll));
  return sizeof(O) == 4 ? static_cast<O>(INT_MIN) : static_cast<O>(LLONG_MIN);
}

// scratch bytes of the fast paths (grouped_fast.cuh); 0 for functions they do not serve
size_t fast_bytes_query(int f, long long rows, long long m, long long K);

inline int num_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace grouped
}  // namespace nbg
