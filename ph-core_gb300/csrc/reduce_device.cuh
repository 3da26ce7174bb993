// reduce_device.cuh -- accumulators and per-output bodies of the reductions,
// shared by the standalone kernels (reduce.cu) and the batched executor (batch.cu).
#pragma once

#include <float.h>

#include <type_traits>

#include "plan.h"

namespace phcu {

enum RedKind { RK_SUM = 0, RK_EXT = 1 };

struct Partial {
  double v;
  long long i;
};

struct RedArgs {
  // input: base points at element (0,...,0) of the view
  const char* in;
  int32_t dtype;
  int32_t op;
  // output space (lexicographic over the kept axes)
  int32_t orank;
  int32_t krank;
  int64_t O;
  int64_t oshape[MAXR];
  int64_t ostride[MAXR];  // input stride of each kept axis
  FastDiv odiv[MAXR];
  // reduced space (one axis, or every axis for a full reduction)
  int64_t K;
  int64_t kshape[MAXR];
  int64_t kstride[MAXR];
  FastDiv kdiv[MAXR];
  int64_t kinner;  // stride of the innermost reduced axis
  // splitting
  int64_t S;
  int64_t chunk;
  // output
  char* out;
  int32_t out_dtype;
  int32_t want_index;
  Partial* partial;  // S x O when S > 1
  uint32_t* status;
};

template <typename T>
struct Lim;
template <>
struct Lim<float> {
  static __device__ __forceinline__ bool nan(float x) { return x != x; }
  // the extreme of a and b ignoring a NaN operand (fmaxf/fminf return the other one)
  static __device__ __forceinline__ float ext(float a, float b, bool is_max) { return is_max ? fmaxf(a, b) : fminf(a, b); }
};
template <>
struct Lim<double> {
  static __device__ __forceinline__ bool nan(double x) { return x != x; }
};
template <>
struct Lim<int32_t> {
  static __device__ __forceinline__ bool nan(int32_t) { return false; }
  static __device__ __forceinline__ int32_t ext(int32_t a, int32_t b, bool is_max) { return is_max ? max(a, b) : min(a, b); }
};
template <>
struct Lim<long long> {
  static __device__ __forceinline__ bool nan(long long) { return false; }
};

// --------------------------------------------------------- accumulators
template <typename T>
struct SumAcc {  // floating point: Neumaier (s, c), value s + c
  T s, c;
  __device__ __forceinline__ void init() { s = 0; c = 0; }
  __device__ __forceinline__ void add(T x) {
    T t = s + x;
    if (fabs((double)s) >= fabs((double)x)) c = c + ((s - t) + x);
    else c = c + ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ void merge(const SumAcc& o) {
    // TwoSum(s, o.s)
    T t = s + o.s;
    T bp = t - s;
    T e = (s - (t - bp)) + (o.s - bp);
    s = t;
    c = (c + o.c) + e;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
  __device__ __forceinline__ void shfl(int d, unsigned mask, int w) {
    SumAcc o;
    o.s = __shfl_down_sync(mask, s, d, w);
    o.c = __shfl_down_sync(mask, c, d, w);
    merge(o);
  }
};
template <>
struct SumAcc<float> {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    if (fabsf(s) >= fabsf(x)) c = c + ((s - t) + x);
    else c = c + ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ void merge(const SumAcc& o) {
    float t = s + o.s;
    float bp = t - s;
    float e = (s - (t - bp)) + (o.s - bp);
    s = t;
    c = (c + o.c) + e;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
  __device__ __forceinline__ void shfl(int d, unsigned mask, int w) {
    SumAcc o;
    o.s = __shfl_down_sync(mask, s, d, w);
    o.c = __shfl_down_sync(mask, c, d, w);
    merge(o);
  }
};
template <>
struct SumAcc<int32_t> {
  long long s;
  __device__ __forceinline__ void init() { s = 0; }
  __device__ __forceinline__ void add(int32_t x) { s += x; }
  __device__ __forceinline__ void merge(const SumAcc& o) { s += o.s; }
  __device__ __forceinline__ double value() const { return (double)s; }
  __device__ __forceinline__ void shfl(int d, unsigned mask, int w) { s += __shfl_down_sync(mask, s, d, w); }
};
template <>
struct SumAcc<long long> {
  long long s;
  __device__ __forceinline__ void init() { s = 0; }
  __device__ __forceinline__ void add(long long x) { s = (long long)((unsigned long long)s + (unsigned long long)x); }
  __device__ __forceinline__ void merge(const SumAcc& o) { add(o.s); }
  __device__ __forceinline__ double value() const { return (double)s; }
  __device__ __forceinline__ void shfl(int d, unsigned mask, int w) { add(__shfl_down_sync(mask, s, d, w)); }
};

template <typename T>
struct ExtAcc {  // (v, i); i < 0 = no candidate yet
  T v;
  long long i;
  __device__ __forceinline__ void init() { v = 0; i = -1; }
  __device__ __forceinline__ static bool better(T a, long long ia, T b, long long ib, bool is_max) {
    // is (a, ia) preferred over (b, ib)?
    if (ia < 0) return false;
    if (ib < 0) return true;
    if (is_max ? (a > b) : (a < b)) return true;
    if (a == b && ia < ib) return true;
    return false;
  }
  // Elements reach one accumulator in increasing k, so a later element only
  // wins on a strict improvement (ties keep the earlier index).
  __device__ __forceinline__ void add(T x, long long k, bool is_max) {
    const bool take = !Lim<T>::nan(x) && (i < 0 || (is_max ? (x > v) : (x < v)));
    if (take) {
      v = x;
      i = k;
    }
  }
  __device__ __forceinline__ void merge(const ExtAcc& o, bool is_max) {
    if (better(o.v, o.i, v, i, is_max)) { v = o.v; i = o.i; }
  }
  __device__ __forceinline__ void shfl(int d, unsigned mask, int w, bool is_max) {
    ExtAcc o;
    o.v = __shfl_down_sync(mask, v, d, w);
    o.i = __shfl_down_sync(mask, i, d, w);
    merge(o, is_max);
  }
};

// ------------------------------------------------------------ helpers
__device__ __forceinline__ int64_t out_offset(const RedArgs& a, uint32_t o) {
  int64_t off = 0;
  for (int d = a.orank - 1; d >= 0; d--) {
    uint32_t q, x;
    a.odiv[d].divmod(o, q, x);
    o = q;
    off += (int64_t)x * a.ostride[d];
  }
  return off;
}

__device__ __forceinline__ int64_t k_offset(const RedArgs& a, uint32_t k) {
  if (a.krank == 1) return (int64_t)k * a.kstride[0];
  int64_t off = 0;
  for (int d = a.krank - 1; d >= 0; d--) {
    uint32_t q, x;
    a.kdiv[d].divmod(k, q, x);
    k = q;
    off += (int64_t)x * a.kstride[d];
  }
  return off;
}

template <typename T>
__device__ __forceinline__ T ld(const char* p) {
  return *(const T*)p;
}

// reinterpretations of loaded 32- / 64-bit words as T
template <typename T>
__device__ __forceinline__ T word32_as(uint32_t u) {
  if constexpr (std::is_same<T, float>::value) return __uint_as_float(u);
  else return (T)(int32_t)u;
}
template <typename T>
__device__ __forceinline__ T word64_as(unsigned long long u) {
  if constexpr (std::is_same<T, double>::value) return __longlong_as_double((long long)u);
  else return (T)(long long)u;
}

__device__ __forceinline__ void store_final(const RedArgs& a, int64_t o, double v, long long vi, bool is_int_sum, long long isum,
                            long long index, uint32_t& st) {
  char* p = a.out + o * dtype_size(a.out_dtype);
  if (a.want_index) {
    if (a.out_dtype == PHCU_I32) *(int32_t*)p = (int32_t)index;
    else *(long long*)p = index;
    return;
  }
  switch (a.out_dtype) {
    case PHCU_F32: *(float*)p = (float)v; break;
    case PHCU_F64: *(double*)p = v; break;
    case PHCU_I32: {
      long long x = is_int_sum ? isum : vi;
      if (x != (int32_t)x) st |= PHCU_ST_OVERFLOW;
      *(int32_t*)p = (int32_t)x;
      break;
    }
    case PHCU_I64: *(long long*)p = is_int_sum ? isum : vi; break;
  }
}

// value of the extremum as (double, long long) for storage
template <typename T>
__device__ __forceinline__ void ext_parts(T v, double& d, long long& l) {
  d = (double)v;
  l = (long long)v;
}

// Finishes one output from its accumulated result (S == 1) or stores a partial.
// An extremum needs the output's first element (the NaN-first rule); a body
// that already loaded it passes it as first_v with known_first set.
template <typename T, int KIND>
__device__ __forceinline__ void finish(const RedArgs& a, int64_t o, int64_t split, const SumAcc<T>& sacc,
                                       const ExtAcc<T>& eacc, uint32_t& st, bool known_first = false,
                                       T first_v = T(0)) {
  if (a.S > 1) {
    Partial& P = a.partial[split * a.O + o];
    if (KIND == RK_SUM) {
      if constexpr (sizeof(T) >= 4 && (std::is_same<T, int32_t>::value || std::is_same<T, long long>::value)) {
        P.v = 0;
        P.i = (long long)sacc.s;
      } else {
        P.v = sacc.value();
        P.i = 0;
        if constexpr (std::is_same<T, float>::value)  // the FP32 pair too, for combine_block
          P.i = (long long)(((unsigned long long)__float_as_uint(sacc.s) << 32) | __float_as_uint(sacc.c));
      }
    } else {
      P.v = (double)eacc.v;
      P.i = eacc.i;
      if constexpr (std::is_same<T, long long>::value) {
        // exact value kept in the index slot's partner: store the int64 bits in v
        P.v = __longlong_as_double((long long)eacc.v);
      }
    }
    return;
  }
  if (KIND == RK_SUM) {
    if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, long long>::value) {
      store_final(a, o, 0, 0, true, (long long)sacc.s, 0, st);
    } else if constexpr (std::is_same<T, float>::value) {
      // s + c rounded once to FP32 (the correctly rounded value of the pair);
      // FP64 conversions cost as much as many loads on this part
      if (a.out_dtype == PHCU_F32 && !a.want_index) *(float*)(a.out + o * 4) = sacc.s + sacc.c;
      else store_final(a, o, sacc.value(), 0, false, 0, 0, st);
    } else {
      store_final(a, o, sacc.value(), 0, false, 0, 0, st);
    }
  } else {
    long long idx = eacc.i;
    T v = eacc.v;
    // first element NaN (or no candidate): the scan never moves off element 0
    const T first = known_first ? first_v : ld<T>(a.in + out_offset(a, (uint32_t)o) * sizeof(T));
    if (idx < 0 || Lim<T>::nan(first)) {
      idx = 0;
      v = first;
    }
    if (a.want_index) {
      store_final(a, o, 0, 0, false, 0, idx, st);
    } else if (std::is_same<T, float>::value && a.out_dtype == PHCU_F32) {
      *(T*)(a.out + o * sizeof(T)) = v;  // the element itself, no conversion
    } else {
      double d;
      long long l;
      ext_parts<T>(v, d, l);
      store_final(a, o, d, l, false, 0, idx, st);
    }
  }
}


// ------------------------------------------------------ per-output bodies
// GROUP: the G lanes of one group reduce elements [k0, k1) of output o; lane 0
// of the group finishes (or stores the partial of split `split`).
template <typename T, int KIND>
__device__ __forceinline__ void group_one_g(const RedArgs& a, int64_t o, int64_t split, const int G, int glane,
                                            unsigned gmask, uint32_t& st) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t k0 = split * a.chunk;
  const int64_t k1 = min(a.K, k0 + a.chunk);
  const char* base = a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T);
  SumAcc<T> sacc;
  ExtAcc<T> eacc;
  sacc.init();
  eacc.init();
  int64_t k = k0 + glane;
  for (; k + 3 * G < k1; k += 4 * G) {  // 4 independent loads in flight per lane
    T x0 = ld<T>(base + k_offset(a, (uint32_t)k) * (int64_t)sizeof(T));
    T x1 = ld<T>(base + k_offset(a, (uint32_t)(k + G)) * (int64_t)sizeof(T));
    T x2 = ld<T>(base + k_offset(a, (uint32_t)(k + 2 * G)) * (int64_t)sizeof(T));
    T x3 = ld<T>(base + k_offset(a, (uint32_t)(k + 3 * G)) * (int64_t)sizeof(T));
    if (KIND == RK_SUM) {
      sacc.add(x0); sacc.add(x1); sacc.add(x2); sacc.add(x3);
    } else {
      eacc.add(x0, k, is_max); eacc.add(x1, k + G, is_max);
      eacc.add(x2, k + 2 * G, is_max); eacc.add(x3, k + 3 * G, is_max);
    }
  }
  for (; k < k1; k += G) {
    T x = ld<T>(base + k_offset(a, (uint32_t)k) * (int64_t)sizeof(T));
    if (KIND == RK_SUM) sacc.add(x);
    else eacc.add(x, k, is_max);
  }
#pragma unroll
  for (int d = G / 2; d >= 1; d >>= 1) {
    if (KIND == RK_SUM) sacc.shfl(d, gmask, G);
    else eacc.shfl(d, gmask, G, is_max);
  }
  if (glane == 0) finish<T, KIND>(a, o, split, sacc, eacc, st);
}

// group_one_g with a compile-time group size (the standalone kernels).
template <typename T, int KIND, int G>
__device__ __forceinline__ void group_one(const RedArgs& a, int64_t o, int64_t split, int glane, unsigned gmask,
                                          uint32_t& st) {
  group_one_g<T, KIND>(a, o, split, G, glane, gmask, st);
}

// GROUP over NO outputs at once (short contiguous axes): each lane keeps NO
// accumulators so NO x 2 loads are in flight per step.
template <typename T, int KIND, int G, int NO>
__device__ __forceinline__ void group_multi(const RedArgs& a, int64_t o0, int64_t split, int glane, unsigned gmask,
                                            uint32_t& st) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t k0 = split * a.chunk;
  const int64_t k1 = min(a.K, k0 + a.chunk);
  const char* base[NO];
  SumAcc<T> sacc[NO];
  ExtAcc<T> eacc[NO];
#pragma unroll
  for (int q = 0; q < NO; q++) {
    const int64_t o = min(o0 + q, a.O - 1);  // past the end: repeat the last output (not stored)
    base[q] = a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T);
    sacc[q].init();
    eacc[q].init();
  }
  int64_t k = k0 + glane;
  for (; k + G < k1; k += 2 * G) {
    const int64_t ka = k_offset(a, (uint32_t)k) * (int64_t)sizeof(T);
    const int64_t kb = k_offset(a, (uint32_t)(k + G)) * (int64_t)sizeof(T);
    T x[NO], y[NO];
#pragma unroll
    for (int q = 0; q < NO; q++) {
      x[q] = ld<T>(base[q] + ka);
      y[q] = ld<T>(base[q] + kb);
    }
#pragma unroll
    for (int q = 0; q < NO; q++) {
      if (KIND == RK_SUM) {
        sacc[q].add(x[q]);
        sacc[q].add(y[q]);
      } else {
        eacc[q].add(x[q], k, is_max);
        eacc[q].add(y[q], k + G, is_max);
      }
    }
  }
  if (k < k1) {
    const int64_t ka = k_offset(a, (uint32_t)k) * (int64_t)sizeof(T);
#pragma unroll
    for (int q = 0; q < NO; q++) {
      const T x = ld<T>(base[q] + ka);
      if (KIND == RK_SUM) sacc[q].add(x);
      else eacc[q].add(x, k, is_max);
    }
  }
#pragma unroll
  for (int q = 0; q < NO; q++) {
#pragma unroll
    for (int d = G / 2; d >= 1; d >>= 1) {
      if (KIND == RK_SUM) sacc[q].shfl(d, gmask, G);
      else eacc[q].shfl(d, gmask, G, is_max);
    }
    if (glane == 0 && o0 + q < a.O) finish<T, KIND>(a, o0 + q, split, sacc[q], eacc[q], st);
  }
}

// 16-byte loads of VN = 16 / sizeof(T) consecutive elements.
template <typename T>
__device__ __forceinline__ void ld16(const char* p, T* x) {
  if constexpr (sizeof(T) == 4) {
    const uint4 v = __ldg((const uint4*)p);
    x[0] = word32_as<T>(v.x);
    x[1] = word32_as<T>(v.y);
    x[2] = word32_as<T>(v.z);
    x[3] = word32_as<T>(v.w);
  } else {
    const ulonglong2 v = __ldg((const ulonglong2*)p);
    x[0] = word64_as<T>(v.x);
    x[1] = word64_as<T>(v.y);
  }
}

// Folds VN consecutive elements (indices k0 .. k0 + VN - 1) into an extremum
// accumulator: the vector's own first extreme (NaNs skipped, strict
// comparison, so ties keep the lower index) is found with a 32-bit local
// index, then offered to the accumulator once; since the accumulator only
// holds lower indices, this equals offering the elements one by one.
template <typename T, int VN>
__device__ __forceinline__ void vec_extreme_into(ExtAcc<T>& acc, const T* x, int64_t k0, bool is_max) {
  T bv = x[0];
  int be = Lim<T>::nan(x[0]) ? -1 : 0;
#pragma unroll
  for (int e = 1; e < VN; e++) {
    const bool take = !Lim<T>::nan(x[e]) && (be < 0 || (is_max ? (x[e] > bv) : (x[e] < bv)));
    bv = take ? x[e] : bv;
    be = take ? e : be;
  }
  if (be >= 0) acc.add(bv, k0 + be, is_max);
}

// Folds U vectors of VN elements of 4-byte type (element (u, e) at index
// k + u * stride + e, so increasing (u, e) is increasing index) into an
// extremum accumulator: the extreme value m over the non-NaN elements (one
// min/max per element), then the first element equal to m (a compare and a
// select per element), offered to the accumulator once.  That element is the
// one a strict-comparison scan skipping NaNs keeps.  Its value is m itself,
// except for zeros, whose sign is taken from the element found.
template <typename T, int U, int VN>
__device__ __forceinline__ void block_extreme_into(ExtAcc<T>& acc, const T (&x)[U][VN], int64_t k, int64_t stride,
                                                   bool is_max) {
  T m = x[0][0];
#pragma unroll
  for (int t = 1; t < U * VN; t++) m = Lim<T>::ext(m, x[t / VN][t % VN], is_max);
  int j = -1;
#pragma unroll
  for (int t = U * VN - 1; t >= 0; t--) j = (x[t / VN][t % VN] == m) ? t : j;
  if (j < 0) return;  // every element NaN
  T val = m;
  if (m == (T)0) {
#pragma unroll
    for (int t = 0; t < U * VN; t++)
      if (t == j) val = x[t / VN][t % VN];
  }
  acc.add(val, k + (int64_t)(j / VN) * stride + (j % VN), is_max);
}

// Folds output e of NF vectors loaded at consecutive reduced positions
// k .. k + NF - 1 (x[j][e] is element k + j of output e) into its extremum
// accumulator: the extreme m over the non-NaN elements, then the first j with
// x[j][e] == m, offered once (zeros take their sign from that element), which
// is what a strict-comparison scan skipping NaNs keeps.
template <typename T, int NF, int VN>
__device__ __forceinline__ void column_extreme_into(ExtAcc<T>& acc, const T (&x)[NF][VN], int e, int64_t k,
                                                    bool is_max) {
  T m = x[0][e];
#pragma unroll
  for (int j = 1; j < NF; j++) m = Lim<T>::ext(m, x[j][e], is_max);
  int jj = -1;
#pragma unroll
  for (int j = NF - 1; j >= 0; j--) jj = (x[j][e] == m) ? j : jj;
  if (jj < 0) return;  // every element NaN
  T val = m;
  if (m == (T)0) {
#pragma unroll
    for (int j = 0; j < NF; j++)
      if (j == jj) val = x[j][e];
  }
  acc.add(val, k + jj, is_max);
}

// GROUP with 16-byte loads along a contiguous reduced axis: lane l of a group
// of G reads vectors l, l + G, l + 2G, ... of each of NO outputs (elements of
// one accumulator arrive in increasing k), then the < VN elements past the last
// whole vector one per lane.  Requires: the reduced axis is one axis of unit
// stride; every output row and every split starts 16-byte aligned.
template <typename T, int KIND, int G, int NO>
__device__ __forceinline__ void group_vec(const RedArgs& a, int64_t o0, int64_t split, int glane, unsigned gmask,
                                          uint32_t& st) {
  constexpr int VN = 16 / sizeof(T);
  constexpr int U = NO <= 2 ? 4 : 1;  // vectors in flight per output and lane
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t k0 = split * a.chunk;
  const int64_t k1 = min(a.K, k0 + a.chunk);
  const int64_t kv1 = k0 + (k1 - k0) / VN * VN;  // end of the whole vectors
  const char* base[NO];
  SumAcc<T> sacc[NO];
  ExtAcc<T> eacc[NO];
#pragma unroll
  for (int q = 0; q < NO; q++) {
    const int64_t o = min(o0 + q, a.O - 1);  // past the end: repeat the last output (not stored)
    base[q] = a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T);
    sacc[q].init();
    eacc[q].init();
  }
  int64_t k = k0 + (int64_t)glane * VN;
  for (; k + (int64_t)(U - 1) * G * VN + VN <= kv1; k += (int64_t)U * G * VN) {
    T x[NO][U][VN];
#pragma unroll
    for (int q = 0; q < NO; q++)
#pragma unroll
      for (int u = 0; u < U; u++) ld16<T>(base[q] + (k + (int64_t)u * G * VN) * (int64_t)sizeof(T), x[q][u]);
#pragma unroll
    for (int q = 0; q < NO; q++) {
      if constexpr (KIND != RK_SUM && sizeof(T) == 4) {
        block_extreme_into<T, U, VN>(eacc[q], x[q], k, (int64_t)G * VN, is_max);
      } else {
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (KIND == RK_SUM) {
#pragma unroll
            for (int e = 0; e < VN; e++) sacc[q].add(x[q][u][e]);
          } else {
            vec_extreme_into<T, VN>(eacc[q], x[q][u], k + (int64_t)u * G * VN, is_max);
          }
        }
      }
    }
  }
  for (; k + VN <= kv1; k += (int64_t)G * VN) {
#pragma unroll
    for (int q = 0; q < NO; q++) {
      T x[VN];
      ld16<T>(base[q] + k * (int64_t)sizeof(T), x);
      if (KIND == RK_SUM) {
#pragma unroll
        for (int e = 0; e < VN; e++) sacc[q].add(x[e]);
      } else {
        vec_extreme_into<T, VN>(eacc[q], x, k, is_max);
      }
    }
  }
  const int64_t kt = kv1 + glane;  // the tail: one element per lane
  if (kt < k1) {
#pragma unroll
    for (int q = 0; q < NO; q++) {
      const T x = ld<T>(base[q] + kt * (int64_t)sizeof(T));
      if (KIND == RK_SUM) sacc[q].add(x);
      else eacc[q].add(x, kt, is_max);
    }
  }
#pragma unroll
  for (int q = 0; q < NO; q++) {
#pragma unroll
    for (int d = G / 2; d >= 1; d >>= 1) {
      if (KIND == RK_SUM) sacc[q].shfl(d, gmask, G);
      else eacc[q].shfl(d, gmask, G, is_max);
    }
    if (glane == 0 && o0 + q < a.O) finish<T, KIND>(a, o0 + q, split, sacc[q], eacc[q], st);
  }
}

// COLUMN with 16-byte loads across outputs: one thread reduces VN consecutive
// outputs o0 .. o0 + VN - 1, which are consecutive in memory (the innermost
// kept axis has unit stride and a length divisible by VN), eight reduced
// positions in flight (four: 2-7% slower for extrema and 4-7% for sums on
// 64x128x128x64, axes 0-2; sixteen: slower for sums).  Requires every output
// row start and every reduced stride to be 16-byte aligned.
constexpr int COL_INFLIGHT = 8;

template <typename T, int KIND>
__device__ __forceinline__ void column_vec(const RedArgs& a, int64_t o0, int64_t split, uint32_t& st) {
  constexpr int VN = 16 / sizeof(T);
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t k0 = split * a.chunk;
  const int64_t k1 = min(a.K, k0 + a.chunk);
  const char* base = a.in + out_offset(a, (uint32_t)o0) * (int64_t)sizeof(T);
  SumAcc<T> sacc[VN];
  ExtAcc<T> eacc[VN];
#pragma unroll
  for (int e = 0; e < VN; e++) {
    sacc[e].init();
    eacc[e].init();
  }
  // element k = 0 of each output, kept from the first batch of split 0 so
  // that finishing an extremum needs no further load
  T first[VN] = {};
  bool have_first = false;
  int64_t k = k0;
  if (a.krank == 1) {
    const int64_t ks = a.kinner * (int64_t)sizeof(T);
    const char* p = base + k0 * ks;
    constexpr int NF = COL_INFLIGHT;
    for (; k + NF - 1 < k1; k += NF, p += NF * ks) {
      T x[NF][VN];
#pragma unroll
      for (int j = 0; j < NF; j++) ld16<T>(p + j * ks, x[j]);
      if constexpr (KIND != RK_SUM) {
        if (k == 0) {
#pragma unroll
          for (int e = 0; e < VN; e++) first[e] = x[0][e];
          have_first = true;
        }
      }
      if constexpr (KIND != RK_SUM && sizeof(T) == 4) {
#pragma unroll
        for (int e = 0; e < VN; e++) column_extreme_into<T, NF, VN>(eacc[e], x, e, k, is_max);
      } else {
#pragma unroll
        for (int j = 0; j < NF; j++)
#pragma unroll
          for (int e = 0; e < VN; e++) {
            if (KIND == RK_SUM) sacc[e].add(x[j][e]);
            else eacc[e].add(x[j][e], k + j, is_max);
          }
      }
    }
    for (; k < k1; k++, p += ks) {
      T x[VN];
      ld16<T>(p, x);
#pragma unroll
      for (int e = 0; e < VN; e++) {
        if (KIND == RK_SUM) sacc[e].add(x[e]);
        else eacc[e].add(x[e], k, is_max);
      }
    }
  } else {
    for (; k < k1; k++) {
      T x[VN];
      ld16<T>(base + k_offset(a, (uint32_t)k) * (int64_t)sizeof(T), x);
#pragma unroll
      for (int e = 0; e < VN; e++) {
        if (KIND == RK_SUM) sacc[e].add(x[e]);
        else eacc[e].add(x[e], k, is_max);
      }
    }
  }
#pragma unroll
  for (int e = 0; e < VN; e++) finish<T, KIND>(a, o0 + e, split, sacc[e], eacc[e], st, have_first, first[e]);
}

// SLAB: the reduced axis sits directly outside the innermost kept axis and
// the two form one contiguous slab of K rows of L elements (L * K elements
// per slab, one slab per value of the outer kept axes).  The block reads a
// slab front to back: thread t takes vector t % LV of each row (LV = L / VN)
// and rows t / LV, t / LV + RPI, ... (RPI = 256 / LV), eight in flight, so a
// warp's loads cover whole rows and the block's 4 KB in a row.  Row partials
// meet in shared memory, where thread l < L folds those of output l in row
// order and finishes it.  Needs a.S == 1 and LV a power of two <= 256.
constexpr int SLAB_THREADS = 256;
template <typename T, int KIND>
using SlabAcc = typename std::conditional<KIND == RK_SUM, SumAcc<T>, ExtAcc<T>>::type;

template <typename T, int KIND>
__device__ __forceinline__ void column_slab(const RedArgs& a, int64_t slab, int L, SlabAcc<T, KIND>* sh, uint32_t& st) {
  constexpr int VN = 16 / sizeof(T);
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int LV = L / VN, RPI = SLAB_THREADS / LV;
  const int lv = threadIdx.x % LV, rr = threadIdx.x / LV;
  const int64_t o0 = slab * L;
  const char* base = a.in + (out_offset(a, (uint32_t)o0) + (int64_t)lv * VN) * (int64_t)sizeof(T);
  const int64_t rs = (int64_t)L * sizeof(T);  // bytes per row
  SlabAcc<T, KIND> acc[VN];
#pragma unroll
  for (int e = 0; e < VN; e++) acc[e].init();
  int64_t k = rr;
  for (; k + (int64_t)(COL_INFLIGHT - 1) * RPI < a.K; k += (int64_t)COL_INFLIGHT * RPI) {
    T x[COL_INFLIGHT][VN];
#pragma unroll
    for (int j = 0; j < COL_INFLIGHT; j++) ld16<T>(base + (k + (int64_t)j * RPI) * rs, x[j]);
#pragma unroll
    for (int j = 0; j < COL_INFLIGHT; j++)
#pragma unroll
      for (int e = 0; e < VN; e++) {
        if constexpr (KIND == RK_SUM) acc[e].add(x[j][e]);
        else acc[e].add(x[j][e], k + (int64_t)j * RPI, is_max);
      }
  }
  for (; k < a.K; k += RPI) {
    T x[VN];
    ld16<T>(base + k * rs, x);
#pragma unroll
    for (int e = 0; e < VN; e++) {
      if constexpr (KIND == RK_SUM) acc[e].add(x[e]);
      else acc[e].add(x[e], k, is_max);
    }
  }
  // partial of row set rr for output lv * VN + e at sh[rr * L + lv * VN + e]
#pragma unroll
  for (int e = 0; e < VN; e++) sh[rr * L + lv * VN + e] = acc[e];
  __syncthreads();
  for (int l = threadIdx.x; l < L; l += SLAB_THREADS) {
    SlabAcc<T, KIND> r = sh[l];
    for (int j = 1; j < RPI; j++) {
      if constexpr (KIND == RK_SUM) r.merge(sh[j * L + l]);
      else r.merge(sh[j * L + l], is_max);
    }
    SumAcc<T> sacc;
    ExtAcc<T> eacc;
    if constexpr (KIND == RK_SUM) {
      sacc = r;
      eacc.init();
    } else {
      eacc = r;
      sacc.init();
    }
    finish<T, KIND>(a, o0 + l, 0, sacc, eacc, st);
  }
  __syncthreads();
}

// COLUMN: one thread reduces elements [k0, k1) of output o.
template <typename T, int KIND>
__device__ __forceinline__ void column_one(const RedArgs& a, int64_t o, int64_t split, uint32_t& st) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t k0 = split * a.chunk;
  const int64_t k1 = min(a.K, k0 + a.chunk);
  const char* base = a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T);
  const int64_t ks = a.kinner * (int64_t)sizeof(T);
  SumAcc<T> sacc;
  ExtAcc<T> eacc;
  sacc.init();
  eacc.init();
  int64_t k = k0;
  if (a.krank == 1) {
    const char* p = base + k0 * ks;
    for (; k + 3 < k1; k += 4, p += 4 * ks) {
      T x0 = ld<T>(p), x1 = ld<T>(p + ks), x2 = ld<T>(p + 2 * ks), x3 = ld<T>(p + 3 * ks);
      if (KIND == RK_SUM) {
        sacc.add(x0); sacc.add(x1); sacc.add(x2); sacc.add(x3);
      } else {
        eacc.add(x0, k, is_max); eacc.add(x1, k + 1, is_max);
        eacc.add(x2, k + 2, is_max); eacc.add(x3, k + 3, is_max);
      }
    }
    for (; k < k1; k++, p += ks) {
      T x = ld<T>(p);
      if (KIND == RK_SUM) sacc.add(x);
      else eacc.add(x, k, is_max);
    }
  } else {
    for (; k < k1; k++) {
      T x = ld<T>(base + k_offset(a, (uint32_t)k) * (int64_t)sizeof(T));
      if (KIND == RK_SUM) sacc.add(x);
      else eacc.add(x, k, is_max);
    }
  }
  finish<T, KIND>(a, o, split, sacc, eacc, st);
}

// Folds the S partials of output o in split order (FP64 for sums) and stores it.
template <typename T, int KIND>
__device__ __forceinline__ void combine_one(const RedArgs& a, int64_t o, uint32_t& st) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  if (KIND == RK_SUM) {
    if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, long long>::value) {
      long long s = 0;
      for (int64_t j = 0; j < a.S; j++)
        s = (long long)((unsigned long long)s + (unsigned long long)a.partial[j * a.O + o].i);
      store_final(a, o, 0, 0, true, s, 0, st);
    } else {
      double s = 0.0, c = 0.0;
      for (int64_t j = 0; j < a.S; j++) {
        double x = a.partial[j * a.O + o].v;
        double t = s + x;
        if (fabs(s) >= fabs(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
      }
      store_final(a, o, s + c, 0, false, 0, 0, st);
    }
  } else {
    ExtAcc<T> e;
    e.init();
    for (int64_t j = 0; j < a.S; j++) {
      const Partial& P = a.partial[j * a.O + o];
      ExtAcc<T> q;
      if constexpr (std::is_same<T, long long>::value) q.v = __double_as_longlong(P.v);
      else q.v = (T)P.v;
      q.i = P.i;
      e.merge(q, is_max);
    }
    long long idx = e.i;
    T v = e.v;
    const T first = ld<T>(a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T));
    if (idx < 0 || Lim<T>::nan(first)) {
      idx = 0;
      v = first;
    }
    if (a.want_index) {
      store_final(a, o, 0, 0, false, 0, idx, st);
    } else if (std::is_same<T, float>::value && a.out_dtype == PHCU_F32) {
      *(T*)(a.out + o * sizeof(T)) = v;  // the element itself, no conversion
    } else {
      double d;
      long long l;
      ext_parts<T>(v, d, l);
      store_final(a, o, d, l, false, 0, idx, st);
    }
  }
}

// Shared scratch of combine_block (one per block, provided by the kernel).
struct CombineScratch {
  double v[256];
  double c[256];
  long long i[256];
};

// All threads of the block fold the S partials of output o (power-of-two
// blockDim <= 256; every thread must call it).  Thread t folds partials
// t, t + blockDim, ... in order; the per-thread results are merged in a fixed
// tree, so the result does not depend on timing.  Thread 0 stores.
template <typename T, int KIND>
__device__ __forceinline__ void combine_block(const RedArgs& a, int64_t o, CombineScratch& cs, uint32_t& st) {
  double* sh_v = cs.v;
  double* sh_c = cs.c;
  long long* sh_i = cs.i;
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int t = threadIdx.x, nt = blockDim.x;
  constexpr bool INT = std::is_same<T, int32_t>::value || std::is_same<T, long long>::value;
  if (KIND == RK_SUM && INT) {
    long long s = 0;
    for (int64_t j = t; j < a.S; j += nt) s = (long long)((unsigned long long)s + (unsigned long long)a.partial[j * a.O + o].i);
    sh_i[t] = s;
    __syncthreads();
    for (int w = nt / 2; w >= 1; w >>= 1) {
      if (t < w) sh_i[t] = (long long)((unsigned long long)sh_i[t] + (unsigned long long)sh_i[t + w]);
      __syncthreads();
    }
    if (t == 0) store_final(a, o, 0, 0, true, sh_i[0], 0, st);
  } else if (KIND == RK_SUM && std::is_same<T, float>::value) {
    // Float32 partials carry their (sum, compensation) pair: fold them as
    // double-float values with FP32 TwoSum (FP64 throughput would make this
    // one block the slowest part of a full reduction)
    float* sv = reinterpret_cast<float*>(sh_v);
    float* sc = reinterpret_cast<float*>(sh_c);
    float s = 0.f, c = 0.f;
    auto fold = [&](unsigned long long w) {
      const float ps = __uint_as_float((uint32_t)(w >> 32)), pc = __uint_as_float((uint32_t)w);
      const float u = s + ps;
      const float bp = u - s;
      const float e = (s - (u - bp)) + (ps - bp);
      s = u;
      c = (c + pc) + e;
    };
    int64_t j = t;
    for (; j + 3 * nt < a.S; j += 4 * nt) {  // four loads in flight, folded in order
      unsigned long long w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) w[q] = (unsigned long long)a.partial[(j + q * nt) * a.O + o].i;
#pragma unroll
      for (int q = 0; q < 4; q++) fold(w[q]);
    }
    for (; j < a.S; j += nt) fold((unsigned long long)a.partial[j * a.O + o].i);
    sv[t] = s;
    sc[t] = c;
    __syncthreads();
    for (int w = nt / 2; w >= 1; w >>= 1) {
      if (t < w) {
        const float x = sv[t], y = sv[t + w];
        const float u = x + y;
        const float bp = u - x;
        const float e = (x - (u - bp)) + (y - bp);
        sv[t] = u;
        sc[t] = (sc[t] + sc[t + w]) + e;
      }
      __syncthreads();
    }
    if (t == 0) store_final(a, o, (double)sv[0] + (double)sc[0], 0, false, 0, 0, st);
  } else if (KIND == RK_SUM) {
    double s = 0.0, c = 0.0;
    for (int64_t j = t; j < a.S; j += nt) {
      const double x = a.partial[j * a.O + o].v;
      const double u = s + x;
      if (fabs(s) >= fabs(x)) c += (s - u) + x;
      else c += (x - u) + s;
      s = u;
    }
    sh_v[t] = s;
    sh_c[t] = c;
    __syncthreads();
    for (int w = nt / 2; w >= 1; w >>= 1) {
      if (t < w) {
        const double x = sh_v[t], y = sh_v[t + w];
        const double u = x + y;
        const double bp = u - x;
        const double e = (x - (u - bp)) + (y - bp);
        sh_v[t] = u;
        sh_c[t] = (sh_c[t] + sh_c[t + w]) + e;
      }
      __syncthreads();
    }
    if (t == 0) store_final(a, o, sh_v[0] + sh_c[0], 0, false, 0, 0, st);
  } else {
    ExtAcc<T> e;
    e.init();
    for (int64_t j = t; j < a.S; j += nt) {
      const Partial& P = a.partial[j * a.O + o];
      ExtAcc<T> q;
      if constexpr (std::is_same<T, long long>::value) q.v = __double_as_longlong(P.v);
      else q.v = (T)P.v;
      q.i = P.i;
      e.merge(q, is_max);
    }
    if constexpr (std::is_same<T, long long>::value) sh_v[t] = __longlong_as_double(e.v);
    else sh_v[t] = (double)e.v;
    sh_i[t] = e.i;
    __syncthreads();
    for (int w = nt / 2; w >= 1; w >>= 1) {
      if (t < w) {
        ExtAcc<T> x, y;
        if constexpr (std::is_same<T, long long>::value) {
          x.v = __double_as_longlong(sh_v[t]);
          y.v = __double_as_longlong(sh_v[t + w]);
        } else {
          x.v = (T)sh_v[t];
          y.v = (T)sh_v[t + w];
        }
        x.i = sh_i[t];
        y.i = sh_i[t + w];
        x.merge(y, is_max);
        if constexpr (std::is_same<T, long long>::value) sh_v[t] = __longlong_as_double(x.v);
        else sh_v[t] = (double)x.v;
        sh_i[t] = x.i;
      }
      __syncthreads();
    }
    if (t == 0) {
      long long idx = sh_i[0];
      T v;
      if constexpr (std::is_same<T, long long>::value) v = __double_as_longlong(sh_v[0]);
      else v = (T)sh_v[0];
      const T first = ld<T>(a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T));
      if (idx < 0 || Lim<T>::nan(first)) {
        idx = 0;
        v = first;
      }
      double d;
      long long l;
      ext_parts<T>(v, d, l);
      store_final(a, o, d, l, false, 0, idx, st);
    }
  }
  __syncthreads();
}

// Host planning of one reduction (shared with the batched executor): fills
// `a` (without scratch) and picks the launch shape.  Returns PHCU_OK, or an
// error; *trivial is set when nothing needs to run (no outputs) and *empty_sum
// when the output must be zero-filled (sum over an empty axis).
struct RedShape {
  int mode;  // 0 = GROUP, 1 = COLUMN
  int G;
  int vec;   // 1: 16-byte loads (group_vec / column_vec)
};
int32_t plan_reduce(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out, int64_t target_threads,
                    RedArgs* a, RedShape* shape, bool* trivial, bool* empty_sum);

}  // namespace phcu
