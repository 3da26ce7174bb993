// reduce.cu -- sum / max / min / argmax / argmin along an axis or over all elements.
//
// Semantics (the reference reaches them through Enumerable, src/multi_indexable.cr:18,
// 656-658, the slices(axis) fold :742-786 and the argmax idiom README.md:56-61):
//  * output element o folds the elements along the axis in increasing index order;
//  * max/min keep the first extreme element (strict > / <), so ties resolve to the
//    lowest index and a NaN never wins unless it is the first element;
//  * Float32 sums are compensated: each thread runs Neumaier's summation in FP32,
//    lanes combine their (sum, compensation) pairs with TwoSum in FP32, and partial
//    results of different blocks are combined in FP64 (the only FP64 arithmetic).
//
// Two launch shapes:
//  GROUP  -- a group of G lanes (G = 4..32) cooperates on one output; lanes read
//            consecutive elements of the reduced axis (that axis is the contiguous one).
//  COLUMN -- one thread per output; consecutive threads own consecutive outputs, which
//            are consecutive in memory, and each thread walks the reduced axis.
// When there are too few outputs to fill the GPU the reduced axis is split into S
// pieces; the pieces' partials go to scratch and a combine kernel folds them in order.
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
};
template <>
struct Lim<double> {
  static __device__ __forceinline__ bool nan(double x) { return x != x; }
};
template <>
struct Lim<int32_t> {
  static __device__ __forceinline__ bool nan(int32_t) { return false; }
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
  __device__ __forceinline__ void add(T x, long long k, bool is_max) {
    if (Lim<T>::nan(x)) return;
    if (better(x, k, v, i, is_max)) { v = x; i = k; }
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

__device__ void store_final(const RedArgs& a, int64_t o, double v, long long vi, bool is_int_sum, long long isum,
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
template <typename T, int KIND>
__device__ __forceinline__ void finish(const RedArgs& a, int64_t o, int64_t split, const SumAcc<T>& sacc,
                                       const ExtAcc<T>& eacc, uint32_t& st) {
  if (a.S > 1) {
    Partial& P = a.partial[split * a.O + o];
    if (KIND == RK_SUM) {
      if constexpr (sizeof(T) >= 4 && (std::is_same<T, int32_t>::value || std::is_same<T, long long>::value)) {
        P.v = 0;
        P.i = (long long)sacc.s;
      } else {
        P.v = sacc.value();
        P.i = 0;
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
    } else {
      store_final(a, o, sacc.value(), 0, false, 0, 0, st);
    }
  } else {
    long long idx = eacc.i;
    T v = eacc.v;
    // first element NaN (or no candidate): the scan never moves off element 0
    const T first = ld<T>(a.in + out_offset(a, (uint32_t)o) * sizeof(T));
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

// ---------------------------------------------------------- GROUP kernel
template <typename T, int KIND, int G>
__global__ void __launch_bounds__(256) reduce_group_kernel(const __grid_constant__ RedArgs a) {
  const int lane = threadIdx.x & 31;
  const int glane = lane & (G - 1);
  const int gid_in_block = threadIdx.x / G;
  const int groups_per_block = blockDim.x / G;
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  uint32_t st = 0;
  const int64_t nwork = a.O * a.S;
  for (int64_t w = (int64_t)blockIdx.x * groups_per_block + gid_in_block; w < nwork;
       w += (int64_t)gridDim.x * groups_per_block) {
    const int64_t o = w % a.O;
    const int64_t split = w / a.O;
    const int64_t k0 = split * a.chunk;
    const int64_t k1 = min(a.K, k0 + a.chunk);
    const char* base = a.in + out_offset(a, (uint32_t)o) * (int64_t)sizeof(T);
    SumAcc<T> sacc;
    ExtAcc<T> eacc;
    sacc.init();
    eacc.init();
    int64_t k = k0 + glane;
    // 4 independent loads in flight per lane
    for (; k + 3 * G < k1; k += 4 * G) {
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
  if (st) atomicOr(a.status, st);
}

// --------------------------------------------------------- COLUMN kernel
template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_column_kernel(const __grid_constant__ RedArgs a) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  uint32_t st = 0;
  const int64_t nwork = a.O * a.S;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = w % a.O;
    const int64_t split = w / a.O;
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
  if (st) atomicOr(a.status, st);
}

// --------------------------------------------------------- combine kernel
// Folds the S partials of every output in split order (FP64 for sums).
template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_combine_kernel(const __grid_constant__ RedArgs a) {
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  uint32_t st = 0;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < a.O; o += (int64_t)gridDim.x * blockDim.x) {
    if (KIND == RK_SUM) {
      if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, long long>::value) {
        long long s = 0;
        for (int64_t j = 0; j < a.S; j++) s = (long long)((unsigned long long)s + (unsigned long long)a.partial[j * a.O + o].i);
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
      double d;
      long long l;
      ext_parts<T>(v, d, l);
      store_final(a, o, d, l, false, 0, idx, st);
    }
  }
  if (st) atomicOr(a.status, st);
}

// --------------------------------------------------------------- launch
template <typename T, int KIND>
static int32_t launch_typed(RedArgs& a, int mode, int G) {
  Context& c = ctx();
  const int threads = 256;
  int64_t work_threads = (mode == 0) ? a.O * a.S * G : a.O * a.S;
  int64_t blocks = (work_threads + threads - 1) / threads;
  int64_t cap = (int64_t)c.sm_count * 8 * 4;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (mode == 0) {
    switch (G) {
      case 32: reduce_group_kernel<T, KIND, 32><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 16: reduce_group_kernel<T, KIND, 16><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 8: reduce_group_kernel<T, KIND, 8><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      default: reduce_group_kernel<T, KIND, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
    }
  } else {
    reduce_column_kernel<T, KIND><<<(unsigned)blocks, threads, 0, c.stream>>>(a);
  }
  count_launch();
  PHCU_TRY(check_launch("reduce kernel"));
  if (a.S > 1) {
    int64_t cb = (a.O + threads - 1) / threads;
    if (cb > cap) cb = cap;
    reduce_combine_kernel<T, KIND><<<(unsigned)cb, threads, 0, c.stream>>>(a);
    count_launch();
    PHCU_TRY(check_launch("reduce combine kernel"));
  }
  return PHCU_OK;
}

template <typename T>
static int32_t launch_kind(RedArgs& a, int mode, int G) {
  if (a.op == PHCU_RED_SUM) return launch_typed<T, RK_SUM>(a, mode, G);
  return launch_typed<T, RK_EXT>(a, mode, G);
}

// Plans and launches a reduction.  `partial_buf` (optional) is caller-provided
// scratch of `partial_cap` Partials; when null, scratch comes from the pool.
int32_t reduce_impl(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out, void* partial_buf,
                    size_t partial_cap) {
  PHCU_TRY(require_ctx());
  PHCU_TRY(check_view(in, "reduce input"));
  PHCU_TRY(check_view(out, "reduce output"));
  if (op < PHCU_RED_SUM || op > PHCU_RED_ARGMIN) return fail(PHCU_ERR_INVALID, "unknown reduction %d", op);
  const int t = in->dtype;
  if (t == PHCU_BOOL) return fail(PHCU_ERR_UNSUPPORTED, "reductions of Bool arrays are not defined");
  const bool want_index = (op == PHCU_RED_ARGMAX || op == PHCU_RED_ARGMIN);
  if (want_index) {
    if (out->dtype != PHCU_I32 && out->dtype != PHCU_I64)
      return fail(PHCU_ERR_INVALID, "argmax/argmin output must be Int32 or Int64");
  } else if (op == PHCU_RED_SUM) {
    bool ok = is_float_t(t) ? is_float_t(out->dtype) : is_int_t(out->dtype);
    if (!ok) return fail(PHCU_ERR_INVALID, "sum output dtype %d does not suit input dtype %d", out->dtype, t);
  } else if (out->dtype != t) {
    return fail(PHCU_ERR_INVALID, "max/min output dtype must equal the input dtype");
  }
  if (axis >= in->rank) return fail(PHCU_ERR_INDEX, "axis %d is not present in a %d-dimensional array", axis, in->rank);

  RedArgs a;
  memset(&a, 0, sizeof(a));
  const int es = dtype_size(t);
  a.in = (const char*)in->base + in->offset * es;
  a.dtype = t;
  a.op = op;
  a.want_index = want_index;
  a.out_dtype = out->dtype;
  a.out = (char*)out->base + out->offset * dtype_size(out->dtype);
  a.status = ctx().status;

  // kept axes and reduced axes
  int64_t osh[MAXR], ost[MAXR], ksh[MAXR], kst[MAXR];
  int orank = 0, krank = 0;
  int64_t O = 1, K = 1;
  for (int i = 0; i < in->rank; i++) {
    bool reduced = axis < 0 || i == axis;
    if (reduced) {
      ksh[krank] = in->shape[i];
      kst[krank] = in->stride[i];
      krank++;
      K *= in->shape[i];
    } else {
      osh[orank] = in->shape[i];
      ost[orank] = in->stride[i];
      orank++;
      O *= in->shape[i];
    }
  }
  if (in->rank == 0) {  // a rank-0 descriptor holds one element
    ksh[0] = 1;
    kst[0] = 0;
    krank = 1;
  }
  const int64_t out_n = (axis < 0) ? 1 : O;
  if (view_size(out) != out_n)
    return fail(PHCU_ERR_SHAPE, "reduction output has %lld elements, expected %lld", (long long)view_size(out),
                (long long)out_n);
  if (O == 0) return PHCU_OK;
  if (K == 0) {
    if (op != PHCU_RED_SUM) return fail(PHCU_ERR_EMPTY, "Empty enumerable");
    // sum of nothing: zeros
    phcu_scalar_t z;
    memset(&z, 0, sizeof(z));
    z.dtype = out->dtype;
    return phcu_fill(out, &z);
  }
  // merge kept axes (drop 1s; merge contiguous neighbours; order kept = lexicographic)
  {
    int r = 0;
    int64_t s2[MAXR], t2[MAXR];
    for (int i = 0; i < orank; i++) {
      if (osh[i] == 1) continue;
      if (r > 0 && t2[r - 1] == ost[i] * osh[i]) {
        s2[r - 1] *= osh[i];
        t2[r - 1] = ost[i];
        continue;
      }
      s2[r] = osh[i];
      t2[r] = ost[i];
      r++;
    }
    orank = r;
    for (int i = 0; i < r; i++) { osh[i] = s2[i]; ost[i] = t2[i]; }
  }
  // reduced axes: order is free for sums/max/min values; argmax needs lexicographic indices
  {
    int r = 0;
    int64_t s2[MAXR], t2[MAXR];
    for (int i = 0; i < krank; i++) {
      if (ksh[i] == 1 && krank > 1) continue;
      if (r > 0 && t2[r - 1] == kst[i] * ksh[i]) {
        s2[r - 1] *= ksh[i];
        t2[r - 1] = kst[i];
        continue;
      }
      s2[r] = ksh[i];
      t2[r] = kst[i];
      r++;
    }
    if (r == 0) { s2[0] = 1; t2[0] = 0; r = 1; }
    krank = r;
    for (int i = 0; i < r; i++) { ksh[i] = s2[i]; kst[i] = t2[i]; }
  }
  a.orank = orank;
  a.O = O;
  for (int i = 0; i < orank; i++) {
    a.oshape[i] = osh[i];
    a.ostride[i] = ost[i];
    a.odiv[i].init((uint32_t)osh[i]);
  }
  a.krank = krank;
  a.K = K;
  for (int i = 0; i < krank; i++) {
    a.kshape[i] = ksh[i];
    a.kstride[i] = kst[i];
    a.kdiv[i].init((uint32_t)ksh[i]);
  }
  a.kinner = kst[krank - 1];

  // launch shape
  Context& c = ctx();
  const int64_t target = (int64_t)c.sm_count * 1024;
  const int64_t inner_out_stride = orank > 0 ? ost[orank - 1] : 0;
  int mode;  // 0 = GROUP, 1 = COLUMN
  int G = 32;
  const bool k_contig = (kst[krank - 1] == 1 || kst[krank - 1] == -1);
  if (orank > 0 && (inner_out_stride == 1 || inner_out_stride == -1) && !(k_contig && O < target / 8)) {
    mode = 1;
  } else {
    mode = 0;
    int64_t per = K / 4;  // elements per lane >= 4
    G = 32;
    while (G > 4 && G > per) G >>= 1;
  }
  int64_t S = 1;
  const int64_t tpw = (mode == 0) ? G : 1;
  if (O * tpw < target) {
    S = (target + O * tpw - 1) / (O * tpw);
    int64_t min_chunk = (mode == 0) ? (int64_t)G * 16 : 32;
    int64_t smax = (K + min_chunk - 1) / min_chunk;
    if (S > smax) S = smax;
    if (S < 1) S = 1;
  }
  a.S = S;
  a.chunk = (K + S - 1) / S;
  a.S = (K + a.chunk - 1) / a.chunk;
  S = a.S;
  void* scratch = nullptr;
  if (S > 1) {
    size_t need = (size_t)S * (size_t)O;
    if (partial_buf) {
      if (need > partial_cap)
        return fail(PHCU_ERR_INVALID, "reduction needs %zu partials, scratch holds %zu", need, partial_cap);
      a.partial = (Partial*)partial_buf;
    } else {
      PHCU_TRY(scratch_alloc(need * sizeof(Partial), &scratch));
      a.partial = (Partial*)scratch;
    }
  }
  int32_t rc;
  switch (t) {
    case PHCU_F32: rc = launch_kind<float>(a, mode, G); break;
    case PHCU_F64: rc = launch_kind<double>(a, mode, G); break;
    case PHCU_I32: rc = launch_kind<int32_t>(a, mode, G); break;
    default: rc = launch_kind<long long>(a, mode, G); break;
  }
  if (scratch) scratch_free(scratch);
  return rc;
}

}  // namespace phcu

using namespace phcu;

extern "C" int32_t phcu_reduce(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out) {
  return reduce_impl(op, in, axis, out, nullptr, 0);
}
