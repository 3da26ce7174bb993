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
#include <algorithm>

#include "async_copy.cuh"
#include "reduce_device.cuh"

namespace phcu {

template <typename T, int KIND, int G>
__global__ void __launch_bounds__(256) reduce_group_kernel(const __grid_constant__ RedArgs a) {
  const int lane = threadIdx.x & 31;
  const int glane = lane & (G - 1);
  const int groups_per_block = blockDim.x / G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  uint32_t st = 0;
  const int64_t nwork = a.O * a.S;
  for (int64_t w = (int64_t)blockIdx.x * groups_per_block + threadIdx.x / G; w < nwork;
       w += (int64_t)gridDim.x * groups_per_block)
    group_one<T, KIND, G>(a, w % a.O, w / a.O, glane, gmask, st);
  if (st) atomicOr(a.status, st);
}

// GROUP over four outputs per group (short contiguous reduced axes).
template <typename T, int KIND, int G>
__global__ void __launch_bounds__(256) reduce_group4_kernel(const __grid_constant__ RedArgs a) {
  constexpr int NO = 4;
  const int lane = threadIdx.x & 31;
  const int glane = lane & (G - 1);
  const int groups_per_block = blockDim.x / G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  uint32_t st = 0;
  const int64_t og = (a.O + NO - 1) / NO;
  const int64_t nwork = og * a.S;
  for (int64_t w = (int64_t)blockIdx.x * groups_per_block + threadIdx.x / G; w < nwork;
       w += (int64_t)gridDim.x * groups_per_block)
    group_multi<T, KIND, G, NO>(a, (w % og) * NO, w / og, glane, gmask, st);
  if (st) atomicOr(a.status, st);
}

// GROUP with 16-byte loads along the reduced axis (NO outputs per group).
template <typename T, int KIND, int G, int NO>
__global__ void __launch_bounds__(256) reduce_group_vec_kernel(const __grid_constant__ RedArgs a) {
  const int lane = threadIdx.x & 31;
  const int glane = lane & (G - 1);
  const int groups_per_block = blockDim.x / G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  uint32_t st = 0;
  const int64_t og = (a.O + NO - 1) / NO;
  const int64_t nwork = og * a.S;
  for (int64_t w = (int64_t)blockIdx.x * groups_per_block + threadIdx.x / G; w < nwork;
       w += (int64_t)gridDim.x * groups_per_block)
    group_vec<T, KIND, G, NO>(a, (w % og) * NO, w / og, glane, gmask, st);
  if (st) atomicOr(a.status, st);
}

// COLUMN with 16-byte loads across 16 / sizeof(T) consecutive outputs.
template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_column_vec_kernel(const __grid_constant__ RedArgs a) {
  constexpr int VN = 16 / sizeof(T);
  uint32_t st = 0;
  const int64_t ov = a.O / VN;
  const int64_t nwork = ov * a.S;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += (int64_t)gridDim.x * blockDim.x)
    column_vec<T, KIND>(a, (w % ov) * VN, w / ov, st);
  if (st) atomicOr(a.status, st);
}

// SLAB: one contiguous K x L slab after another per block (column_slab).
template <typename T, int KIND>
__global__ void __launch_bounds__(SLAB_THREADS, 4) reduce_slab_kernel(const __grid_constant__ RedArgs a) {
  constexpr int VN = 16 / sizeof(T);
  __shared__ __align__(16) unsigned char raw[SLAB_THREADS * VN * sizeof(SlabAcc<T, KIND>)];
  SlabAcc<T, KIND>* sh = reinterpret_cast<SlabAcc<T, KIND>*>(raw);
  uint32_t st = 0;
  const int L = (int)a.oshape[a.orank - 1];
  const int64_t nslabs = a.O / L;
  for (int64_t s = blockIdx.x; s < nslabs; s += gridDim.x) column_slab<T, KIND>(a, s, L, sh, st);
  if (st) atomicOr(a.status, st);
}

template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_column_kernel(const __grid_constant__ RedArgs a) {
  uint32_t st = 0;
  const int64_t nwork = a.O * a.S;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += (int64_t)gridDim.x * blockDim.x)
    column_one<T, KIND>(a, w % a.O, w / a.O, st);
  if (st) atomicOr(a.status, st);
}

template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_combine_kernel(const __grid_constant__ RedArgs a) {
  uint32_t st = 0;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < a.O; o += (int64_t)gridDim.x * blockDim.x)
    combine_one<T, KIND>(a, o, st);
  if (st) atomicOr(a.status, st);
}

// One block per output: used when each output has many partials.
template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_combine_block_kernel(const __grid_constant__ RedArgs a) {
  __shared__ CombineScratch cs;
  uint32_t st = 0;
  for (int64_t o = blockIdx.x; o < a.O; o += gridDim.x) combine_block<T, KIND>(a, o, cs, st);
  if (st) atomicOr(a.status, st);
}

// Full reduction of one contiguous, 16-byte aligned run of K elements in one
// launch: block b folds a contiguous range of whole vectors (each thread takes
// vectors t, t + 256, ... in order, four in flight), the block's lanes combine
// in a fixed tree, thread 0 stores the block's partial (slot b of S = gridDim
// partials), and the block that arrives last (counter after __threadfence)
// folds the S partials in block order, stores the result and resets the
// counter.  The last block also takes the K % VN elements past the last vector.
template <typename T, int KIND>
__global__ void __launch_bounds__(256) reduce_all_kernel(const __grid_constant__ RedArgs a, unsigned* arrive) {
  constexpr int VN = 16 / sizeof(T);
  __shared__ CombineScratch cs;
  __shared__ int last;
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  const int64_t nv = a.K / VN;
  const int64_t per = (nv + gridDim.x - 1) / gridDim.x;
  const int64_t v0 = (int64_t)blockIdx.x * per, v1 = min(nv, v0 + per);
  uint32_t st = 0;
  SumAcc<T> sacc;
  ExtAcc<T> eacc;
  sacc.init();
  eacc.init();
  int64_t v = v0 + threadIdx.x;
  for (; v + 3 * (int64_t)blockDim.x < v1; v += 4 * (int64_t)blockDim.x) {
    T x[4][VN];
#pragma unroll
    for (int u = 0; u < 4; u++) ld16<T>(a.in + (v + u * (int64_t)blockDim.x) * 16, x[u]);
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (KIND == RK_SUM) {
#pragma unroll
        for (int e = 0; e < VN; e++) sacc.add(x[u][e]);
      } else {
        vec_extreme_into<T, VN>(eacc, x[u], (v + u * (int64_t)blockDim.x) * VN, is_max);
      }
    }
  }
  for (; v < v1; v += blockDim.x) {
    T x[VN];
    ld16<T>(a.in + v * 16, x);
    if (KIND == RK_SUM) {
#pragma unroll
      for (int e = 0; e < VN; e++) sacc.add(x[e]);
    } else {
      vec_extreme_into<T, VN>(eacc, x, v * VN, is_max);
    }
  }
  if (blockIdx.x == gridDim.x - 1) {  // the elements past the last whole vector
    const int64_t k = nv * VN + threadIdx.x;
    if (k < a.K) {
      const T x = ld<T>(a.in + k * (int64_t)sizeof(T));
      if (KIND == RK_SUM) sacc.add(x);
      else eacc.add(x, k, is_max);
    }
  }
  // lanes of a warp, then the warps in order
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    if (KIND == RK_SUM) sacc.shfl(d, 0xffffffffu, 32);
    else eacc.shfl(d, 0xffffffffu, 32, is_max);
  }
  __shared__ SumAcc<T> ws[32];
  __shared__ ExtAcc<T> we[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    ws[warp] = sacc;
    we[warp] = eacc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; w++) {
      if (KIND == RK_SUM) ws[0].merge(ws[w]);
      else we[0].merge(we[w], is_max);
    }
    RedArgs b = a;
    b.S = gridDim.x;
    finish<T, KIND>(b, 0, blockIdx.x, ws[0], we[0], st);  // the block's partial, slot blockIdx.x
    __threadfence();
    last = atomicAdd(arrive, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    RedArgs b = a;
    b.S = gridDim.x;
    b.O = 1;
    combine_block<T, KIND>(b, 0, cs, st);
    if (threadIdx.x == 0) *arrive = 0;
  }
  if (st) atomicOr(a.status, st);
}

// ------------------------------------------------ rows staged by bulk copies
// Reductions of short contiguous rows laid back to back (the innermost axis of
// a contiguous array; 4-byte elements, rows of 32-96 elements): a persistent
// block takes tiles of ROWS_PER_TILE rows; one thread issues one bulk copy of
// the whole tile (contiguous, 16-byte aligned) into a two-stage ring and the
// copy of tile i + 2 as soon as every thread has finished tile i.  Thread r
// reduces row r from shared memory: its vectors are read starting at vector
// r (mod the row's vector count), so the eight threads of a quarter-warp hit
// eight different bank groups.  Per element a sum costs its compensated add
// and an extremum one min/max plus a compare and a select (the first index
// holding the extreme value); no cross-lane combine.  A copy that has not
// landed after TMA_WAIT_NS sets PHCU_ST_TIMEOUT and ends the block.
constexpr int ROWS_PER_TILE = 256;
constexpr int ROWS_MAX_BYTES = 384;  // row length limit: two 96 KiB stages

template <typename T, int KIND>
__global__ void __launch_bounds__(ROWS_PER_TILE, 1) reduce_rows_kernel(const __grid_constant__ RedArgs a) {
  static_assert(sizeof(T) == 4, "4-byte elements");
  constexpr int VN = 4;
  extern __shared__ __align__(128) unsigned char rows_smem[];
  __shared__ __align__(8) uint64_t bars[2];
  const int K = (int)a.K;
  const int NV = K / VN;
  const uint32_t row_bytes = (uint32_t)K * sizeof(T);
  const uint32_t stage_bytes = ROWS_PER_TILE * row_bytes;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(rows_smem);
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&bars[0]);
  const int64_t ntiles = (a.O + ROWS_PER_TILE - 1) / ROWS_PER_TILE;
  const int64_t g = gridDim.x;
  const bool is_max = (a.op == PHCU_RED_MAX || a.op == PHCU_RED_ARGMAX);
  auto issue = [&](int64_t tile, int stg) {
    const int64_t r0 = tile * ROWS_PER_TILE;
    const uint32_t bytes = (uint32_t)min((int64_t)ROWS_PER_TILE, a.O - r0) * row_bytes;
    mbar_expect_tx(bar0 + 8u * stg, bytes);
    bulk_load_1d(sb + stg * stage_bytes, a.in + r0 * row_bytes, bytes, bar0 + 8u * stg);
  };
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t st = 0;
  int64_t t = blockIdx.x;
  if (threadIdx.x == 0) {
    if (t < ntiles) issue(t, 0);
    if (t + g < ntiles) issue(t + g, 1);
  }
  const int r = threadIdx.x;
  for (uint32_t i = 0; t < ntiles; i++, t += g) {
    const int stg = i & 1;
    const bool ok = mbar_wait_bounded(bar0 + 8u * stg, (i >> 1) & 1u, TMA_WAIT_NS);
    if (!__syncthreads_and(ok)) {
      st |= PHCU_ST_TIMEOUT;
      if (threadIdx.x == 0 && t + g < ntiles) mbar_wait_bounded(bar0 + 8u * (stg ^ 1), ((i + 1) >> 1) & 1u, TMA_WAIT_NS);
      break;
    }
    const int64_t o = t * ROWS_PER_TILE + r;
    if (o < a.O) {
      const unsigned char* row = rows_smem + stg * stage_bytes + (size_t)r * row_bytes;
      const uint4* rv = reinterpret_cast<const uint4*>(row);
      int q = r % NV;  // first vector read by this thread
      if (KIND == RK_SUM) {
        SumAcc<T> acc;
        acc.init();
        for (int j = 0; j < NV; j++) {
          const uint4 u = rv[q];
          acc.add(word32_as<T>(u.x));
          acc.add(word32_as<T>(u.y));
          acc.add(word32_as<T>(u.z));
          acc.add(word32_as<T>(u.w));
          q = (q + 1 == NV) ? 0 : q + 1;
        }
        if constexpr (std::is_same<T, float>::value) store_final(a, o, acc.value(), 0, false, 0, 0, st);
        else store_final(a, o, 0, 0, true, (long long)acc.s, 0, st);
      } else {
        // the extreme value over the non-NaN elements, then its first index
        T m = word32_as<T>(rv[0].x);
        for (int j = 0; j < NV; j++) {
          const uint4 u = rv[q];
          m = Lim<T>::ext(m, word32_as<T>(u.x), is_max);
          m = Lim<T>::ext(m, word32_as<T>(u.y), is_max);
          m = Lim<T>::ext(m, word32_as<T>(u.z), is_max);
          m = Lim<T>::ext(m, word32_as<T>(u.w), is_max);
          q = (q + 1 == NV) ? 0 : q + 1;
        }
        int best = K;
        for (int j = 0; j < NV; j++) {
          const uint4 u = rv[q];
          const int k0 = q * VN;
          best = min(best, word32_as<T>(u.x) == m ? k0 : K);
          best = min(best, word32_as<T>(u.y) == m ? k0 + 1 : K);
          best = min(best, word32_as<T>(u.z) == m ? k0 + 2 : K);
          best = min(best, word32_as<T>(u.w) == m ? k0 + 3 : K);
          q = (q + 1 == NV) ? 0 : q + 1;
        }
        const T* re = reinterpret_cast<const T*>(row);
        // a NaN first element (or no candidate) wins: the scan never moves off element 0
        if (best == K || Lim<T>::nan(re[0])) best = 0;
        const T v = re[best];  // the element itself (the sign of a zero)
        double d;
        long long l;
        ext_parts<T>(v, d, l);
        store_final(a, o, d, l, false, 0, best, st);
      }
    }
    __syncthreads();  // every thread is done with this stage
    if (threadIdx.x == 0 && t + 2 * g < ntiles) {
      fence_proxy_async();
      issue(t + 2 * g, stg);
    }
  }
  if (st) atomicOr(a.status, st);
}

// Whether the staged row reduction applies: one contiguous reduced axis of
// 32-96 four-byte elements (whole 16-byte vectors), rows back to back from a
// 16-byte aligned start, no split, enough rows for every SM.
static bool rows_fit(const RedArgs& a, const RedShape& sh) {
  const int es = dtype_size(a.dtype);
  return sh.mode == 0 && es == 4 && a.S == 1 && a.krank == 1 && a.kinner == 1 && a.orank == 1 &&
         a.ostride[0] == a.K && a.K >= 32 && a.K * es <= ROWS_MAX_BYTES && (a.K * es) % 16 == 0 &&
         ((uintptr_t)a.in % 16) == 0 && a.O >= (int64_t)ROWS_PER_TILE * ctx().sm_count;
}

template <typename T, int KIND>
static int32_t launch_rows(const RedArgs& a) {
  const size_t smem = 2 * (size_t)ROWS_PER_TILE * (size_t)a.K * sizeof(T);
  const int per_sm = blocks_per_sm((const void*)reduce_rows_kernel<T, KIND>, ROWS_PER_TILE, smem);
  const int64_t ntiles = (a.O + ROWS_PER_TILE - 1) / ROWS_PER_TILE;
  const int64_t grid = std::min<int64_t>(ntiles, (int64_t)ctx().sm_count * per_sm);
  reduce_rows_kernel<T, KIND><<<(unsigned)grid, ROWS_PER_TILE, smem, ctx().stream>>>(a);
  count_launch();
  return check_launch("reduce_rows_kernel");
}

static int32_t launch_rows_any(const RedArgs& a) {
  const bool sum = a.op == PHCU_RED_SUM;
  if (a.dtype == PHCU_F32) return sum ? launch_rows<float, RK_SUM>(a) : launch_rows<float, RK_EXT>(a);
  return sum ? launch_rows<int32_t, RK_SUM>(a) : launch_rows<int32_t, RK_EXT>(a);
}

// Whether the one-launch full reduction applies: one contiguous reduced run,
// 16-byte aligned, long enough to need many blocks.
static bool full_run(const RedArgs& a, const RedShape& sh) {
  return a.O == 1 && a.krank == 1 && a.kinner == 1 && sh.vec && a.K >= (int64_t)1 << 16 &&
         ((uintptr_t)a.in % 16) == 0;
}

template <typename T, int KIND>
static int32_t launch_all(const RedArgs& a, unsigned* arrive) {
  reduce_all_kernel<T, KIND><<<(unsigned)a.S, 256, 0, ctx().stream>>>(a, arrive);
  count_launch();
  return check_launch("reduce_all_kernel");
}

// Blocks of a one-launch full reduction: four per SM, at most one per 4096
// vectors (so every block has work for each of its threads).
static int64_t full_run_blocks(const RedArgs& a) {
  const int64_t want = (a.K / (16 / dtype_size(a.dtype)) + 4095) / 4096;
  return std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx().sm_count * 4, want));
}

static int32_t launch_full_run(const RedArgs& a, unsigned* arrive) {
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32: return sum ? launch_all<float, RK_SUM>(a, arrive) : launch_all<float, RK_EXT>(a, arrive);
    case PHCU_F64: return sum ? launch_all<double, RK_SUM>(a, arrive) : launch_all<double, RK_EXT>(a, arrive);
    case PHCU_I32: return sum ? launch_all<int32_t, RK_SUM>(a, arrive) : launch_all<int32_t, RK_EXT>(a, arrive);
    default: return sum ? launch_all<long long, RK_SUM>(a, arrive) : launch_all<long long, RK_EXT>(a, arrive);
  }
}

// Whether a COLUMN sum reads whole contiguous slabs (column_slab): one
// reduced axis whose stride is the length L of the innermost kept axis (unit
// stride), L / VN a power of two up to 256, one split, and at least two slabs
// per SM.  The axis-2 sum of 64x128x128x64 runs at 0.88 of the copy peak so
// (COLUMN: 0.73); extrema stay in COLUMN (0.76 there, 0.44-0.48 as slabs).
static bool slab_fit(const RedArgs& a, const RedShape& sh) {
  if (!(sh.vec && sh.mode == 1 && a.S == 1 && a.krank == 1 && a.orank >= 1)) return false;
  const int64_t L = a.oshape[a.orank - 1];
  const int64_t lv = L / (16 / dtype_size(a.dtype));
  return a.ostride[a.orank - 1] == 1 && a.kstride[0] == L && lv >= 1 && lv <= SLAB_THREADS && (lv & (lv - 1)) == 0 &&
         a.O / L >= 2 * (int64_t)ctx().sm_count;
}

// COLUMN blocks of 128 threads: finer blocks spread the outputs evenly over
// the SMs (axis 2 of 64x128x128x64: 1,024 blocks, 6.7 per SM, instead of 512
// at 3.4); every COLUMN entry of that layout gained 0-3% (64 threads: the same).
#ifndef PHCU_COL_THREADS
#define PHCU_COL_THREADS 128
#endif
template <typename T, int KIND>
static int32_t launch_typed(const RedArgs& a, const RedShape& sh) {
  Context& c = ctx();
  const int threads = 256;
  constexpr int VN = 16 / sizeof(T);
  // four outputs per group when the reduced axis is short and outputs are many
  const bool four = sh.mode == 0 && a.K <= (sh.vec ? 2 * VN : 8) * sh.G && a.O >= 4096;
  // two outputs per group for an extremum whose rows one pass of the group covers: eight vectors in
  // flight per lane (axis-3 max/argmax of 64x128x128x64 68 -> 63 us; sums lose, 57 -> 65 us)
  const bool two = !four && KIND == RK_EXT && sh.mode == 0 && sh.vec && a.K <= 4 * VN * sh.G && a.O >= 4096;
  int64_t work_threads = (sh.mode == 0) ? (four ? (a.O + 3) / 4 : two ? (a.O + 1) / 2 : a.O) * a.S * sh.G
                                        : (sh.vec ? a.O / VN : a.O) * a.S;
  const int col_threads = PHCU_COL_THREADS;
  int64_t blocks = (work_threads + threads - 1) / threads;
  if (sh.vec && sh.mode == 1) blocks = (work_threads + col_threads - 1) / col_threads;
  int64_t cap = (int64_t)c.sm_count * 8 * 4;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  bool slab = false;
  if constexpr (KIND == RK_SUM) slab = slab_fit(a, sh);
  if (slab) {
    if constexpr (KIND == RK_SUM) {
      const int64_t nslabs = a.O / a.oshape[a.orank - 1];
      const int per_sm = blocks_per_sm((const void*)reduce_slab_kernel<T, KIND>, SLAB_THREADS, 0);
      const int64_t grid = std::min<int64_t>(nslabs, (int64_t)c.sm_count * per_sm);
      reduce_slab_kernel<T, KIND><<<(unsigned)grid, SLAB_THREADS, 0, c.stream>>>(a);
    }
  } else if (sh.vec && sh.mode == 1) {
    reduce_column_vec_kernel<T, KIND><<<(unsigned)blocks, col_threads, 0, c.stream>>>(a);
  } else if (sh.vec && four) {
    switch (sh.G) {
      case 32: reduce_group_vec_kernel<T, KIND, 32, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 16: reduce_group_vec_kernel<T, KIND, 16, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 8: reduce_group_vec_kernel<T, KIND, 8, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      default: reduce_group_vec_kernel<T, KIND, 4, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
    }
  } else if (sh.vec && two) {
    switch (sh.G) {
      case 32: reduce_group_vec_kernel<T, KIND, 32, 2><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 16: reduce_group_vec_kernel<T, KIND, 16, 2><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 8: reduce_group_vec_kernel<T, KIND, 8, 2><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      default: reduce_group_vec_kernel<T, KIND, 4, 2><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
    }
  } else if (sh.vec) {
    switch (sh.G) {
      case 32: reduce_group_vec_kernel<T, KIND, 32, 1><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 16: reduce_group_vec_kernel<T, KIND, 16, 1><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 8: reduce_group_vec_kernel<T, KIND, 8, 1><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      default: reduce_group_vec_kernel<T, KIND, 4, 1><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
    }
  } else if (four) {
    switch (sh.G) {
      case 32: reduce_group4_kernel<T, KIND, 32><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 16: reduce_group4_kernel<T, KIND, 16><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      case 8: reduce_group4_kernel<T, KIND, 8><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
      default: reduce_group4_kernel<T, KIND, 4><<<(unsigned)blocks, threads, 0, c.stream>>>(a); break;
    }
  } else if (sh.mode == 0) {
    switch (sh.G) {
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
    if (a.S >= 32) {
      int64_t cb = a.O < cap ? a.O : cap;
      reduce_combine_block_kernel<T, KIND><<<(unsigned)cb, threads, 0, c.stream>>>(a);
    } else {
      int64_t cb = (a.O + threads - 1) / threads;
      if (cb > cap) cb = cap;
      reduce_combine_kernel<T, KIND><<<(unsigned)cb, threads, 0, c.stream>>>(a);
    }
    count_launch();
    PHCU_TRY(check_launch("reduce combine kernel"));
  }
  return PHCU_OK;
}

static int32_t launch_reduce(const RedArgs& a, const RedShape& sh) {
  if (rows_fit(a, sh)) return launch_rows_any(a);
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32: return sum ? launch_typed<float, RK_SUM>(a, sh) : launch_typed<float, RK_EXT>(a, sh);
    case PHCU_F64: return sum ? launch_typed<double, RK_SUM>(a, sh) : launch_typed<double, RK_EXT>(a, sh);
    case PHCU_I32: return sum ? launch_typed<int32_t, RK_SUM>(a, sh) : launch_typed<int32_t, RK_EXT>(a, sh);
    default: return sum ? launch_typed<long long, RK_SUM>(a, sh) : launch_typed<long long, RK_EXT>(a, sh);
  }
}

// Launches an already planned reduction the way phcu_reduce does, split
// partials in stream-ordered pool scratch (the batched executor's per-op replay).
int32_t launch_reduce_pooled(RedArgs a, const RedShape& sh) {
  void* scratch = nullptr;
  if (a.S > 1) {
    PHCU_TRY(scratch_alloc((size_t)a.S * (size_t)a.O * sizeof(Partial), &scratch));
    a.partial = (Partial*)scratch;
  }
  const int32_t rc = launch_reduce(a, sh);
  if (scratch) scratch_free(scratch);
  return rc;
}

static void merge_axes(int64_t* sh, int64_t* st, int& rank, bool keep_one) {
  int r = 0;
  int64_t s2[MAXR], t2[MAXR];
  for (int i = 0; i < rank; i++) {
    if (sh[i] == 1 && !(keep_one && rank == 1)) continue;
    if (r > 0 && t2[r - 1] == st[i] * sh[i]) {
      s2[r - 1] *= sh[i];
      t2[r - 1] = st[i];
      continue;
    }
    s2[r] = sh[i];
    t2[r] = st[i];
    r++;
  }
  rank = r;
  for (int i = 0; i < r; i++) {
    sh[i] = s2[i];
    st[i] = t2[i];
  }
}

int32_t plan_reduce(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out, int64_t target,
                    RedArgs* pa, RedShape* shape, bool* trivial, bool* empty_sum) {
  *trivial = false;
  *empty_sum = false;
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
  // the kernels write the output as one row-major run from its first element
  // (check_view bounds the element count, so the running product stays small)
  int64_t expect = 1;
  for (int i = out->rank - 1; i >= 0 && view_size(out) > 0; i--) {
    if (out->shape[i] != 1 && out->stride[i] != expect)
      return fail(PHCU_ERR_INVALID, "reduction output must be contiguous and row-major (axis %d has stride %lld)", i,
                  (long long)out->stride[i]);
    expect *= out->shape[i];
  }

  RedArgs& a = *pa;
  memset(&a, 0, sizeof(a));
  a.in = (const char*)in->base + in->offset * dtype_size(t);
  a.dtype = t;
  a.op = op;
  a.want_index = want_index;
  a.out_dtype = out->dtype;
  a.out = (char*)out->base + out->offset * dtype_size(out->dtype);
  a.status = ctx().status;

  int64_t osh[MAXR], ost[MAXR], ksh[MAXR], kst[MAXR];
  int orank = 0, krank = 0;
  int64_t O = 1, K = 1;
  for (int i = 0; i < in->rank; i++) {
    if (axis < 0 || i == axis) {
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
  if (in->rank == 0) {
    ksh[0] = 1;
    kst[0] = 0;
    krank = 1;
  }
  const int64_t out_n = (axis < 0) ? 1 : O;
  if (view_size(out) != out_n)
    return fail(PHCU_ERR_SHAPE, "reduction output has %lld elements, expected %lld", (long long)view_size(out),
                (long long)out_n);
  if (O == 0) {
    *trivial = true;
    return PHCU_OK;
  }
  if (K == 0) {
    if (op != PHCU_RED_SUM) return fail(PHCU_ERR_EMPTY, "Empty enumerable");
    *empty_sum = true;
    return PHCU_OK;
  }
  // kept axes: lexicographic order is the output order; reduced axes:
  // lexicographic order is the index order argmax reports
  merge_axes(osh, ost, orank, false);
  merge_axes(ksh, kst, krank, true);
  if (krank == 0) {
    ksh[0] = 1;
    kst[0] = 0;
    krank = 1;
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

  const int64_t inner_out_stride = orank > 0 ? ost[orank - 1] : 0;
  const bool k_contig = (kst[krank - 1] == 1 || kst[krank - 1] == -1);
  const int64_t ao = inner_out_stride < 0 ? -inner_out_stride : inner_out_stride;
  const int64_t ak = kst[krank - 1] < 0 ? -kst[krank - 1] : kst[krank - 1];
  int mode, G = 32;
  if (orank > 0 && ao == 1 && !(k_contig && O < target / 8)) {
    mode = 1;
  } else if (orank > 0 && !k_contig && ao < ak && O >= target / 8) {
    mode = 1;  // neither axis contiguous: neighbouring threads read closer along the outputs
  } else {
    mode = 0;
  }
  // 16-byte loads: every output row (and, for COLUMN, every reduced step) must
  // start 16-byte aligned; GROUP also needs the reduced axis to be one axis of
  // unit stride, COLUMN a unit-stride innermost kept axis whose length the
  // vector divides.
  const int es = dtype_size(t);
  const int VN = 16 / es;
  bool vec = ((uintptr_t)a.in % 16) == 0;
  for (int i = 0; i < orank - (mode == 1 ? 1 : 0); i++) vec = vec && (ost[i] * es) % 16 == 0;
  if (mode == 0) {
    vec = vec && krank == 1 && kst[0] == 1 && K >= VN;
  } else {
    vec = vec && ost[orank - 1] == 1 && osh[orank - 1] % VN == 0;
    for (int i = 0; i < krank; i++) vec = vec && (kst[i] * es) % 16 == 0;
  }
  if (mode == 0) {
    // lanes per output: at least 4 elements (4 vectors) per lane, so short
    // rows spend their time loading rather than combining across lanes
    const int64_t per = vec ? K / (4 * VN) : K / 4;
    while (G > 4 && G > per) G >>= 1;
  }
  int64_t S = 1;
  const int64_t units = (mode == 0) ? O * G : O;
  if (units < target) {
    S = (target + units - 1) / units;
    int64_t min_chunk = (mode == 0) ? (int64_t)G * 16 : 32;
    int64_t smax = (K + min_chunk - 1) / min_chunk;
    if (S > smax) S = smax;
    if (S < 1) S = 1;
  }
  a.chunk = (K + S - 1) / S;
  if (vec && mode == 0) a.chunk = (a.chunk + VN - 1) / VN * VN;  // splits start on whole vectors
  a.S = (K + a.chunk - 1) / a.chunk;
  shape->mode = mode;
  shape->G = G;
  shape->vec = vec ? 1 : 0;
  return PHCU_OK;
}

// Plans and launches a reduction.  `partial_buf` (optional) is caller-provided
// scratch of `partial_cap` Partials; when null, scratch comes from the pool.
int32_t reduce_impl(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out, void* partial_buf,
                    size_t partial_cap) {
  RedArgs a;
  RedShape sh;
  bool trivial, empty_sum;
  // planning checks the arguments and touches no device state, so it comes
  // first and argument errors read the same with or without a context
  PHCU_TRY(plan_reduce(op, in, axis, out, (int64_t)ctx().sm_count * 1024, &a, &sh, &trivial, &empty_sum));
  PHCU_TRY(require_ctx());
  if (trivial) return PHCU_OK;
  if (empty_sum) {
    phcu_scalar_t z;
    memset(&z, 0, sizeof(z));
    z.dtype = out->dtype;
    return phcu_fill(out, &z);
  }
  void* scratch = nullptr;
  if (full_run(a, sh)) {
    // S block partials and the arrival counter (zeroed here, reset by the last block)
    a.S = full_run_blocks(a);
    a.chunk = a.K;
    const size_t need = (size_t)a.S + 1;
    if (partial_buf) {
      if (need > partial_cap)
        return fail(PHCU_ERR_UNSUPPORTED,
                    "reduction needs %zu partials but the allocation-free scratch holds %zu; use phcu_reduce", need,
                    partial_cap);
      a.partial = (Partial*)partial_buf;
    } else {
      PHCU_TRY(scratch_alloc(need * sizeof(Partial), &scratch));
      a.partial = (Partial*)scratch;
    }
    unsigned* arrive = (unsigned*)(a.partial + a.S);
    cudaError_t e = cudaMemsetAsync(arrive, 0, sizeof(unsigned), ctx().stream);
    int32_t rc = e == cudaSuccess ? launch_full_run(a, arrive) : cuda_fail(e, "cudaMemsetAsync(reduction counter)");
    if (scratch) scratch_free(scratch);
    return rc;
  }
  if (a.S > 1) {
    size_t need = (size_t)a.S * (size_t)a.O;
    if (partial_buf) {
      if (need > partial_cap)
        return fail(PHCU_ERR_UNSUPPORTED,
                    "reduction needs %zu partials but the allocation-free scratch holds %zu; use phcu_reduce", need,
                    partial_cap);
      a.partial = (Partial*)partial_buf;
    } else {
      PHCU_TRY(scratch_alloc(need * sizeof(Partial), &scratch));
      a.partial = (Partial*)scratch;
    }
  }
  int32_t rc = launch_reduce(a, sh);
  if (scratch) scratch_free(scratch);
  return rc;
}

// ------------------------------------------------ allocation-free variant
// Scratch for phcu_reduce_noalloc: the partial results of split reductions.
// It lives in the library's device image, so every GPU that loads the library
// holds these 4 MiB until the process exits, and no call ever allocates.
constexpr size_t NOALLOC_PARTIALS = size_t(1) << 18;
static __device__ __align__(256) Partial g_noalloc_partials[NOALLOC_PARTIALS];

// Device address of g_noalloc_partials, looked up once per device (the host
// symbol is only a stand-in: it must never be handed to a kernel).  Cleared
// when the library's context is released: a device reset between
// phcu_shutdown and the next phcu_init reloads the module, and the array may
// then sit at another address.
static void* g_noalloc_addr[64] = {nullptr};

void release_noalloc_scratch() {
  for (auto& p : g_noalloc_addr) p = nullptr;
}

static int32_t noalloc_scratch(void** out) {
  int dev = 0;
  PHCU_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PHCU_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(reduction scratch)");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return PHCU_OK;
}

}  // namespace phcu

using namespace phcu;

extern "C" int32_t phcu_reduce(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out) {
  return reduce_impl(op, in, axis, out, nullptr, 0);
}

extern "C" int32_t phcu_reduce_noalloc(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out) {
  PHCU_TRY(require_ctx());
  void* scratch = nullptr;
  PHCU_TRY(noalloc_scratch(&scratch));
  // Every split writes its own partials before the combine reads them, so the
  // scratch needs no clearing between calls.
  return reduce_impl(op, in, axis, out, scratch, NOALLOC_PARTIALS);
}
