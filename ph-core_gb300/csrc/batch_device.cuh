// batch_device.cuh -- work items, bodies and the persistent kernel of the
// batched executor (batch.cu holds the host side).  Each instantiation of
// batch_kernel lives in its own translation unit (batch_k*.cu), so they
// compile in parallel.
//
// The bodies are those of the standalone kernels: ROW and TILE with the
// reduced interpreter for pre-decoded programs (copies and single operators
// included) or the general one otherwise, and the element-load reduction
// bodies (GROUP with the planner's lanes per output, or COLUMN).
#pragma once

#include "eval_device.cuh"
#include "reduce_device.cuh"

namespace phcu {

enum BKind : int32_t { BK_ROW = 0, BK_TILE = 1, BK_REDUCE = 2 };

// Body classes, in item order (one launch each): the layout and, for the
// elementwise layouts, the interpreter (general or pre-decoded).
enum BClass : int32_t { BC_ROW = 0, BC_ROW_FX = 1, BC_TILE = 2, BC_TILE_FX = 3, BC_REDUCE = 4, BC_COUNT = 5 };
__host__ __device__ inline int body_class(int kind, int fast) {
  return kind == BK_REDUCE ? BC_REDUCE : kind * 2 + (fast == FAST_FX);
}

// What a block needs to run one task's items (staged in shared memory).
struct BHead {
  int32_t kind;
  int32_t fast;     // ROW / TILE: FAST_FX (pre-decoded program) or FAST_NONE
  int32_t vec;      // ROW: elements per chunk (1 or 4)
  int32_t rmode;    // REDUCE: 0 GROUP, 1 COLUMN
  int32_t rG;       // REDUCE GROUP: lanes per output
  int32_t counter;  // REDUCE split over several items: arrival counter, else -1
  int64_t item0, nitems, per_item, nunits;
};

struct BTask {
  BHead h;
  int32_t prog;
  int32_t pad;  // reduction: index of its per-op replay plan (host side)
  int64_t bytes;
  int64_t order_key;
  EvalPlan ep;
  RedArgs ra;
};

constexpr int BATCH_THREADS = 256;
#ifndef PHCU_BATCH_MIN_BLOCKS
#define PHCU_BATCH_MIN_BLOCKS 3
#endif
constexpr int BATCH_MIN_BLOCKS = PHCU_BATCH_MIN_BLOCKS;
#ifndef PHCU_BATCH_ROW_FX_BLOCKS
#define PHCU_BATCH_ROW_FX_BLOCKS 4
#endif
// The bodies are inlined into the kernel.  As separate functions (built with
// PHCU_BATCH_NOINLINE) each keeps its own register allocation but the calls
// spill: the 10,000-task workload took 3.59 ms so, 3.35 ms inlined, and
// 4.27 / 4.37 ms at two blocks per SM (128 registers, inlined / separate).
#ifdef PHCU_BATCH_NOINLINE
#define PHCU_BODY __noinline__
#else
#define PHCU_BODY __forceinline__
#endif

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// ------------------------------------------------------------ ROW bodies
// Chunks [u0, u1) of VEC elements; a thread takes U chunks blockDim apart per pass.
template <typename S, int NIN, int VEC, int U, bool STASH, int FAST>
__device__ __forceinline__ void row_item(const EvalPlan& p, const phcu_program_t& prog, int64_t u0, int64_t u1,
                                         uint32_t& st) {
  const uint32_t step = blockDim.x;
  for (int64_t c = u0 + threadIdx.x; c < u1; c += (int64_t)step * U)
    row_group<S, NIN, VEC, U, STASH, FAST>(p, prog, (uint32_t)c, step, (uint32_t)u1, st);
}

// Elements per thread per pass: 4 (8 for pre-decoded 32-bit programs, as in
// the standalone ROW kernel, spilled in the batch kernel at 80 registers:
// 2.02 ms against 2.00 ms with 4 at four blocks per SM); single-element
// chunks take half as many.
#ifndef PHCU_BATCH_FX_V
#define PHCU_BATCH_FX_V 4
#endif
template <typename S, int FAST>
constexpr int batch_v() {
  return (sizeof(S) == 8 || FAST == FAST_NONE) ? 4 : PHCU_BATCH_FX_V;
}

// One function per body and chunk width: each gets its own register allocation.
template <typename S, int NIN, int VEC, int FAST>
__device__ PHCU_BODY void run_row_body(const EvalPlan& p, const phcu_program_t& prog, int64_t u0, int64_t u1,
                                          uint32_t& st) {
  constexpr int V = batch_v<S, FAST>();
  row_item<S, NIN, VEC, VEC == 4 ? V / 4 : V / 2, FAST == FAST_NONE, FAST>(p, prog, u0, u1, st);
}

// ----------------------------------------------------------- TILE bodies
template <typename S, int NIN, int FAST>
__device__ PHCU_BODY void run_tile_body(const EvalPlan& p, const phcu_program_t& prog, int64_t u0, int64_t u1,
                                           S* tiles, uint32_t& st) {
  for (int64_t t = u0; t < u1; t++) tile_body<S, NIN, FAST == FAST_NONE, FAST>(p, prog, (uint64_t)t, tiles, st);
}

// ------------------------------------------------------ REDUCE bodies
// Units [u0, u1) are (output, split) pairs; GROUP (G lanes per unit) or
// COLUMN (one thread per unit), element loads.
template <typename T, int KIND>
__device__ __forceinline__ void red_units(const BHead& h, const RedArgs& a, int64_t u0, int64_t u1, uint32_t& st) {
  if (h.rmode == 1) {
    for (int64_t w = u0 + threadIdx.x; w < u1; w += blockDim.x) column_one<T, KIND>(a, w % a.O, w / a.O, st);
    return;
  }
  const int G = h.rG;
  const int lane = threadIdx.x & 31;
  const int glane = lane & (G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  const int groups = blockDim.x / G;
  for (int64_t w = u0 + threadIdx.x / G; w < u1; w += groups)
    group_one_g<T, KIND>(a, w % a.O, w / a.O, G, glane, gmask, st);
}

template <typename T, int KIND>
__device__ __forceinline__ void red_combine(const RedArgs& a, CombineScratch& cs, uint32_t& st) {
  if (a.S >= 32) {
    for (int64_t o = 0; o < a.O; o++) combine_block<T, KIND>(a, o, cs, st);  // uniform loop: all threads
  } else {
    for (int64_t o = threadIdx.x; o < a.O; o += blockDim.x) combine_one<T, KIND>(a, o, st);
  }
}

template <bool WIDE>
__device__ PHCU_BODY void run_reduce(const BHead& h, const RedArgs& a, int64_t u0, int64_t u1, uint32_t& st) {
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32:
      if (sum) red_units<float, RK_SUM>(h, a, u0, u1, st);
      else red_units<float, RK_EXT>(h, a, u0, u1, st);
      break;
    case PHCU_I32:
      if (sum) red_units<int32_t, RK_SUM>(h, a, u0, u1, st);
      else red_units<int32_t, RK_EXT>(h, a, u0, u1, st);
      break;
    case PHCU_F64:
      if constexpr (WIDE) {
        if (sum) red_units<double, RK_SUM>(h, a, u0, u1, st);
        else red_units<double, RK_EXT>(h, a, u0, u1, st);
      }
      break;
    default:
      if constexpr (WIDE) {
        if (sum) red_units<long long, RK_SUM>(h, a, u0, u1, st);
        else red_units<long long, RK_EXT>(h, a, u0, u1, st);
      }
  }
}

template <bool WIDE>
__device__ PHCU_BODY void run_combine(const RedArgs& a, CombineScratch& cs, uint32_t& st) {
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32:
      if (sum) red_combine<float, RK_SUM>(a, cs, st);
      else red_combine<float, RK_EXT>(a, cs, st);
      break;
    case PHCU_I32:
      if (sum) red_combine<int32_t, RK_SUM>(a, cs, st);
      else red_combine<int32_t, RK_EXT>(a, cs, st);
      break;
    case PHCU_F64:
      if constexpr (WIDE) {
        if (sum) red_combine<double, RK_SUM>(a, cs, st);
        else red_combine<double, RK_EXT>(a, cs, st);
      }
      break;
    default:
      if constexpr (WIDE) {
        if (sum) red_combine<long long, RK_SUM>(a, cs, st);
        else red_combine<long long, RK_EXT>(a, cs, st);
      }
  }
}

struct BatchArgs {
  const BTask* tasks;
  const int32_t* item_task;
  const phcu_program_t* progs;
  unsigned long long* ticket;  // this launch's own counter, from 0
  uint32_t* counters;
  uint32_t* status;
  int64_t item_begin, item_end;  // the items of this launch's body class
  uint64_t deadline_ns;          // global-timer budget per launch
};

// Resident blocks per SM of each class's kernel: four for the pre-decoded
// ROW body with 32-bit slots (64 registers; 10,000-task batch 2.15 -> 2.00
// ms), three (80 registers) for the rest.
template <typename S, int CLASS>
constexpr int batch_min_blocks() {
  return (CLASS == BC_ROW_FX && sizeof(S) == 4) ? PHCU_BATCH_ROW_FX_BLOCKS : BATCH_MIN_BLOCKS;
}

// One persistent kernel per body class (BClass), each compiled with only that
// class's bodies, so each gets the register allocation its own bodies need.
// S: program slot width; NIN: inputs per program (2 or 4); WIDE: reductions
// of 64-bit elements.  Blocks take the class's items with an atomic ticket
// until they (or the global-timer deadline) run out; a task's plan (and
// program) is copied into shared memory when the block's task changes.
template <typename S, int NIN, bool WIDE, int CLASS>
__global__ void __launch_bounds__(BATCH_THREADS, batch_min_blocks<S, CLASS>())
    batch_kernel(const __grid_constant__ BatchArgs A) {
  extern __shared__ __align__(16) unsigned char tiles_raw[];
  S* tiles = reinterpret_cast<S*>(tiles_raw);
  constexpr size_t PB = CLASS == BC_REDUCE ? sizeof(RedArgs) : sizeof(EvalPlan);
  __shared__ __align__(16) unsigned char s_plan[PB];
  // the program (elementwise classes) or the fold scratch (reductions)
  __shared__ __align__(16) unsigned char s_aux[CLASS == BC_REDUCE ? sizeof(CombineScratch) : sizeof(phcu_program_t)];
  __shared__ BHead s_head;
  __shared__ long long s_item;
  __shared__ int s_flag;
  const phcu_program_t& s_prog = *reinterpret_cast<const phcu_program_t*>(s_aux);
  uint32_t st = 0;
  int cur = -1;  // task whose plan is in shared memory
  const uint64_t t_start = global_ns();
  for (;;) {
    if (threadIdx.x == 0) {
      long long it = A.item_begin + (long long)atomicAdd(A.ticket, 1ull);
      if (global_ns() - t_start > A.deadline_ns) {
        st |= PHCU_ST_TIMEOUT;
        it = A.item_end;  // give up: the host sees TIMEOUT in the status word
      }
      s_item = it;
    }
    __syncthreads();
    const long long item = s_item;
    if (item >= A.item_end) break;
    const int ti = A.item_task[item];
    if (ti != cur) {  // uniform: every thread read the same item
      const BTask& T = A.tasks[ti];
      const uint32_t* src = CLASS == BC_REDUCE ? (const uint32_t*)&T.ra : (const uint32_t*)&T.ep;
      for (int i = threadIdx.x; i < (int)(PB / 4); i += blockDim.x) ((uint32_t*)s_plan)[i] = src[i];
      if constexpr (CLASS != BC_REDUCE) {
        const uint32_t* ps = (const uint32_t*)&A.progs[T.prog];
        for (int i = threadIdx.x; i < (int)(sizeof(phcu_program_t) / 4); i += blockDim.x)
          ((uint32_t*)s_aux)[i] = ps[i];
      }
      if (threadIdx.x == 0) s_head = T.h;
      cur = ti;
      __syncthreads();
    }
    const BHead& h = s_head;
    const int64_t local = item - h.item0;
    const int64_t u0 = local * h.per_item;
    const int64_t u1 = min(h.nunits, u0 + h.per_item);
    if constexpr (CLASS == BC_ROW || CLASS == BC_ROW_FX) {
      constexpr int FAST = CLASS == BC_ROW_FX ? FAST_FX : FAST_NONE;
      const EvalPlan& p = *reinterpret_cast<const EvalPlan*>(s_plan);
      if (h.vec == 4) run_row_body<S, NIN, 4, FAST>(p, s_prog, u0, u1, st);
      else run_row_body<S, NIN, 1, FAST>(p, s_prog, u0, u1, st);
    } else if constexpr (CLASS == BC_TILE || CLASS == BC_TILE_FX) {
      constexpr int FAST = CLASS == BC_TILE_FX ? FAST_FX : FAST_NONE;
      run_tile_body<S, NIN, FAST>(*reinterpret_cast<const EvalPlan*>(s_plan), s_prog, u0, u1, tiles, st);
    } else {
      const RedArgs& a = *reinterpret_cast<const RedArgs*>(s_plan);
      run_reduce<WIDE>(h, a, u0, u1, st);
      if (h.counter >= 0) {
        __syncthreads();
        if (threadIdx.x == 0) {
          __threadfence();
          const uint32_t arrived = atomicAdd(&A.counters[h.counter], 1u);
          s_flag = (arrived == (uint32_t)(h.nitems - 1));
        }
        __syncthreads();
        if (s_flag) {
          __threadfence();
          run_combine<WIDE>(a, *reinterpret_cast<CombineScratch*>(s_aux), st);
        }
      }
    }
    __syncthreads();  // s_item (and, for a new task, the staged plan) is rewritten next
  }
  if (st) atomicOr(A.status, st);
}

using BatchKernel = void (*)(BatchArgs);

// The instantiations (batch_k32n2.cu, batch_k32n4.cu, batch_k64.cu): the
// elementwise classes per slot width and input count, the reductions narrow
// (32-bit elements) and wide (every element type).
template <typename S, int NIN>
inline BatchKernel batch_kernel_ew(int cls) {
  switch (cls) {
    case BC_ROW: return batch_kernel<S, NIN, false, BC_ROW>;
    case BC_ROW_FX: return batch_kernel<S, NIN, false, BC_ROW_FX>;
    case BC_TILE: return batch_kernel<S, NIN, false, BC_TILE>;
    default: return batch_kernel<S, NIN, false, BC_TILE_FX>;
  }
}
BatchKernel batch_kernel_u32_nin2(int cls);
BatchKernel batch_kernel_u32_nin4(int cls);
BatchKernel batch_kernel_u64(int cls);
BatchKernel batch_kernel_reduce(bool wide);

}  // namespace phcu
