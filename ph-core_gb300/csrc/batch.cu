// batch.cu -- persistent batched executor for thousands of small, uneven
// array operations (no reference counterpart: the reference materialises one
// NArray per operation, src/multi_indexable.cr:1026-1078).
//
// Every task (a fused elementwise program over strided views, or a reduction)
// is planned once on the host exactly as the standalone entry points plan it,
// then cut into work items (a range of row chunks, of transpose tiles, or of
// reduction outputs).  One persistent launch of about one block per SM slot
// drains the item list through a device work queue: each block takes the next
// item with an atomic ticket, copies that task's plan and program into shared
// memory and runs the same device bodies as the standalone kernels.  Split
// reductions write partials; the block that finishes a task's last item
// (atomic arrival counter after a __threadfence) folds them, so no block ever
// waits on another.  A global-timer deadline bounds the loop (status TIMEOUT).
//
// Mode 1 replays the same plans as one ordinary launch per task (the per-op
// baseline); mode 2 captures those launches once in a CUDA graph.
#include <algorithm>
#include <vector>

#include "eval_device.cuh"
#include "reduce_device.cuh"

namespace phcu {

int32_t launch_eval_plan(const EvalPlan& plan, const phcu_program_t& prog);  // eval.cu
int32_t launch_reduce_plan(const RedArgs& a, int mode, int G);                // reduce.cu

enum BKind : int32_t { BK_ROW = 0, BK_TILE = 1, BK_REDUCE = 2 };

struct BTask {
  int32_t kind;
  int32_t vec;
  int32_t prog;
  int32_t rmode;  // reduce: 0 GROUP (32 lanes), 1 COLUMN
  int32_t rG;     // reduce group size of the standalone replay
  int32_t counter;
  int64_t item0, nitems;
  int64_t per_item, nunits;
  int64_t bytes;
  EvalPlan ep;
  RedArgs ra;
};

constexpr int BATCH_THREADS = 256;
constexpr int64_t DEFAULT_CHUNK = 8192;

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

template <int KIND, typename T>
__device__ __forceinline__ void batch_reduce_units(const RedArgs& a, int rmode, int64_t u0, int64_t u1, uint32_t& st) {
  if (rmode == 1) {
    for (int64_t w = u0 + threadIdx.x; w < u1; w += blockDim.x) column_one<T, KIND>(a, w % a.O, w / a.O, st);
  } else {
    const int lane = threadIdx.x & 31;
    for (int64_t w = u0 + (threadIdx.x >> 5); w < u1; w += blockDim.x >> 5)
      group_one<T, KIND, 32>(a, w % a.O, w / a.O, lane, 0xffffffffu, st);
  }
}

template <int KIND, typename T>
__device__ __forceinline__ void batch_combine(const RedArgs& a, CombineScratch& cs, uint32_t& st) {
  if (a.S >= 32) {
    for (int64_t o = 0; o < a.O; o++) combine_block<T, KIND>(a, o, cs, st);  // uniform loop: all threads
  } else {
    for (int64_t o = threadIdx.x; o < a.O; o += blockDim.x) combine_one<T, KIND>(a, o, st);
  }
}

__device__ __forceinline__ void dispatch_reduce(const RedArgs& a, int rmode, int64_t u0, int64_t u1, uint32_t& st) {
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32:
      if (sum) batch_reduce_units<RK_SUM, float>(a, rmode, u0, u1, st);
      else batch_reduce_units<RK_EXT, float>(a, rmode, u0, u1, st);
      break;
    case PHCU_I32:
      if (sum) batch_reduce_units<RK_SUM, int32_t>(a, rmode, u0, u1, st);
      else batch_reduce_units<RK_EXT, int32_t>(a, rmode, u0, u1, st);
      break;
    case PHCU_F64:
      if (sum) batch_reduce_units<RK_SUM, double>(a, rmode, u0, u1, st);
      else batch_reduce_units<RK_EXT, double>(a, rmode, u0, u1, st);
      break;
    default:
      if (sum) batch_reduce_units<RK_SUM, long long>(a, rmode, u0, u1, st);
      else batch_reduce_units<RK_EXT, long long>(a, rmode, u0, u1, st);
  }
}

__device__ __forceinline__ void dispatch_combine(const RedArgs& a, CombineScratch& cs, uint32_t& st) {
  const bool sum = a.op == PHCU_RED_SUM;
  switch (a.dtype) {
    case PHCU_F32:
      if (sum) batch_combine<RK_SUM, float>(a, cs, st);
      else batch_combine<RK_EXT, float>(a, cs, st);
      break;
    case PHCU_I32:
      if (sum) batch_combine<RK_SUM, int32_t>(a, cs, st);
      else batch_combine<RK_EXT, int32_t>(a, cs, st);
      break;
    case PHCU_F64:
      if (sum) batch_combine<RK_SUM, double>(a, cs, st);
      else batch_combine<RK_EXT, double>(a, cs, st);
      break;
    default:
      if (sum) batch_combine<RK_SUM, long long>(a, cs, st);
      else batch_combine<RK_EXT, long long>(a, cs, st);
  }
}

struct BatchArgs {
  const BTask* tasks;
  const int32_t* item_task;
  const phcu_program_t* progs;
  unsigned long long* ticket;
  uint32_t* counters;
  uint32_t* status;
  int64_t n_items;
  uint64_t deadline_ns;  // global-timer budget per launch
};

template <typename S>
__global__ void __launch_bounds__(BATCH_THREADS, 2) batch_kernel(const __grid_constant__ BatchArgs A) {
  extern __shared__ __align__(16) unsigned char tiles_raw[];
  S* tiles = reinterpret_cast<S*>(tiles_raw);
  constexpr int E = 4;  // elements per thread per row pass (the kernel carries every code path)
  __shared__ __align__(16) unsigned char s_plan[sizeof(EvalPlan) > sizeof(RedArgs) ? sizeof(EvalPlan)
                                                                                    : sizeof(RedArgs)];
  __shared__ __align__(16) unsigned char s_prog[sizeof(phcu_program_t)];
  __shared__ long long s_item;
  __shared__ int s_flag;
  __shared__ CombineScratch s_combine;
  uint32_t st = 0;
  const uint64_t t_start = global_ns();
  for (;;) {
    if (threadIdx.x == 0) {
      long long it = (long long)atomicAdd(A.ticket, 1ull);
      if (global_ns() - t_start > A.deadline_ns) {
        st |= PHCU_ST_TIMEOUT;
        it = A.n_items;  // give up: the host sees TIMEOUT in the status word
      }
      s_item = it;
    }
    __syncthreads();
    const long long item = s_item;
    if (item >= A.n_items) break;
    const BTask& T = A.tasks[A.item_task[item]];
    const int kind = T.kind;
    const int64_t local = item - T.item0;
    const int64_t u0 = local * T.per_item;
    const int64_t u1 = min(T.nunits, u0 + T.per_item);
    // stage the plan (and program) of this task in shared memory
    {
      const uint32_t* src = (kind == BK_REDUCE) ? (const uint32_t*)&T.ra : (const uint32_t*)&T.ep;
      const int words = (int)((kind == BK_REDUCE ? sizeof(RedArgs) : sizeof(EvalPlan)) / 4);
      uint32_t* dst = (uint32_t*)s_plan;
      for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
      if (kind != BK_REDUCE) {
        const uint32_t* ps = (const uint32_t*)&A.progs[T.prog];
        uint32_t* pd = (uint32_t*)s_prog;
        for (int i = threadIdx.x; i < (int)(sizeof(phcu_program_t) / 4); i += blockDim.x) pd[i] = ps[i];
      }
    }
    __syncthreads();
    if (kind == BK_ROW) {
      const EvalPlan& p = *reinterpret_cast<const EvalPlan*>(s_plan);
      const phcu_program_t& prog = *reinterpret_cast<const phcu_program_t*>(s_prog);
      const uint32_t step = blockDim.x;
      switch (T.vec) {
        case 4:
          for (int64_t c = u0 + threadIdx.x; c < u1; c += (int64_t)step * (E / 4))
            row_group<S, MAXIN, 4, E / 4, true, FAST_NONE>(p, prog, (uint32_t)c, step, (uint32_t)u1, st);
          break;
        case 2:
          for (int64_t c = u0 + threadIdx.x; c < u1; c += (int64_t)step * (E / 2))
            row_group<S, MAXIN, 2, E / 2, true, FAST_NONE>(p, prog, (uint32_t)c, step, (uint32_t)u1, st);
          break;
        default:
          for (int64_t c = u0 + threadIdx.x; c < u1; c += (int64_t)step * E)
            row_group<S, MAXIN, 1, E, true, FAST_NONE>(p, prog, (uint32_t)c, step, (uint32_t)u1, st);
      }
    } else if (kind == BK_TILE) {
      const EvalPlan& p = *reinterpret_cast<const EvalPlan*>(s_plan);
      const phcu_program_t& prog = *reinterpret_cast<const phcu_program_t*>(s_prog);
      for (int64_t t = u0; t < u1; t++) tile_body<S, MAXIN, true, FAST_NONE>(p, prog, (uint64_t)t, tiles, st);
    } else {
      const RedArgs& a = *reinterpret_cast<const RedArgs*>(s_plan);
      dispatch_reduce(a, T.rmode, u0, u1, st);
      if (a.S > 1) {
        __syncthreads();
        if (threadIdx.x == 0) {
          __threadfence();
          const uint32_t arrived = atomicAdd(&A.counters[T.counter], 1u);
          s_flag = (arrived == (uint32_t)(T.nitems - 1));
        }
        __syncthreads();
        if (s_flag) {
          __threadfence();
          dispatch_combine(a, s_combine, st);
        }
      }
    }
    __syncthreads();  // s_plan / s_item are rewritten by the next item
  }
  if (st) atomicOr(A.status, st);
}

struct Batch {
  std::vector<BTask> host_tasks;
  std::vector<phcu_program_t> host_progs;
  BTask* d_tasks = nullptr;
  int32_t* d_item_task = nullptr;
  phcu_program_t* d_progs = nullptr;
  unsigned long long* d_ticket = nullptr;
  uint32_t* d_counters = nullptr;
  Partial* d_partials = nullptr;
  int64_t n_items = 0;
  int32_t n_counters = 0;
  int64_t bytes = 0;
  size_t smem = 0;
  int max_staged = 0;
  bool narrow = true;  // every program fits 32-bit slots
  int grid = 0;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
};

static void free_batch(Batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_tasks);
  cudaFree(b->d_item_task);
  cudaFree(b->d_progs);
  cudaFree(b->d_ticket);
  cudaFree(b->d_counters);
  cudaFree(b->d_partials);
  delete b;
}

static int64_t eval_bytes(const EvalPlan& p) {
  int64_t per = dtype_size(p.out.dtype);
  for (int k = 0; k < p.nin; k++) per += dtype_size(p.in[k].dtype);
  return per * p.sp.n;
}

int32_t batch_prepare(const phcu_task_t* tasks, int32_t n, const phcu_program_t* programs, int32_t nprog,
                      Batch** out) {
  PHCU_TRY(require_ctx());
  if (n < 0 || (n > 0 && !tasks)) return fail(PHCU_ERR_INVALID, "batch: bad task list");
  if (nprog < 0 || (nprog > 0 && !programs)) return fail(PHCU_ERR_INVALID, "batch: bad program table");
  Batch* b = new Batch();
  b->host_progs.assign(programs, programs + (programs ? nprog : 0));
  // program used for zero-filling empty sums
  std::vector<std::pair<int, int>> fill_prog;  // (dtype, index)
  auto zero_prog = [&](int dtype) {
    for (auto& f : fill_prog)
      if (f.first == dtype) return f.second;
    phcu_program_t P;
    memset(&P, 0, sizeof(P));
    P.n_instr = 1;
    P.out_type = dtype;
    P.code[0].op = PHCU_I_LD;
    P.code[0].src = PHCU_SRC_IMM;
    P.code[0].type = (uint8_t)dtype;
    P.code[0].btype = (uint8_t)dtype;
    b->host_progs.push_back(P);
    fill_prog.push_back({dtype, (int)b->host_progs.size() - 1});
    return (int)b->host_progs.size() - 1;
  };
  const int64_t target = (int64_t)ctx().sm_count * 1024;
  size_t partial_total = 0;
  std::vector<size_t> partial_off;
  int64_t items = 0;
  for (int i = 0; i < n; i++) {
    const phcu_task_t& t = tasks[i];
    BTask bt;
    memset(&bt, 0, sizeof(bt));
    const int64_t chunk = t.chunk > 0 ? t.chunk : DEFAULT_CHUNK;
    if (t.kind == PHCU_TASK_EVAL) {
      if (t.prog < 0 || t.prog >= nprog) {
        free_batch(b);
        return fail(PHCU_ERR_INVALID, "batch task %d: program %d out of range", i, t.prog);
      }
      if (t.n_inputs < 0 || t.n_inputs > MAXIN) {
        free_batch(b);
        return fail(PHCU_ERR_INVALID, "batch task %d: %d inputs", i, t.n_inputs);
      }
      int32_t rc = check_view(&t.out, "batch output");
      for (int k = 0; k < t.n_inputs && rc == PHCU_OK; k++) rc = check_input_view(&t.in[k], "batch input");
      if (rc == PHCU_OK) rc = check_program(&programs[t.prog], t.n_inputs);
      if (rc == PHCU_OK && programs[t.prog].out_type != t.out.dtype)
        rc = fail(PHCU_ERR_INVALID, "batch task %d: program result type differs from the output", i);
      const phcu_view_t* ins[MAXIN];
      for (int k = 0; k < t.n_inputs; k++) ins[k] = &t.in[k];
      if (rc == PHCU_OK) rc = make_plan(&t.out, ins, t.n_inputs, &bt.ep, t.layout == 1 ? MODE_ROW : -1);
      if (rc != PHCU_OK) {
        free_batch(b);
        return rc;
      }
      if (bt.ep.mode == MODE_EMPTY) continue;
      bt.prog = t.prog;
      bt.bytes = eval_bytes(bt.ep);
      if (!program_is_32bit(programs[t.prog], bt.ep)) b->narrow = false;
      if (bt.ep.mode == MODE_TILE) {
        bt.kind = BK_TILE;
        bt.nunits = bt.ep.tiles_w * bt.ep.tiles_r * bt.ep.nbatch;
        bt.per_item = std::max<int64_t>(1, chunk / (TILE * TILE));
        b->max_staged = std::max(b->max_staged, __builtin_popcount(bt.ep.staged));
      } else {
        bt.kind = BK_ROW;
        // the batch kernel walks chunks of at most 4 (an 8-aligned plan is 4-aligned)
        bt.vec = std::min(bt.ep.vec, 4);
        bt.nunits = bt.ep.sp.n / bt.vec;
        bt.per_item = std::max<int64_t>(1, chunk / bt.vec);
      }
    } else if (t.kind == PHCU_TASK_REDUCE) {
      RedShape sh;
      bool trivial, empty_sum;
      int32_t rc = plan_reduce(t.red_op, &t.in[0], t.axis, &t.out, target, &bt.ra, &sh, &trivial, &empty_sum);
      if (rc != PHCU_OK) {
        free_batch(b);
        return rc;
      }
      if (trivial) continue;
      if (empty_sum) {
        const phcu_view_t* none[1] = {nullptr};
        rc = make_plan(&t.out, none, 0, &bt.ep, MODE_ROW);
        if (rc != PHCU_OK) {
          free_batch(b);
          return rc;
        }
        bt.kind = BK_ROW;
        bt.vec = std::min(bt.ep.vec, 4);
        bt.prog = zero_prog(t.out.dtype);
        bt.nunits = bt.ep.sp.n / bt.vec;
        bt.per_item = std::max<int64_t>(1, chunk / bt.vec);
        bt.bytes = bt.ep.sp.n * dtype_size(t.out.dtype);
        if (dtype_size(t.out.dtype) == 8) b->narrow = false;
      } else {
        bt.kind = BK_REDUCE;
        bt.rG = sh.G;
        bt.rmode = (t.layout == 1) ? (sh.mode == 1 ? 0 : 1) : sh.mode;
        if (bt.rmode == 1 && bt.ra.orank == 0) bt.rmode = 0;
        bt.nunits = bt.ra.O * bt.ra.S;
        bt.per_item = std::max<int64_t>(1, chunk / std::max<int64_t>(1, bt.ra.chunk));
        bt.bytes = view_size(&t.in[0]) * dtype_size(t.in[0].dtype) + bt.ra.O * dtype_size(t.out.dtype);
        if (bt.ra.S > 1) {
          bt.counter = b->n_counters++;
          partial_off.push_back(partial_total);
          partial_total += (size_t)bt.ra.S * (size_t)bt.ra.O;
        } else {
          bt.counter = -1;
        }
      }
    } else {
      free_batch(b);
      return fail(PHCU_ERR_INVALID, "batch task %d: unknown kind %d", i, t.kind);
    }
    bt.item0 = items;
    bt.nitems = (bt.nunits + bt.per_item - 1) / bt.per_item;
    items += bt.nitems;
    b->bytes += bt.bytes;
    b->host_tasks.push_back(bt);
  }
  b->n_items = items;
  if (items >= INT32_MAX) {
    free_batch(b);
    return fail(PHCU_ERR_UNSUPPORTED, "batch: too many work items");
  }
  cudaStream_t s = stream();
  if (partial_total) {
    cudaError_t e = cudaMalloc(&b->d_partials, partial_total * sizeof(Partial));
    if (e != cudaSuccess) {
      free_batch(b);
      return cuda_fail(e, "cudaMalloc(batch partials)");
    }
    int k = 0;
    for (auto& bt : b->host_tasks)
      if (bt.kind == BK_REDUCE && bt.ra.S > 1) bt.ra.partial = b->d_partials + partial_off[k++];
  }
  std::vector<int32_t> item_task((size_t)items);
  for (size_t i = 0; i < b->host_tasks.size(); i++) {
    const BTask& bt = b->host_tasks[i];
    for (int64_t j = 0; j < bt.nitems; j++) item_task[(size_t)(bt.item0 + j)] = (int32_t)i;
  }
  for (phcu_program_t& P : b->host_progs) predecode_program(&P);
  cudaError_t e = cudaSuccess;
  const size_t nt = std::max<size_t>(1, b->host_tasks.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tasks, nt * sizeof(BTask));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_item_task, std::max<size_t>(1, item_task.size()) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_progs, std::max<size_t>(1, b->host_progs.size()) * sizeof(phcu_program_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ticket, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, std::max(1, b->n_counters) * sizeof(uint32_t));
  if (e != cudaSuccess) {
    free_batch(b);
    return cuda_fail(e, "cudaMalloc(batch)");
  }
  if (!b->host_tasks.empty())
    e = cudaMemcpyAsync(b->d_tasks, b->host_tasks.data(), b->host_tasks.size() * sizeof(BTask),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !item_task.empty())
    e = cudaMemcpyAsync(b->d_item_task, item_task.data(), item_task.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !b->host_progs.empty())
    e = cudaMemcpyAsync(b->d_progs, b->host_progs.data(), b->host_progs.size() * sizeof(phcu_program_t),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    free_batch(b);
    return cuda_fail(e, "batch upload");
  }
  b->smem = (size_t)b->max_staged * TILE * (TILE + 1) * (b->narrow ? 4 : 8);
  int per_sm = 0;
  // static + dynamic shared memory above the default 48 KiB needs an opt-in
  auto prepare_kernel = [&](const void* fn) -> int32_t {
    cudaFuncAttributes fa;
    cudaError_t e2 = cudaFuncGetAttributes(&fa, fn);
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFuncGetAttributes(batch_kernel)");
    if (fa.sharedSizeBytes + b->smem > 48 * 1024) {
      e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem);
      if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFuncSetAttribute(batch_kernel)");
    }
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BATCH_THREADS, b->smem);
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(batch_kernel)");
    return PHCU_OK;
  };
  int32_t prc = b->narrow ? prepare_kernel((const void*)batch_kernel<uint32_t>)
                          : prepare_kernel((const void*)batch_kernel<uint64_t>);
  if (prc != PHCU_OK) {
    free_batch(b);
    return prc;
  }
  if (per_sm < 1) per_sm = 1;
  b->grid = ctx().sm_count * per_sm;
  *out = b;
  return PHCU_OK;
}

int32_t batch_launch(Batch* b, int mode) {
  PHCU_TRY(require_ctx());
  cudaStream_t s = stream();
  if (b->n_items == 0) return PHCU_OK;
  if (mode == 0) {
    PHCU_CUDA(cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned long long), s));
    if (b->n_counters) PHCU_CUDA(cudaMemsetAsync(b->d_counters, 0, b->n_counters * sizeof(uint32_t), s));
    BatchArgs A;
    A.tasks = b->d_tasks;
    A.item_task = b->d_item_task;
    A.progs = b->d_progs;
    A.ticket = b->d_ticket;
    A.counters = b->d_counters;
    A.status = ctx().status;
    A.n_items = b->n_items;
    A.deadline_ns = 20ull * 1000 * 1000 * 1000;  // 20 s
    int grid = (int)std::min<int64_t>(b->grid, b->n_items);
    if (b->narrow) batch_kernel<uint32_t><<<grid, BATCH_THREADS, b->smem, s>>>(A);
    else batch_kernel<uint64_t><<<grid, BATCH_THREADS, b->smem, s>>>(A);
    count_launch();
    return check_launch("batch_kernel");
  }
  if (mode == 2 && b->graph && b->graph_stream == s) {
    PHCU_CUDA(cudaGraphLaunch(b->graph, s));
    count_launch((unsigned)b->host_tasks.size());
    return PHCU_OK;
  }
  bool capture = (mode == 2);
  if (capture) PHCU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  unsigned long long before = ctx().launches;
  int32_t rc = PHCU_OK;
  for (const BTask& bt : b->host_tasks) {
    if (bt.kind == BK_REDUCE) rc = launch_reduce_plan(bt.ra, bt.rmode == 1 ? 1 : 0, bt.rmode == 1 ? 1 : bt.rG);
    else rc = launch_eval_plan(bt.ep, b->host_progs[bt.prog]);
    if (rc != PHCU_OK) break;
  }
  if (capture) {
    cudaGraph_t g;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    ctx().launches = before;
    if (rc != PHCU_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(batch)");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate(batch)");
    b->graph_stream = s;
    PHCU_CUDA(cudaGraphLaunch(b->graph, s));
    count_launch((unsigned)b->host_tasks.size());
  }
  return rc;
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_batch_prepare(const phcu_task_t* tasks, int32_t n_tasks, const phcu_program_t* programs,
                           int32_t n_programs, void** batch) {
  if (!batch) return fail(PHCU_ERR_INVALID, "batch: null handle pointer");
  Batch* b = nullptr;
  PHCU_TRY(batch_prepare(tasks, n_tasks, programs, n_programs, &b));
  *batch = b;
  return PHCU_OK;
}

int32_t phcu_batch_launch(void* batch, int32_t mode) {
  if (!batch) return fail(PHCU_ERR_INVALID, "batch: null handle");
  if (mode < 0 || mode > 2) return fail(PHCU_ERR_INVALID, "batch: unknown mode %d", mode);
  return batch_launch((Batch*)batch, mode);
}

int32_t phcu_batch_info(void* batch, int64_t* n_tasks, int64_t* n_items, int64_t* bytes) {
  if (!batch) return fail(PHCU_ERR_INVALID, "batch: null handle");
  Batch* b = (Batch*)batch;
  if (n_tasks) *n_tasks = (int64_t)b->host_tasks.size();
  if (n_items) *n_items = b->n_items;
  if (bytes) *bytes = b->bytes;
  return PHCU_OK;
}

int32_t phcu_batch_destroy(void* batch) {
  if (batch) {
    cudaStreamSynchronize(stream());
    free_batch((Batch*)batch);
  }
  return PHCU_OK;
}

int32_t phcu_batch_run(const phcu_task_t* tasks, int32_t n_tasks, const phcu_program_t* programs,
                       int32_t n_programs, int32_t mode) {
  void* b = nullptr;
  PHCU_TRY(phcu_batch_prepare(tasks, n_tasks, programs, n_programs, &b));
  int32_t rc = phcu_batch_launch(b, mode);
  phcu_batch_destroy(b);
  return rc;
}

}  // extern "C"
