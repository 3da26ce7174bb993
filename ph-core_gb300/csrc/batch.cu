// batch.cu -- persistent batched executor for thousands of small, uneven
// array operations (no reference counterpart: the reference materialises one
// NArray per operation, src/multi_indexable.cr:1026-1078).  Host side; the
// kernel and its bodies are in batch_device.cuh.
//
// Every task (a fused elementwise program over strided views, or a reduction)
// is planned once on the host exactly as the standalone entry points plan it,
// given the body the standalone launch would use (the reduced interpreter for
// pre-decoded programs, the general one otherwise; for reductions GROUP with
// the planner's lanes per output, or COLUMN), and cut into work items (a range
// of row chunks, of transpose tiles, or of reduction outputs x splits).  Tasks
// are ordered by body, so the blocks resident at any moment mostly run the
// same code, and by size within a body, largest first, so small items fill the
// tail.  One persistent launch of one block per resident slot drains the item
// list through a device work queue (an atomic ticket).  Split reductions write
// partials; the block that finishes a task's last item (atomic arrival counter
// after a __threadfence) folds them, so no block ever waits on another.  A
// global-timer deadline bounds the loop (status TIMEOUT).  The kernel is
// instantiated for what a batch needs (slot width, inputs per program, 64-bit
// reductions), so a batch of 32-bit operators does not carry the register
// demand of the general case.
//
// Mode 1 replays the same plans as one ordinary launch per task (the per-op
// baseline); mode 2 captures those launches once in a CUDA graph.
#include <algorithm>
#include <vector>

#include "batch_device.cuh"

namespace phcu {

int32_t launch_eval_plan(const EvalPlan& plan, const phcu_program_t& prog);  // eval.cu
int32_t launch_reduce_pooled(RedArgs a, const RedShape& sh);                  // reduce.cu

constexpr int64_t DEFAULT_CHUNK = 32768;  // elements per work item (16384: 3.19 ms, 32768: 3.15 ms on 10,000 tasks)
constexpr int64_t WALK_ELEMS = 512;       // reduced elements one thread walks per unit, about at most

static BatchKernel pick_kernel(int cls, bool narrow, int nin, bool wide) {
  if (cls == BC_REDUCE) return batch_kernel_reduce(wide);
  if (narrow) return nin <= 2 ? batch_kernel_u32_nin2(cls) : batch_kernel_u32_nin4(cls);
  return batch_kernel_u64(cls);
}

// One launch per body class present: its kernel, launch shape and items.
struct Phase {
  BatchKernel kernel = nullptr;
  size_t smem = 0;
  int grid = 0;
  int64_t begin = 0, end = 0;
};

// The per-op replay of a reduction task: the standalone plan and launch shape.
struct Replay {
  RedArgs ra;
  RedShape sh;
};

struct Batch {
  std::vector<BTask> host_tasks;
  std::vector<Replay> replays;  // indexed by BTask::pad of reduction tasks
  std::vector<phcu_program_t> host_progs;
  BTask* d_tasks = nullptr;
  int32_t* d_item_task = nullptr;
  phcu_program_t* d_progs = nullptr;
  unsigned long long* d_ticket = nullptr;  // one counter per phase
  uint32_t* d_counters = nullptr;
  Partial* d_partials = nullptr;
  int64_t n_items = 0;
  int32_t n_counters = 0;
  int64_t bytes = 0;
  Phase phases[BC_COUNT];  // one per body class
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
  for (int k = 0; k < p.nin; k++)
    if (p.in[k].vmode != VM_INDEX) per += dtype_size(p.in[k].dtype);
  return per * p.sp.n;
}

// Pre-decoded programs (every instruction has a pre-decoded form) run the
// reduced interpreter, the rest the general one.
static int eval_fast(const phcu_program_t& P) {
  return (!program_uses_stash(P) && program_is_fx(P)) ? FAST_FX : FAST_NONE;
}

// Splits the reduced axis of a long reduction so that no thread walks much
// more than WALK_ELEMS elements of one unit (G lanes share a GROUP unit): the
// batch has parallelism across tasks, so splits only bound a task's critical
// path (the standalone planner splits to fill the whole GPU with one task).
static void batch_splits(RedArgs& a, int rmode, int G) {
  const int64_t K = a.K;
  const int64_t span = WALK_ELEMS * (rmode == 0 ? G : 1);
  const int64_t S = K > 2 * span ? (K + span - 1) / span : 1;
  const int64_t chunk = (K + S - 1) / S;
  a.chunk = chunk;
  a.S = (K + chunk - 1) / chunk;
}

int32_t batch_prepare(const phcu_task_t* tasks, int32_t n, const phcu_program_t* programs, int32_t nprog,
                      Batch** out) {
  PHCU_TRY(require_ctx());
  if (n < 0 || (n > 0 && !tasks)) return fail(PHCU_ERR_INVALID, "batch: bad task list");
  if (nprog < 0 || (nprog > 0 && !programs)) return fail(PHCU_ERR_INVALID, "batch: bad program table");
  Batch* b = new Batch();
  b->host_progs.assign(programs, programs + (programs ? nprog : 0));
  for (phcu_program_t& P : b->host_progs) predecode_program(&P);
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
    predecode_program(&P);
    b->host_progs.push_back(P);
    fill_prog.push_back({dtype, (int)b->host_progs.size() - 1});
    return (int)b->host_progs.size() - 1;
  };
  bool narrow = true, wide = false;  // elementwise programs all 32-bit; any 64-bit reduction
  int nin_max = 0, max_staged = 0;
  auto fail_batch = [&](int32_t rc) {
    free_batch(b);
    return rc;
  };
  auto plan_row = [](BTask& bt, int64_t chunk) {
    bt.h.kind = BK_ROW;
    bt.h.vec = bt.ep.vec >= 4 ? 4 : 1;  // a 2-aligned plan walks single elements
    bt.h.nunits = bt.ep.sp.n / bt.h.vec;
    bt.h.per_item = std::max<int64_t>(1, chunk / bt.h.vec);
  };
  const int64_t target = (int64_t)ctx().sm_count * 1024;
  for (int i = 0; i < n; i++) {
    const phcu_task_t& t = tasks[i];
    BTask bt;
    memset(&bt, 0, sizeof(bt));
    bt.h.counter = -1;
    // elements per work item, within [2^10, 2^16]: one item is one block's
    // work, and a much larger one would leave that block last in the launch
    const int64_t chunk = std::min<int64_t>(std::max<int64_t>(t.chunk > 0 ? t.chunk : DEFAULT_CHUNK, 1 << 10), 1 << 16);
    if (t.kind == PHCU_TASK_EVAL) {
      if (t.prog < 0 || t.prog >= nprog)
        return fail_batch(fail(PHCU_ERR_INVALID, "batch task %d: program %d out of range", i, t.prog));
      if (t.n_inputs < 0 || t.n_inputs > MAXIN)
        return fail_batch(fail(PHCU_ERR_INVALID, "batch task %d: %d inputs", i, t.n_inputs));
      int32_t rc = check_view(&t.out, "batch output");
      for (int k = 0; k < t.n_inputs && rc == PHCU_OK; k++) rc = check_input_view(&t.in[k], "batch input");
      if (rc == PHCU_OK) rc = check_program(&programs[t.prog], t.n_inputs);
      if (rc == PHCU_OK && programs[t.prog].out_type != t.out.dtype)
        rc = fail(PHCU_ERR_INVALID, "batch task %d: program result type differs from the output", i);
      const phcu_view_t* ins[MAXIN];
      for (int k = 0; k < t.n_inputs; k++) ins[k] = &t.in[k];
      if (rc == PHCU_OK) rc = make_plan(&t.out, ins, t.n_inputs, &bt.ep, t.layout == 1 ? MODE_ROW : -1);
      if (rc != PHCU_OK) return fail_batch(rc);
      if (bt.ep.mode == MODE_EMPTY) continue;
      const phcu_program_t& P = b->host_progs[t.prog];
      bt.prog = t.prog;
      bt.bytes = eval_bytes(bt.ep);
      bt.h.fast = eval_fast(P);
      nin_max = std::max(nin_max, t.n_inputs);
      if (!program_is_32bit(P, bt.ep)) narrow = false;
      if (bt.ep.mode == MODE_TILE) {
        bt.h.kind = BK_TILE;
        bt.h.nunits = bt.ep.tiles_w * bt.ep.tiles_r * bt.ep.nbatch;
        bt.h.per_item = std::max<int64_t>(1, chunk / (TILE * TILE));
        max_staged = std::max(max_staged, __builtin_popcount(bt.ep.staged));
      } else {
        plan_row(bt, chunk);
      }
    } else if (t.kind == PHCU_TASK_REDUCE) {
      RedShape sh;
      bool trivial, empty_sum;
      int32_t rc = plan_reduce(t.red_op, &t.in[0], t.axis, &t.out, target, &bt.ra, &sh, &trivial, &empty_sum);
      if (rc != PHCU_OK) return fail_batch(rc);
      if (trivial) continue;
      if (empty_sum) {
        const phcu_view_t* none[1] = {nullptr};
        rc = make_plan(&t.out, none, 0, &bt.ep, MODE_ROW);
        if (rc != PHCU_OK) return fail_batch(rc);
        bt.prog = zero_prog(t.out.dtype);
        bt.h.fast = eval_fast(b->host_progs[bt.prog]);
        plan_row(bt, chunk);
        bt.bytes = bt.ep.sp.n * dtype_size(t.out.dtype);
        if (dtype_size(t.out.dtype) == 8) narrow = false;
      } else {
        // a reduction keeps the planner's layout (GROUP or COLUMN): the other
        // one, once offered to the tuner, ran the 10,000-task batch's
        // reductions 4-5x slower
        bt.h.kind = BK_REDUCE;
        const int rmode = sh.mode;
        bt.h.rmode = rmode;
        bt.h.rG = rmode == 0 ? sh.G : 1;
        // the per-op replay runs the standalone plan (its splits, vector loads)
        Replay rp{bt.ra, sh};
        bt.pad = (int32_t)b->replays.size();
        b->replays.push_back(rp);
        if (dtype_size(bt.ra.dtype) == 8) wide = true;
        batch_splits(bt.ra, rmode, bt.h.rG);
        bt.h.nunits = bt.ra.O * bt.ra.S;
        // at least one unit for every group of lanes of the block: a smaller
        // item leaves threads idle at the item's closing barrier
        bt.h.per_item = std::max<int64_t>(chunk / std::max<int64_t>(1, bt.ra.chunk), BATCH_THREADS / bt.h.rG);
        bt.bytes = view_size(&t.in[0]) * dtype_size(t.in[0].dtype) + bt.ra.O * dtype_size(t.out.dtype);
      }
    } else {
      return fail_batch(fail(PHCU_ERR_INVALID, "batch task %d: unknown kind %d", i, t.kind));
    }
    bt.h.nitems = (bt.h.nunits + bt.h.per_item - 1) / bt.h.per_item;
    // order: body class, then layout, chunk width or operator, then size, largest first
    bt.order_key = body_class(bt.h.kind, bt.h.fast) * 8 +
                   (bt.h.kind == BK_REDUCE ? bt.h.rmode * 2 + (bt.ra.op == PHCU_RED_SUM) : (bt.h.vec == 4));
    b->bytes += bt.bytes;
    b->host_tasks.push_back(bt);
  }
  std::stable_sort(b->host_tasks.begin(), b->host_tasks.end(), [](const BTask& x, const BTask& y) {
    if (x.order_key != y.order_key) return x.order_key < y.order_key;
    return x.bytes > y.bytes;
  });
  // items (contiguous per task) and the partials of split reductions
  int64_t items = 0;
  size_t partial_total = 0;
  std::vector<size_t> partial_off(b->host_tasks.size(), 0);
  for (size_t i = 0; i < b->host_tasks.size(); i++) {
    BTask& bt = b->host_tasks[i];
    bt.h.item0 = items;
    items += bt.h.nitems;
    if (bt.h.kind == BK_REDUCE && bt.ra.S > 1) {
      bt.h.counter = b->n_counters++;  // the block finishing the last item folds the partials
      partial_off[i] = partial_total;
      partial_total += (size_t)bt.ra.S * (size_t)bt.ra.O;
    }
  }
  b->n_items = items;
  if (items >= INT32_MAX) return fail_batch(fail(PHCU_ERR_UNSUPPORTED, "batch: too many work items"));
  cudaStream_t s = stream();
  if (partial_total) {
    cudaError_t e = cudaMalloc(&b->d_partials, partial_total * sizeof(Partial));
    if (e != cudaSuccess) return fail_batch(cuda_fail(e, "cudaMalloc(batch partials)"));
    for (size_t i = 0; i < b->host_tasks.size(); i++) {
      BTask& bt = b->host_tasks[i];
      if (bt.h.kind == BK_REDUCE && bt.ra.S > 1) bt.ra.partial = b->d_partials + partial_off[i];
    }
  }
  std::vector<int32_t> item_task((size_t)items);
  for (size_t i = 0; i < b->host_tasks.size(); i++) {
    const BTask& bt = b->host_tasks[i];
    for (int64_t j = 0; j < bt.h.nitems; j++) item_task[(size_t)(bt.h.item0 + j)] = (int32_t)i;
  }
  cudaError_t e = cudaSuccess;
  const size_t nt = std::max<size_t>(1, b->host_tasks.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tasks, nt * sizeof(BTask));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_item_task, std::max<size_t>(1, item_task.size()) * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMalloc(&b->d_progs, std::max<size_t>(1, b->host_progs.size()) * sizeof(phcu_program_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ticket, BC_COUNT * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, std::max(1, b->n_counters) * sizeof(uint32_t));
  if (e != cudaSuccess) return fail_batch(cuda_fail(e, "cudaMalloc(batch)"));
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
  if (e != cudaSuccess) return fail_batch(cuda_fail(e, "batch upload"));
  // the items of each body class are contiguous (the order key starts with
  // the class); each class gets its own kernel and launch
  for (const BTask& bt : b->host_tasks) {
    Phase& ph = b->phases[body_class(bt.h.kind, bt.h.fast)];
    if (ph.end == 0) ph.begin = bt.h.item0;
    ph.end = bt.h.item0 + bt.h.nitems;
  }
  for (int cls = 0; cls < BC_COUNT; cls++) {
    Phase& ph = b->phases[cls];
    if (ph.end <= ph.begin) continue;
    ph.kernel = pick_kernel(cls, narrow, nin_max, wide);
    ph.smem = (cls == BC_TILE || cls == BC_TILE_FX) ? (size_t)max_staged * TILE * (TILE + 1) * (narrow ? 4 : 8) : 0;
    // static + dynamic shared memory above the default 48 KiB needs an opt-in
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, (const void*)ph.kernel);
    if (e != cudaSuccess) return fail_batch(cuda_fail(e, "cudaFuncGetAttributes(batch_kernel)"));
    if (fa.sharedSizeBytes + ph.smem > 48 * 1024) {
      e = cudaFuncSetAttribute((const void*)ph.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ph.smem);
      if (e != cudaSuccess) return fail_batch(cuda_fail(e, "cudaFuncSetAttribute(batch_kernel)"));
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)ph.kernel, BATCH_THREADS, ph.smem);
    if (e != cudaSuccess) return fail_batch(cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(batch)"));
    if (per_sm < 1) per_sm = 1;
    ph.grid = (int)std::min<int64_t>((int64_t)ctx().sm_count * per_sm, ph.end - ph.begin);
  }
  *out = b;
  return PHCU_OK;
}

int32_t batch_launch(Batch* b, int mode) {
  PHCU_TRY(require_ctx());
  cudaStream_t s = stream();
  if (b->n_items == 0) return PHCU_OK;
  if (mode == 0) {
    PHCU_CUDA(cudaMemsetAsync(b->d_ticket, 0, BC_COUNT * sizeof(unsigned long long), s));
    if (b->n_counters) PHCU_CUDA(cudaMemsetAsync(b->d_counters, 0, b->n_counters * sizeof(uint32_t), s));
    // The class kernels run side by side: the first on the library stream,
    // each later one on a side stream forked from it, all joined back.  Each
    // fills the GPU, so a later class mostly takes over SMs as the earlier
    // classes' blocks run out of items (10,000 uneven tasks: 2.00 -> 1.91 ms;
    // a fixed split of blocks per SM between the classes ran 2.4-3.6 ms).
    Context& c = ctx();
    PHCU_CUDA(cudaEventRecord(c.ev_fork, s));  // after the memsets, before the first class
    int nside = 0;
    bool first = true;
    for (int cls = 0; cls < BC_COUNT; cls++) {
      const Phase& ph = b->phases[cls];
      if (!ph.kernel) continue;
      cudaStream_t ls = s;
      if (!first) {
        ls = c.side[nside];
        PHCU_CUDA(cudaStreamWaitEvent(ls, c.ev_fork, 0));
      }
      BatchArgs A;
      A.tasks = b->d_tasks;
      A.item_task = b->d_item_task;
      A.progs = b->d_progs;
      A.ticket = b->d_ticket + cls;
      A.counters = b->d_counters;
      A.status = ctx().status;
      A.item_begin = ph.begin;
      A.item_end = ph.end;
      A.deadline_ns = 20ull * 1000 * 1000 * 1000;  // 20 s
      ph.kernel<<<ph.grid, BATCH_THREADS, ph.smem, ls>>>(A);
      count_launch();
      int32_t rc = check_launch("batch_kernel");
      if (!first && rc == PHCU_OK) {
        const cudaError_t e = cudaEventRecord(c.ev_join[nside], ls);
        if (e == cudaSuccess) nside++;
        else rc = cuda_fail(e, "cudaEventRecord(batch join)");
      }
      first = false;
      if (rc != PHCU_OK) {  // join what was forked, then report
        for (int i = 0; i < nside; i++) cudaStreamWaitEvent(s, c.ev_join[i], 0);
        return rc;
      }
    }
    for (int i = 0; i < nside; i++) PHCU_CUDA(cudaStreamWaitEvent(s, c.ev_join[i], 0));
    return PHCU_OK;
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
    if (bt.h.kind == BK_REDUCE) rc = launch_reduce_pooled(b->replays[(size_t)bt.pad].ra, b->replays[(size_t)bt.pad].sh);
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
