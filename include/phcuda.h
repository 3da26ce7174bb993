/*
 * phcuda.h -- C-ABI of libphcuda.so, the GB300 (sm_103a) device backend for
 * Phase n-dimensional arrays (in-phase/ph-core).
 *
 * This is the boundary a `Phase::CuNArray` binds through a Crystal `lib`
 * block.  Region canonicalisation (RangeSyntax / IndexRegion) and shape
 * validation stay in the caller, exactly as in the reference; the library
 * receives already-canonical affine view descriptors.  Every entry point
 * returns an int32 status (PHCU_OK == 0); the message of the last failure on
 * the calling thread is available from phcu_last_error().
 *
 * Ownership: the caller owns every device buffer it allocated with
 * phcu_alloc and frees it with phcu_free; views borrow buffers.  Descriptors
 * and programs are copied by value at call time.
 * Threading: one host thread drives one context; calls are stream-ordered and
 * asynchronous except phcu_download, phcu_sync, phcu_status_word and the
 * timers.  Errors found by kernels (Int32 overflow, division by zero, a
 * negative integer exponent) are recorded in a device status word and
 * surface at the next phcu_status_word() call.
 *
 * Each declaration cites the reference interface (file:line inside ph-core)
 * whose work it replaces.
 */
#ifndef PHCUDA_H
#define PHCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PHCU_API __attribute__((visibility("default")))
#else
#define PHCU_API
#endif

#define PHCU_VERSION_MAJOR 1
#define PHCU_VERSION_MINOR 0
#define PHCU_MAX_RANK 8
#define PHCU_MAX_INPUTS 4
#define PHCU_MAX_INSTR 24

/* ------------------------------------------------------------- status codes
 * Mapped by the binding onto the reference's exceptions:
 * ShapeError / DimensionError (src/exceptions/exceptions.cr:4,18), IndexError,
 * OverflowError, DivisionByZeroError, ArgumentError, Enumerable::EmptyError. */
enum {
  PHCU_OK = 0,
  PHCU_ERR_SHAPE = 1,
  PHCU_ERR_DIM = 2,
  PHCU_ERR_INDEX = 3,
  PHCU_ERR_OVERFLOW = 4,
  PHCU_ERR_DIVZERO = 5,
  PHCU_ERR_ARGUMENT = 6,
  PHCU_ERR_UNBOUNDED = 7,
  PHCU_ERR_EMPTY = 8,
  PHCU_ERR_UNSUPPORTED = 9,
  PHCU_ERR_OOM = 10,
  PHCU_ERR_TIMEOUT = 11,
  PHCU_ERR_CUDA = 12,
  PHCU_ERR_OOB = 13,
  PHCU_ERR_INVALID = 14,
  PHCU_ERR_NOT_INIT = 15
};

/* bits of the device status word */
enum {
  PHCU_ST_OVERFLOW = 1u,
  PHCU_ST_DIVZERO = 2u,
  PHCU_ST_ARGUMENT = 4u,
  PHCU_ST_TIMEOUT = 8u,
  PHCU_ST_OOB = 16u
};

/* element types: Crystal Bool, Int32, Int64, Float32, Float64 */
enum { PHCU_BOOL = 0, PHCU_I32 = 1, PHCU_I64 = 2, PHCU_F32 = 3, PHCU_F64 = 4 };

/* An index operand: a phcu_view_t of this dtype is an input of phcu_eval (or
 * of a batch task) whose element at view coordinate c is the Int32 value
 * offset + sum_i c_i * stride[i], computed and never loaded (`base` is
 * ignored and may be null).  Row-major strides of the output shape give each
 * element's lexicographic index (the idx of NArray#map_with_index,
 * src/n_array.cr:605-611); stride 1 on axis d and 0 elsewhere gives its
 * coordinate along d (MultiIndexable#map_with_coord, src/multi_indexable.cr:708-712).
 * In the program it is read as an Int32 input. */
enum { PHCU_INDEX = 5 };

/* infix operators (src/multi_indexable.cr:958-981) */
enum {
  PHCU_OP_ADD = 0, PHCU_OP_SUB, PHCU_OP_MUL, PHCU_OP_DIV, PHCU_OP_FLOORDIV, PHCU_OP_MOD, PHCU_OP_POW,
  PHCU_OP_WADD, PHCU_OP_WSUB, PHCU_OP_WMUL, PHCU_OP_WPOW,
  PHCU_OP_AND, PHCU_OP_OR, PHCU_OP_XOR,
  PHCU_OP_GT, PHCU_OP_LT, PHCU_OP_GE, PHCU_OP_LE, PHCU_OP_CMP, PHCU_OP_EQ,
  PHCU_OP_NBINARY
};
/* unary operators (src/multi_indexable.cr:983-985) */
enum { PHCU_UOP_POS = 0, PHCU_UOP_NEG = 1, PHCU_UOP_NOT = 2 };

/* reductions (Enumerable#sum/#max/#min, src/multi_indexable.cr:18; argmax idiom README.md:56-61) */
enum { PHCU_RED_SUM = 0, PHCU_RED_MAX = 1, PHCU_RED_MIN = 2, PHCU_RED_ARGMAX = 3, PHCU_RED_ARGMIN = 4 };

/* --------------------------------------------------------- view descriptor
 * An affine view of a row-major device buffer: element (c_0..c_{r-1}) of the
 * view lives at base + (offset + sum_i c_i * stride[i]) * sizeof(dtype).
 * Strides are signed element counts.  This is the folded form of a View's
 * Region/Permute/Reverse transform chain (src/view_util/transforms.cr:191-305)
 * over an NArray buffer (src/buffered/buffered.cr:15-52). */
typedef struct {
  void* base;
  int32_t dtype;
  int32_t rank;
  int64_t offset;
  int64_t shape[PHCU_MAX_RANK];
  int64_t stride[PHCU_MAX_RANK];
} phcu_view_t;

/* ------------------------------------------------------- fused programs
 * A program is a fixed-opcode accumulator machine evaluated per element by a
 * single templated kernel (no JIT).  Registers: ACC, two stash slots S0/S1,
 * the inputs IN[k] (loaded from the input views) and one immediate per
 * instruction.  `src` selects operand B: 0..3 = IN[k], 8 = immediate,
 * 9 = S0, 10 = S1.  `type` is the compute type of the instruction, `btype`
 * the stored type of operand B (converted to `type` on the fly); flag bit 0
 * swaps the operands (ACC = B op ACC).  Binary opcodes reuse PHCU_OP_*
 * numbering; the extra opcodes are below. */
enum {
  PHCU_I_LD = 64,   /* ACC = B */
  PHCU_I_ST0 = 65,  /* S0 = ACC */
  PHCU_I_ST1 = 66,  /* S1 = ACC */
  PHCU_I_CVT = 67,  /* ACC = (imm.i type) ACC, ACC of `type` */
  PHCU_I_NEG = 68,
  PHCU_I_NOT = 69,
  PHCU_I_POS = 70,
  PHCU_I_SEL = 71   /* ACC = (S0 & 1) ? B : ACC  (S0 holds a Bool mask; masked writes,
                       multi_writable.cr:127-172, n_array.cr:510-551) */
};
enum { PHCU_SRC_IMM = 8, PHCU_SRC_S0 = 9, PHCU_SRC_S1 = 10 };

typedef struct {
  uint8_t op;
  uint8_t src;
  uint8_t type;
  uint8_t btype;
  uint8_t flags;
  uint8_t pad[3];
  union {
    double f;
    int64_t i;
  } imm;
} phcu_instr_t;

typedef struct {
  int32_t n_instr;
  int32_t out_type; /* type of ACC after the last instruction */
  phcu_instr_t code[PHCU_MAX_INSTR];
} phcu_program_t;

typedef struct {
  int32_t dtype;
  int32_t pad;
  union {
    double f;
    int64_t i;
  } v;
} phcu_scalar_t;

/* ----------------------------------------------------------------- context */

/* Creates the context on `device` (library stream, memory pool, status word).
 * Replaces nothing in the reference (pure-CPU); required before any call. */
PHCU_API int32_t phcu_init(int32_t device);
PHCU_API int32_t phcu_shutdown(void);
/* Use an external CUDA stream (cudaStream_t) for every later call; NULL
 * restores the library's own stream. */
PHCU_API int32_t phcu_set_stream(void* stream);
PHCU_API int32_t phcu_get_stream(void** stream);
PHCU_API int32_t phcu_sync(void);
/* Copies the message of the last failure on this thread (always NUL-terminated). */
PHCU_API int32_t phcu_last_error(char* buf, size_t len);
/* Reads (after a sync) and optionally clears the device status word. */
PHCU_API int32_t phcu_status_word(uint32_t* out, int32_t clear);
PHCU_API int32_t phcu_version(int32_t* major, int32_t* minor);
/* Device facts: SM count, L2 bytes, max shared memory per block, clock kHz. */
PHCU_API int32_t phcu_device_info(int32_t* sm_count, int64_t* l2_bytes, int32_t* smem_per_block,
                         int32_t* clock_khz);

/* ------------------------------------------------------------------ memory
 * Device storage of a CuNArray; replaces the Slice(T) buffer of NArray
 * (src/n_array.cr:19, 47-79). */
PHCU_API int32_t phcu_alloc(size_t bytes, void** dptr);
PHCU_API int32_t phcu_free(void* dptr);
/* Pinned host staging buffers for asynchronous copies. */
PHCU_API int32_t phcu_host_alloc(size_t bytes, void** hptr);
PHCU_API int32_t phcu_host_free(void* hptr);
/* Host -> device copy, stream-ordered (NArray.of_buffer, src/n_array.cr:76-79). */
PHCU_API int32_t phcu_upload(void* dst, const void* src, size_t bytes);
/* Device -> host copy; returns when the data is on the host (to_narr). */
PHCU_API int32_t phcu_download(void* dst, const void* src, size_t bytes);
/* Overlapped transfers (the bulk copies behind NArray#to_narr / of_buffer,
 * src/view.cr:123-126, src/n_array.cr:76-79, for callers that pipeline many
 * results).  phcu_download_async starts a device -> host copy that waits for
 * the work enqueued so far and then runs on the library's device-to-host
 * stream while later kernels proceed; phcu_upload_async copies host -> device
 * on a host-to-device stream after the work enqueued so far, and later
 * library work waits for it (it does not wait for outstanding downloads).
 * Until phcu_transfer_wait (or phcu_sync) returns, the host buffers must stay
 * untouched and pinned (phcu_host_alloc), a download's source must not be
 * written or freed, and an upload's destination must not be the source of an
 * unfinished download. */
PHCU_API int32_t phcu_download_async(void* dst, const void* src, size_t bytes);
PHCU_API int32_t phcu_upload_async(void* dst, const void* src, size_t bytes);
PHCU_API int32_t phcu_transfer_wait(void);
PHCU_API int32_t phcu_memset(void* dptr, int32_t value, size_t bytes);

/* ---------------------------------------------------------------- hot path */

/* Strided gather/scatter: dst[i] = src[i] for every lexicographic i of the
 * common shape.  Replaces NArray#unsafe_fetch_chunk (src/n_array.cr:450-453),
 * View#to_narr (src/view.cr:123-126), NArray#unsafe_set_chunk
 * (src/n_array.cr:484-492), MultiWritable#unsafe_set_chunk
 * (src/multi_writable.cr:29-36) and MutableView#unsafe_set_element
 * (src/mutable_view.cr:16-18).  Shapes must have equal sizes and be
 * compatible up to trailing ones (ShapeUtil.compatible_shapes?,
 * src/shape_util.cr:6-32); dtypes equal (else PHCU_ERR_INVALID).  A source
 * that overlaps the destination is staged through a temporary first. */
PHCU_API int32_t phcu_copy(const phcu_view_t* dst, const phcu_view_t* src);

/* dst[i] = value for every i.  Replaces NArray#unsafe_set_chunk(region, value)
 * (src/n_array.cr:495-500) and MultiWritable#unsafe_set_chunk(region, value)
 * (src/multi_writable.cr:40-44); value has dst's dtype. */
PHCU_API int32_t phcu_fill(const phcu_view_t* dst, const phcu_scalar_t* value);

/* Fused elementwise program over n_inputs strided views into out.  Replaces
 * map_with/each_with (src/multi_indexable.cr:1026-1102), NArray#map
 * (src/n_array.cr:589-595) and ProcView#unsafe_fetch_element
 * (src/proc_view.cr:28-30); one kernel for a whole infix/process chain. */
PHCU_API int32_t phcu_eval(const phcu_program_t* prog, const phcu_view_t* inputs, int32_t n_inputs,
                  const phcu_view_t* out);

/* One infix operator between two views (def_elementwise_binary,
 * src/multi_indexable.cr:931-945); out dtype must be the Crystal result type. */
PHCU_API int32_t phcu_binary(int32_t op, const phcu_view_t* a, const phcu_view_t* b, const phcu_view_t* out);
/* `view op scalar` (src/multi_indexable.cr:949-951) or, with scalar_left,
 * `scalar op view` (src/patches/number.cr:9-13). */
PHCU_API int32_t phcu_binary_scalar(int32_t op, const phcu_view_t* a, const phcu_scalar_t* s,
                           int32_t scalar_left, const phcu_view_t* out);
/* Unary +, -, ~ (src/multi_indexable.cr:983-985). */
PHCU_API int32_t phcu_unary(int32_t uop, const phcu_view_t* a, const phcu_view_t* out);
/* Crystal result dtype of `a op b` (or PHCU_ERR_UNSUPPORTED). */
PHCU_API int32_t phcu_result_dtype(int32_t op, int32_t ta, int32_t tb, int32_t* tout);

/* Reduction of `in` along `axis` (axis < 0: every element, lexicographic
 * order) into the contiguous `out` (shape = in.shape without axis; one
 * element for axis < 0).  Replaces Enumerable#sum/#max/#min over each and the
 * slices(axis) fold (src/multi_indexable.cr:18, 656-658, 742-786) and the
 * argmax idiom (README.md:56-61: first maximum wins; NaN never wins unless it
 * is the first element).  SUM of Float32 accumulates compensated FP32 per
 * thread and combines across blocks in FP64; out dtype F32 or F64.  ARGMAX /
 * ARGMIN write the index along the axis (lexicographic index for axis < 0)
 * as I32 or I64. */
PHCU_API int32_t phcu_reduce(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out);

/* phcu_reduce for callers that cannot allocate device memory: a host that has
 * handed all device memory to its own pool, an embedded runtime, or code that
 * runs inside a region where cudaMalloc would synchronise or fail.  It has no
 * counterpart in the reference (which has no device code); results equal
 * phcu_reduce's.  Split reductions keep their partials in a static device
 * array of 2^18 partials (4 MiB) that every GPU loading the library holds
 * until the process exits; a reduction that would need more partials is
 * rejected with PHCU_ERR_UNSUPPORTED (phcu_reduce handles it).  The first call
 * on a device after phcu_init looks the array up (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  Every call shares the array: calls that
 * overlap on the GPU (different streams, no ordering) race.  No call allocates
 * or frees memory. */
PHCU_API int32_t phcu_reduce_noalloc(int32_t op, const phcu_view_t* in, int32_t axis, const phcu_view_t* out);

/* Explicit 2-D heat step on an n x m Float32 grid (examples/heat_equation.cr:38-51
 * generalised to 2-D shifted views): out interior = c + (up+down+left+right-c*4)*coef
 * evaluated left to right without FMA; boundary copied.  u and out are
 * contiguous and distinct. */
PHCU_API int32_t phcu_heat_step(const float* u, float* out, int64_t n, int64_t m, float coef);
/* `steps` heat steps ping-ponging between u and tmp (result ends in u).
 * use_graph != 0 captures the steps once into a CUDA graph and replays it. */
PHCU_API int32_t phcu_heat_run(float* u, float* tmp, int64_t n, int64_t m, float coef, int32_t steps,
                      int32_t use_graph);
/* The same run in Float64 (the reference run the Float32 error is measured against). */
PHCU_API int32_t phcu_heat_run_f64(double* u, double* tmp, int64_t n, int64_t m, double coef, int32_t steps,
                                   int32_t use_graph);

/* ------------------------------------------------------------------ graphs
 * Stream capture of a sequence of calls (no reference counterpart: replaces
 * repeated host-driven step loops such as examples/heat_equation.cr:26-36). */
PHCU_API int32_t phcu_graph_begin(void);
PHCU_API int32_t phcu_graph_end(void** graph_exec);
PHCU_API int32_t phcu_graph_launch(void* graph_exec);
PHCU_API int32_t phcu_graph_destroy(void* graph_exec);

/* ------------------------------------------------------- timing / counters */
PHCU_API int32_t phcu_timer_start(void** timer);
PHCU_API int32_t phcu_timer_stop(void* timer, float* ms); /* waits for the stop event */
/* Number of kernels this library launched since phcu_init. */
PHCU_API int32_t phcu_launch_count(uint64_t* n);
/* Writes a scratch buffer larger than L2 so the next kernel starts cold. */
PHCU_API int32_t phcu_l2_flush(void);

/* --------------------------------------------------------- batched executor
 * Thousands of small, uneven array operations in one persistent launch,
 * driven by a device work queue (an atomic ticket counter).  No reference
 * counterpart: the reference runs one materialising pass per operation
 * (src/multi_indexable.cr:1026-1078). */
enum { PHCU_TASK_EVAL = 0, PHCU_TASK_REDUCE = 1 };
typedef struct {
  int32_t kind;     /* PHCU_TASK_EVAL or PHCU_TASK_REDUCE */
  int32_t red_op;   /* PHCU_RED_* for REDUCE */
  int32_t axis;     /* reduce axis (REDUCE) */
  int32_t n_inputs; /* EVAL: 0..PHCU_MAX_INPUTS; REDUCE: 1 */
  int32_t prog;     /* index into the program table (EVAL) */
  int32_t chunk;    /* elements per work item (0 = library default 32768; clamped to [1024, 65536]) */
  int32_t layout;   /* EVAL: 0 = planner's launch shape, 1 = ROW; a REDUCE task
                       always takes the planner's layout */
  int32_t pad;
  phcu_view_t in[PHCU_MAX_INPUTS];
  phcu_view_t out;
} phcu_task_t;

/* Plans every task once and uploads the work list; the handle is replayed by
 * phcu_batch_launch.  The tasks' outputs must not alias their inputs or each
 * other; buffers must outlive the handle. */
PHCU_API int32_t phcu_batch_prepare(const phcu_task_t* tasks, int32_t n_tasks, const phcu_program_t* programs,
                                    int32_t n_programs, void** batch);
/* mode 0: the persistent launches over the device work queue, one per body
 * class present (tasks grouped by kernel kind), side by side: the first on
 * the library stream, the others on side streams forked from it, which the
 * library stream then waits for, so later work on it sees every result;
 * mode 1: one ordinary launch per task (the per-op baseline); mode 2: the
 * per-op launches captured once in a CUDA graph and replayed. */
PHCU_API int32_t phcu_batch_launch(void* batch, int32_t mode);
/* Planned task count (empty tasks dropped), work items and algorithmic bytes. */
PHCU_API int32_t phcu_batch_info(void* batch, int64_t* n_tasks, int64_t* n_items, int64_t* bytes);
PHCU_API int32_t phcu_batch_destroy(void* batch);
/* prepare + launch(mode) + destroy */
PHCU_API int32_t phcu_batch_run(const phcu_task_t* tasks, int32_t n_tasks, const phcu_program_t* programs,
                       int32_t n_programs, int32_t mode);

/* ------------------------------------------------------- autotuner and MLP
 * Launch configurations for the standalone kernels, chosen by exhaustive
 * timing or predicted by a small MLP (24 -> 64 -> 64 -> 1, log-time) trained
 * on the GPU by the library's own kernels. */
#define PHCU_TUNE_FEATURES 24
#define PHCU_MLP_H1 64
#define PHCU_MLP_H2 64
#define PHCU_MLP_PARAMS (PHCU_MLP_H1 * PHCU_TUNE_FEATURES + PHCU_MLP_H1 + PHCU_MLP_H2 * PHCU_MLP_H1 + \
                         PHCU_MLP_H2 + PHCU_MLP_H2 + 1)
/* Number of candidate launch configurations. */
PHCU_API int32_t phcu_tune_n_configs(int32_t* n);
/* Feature vector of (task, config) as the tuner sees it. */
PHCU_API int32_t phcu_tune_features(const phcu_task_t* task, int32_t config, float* features);
/* Times `task` under every config (reps each, median); ms[n_configs].  The
 * task runs as a batch of copies that fills the GPU (up to 512, about 2^25
 * elements in all), each copy writing its own scratch output of the task's
 * shape, and ms is the time per copy: its cost inside a large batch.  The
 * task's own output is not written. */
PHCU_API int32_t phcu_tune_measure(const phcu_task_t* task, const phcu_program_t* programs, int32_t reps,
                          float* ms);
/* Runs `task` once under `config` (standalone kernels). */
PHCU_API int32_t phcu_task_run_config(const phcu_task_t* task, const phcu_program_t* programs, int32_t config);
/* MLP on device memory (params: PHCU_MLP_PARAMS floats). */
PHCU_API int32_t phcu_mlp_init(float* params_dev, uint64_t seed);
PHCU_API int32_t phcu_mlp_forward(const float* params_dev, const float* x_dev, int32_t batch, float* y_dev);
/* One forward+backward pass: loss (host) and grad (device, PHCU_MLP_PARAMS). */
PHCU_API int32_t phcu_mlp_grad(const float* params_dev, const float* x_dev, const float* y_dev,
                      int32_t batch, float* grad_dev, float* loss);
/* Adam training over n samples for `epochs` epochs of minibatches. */
PHCU_API int32_t phcu_mlp_train(float* params_dev, const float* x_dev, const float* y_dev, int32_t n,
                       int32_t epochs, int32_t batch, float lr, uint64_t seed, float* final_loss);

#ifdef __cplusplus
}
#endif
#endif
