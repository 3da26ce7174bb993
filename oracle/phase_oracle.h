/*
 * phase_oracle.h -- CPU restatement of the reference (in-phase/ph-core, Crystal)
 * semantics for the device-array hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path and
 * the timed CPU baseline ("port" of the reference's own loops).  Product code
 * (the libphcuda.so C-ABI and the phase_cu host package) never links, imports or
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * and reference legs use it.
 *
 * Parity status: the region/index/gather/scatter/integer-op semantics are
 * pinned by the reference's own known-answer specs (tests/golden); Float32
 * arithmetic, division, floor-division, modulo, powers, sums, max and argmax
 * have no reference test that pins them ("parity unpinned" for those), so the
 * Crystal 1.0 stdlib semantics they follow are stated beside each function.
 *
 * Every function names the reference file:line it restates.  Compiled with
 * -O2 -ffp-contract=off (no FMA contraction, no fast-math).
 */
#ifndef PHASE_ORACLE_H
#define PHASE_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_RANK 8
#define ORA_MAX_TF 16

/* status / error codes (same numbering as the product C-ABI, checked by a test) */
enum {
  ORA_OK = 0,
  ORA_ERR_SHAPE = 1,      /* Phase::ShapeError        (src/exceptions/exceptions.cr:4)  */
  ORA_ERR_DIM = 2,        /* Phase::DimensionError    (src/exceptions/exceptions.cr:18) */
  ORA_ERR_INDEX = 3,      /* IndexError (stdlib), raised by RangeSyntax/CoordUtil       */
  ORA_ERR_OVERFLOW = 4,   /* OverflowError (Crystal checked Int32 arithmetic)           */
  ORA_ERR_DIVZERO = 5,    /* DivisionByZeroError                                        */
  ORA_ERR_ARGUMENT = 6,   /* ArgumentError (e.g. negative integer exponent)             */
  ORA_ERR_UNBOUNDED = 7,  /* generic Exception: unbounded literal without bound shape   */
  ORA_ERR_EMPTY = 8,      /* Enumerable::EmptyError (max of an empty collection)        */
  ORA_ERR_UNSUPPORTED = 9
};

/* device-side status bits recorded during elementwise evaluation */
enum {
  ORA_ST_OVERFLOW = 1u,
  ORA_ST_DIVZERO = 2u,
  ORA_ST_ARGUMENT = 4u
};

/* element types (Crystal Bool, Int32, Int64, Float32, Float64) */
enum { ORA_BOOL = 0, ORA_I32 = 1, ORA_I64 = 2, ORA_F32 = 3, ORA_F64 = 4 };

/* infix operators of MultiIndexable (src/multi_indexable.cr:958-981) */
enum {
  ORA_OP_ADD = 0, ORA_OP_SUB, ORA_OP_MUL, ORA_OP_DIV, ORA_OP_FLOORDIV, ORA_OP_MOD, ORA_OP_POW,
  ORA_OP_WADD, ORA_OP_WSUB, ORA_OP_WMUL, ORA_OP_WPOW,
  ORA_OP_AND, ORA_OP_OR, ORA_OP_XOR,
  ORA_OP_GT, ORA_OP_LT, ORA_OP_GE, ORA_OP_LE, ORA_OP_CMP, ORA_OP_EQ,
  ORA_OP_NBINARY
};
/* unary operators (src/multi_indexable.cr:983-985) */
enum { ORA_UOP_POS = 0, ORA_UOP_NEG = 1, ORA_UOP_NOT = 2 };

/* reductions (Enumerable#sum/#max/#min via include Enumerable(T),
 * src/multi_indexable.cr:18; argmax idiom README.md:56-61) */
enum { ORA_RED_SUM = 0, ORA_RED_MAX = 1, ORA_RED_MIN = 2, ORA_RED_ARGMAX = 3, ORA_RED_ARGMIN = 4 };

/* ---------------------------------------------------------------- regions */

/* One element of a region literal: an Int (kind 0) or a Range with optional
 * first/last/step and exclusivity (kind 1).  This is the parsed form produced
 * by RangeSyntax.parse_range (src/range_syntax/range_syntax.cr:42-68). */
typedef struct {
  int32_t kind;       /* 0 = integer index, 1 = range */
  int32_t has_first, has_last, has_step, exclusive;
  int32_t pad;
  int64_t first, last, step;
} ora_lit_t;

typedef struct {
  int64_t first, step, last, size;
} ora_range_t;

/* IndexRegion (src/index_region.cr:40-120): proper-rank first/step/last/shape,
 * degeneracy per axis, drop flag and the derived reduced shape. */
typedef struct {
  int32_t rank;            /* proper dimensions */
  int32_t drop;
  int32_t reduced_rank;
  int32_t pad;
  int64_t first[ORA_MAX_RANK];
  int64_t step[ORA_MAX_RANK];
  int64_t last[ORA_MAX_RANK];
  int64_t shape[ORA_MAX_RANK];          /* proper shape */
  int32_t degeneracy[ORA_MAX_RANK];
  int64_t reduced_shape[ORA_MAX_RANK];
} ora_region_t;

int ora_get_size(int64_t first, int64_t last, int64_t step, int64_t* size);
int ora_infer_range(const ora_lit_t* lit, int64_t bound, ora_range_t* out);
int ora_canonicalize_range(const ora_lit_t* lit, int64_t bound, ora_range_t* out);
int ora_canonicalize_index(int64_t index, int64_t size, int64_t* out);
int ora_compatible_shapes(const int64_t* s1, int r1, const int64_t* s2, int r2);

int ora_region_new(const ora_lit_t* lits, int nlits, const int64_t* bound, int rank, int drop,
                   ora_region_t* out);
int ora_region_new_absolute(const ora_lit_t* lits, int nlits, int drop, ora_region_t* out);
int ora_region_new_trim(const ora_lit_t* lits, int nlits, const int64_t* bound /* may be NULL */,
                        const int64_t* trim_to, int rank, int drop, ora_region_t* out);
int ora_region_cover(const int64_t* shape, int rank, ora_region_t* out);
int ora_region_trim(ora_region_t* r, const int64_t* bound, int rank);
int ora_region_fits_in(const ora_region_t* r, const int64_t* bound, int rank, int* fits);
int ora_region_reverse(ora_region_t* r);
int ora_region_translate(ora_region_t* r, const int64_t* offset, int n);
int ora_region_includes(const ora_region_t* r, const int64_t* coord, int n);
int ora_region_local_to_absolute(const ora_region_t* r, const int64_t* local, int64_t* absolute);

/* ------------------------------------------------------------- transforms */

enum { ORA_TF_REGION = 0, ORA_TF_PERMUTE = 1, ORA_TF_REVERSE = 2, ORA_TF_RESHAPE = 3 };

/* One coordinate transform of a View (src/view_util/transforms.cr). */
typedef struct {
  int32_t kind;
  int32_t in_rank;                     /* rank of the view-side coordinate */
  int32_t out_rank;                    /* rank of the source-side coordinate */
  int32_t pad;
  ora_region_t region;                 /* REGION */
  int32_t pattern[ORA_MAX_RANK];       /* PERMUTE */
  int64_t shape[ORA_MAX_RANK];         /* REVERSE: shape; RESHAPE: source shape */
  int64_t new_shape[ORA_MAX_RANK];     /* RESHAPE: view shape */
} ora_xf_t;

/* An operand: an NArray buffer (row-major) seen through a View transform chain
 * (newest first, as ComposedTransform stores it, transforms.cr:46-48). */
typedef struct {
  void* buf;
  int32_t dtype;
  int32_t base_rank;
  int64_t base_shape[ORA_MAX_RANK];
  int32_t ntf;
  int32_t rank;                        /* view rank */
  int64_t shape[ORA_MAX_RANK];         /* view shape */
  ora_xf_t tf[ORA_MAX_TF];
} ora_operand_t;

int ora_xf_apply(const ora_xf_t* t, const int64_t* in, int64_t* out);
int ora_operand_offset(const ora_operand_t* a, const int64_t* coord, int64_t* index);

/* --------------------------------------------------------- bulk operations */

int ora_dtype_size(int dtype);

/* View#to_narr / get_chunk on a view: lexicographic gather (view.cr:123-126). */
int ora_gather(const ora_operand_t* a, void* out, int nthreads);
/* Slabs [lo, hi) of the lexicographic output of gather / map_binary / scatter,
 * each element at its own position (bounded timing samples of a full-size
 * operation; ora_scatter_range requires a source that does not alias dst). */
int ora_gather_range(const ora_operand_t* a, void* out, int64_t lo, int64_t hi, int nthreads);
int ora_map_binary_range(int op, const ora_operand_t* a, const ora_operand_t* b, void* out, int64_t lo, int64_t hi,
                         uint32_t* status, int nthreads);
int ora_scatter_range(const ora_operand_t* dst, const ora_operand_t* src, int64_t lo, int64_t hi, int nthreads);
/* NArray#unsafe_fetch_chunk with the buffer-index odometer (n_array.cr:450-453). */
int ora_narray_fetch_chunk(const void* buf, int dtype, const int64_t* shape, int rank,
                           const ora_region_t* region, void* out, int nthreads);
/* NArray#unsafe_set_chunk, array and scalar source (n_array.cr:484-500). */
int ora_narray_set_chunk(void* buf, int dtype, const int64_t* shape, int rank,
                         const ora_region_t* region, const void* src_lex);
int ora_narray_set_chunk_scalar(void* buf, int dtype, const int64_t* shape, int rank,
                                const ora_region_t* region, const void* value);
/* MultiWritable#unsafe_set_chunk through a MutableView (multi_writable.cr:29-36,
 * mutable_view.cr:16-18): dst view <- src operand, element by element in lex order. */
int ora_scatter(const ora_operand_t* dst, const ora_operand_t* src);
int ora_scatter_scalar(const ora_operand_t* dst, const void* value);

/* Elementwise maps with Crystal number semantics (multi_indexable.cr:931-985,
 * 1026-1102; n_array.cr:589-595; patches/number.cr:4-22). */
int ora_result_dtype(int op, int ta, int tb, int* tout);
int ora_map_binary(int op, const ora_operand_t* a, const ora_operand_t* b, void* out,
                   uint32_t* status, int nthreads);
int ora_map_binary_scalar(int op, const ora_operand_t* a, const void* scalar, int scalar_dtype,
                          int scalar_left, void* out, uint32_t* status, int nthreads);
int ora_map_unary(int uop, const ora_operand_t* a, void* out, uint32_t* status);
int ora_cast(const void* in, int tin, void* out, int tout, int64_t n);

/* Reductions.  ora_reduce follows the reference's own path (FP32 left folds over
 * slices / sequential scans; integer sums with overflow check).  ora_reduce_f64
 * is the FP64 oracle for sums.  axis < 0 reduces every element (lex order). */
int ora_reduce(int op, const void* in, int dtype, const int64_t* shape, int rank, int axis,
               void* out, int out_dtype);
int ora_reduce_f64(const void* in, int dtype, const int64_t* shape, int rank, int axis,
                   double* out);

/* One explicit heat step on an n x m grid (examples/heat_equation.cr:38-51
 * generalised to 2-D shifted views), Jacobi update of the interior, zero-copy
 * of the boundary. */
int ora_heat_step_f32(const float* u, float* out, int64_t n, int64_t m, float coef);
int ora_heat_step_f64(const double* u, double* out, int64_t n, int64_t m, double coef);
int ora_heat_run_f32(float* u, float* tmp, int64_t n, int64_t m, float coef, int steps, int nthreads);
int ora_heat_run_f64(double* u, double* tmp, int64_t n, int64_t m, double coef, int steps, int nthreads);

/* MLP oracle (24 -> 64 -> 64 -> 1, ReLU, MSE) for gradient checks: forward and
 * backward in double for a batch. */
int ora_mlp_forward_backward(const float* params, int in_dim, int h1, int h2, const float* x,
                             const float* y, int batch, double* loss, double* grad);

#ifdef __cplusplus
}
#endif
#endif
