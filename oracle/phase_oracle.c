/*
 * phase_oracle.c -- CPU restatement of the reference (in-phase/ph-core) hot
 * path.  TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the
 * timed CPU baseline.  Nothing in the product links or calls this file.
 *
 * The loops deliberately keep the reference's algorithms: lexicographic
 * odometers over coordinates, one coordinate -> buffer index dot product per
 * operand per element, per-element View transform chains, one materialised
 * pass per infix operator, sequential folds for reductions.  Multi-threaded
 * variants split the lexicographic output range into contiguous pieces and
 * run the same per-element loop on each piece (the reference itself is
 * single-threaded; threads are only used to time the port on all host cores).
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared -pthread (see oracle/Makefile).
 */
#include "phase_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ================================================================ helpers */

int ora_dtype_size(int dtype) {
  switch (dtype) {
    case ORA_BOOL: return 1;
    case ORA_I32: return 4;
    case ORA_I64: return 8;
    case ORA_F32: return 4;
    case ORA_F64: return 8;
  }
  return 0;
}

static int64_t sign64(int64_t x) { return (x > 0) - (x < 0); }
static int64_t cmp64(int64_t a, int64_t b) { return (a > b) - (a < b); }

/* Crystal Int#// for positive divisors (floor division). */
static int64_t floordiv64(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q -= 1;
  return q;
}
static int64_t floormod64(int64_t a, int64_t b) {
  int64_t r = a % b;
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}

static int64_t shape_size(const int64_t* shape, int rank) {
  /* ShapeUtil.shape_to_size (src/shape_util.cr:41-50): [] -> 0, else product */
  if (rank == 0) return 0;
  int64_t n = 1;
  for (int i = 0; i < rank; i++) n *= shape[i];
  return n;
}

static void axis_strides(const int64_t* shape, int rank, int64_t* st) {
  /* Buffered.axis_strides (src/buffered/buffered.cr:15-24) */
  if (rank == 0) return;
  st[rank - 1] = 1;
  for (int i = rank - 2; i >= 0; i--) st[i] = st[i + 1] * shape[i + 1];
}

static void index_to_coord(int64_t index, const int64_t* shape, int rank, int64_t* coord) {
  /* Buffered.index_to_coord (src/buffered/buffered.cr:65-76) */
  for (int d = rank - 1; d >= 0; d--) {
    coord[d] = index % shape[d];
    index /= shape[d];
  }
}

/* ============================================================ RangeSyntax */

/* RangeSyntax.get_size (src/range_syntax/range_syntax.cr:7-17) */
int ora_get_size(int64_t first, int64_t last, int64_t step, int64_t* size) {
  if (last != first && sign64(step) != cmp64(last, first)) return ORA_ERR_INDEX;
  if (step == 0) { /* a..0..a: Crystal's Int#// would raise; treated as a step conflict */
    return ORA_ERR_INDEX;
  }
  if (last >= first) *size = floordiv64(last - first, step) + 1;
  else *size = floordiv64(first - last, -step) + 1;
  return ORA_OK;
}

/* CoordUtil.canonicalize_index_unsafe (src/coord_util.cr:76-82) */
static int64_t canon_unsafe(int64_t index, int64_t size) { return index < 0 ? size + index : index; }

/* CoordUtil.canonicalize_index / has_index? (src/coord_util.cr:20-22, 43-48) */
int ora_canonicalize_index(int64_t index, int64_t size, int64_t* out) {
  if (!(index < size && index >= -size)) return ORA_ERR_INDEX;
  *out = canon_unsafe(index, size);
  return ORA_OK;
}

/* RangeSyntax.infer_range (src/range_syntax/range_syntax.cr:84-136) */
int ora_infer_range(const ora_lit_t* lit, int64_t bound, ora_range_t* out) {
  if (lit->kind == 0) { /* integer index: range_syntax.cr:84-87 */
    int64_t c = canon_unsafe(lit->first, bound);
    out->first = c; out->step = 1; out->last = c; out->size = 1;
    return ORA_OK;
  }
  int64_t first, temp_last, step;
  if (!lit->has_step) {
    first = lit->has_first ? canon_unsafe(lit->first, bound) : 0;
    temp_last = lit->has_last ? canon_unsafe(lit->last, bound) : bound - 1;
    step = (temp_last >= first) ? 1 : -1;
  } else {
    step = lit->step;
    first = lit->has_first ? canon_unsafe(lit->first, bound) : (step > 0 ? 0 : bound - 1);
    temp_last = lit->has_last ? canon_unsafe(lit->last, bound) : (step > 0 ? bound - 1 : 0);
  }
  if (lit->has_last && lit->exclusive) {
    if (temp_last == first) { /* spans no integers: {0, 0, 0, 0} */
      out->first = 0; out->step = 0; out->last = 0; out->size = 0;
      return ORA_OK;
    }
    temp_last -= sign64(step);
  }
  if (first < 0 || temp_last < 0) return ORA_ERR_INDEX;
  int64_t size;
  int rc = ora_get_size(first, temp_last, step, &size);
  if (rc) return rc;
  out->first = first;
  out->step = step;
  out->size = size;
  out->last = first + step * (size - 1);
  return ORA_OK;
}

/* RangeSyntax.canonicalize_range (src/range_syntax/range_syntax.cr:145-153) */
int ora_canonicalize_range(const ora_lit_t* lit, int64_t bound, ora_range_t* out) {
  int rc = ora_infer_range(lit, bound, out);
  if (rc) return rc;
  /* range_valid? (range_syntax.cr:138-140): both endpoints in 0...bound */
  if (!(out->last >= 0 && out->last < bound && out->first >= 0 && out->first < bound))
    return ORA_ERR_INDEX;
  return ORA_OK;
}

/* ShapeUtil.compatible_shapes? (src/shape_util.cr:6-32) */
int ora_compatible_shapes(const int64_t* s1, int r1, const int64_t* s2, int r2) {
  if (r1 == 0 || r2 == 0) return r1 == r2;
  const int64_t* larger = r1 > r2 ? s1 : s2;
  int shared = r1 > r2 ? r2 : r1;
  int lr = r1 > r2 ? r1 : r2;
  for (int i = 0; i < shared; i++)
    if (s1[i] != s2[i]) return 0;
  for (int i = shared; i < lr; i++)
    if (larger[i] != 1) return 0;
  return 1;
}

/* ============================================================ IndexRegion */

/* IndexRegion.compute_reduced_shape (src/index_region.cr:304-317) */
static void compute_reduced(ora_region_t* r) {
  if (r->drop) {
    int k = 0;
    for (int i = 0; i < r->rank; i++)
      if (!r->degeneracy[i]) r->reduced_shape[k++] = r->shape[i];
    if (k == 0) {
      r->reduced_shape[0] = shape_size(r->shape, r->rank);
      k = 1;
    }
    r->reduced_rank = k;
  } else {
    for (int i = 0; i < r->rank; i++) r->reduced_shape[i] = r->shape[i];
    r->reduced_rank = r->rank;
  }
}

/* RangeSyntax.ensure_nonnegative (range_syntax.cr:70-82) */
static int ensure_nonneg(const ora_lit_t* l) {
  if (l->kind == 0) return l->first < 0 ? ORA_ERR_INDEX : ORA_OK;
  if (l->has_first && l->first < 0) return ORA_ERR_INDEX;
  if (l->has_last && l->last < 0) return ORA_ERR_INDEX;
  return ORA_OK;
}

/* RangeSyntax.bounded? (range_syntax.cr:19-35) */
static int lit_bounded(const ora_lit_t* l) {
  if (l->kind == 0) return 1;
  if (!l->has_step || l->step >= 0) return l->has_last;
  return l->has_first;
}

/* IndexRegion.new(region_literal, bound_shape, drop) (src/index_region.cr:192-224) */
int ora_region_new(const ora_lit_t* lits, int nlits, const int64_t* bound, int rank, int drop,
                   ora_region_t* out) {
  memset(out, 0, sizeof(*out));
  if (rank > ORA_MAX_RANK) return ORA_ERR_DIM;
  if (nlits > rank) return ORA_ERR_DIM;
  out->rank = rank;
  out->drop = drop;
  for (int i = 0; i < rank; i++) out->step[i] = 1;
  for (int i = 0; i < nlits; i++) {
    ora_range_t r;
    int rc = ora_canonicalize_range(&lits[i], bound[i], &r);
    if (rc) return rc;
    out->first[i] = r.first;
    out->step[i] = r.step;
    out->last[i] = r.last;
    out->shape[i] = r.size;
    if (lits[i].kind == 0) out->degeneracy[i] = drop;
  }
  for (int i = nlits; i < rank; i++) {
    out->last[i] = bound[i] - 1;
    out->shape[i] = bound[i];
  }
  compute_reduced(out);
  return ORA_OK;
}

/* IndexRegion.new(region_literal, drop) without a bound (src/index_region.cr:255-283) */
int ora_region_new_absolute(const ora_lit_t* lits, int nlits, int drop, ora_region_t* out) {
  memset(out, 0, sizeof(*out));
  if (nlits > ORA_MAX_RANK) return ORA_ERR_DIM;
  out->rank = nlits;
  out->drop = drop;
  for (int i = 0; i < nlits; i++) {
    int rc = ensure_nonneg(&lits[i]);
    if (rc) return rc;
    if (!lit_bounded(&lits[i])) return ORA_ERR_UNBOUNDED;
    if (lits[i].kind == 0) out->degeneracy[i] = 1;
    ora_range_t r;
    rc = ora_infer_range(&lits[i], 0, &r);
    if (rc) return rc;
    out->first[i] = r.first;
    out->step[i] = r.step;
    out->last[i] = r.last;
    out->shape[i] = r.size;
  }
  compute_reduced(out);
  return ORA_OK;
}

/* IndexRegion.trim_axis (src/index_region.cr:684-702) */
static void trim_axis(int64_t nb, int64_t* first, int64_t* step, int64_t* last, int64_t* size) {
  if (*first >= nb) {
    if (*last >= nb) {
      *first = 0; *step = 0; *last = 0; *size = 0;
      return;
    } else if (*step < 0) {
      int64_t as = *step < 0 ? -*step : *step;
      int64_t span = (nb - 1) - *last;
      *size = floordiv64(span, as) + 1;
      span -= floormod64(span, as);
      *first = *last + span;
      return;
    }
  } else if (*step > 0 && *last >= nb) {
    int64_t as = *step;
    int64_t span = (nb - 1) - *first;
    span -= floormod64(span, as);
    *size = floordiv64(span, as) + 1;
    *last = *first + span;
  }
}

/* IndexRegion#trim! (src/index_region.cr:502-515) */
int ora_region_trim(ora_region_t* r, const int64_t* bound, int rank) {
  if (rank != r->rank) return ORA_ERR_DIM;
  for (int i = 0; i < rank; i++)
    trim_axis(bound[i], &r->first[i], &r->step[i], &r->last[i], &r->shape[i]);
  compute_reduced(r);
  return ORA_OK;
}

/* IndexRegion.new(region_literal, bound_shape?, drop, trim_to:) (src/index_region.cr:137-169) */
int ora_region_new_trim(const ora_lit_t* lits, int nlits, const int64_t* bound,
                        const int64_t* trim_to, int rank, int drop, ora_region_t* out) {
  memset(out, 0, sizeof(*out));
  if (rank > ORA_MAX_RANK || nlits > rank) return ORA_ERR_DIM;
  out->rank = rank;
  out->drop = drop;
  int allow_relative = bound != NULL;
  const int64_t* bs = bound ? bound : trim_to;
  for (int i = 0; i < rank; i++) out->step[i] = 1;
  for (int i = 0; i < nlits; i++) {
    if (!allow_relative) {
      int rc = ensure_nonneg(&lits[i]);
      if (rc) return rc;
    }
    ora_range_t r;
    int rc = ora_infer_range(&lits[i], bs[i], &r);
    if (rc) return rc;
    out->first[i] = r.first;
    out->step[i] = r.step;
    out->last[i] = r.last;
    out->shape[i] = r.size;
    if (lits[i].kind == 0) out->degeneracy[i] = drop;
  }
  for (int i = nlits; i < rank; i++) {
    out->last[i] = bs[i] - 1;
    out->shape[i] = bs[i];
  }
  compute_reduced(out);
  return ora_region_trim(out, trim_to, rank);
}

/* IndexRegion.cover (src/index_region.cr:232-238) */
int ora_region_cover(const int64_t* shape, int rank, ora_region_t* out) {
  memset(out, 0, sizeof(*out));
  if (rank > ORA_MAX_RANK) return ORA_ERR_DIM;
  out->rank = rank;
  out->drop = 1;
  for (int i = 0; i < rank; i++) {
    out->first[i] = 0;
    out->step[i] = shape[i] == 0 ? 0 : 1;
    out->last[i] = shape[i] - 1 > 0 ? shape[i] - 1 : 0;
    out->shape[i] = shape[i];
  }
  compute_reduced(out);
  return ORA_OK;
}

/* IndexRegion#fits_in? (src/index_region.cr:468-478) */
int ora_region_fits_in(const ora_region_t* r, const int64_t* bound, int rank, int* fits) {
  if (rank != r->rank) return ORA_ERR_DIM;
  *fits = 1;
  for (int i = 0; i < rank; i++) {
    int64_t m = r->first[i] > r->last[i] ? r->first[i] : r->last[i];
    if (bound[i] <= m) { *fits = 0; break; }
  }
  return ORA_OK;
}

/* IndexRegion#reverse! (src/index_region.cr:533-537) */
int ora_region_reverse(ora_region_t* r) {
  for (int i = 0; i < r->rank; i++) {
    int64_t t = r->first[i];
    r->first[i] = r->last[i];
    r->last[i] = t;
    r->step[i] = -r->step[i];
  }
  return ORA_OK;
}

/* IndexRegion#translate! (src/index_region.cr:577-585) */
int ora_region_translate(ora_region_t* r, const int64_t* offset, int n) {
  for (int i = 0; i < n; i++)
    if (offset[i] < 0 && (r->first[i] < -offset[i] || r->last[i] < -offset[i])) return ORA_ERR_INDEX;
  for (int i = 0; i < n; i++) {
    r->first[i] += offset[i];
    r->last[i] += offset[i];
  }
  return ORA_OK;
}

/* IndexRegion#includes? (src/index_region.cr:445-458); returns 1/0 */
int ora_region_includes(const ora_region_t* r, const int64_t* coord, int n) {
  if (n != r->rank) return 0;
  for (int i = 0; i < n; i++) {
    int64_t lo = r->step[i] > 0 ? r->first[i] : r->last[i];
    int64_t hi = r->step[i] > 0 ? r->last[i] : r->first[i];
    if (coord[i] < lo || coord[i] > hi) return 0;
    if (r->step[i] == 0) return 0;
    if (floormod64(coord[i] - r->first[i], r->step[i]) != 0) return 0;
  }
  return 1;
}

/* IndexRegion#local_to_absolute_unsafe (src/index_region.cr:621-637) */
int ora_region_local_to_absolute(const ora_region_t* r, const int64_t* local, int64_t* absolute) {
  if (r->drop) {
    int la = 0;
    for (int i = 0; i < r->rank; i++) {
      if (r->degeneracy[i]) absolute[i] = r->first[i];
      else { absolute[i] = r->first[i] + local[la] * r->step[i]; la++; }
    }
  } else {
    for (int i = 0; i < r->rank; i++) absolute[i] = r->first[i] + local[i] * r->step[i];
  }
  return ORA_OK;
}

/* ============================================================= transforms */

/* CoordTransform#apply for each transform kind (src/view_util/transforms.cr) */
int ora_xf_apply(const ora_xf_t* t, const int64_t* in, int64_t* out) {
  switch (t->kind) {
    case ORA_TF_REGION: /* RegionTransform#apply (transforms.cr:214-220) */
      return ora_region_local_to_absolute(&t->region, in, out);
    case ORA_TF_PERMUTE: /* PermuteTransform#unpermute (transforms.cr:255-270) */
      for (int i = 0; i < t->in_rank; i++) out[t->pattern[i]] = in[i];
      return ORA_OK;
    case ORA_TF_REVERSE: /* ReverseTransform#apply (transforms.cr:298-304) */
      for (int i = 0; i < t->in_rank; i++) out[i] = t->shape[i] - 1 - in[i];
      return ORA_OK;
    case ORA_TF_RESHAPE: { /* ReshapeTransform#apply (transforms.cr:184-188) */
      int64_t vst[ORA_MAX_RANK];
      axis_strides(t->new_shape, t->in_rank, vst);
      int64_t index = 0;
      for (int i = 0; i < t->in_rank; i++) index += in[i] * vst[i];
      index_to_coord(index, t->shape, t->out_rank, out);
      return ORA_OK;
    }
  }
  return ORA_ERR_UNSUPPORTED;
}

/* View#unsafe_fetch_element -> ComposedTransform#apply (transforms.cr:77-91)
 * -> NArray#unsafe_fetch_element (n_array.cr:456-458, buffered.cr:44-52) */
int ora_operand_offset(const ora_operand_t* a, const int64_t* coord, int64_t* index) {
  int64_t c0[ORA_MAX_RANK], c1[ORA_MAX_RANK];
  const int64_t* cur = coord;
  int64_t* nxt = c0;
  for (int k = 0; k < a->ntf; k++) {
    ora_xf_apply(&a->tf[k], cur, nxt);
    cur = nxt;
    nxt = (nxt == c0) ? c1 : c0;
  }
  int64_t st[ORA_MAX_RANK];
  axis_strides(a->base_shape, a->base_rank, st);
  int64_t idx = 0;
  for (int i = 0; i < a->base_rank; i++) idx += cur[i] * st[i];
  *index = idx;
  return ORA_OK;
}

/* Fast path for operands without transforms: coord . axis_strides */
typedef struct {
  const ora_operand_t* op;
  int64_t st[ORA_MAX_RANK];
  int plain;
  int es;
} opctx_t;

static void opctx_init(opctx_t* c, const ora_operand_t* a) {
  c->op = a;
  c->plain = a->ntf == 0;
  c->es = ora_dtype_size(a->dtype);
  axis_strides(a->base_shape, a->base_rank, c->st);
}

static inline int64_t opctx_index(const opctx_t* c, const int64_t* coord) {
  if (c->plain) {
    int64_t idx = 0;
    for (int i = 0; i < c->op->base_rank; i++) idx += coord[i] * c->st[i];
    return idx;
  }
  int64_t idx;
  ora_operand_offset(c->op, coord, &idx);
  return idx;
}

/* LexIterator#advance! (src/iterators/lex_iterator.cr:13-25) over a cover region */
static inline void lex_advance(int64_t* coord, const int64_t* shape, int rank) {
  for (int i = rank - 1; i >= 0; i--) {
    if (coord[i] == shape[i] - 1) {
      coord[i] = 0;
      if (i == 0) return;
    } else {
      coord[i] += 1;
      return;
    }
  }
}

/* ================================================================ threads */

typedef struct {
  void (*fn)(void* arg, int64_t lo, int64_t hi);
  void* arg;
  int64_t lo, hi;
} job_t;

static void* job_run(void* p) {
  job_t* j = (job_t*)p;
  j->fn(j->arg, j->lo, j->hi);
  return NULL;
}

static void parallel_for(int64_t n, int nthreads, void (*fn)(void*, int64_t, int64_t), void* arg) {
  if (n <= 0) return;
  if (nthreads <= 1 || n < 4096) {
    fn(arg, 0, n);
    return;
  }
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  job_t jobs[256];
  for (int t = 0; t < nthreads; t++) {
    jobs[t].fn = fn;
    jobs[t].arg = arg;
    jobs[t].lo = n * t / nthreads;
    jobs[t].hi = n * (t + 1) / nthreads;
    pthread_create(&th[t], NULL, job_run, &jobs[t]);
  }
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* parallel_for over the piece [lo, hi) of an index range */
typedef struct {
  void (*fn)(void*, int64_t, int64_t);
  void* arg;
  int64_t base;
} offset_arg_t;

static void offset_piece(void* p, int64_t lo, int64_t hi) {
  offset_arg_t* o = (offset_arg_t*)p;
  o->fn(o->arg, o->base + lo, o->base + hi);
}

static void parallel_for_range(int64_t lo, int64_t hi, int nthreads, void (*fn)(void*, int64_t, int64_t),
                               void* arg) {
  offset_arg_t o = {fn, arg, lo};
  parallel_for(hi - lo, nthreads, offset_piece, &o);
}

/* ================================================================= gather */

typedef struct {
  const ora_operand_t* a;
  char* out;
} gather_arg_t;

static void gather_piece(void* p, int64_t lo, int64_t hi) {
  gather_arg_t* g = (gather_arg_t*)p;
  opctx_t c;
  opctx_init(&c, g->a);
  int64_t coord[ORA_MAX_RANK];
  index_to_coord(lo, g->a->shape, g->a->rank, coord);
  const char* src = (const char*)g->a->buf;
  for (int64_t i = lo; i < hi; i++) {
    int64_t idx = opctx_index(&c, coord);
    memcpy(g->out + i * c.es, src + idx * c.es, c.es);
    lex_advance(coord, g->a->shape, g->a->rank);
  }
}

/* View#to_narr (src/view.cr:123-126): NArray.build(shape) { unsafe_fetch_element(coord) } */
int ora_gather(const ora_operand_t* a, void* out, int nthreads) {
  int64_t n = shape_size(a->shape, a->rank);
  gather_arg_t g = {a, (char*)out};
  parallel_for(n, nthreads, gather_piece, &g);
  return ORA_OK;
}

/* The elements [lo, hi) (lexicographic positions) of ora_gather's output,
 * written at their positions in `out`: a slab of the same operation for a
 * bounded timing sample. */
int ora_gather_range(const ora_operand_t* a, void* out, int64_t lo, int64_t hi, int nthreads) {
  int64_t n = shape_size(a->shape, a->rank);
  if (lo < 0 || hi > n || lo > hi) return ORA_ERR_INDEX;
  gather_arg_t g = {a, (char*)out};
  parallel_for_range(lo, hi, nthreads, gather_piece, &g);
  return ORA_OK;
}

typedef struct {
  const char* buf;
  int es;
  const int64_t* shape;
  int rank;
  const ora_region_t* region;
  char* out;
} chunk_arg_t;

static void chunk_piece(void* p, int64_t lo, int64_t hi) {
  chunk_arg_t* g = (chunk_arg_t*)p;
  const ora_region_t* r = g->region;
  int rank = r->rank;
  int64_t bst[ORA_MAX_RANK], coord[ORA_MAX_RANK], local[ORA_MAX_RANK];
  axis_strides(g->shape, g->rank, bst);
  /* position the odometer at lexicographic element `lo` of the region */
  index_to_coord(lo, r->shape, rank, local);
  int64_t bidx = 0;
  for (int i = 0; i < rank; i++) {
    coord[i] = r->first[i] + local[i] * r->step[i];
    bidx += bst[i] * coord[i];
  }
  for (int64_t i = lo; i < hi; i++) {
    memcpy(g->out + i * g->es, g->buf + bidx * g->es, g->es);
    /* Indexed::LexIterator#advance! (src/buffered/indexed/lex_iterator.cr:7-21) */
    for (int d = rank - 1; d >= 0; d--) {
      if (coord[d] == r->last[d]) {
        bidx -= (coord[d] - r->first[d]) * bst[d];
        coord[d] = r->first[d];
        if (d == 0) break;
      } else {
        coord[d] += r->step[d];
        bidx += bst[d] * r->step[d];
        break;
      }
    }
  }
}

/* NArray#unsafe_fetch_chunk (src/n_array.cr:450-453) with the indexed
 * odometer of src/buffered/indexed/stride_iterator.cr:10-22 */
int ora_narray_fetch_chunk(const void* buf, int dtype, const int64_t* shape, int rank,
                           const ora_region_t* region, void* out, int nthreads) {
  if (region->rank != rank) return ORA_ERR_DIM;
  int64_t n = shape_size(region->shape, region->rank);
  for (int i = 0; i < rank; i++)
    if (region->shape[i] == 0) n = 0;
  chunk_arg_t g = {(const char*)buf, ora_dtype_size(dtype), shape, rank, region, (char*)out};
  parallel_for(n, nthreads, chunk_piece, &g);
  return ORA_OK;
}

/* NArray#unsafe_set_chunk(region, src) (src/n_array.cr:484-492) */
int ora_narray_set_chunk(void* buf, int dtype, const int64_t* shape, int rank,
                         const ora_region_t* region, const void* src_lex) {
  if (region->rank != rank) return ORA_ERR_DIM;
  int es = ora_dtype_size(dtype);
  int64_t n = shape_size(region->shape, rank);
  for (int i = 0; i < rank; i++)
    if (region->shape[i] == 0) n = 0;
  int64_t bst[ORA_MAX_RANK], coord[ORA_MAX_RANK];
  axis_strides(shape, rank, bst);
  int64_t bidx = 0;
  for (int i = 0; i < rank; i++) {
    coord[i] = region->first[i];
    bidx += bst[i] * coord[i];
  }
  char* b = (char*)buf;
  const char* s = (const char*)src_lex;
  for (int64_t i = 0; i < n; i++) {
    memcpy(b + bidx * es, s + i * es, es);
    for (int d = rank - 1; d >= 0; d--) {
      if (coord[d] == region->last[d]) {
        bidx -= (coord[d] - region->first[d]) * bst[d];
        coord[d] = region->first[d];
        if (d == 0) break;
      } else {
        coord[d] += region->step[d];
        bidx += bst[d] * region->step[d];
        break;
      }
    }
  }
  return ORA_OK;
}

/* NArray#unsafe_set_chunk(region, value) (src/n_array.cr:495-500) */
int ora_narray_set_chunk_scalar(void* buf, int dtype, const int64_t* shape, int rank,
                                const ora_region_t* region, const void* value) {
  if (region->rank != rank) return ORA_ERR_DIM;
  int es = ora_dtype_size(dtype);
  int64_t n = shape_size(region->shape, rank);
  for (int i = 0; i < rank; i++)
    if (region->shape[i] == 0) n = 0;
  int64_t bst[ORA_MAX_RANK], coord[ORA_MAX_RANK];
  axis_strides(shape, rank, bst);
  int64_t bidx = 0;
  for (int i = 0; i < rank; i++) {
    coord[i] = region->first[i];
    bidx += bst[i] * coord[i];
  }
  char* b = (char*)buf;
  for (int64_t i = 0; i < n; i++) {
    memcpy(b + bidx * es, value, es);
    for (int d = rank - 1; d >= 0; d--) {
      if (coord[d] == region->last[d]) {
        bidx -= (coord[d] - region->first[d]) * bst[d];
        coord[d] = region->first[d];
        if (d == 0) break;
      } else {
        coord[d] += region->step[d];
        bidx += bst[d] * region->step[d];
        break;
      }
    }
  }
  return ORA_OK;
}

/* MultiWritable#unsafe_set_chunk(region, src) through a MutableView:
 * src.each zipped with the destination's lexicographic coordinates
 * (src/multi_writable.cr:29-36; src/mutable_view.cr:16-18).  Writes happen one
 * element at a time in lexicographic order, so a source that aliases the
 * destination observes earlier writes, exactly as in the reference. */
int ora_scatter(const ora_operand_t* dst, const ora_operand_t* src) {
  int64_t n = shape_size(dst->shape, dst->rank);
  int64_t ns = shape_size(src->shape, src->rank);
  if (!ora_compatible_shapes(src->shape, src->rank, dst->shape, dst->rank)) return ORA_ERR_SHAPE;
  if (n != ns) return ORA_ERR_SHAPE;
  opctx_t cd, cs;
  opctx_init(&cd, dst);
  opctx_init(&cs, src);
  if (cd.es != cs.es) return ORA_ERR_UNSUPPORTED;
  int64_t dc[ORA_MAX_RANK] = {0}, sc[ORA_MAX_RANK] = {0};
  char* d = (char*)dst->buf;
  const char* s = (const char*)src->buf;
  for (int64_t i = 0; i < n; i++) {
    int64_t si = opctx_index(&cs, sc);
    int64_t di = opctx_index(&cd, dc);
    memmove(d + di * cd.es, s + si * cs.es, cd.es);
    lex_advance(sc, src->shape, src->rank);
    lex_advance(dc, dst->shape, dst->rank);
  }
  return ORA_OK;
}

/* The writes [lo, hi) of ora_scatter, split over threads: only for a source
 * that does not alias the destination (element order is then irrelevant);
 * a slab of the same operation for a bounded timing sample. */
typedef struct {
  const ora_operand_t *dst, *src;
} scatter_arg_t;

static void scatter_piece(void* p, int64_t lo, int64_t hi) {
  scatter_arg_t* a = (scatter_arg_t*)p;
  opctx_t cd, cs;
  opctx_init(&cd, a->dst);
  opctx_init(&cs, a->src);
  int64_t dc[ORA_MAX_RANK], sc[ORA_MAX_RANK];
  index_to_coord(lo, a->dst->shape, a->dst->rank, dc);
  index_to_coord(lo, a->src->shape, a->src->rank, sc);
  char* d = (char*)a->dst->buf;
  const char* s = (const char*)a->src->buf;
  for (int64_t i = lo; i < hi; i++) {
    memcpy(d + opctx_index(&cd, dc) * cd.es, s + opctx_index(&cs, sc) * cs.es, cd.es);
    lex_advance(sc, a->src->shape, a->src->rank);
    lex_advance(dc, a->dst->shape, a->dst->rank);
  }
}

int ora_scatter_range(const ora_operand_t* dst, const ora_operand_t* src, int64_t lo, int64_t hi, int nthreads) {
  int64_t n = shape_size(dst->shape, dst->rank);
  if (!ora_compatible_shapes(src->shape, src->rank, dst->shape, dst->rank)) return ORA_ERR_SHAPE;
  if (n != shape_size(src->shape, src->rank)) return ORA_ERR_SHAPE;
  if (ora_dtype_size(dst->dtype) != ora_dtype_size(src->dtype)) return ORA_ERR_UNSUPPORTED;
  if (lo < 0 || hi > n || lo > hi) return ORA_ERR_INDEX;
  scatter_arg_t a = {dst, src};
  parallel_for_range(lo, hi, nthreads, scatter_piece, &a);
  return ORA_OK;
}

/* MultiWritable#unsafe_set_chunk(region, value) (src/multi_writable.cr:40-44) */
int ora_scatter_scalar(const ora_operand_t* dst, const void* value) {
  int64_t n = shape_size(dst->shape, dst->rank);
  opctx_t cd;
  opctx_init(&cd, dst);
  int64_t dc[ORA_MAX_RANK] = {0};
  char* d = (char*)dst->buf;
  for (int64_t i = 0; i < n; i++) {
    int64_t di = opctx_index(&cd, dc);
    memcpy(d + di * cd.es, value, cd.es);
    lex_advance(dc, dst->shape, dst->rank);
  }
  return ORA_OK;
}

/* ======================================================= number semantics */
/*
 * Crystal 1.0 stdlib number semantics (not vendored in the reference; the
 * reference reaches them through `elem.{{name.id}} other_elem`,
 * src/multi_indexable.cr:943,950 and src/patches/number.cr:12).  Stated
 * assumptions:
 *  - Int `+ - *` are checked: overflow raises OverflowError; `&+ &- &*` wrap.
 *  - Int / Int -> Float64 (both converted to Float64, IEEE division).
 *  - Int // Int floors; zero divisor -> DivisionByZeroError; MIN // -1 -> OverflowError.
 *  - Int % Int is the floored modulo (sign of the divisor); zero divisor raises;
 *    MIN % -1 == 0.
 *  - Int ** Int: exponent < 0 -> ArgumentError; binary exponentiation with
 *    checked multiplies (`&**` wraps).
 *  - Float // Float = floor(a / b); Float % Float = a - b * floor(a / b), zero
 *    divisor raises DivisionByZeroError.
 *  - Float ** Int is LLVM powi: binary exponentiation (compiler-rt __powisf2
 *    method, restated below), x ** 2 == x * x.  Float ** Float is libm pow.
 *  - Mixed Float32/Int -> Float32; anything with Float64 -> Float64; mixed
 *    Int32/Int64 -> the receiver's type; comparisons -> Bool; <=> -> Int32
 *    (NaN compares as 0).
 */

typedef union {
  int64_t i;
  double f;
} val_t;

static val_t load_val(const void* p, int dtype) {
  val_t v;
  switch (dtype) {
    case ORA_BOOL: v.i = *(const uint8_t*)p ? 1 : 0; break;
    case ORA_I32: v.i = *(const int32_t*)p; break;
    case ORA_I64: v.i = *(const int64_t*)p; break;
    case ORA_F32: v.f = *(const float*)p; break;
    case ORA_F64: v.f = *(const double*)p; break;
    default: v.i = 0;
  }
  return v;
}

static int is_float(int t) { return t == ORA_F32 || t == ORA_F64; }
static int is_int(int t) { return t == ORA_I32 || t == ORA_I64; }

int ora_result_dtype(int op, int ta, int tb, int* tout) {
  if (ta == ORA_BOOL || tb == ORA_BOOL) {
    if (ta == ORA_BOOL && tb == ORA_BOOL &&
        (op == ORA_OP_AND || op == ORA_OP_OR || op == ORA_OP_XOR || op == ORA_OP_EQ)) {
      *tout = ORA_BOOL;
      return ORA_OK;
    }
    if (op == ORA_OP_EQ) { *tout = ORA_BOOL; return ORA_OK; }
    return ORA_ERR_UNSUPPORTED;
  }
  if (op == ORA_OP_GT || op == ORA_OP_LT || op == ORA_OP_GE || op == ORA_OP_LE || op == ORA_OP_EQ) {
    *tout = ORA_BOOL;
    return ORA_OK;
  }
  if (op == ORA_OP_CMP) { *tout = ORA_I32; return ORA_OK; }
  if (op == ORA_OP_AND || op == ORA_OP_OR || op == ORA_OP_XOR) {
    if (!is_int(ta) || !is_int(tb)) return ORA_ERR_UNSUPPORTED;
    *tout = ta;
    return ORA_OK;
  }
  if (is_int(ta) && is_int(tb)) {
    *tout = (op == ORA_OP_DIV) ? ORA_F64 : ta;
    return ORA_OK;
  }
  if (op == ORA_OP_WADD || op == ORA_OP_WSUB || op == ORA_OP_WMUL || op == ORA_OP_WPOW)
    return ORA_ERR_UNSUPPORTED;
  if (is_int(ta) && is_float(tb) && op == ORA_OP_POW) { *tout = ORA_F64; return ORA_OK; }
  *tout = (ta == ORA_F64 || tb == ORA_F64) ? ORA_F64 : ORA_F32;
  return ORA_OK;
}

/* compiler-rt's __powisf2 / __powidf2 method: binary exponentiation, reciprocal
 * for negative exponents (restated from its published description). */
static float powi_f32(float a, int32_t b) {
  int recip = b < 0;
  float r = 1.0f;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0f / r : r;
}
static double powi_f64(double a, int32_t b) {
  int recip = b < 0;
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

static int fits(int64_t x, int t) {
  if (t == ORA_I32) return x >= INT32_MIN && x <= INT32_MAX;
  return 1;
}

static int64_t wrap(int64_t x, int t) {
  if (t == ORA_I32) return (int64_t)(int32_t)(uint32_t)(uint64_t)x;
  return x;
}

/* checked integer helpers in the width of type t */
static int64_t iadd(int64_t a, int64_t b, int t, uint32_t* st) {
  if (t == ORA_I32) {
    int64_t r = a + b;
    if (!fits(r, t)) *st |= ORA_ST_OVERFLOW;
    return wrap(r, t);
  }
  int64_t r;
  if (__builtin_add_overflow(a, b, &r)) *st |= ORA_ST_OVERFLOW;
  return r;
}
static int64_t isub(int64_t a, int64_t b, int t, uint32_t* st) {
  if (t == ORA_I32) {
    int64_t r = a - b;
    if (!fits(r, t)) *st |= ORA_ST_OVERFLOW;
    return wrap(r, t);
  }
  int64_t r;
  if (__builtin_sub_overflow(a, b, &r)) *st |= ORA_ST_OVERFLOW;
  return r;
}
static int64_t imul(int64_t a, int64_t b, int t, uint32_t* st) {
  if (t == ORA_I32) {
    int64_t r = a * b;
    if (!fits(r, t)) *st |= ORA_ST_OVERFLOW;
    return wrap(r, t);
  }
  int64_t r;
  if (__builtin_mul_overflow(a, b, &r)) *st |= ORA_ST_OVERFLOW;
  return r;
}
static int64_t wadd(int64_t a, int64_t b, int t) { return wrap((int64_t)((uint64_t)a + (uint64_t)b), t); }
static int64_t wsub(int64_t a, int64_t b, int t) { return wrap((int64_t)((uint64_t)a - (uint64_t)b), t); }
static int64_t wmul(int64_t a, int64_t b, int t) { return wrap((int64_t)((uint64_t)a * (uint64_t)b), t); }

/* Int#** (checked) / Int#&** (wrapping): binary exponentiation */
static int64_t ipow(int64_t base, int64_t e, int t, int wrapping, uint32_t* st) {
  if (e < 0) {
    *st |= ORA_ST_ARGUMENT;
    return 0;
  }
  int64_t result = 1, k = base;
  while (e > 0) {
    if (e & 1) result = wrapping ? wmul(result, k, t) : imul(result, k, t, st);
    e >>= 1;
    if (e > 0) k = wrapping ? wmul(k, k, t) : imul(k, k, t, st);
  }
  return result;
}

static int64_t int_min(int t) { return t == ORA_I32 ? (int64_t)INT32_MIN : INT64_MIN; }

static val_t apply_binary(int op, val_t a, int ta, val_t b, int tb, int tout, uint32_t* st) {
  val_t r;
  r.i = 0;
  if (ta == ORA_BOOL && tb == ORA_BOOL) {
    switch (op) {
      case ORA_OP_AND: r.i = a.i & b.i; break;
      case ORA_OP_OR: r.i = a.i | b.i; break;
      case ORA_OP_XOR: r.i = a.i ^ b.i; break;
      case ORA_OP_EQ: r.i = a.i == b.i; break;
    }
    return r;
  }
  if (ta == ORA_BOOL || tb == ORA_BOOL) { r.i = 0; return r; } /* Bool == number -> false */
  int both_int = is_int(ta) && is_int(tb);
  if (both_int) {
    int t = ta; /* receiver type */
    int64_t x = a.i, y = b.i;
    switch (op) {
      case ORA_OP_ADD: r.i = iadd(x, y, t, st); break;
      case ORA_OP_SUB: r.i = isub(x, y, t, st); break;
      case ORA_OP_MUL: r.i = imul(x, y, t, st); break;
      case ORA_OP_DIV: r.f = (double)x / (double)y; break;
      case ORA_OP_FLOORDIV:
        if (y == 0) { *st |= ORA_ST_DIVZERO; r.i = 0; break; }
        if (x == int_min(t) && y == -1) { *st |= ORA_ST_OVERFLOW; r.i = x; break; }
        r.i = floordiv64(x, y);
        break;
      case ORA_OP_MOD:
        if (y == 0) { *st |= ORA_ST_DIVZERO; r.i = 0; break; }
        if (y == -1) { r.i = 0; break; }
        r.i = floormod64(x, y);
        break;
      case ORA_OP_POW: r.i = ipow(x, y, t, 0, st); break;
      case ORA_OP_WADD: r.i = wadd(x, y, t); break;
      case ORA_OP_WSUB: r.i = wsub(x, y, t); break;
      case ORA_OP_WMUL: r.i = wmul(x, y, t); break;
      case ORA_OP_WPOW: r.i = ipow(x, y, t, 1, st); break;
      case ORA_OP_AND: r.i = wrap(x & y, t); break;
      case ORA_OP_OR: r.i = wrap(x | y, t); break;
      case ORA_OP_XOR: r.i = wrap(x ^ y, t); break;
      case ORA_OP_GT: r.i = x > y; break;
      case ORA_OP_LT: r.i = x < y; break;
      case ORA_OP_GE: r.i = x >= y; break;
      case ORA_OP_LE: r.i = x <= y; break;
      case ORA_OP_EQ: r.i = x == y; break;
      case ORA_OP_CMP: r.i = cmp64(x, y); break;
    }
    return r;
  }
  /* at least one float operand */
  if (op == ORA_OP_POW && is_float(ta) && is_int(tb)) {
    if (ta == ORA_F32) r.f = (double)powi_f32((float)a.f, (int32_t)b.i);
    else r.f = powi_f64(a.f, (int32_t)b.i);
    return r;
  }
  if (tout == ORA_F32 || (tout == ORA_BOOL && ta != ORA_F64 && tb != ORA_F64) ||
      (tout == ORA_I32 && ta != ORA_F64 && tb != ORA_F64)) {
    float x = is_int(ta) ? (float)a.i : (float)a.f;
    float y = is_int(tb) ? (float)b.i : (float)b.f;
    float z = 0.0f;
    switch (op) {
      case ORA_OP_ADD: z = x + y; break;
      case ORA_OP_SUB: z = x - y; break;
      case ORA_OP_MUL: z = x * y; break;
      case ORA_OP_DIV: z = x / y; break;
      case ORA_OP_FLOORDIV: z = floorf(x / y); break;
      case ORA_OP_MOD: {
        if (y == 0.0f) { *st |= ORA_ST_DIVZERO; z = 0.0f; break; }
        float q = floorf(x / y);
        float m = y * q;
        z = x - m;
        break;
      }
      case ORA_OP_POW: z = powf(x, y); break;
      case ORA_OP_GT: r.i = x > y; return r;
      case ORA_OP_LT: r.i = x < y; return r;
      case ORA_OP_GE: r.i = x >= y; return r;
      case ORA_OP_LE: r.i = x <= y; return r;
      case ORA_OP_EQ: r.i = x == y; return r;
      case ORA_OP_CMP: r.i = (x > y) - (x < y); return r;
    }
    r.f = (double)z;
    return r;
  }
  {
    double x = is_int(ta) ? (double)a.i : a.f;
    double y = is_int(tb) ? (double)b.i : b.f;
    double z = 0.0;
    switch (op) {
      case ORA_OP_ADD: z = x + y; break;
      case ORA_OP_SUB: z = x - y; break;
      case ORA_OP_MUL: z = x * y; break;
      case ORA_OP_DIV: z = x / y; break;
      case ORA_OP_FLOORDIV: z = floor(x / y); break;
      case ORA_OP_MOD: {
        if (y == 0.0) { *st |= ORA_ST_DIVZERO; z = 0.0; break; }
        double q = floor(x / y);
        double m = y * q;
        z = x - m;
        break;
      }
      case ORA_OP_POW: z = pow(x, y); break;
      case ORA_OP_GT: r.i = x > y; return r;
      case ORA_OP_LT: r.i = x < y; return r;
      case ORA_OP_GE: r.i = x >= y; return r;
      case ORA_OP_LE: r.i = x <= y; return r;
      case ORA_OP_EQ: r.i = x == y; return r;
      case ORA_OP_CMP: r.i = (x > y) - (x < y); return r;
    }
    r.f = z;
    return r;
  }
}

static void store_val(void* p, int dtype, val_t v) {
  switch (dtype) {
    case ORA_BOOL: *(uint8_t*)p = v.i ? 1 : 0; break;
    case ORA_I32: *(int32_t*)p = (int32_t)v.i; break;
    case ORA_I64: *(int64_t*)p = v.i; break;
    case ORA_F32: *(float*)p = (float)v.f; break;
    case ORA_F64: *(double*)p = v.f; break;
  }
}

typedef struct {
  int op;
  const ora_operand_t* a;
  const ora_operand_t* b; /* NULL for scalar */
  val_t scalar;
  int scalar_dtype, scalar_left;
  int tout;
  char* out;
  uint32_t status;
  pthread_mutex_t mu;
} map_arg_t;

static void map_piece(void* p, int64_t lo, int64_t hi) {
  map_arg_t* m = (map_arg_t*)p;
  opctx_t ca, cb;
  opctx_init(&ca, m->a);
  if (m->b) opctx_init(&cb, m->b);
  int oes = ora_dtype_size(m->tout);
  int64_t coord[ORA_MAX_RANK];
  index_to_coord(lo, m->a->shape, m->a->rank, coord);
  const char* abuf = (const char*)m->a->buf;
  const char* bbuf = m->b ? (const char*)m->b->buf : NULL;
  uint32_t st = 0;
  int ta = m->a->dtype;
  for (int64_t i = lo; i < hi; i++) {
    /* MultiIndexable.each_with (src/multi_indexable.cr:1080-1102): every
     * operand is fetched at the same lexicographic coordinate */
    val_t x = load_val(abuf + opctx_index(&ca, coord) * ca.es, ta);
    val_t r;
    if (m->b) {
      val_t y = load_val(bbuf + opctx_index(&cb, coord) * cb.es, m->b->dtype);
      r = apply_binary(m->op, x, ta, y, m->b->dtype, m->tout, &st);
    } else if (m->scalar_left) {
      r = apply_binary(m->op, m->scalar, m->scalar_dtype, x, ta, m->tout, &st);
    } else {
      r = apply_binary(m->op, x, ta, m->scalar, m->scalar_dtype, m->tout, &st);
    }
    store_val(m->out + i * oes, m->tout, r);
    lex_advance(coord, m->a->shape, m->a->rank);
  }
  pthread_mutex_lock(&m->mu);
  m->status |= st;
  pthread_mutex_unlock(&m->mu);
}

/* def_elementwise_binary -> map_with (src/multi_indexable.cr:931-945, 1026-1078) */
int ora_map_binary(int op, const ora_operand_t* a, const ora_operand_t* b, void* out,
                   uint32_t* status, int nthreads) {
  if (a->rank != b->rank) return ORA_ERR_SHAPE;
  for (int i = 0; i < a->rank; i++)
    if (a->shape[i] != b->shape[i]) return ORA_ERR_SHAPE;
  int tout;
  int rc = ora_result_dtype(op, a->dtype, b->dtype, &tout);
  if (rc) return rc;
  map_arg_t m;
  memset(&m, 0, sizeof(m));
  m.op = op; m.a = a; m.b = b; m.tout = tout; m.out = (char*)out;
  pthread_mutex_init(&m.mu, NULL);
  parallel_for(shape_size(a->shape, a->rank), nthreads, map_piece, &m);
  pthread_mutex_destroy(&m.mu);
  *status = m.status;
  return ORA_OK;
}

/* The elements [lo, hi) of ora_map_binary's output (a timing slab). */
int ora_map_binary_range(int op, const ora_operand_t* a, const ora_operand_t* b, void* out, int64_t lo, int64_t hi,
                         uint32_t* status, int nthreads) {
  if (a->rank != b->rank) return ORA_ERR_SHAPE;
  for (int i = 0; i < a->rank; i++)
    if (a->shape[i] != b->shape[i]) return ORA_ERR_SHAPE;
  if (lo < 0 || hi > shape_size(a->shape, a->rank) || lo > hi) return ORA_ERR_INDEX;
  int tout;
  int rc = ora_result_dtype(op, a->dtype, b->dtype, &tout);
  if (rc) return rc;
  map_arg_t m;
  memset(&m, 0, sizeof(m));
  m.op = op; m.a = a; m.b = b; m.tout = tout; m.out = (char*)out;
  pthread_mutex_init(&m.mu, NULL);
  parallel_for_range(lo, hi, nthreads, map_piece, &m);
  pthread_mutex_destroy(&m.mu);
  *status = m.status;
  return ORA_OK;
}

/* `narr <op> scalar` -> map (multi_indexable.cr:949-951, n_array.cr:589-595);
 * `scalar <op> narr` (src/patches/number.cr:9-13) */
int ora_map_binary_scalar(int op, const ora_operand_t* a, const void* scalar, int scalar_dtype,
                          int scalar_left, void* out, uint32_t* status, int nthreads) {
  int tout;
  int rc = scalar_left ? ora_result_dtype(op, scalar_dtype, a->dtype, &tout)
                       : ora_result_dtype(op, a->dtype, scalar_dtype, &tout);
  if (rc) return rc;
  map_arg_t m;
  memset(&m, 0, sizeof(m));
  m.op = op; m.a = a; m.b = NULL; m.tout = tout; m.out = (char*)out;
  m.scalar = load_val(scalar, scalar_dtype);
  m.scalar_dtype = scalar_dtype;
  m.scalar_left = scalar_left;
  pthread_mutex_init(&m.mu, NULL);
  parallel_for(shape_size(a->shape, a->rank), nthreads, map_piece, &m);
  pthread_mutex_destroy(&m.mu);
  *status = m.status;
  return ORA_OK;
}

/* def_elementwise_unary (src/multi_indexable.cr:947-955, 983-985) */
int ora_map_unary(int uop, const ora_operand_t* a, void* out, uint32_t* status) {
  int t = a->dtype;
  if (uop == ORA_UOP_NOT && !is_int(t)) return ORA_ERR_UNSUPPORTED;
  if (t == ORA_BOOL) return ORA_ERR_UNSUPPORTED;
  opctx_t ca;
  opctx_init(&ca, a);
  int64_t n = shape_size(a->shape, a->rank);
  int64_t coord[ORA_MAX_RANK] = {0};
  uint32_t st = 0;
  for (int64_t i = 0; i < n; i++) {
    val_t x = load_val((const char*)a->buf + opctx_index(&ca, coord) * ca.es, t);
    val_t r = x;
    if (uop == ORA_UOP_NEG) {
      if (is_int(t)) {
        if (x.i == int_min(t)) { st |= ORA_ST_OVERFLOW; r.i = x.i; }
        else r.i = -x.i;
      } else if (t == ORA_F32) {
        r.f = (double)(-(float)x.f);
      } else {
        r.f = -x.f;
      }
    } else if (uop == ORA_UOP_NOT) {
      r.i = wrap(~x.i, t);
    }
    store_val((char*)out + i * ca.es, t, r);
    lex_advance(coord, a->shape, a->rank);
  }
  *status = st;
  return ORA_OK;
}

int ora_cast(const void* in, int tin, void* out, int tout, int64_t n) {
  int ei = ora_dtype_size(tin), eo = ora_dtype_size(tout);
  for (int64_t i = 0; i < n; i++) {
    val_t v = load_val((const char*)in + i * ei, tin);
    val_t r;
    if (is_int(tin) && is_float(tout)) r.f = tout == ORA_F32 ? (double)(float)v.i : (double)v.i;
    else if (is_float(tin) && is_int(tout)) r.i = (int64_t)v.f;
    else r = v;
    store_val((char*)out + i * eo, tout, r);
  }
  return ORA_OK;
}

/* ============================================================= reductions */

/*
 * The reference has no reduction API of its own: `sum`/`max`/`min` come from
 * Crystal's Enumerable (included at src/multi_indexable.cr:18, iterating `each`
 * in lexicographic order, :656-658), an axis reduction in Phase style is a left
 * fold over `slices(axis)` (src/multi_indexable.cr:742-786), and argmax is the
 * README idiom (README.md:56-61): start at the first element and replace only
 * on strict `>`, so the first maximum wins and NaNs never win unless the first
 * element is NaN.
 *
 * For axis k the output has the input shape without axis k (lexicographic);
 * output element o folds the elements along k in increasing index order.
 */
static void red_geometry(const int64_t* shape, int rank, int axis, int64_t* outer, int64_t* K,
                         int64_t* inner) {
  int64_t o = 1, in = 1;
  for (int i = 0; i < axis; i++) o *= shape[i];
  for (int i = axis + 1; i < rank; i++) in *= shape[i];
  *outer = o;
  *K = shape[axis];
  *inner = in;
}

int ora_reduce(int op, const void* in, int dtype, const int64_t* shape, int rank, int axis,
               void* out, int out_dtype) {
  int64_t outer, K, inner;
  if (axis < 0) {
    outer = 1;
    K = shape_size(shape, rank);
    inner = 1;
  } else {
    if (axis >= rank) return ORA_ERR_INDEX;
    red_geometry(shape, rank, axis, &outer, &K, &inner);
  }
  int es = ora_dtype_size(dtype), oes = ora_dtype_size(out_dtype);
  const char* src = (const char*)in;
  int isf = is_float(dtype);
  if (K == 0 && op != ORA_RED_SUM) return ORA_ERR_EMPTY;
  uint32_t st = 0;
  for (int64_t o = 0; o < outer; o++) {
    for (int64_t j = 0; j < inner; j++) {
      const char* base = src + (o * K * inner + j) * es;
      val_t r;
      if (op == ORA_RED_SUM) {
        if (isf) {
          if (dtype == ORA_F32) {
            float acc = 0.0f; /* sequential FP32 left fold (Enumerable#sum) */
            for (int64_t k = 0; k < K; k++) acc = acc + *(const float*)(base + k * inner * es);
            r.f = acc;
          } else {
            double acc = 0.0;
            for (int64_t k = 0; k < K; k++) acc = acc + *(const double*)(base + k * inner * es);
            r.f = acc;
          }
        } else {
          int64_t acc = 0;
          for (int64_t k = 0; k < K; k++)
            acc = iadd(acc, load_val(base + k * inner * es, dtype).i, dtype, &st);
          r.i = acc;
        }
        store_val((char*)out + (o * inner + j) * oes, out_dtype, r);
      } else {
        int want_max = (op == ORA_RED_MAX || op == ORA_RED_ARGMAX);
        val_t best = load_val(base, dtype);
        int64_t bi = 0;
        for (int64_t k = 1; k < K; k++) {
          val_t v = load_val(base + k * inner * es, dtype);
          int better;
          if (isf) better = want_max ? (v.f > best.f) : (v.f < best.f);
          else better = want_max ? (v.i > best.i) : (v.i < best.i);
          if (better) { best = v; bi = k; }
        }
        if (op == ORA_RED_ARGMAX || op == ORA_RED_ARGMIN) {
          val_t iv;
          iv.i = bi;
          store_val((char*)out + (o * inner + j) * oes, out_dtype, iv);
        } else {
          store_val((char*)out + (o * inner + j) * oes, out_dtype, best);
        }
      }
    }
  }
  if (st & ORA_ST_OVERFLOW) return ORA_ERR_OVERFLOW;
  return ORA_OK;
}

/* FP64 oracle for sums: every FP32 input is exact in double; the terms are
 * accumulated in double with Neumaier compensation, so the result is the
 * exact sum to within a few ulps of double. */
int ora_reduce_f64(const void* in, int dtype, const int64_t* shape, int rank, int axis,
                   double* out) {
  int64_t outer, K, inner;
  if (axis < 0) {
    outer = 1;
    K = shape_size(shape, rank);
    inner = 1;
  } else {
    if (axis >= rank) return ORA_ERR_INDEX;
    red_geometry(shape, rank, axis, &outer, &K, &inner);
  }
  int es = ora_dtype_size(dtype);
  const char* src = (const char*)in;
  for (int64_t o = 0; o < outer; o++) {
    for (int64_t j = 0; j < inner; j++) {
      const char* base = src + (o * K * inner + j) * es;
      double s = 0.0, c = 0.0;
      for (int64_t k = 0; k < K; k++) {
        val_t v = load_val(base + k * inner * es, dtype);
        double x = is_float(dtype) ? v.f : (double)v.i;
        double t = s + x;
        if (fabs(s) >= fabs(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
      }
      out[o * inner + j] = s + c;
    }
  }
  return ORA_OK;
}

/* ================================================================== heat */

/* One step of the Phase heat program on an n x m grid:
 *   c   = u[1..-2, 1..-2]
 *   lap = u[0..-3, 1..-2] + u[2.., 1..-2] + u[1..-2, 0..-3] + u[1..-2, 2..] - c * 4
 *   u[1..-2, 1..-2] = c + lap * coef
 * Each infix op is evaluated left to right in the element type
 * (examples/heat_equation.cr:38-51 pattern generalised to 2-D). */
typedef struct {
  const void* u;
  void* out;
  int64_t n, m;
  double coef;
  int f64;
} heat_arg_t;

static void heat_rows(void* p, int64_t lo, int64_t hi) {
  heat_arg_t* h = (heat_arg_t*)p;
  int64_t n = h->n, m = h->m;
  for (int64_t i = lo; i < hi; i++) {
    if (h->f64) {
      const double* u = (const double*)h->u;
      double* o = (double*)h->out;
      for (int64_t j = 0; j < m; j++) {
        if (i == 0 || i == n - 1 || j == 0 || j == m - 1) { o[i * m + j] = u[i * m + j]; continue; }
        double c = u[i * m + j];
        double lap = u[(i - 1) * m + j] + u[(i + 1) * m + j];
        lap = lap + u[i * m + j - 1];
        lap = lap + u[i * m + j + 1];
        double c4 = c * 4.0;
        lap = lap - c4;
        double d = lap * h->coef;
        o[i * m + j] = c + d;
      }
    } else {
      const float* u = (const float*)h->u;
      float* o = (float*)h->out;
      float coef = (float)h->coef;
      for (int64_t j = 0; j < m; j++) {
        if (i == 0 || i == n - 1 || j == 0 || j == m - 1) { o[i * m + j] = u[i * m + j]; continue; }
        float c = u[i * m + j];
        float lap = u[(i - 1) * m + j] + u[(i + 1) * m + j];
        lap = lap + u[i * m + j - 1];
        lap = lap + u[i * m + j + 1];
        float c4 = c * 4.0f;
        lap = lap - c4;
        float d = lap * coef;
        o[i * m + j] = c + d;
      }
    }
  }
}

int ora_heat_step_f32(const float* u, float* out, int64_t n, int64_t m, float coef) {
  heat_arg_t h = {u, out, n, m, coef, 0};
  heat_rows(&h, 0, n);
  return ORA_OK;
}

int ora_heat_step_f64(const double* u, double* out, int64_t n, int64_t m, double coef) {
  heat_arg_t h = {u, out, n, m, coef, 1};
  heat_rows(&h, 0, n);
  return ORA_OK;
}

static int heat_run(void* u, void* tmp, int64_t n, int64_t m, double coef, int steps, int nthreads,
                    int f64) {
  int es = f64 ? 8 : 4;
  void* a = u;
  void* b = tmp;
  for (int s = 0; s < steps; s++) {
    heat_arg_t h = {a, b, n, m, coef, f64};
    if (nthreads > 1 && n > 64) {
      /* rows are independent within a step */
      parallel_for(n, nthreads, heat_rows, &h);
    } else {
      heat_rows(&h, 0, n);
    }
    void* t = a;
    a = b;
    b = t;
  }
  if (a != u) memcpy(u, a, (size_t)(n * m * es));
  return ORA_OK;
}

int ora_heat_run_f32(float* u, float* tmp, int64_t n, int64_t m, float coef, int steps, int nthreads) {
  return heat_run(u, tmp, n, m, coef, steps, nthreads, 0);
}

int ora_heat_run_f64(double* u, double* tmp, int64_t n, int64_t m, double coef, int steps, int nthreads) {
  return heat_run(u, tmp, n, m, coef, steps, nthreads, 1);
}

/* =================================================================== MLP */

/* Reference forward/backward of the tuner MLP in double:
 *   h1 = relu(W1 x + b1); h2 = relu(W2 h1 + b2); yhat = W3 h2 + b3
 *   loss = mean((yhat - y)^2)
 * Parameter layout (float): W1[h1][in], b1[h1], W2[h2][h1], b2[h2], W3[h2], b3[1].
 * grad has the same layout (double). */
int ora_mlp_forward_backward(const float* params, int in_dim, int h1, int h2, const float* x,
                             const float* y, int batch, double* loss, double* grad) {
  const float* W1 = params;
  const float* b1 = W1 + (size_t)h1 * in_dim;
  const float* W2 = b1 + h1;
  const float* b2 = W2 + (size_t)h2 * h1;
  const float* W3 = b2 + h2;
  const float* b3 = W3 + h2;
  size_t np = (size_t)h1 * in_dim + h1 + (size_t)h2 * h1 + h2 + h2 + 1;
  memset(grad, 0, np * sizeof(double));
  double* gW1 = grad;
  double* gb1 = gW1 + (size_t)h1 * in_dim;
  double* gW2 = gb1 + h1;
  double* gb2 = gW2 + (size_t)h2 * h1;
  double* gW3 = gb2 + h2;
  double* gb3 = gW3 + h2;
  double* a1 = (double*)malloc(sizeof(double) * h1);
  double* a2 = (double*)malloc(sizeof(double) * h2);
  double* d1 = (double*)malloc(sizeof(double) * h1);
  double* d2 = (double*)malloc(sizeof(double) * h2);
  double L = 0.0;
  for (int s = 0; s < batch; s++) {
    const float* xs = x + (size_t)s * in_dim;
    for (int i = 0; i < h1; i++) {
      double z = b1[i];
      for (int k = 0; k < in_dim; k++) z += (double)W1[(size_t)i * in_dim + k] * xs[k];
      a1[i] = z > 0 ? z : 0;
    }
    for (int i = 0; i < h2; i++) {
      double z = b2[i];
      for (int k = 0; k < h1; k++) z += (double)W2[(size_t)i * h1 + k] * a1[k];
      a2[i] = z > 0 ? z : 0;
    }
    double yh = b3[0];
    for (int k = 0; k < h2; k++) yh += (double)W3[k] * a2[k];
    double e = yh - y[s];
    L += e * e;
    double dy = 2.0 * e / batch;
    gb3[0] += dy;
    for (int k = 0; k < h2; k++) {
      gW3[k] += dy * a2[k];
      d2[k] = a2[k] > 0 ? dy * W3[k] : 0.0;
    }
    for (int i = 0; i < h2; i++) {
      gb2[i] += d2[i];
      for (int k = 0; k < h1; k++) gW2[(size_t)i * h1 + k] += d2[i] * a1[k];
    }
    for (int k = 0; k < h1; k++) {
      double acc = 0.0;
      for (int i = 0; i < h2; i++) acc += d2[i] * W2[(size_t)i * h1 + k];
      d1[k] = a1[k] > 0 ? acc : 0.0;
    }
    for (int i = 0; i < h1; i++) {
      gb1[i] += d1[i];
      for (int k = 0; k < in_dim; k++) gW1[(size_t)i * in_dim + k] += d1[i] * xs[k];
    }
  }
  *loss = L / batch;
  free(a1); free(a2); free(d1); free(d2);
  return ORA_OK;
}
