// plan.cu -- host-side view compiler.
//
// A View in the reference is a source buffer plus a chain of coordinate
// transforms applied per element (src/view.cr:109-117, src/view_util/transforms.cr).
// The caller folds Region/Permute/Reverse into one affine descriptor
// (phcu_view_t); this file turns the descriptors of one operation (output +
// inputs) into a canonical iteration space:
//   1. drop size-1 axes (lexicographic order is unchanged);
//   2. flip every axis the output walks backwards (element order is free for
//      elementwise work, so all operands flip together);
//   3. order axes by decreasing output stride (innermost = output-contiguous);
//   4. merge neighbouring axes that are contiguous for every operand;
//   5. pick ROW (inner axis shared) or TILE (inputs contiguous along another
//      axis: staged through shared memory) and per-operand vector modes.
#include <algorithm>

#include "plan.h"

namespace phcu {

int64_t view_size(const phcu_view_t* v) {
  if (v->rank == 0) return 1;  // rank-0 descriptors address one element
  int64_t n = 1;
  for (int i = 0; i < v->rank; i++) n *= v->shape[i];
  return n;
}

int32_t check_view(const phcu_view_t* v, const char* what) {
  if (!v) return fail(PHCU_ERR_INVALID, "%s: null view", what);
  if (!dtype_valid(v->dtype)) return fail(PHCU_ERR_INVALID, "%s: bad dtype %d", what, v->dtype);
  if (v->rank < 0 || v->rank > MAXR) return fail(PHCU_ERR_DIM, "%s: rank %d outside 0..%d", what, v->rank, MAXR);
  bool empty = false;
  for (int i = 0; i < v->rank; i++) {
    if (v->shape[i] < 0) return fail(PHCU_ERR_DIM, "%s: negative extent on axis %d", what, i);
    if (v->shape[i] == 0) empty = true;
  }
  if (empty) return PHCU_OK;
  // the element count, refused before the product could wrap: n * s stays
  // within the limit exactly when n <= limit / s (integer division)
  const int64_t limit = (int64_t)UINT32_MAX - 1;
  int64_t n = 1;
  for (int i = 0; i < v->rank; i++) {
    if (n > limit / v->shape[i])
      return fail(PHCU_ERR_UNSUPPORTED, "%s: more than 2^32-2 elements (the per-operation limit)", what);
    n *= v->shape[i];
  }
  if (!v->base) return fail(PHCU_ERR_INVALID, "%s: null base pointer", what);
  return PHCU_OK;
}

int32_t check_input_view(const phcu_view_t* v, const char* what) {
  if (!is_index_view(v)) return check_view(v, what);
  // an index operand: the shape rules of check_view, no storage
  phcu_view_t t = *v;
  t.dtype = PHCU_I32;
  t.base = (void*)&t;  // any non-null address: it is never read
  return check_view(&t, what);
}

void view_extent(const phcu_view_t* v, uintptr_t* lo, uintptr_t* hi) {
  int es = dtype_size(v->dtype);
  int64_t mn = v->offset, mx = v->offset;
  for (int i = 0; i < v->rank; i++) {
    if (v->shape[i] <= 0) { *lo = *hi = (uintptr_t)v->base; return; }
    int64_t span = (v->shape[i] - 1) * v->stride[i];
    if (span < 0) mn += span; else mx += span;
  }
  *lo = (uintptr_t)v->base + (uintptr_t)(mn * es);
  *hi = (uintptr_t)v->base + (uintptr_t)((mx + 1) * es);
}

bool views_overlap(const phcu_view_t* a, const phcu_view_t* b) {
  if (is_index_view(a) || is_index_view(b)) return false;  // index operands have no storage
  uintptr_t al, ah, bl, bh;
  view_extent(a, &al, &ah);
  view_extent(b, &bl, &bh);
  if (al == ah || bl == bh) return false;
  return al < bh && bl < ah;
}

bool views_identical(const phcu_view_t* a, const phcu_view_t* b) {
  if (a->base != b->base || a->offset != b->offset || a->dtype != b->dtype) return false;
  // compare the non-unit axes
  int ia = 0, ib = 0;
  for (;;) {
    while (ia < a->rank && a->shape[ia] == 1) ia++;
    while (ib < b->rank && b->shape[ib] == 1) ib++;
    if (ia == a->rank || ib == b->rank) return ia == a->rank && ib == b->rank;
    if (a->shape[ia] != b->shape[ib] || a->stride[ia] != b->stride[ib]) return false;
    ia++;
    ib++;
  }
}

namespace {

struct Axis {
  int64_t n;
  int64_t st[MAXIN + 1];
};

}  // namespace

int32_t make_plan(const phcu_view_t* out, const phcu_view_t* const* ins, int nin, EvalPlan* p,
                  int force_mode) {
  memset(p, 0, sizeof(*p));
  const int nops = nin + 1;
  const phcu_view_t* ops[MAXIN + 1];
  ops[0] = out;
  for (int k = 0; k < nin; k++) ops[k + 1] = ins[k];

  // 1. non-unit axes of every operand; shapes must agree
  int64_t shp[MAXIN + 1][MAXR], str[MAXIN + 1][MAXR];
  int rk[MAXIN + 1];
  int64_t off[MAXIN + 1];
  bool empty = false;
  for (int k = 0; k < nops; k++) {
    rk[k] = 0;
    off[k] = ops[k]->offset;
    for (int i = 0; i < ops[k]->rank; i++) {
      if (ops[k]->shape[i] == 0) empty = true;
      if (ops[k]->shape[i] == 1) continue;
      shp[k][rk[k]] = ops[k]->shape[i];
      str[k][rk[k]] = ops[k]->stride[i];
      rk[k]++;
    }
  }
  int64_t n = view_size(out);
  for (int k = 1; k < nops; k++)
    if (view_size(ops[k]) != n) return fail(PHCU_ERR_SHAPE, "operand %d has %lld elements, output has %lld", k,
                                           (long long)view_size(ops[k]), (long long)n);
  if (empty || n == 0) {
    p->mode = MODE_EMPTY;
    return PHCU_OK;
  }
  for (int k = 1; k < nops; k++) {
    if (rk[k] != rk[0]) return fail(PHCU_ERR_SHAPE, "operand %d shape is not compatible with the output shape", k);
    for (int i = 0; i < rk[0]; i++)
      if (shp[k][i] != shp[0][i])
        return fail(PHCU_ERR_SHAPE, "operand %d shape is not compatible with the output shape", k);
  }
  // an output axis of stride 0 would have every one of its elements written
  // to one place, by different threads
  for (int i = 0; i < rk[0]; i++)
    if (str[0][i] == 0) return fail(PHCU_ERR_INVALID, "the output view has stride 0 on an axis of extent %lld",
                                    (long long)shp[0][i]);
  int rank = rk[0];
  Axis ax[MAXR];
  for (int i = 0; i < rank; i++) {
    ax[i].n = shp[0][i];
    for (int k = 0; k < nops; k++) ax[i].st[k] = str[k][i];
  }

  // 2. walk every axis forwards for the output
  for (int i = 0; i < rank; i++) {
    if (ax[i].st[0] < 0) {
      for (int k = 0; k < nops; k++) {
        off[k] += (ax[i].n - 1) * ax[i].st[k];
        ax[i].st[k] = -ax[i].st[k];
      }
    }
  }
  // 3. innermost axis = smallest output stride (stable: lexicographic order kept on ties)
  std::stable_sort(ax, ax + rank, [](const Axis& a, const Axis& b) {
    int64_t sa = a.st[0] < 0 ? -a.st[0] : a.st[0];
    int64_t sb = b.st[0] < 0 ? -b.st[0] : b.st[0];
    return sa > sb;
  });
  // 4. merge contiguous neighbours
  int r = 0;
  Axis m[MAXR];
  for (int i = 0; i < rank; i++) {
    if (r > 0) {
      Axis& prev = m[r - 1];
      bool ok = true;
      for (int k = 0; k < nops; k++)
        if (prev.st[k] != ax[i].st[k] * ax[i].n) { ok = false; break; }
      if (ok) {
        prev.n *= ax[i].n;
        for (int k = 0; k < nops; k++) prev.st[k] = ax[i].st[k];
        continue;
      }
    }
    m[r++] = ax[i];
  }
  if (r == 0) {  // a single element
    m[0].n = 1;
    for (int k = 0; k < nops; k++) m[0].st[k] = 0;
    r = 1;
  }

  p->sp.rank = r;
  p->sp.n = n;
  for (int i = 0; i < r; i++) {
    p->sp.shape[i] = m[i].n;
    p->sp.div[i].init((uint32_t)m[i].n);
  }
  Operand* dst[MAXIN + 1];
  dst[0] = &p->out;
  for (int k = 0; k < nin; k++) dst[k + 1] = &p->in[k];
  bool any_index = false;
  for (int k = 0; k < nops; k++) {
    if (is_index_view(ops[k])) {
      // an index operand: the value of canonical element 0 travels in `base`
      any_index = true;
      dst[k]->base = (const char*)(uintptr_t)off[k];
      dst[k]->dtype = PHCU_I32;
      for (int i = 0; i < r; i++) dst[k]->stride[i] = m[i].st[k];
      for (int i = r; i < MAXR; i++) dst[k]->stride[i] = 0;
      dst[k]->vmode = VM_INDEX;
      continue;
    }
    int es = dtype_size(ops[k]->dtype);
    dst[k]->base = (const char*)ops[k]->base + off[k] * es;
    dst[k]->dtype = ops[k]->dtype;
    for (int i = 0; i < r; i++) dst[k]->stride[i] = m[i].st[k];
    for (int i = r; i < MAXR; i++) dst[k]->stride[i] = 0;
    dst[k]->vmode = VM_SCALAR;
  }
  p->nin = nin;

  // 5. mode
  const int W = r - 1;
  int mode = MODE_ROW;
  int raxis = -1;
  uint32_t staged = 0;
  // index operands are computed by the ROW body only
  if (!any_index && r >= 2 && p->out.stride[W] == 1 && m[W].n >= 8) {
    // candidate inputs: contiguous along some other axis R, far apart along W
    // (staging inputs that step 2-4 elements along R as well made the
    // 10,000-task batch 4% slower: kept out)
    auto stage = [](int64_t sa, int64_t sw) { return (sa == 1 || sa == -1) && (sw > 2 || sw < -2); };
    int best = -1;
    int64_t best_bytes = 0;
    for (int a = 0; a < W; a++) {
      if (m[a].n < 8) continue;
      int64_t bytes = 0;
      for (int k = 0; k < nin; k++)
        if (stage(p->in[k].stride[a], p->in[k].stride[W])) bytes += dtype_size(p->in[k].dtype);
      if (bytes > best_bytes) { best_bytes = bytes; best = a; }
    }
    if (best >= 0) {
      mode = MODE_TILE;
      raxis = best;
      for (int k = 0; k < nin; k++)
        if (stage(p->in[k].stride[best], p->in[k].stride[W])) staged |= 1u << k;
    }
  }
  if (force_mode == MODE_ROW) mode = MODE_ROW;
  if (force_mode == MODE_TILE && raxis >= 0 && !any_index) mode = MODE_TILE;

  if (mode == MODE_TILE) {
    p->mode = MODE_TILE;
    p->raxis = raxis;
    p->staged = staged;
    p->tiles_w = (m[W].n + TILE - 1) / TILE;
    p->tiles_r = (m[raxis].n + TILE - 1) / TILE;
    int64_t nb = 1;
    for (int a = 0; a < W; a++)
      if (a != raxis) nb *= m[a].n;
    p->nbatch = nb;
    p->tdiv_w.init((uint32_t)p->tiles_w);
    p->tdiv_r.init((uint32_t)p->tiles_r);
    return PHCU_OK;
  }

  p->mode = MODE_ROW;
  const int64_t L = m[W].n;
  // Elements per thread-chunk (a chunk never crosses a row): the widest of
  // 8, 4, 2 that divides the row and that every unit-stride operand can use
  // with aligned vector accesses; if none fits them all, the widest dividing
  // the row, with the misaligned operands on scalar accesses.
  auto vec_ok = [&](const Operand* o, int v) {
    const int es = dtype_size(o->dtype);
    const int64_t sw = o->stride[W];
    for (int a = 0; a < W; a++)
      if (o->stride[a] % v != 0) return false;
    int64_t align = (int64_t)v * es;
    if (align > 16) align = 16;
    uintptr_t lo = (uintptr_t)o->base;
    if (sw == -1) lo -= (uintptr_t)((v - 1) * es);
    return (lo % align) == 0;
  };
  int vec = 1;
  for (int v : {8, 4, 2}) {
    if (L % v != 0) continue;
    bool all = true;
    for (int k = 0; k < nops; k++) {
      const int64_t sw = dst[k]->stride[W];
      if (dst[k]->vmode != VM_INDEX && (sw == 1 || sw == -1) && !vec_ok(dst[k], v)) all = false;
    }
    if (all) {
      vec = v;
      break;
    }
  }
  if (vec == 1) vec = (L % 4 == 0) ? 4 : (L % 2 == 0) ? 2 : 1;
  p->vec = vec;
  for (int k = 0; k < nops; k++) {
    Operand* o = dst[k];
    const int64_t sw = o->stride[W];
    if (o->vmode == VM_INDEX || vec == 1 || (sw != 1 && sw != -1)) continue;
    // an operand aligned for `vec` is also aligned for the 4-element chunks a
    // kernel may use instead of 8
    if (vec_ok(o, vec)) o->vmode = (sw == 1) ? VM_VEC : VM_VEC_REV;
  }
  p->nrows = n / L;
  p->lendiv.init((uint32_t)L);
  return PHCU_OK;
}

}  // namespace phcu
