// phase.hpp -- C++ host side of the GB300 backend for Phase n-dimensional
// arrays: the reference's MultiIndexable / MultiWritable surface
// (src/multi_indexable.cr, src/multi_writable.cr, src/n_array.cr,
// src/view.cr, src/index_region.cr, src/range_syntax/range_syntax.cr) over
// the C ABI of libphcuda.so (include/phcuda.h).  Header-only C++17; link
// against libphcuda.so.
//
// As in the reference, index validation stays on the host: region literals
// are canonicalised here (RangeSyntax / IndexRegion) and raise IndexError,
// DimensionError or ShapeError before any device call.  A view is an affine
// descriptor (offset, shape, signed strides) over an array's device buffer;
// nothing is copied until an operation materialises it.  Every bulk
// operation is one call into the library; there is no CPU path.
//
// Surface: CuNArray<T> (arrays), CuView<T> (region / permute / reverse /
// reshape views), CuProcView<T> (fused expressions: one device program per
// materialisation), the infix operators with Crystal's result types and the
// comparisons (Bool arrays), reductions, chunk and element reads and writes,
// slices, masked writes, equals?, the in-place maps (map!, map_with!,
// map_with_index!, map_with_coord!), tile, concatenate and push.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "phcuda.h"

namespace phase {

// ------------------------------------------------------------------ errors
// The reference's exception taxonomy (contributing/standards.md, stdlib).
struct PhaseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct ShapeError : PhaseError {
  using PhaseError::PhaseError;
};
struct DimensionError : ShapeError {
  using ShapeError::ShapeError;
};
struct IndexError : PhaseError {
  using PhaseError::PhaseError;
};
struct OverflowError : PhaseError {
  using PhaseError::PhaseError;
};
struct DivisionByZeroError : PhaseError {
  using PhaseError::PhaseError;
};
struct ArgumentError : PhaseError {
  using PhaseError::PhaseError;
};
struct EmptyError : PhaseError {
  using PhaseError::PhaseError;
};
struct DeviceError : PhaseError {
  using PhaseError::PhaseError;
};
// A fused expression the device program cannot hold (more than
// PHCU_MAX_INPUTS distinct views, PHCU_MAX_INSTR instructions or two nested
// stashes), or an operator Crystal does not define for the operand types.
struct NotImplementedError : PhaseError {
  using PhaseError::PhaseError;
};

inline std::string last_error() {
  char buf[512];
  buf[0] = 0;
  phcu_last_error(buf, sizeof(buf));
  return buf;
}

// Maps a library status code onto the reference's exceptions.
inline void check(int32_t rc, const char* what = "") {
  if (rc == PHCU_OK) return;
  const std::string msg = std::string(what) + (what[0] ? ": " : "") + last_error();
  switch (rc) {
    case PHCU_ERR_SHAPE: throw ShapeError(msg);
    case PHCU_ERR_DIM: throw DimensionError(msg);
    case PHCU_ERR_INDEX: throw IndexError(msg);
    case PHCU_ERR_OVERFLOW: throw OverflowError(msg);
    case PHCU_ERR_DIVZERO: throw DivisionByZeroError(msg);
    case PHCU_ERR_ARGUMENT: throw ArgumentError(msg);
    case PHCU_ERR_EMPTY: throw EmptyError(msg);
    default: throw DeviceError(msg);
  }
}

// Reads and clears the device status word that kernels set for checked
// integer arithmetic; raises what the reference would have raised.
inline void check_status() {
  uint32_t w = 0;
  check(phcu_status_word(&w, 1), "phcu_status_word");
  if (w & PHCU_ST_DIVZERO) throw DivisionByZeroError("Division by 0");
  if (w & PHCU_ST_OVERFLOW) throw OverflowError("Arithmetic overflow");
  if (w & PHCU_ST_ARGUMENT) throw ArgumentError("Cannot raise an integer to a negative integer power");
  if (w & PHCU_ST_TIMEOUT) throw DeviceError("device work timed out");
}

// ------------------------------------------------------------------ dtypes
template <typename T>
struct DType;
template <>
struct DType<float> {
  static constexpr int32_t id = PHCU_F32;
  static constexpr const char* name = "Float32";
};
template <>
struct DType<double> {
  static constexpr int32_t id = PHCU_F64;
  static constexpr const char* name = "Float64";
};
template <>
struct DType<int32_t> {
  static constexpr int32_t id = PHCU_I32;
  static constexpr const char* name = "Int32";
};
template <>
struct DType<int64_t> {
  static constexpr int32_t id = PHCU_I64;
  static constexpr const char* name = "Int64";
};

// Crystal's Bool as a one-byte device element: the result of the elementwise
// comparisons and the mask of masked writes.  (std::vector<bool> packs bits,
// so host copies of Bool arrays use this one-byte type instead.)
struct Bool {
  uint8_t v = 0;
  Bool() = default;
  Bool(bool b) : v(b ? 1 : 0) {}
  operator bool() const { return v != 0; }
};
static_assert(sizeof(Bool) == 1, "Bool is one byte on the device");
template <>
struct DType<Bool> {
  static constexpr int32_t id = PHCU_BOOL;
  static constexpr const char* name = "Bool";
};

// -------------------------------------------------------- region literals
// One entry of a region literal: an integer index (the axis is dropped) or a
// Crystal range `first..last`, `first...last`, `first..step..last` with any of
// first / last / step omitted.
struct Lit {
  bool is_index = false;
  int64_t index = 0;
  std::optional<int64_t> first, last, step;
  bool exclusive = false;
};
inline Lit idx(int64_t i) {
  Lit l;
  l.is_index = true;
  l.index = i;
  return l;
}
inline Lit rng(std::optional<int64_t> first = std::nullopt, std::optional<int64_t> last = std::nullopt,
               std::optional<int64_t> step = std::nullopt, bool exclusive = false) {
  Lit l;
  l.first = first;
  l.last = last;
  l.step = step;
  l.exclusive = exclusive;
  return l;
}
inline Lit all() { return rng(); }

// {first, step, last, size} of one axis.
struct AxisRange {
  int64_t first = 0, step = 1, last = 0, size = 0;
};

namespace detail {
inline int64_t sign(int64_t x) { return (x > 0) - (x < 0); }
inline int64_t canon_unsafe(int64_t i, int64_t bound) { return i < 0 ? bound + i : i; }
}  // namespace detail

// RangeSyntax.get_size (range_syntax.cr:7-17).
inline int64_t get_size(int64_t first, int64_t last, int64_t step) {
  if (last != first && detail::sign(step) != detail::sign(last - first))
    throw IndexError("Could not get size of range - step direction disagrees with first and last.");
  if (step == 0) throw IndexError("Could not get size of range - zero step.");
  if (last >= first) return (last - first) / step + 1;
  return (first - last) / (-step) + 1;
}

// RangeSyntax.infer_range (range_syntax.cr:84-136).
inline AxisRange infer_range(const Lit& l, int64_t bound) {
  if (l.is_index) {
    const int64_t c = detail::canon_unsafe(l.index, bound);
    return {c, 1, c, 1};
  }
  int64_t first, temp_last, step;
  if (!l.step) {
    first = l.first ? detail::canon_unsafe(*l.first, bound) : 0;
    temp_last = l.last ? detail::canon_unsafe(*l.last, bound) : bound - 1;
    step = temp_last >= first ? 1 : -1;
  } else {
    step = *l.step;
    first = l.first ? detail::canon_unsafe(*l.first, bound) : (step > 0 ? 0 : bound - 1);
    temp_last = l.last ? detail::canon_unsafe(*l.last, bound) : (step > 0 ? bound - 1 : 0);
  }
  if (l.last && l.exclusive) {
    if (temp_last == first) return {0, 0, 0, 0};
    temp_last -= detail::sign(step);
  }
  if (first < 0 || temp_last < 0)
    throw IndexError("Invalid index: At least one endpoint of the range is negative after canonicalization.");
  int64_t size;
  try {
    size = get_size(first, temp_last, step);
  } catch (const IndexError&) {
    throw IndexError("Could not canonicalize range: Conflict between implicit direction of the range and the step");
  }
  return {first, step, first + step * (size - 1), size};
}

// RangeSyntax.canonicalize_range (range_syntax.cr:145-153).
inline AxisRange canonicalize_range(const Lit& l, int64_t bound) {
  const AxisRange r = infer_range(l, bound);
  if (!(0 <= r.last && r.last < bound && 0 <= r.first && r.first < bound))
    throw IndexError("Could not canonicalize range: not a sensible index range for an axis of length " +
                     std::to_string(bound) + ".");
  return r;
}

// ShapeUtil.shape_to_size (shape_util.cr:41-50).
inline int64_t shape_to_size(const std::vector<int64_t>& shape) {
  if (shape.empty()) return 0;
  int64_t n = 1;
  for (int64_t s : shape) n *= s;
  return n;
}

// IndexRegion.new(region_literal, bound_shape, drop) (index_region.cr:192-224):
// per proper axis {first, step, last, size}; an integer index is a degenerate
// axis, dropped from the reduced shape when `drop`.
struct IndexRegion {
  std::vector<AxisRange> axes;
  std::vector<bool> degenerate;
  bool drop = true;

  static IndexRegion make(const std::vector<Lit>& lits, const std::vector<int64_t>& bound, bool drop = true) {
    if (lits.size() > bound.size())
      throw DimensionError("The region literal had more dimensions than its bound shape.");
    IndexRegion r;
    r.drop = drop;
    r.axes.resize(bound.size());
    r.degenerate.assign(bound.size(), false);
    for (size_t i = 0; i < lits.size(); i++) {
      r.axes[i] = canonicalize_range(lits[i], bound[i]);
      if (lits[i].is_index) r.degenerate[i] = drop;
    }
    for (size_t a = lits.size(); a < bound.size(); a++) r.axes[a] = {0, 1, bound[a] - 1, bound[a]};
    return r;
  }

  // IndexRegion.cover (index_region.cr:232-238).
  static IndexRegion cover(const std::vector<int64_t>& bound) {
    IndexRegion r;
    for (int64_t n : bound) r.axes.push_back({0, n == 0 ? 0 : 1, std::max<int64_t>(0, n - 1), n});
    r.degenerate.assign(bound.size(), false);
    return r;
  }

  // IndexRegion.new(region_literal, drop) without a bound (index_region.cr:255-283):
  // negative indices have no meaning, and every range needs its far end.
  static IndexRegion absolute(const std::vector<Lit>& lits, bool drop = true) {
    IndexRegion r;
    r.drop = drop;
    for (const Lit& l : lits) {
      if (l.is_index) {
        if (l.index < 0) throw IndexError("Negative indices have no meaning when a bounding shape is not provided.");
      } else {
        if ((l.first && *l.first < 0) || (l.last && *l.last < 0))
          throw IndexError("Negative indices have no meaning when a bounding shape is not provided.");
        const bool bounded = (!l.step || *l.step >= 0) ? (bool)l.last : (bool)l.first;
        if (!bounded)
          throw ArgumentError("Cannot create IndexRegion without an explicit upper bound unless you provide a "
                              "bounding shape");
      }
      r.axes.push_back(infer_range(l, 0));
      r.degenerate.push_back(l.is_index);
    }
    return r;
  }

  // IndexRegion#fits_in? (index_region.cr:468-478).
  bool fits_in(const std::vector<int64_t>& bound) const {
    if (bound.size() != axes.size())
      throw DimensionError("The bound shape provided had a different number of dimensions than this IndexRegion.");
    for (size_t i = 0; i < axes.size(); i++)
      if (bound[i] <= std::max(axes[i].first, axes[i].last)) return false;
    return true;
  }

  // IndexRegion#trim! (index_region.cr:502-515, trim_axis :684-702).
  IndexRegion& trim(const std::vector<int64_t>& bound) {
    if (bound.size() != axes.size()) throw DimensionError("Cannot trim a region to a shape of another rank");
    for (size_t a = 0; a < axes.size(); a++) {
      AxisRange& x = axes[a];
      const int64_t nb = bound[a], as = x.step < 0 ? -x.step : x.step;
      if (x.first >= nb) {
        if (x.last >= nb) {
          x = {0, 0, 0, 0};
        } else if (x.step < 0) {
          int64_t span = (nb - 1) - x.last;
          x.size = span / as + 1;
          span -= span % as;
          x.first = x.last + span;
        }
      } else if (x.step > 0 && x.last >= nb) {
        int64_t span = (nb - 1) - x.first;
        span -= span % as;
        x.size = span / as + 1;
        x.last = x.first + span;
      }
    }
    return *this;
  }

  // IndexRegion#reverse! (index_region.cr:533-537).
  IndexRegion& reverse() {
    for (AxisRange& x : axes) {
      std::swap(x.first, x.last);
      x.step = -x.step;
    }
    return *this;
  }

  // IndexRegion#translate! (index_region.cr:577-585).
  IndexRegion& translate(const std::vector<int64_t>& offset) {
    for (size_t a = 0; a < offset.size() && a < axes.size(); a++)
      if (offset[a] < 0 && (axes[a].first < -offset[a] || axes[a].last < -offset[a]))
        throw IndexError("Can't translate to negative indices");
    for (size_t a = 0; a < offset.size() && a < axes.size(); a++) {
      axes[a].first += offset[a];
      axes[a].last += offset[a];
    }
    return *this;
  }

  // IndexRegion#includes? (index_region.cr:445-458).
  bool includes(const std::vector<int64_t>& coord) const {
    if (coord.size() != axes.size()) return false;
    for (size_t i = 0; i < axes.size(); i++) {
      const AxisRange& x = axes[i];
      const int64_t lo = x.step > 0 ? x.first : x.last, hi = x.step > 0 ? x.last : x.first;
      if (coord[i] < lo || coord[i] > hi || x.step == 0) return false;
      if ((coord[i] - x.first) % x.step != 0) return false;
    }
    return true;
  }

  // IndexRegion#local_to_absolute_unsafe (index_region.cr:621-637): a
  // coordinate of the region's (reduced) shape to one of the bound shape.
  std::vector<int64_t> local_to_absolute(const std::vector<int64_t>& coord) const {
    std::vector<int64_t> out;
    size_t la = 0;
    for (size_t i = 0; i < axes.size(); i++) {
      if (drop && degenerate[i]) {
        out.push_back(axes[i].first);
      } else {
        out.push_back(axes[i].first + coord[la] * axes[i].step);
        la++;
      }
    }
    return out;
  }

  // IndexRegion#shape (index_region.cr:304-317): the kept axes' sizes, or
  // [size] when every axis is dropped.
  std::vector<int64_t> shape() const {
    std::vector<int64_t> s, proper;
    for (size_t i = 0; i < axes.size(); i++) {
      proper.push_back(axes[i].size);
      if (!(drop && degenerate[i])) s.push_back(axes[i].size);
    }
    if (drop && s.empty()) s.push_back(shape_to_size(proper));
    return s;
  }
};

// ------------------------------------------------------------- device side
// The library context: one device per process.
inline void init(int device = 0) { check(phcu_init(device), "phcu_init"); }

// A device allocation, released stream-ordered when the last array or view
// that refers to it goes away (views alias their source, src/view.cr:21-26).
struct Buffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  explicit Buffer(size_t n) : bytes(n) { check(phcu_alloc(n, &ptr), "phcu_alloc"); }
  ~Buffer() {
    if (ptr) phcu_free(ptr);
  }
  Buffer(const Buffer&) = delete;
  Buffer& operator=(const Buffer&) = delete;
};

// A view's layout over its buffer, in elements.
struct Affine {
  int64_t offset = 0;
  std::vector<int64_t> shape, stride;
};

inline std::vector<int64_t> row_major(const std::vector<int64_t>& shape) {
  std::vector<int64_t> st(shape.size());
  int64_t s = 1;
  for (size_t i = shape.size(); i-- > 0;) {
    st[i] = s;
    s *= shape[i];
  }
  return st;
}

namespace detail {
// Whether writing `src` into `dst` (two layouts over one buffer, equal element
// counts) element by element in lexicographic order, as the reference's
// MultiWritable#unsafe_set_chunk does (multi_writable.cr:29-44), can differ
// from reading the whole source first, as the device does: some element is
// read at step i after a step j < i changed it (S(i) = D(j), S(j) != D(j)).
// Exact up to 2^22 elements; above, false only for a destination walked in
// increasing address order whose every read is at or past the write of its
// step.  A destination that writes an element twice counts as differing.
inline bool sequential_order_differs(const Affine& dst, const Affine& src) {
  std::vector<std::pair<int64_t, int64_t>> d, s;  // (extent, stride) of the non-unit axes
  for (size_t i = 0; i < dst.shape.size(); i++)
    if (dst.shape[i] != 1) d.push_back({dst.shape[i], dst.stride[i]});
  for (size_t i = 0; i < src.shape.size(); i++)
    if (src.shape[i] != 1) s.push_back({src.shape[i], src.stride[i]});
  int64_t n = 1;
  for (auto& a : d) n *= a.first;
  if (n == 0) return false;
  if (dst.offset == src.offset && d == s) return false;  // each step reads the element it writes
  auto span = [](const std::vector<std::pair<int64_t, int64_t>>& v, int64_t off, int64_t* lo, int64_t* hi) {
    *lo = *hi = off;
    for (auto& a : v) {
      const int64_t e = (a.first - 1) * a.second;
      if (e < 0) *lo += e;
      else *hi += e;
    }
  };
  int64_t dlo, dhi, slo, shi;
  span(d, dst.offset, &dlo, &dhi);
  span(s, src.offset, &slo, &shi);
  if (shi < dlo || dhi < slo) return false;  // disjoint
  auto addresses = [n](const std::vector<std::pair<int64_t, int64_t>>& v, int64_t off) {
    std::vector<int64_t> a(1, off);
    a.reserve((size_t)n);
    for (auto& ax : v) {
      std::vector<int64_t> b;
      b.reserve(a.size() * (size_t)ax.first);
      for (int64_t x : a)
        for (int64_t k = 0; k < ax.first; k++) b.push_back(x + k * ax.second);
      a.swap(b);
    }
    return a;
  };
  if (n <= ((int64_t)1 << 22)) {
    const std::vector<int64_t> da = addresses(d, dst.offset), sa = addresses(s, src.offset);
    std::vector<std::pair<int64_t, int64_t>> order((size_t)n);  // (address, step)
    for (int64_t j = 0; j < n; j++) order[(size_t)j] = {da[(size_t)j], j};
    std::sort(order.begin(), order.end());
    for (size_t k = 1; k < order.size(); k++)
      if (order[k].first == order[k - 1].first) return true;  // an element written twice
    for (int64_t i = 0; i < n; i++) {
      auto it = std::lower_bound(order.begin(), order.end(), std::make_pair(sa[(size_t)i], (int64_t)INT64_MIN));
      if (it == order.end() || it->first != sa[(size_t)i]) continue;
      const int64_t j = it->second;
      if (j < i && sa[(size_t)j] != da[(size_t)j]) return true;
    }
    return false;
  }
  bool monotone = true;
  int64_t inner = 0;
  for (size_t k = d.size(); k-- > 0;) {
    monotone = monotone && d[k].second > inner;
    inner += (d[k].first - 1) * d[k].second;
  }
  if (!monotone || d.size() != s.size()) return true;
  int64_t gap = src.offset - dst.offset;
  for (size_t k = 0; k < d.size(); k++) {
    if (d[k].first != s[k].first) return true;
    gap += std::min<int64_t>(0, (d[k].first - 1) * (s[k].second - d[k].second));
  }
  return gap < 0;
}
}  // namespace detail

inline phcu_view_t make_view(void* base, int32_t dtype, const Affine& a) {
  if (a.shape.size() > (size_t)PHCU_MAX_RANK)
    throw DimensionError("rank " + std::to_string(a.shape.size()) + " exceeds the device limit of " +
                         std::to_string(PHCU_MAX_RANK));
  phcu_view_t v;
  std::memset(&v, 0, sizeof(v));
  v.base = base;
  v.dtype = dtype;
  v.rank = (int32_t)a.shape.size();
  v.offset = a.offset;
  for (size_t i = 0; i < a.shape.size(); i++) {
    v.shape[i] = a.shape[i];
    v.stride[i] = a.stride[i];
  }
  return v;
}

// RegionTransform (src/view_util/transforms.cr:191-222) folded into the layout.
inline Affine affine_region(const Affine& a, const IndexRegion& r) {
  Affine o;
  o.offset = a.offset;
  std::vector<int64_t> proper;
  for (size_t i = 0; i < r.axes.size(); i++) {
    proper.push_back(r.axes[i].size);
    if (r.axes[i].size > 0) o.offset += r.axes[i].first * a.stride[i];
    if (r.drop && r.degenerate[i]) continue;
    o.shape.push_back(r.axes[i].size);
    o.stride.push_back(r.axes[i].step * a.stride[i]);
  }
  if (o.shape.empty()) {  // every axis dropped: shape [size] (index_region.cr:304-317)
    o.shape = {shape_to_size(proper)};
    o.stride = {0};
  }
  return o;
}

// PermuteTransform (transforms.cr:224-271): view axis i is source axis order[i].
inline Affine affine_permute(const Affine& a, const std::vector<int>& order) {
  const size_t n = a.shape.size();
  std::vector<bool> seen(n, false);
  if (order.size() != n) throw IndexError("a permutation must name every axis once");
  for (int o : order) {
    if (o < 0 || (size_t)o >= n || seen[o]) throw IndexError("a permutation must name every axis once");
    seen[o] = true;
  }
  Affine p;
  p.offset = a.offset;
  for (int o : order) {
    p.shape.push_back(a.shape[o]);
    p.stride.push_back(a.stride[o]);
  }
  return p;
}

// ReverseTransform (transforms.cr:273-305): every axis reversed.
inline Affine affine_reverse(const Affine& a) {
  Affine r = a;
  for (size_t i = 0; i < a.shape.size(); i++) {
    if (a.shape[i] > 0) r.offset += (a.shape[i] - 1) * a.stride[i];
    r.stride[i] = -a.stride[i];
  }
  return r;
}

// ReshapeTransform (transforms.cr:118-189) as strides, when the view's layout
// allows it: the lexicographic order is regrouped without moving elements.
// Empty when the new shape cannot be expressed with strides.
inline std::optional<Affine> affine_reshape(const Affine& a, const std::vector<int64_t>& ns) {
  if (shape_to_size(ns) == 0 || shape_to_size(a.shape) == 0) return Affine{a.offset, ns, row_major(ns)};
  std::vector<std::pair<int64_t, int64_t>> old;  // (extent, stride) of the axes longer than 1
  for (size_t i = 0; i < a.shape.size(); i++)
    if (a.shape[i] != 1) old.push_back({a.shape[i], a.stride[i]});
  std::vector<int64_t> nst(ns.size(), 0);
  size_t oi = 0, ni = 0;
  const size_t on = old.size(), nn = ns.size();
  while (ni < nn && oi < on) {
    if (ns[ni] == 1) {
      nst[ni++] = 0;
      continue;
    }
    // old axes [oi, oj) and new axes [ni, nj) of equal element count
    int64_t op = old[oi].first, np = ns[ni];
    size_t oj = oi + 1, nj = ni + 1;
    while (op != np) {
      if (op < np) {
        if (oj >= on) return std::nullopt;
        op *= old[oj++].first;
      } else {
        if (nj >= nn) return std::nullopt;
        np *= ns[nj++];
      }
    }
    for (size_t k = oi; k + 1 < oj; k++)  // the old group must be contiguous in itself
      if (old[k].second != old[k + 1].second * old[k + 1].first) return std::nullopt;
    int64_t st = old[oj - 1].second;
    for (size_t k = nj; k-- > ni;) {
      nst[k] = st;
      st *= ns[k];
    }
    oi = oj;
    ni = nj;
  }
  for (; ni < nn; ni++) {
    if (ns[ni] != 1) return std::nullopt;
    nst[ni] = 0;
  }
  return Affine{a.offset, ns, nst};
}

template <typename T>
class CuNArray;
template <typename T>
class CuProcView;

// A strided, aliasing view of an array (src/view.cr): region, permute and
// reverse rewrite the layout; materialising takes one gather kernel.
template <typename T>
class CuView {
 public:
  CuView(std::shared_ptr<Buffer> buf, Affine a) : buf_(std::move(buf)), aff_(std::move(a)) {}

  const std::vector<int64_t>& shape() const { return aff_.shape; }
  int64_t size() const { return shape_to_size(aff_.shape); }
  size_t dimensions() const { return aff_.shape.size(); }
  phcu_view_t desc() const { return make_view(buf_->ptr, DType<T>::id, aff_); }
  const Affine& layout() const { return aff_; }
  const std::shared_ptr<Buffer>& buffer() const { return buf_; }

  // View#view / #restrict_to (view.cr:43-56).
  CuView view(const std::vector<Lit>& region) const {
    return CuView(buf_, affine_region(aff_, IndexRegion::make(region, aff_.shape)));
  }
  // View#permute! (view.cr:72-81); no order reverses the axes.
  CuView permute(std::vector<int> order = {}) const {
    if (order.empty())
      for (size_t i = aff_.shape.size(); i-- > 0;) order.push_back((int)i);
    return CuView(buf_, affine_permute(aff_, order));
  }
  // View#reverse! (view.cr:96-99).
  CuView reverse() const { return CuView(buf_, affine_reverse(aff_)); }
  // View#reshape (view.cr:58-70): the same elements in lexicographic order
  // under a new shape; a layout that strides cannot express is copied first.
  CuView reshape(const std::vector<int64_t>& new_shape) const;

  // View#to_narr (view.cr:123-126): one gather into a new contiguous array.
  CuNArray<T> to_cu() const;
  std::vector<T> to_vector() const;

  // MultiIndexable#process (view.cr:119-121, proc_view.cr:6-35): a lazy
  // elementwise program over this view; f maps a Sym<T> to a Sym<R> (or a
  // constant).  Nothing runs until the result is materialised.
  CuProcView<T> process() const;
  template <typename F>
  auto process(F f) const;

 protected:
  std::shared_ptr<Buffer> buf_;
  Affine aff_;
};

namespace detail {
// defined with the fused expressions below
inline std::string shape_text(const std::vector<int64_t>& s);
inline int64_t slot_bits(float v);
inline int64_t slot_bits(double v);
inline int64_t slot_bits(int32_t v);
inline int64_t slot_bits(int64_t v);
}  // namespace detail

// A device-resident NArray (src/n_array.cr): one row-major buffer.  Copies of
// a CuNArray share the buffer, as Crystal references to one NArray do;
// clone() makes an independent copy (NArray#clone, n_array.cr:372-374).
template <typename T>
class CuNArray : public CuView<T> {
 public:
  explicit CuNArray(std::vector<int64_t> shape)
      : CuView<T>(std::make_shared<Buffer>((size_t)std::max<int64_t>(1, count(shape)) * sizeof(T)),
                  Affine{0, shape, row_major(shape)}) {}

  // NArray.of_buffer (n_array.cr:76-79): shape plus lexicographic elements.
  static CuNArray of_buffer(const std::vector<int64_t>& shape, const std::vector<T>& elems) {
    if ((int64_t)elems.size() != count(shape))
      throw ShapeError("Cannot create NArray: the shape's size and the buffer's size differ.");
    CuNArray a(shape);
    if (!elems.empty()) check(phcu_upload(a.buf_->ptr, elems.data(), elems.size() * sizeof(T)), "phcu_upload");
    return a;
  }
  // NArray.fill (n_array.cr:230-232).
  static CuNArray fill(const std::vector<int64_t>& shape, T value) {
    CuNArray a(shape);
    a.fill_view(a.desc(), value);
    return a;
  }

  CuNArray clone() const { return this->to_cu(); }

  std::vector<T> to_vector() const {
    std::vector<T> h((size_t)this->size());
    if (!h.empty()) check(phcu_download(h.data(), this->buf_->ptr, h.size() * sizeof(T)), "phcu_download");
    return h;
  }

  // MultiIndexable#get_chunk / #[] (multi_indexable.cr:330-413): a copy.
  CuNArray get_chunk(const std::vector<Lit>& region) const { return this->view(region).to_cu(); }

  // MultiWritable#set_chunk / #[]= (multi_writable.cr:55-84): a strided copy
  // of src into the region, or the value into every element of it.
  void set_chunk(const std::vector<Lit>& region, const CuView<T>& src) {
    const CuView<T> dst = this->view(region);
    if (dst.shape() != src.shape())
      throw ShapeError("Cannot set chunk: the source's shape differs from the region's shape.");
    refuse_reordered_alias(dst, src.buffer().get(), src.layout());
    const phcu_view_t d = dst.desc(), s = src.desc();
    check(phcu_copy(&d, &s), "phcu_copy");
  }
  void set_chunk(const std::vector<Lit>& region, T value) { fill_view(this->view(region).desc(), value); }
  // A fused source is evaluated first, then copied in.  The reference reads
  // its operands element by element while it writes, so an operand that
  // aliases the region in another element order is refused.
  void set_chunk(const std::vector<Lit>& region, const CuProcView<T>& src);

  // MultiIndexable#get / #unsafe_fetch_element (multi_indexable.cr, n_array.cr:456-458)
  // and MultiWritable#set_element / #unsafe_set_element (n_array.cr:503-505):
  // one element, negative indices counted from the end (CoordUtil).  Slow
  // paths: one download or one fill per element.
  T get(const std::vector<int64_t>& coord) const { return this->view(coord_lits(coord)).to_vector()[0]; }
  void set_element(const std::vector<int64_t>& coord, T value) { set_chunk(coord_lits(coord), value); }

  // MultiIndexable#slices / #each_slice (multi_indexable.cr:742-786): the
  // chunks with axis `axis` fixed at 0, 1, ... and dropped.
  std::vector<CuNArray> slices(int axis = 0) const {
    const int d = (int)this->dimensions();
    if (axis < 0 || axis >= d)
      throw IndexError("axis " + std::to_string(axis) + " is not present in a " + std::to_string(d) +
                       "-dimensional MultiIndexable");
    std::vector<CuNArray> out;
    for (int64_t i = 0; i < this->shape()[axis]; i++) {
      std::vector<Lit> lits((size_t)d, all());
      lits[(size_t)axis] = idx(i);
      out.push_back(get_chunk(lits));
    }
    return out;
  }

  // NArray#[]=(mask, value) and MultiWritable#set_mask (n_array.cr:510-551,
  // multi_writable.cr:127-172): value, or the element of src, wherever mask
  // holds true; one in-place select kernel.
  void set_mask(const CuView<Bool>& mask, T value) { masked_write(mask, nullptr, value); }
  void set_mask(const CuView<Bool>& mask, const CuView<T>& src) { masked_write(mask, &src, T(0)); }

  // Mutable#map! (mutable.cr:29-33, n_array.cr:621-627): self = f(self), and
  // Mutable#map_with! (mutable.cr:54-67): self = f(self, other), each one
  // program written into the array itself.  The block returns a Sym of the
  // array's element type.
  template <typename F>
  CuNArray& map_inplace(F f);
  template <typename U, typename F>
  CuNArray& map_with_inplace(const CuView<U>& other, F f);
  // NArray#map_with_index! (n_array.cr:631-637) and #map_with_coord!
  // (mutable.cr:16-20, n_array.cr:641-650): the block also receives the
  // element's lexicographic index, or its coordinates, as Int32 Syms computed
  // on the device (index operands, never stored).
  template <typename F>
  CuNArray& map_with_index_inplace(F f);
  template <typename F>
  CuNArray& map_with_coord_inplace(F f);

  // NArray#reshape (n_array.cr:429-437): the same buffer under a new shape.
  CuNArray reshape(const std::vector<int64_t>& new_shape) const {
    if (count(new_shape) != count(this->shape()))
      throw ShapeError("Cannot create NArray: Given shape does not match number of elements in buffer.");
    return CuNArray(this->buf_, new_shape);
  }

  // NArray.tile (n_array.cr:242-252): src repeated counts[i] times along axis
  // i.  One strided copy: the output seen as [c0, s0, c1, s1, ...] receives
  // the source read with stride 0 along every c axis (leading axes walked on
  // the host where that view would pass the device's rank limit).
  static CuNArray tile(const CuView<T>& src, const std::vector<int64_t>& counts) {
    const std::vector<int64_t>& ss = src.shape();
    const size_t R = ss.size();
    if (counts.size() < R)
      throw IndexError("tile: " + std::to_string(counts.size()) + " counts for a " + std::to_string(R) +
                       "-dimensional source");
    std::vector<int64_t> shape(R);
    for (size_t i = 0; i < R; i++) {
      if (counts[i] < 0) throw ArgumentError("tile: negative count");
      shape[i] = ss[i] * counts[i];
    }
    CuNArray out(shape);
    if (shape_to_size(shape) == 0) return out;
    const std::vector<int64_t> ost = row_major(shape);
    const size_t lead = 2 * R > (size_t)PHCU_MAX_RANK ? 2 * R - (size_t)PHCU_MAX_RANK : 0;
    int64_t nprefix = 1;
    for (size_t i = 0; i < lead; i++) nprefix *= counts[i];
    for (int64_t pfx = 0; pfx < nprefix; pfx++) {
      Affine d{0, {}, {}}, s{src.layout().offset, {}, {}};
      int64_t rest = pfx;
      for (size_t i = lead; i-- > 0;) {  // this prefix's copy index along each leading axis
        const int64_t ci = rest % counts[i];
        rest /= counts[i];
        d.offset += ci * ss[i] * ost[i];
      }
      for (size_t i = 0; i < R; i++) {
        if (i < lead) {
          d.shape.push_back(ss[i]);
          d.stride.push_back(ost[i]);
          s.shape.push_back(ss[i]);
          s.stride.push_back(src.layout().stride[i]);
        } else {
          d.shape.insert(d.shape.end(), {counts[i], ss[i]});
          d.stride.insert(d.stride.end(), {ss[i] * ost[i], ost[i]});
          s.shape.insert(s.shape.end(), {counts[i], ss[i]});
          s.stride.insert(s.stride.end(), {0, src.layout().stride[i]});
        }
      }
      const phcu_view_t dv = make_view(out.buf_->ptr, DType<T>::id, d);
      const phcu_view_t sv = make_view(src.buffer()->ptr, DType<T>::id, s);
      check(phcu_copy(&dv, &sv), "phcu_copy");
    }
    return out;
  }

  // NArray.concatenate (n_array.cr:719-749): one strided copy of each operand
  // into its slab of the output along `axis`.
  static CuNArray concatenate(const std::vector<CuView<T>>& parts, int axis = 0) {
    if (parts.empty()) throw ArgumentError("concatenate: no arrays");
    const std::vector<int64_t>& first = parts[0].shape();
    const int rank = (int)first.size();
    const int ax = axis < 0 ? axis + rank : axis;
    if (ax < 0 || ax >= rank)
      throw IndexError("axis " + std::to_string(axis) + " is not present in a " + std::to_string(rank) +
                       "-dimensional MultiIndexable");
    std::vector<int64_t> shape = first;
    shape[(size_t)ax] = 0;
    for (const CuView<T>& p : parts) {
      bool ok = (int)p.dimensions() == rank;
      for (int i = 0; ok && i < rank; i++) ok = i == ax || p.shape()[(size_t)i] == first[(size_t)i];
      if (!ok)
        throw DimensionError("Cannot concatenate these arrays along axis " + std::to_string(axis) +
                             ": shapes do not match");
      shape[(size_t)ax] += p.shape()[(size_t)ax];
    }
    CuNArray out(shape);
    const std::vector<int64_t> ost = row_major(shape);
    int64_t pos = 0;
    for (const CuView<T>& p : parts) {
      const int64_t k = p.shape()[(size_t)ax];
      if (k > 0 && p.size() > 0) {
        std::vector<int64_t> sub = shape;
        sub[(size_t)ax] = k;
        const phcu_view_t dv = make_view(out.buf_->ptr, DType<T>::id, Affine{pos * ost[(size_t)ax], sub, ost});
        const phcu_view_t sv = p.desc();
        check(phcu_copy(&dv, &sv), "phcu_copy");
      }
      pos += k;
    }
    return out;
  }

  // NArray#push / #<< (n_array.cr:682-712): appends along axis 0; the array
  // takes the concatenation's buffer.
  CuNArray& push(const CuView<T>& other) {
    *this = concatenate({*this, other}, 0);
    return *this;
  }

 private:
  static int64_t count(const std::vector<int64_t>& shape) {
    for (int64_t s : shape)
      if (s < 0) throw DimensionError("Cannot create NArray: One or more of the provided dimensions was negative.");
    return shape.empty() ? 1 : shape_to_size(shape);
  }
  static void refuse_reordered_alias(const CuView<T>& dst, const Buffer* src_buf, const Affine& src) {
    if (src_buf == dst.buffer().get() && detail::sequential_order_differs(dst.layout(), src))
      throw NotImplementedError(
          "set_chunk: the source overlaps the destination in another element order, so the reference's "
          "element-by-element write would read elements it has already written, while the device reads the "
          "whole source first; write a copy of the source (clone) instead");
  }
  static void fill_view(const phcu_view_t& v, T value) {
    phcu_scalar_t s;
    std::memset(&s, 0, sizeof(s));
    s.dtype = DType<T>::id;
    if (std::is_floating_point<T>::value) s.v.f = (double)value;
    else s.v.i = (int64_t)value;
    check(phcu_fill(&v, &s), "phcu_fill");
  }
  std::vector<Lit> coord_lits(const std::vector<int64_t>& coord) const {
    if (coord.size() != this->dimensions())
      throw DimensionError("Could not canonicalize coordinate " + detail::shape_text(coord) + " to fit in shape " +
                           detail::shape_text(this->shape()));
    std::vector<Lit> lits;
    for (int64_t c : coord) lits.push_back(idx(c));
    return lits;
  }
  // Program: S0 = mask; ACC = self; ACC = S0 ? source : ACC, with the source
  // an input view or the value as an immediate; inputs {mask, source, self}.
  void masked_write(const CuView<Bool>& mask, const CuView<T>* src, T value) {
    if (mask.shape() != this->shape())
      throw ShapeError("Cannot perform masking: mask shape " + detail::shape_text(mask.shape()) +
                       " does not match array shape " + detail::shape_text(this->shape()) + ".");
    if (src && src->shape() != this->shape())
      throw ShapeError("Cannot perform masking: source shape " + detail::shape_text(src->shape()) +
                       " does not match array shape " + detail::shape_text(this->shape()) + ".");
    if (src) refuse_reordered_alias(*this, src->buffer().get(), src->layout());
    phcu_program_t p;
    std::memset(&p, 0, sizeof(p));
    const int32_t t = DType<T>::id;
    auto emit = [&p](int32_t op, int32_t sr, int32_t ty, int32_t bt, int64_t imm) {
      phcu_instr_t& c = p.code[p.n_instr++];
      c.op = (uint8_t)op;
      c.src = (uint8_t)sr;
      c.type = (uint8_t)ty;
      c.btype = (uint8_t)bt;
      c.imm.i = imm;
    };
    emit(PHCU_I_LD, 0, PHCU_BOOL, PHCU_BOOL, 0);
    emit(PHCU_I_ST0, 0, PHCU_BOOL, 0, 0);
    emit(PHCU_I_LD, 2, t, t, 0);
    if (src) emit(PHCU_I_SEL, 1, t, t, 0);
    else emit(PHCU_I_SEL, PHCU_SRC_IMM, t, t, detail::slot_bits(value));
    p.out_type = t;
    const phcu_view_t me = this->desc();
    phcu_view_t ins[3] = {mask.desc(), src ? src->desc() : me, me};
    check(phcu_eval(&p, ins, 3, &me), "phcu_eval");
  }
  template <typename R>
  void write_self(const CuProcView<R>& pv);
  CuNArray(std::shared_ptr<Buffer> buf, const std::vector<int64_t>& shape)
      : CuView<T>(std::move(buf), Affine{0, shape, row_major(shape)}) {}
};

template <typename T>
CuView<T> CuView<T>::reshape(const std::vector<int64_t>& new_shape) const {
  if (shape_to_size(new_shape) != size()) {
    auto text = [](const std::vector<int64_t>& v) {
      std::string t;
      for (size_t i = 0; i < v.size(); i++) t += (i ? "x" : "") + std::to_string(v[i]);
      return t;
    };
    throw ShapeError("Cannot change shape from " + text(aff_.shape) + " (" + std::to_string(size()) +
                     " elements) to " + text(new_shape) + " (" + std::to_string(shape_to_size(new_shape)) +
                     " elements) because reshape cannot add or remove elements.");
  }
  if (const std::optional<Affine> r = affine_reshape(aff_, new_shape)) return CuView(buf_, *r);
  const CuNArray<T> m = to_cu();  // not expressible with strides: read now into a contiguous copy
  return CuView(m.buffer(), Affine{0, new_shape, row_major(new_shape)});
}

template <typename T>
CuNArray<T> CuView<T>::to_cu() const {
  CuNArray<T> out(aff_.shape);
  const phcu_view_t d = out.desc(), s = desc();
  check(phcu_copy(&d, &s), "phcu_copy");
  return out;
}

template <typename T>
std::vector<T> CuView<T>::to_vector() const {
  return to_cu().to_vector();
}

// ------------------------------------------------------ infix operators
// def_elementwise_binary (multi_indexable.cr:931-945): the operands' shapes
// must match, the result has Crystal's type (Int32 / Int32 is Float64), and
// checked integer arithmetic raises OverflowError / DivisionByZeroError after
// the operation, as the reference does.
template <typename T>
struct DivResult {
  using type = T;
};
template <>
struct DivResult<int32_t> {
  using type = double;
};
template <>
struct DivResult<int64_t> {
  using type = double;
};

namespace detail {
inline bool can_raise(int32_t op, bool integral) {
  return integral && (op == PHCU_OP_ADD || op == PHCU_OP_SUB || op == PHCU_OP_MUL || op == PHCU_OP_FLOORDIV ||
                      op == PHCU_OP_MOD || op == PHCU_OP_POW);
}

template <typename R, typename T>
CuNArray<R> binary(int32_t op, const CuView<T>& a, const CuView<T>& b) {
  if (a.shape() != b.shape())
    throw ShapeError("Could not apply the elementwise operator: the operands' shapes differ.");
  int32_t t = -1;
  check(phcu_result_dtype(op, DType<T>::id, DType<T>::id, &t), "phcu_result_dtype");
  if (t != DType<R>::id) throw ArgumentError("unexpected result type of an elementwise operator");
  CuNArray<R> out(a.shape());
  const phcu_view_t x = a.desc(), y = b.desc(), o = out.desc();
  check(phcu_binary(op, &x, &y, &o), "phcu_binary");
  if (can_raise(op, std::is_integral<T>::value)) check_status();
  return out;
}

template <typename T>
CuNArray<T> binary_scalar(int32_t op, const CuView<T>& a, T value, bool scalar_left) {
  CuNArray<T> out(a.shape());
  phcu_scalar_t s;
  std::memset(&s, 0, sizeof(s));
  s.dtype = DType<T>::id;
  if (std::is_floating_point<T>::value) s.v.f = (double)value;
  else s.v.i = (int64_t)value;
  const phcu_view_t x = a.desc(), o = out.desc();
  check(phcu_binary_scalar(op, &x, &s, scalar_left ? 1 : 0, &o), "phcu_binary_scalar");
  if (can_raise(op, std::is_integral<T>::value)) check_status();
  return out;
}
}  // namespace detail

template <typename T>
CuNArray<T> operator+(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_ADD, a, b); }
template <typename T>
CuNArray<T> operator-(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_SUB, a, b); }
template <typename T>
CuNArray<T> operator*(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_MUL, a, b); }
template <typename T>
CuNArray<typename DivResult<T>::type> operator/(const CuView<T>& a, const CuView<T>& b) {
  return detail::binary<typename DivResult<T>::type>(PHCU_OP_DIV, a, b);
}
template <typename T>
CuNArray<T> operator+(const CuView<T>& a, T v) { return detail::binary_scalar<T>(PHCU_OP_ADD, a, v, false); }
template <typename T>
CuNArray<T> operator-(const CuView<T>& a, T v) { return detail::binary_scalar<T>(PHCU_OP_SUB, a, v, false); }
template <typename T>
CuNArray<T> operator-(T v, const CuView<T>& a) { return detail::binary_scalar<T>(PHCU_OP_SUB, a, v, true); }
template <typename T>
CuNArray<T> operator*(const CuView<T>& a, T v) { return detail::binary_scalar<T>(PHCU_OP_MUL, a, v, false); }

// Crystal's wrapping integer operators &+ &- &*.
template <typename T>
CuNArray<T> wadd(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_WADD, a, b); }
template <typename T>
CuNArray<T> wsub(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_WSUB, a, b); }
template <typename T>
CuNArray<T> wmul(const CuView<T>& a, const CuView<T>& b) { return detail::binary<T>(PHCU_OP_WMUL, a, b); }

// The elementwise comparisons > < >= <= and #eq (multi_indexable.cr:899-913):
// Bool arrays, the masks of set_mask.
template <typename T>
CuNArray<Bool> gt(const CuView<T>& a, const CuView<T>& b) { return detail::binary<Bool>(PHCU_OP_GT, a, b); }
template <typename T>
CuNArray<Bool> lt(const CuView<T>& a, const CuView<T>& b) { return detail::binary<Bool>(PHCU_OP_LT, a, b); }
template <typename T>
CuNArray<Bool> ge(const CuView<T>& a, const CuView<T>& b) { return detail::binary<Bool>(PHCU_OP_GE, a, b); }
template <typename T>
CuNArray<Bool> le(const CuView<T>& a, const CuView<T>& b) { return detail::binary<Bool>(PHCU_OP_LE, a, b); }
template <typename T>
CuNArray<Bool> eq(const CuView<T>& a, const CuView<T>& b) { return detail::binary<Bool>(PHCU_OP_EQ, a, b); }

// MultiIndexable#equals? / #== (multi_indexable.cr:74-84, 871-879): same shape
// and equal elements.  The comparison, a Bool -> Int32 conversion and the
// minimum run on the device; one Int32 comes back.
template <typename T>
bool equals(const CuView<T>& a, const CuView<T>& b) {
  if (a.shape() != b.shape()) return false;
  if (a.size() == 0) return true;
  const CuNArray<Bool> same = eq(a, b);
  CuNArray<int32_t> flags(a.shape());
  phcu_program_t p;
  std::memset(&p, 0, sizeof(p));
  p.n_instr = 2;
  p.out_type = PHCU_I32;
  p.code[0].op = PHCU_I_LD;
  p.code[0].type = p.code[0].btype = PHCU_BOOL;
  p.code[1].op = PHCU_I_CVT;
  p.code[1].type = p.code[1].btype = PHCU_BOOL;
  p.code[1].imm.i = PHCU_I32;
  const phcu_view_t in = same.desc(), o = flags.desc();
  check(phcu_eval(&p, &in, 1, &o), "phcu_eval");
  CuNArray<int32_t> m(std::vector<int64_t>{1});
  const phcu_view_t fv = flags.desc(), mv = m.desc();
  check(phcu_reduce(PHCU_RED_MIN, &fv, -1, &mv), "phcu_reduce");
  return m.to_vector()[0] == 1;
}

// ---------------------------------------------------- fused expressions
// ProcView (src/proc_view.cr:6-35) and chained infix operators build an
// expression over up to PHCU_MAX_INPUTS aliasing views; materialising it
// compiles the expression into the library's accumulator program
// (phcu_program_t) and runs ONE phcu_eval, instead of the reference's one
// map_with pass per operator (multi_indexable.cr:1026-1078).
namespace detail {
constexpr bool is_int_type(int32_t t) { return t == PHCU_I32 || t == PHCU_I64; }
constexpr bool is_float_type(int32_t t) { return t == PHCU_F32 || t == PHCU_F64; }

// Crystal's result type of `a op b` for numeric operands (Number#+ and
// friends; Int / Int is Float64, Int ** Float is Float64), or -1 where
// Crystal defines no such operator (bitwise or wrapping operators on floats).
constexpr int32_t result_type(int32_t op, int32_t ta, int32_t tb) {
  if (op == PHCU_OP_GT || op == PHCU_OP_LT || op == PHCU_OP_GE || op == PHCU_OP_LE || op == PHCU_OP_EQ)
    return PHCU_BOOL;
  if (op == PHCU_OP_CMP) return PHCU_I32;
  if (op == PHCU_OP_AND || op == PHCU_OP_OR || op == PHCU_OP_XOR)
    return is_int_type(ta) && is_int_type(tb) ? ta : -1;
  if (is_int_type(ta) && is_int_type(tb)) return op == PHCU_OP_DIV ? PHCU_F64 : ta;
  if (op == PHCU_OP_WADD || op == PHCU_OP_WSUB || op == PHCU_OP_WMUL || op == PHCU_OP_WPOW) return -1;
  if (is_int_type(ta) && is_float_type(tb) && op == PHCU_OP_POW) return PHCU_F64;
  return ta == PHCU_F64 || tb == PHCU_F64 ? PHCU_F64 : PHCU_F32;
}

// The type an instruction computes in: Float32 ** Int keeps the float and
// takes an integer exponent (repeated squaring, x ** 2 == x * x).
constexpr int32_t compute_type(int32_t op, int32_t ta, int32_t tb) {
  if (is_int_type(ta) && is_int_type(tb)) return ta;
  if (op == PHCU_OP_POW && is_float_type(ta) && is_int_type(tb)) return ta;
  if (is_int_type(ta) && is_float_type(tb) && op == PHCU_OP_POW) return PHCU_F64;
  return ta == PHCU_F64 || tb == PHCU_F64 ? PHCU_F64 : PHCU_F32;
}

// Operators whose kernel may set the status word: checked Int arithmetic
// (OverflowError, DivisionByZeroError, negative exponents) and `%`.
constexpr bool program_can_raise(int32_t op, int32_t ta, int32_t tb) {
  if (is_int_type(ta) && is_int_type(tb))
    return op == PHCU_OP_ADD || op == PHCU_OP_SUB || op == PHCU_OP_MUL || op == PHCU_OP_FLOORDIV ||
           op == PHCU_OP_MOD || op == PHCU_OP_POW || op == PHCU_OP_WPOW;
  return op == PHCU_OP_MOD;
}

// One node of an expression tree.
struct Expr {
  enum Kind { IN, CONST, BIN, UN } kind = IN;
  int32_t op = 0;          // BIN: PHCU_OP_*; UN: PHCU_I_NEG / PHCU_I_NOT / PHCU_I_POS
  int32_t t = 0;           // type of the node's value
  int32_t ta = 0, tb = 0;  // BIN: types of the operands
  int32_t slot = 0;        // IN: input slot
  int64_t bits = 0;        // CONST: the value's bit pattern in a program slot
  std::shared_ptr<const Expr> a, b;
};
using ExprP = std::shared_ptr<const Expr>;

inline ExprP input(int32_t slot, int32_t t) {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::IN;
  e->slot = slot;
  e->t = t;
  return e;
}

// The bit pattern of a constant in a 64-bit program slot: Float32 and Int32
// fill the low 32 bits (the rest zero), Float64 and Int64 all 64.
inline int64_t slot_bits(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  return (int64_t)u;
}
inline int64_t slot_bits(double v) {
  int64_t u;
  std::memcpy(&u, &v, 8);
  return u;
}
inline int64_t slot_bits(int32_t v) { return (int64_t)(uint32_t)v; }
inline int64_t slot_bits(int64_t v) { return v; }

template <typename S>
ExprP constant(S v) {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::CONST;
  e->t = DType<S>::id;
  e->bits = slot_bits(v);
  return e;
}

inline ExprP binary_expr(int32_t op, ExprP a, ExprP b) {
  const int32_t t = result_type(op, a->t, b->t);
  if (t < 0) throw NotImplementedError("the operator is not defined for these operand types");
  auto e = std::make_shared<Expr>();
  e->kind = Expr::BIN;
  e->op = op;
  e->ta = a->t;
  e->tb = b->t;
  e->t = t;
  e->a = std::move(a);
  e->b = std::move(b);
  return e;
}

inline ExprP unary_expr(int32_t op, ExprP a) {
  auto e = std::make_shared<Expr>();
  e->kind = Expr::UN;
  e->op = op;
  e->t = a->t;
  e->a = std::move(a);
  return e;
}

// The same tree with every input slot k replaced by map(k).
template <typename M>
ExprP relabel(const ExprP& e, const M& map) {
  if (e->kind == Expr::CONST) return e;
  auto n = std::make_shared<Expr>(*e);
  if (e->kind == Expr::IN) n->slot = map(e->slot);
  if (e->a) n->a = relabel(e->a, map);
  if (e->b) n->b = relabel(e->b, map);
  return n;
}

// Expression tree -> accumulator program.  Leaves (an input or a constant)
// become operand B of an instruction; a binary node whose operands are both
// compound evaluates the right one first into a stash register (S0, then S1
// one level deeper), so a program needs no stack.
class ProgramCompiler {
 public:
  phcu_program_t prog;
  bool raises = false;

  ProgramCompiler() { std::memset(&prog, 0, sizeof(prog)); }

  void run(const ExprP& e, int32_t out_type) {
    gen(*e, 0);
    if (e->t != out_type) emit(PHCU_I_CVT, 0, e->t, 0, out_type);
    prog.out_type = out_type;
  }

 private:
  void emit(int32_t op, int32_t src, int32_t t, int32_t bt, int64_t imm, int32_t flags = 0) {
    if (prog.n_instr >= PHCU_MAX_INSTR)
      throw NotImplementedError("fused program longer than " + std::to_string(PHCU_MAX_INSTR) + " instructions");
    phcu_instr_t& c = prog.code[prog.n_instr++];
    c.op = (uint8_t)op;
    c.src = (uint8_t)src;
    c.type = (uint8_t)t;
    c.btype = (uint8_t)bt;
    c.flags = (uint8_t)flags;
    c.imm.i = imm;
  }
  static bool leaf(const Expr& e) { return e.kind == Expr::IN || e.kind == Expr::CONST; }
  static int32_t src_of(const Expr& e) { return e.kind == Expr::IN ? e.slot : PHCU_SRC_IMM; }
  static int64_t imm_of(const Expr& e) { return e.kind == Expr::IN ? 0 : e.bits; }

  void gen(const Expr& e, int depth) {
    if (leaf(e)) {
      emit(PHCU_I_LD, src_of(e), e.t, e.t, imm_of(e));
      return;
    }
    if (e.kind == Expr::UN) {
      gen(*e.a, depth);
      if (e.op == PHCU_I_NEG && is_int_type(e.t)) raises = true;
      emit(e.op, 0, e.t, 0, 0);
      return;
    }
    const Expr& l = *e.a;
    const Expr& r = *e.b;
    const int32_t T = compute_type(e.op, e.ta, e.tb);
    if (program_can_raise(e.op, e.ta, e.tb)) raises = true;
    if (leaf(r)) {
      gen(l, depth);
      if (e.ta != T) emit(PHCU_I_CVT, 0, e.ta, 0, T);
      emit(e.op, src_of(r), T, r.t, imm_of(r));
    } else if (leaf(l) && e.op != PHCU_OP_POW) {  // ACC = B op ACC
      gen(r, depth);
      if (e.tb != T) emit(PHCU_I_CVT, 0, e.tb, 0, T);
      emit(e.op, src_of(l), T, l.t, imm_of(l), 1);
    } else {
      if (depth >= 2) throw NotImplementedError("expression too deep for the two stash registers");
      gen(r, depth);
      emit(depth == 0 ? PHCU_I_ST0 : PHCU_I_ST1, 0, e.tb, 0, 0);
      gen(l, depth + 1);
      if (e.ta != T) emit(PHCU_I_CVT, 0, e.ta, 0, T);
      emit(e.op, depth == 0 ? PHCU_SRC_S0 : PHCU_SRC_S1, T, e.tb, 0);
    }
    int32_t rt = T;
    if (e.op == PHCU_OP_GT || e.op == PHCU_OP_LT || e.op == PHCU_OP_GE || e.op == PHCU_OP_LE || e.op == PHCU_OP_EQ)
      rt = PHCU_BOOL;
    else if (e.op == PHCU_OP_CMP)
      rt = PHCU_I32;
    else if (e.op == PHCU_OP_DIV && is_int_type(T))
      rt = PHCU_F64;
    if (rt != e.t) emit(PHCU_I_CVT, 0, rt, 0, e.t);
  }
};

inline phcu_program_t compile_program(const ExprP& e, int32_t out_type, bool* raises) {
  ProgramCompiler c;
  c.run(e, out_type);
  if (raises) *raises = c.raises;
  return c.prog;
}

template <int32_t ID>
struct TypeOf;
template <>
struct TypeOf<PHCU_F32> {
  using type = float;
};
template <>
struct TypeOf<PHCU_F64> {
  using type = double;
};
template <>
struct TypeOf<PHCU_I32> {
  using type = int32_t;
};
template <>
struct TypeOf<PHCU_I64> {
  using type = int64_t;
};
}  // namespace detail

// The element type of `a op b` for element types A and B, as Crystal types it.
template <int32_t OP, typename A, typename B>
using BinResult = typename detail::TypeOf<detail::result_type(OP, DType<A>::id, DType<B>::id)>::type;

// The element handed to a process() block: operators on it record the
// expression instead of computing, so the blocks of a chain compose into one
// program (proc_view.cr:32-35).
template <typename T>
struct Sym {
  using value_type = T;
  detail::ExprP e;
  // Operand `slot` of a program (for building expressions by hand).
  static Sym input(int32_t slot) { return Sym{detail::input(slot, DType<T>::id)}; }
};

namespace detail {
template <typename S>
struct IsLiteral : std::false_type {};
template <>
struct IsLiteral<float> : std::true_type {};
template <>
struct IsLiteral<double> : std::true_type {};
template <>
struct IsLiteral<int32_t> : std::true_type {};
template <>
struct IsLiteral<int64_t> : std::true_type {};
template <typename X>
struct IsSym : std::false_type {};
template <typename T>
struct IsSym<Sym<T>> : std::true_type {};

// One operand view of a fused expression: the buffer it keeps alive and its
// layout.
struct Leaf {
  std::shared_ptr<Buffer> buf;
  Affine aff;
  int32_t dtype = 0;
  phcu_view_t desc() const { return make_view(buf ? buf->ptr : nullptr, dtype, aff); }
  bool same(const Leaf& o) const {
    return buf.get() == o.buf.get() && dtype == o.dtype && aff.offset == o.aff.offset && aff.shape == o.aff.shape &&
           aff.stride == o.aff.stride;
  }
};

inline size_t type_bytes(int32_t t) { return t == PHCU_BOOL ? 1 : (t == PHCU_I64 || t == PHCU_F64) ? 8 : 4; }

inline void leaf_slots(const Expr& e, std::vector<int32_t>& acc) {
  if (e.kind == Expr::IN) {
    if (std::find(acc.begin(), acc.end(), e.slot) == acc.end()) acc.push_back(e.slot);
    return;
  }
  if (e.a) leaf_slots(*e.a, acc);
  if (e.b) leaf_slots(*e.b, acc);
}

inline int expr_size(const Expr& e) {
  if (e.kind == Expr::IN || e.kind == Expr::CONST) return 0;
  return 1 + (e.a ? expr_size(*e.a) : 0) + (e.b ? expr_size(*e.b) : 0);
}

// Whether an expression over `nleaves` views compiles into one program.
inline bool fits(const ExprP& e, size_t nleaves, int32_t out_type) {
  if (nleaves > (size_t)PHCU_MAX_INPUTS) return false;
  try {
    compile_program(e, out_type, nullptr);
  } catch (const NotImplementedError&) {
    return false;
  }
  return true;
}

inline void operator_nodes(const ExprP& e, std::vector<ExprP>& acc) {
  for (const ExprP* c : {&e->a, &e->b}) {
    if (!*c) continue;
    if ((*c)->kind == Expr::BIN || (*c)->kind == Expr::UN) acc.push_back(*c);
    operator_nodes(*c, acc);
  }
}

inline ExprP replace_node(const ExprP& e, const Expr* old, const ExprP& with) {
  if (e.get() == old) return with;
  if (e->kind == Expr::IN || e->kind == Expr::CONST) return e;
  auto n = std::make_shared<Expr>(*e);
  if (e->a) n->a = replace_node(e->a, old, with);
  if (e->b) n->b = replace_node(e->b, old, with);
  return n;
}

// Splits an expression that one device program cannot hold (more than
// PHCU_MAX_INPUTS distinct views, more than PHCU_MAX_INSTR instructions, or
// nesting deeper than the two stash registers): the largest operator
// sub-expression that fits is evaluated into a temporary array of its own
// type, which becomes a new leaf, until the rest fits.  ProcView composes
// without limit (proc_view.cr:32-35); every operator still runs once per
// element in its own type, so the results equal the unsplit expression's.
// `raises` collects whether any piece can set the status word.
inline void split_to_fit(std::vector<Leaf>& leaves, ExprP& expr, const std::vector<int64_t>& shape,
                         int32_t out_type, bool* raises) {
  for (;;) {
    std::vector<int32_t> used;
    leaf_slots(*expr, used);
    if (fits(expr, used.size(), out_type)) break;
    std::vector<ExprP> nodes;
    operator_nodes(expr, nodes);
    ExprP best;
    for (const ExprP& n : nodes) {
      std::vector<int32_t> ids;
      leaf_slots(*n, ids);
      if (fits(n, ids.size(), n->t) && (!best || expr_size(*n) > expr_size(*best))) best = n;
    }
    if (!best) throw NotImplementedError("expression cannot be split into device programs");
    // the piece over its own leaves
    std::vector<int32_t> ids;
    leaf_slots(*best, ids);
    std::sort(ids.begin(), ids.end());
    ExprP piece = relabel(best, [&ids](int32_t k) {
      return (int32_t)(std::lower_bound(ids.begin(), ids.end(), k) - ids.begin());
    });
    bool r = false;
    const phcu_program_t p = compile_program(piece, best->t, &r);
    if (raises) *raises = *raises || r;
    const int64_t n = shape_to_size(shape);
    Leaf tmp{std::make_shared<Buffer>((size_t)std::max<int64_t>(n, 1) * type_bytes(best->t)),
             Affine{0, shape, row_major(shape)}, best->t};
    phcu_view_t ins[PHCU_MAX_INPUTS];
    std::memset(ins, 0, sizeof(ins));
    for (size_t k = 0; k < ids.size(); k++) ins[k] = leaves[(size_t)ids[k]].desc();
    const phcu_view_t o = tmp.desc();
    check(phcu_eval(&p, ins, (int32_t)ids.size(), &o), "phcu_eval");
    leaves.push_back(tmp);
    expr = replace_node(expr, best.get(), input((int32_t)leaves.size() - 1, best->t));
    // drop the leaves nothing reads any more
    std::vector<int32_t> keep;
    leaf_slots(*expr, keep);
    std::sort(keep.begin(), keep.end());
    std::vector<Leaf> kept;
    for (int32_t k : keep) kept.push_back(leaves[(size_t)k]);
    expr = relabel(expr, [&keep](int32_t k) {
      return (int32_t)(std::lower_bound(keep.begin(), keep.end(), k) - keep.begin());
    });
    leaves = std::move(kept);
  }
}

inline std::string shape_text(const std::vector<int64_t>& s) {
  std::string t = "[";
  for (size_t i = 0; i < s.size(); i++) t += (i ? ", " : "") + std::to_string(s[i]);
  return t + "]";
}

inline const char* op_name(int32_t op) {
  static const char* names[] = {"+", "-", "*", "/", "//", "%", "**", "&+", "&-", "&*", "&**", "&", "|", "^"};
  return op >= 0 && op < (int32_t)(sizeof(names) / sizeof(names[0])) ? names[op] : "?";
}
}  // namespace detail

// A lazy elementwise program over up to PHCU_MAX_INPUTS aliasing operand views
// (ProcView, src/proc_view.cr:6-35).  process() composes blocks; infix
// operators with other fused expressions, views, arrays or constants extend
// the program; the whole chain runs as ONE kernel when it is materialised
// (to_cu / to_vector / get_chunk / a reduction / set_chunk).  Identical
// operand views share one input slot.
template <typename T>
class CuProcView {
 public:
  CuProcView(std::vector<detail::Leaf> leaves, detail::ExprP expr, std::vector<int64_t> shape)
      : leaves_(std::move(leaves)), expr_(std::move(expr)), shape_(std::move(shape)) {
    std::vector<detail::Leaf> kept;
    std::vector<int32_t> slot(leaves_.size());
    for (size_t i = 0; i < leaves_.size(); i++) {
      size_t j = 0;
      while (j < kept.size() && !kept[j].same(leaves_[i])) j++;
      if (j == kept.size()) kept.push_back(leaves_[i]);
      slot[i] = (int32_t)j;
    }
    if (kept.size() != leaves_.size()) {
      expr_ = detail::relabel(expr_, [&slot](int32_t k) { return slot[k]; });
      leaves_ = std::move(kept);
    }
  }

  const std::vector<int64_t>& shape() const { return shape_; }
  int64_t size() const { return shape_to_size(shape_); }
  size_t dimensions() const { return shape_.size(); }
  const std::vector<detail::Leaf>& leaves() const { return leaves_; }
  const detail::ExprP& expr() const { return expr_; }

  // ProcView#process (proc_view.cr:32-35): another block on the result.
  template <typename F>
  auto process(F f) const {
    auto r = f(Sym<T>{expr_});
    using R = decltype(r);
    if constexpr (detail::IsLiteral<R>::value) {
      return CuProcView<R>(leaves_, detail::constant(r), shape_);  // a constant block
    } else {
      static_assert(detail::IsSym<R>::value, "a process block returns a Sym or a constant");
      return CuProcView<typename R::value_type>(leaves_, r.e, shape_);
    }
  }

  // Index transforms commute with an elementwise program, so view / permute /
  // reverse apply to every operand and the program stays as it is.
  CuProcView view(const std::vector<Lit>& region) const {
    const IndexRegion r = IndexRegion::make(region, shape_);
    std::vector<detail::Leaf> ls = leaves_;
    for (auto& l : ls) l.aff = affine_region(l.aff, r);
    return CuProcView(std::move(ls), expr_, affine_region(Affine{0, shape_, row_major(shape_)}, r).shape);
  }
  CuProcView permute(std::vector<int> order = {}) const {
    if (order.empty())
      for (size_t i = shape_.size(); i-- > 0;) order.push_back((int)i);
    std::vector<detail::Leaf> ls = leaves_;
    for (auto& l : ls) l.aff = affine_permute(l.aff, order);
    return CuProcView(std::move(ls), expr_, affine_permute(Affine{0, shape_, row_major(shape_)}, order).shape);
  }
  CuProcView reverse() const {
    std::vector<detail::Leaf> ls = leaves_;
    for (auto& l : ls) l.aff = affine_reverse(l.aff);
    return CuProcView(std::move(ls), expr_, shape_);
  }

  // The device program this expression compiles to; `raises` tells whether
  // it can set the status word (checked Int arithmetic).
  phcu_program_t program(bool* raises = nullptr) const {
    return detail::compile_program(expr_, DType<T>::id, raises);
  }

  // One phcu_eval into a new contiguous array (more than one when the
  // expression is larger than one device program: see detail::split_to_fit).
  CuNArray<T> to_cu() const {
    CuNArray<T> out(shape_);
    eval_into(out.desc());
    return out;
  }
  // The same into an existing view of this shape (an in-place map).
  void eval_into(const phcu_view_t& o) const {
    bool raises = false;
    std::vector<detail::Leaf> leaves = leaves_;
    detail::ExprP expr = expr_;
    detail::split_to_fit(leaves, expr, shape_, DType<T>::id, &raises);
    bool r = false;
    const phcu_program_t p = detail::compile_program(expr, DType<T>::id, &r);
    raises = raises || r;
    phcu_view_t ins[PHCU_MAX_INPUTS];
    std::memset(ins, 0, sizeof(ins));
    for (size_t k = 0; k < leaves.size(); k++) ins[k] = leaves[k].desc();
    check(phcu_eval(&p, ins, (int32_t)leaves.size(), &o), "phcu_eval");
    if (raises) check_status();
  }
  std::vector<T> to_vector() const { return to_cu().to_vector(); }
  // MultiIndexable#get_chunk: evaluates the region's elements only.
  CuNArray<T> get_chunk(const std::vector<Lit>& region) const { return view(region).to_cu(); }

 private:
  std::vector<detail::Leaf> leaves_;
  detail::ExprP expr_;
  std::vector<int64_t> shape_;
};

template <typename T>
void CuNArray<T>::set_chunk(const std::vector<Lit>& region, const CuProcView<T>& src) {
  const CuView<T> dst = this->view(region);
  for (const detail::Leaf& l : src.leaves()) refuse_reordered_alias(dst, l.buf.get(), l.aff);
  set_chunk(region, src.to_cu());
}

// In-place maps: the program is written into the array itself.  Every
// operand must read the array in its own element order (the reference reads
// and writes element by element); the array itself always does.
template <typename T>
template <typename R>
void CuNArray<T>::write_self(const CuProcView<R>& pv) {
  static_assert(std::is_same<R, T>::value, "an in-place map keeps the array's element type");
  for (const detail::Leaf& l : pv.leaves()) refuse_reordered_alias(*this, l.buf.get(), l.aff);
  pv.eval_into(this->desc());
}

template <typename T>
template <typename F>
CuNArray<T>& CuNArray<T>::map_inplace(F f) {
  write_self(this->process(f));
  return *this;
}

template <typename T>
template <typename U, typename F>
CuNArray<T>& CuNArray<T>::map_with_inplace(const CuView<U>& other, F f) {
  if (other.shape() != this->shape())
    throw ShapeError("The shape of this MultiIndexable (" + detail::shape_text(this->shape()) +
                     ") does not match the shape of the one provided (" + detail::shape_text(other.shape()) + ").");
  auto r = f(Sym<T>::input(0), Sym<U>::input(1));
  static_assert(detail::IsSym<decltype(r)>::value, "a map_with! block returns a Sym");
  using R = typename decltype(r)::value_type;
  write_self(CuProcView<R>({detail::Leaf{this->buf_, this->aff_, DType<T>::id},
                            detail::Leaf{other.buffer(), other.layout(), DType<U>::id}},
                           r.e, this->shape()));
  return *this;
}

template <typename T>
template <typename F>
CuNArray<T>& CuNArray<T>::map_with_index_inplace(F f) {
  auto r = f(Sym<T>::input(0), Sym<int32_t>::input(1));
  static_assert(detail::IsSym<decltype(r)>::value, "a map_with_index! block returns a Sym");
  using R = typename decltype(r)::value_type;
  const std::vector<int64_t>& sh = this->shape();
  write_self(CuProcView<R>({detail::Leaf{this->buf_, this->aff_, DType<T>::id},
                            detail::Leaf{nullptr, Affine{0, sh, row_major(sh)}, PHCU_INDEX}},
                           r.e, sh));
  return *this;
}

template <typename T>
template <typename F>
CuNArray<T>& CuNArray<T>::map_with_coord_inplace(F f) {
  const std::vector<int64_t>& sh = this->shape();
  std::vector<detail::Leaf> leaves = {detail::Leaf{this->buf_, this->aff_, DType<T>::id}};
  std::vector<Sym<int32_t>> coord;
  for (size_t d = 0; d < sh.size(); d++) {  // coordinate d: stride 1 on axis d, 0 elsewhere
    std::vector<int64_t> st(sh.size(), 0);
    st[d] = 1;
    leaves.push_back(detail::Leaf{nullptr, Affine{0, sh, st}, PHCU_INDEX});
    coord.push_back(Sym<int32_t>::input((int32_t)(d + 1)));
  }
  auto r = f(Sym<T>::input(0), coord);
  static_assert(detail::IsSym<decltype(r)>::value, "a map_with_coord! block returns a Sym");
  using R = typename decltype(r)::value_type;
  write_self(CuProcView<R>(std::move(leaves), r.e, sh));
  return *this;
}

template <typename T>
CuProcView<T> CuView<T>::process() const {
  return CuProcView<T>({detail::Leaf{buf_, aff_, DType<T>::id}}, detail::input(0, DType<T>::id), aff_.shape);
}

template <typename T>
template <typename F>
auto CuView<T>::process(F f) const {
  return process().process(f);
}

namespace detail {
template <typename T>
CuProcView<T> lift(const CuView<T>& v) {
  return v.process();
}

template <int32_t OP, typename A, typename B>
CuProcView<BinResult<OP, A, B>> combine(const CuProcView<A>& a, const CuProcView<B>& b) {
  if (a.shape() != b.shape())
    throw ShapeError("The shape of this MultiIndexable (" + shape_text(a.shape()) +
                     ") does not match the shape of the one provided (" + shape_text(b.shape()) + "), so '" +
                     op_name(OP) + "' cannot be applied element-wise.");
  std::vector<Leaf> leaves = a.leaves();
  const int32_t base = (int32_t)leaves.size();
  leaves.insert(leaves.end(), b.leaves().begin(), b.leaves().end());
  ExprP rhs = relabel(b.expr(), [base](int32_t k) { return k + base; });
  return CuProcView<BinResult<OP, A, B>>(std::move(leaves), binary_expr(OP, a.expr(), rhs), a.shape());
}
}  // namespace detail

// The lazy operators: on two Syms or a Sym and a constant (inside process
// blocks), and on a fused expression with another one, a view / array or a
// constant.  Constants take Crystal's literal types: int -> Int32, long
// (int64_t) -> Int64, float -> Float32, double -> Float64.  Eager operators
// between two plain views stay as they are (one kernel each).
#define PHASE_LAZY_BINARY(NAME, OPCODE)                                                                       \
  template <typename A, typename B>                                                                           \
  Sym<BinResult<OPCODE, A, B>> NAME(const Sym<A>& a, const Sym<B>& b) {                                       \
    return {detail::binary_expr(OPCODE, a.e, b.e)};                                                           \
  }                                                                                                           \
  template <typename A, typename S, typename = std::enable_if_t<detail::IsLiteral<S>::value>>                 \
  Sym<BinResult<OPCODE, A, S>> NAME(const Sym<A>& a, S s) {                                                   \
    return {detail::binary_expr(OPCODE, a.e, detail::constant(s))};                                           \
  }                                                                                                           \
  template <typename S, typename B, typename = std::enable_if_t<detail::IsLiteral<S>::value>>                 \
  Sym<BinResult<OPCODE, S, B>> NAME(S s, const Sym<B>& b) {                                                   \
    return {detail::binary_expr(OPCODE, detail::constant(s), b.e)};                                           \
  }                                                                                                           \
  template <typename A, typename B>                                                                           \
  CuProcView<BinResult<OPCODE, A, B>> NAME(const CuProcView<A>& a, const CuProcView<B>& b) {                  \
    return detail::combine<OPCODE>(a, b);                                                                     \
  }                                                                                                           \
  template <typename A, typename B>                                                                           \
  CuProcView<BinResult<OPCODE, A, B>> NAME(const CuProcView<A>& a, const CuView<B>& b) {                      \
    return detail::combine<OPCODE>(a, detail::lift(b));                                                       \
  }                                                                                                           \
  template <typename A, typename B>                                                                           \
  CuProcView<BinResult<OPCODE, A, B>> NAME(const CuView<A>& a, const CuProcView<B>& b) {                      \
    return detail::combine<OPCODE>(detail::lift(a), b);                                                       \
  }                                                                                                           \
  template <typename A, typename S, typename = std::enable_if_t<detail::IsLiteral<S>::value>>                 \
  CuProcView<BinResult<OPCODE, A, S>> NAME(const CuProcView<A>& a, S s) {                                     \
    return CuProcView<BinResult<OPCODE, A, S>>(a.leaves(), detail::binary_expr(OPCODE, a.expr(),              \
                                                                               detail::constant(s)),          \
                                               a.shape());                                                    \
  }                                                                                                           \
  template <typename S, typename B, typename = std::enable_if_t<detail::IsLiteral<S>::value>>                 \
  CuProcView<BinResult<OPCODE, S, B>> NAME(S s, const CuProcView<B>& b) {                                     \
    return CuProcView<BinResult<OPCODE, S, B>>(b.leaves(), detail::binary_expr(OPCODE, detail::constant(s),   \
                                                                               b.expr()),                     \
                                               b.shape());                                                    \
  }

PHASE_LAZY_BINARY(operator+, PHCU_OP_ADD)
PHASE_LAZY_BINARY(operator-, PHCU_OP_SUB)
PHASE_LAZY_BINARY(operator*, PHCU_OP_MUL)
PHASE_LAZY_BINARY(operator/, PHCU_OP_DIV)
PHASE_LAZY_BINARY(operator%, PHCU_OP_MOD)
PHASE_LAZY_BINARY(operator&, PHCU_OP_AND)
PHASE_LAZY_BINARY(operator|, PHCU_OP_OR)
PHASE_LAZY_BINARY(operator^, PHCU_OP_XOR)
PHASE_LAZY_BINARY(floordiv, PHCU_OP_FLOORDIV)  // Crystal //
PHASE_LAZY_BINARY(pow, PHCU_OP_POW)            // Crystal **
PHASE_LAZY_BINARY(wadd, PHCU_OP_WADD)          // Crystal &+
PHASE_LAZY_BINARY(wsub, PHCU_OP_WSUB)          // Crystal &-
PHASE_LAZY_BINARY(wmul, PHCU_OP_WMUL)          // Crystal &*
PHASE_LAZY_BINARY(wpow, PHCU_OP_WPOW)          // Crystal &**
#undef PHASE_LAZY_BINARY

// Unary minus (multi_indexable.cr:983-985); checked for Int operands.
template <typename T>
Sym<T> operator-(const Sym<T>& a) {
  return {detail::unary_expr(PHCU_I_NEG, a.e)};
}
template <typename T>
CuProcView<T> operator-(const CuProcView<T>& a) {
  return CuProcView<T>(a.leaves(), detail::unary_expr(PHCU_I_NEG, a.expr()), a.shape());
}

// ------------------------------------------------------------ reductions
// Enumerable#sum / #max / #min over the slices along an axis (multi_indexable.cr:
// 18, 742-786) and the argmax idiom (README.md:56-61: the first maximum wins).
namespace detail {
template <typename R, typename T>
CuNArray<R> reduce_axis(int32_t op, const CuView<T>& a, int axis) {
  const int d = (int)a.dimensions();
  if (axis < 0) axis += d;
  if (axis < 0 || axis >= d)
    throw IndexError("axis " + std::to_string(axis) + " is not present in a " + std::to_string(d) +
                     "-dimensional MultiIndexable");
  if (a.shape()[axis] == 0 && op != PHCU_RED_SUM) throw EmptyError("Empty enumerable");
  std::vector<int64_t> os = a.shape();
  os.erase(os.begin() + axis);
  CuNArray<R> out(os.empty() ? std::vector<int64_t>{1} : os);
  const phcu_view_t in = a.desc(), o = out.desc();
  check(phcu_reduce(op, &in, axis, &o), "phcu_reduce");
  if (op == PHCU_RED_SUM && std::is_integral<T>::value) check_status();
  return out;
}

template <typename R, typename T>
R reduce_all(int32_t op, const CuView<T>& a) {
  CuNArray<R> out(std::vector<int64_t>{1});
  const phcu_view_t in = a.desc(), o = out.desc();
  check(phcu_reduce(op, &in, -1, &o), "phcu_reduce");
  if (op == PHCU_RED_SUM && std::is_integral<T>::value) check_status();
  return out.to_vector()[0];
}

inline std::vector<int64_t> unravel(int64_t i, const std::vector<int64_t>& shape) {
  std::vector<int64_t> c(shape.size());
  for (size_t k = shape.size(); k-- > 0;) {
    c[k] = i % shape[k];
    i /= shape[k];
  }
  return c;
}
}  // namespace detail

template <typename T>
CuNArray<T> sum(const CuView<T>& a, int axis) { return detail::reduce_axis<T>(PHCU_RED_SUM, a, axis); }
template <typename T>
CuNArray<T> max(const CuView<T>& a, int axis) { return detail::reduce_axis<T>(PHCU_RED_MAX, a, axis); }
template <typename T>
CuNArray<T> min(const CuView<T>& a, int axis) { return detail::reduce_axis<T>(PHCU_RED_MIN, a, axis); }
template <typename T>
CuNArray<int32_t> argmax(const CuView<T>& a, int axis) { return detail::reduce_axis<int32_t>(PHCU_RED_ARGMAX, a, axis); }
template <typename T>
CuNArray<int32_t> argmin(const CuView<T>& a, int axis) { return detail::reduce_axis<int32_t>(PHCU_RED_ARGMIN, a, axis); }

// Over every element: the sum (zero when empty), the extreme values (EmptyError
// when empty) and the coordinate of the first maximum / minimum.
template <typename T>
T sum(const CuView<T>& a) {
  return a.size() == 0 ? T(0) : detail::reduce_all<T>(PHCU_RED_SUM, a);
}
template <typename T>
T max(const CuView<T>& a) {
  if (a.size() == 0) throw EmptyError("Empty enumerable");
  return detail::reduce_all<T>(PHCU_RED_MAX, a);
}
template <typename T>
T min(const CuView<T>& a) {
  if (a.size() == 0) throw EmptyError("Empty enumerable");
  return detail::reduce_all<T>(PHCU_RED_MIN, a);
}
template <typename T>
std::vector<int64_t> argmax(const CuView<T>& a) {
  if (a.size() == 0) throw EmptyError("Empty enumerable");
  return detail::unravel(detail::reduce_all<int64_t>(PHCU_RED_ARGMAX, a), a.shape());
}
template <typename T>
std::vector<int64_t> argmin(const CuView<T>& a) {
  if (a.size() == 0) throw EmptyError("Empty enumerable");
  return detail::unravel(detail::reduce_all<int64_t>(PHCU_RED_ARGMIN, a), a.shape());
}


// Reductions of a fused expression: the program runs once into a temporary,
// then the reduction kernel reads it.
template <typename T>
CuNArray<T> sum(const CuProcView<T>& a, int axis) { return sum(a.to_cu(), axis); }
template <typename T>
CuNArray<T> max(const CuProcView<T>& a, int axis) { return max(a.to_cu(), axis); }
template <typename T>
CuNArray<T> min(const CuProcView<T>& a, int axis) { return min(a.to_cu(), axis); }
template <typename T>
CuNArray<int32_t> argmax(const CuProcView<T>& a, int axis) { return argmax(a.to_cu(), axis); }
template <typename T>
CuNArray<int32_t> argmin(const CuProcView<T>& a, int axis) { return argmin(a.to_cu(), axis); }
template <typename T>
T sum(const CuProcView<T>& a) { return sum(a.to_cu()); }
template <typename T>
T max(const CuProcView<T>& a) { return max(a.to_cu()); }
template <typename T>
T min(const CuProcView<T>& a) { return min(a.to_cu()); }
template <typename T>
std::vector<int64_t> argmax(const CuProcView<T>& a) { return argmax(a.to_cu()); }
template <typename T>
std::vector<int64_t> argmin(const CuProcView<T>& a) { return argmin(a.to_cu()); }

}  // namespace phase
