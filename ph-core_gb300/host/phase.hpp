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

template <typename T>
class CuNArray;

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

  // View#to_narr (view.cr:123-126): one gather into a new contiguous array.
  CuNArray<T> to_cu() const;
  std::vector<T> to_vector() const;

 protected:
  std::shared_ptr<Buffer> buf_;
  Affine aff_;
};

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
    const phcu_view_t d = dst.desc(), s = src.desc();
    check(phcu_copy(&d, &s), "phcu_copy");
  }
  void set_chunk(const std::vector<Lit>& region, T value) { fill_view(this->view(region).desc(), value); }

 private:
  static int64_t count(const std::vector<int64_t>& shape) {
    for (int64_t s : shape)
      if (s < 0) throw DimensionError("Cannot create NArray: One or more of the provided dimensions was negative.");
    return shape.empty() ? 1 : shape_to_size(shape);
  }
  static void fill_view(const phcu_view_t& v, T value) {
    phcu_scalar_t s;
    std::memset(&s, 0, sizeof(s));
    s.dtype = DType<T>::id;
    if (std::is_floating_point<T>::value) s.v.f = (double)value;
    else s.v.i = (int64_t)value;
    check(phcu_fill(&v, &s), "phcu_fill");
  }
};

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

}  // namespace phase
