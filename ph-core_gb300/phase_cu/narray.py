"""Phase::CuNArray and its views: the MultiIndexable/MultiWritable surface on
device memory.

Mirrors the reference operator API (src/multi_indexable.cr, src/multi_writable.cr,
src/n_array.cr, src/view.cr, src/proc_view.cr, src/mutable_view.cr): same
method names (snake_case), argument meaning and exceptions.  Every bulk
method runs one library call; nothing is evaluated element by element on the
host.  Region validation happens here (as in the reference); the library
receives affine view descriptors.

  CuNArray       -- owns a contiguous row-major device buffer (NArray)
  CuView         -- lazy aliasing view: base buffer + affine map (View)
  CuMutableView  -- writable view (MutableView)
  CuProcView     -- lazy elementwise program over views (ProcView); infix
                    operators on it stay lazy and compile into ONE kernel
"""
import ctypes
import os

import numpy as np

from . import _abi as A
from .errors import ArgumentError, DimensionError, EmptyError, ShapeError
from .region import IndexRegion, check_region_fits, compatible_shapes, normalise_literal, shape_to_size

# ----------------------------------------------------------------- context
_ready = False


class config:
    """eager_errors: after an operation that can raise (checked integer
    arithmetic, float modulo), wait for it and raise like the reference does.
    When False, device errors surface at the next check_errors() call."""

    eager_errors = True


def init(device=None):
    global _ready
    if _ready:
        return
    lib = A.load()
    dev = int(os.environ.get("PHCU_DEVICE", "0")) if device is None else int(device)
    A.check(lib.phcu_init(dev), "phcu_init")
    _ready = True


def lib():
    init()
    return A.load()


def sync():
    A.call("phcu_sync") if _ready else None


def check_errors():
    """Reads and clears the device status word; raises the matching exception."""
    init()
    w = ctypes.c_uint32(0)
    A.check(lib().phcu_status_word(ctypes.byref(w), 1), "phcu_status_word")
    v = w.value
    if v & A.ST_DIVZERO:
        from .errors import DivisionByZeroError
        raise DivisionByZeroError("Division by 0")
    if v & A.ST_OVERFLOW:
        raise OverflowError("Arithmetic overflow")
    if v & A.ST_ARGUMENT:
        raise ArgumentError("Cannot raise an integer to a negative integer power, use floats for that")
    if v & A.ST_TIMEOUT:
        from .errors import DeviceError
        raise DeviceError("device work queue timed out")


# ------------------------------------------------------------------ dtypes
_NP = {A.BOOL: np.bool_, A.I32: np.int32, A.I64: np.int64, A.F32: np.float32, A.F64: np.float64}
_FROM_NP = {np.dtype(np.bool_): A.BOOL, np.dtype(np.int32): A.I32, np.dtype(np.int64): A.I64,
            np.dtype(np.float32): A.F32, np.dtype(np.float64): A.F64}

Bool, Int32, Int64, Float32, Float64 = A.BOOL, A.I32, A.I64, A.F32, A.F64


def dtype_of_numpy(dt):
    dt = np.dtype(dt)
    if dt not in _FROM_NP:
        raise TypeError("unsupported element type %s" % dt)
    return _FROM_NP[dt]


def np_dtype(t):
    return _NP[t]


def _is_int(t):
    return t in (A.I32, A.I64)


def _is_float(t):
    return t in (A.F32, A.F64)


def scalar_dtype(v):
    """Crystal literal type of a Python scalar: int -> Int32 (Int64 if it does
    not fit), float -> Float64, bool -> Bool; numpy scalars keep their type."""
    if isinstance(v, (bool, np.bool_)):
        return A.BOOL
    if isinstance(v, np.generic):
        return dtype_of_numpy(v.dtype)
    if isinstance(v, int):
        return A.I32 if -2 ** 31 <= v < 2 ** 31 else A.I64
    if isinstance(v, float):
        return A.F64
    raise TypeError("unsupported scalar %r" % (v,))


def result_dtype(op, ta, tb):
    """Crystal result type of `a op b` (same rules as the library)."""
    if ta == A.BOOL or tb == A.BOOL:
        if op == A.OP_EQ:
            return A.BOOL
        if ta == A.BOOL and tb == A.BOOL and op in (A.OP_AND, A.OP_OR, A.OP_XOR):
            return A.BOOL
        raise NotImplementedError("operator is not defined for Bool operands")
    if op in (A.OP_GT, A.OP_LT, A.OP_GE, A.OP_LE, A.OP_EQ):
        return A.BOOL
    if op == A.OP_CMP:
        return A.I32
    if op in (A.OP_AND, A.OP_OR, A.OP_XOR):
        if not (_is_int(ta) and _is_int(tb)):
            raise NotImplementedError("bitwise operator on a float operand")
        return ta
    if _is_int(ta) and _is_int(tb):
        return A.F64 if op == A.OP_DIV else ta
    if op in (A.OP_WADD, A.OP_WSUB, A.OP_WMUL, A.OP_WPOW):
        raise NotImplementedError("wrapping operator on a float operand")
    if _is_int(ta) and _is_float(tb) and op == A.OP_POW:
        return A.F64
    return A.F64 if A.F64 in (ta, tb) else A.F32


def _compute_type(op, ta, tb):
    if ta == A.BOOL and tb == A.BOOL:
        return A.BOOL
    if _is_int(ta) and _is_int(tb):
        return ta
    if op == A.OP_POW and _is_float(ta) and _is_int(tb):
        return ta
    if _is_int(ta) and _is_float(tb) and op == A.OP_POW:
        return A.F64
    return A.F64 if A.F64 in (ta, tb) else A.F32


def _slot_bits(value, t):
    """Bit pattern of a value in a 64-bit program slot of type t."""
    if t == A.F32:
        return int(np.array(value, dtype=np.float32).view(np.uint32))
    if t == A.F64:
        return int(np.array(value, dtype=np.float64).view(np.int64))
    if t == A.I32:
        return int(np.array(int(value), dtype=np.int64).astype(np.int32).view(np.uint32))
    if t == A.BOOL:
        return 1 if value else 0
    return int(np.int64(int(value)))


def _cast_scalar(value, t):
    return np.array(value).astype(_NP[t])[()]


# --------------------------------------------------------------- buffers
class _Buffer:
    """Device allocation owned by a CuNArray (freed when the last user goes)."""

    __slots__ = ("ptr", "nbytes", "__weakref__")

    def __init__(self, nbytes):
        init()
        p = ctypes.c_void_p()
        A.check(lib().phcu_alloc(max(int(nbytes), 1), ctypes.byref(p)), "phcu_alloc")
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def __del__(self):
        try:
            if self.ptr and A._lib is not None:
                A._lib.phcu_free(self.ptr)
        except Exception:
            pass
        self.ptr = None


def _row_major(shape):
    st = [0] * len(shape)
    s = 1
    for i in range(len(shape) - 1, -1, -1):
        st[i] = s
        s *= shape[i]
    return st


def _make_view(buf, dtype, offset, shape, stride):
    v = A.View()
    v.base = buf.ptr if buf is not None else None
    v.dtype = dtype
    v.rank = len(shape)
    v.offset = offset
    if len(shape) > A.MAX_RANK:
        raise DimensionError("rank %d exceeds the device limit of %d" % (len(shape), A.MAX_RANK))
    for i, (n, s) in enumerate(zip(shape, stride)):
        v.shape[i] = n
        v.stride[i] = s
    return v


# ------------------------------------------------- affine transform algebra
def _affine_region(offset, shape, stride, region):
    """Folds a RegionTransform (transforms.cr:191-222) into (offset, shape, stride)."""
    off = offset
    nshape, nstride = [], []
    for i in range(region.proper_dimensions):
        if region.proper_shape[i] > 0:
            off += region.first[i] * stride[i]
        if region.drop and region.degeneracy[i]:
            continue
        nshape.append(region.proper_shape[i])
        nstride.append(region.step[i] * stride[i])
    if not nshape:  # every axis dropped: shape [size] (index_region.cr:304-317)
        nshape, nstride = [shape_to_size(region.proper_shape)], [0]
    return off, nshape, nstride


def _affine_permute(offset, shape, stride, order):
    """PermuteTransform (transforms.cr:224-271): view axis i is source axis order[i]."""
    return offset, [shape[o] for o in order], [stride[o] for o in order]


def _affine_reverse(offset, shape, stride):
    """ReverseTransform (transforms.cr:273-305): every axis reversed."""
    off = offset
    for n, s in zip(shape, stride):
        if n > 0:
            off += (n - 1) * s
    return off, list(shape), [-s for s in stride]


def _affine_reshape(offset, shape, stride, new_shape):
    """ReshapeTransform (transforms.cr:118-189) when it stays affine: the lexicographic
    order of the view is regrouped without moving elements.  Returns None when the
    view's layout cannot express the new shape with strides."""
    old = [(n, s) for n, s in zip(shape, stride) if n != 1]
    new = list(new_shape)
    if shape_to_size(new) == 0 or shape_to_size(list(shape)) == 0:
        return offset, new, _row_major(new)
    nst = [0] * len(new)
    oi, ni = 0, 0
    on, nn = len(old), len(new)
    while ni < nn and oi < on:
        if new[ni] == 1:
            nst[ni] = 0
            ni += 1
            continue
        # group old axes [oi, oj) with new axes [ni, nj) of equal element count
        op, np_ = old[oi][0], new[ni]
        oj, nj = oi + 1, ni + 1
        while op != np_:
            if op < np_:
                if oj >= on:
                    return None
                op *= old[oj][0]
                oj += 1
            else:
                if nj >= nn:
                    return None
                np_ *= new[nj]
                nj += 1
        for k in range(oi, oj - 1):  # the old group must be contiguous in itself
            if old[k][1] != old[k + 1][1] * old[k + 1][0]:
                return None
        s = old[oj - 1][1]
        for k in range(nj - 1, ni - 1, -1):
            nst[k] = s
            s *= new[k]
        oi, ni = oj, nj
    while ni < nn:
        if new[ni] != 1:
            return None
        nst[ni] = 0
        ni += 1
    return offset, new, nst


# =========================================================== common surface
class _Indexable:
    """Shared MultiIndexable surface (src/multi_indexable.cr)."""

    dtype = A.F32

    # ------------------------------------------------ required by subclasses
    def _desc(self):
        """(buffer, offset, shape, stride) of an affine operand."""
        raise NotImplementedError

    # -------------------------------------------------------------- shape
    @property
    def shape(self):
        """A copy of the shape (multi_indexable.cr:45-47)."""
        return list(self._shape)

    @property
    def size(self):
        return shape_to_size(self._shape)

    @property
    def dimensions(self):
        return len(self._shape)

    def is_empty(self):
        return self.size == 0

    def is_scalar(self):
        return self.size == 1

    @property
    def np_dtype(self):
        return _NP[self.dtype]

    # -------------------------------------------------------- materialise
    def to_cu(self):
        """Materialises into a new contiguous CuNArray (one gather kernel)."""
        out = CuNArray.empty(self._shape, self.dtype)
        _copy_into(out._view(), self._cview())
        return out

    def to_narr(self):
        """Downloads into a numpy array (the host-side NArray)."""
        a = self if isinstance(self, CuNArray) else self.to_cu()
        host = np.empty(a._shape, dtype=_NP[a.dtype])
        if host.nbytes:
            A.check(lib().phcu_download(host.ctypes.data, a._buf.ptr, host.nbytes), "phcu_download")
        return host

    to_numpy = to_narr

    def _cview(self):
        buf, off, shape, stride = self._desc()
        return _make_view(buf, self.dtype, off, shape, stride)

    # -------------------------------------------------------------- access
    def get(self, *coord):
        """MultiIndexable#get (canonicalised, bounds-checked) -> Python scalar."""
        from .region import canonicalize_index

        coord = normalise_literal(coord)
        if len(coord) != self.dimensions:
            raise DimensionError("Could not canonicalize coordinate %r to fit in shape %r" % (coord, self.shape))
        coord = [canonicalize_index(c, n) for c, n in zip(coord, self._shape)]
        return self._fetch_element(coord)

    get_element = get

    def _fetch_element(self, coord):
        buf, off, shape, stride = self._desc()
        idx = off + sum(c * s for c, s in zip(coord, stride))
        host = np.empty(1, dtype=_NP[self.dtype])
        es = host.itemsize
        A.check(lib().phcu_download(host.ctypes.data, buf.ptr + idx * es, es), "phcu_download")
        return host[0].item()

    def get_chunk(self, *region_literal, drop=True):
        """MultiIndexable#get_chunk / #[] (multi_indexable.cr:354-356, 523-525)."""
        lits = normalise_literal(region_literal)
        if len(lits) == 1 and isinstance(lits[0], IndexRegion):
            region = lits[0]
            check_region_fits(region, self._shape)
        else:
            region = IndexRegion.new(lits, self._shape, drop)
        return self._unsafe_fetch_chunk(region)

    def __getitem__(self, key):
        if not isinstance(key, tuple):
            key = (key,)
        return self.get_chunk(*key)

    def get_available(self, *region_literal, drop=True):
        """MultiIndexable#get_available (multi_indexable.cr:397-413)."""
        lits = normalise_literal(region_literal)
        region = IndexRegion.trimmed(lits, self._shape, bound_shape=self._shape, drop=drop)
        return self._unsafe_fetch_chunk(region)

    def has_region(self, *region_literal):
        try:
            IndexRegion.new(normalise_literal(region_literal), self._shape)
            return True
        except (IndexError, DimensionError):
            return False

    def _unsafe_fetch_chunk(self, region):
        # default (NArray): a copy (n_array.cr:450-453)
        return self._region_view(region).to_cu()

    def _region_view(self, region):
        buf, off, shape, stride = self._desc()
        o, s, st = _affine_region(off, shape, stride, region)
        return CuView(self._base(), buf, self.dtype, o, s, st)

    def _base(self):
        return self

    # --------------------------------------------------------------- views
    def view(self, *region):
        """MultiIndexable#view (multi_indexable.cr:881-887): an aliasing CuView."""
        buf, off, shape, stride = self._desc()
        v = CuView(self._base(), buf, self.dtype, off, shape, stride)
        lits = normalise_literal(region)
        if lits:
            return v._restrict(lits)
        return v

    def process(self, fn=None):
        """MultiIndexable#process (multi_indexable.cr:889-895): a lazy CuProcView.
        `fn` receives a symbolic element and returns an expression built with
        infix operators, e.g. x.process(lambda e: (e + 4) ** 2)."""
        pv = CuProcView._leaf(self)
        return pv.process(fn) if fn is not None else pv

    def _as_leaf(self):
        """This operand as a read-only CuView leaf of a program."""
        buf, off, shape, stride = self._desc()
        return CuView(self._base(), buf, self.dtype, off, shape, stride)

    def _as_proc(self):
        return self if isinstance(self, CuProcView) else CuProcView._leaf(self)

    def process_with_index(self, fn):
        """Lazy form of map_with_index: fn(element, index) with the element's
        lexicographic index as an Int32 symbol (an index operand computed on the
        device, never stored)."""
        pv = self._as_proc()
        idx = CuIndexView.lex(self.shape)
        leaves = list(pv._leaves) + [idx]
        out = fn(_Sym(pv._expr, pv.dtype), _Sym(("in", len(leaves) - 1, A.I32), A.I32))
        return CuProcView._of_result(leaves, out, self.shape)

    def process_with_coord(self, fn):
        """Lazy form of map_with_coord: fn(element, coord), coord a list of
        Int32 symbols, one per axis (index operands computed on the device)."""
        pv = self._as_proc()
        leaves = list(pv._leaves)
        coord = []
        for d in range(self.dimensions):
            leaves.append(CuIndexView.axis(self.shape, d))
            coord.append(_Sym(("in", len(leaves) - 1, A.I32), A.I32))
        out = fn(_Sym(pv._expr, pv.dtype), coord)
        return CuProcView._of_result(leaves, out, self.shape)

    def map(self, fn):
        """MultiIndexable#map / NArray#map (multi_indexable.cr:722-726,
        n_array.cr:589-595): a new array of fn(element), one kernel."""
        return self.process(fn).to_cu()

    def map_with_index(self, fn):
        """NArray#map_with_index (n_array.cr:605-611): a new array of
        fn(element, lexicographic index), one kernel."""
        return self.process_with_index(fn).to_cu()

    def map_with_coord(self, fn):
        """MultiIndexable#map_with_coord (multi_indexable.cr:708-712,
        n_array.cr:614-618): a new array of fn(element, coord), one kernel."""
        return self.process_with_coord(fn).to_cu()

    def process_with(self, *args):
        """Lazy form of map_with: the last argument is the block, called with
        this element and the elements of every MultiIndexable argument (scalar
        arguments are passed as they are)."""
        *others, fn = args
        if not callable(fn):
            raise ArgumentError("map_with: the last argument must be the block")
        pv = self._as_proc()
        leaves = list(pv._leaves)
        syms = []
        for o in others:
            if isinstance(o, _Indexable):
                if o.shape != self.shape:
                    raise ShapeError("The shape of this MultiIndexable (%r) does not match the shape of the one "
                                     "provided (%r), so 'map_with' cannot be applied element-wise."
                                     % (self.shape, o.shape))
                op = o._as_proc()
                base = len(leaves)
                leaves += op._leaves
                syms.append(_Sym(_shift(op._expr, base), op.dtype))
            else:
                syms.append(o)
        out = fn(_Sym(pv._expr, pv.dtype), *syms)
        return CuProcView._of_result(leaves, out, self.shape)

    def map_with(self, *args):
        """MultiIndexable#map_with (multi_indexable.cr:1026-1078): a new array of
        fn(element, *argument elements); the last argument is the block."""
        return self.process_with(*args).to_cu()

    # in-place forms (Mutable#map!, #map_with!, #map_with_coord!; NArray#map_with_index!)
    def _write_self(self, pv):
        if not isinstance(self, (CuNArray, CuMutableView)):
            raise NotImplementedError("%s is read-only: in-place maps need a CuNArray or a CuMutableView"
                                      % type(self).__name__)
        mine = self._desc()
        for leaf in pv._leaves:
            if not isinstance(leaf, CuIndexView):
                _refuse_reordered_alias(mine, leaf._desc(), "in-place map")
        out = self._cview()
        pv._eval_into(out, self.dtype)
        return self

    def map_inplace(self, fn):
        """Mutable#map! / NArray#map! (mutable.cr:29-33, n_array.cr:621-627):
        self = fn(self), one kernel."""
        return self._write_self(self.process(fn))

    def map_with_index_inplace(self, fn):
        """NArray#map_with_index! (n_array.cr:631-637): self = fn(self, index)."""
        return self._write_self(self.process_with_index(fn))

    def map_with_coord_inplace(self, fn):
        """Mutable#map_with_coord! / NArray#map_with_coord! (mutable.cr:16-20,
        n_array.cr:641-650): self = fn(self, coord)."""
        return self._write_self(self.process_with_coord(fn))

    def map_with_inplace(self, *args):
        """Mutable#map_with! (mutable.cr:54-67): self = fn(self, *argument
        elements); the last argument is the block."""
        return self._write_self(self.process_with(*args))

    # --------------------------------------------------- iteration (host)
    def each(self):
        return iter(self.to_narr().reshape(-1).tolist())

    def fast_each(self):
        return self.each()

    def each_with_coord(self):
        a = self.to_narr()
        for idx in np.ndindex(*a.shape):
            yield a[idx].item(), list(idx)

    def to_a(self):
        return self.to_narr().reshape(-1).tolist()

    # -------------------------------------------------------------- slices
    def each_slice(self, axis=0):
        """MultiIndexable#each_slice (multi_indexable.cr:742-748): axis `axis` fixed
        and dropped, in increasing index order."""
        if not (0 <= axis < self.dimensions):
            raise IndexError("axis %d is not present in a %d-dimensional MultiIndexable" % (axis, self.dimensions))
        for i in range(self._shape[axis]):
            lits = [slice(None)] * self.dimensions
            lits[axis] = i
            yield self.get_chunk(*lits)

    def slices(self, axis=0):
        return list(self.each_slice(axis))

    # ------------------------------------------- materialising transforms
    def permute(self, *order):
        """MultiIndexable#permute (multi_indexable.cr:795-803): a permuted copy."""
        return self.view().permute(*order).to_cu()

    def reverse(self):
        return self.view().reverse().to_cu()

    def reshape(self, *new_shape):
        return self.view().reshape(*new_shape).to_cu()

    # ------------------------------------------------------------ compare
    def equals(self, other):
        """MultiIndexable#equals? with == (multi_indexable.cr:871-879): the
        elementwise comparison and the all-reduction run on the device; one
        Int32 comes back."""
        if self.shape != other.shape:
            return False
        if self.size == 0:
            return True
        same = self.eq(other)
        flags = CuNArray.empty(self._shape, A.I32)
        P = A.Program()
        P.n_instr = 2
        P.out_type = A.I32
        for i, (op, t, imm) in enumerate(((A.I_LD, A.BOOL, 0), (A.I_CVT, A.BOOL, A.I32))):
            c = P.code[i]
            c.op, c.src, c.type, c.btype, c.flags = op, 0, t, t, 0
            c.imm.i = imm
        ins = (A.View * 1)(same._cview())
        A.check(lib().phcu_eval(ctypes.byref(P), ins, 1, ctypes.byref(flags._view())), "phcu_eval")
        return flags.min() == 1

    def __eq__(self, other):
        """MultiIndexable#== (multi_indexable.cr:74-84): same type, shape and elements."""
        if not isinstance(other, _Indexable):
            return False
        return self.equals(other)

    __hash__ = None

    def eq(self, other):
        """Elementwise equality -> Bool array (multi_indexable.cr:899-913)."""
        if isinstance(other, _Indexable) and self.shape != other.shape:
            raise DimensionError("Cannot compute the element-wise equality between this MultiIndexable (shape: %r) "
                                 "and the one provided (shape: %r)." % (self.shape, other.shape))
        return self._binary(A.OP_EQ, other)

    # ------------------------------------------------------------ infix ops
    def _binary(self, op, other, reflected=False):
        if isinstance(other, CuProcView):
            me = CuProcView._leaf(self)
            return me._binary(op, other, reflected)
        if isinstance(other, _Indexable):
            a, b = (other, self) if reflected else (self, other)
            if a._shape != b._shape:
                name = _OP_NAMES.get(op, str(op))
                if a.is_scalar() or b.is_scalar():
                    raise ShapeError("The shape of this MultiIndexable (%r) does not match the shape of the one "
                                     "provided (%r), so '%s' cannot be applied element-wise. Did you mean to call "
                                     "to_scalar on one of the arguments?" % (a.shape, b.shape, name))
                raise ShapeError("The shape of this MultiIndexable (%r) does not match the shape of the one provided "
                                 "(%r), so '%s' cannot be applied element-wise." % (a.shape, b.shape, name))
            tout = result_dtype(op, a.dtype, b.dtype)
            out = CuNArray.empty(self._shape, tout)
            A.check(lib().phcu_binary(op, ctypes.byref(a._cview()), ctypes.byref(b._cview()),
                                      ctypes.byref(out._view())), "phcu_binary")
            _after(op, a.dtype, b.dtype)
            return out
        # scalar operand
        st = scalar_dtype(other)
        ta, tb = (st, self.dtype) if reflected else (self.dtype, st)
        tout = result_dtype(op, ta, tb)
        out = CuNArray.empty(self._shape, tout)
        s = A.Scalar()
        s.dtype = st
        if _is_float(st):
            s.v.f = float(other)
        else:
            s.v.i = int(other)
        A.check(lib().phcu_binary_scalar(op, ctypes.byref(self._cview()), ctypes.byref(s), 1 if reflected else 0,
                                         ctypes.byref(out._view())), "phcu_binary_scalar")
        _after(op, ta, tb)
        return out

    def __add__(self, o): return self._binary(A.OP_ADD, o)
    def __radd__(self, o): return self._binary(A.OP_ADD, o, True)
    def __sub__(self, o): return self._binary(A.OP_SUB, o)
    def __rsub__(self, o): return self._binary(A.OP_SUB, o, True)
    def __mul__(self, o): return self._binary(A.OP_MUL, o)
    def __rmul__(self, o): return self._binary(A.OP_MUL, o, True)
    def __truediv__(self, o): return self._binary(A.OP_DIV, o)
    def __rtruediv__(self, o): return self._binary(A.OP_DIV, o, True)
    def __floordiv__(self, o): return self._binary(A.OP_FLOORDIV, o)
    def __rfloordiv__(self, o): return self._binary(A.OP_FLOORDIV, o, True)
    def __mod__(self, o): return self._binary(A.OP_MOD, o)
    def __rmod__(self, o): return self._binary(A.OP_MOD, o, True)
    def __pow__(self, o): return self._binary(A.OP_POW, o)
    def __rpow__(self, o): return self._binary(A.OP_POW, o, True)
    def __and__(self, o): return self._binary(A.OP_AND, o)
    def __rand__(self, o): return self._binary(A.OP_AND, o, True)
    def __or__(self, o): return self._binary(A.OP_OR, o)
    def __ror__(self, o): return self._binary(A.OP_OR, o, True)
    def __xor__(self, o): return self._binary(A.OP_XOR, o)
    def __rxor__(self, o): return self._binary(A.OP_XOR, o, True)
    def __gt__(self, o): return self._binary(A.OP_GT, o)
    def __lt__(self, o): return self._binary(A.OP_LT, o)
    def __ge__(self, o): return self._binary(A.OP_GE, o)
    def __le__(self, o): return self._binary(A.OP_LE, o)

    def wadd(self, o):
        """Crystal `&+` (wrapping addition)."""
        return self._binary(A.OP_WADD, o)

    def wsub(self, o):
        """Crystal `&-`."""
        return self._binary(A.OP_WSUB, o)

    def wmul(self, o):
        """Crystal `&*`."""
        return self._binary(A.OP_WMUL, o)

    def wpow(self, o):
        """Crystal `&**`."""
        return self._binary(A.OP_WPOW, o)

    def cmp(self, o):
        """Crystal `<=>` elementwise -> Int32 array."""
        return self._binary(A.OP_CMP, o)

    def _unary(self, uop):
        if self.dtype == A.BOOL or (uop == A.UOP_NOT and not _is_int(self.dtype)):
            raise NotImplementedError("unary operator not defined for %s" % A.DTYPE_NAMES[self.dtype])
        out = CuNArray.empty(self._shape, self.dtype)
        A.check(lib().phcu_unary(uop, ctypes.byref(self._cview()), ctypes.byref(out._view())), "phcu_unary")
        if uop == A.UOP_NEG and _is_int(self.dtype) and config.eager_errors:
            check_errors()
        return out

    def __neg__(self): return self._unary(A.UOP_NEG)
    def __pos__(self): return self._unary(A.UOP_POS)
    def __invert__(self): return self._unary(A.UOP_NOT)

    # ---------------------------------------------------------- reductions
    def _reduce(self, op, axis, out_dtype=None):
        if self.dtype == A.BOOL and op == A.RED_SUM:
            raise NotImplementedError("sum of Bool")
        src = self
        if axis is None:
            n = self.size
            if n == 0:
                if op == A.RED_SUM:
                    return _NP[self.dtype](0).item()
                raise EmptyError("Empty enumerable")
            oshape = [1]
        else:
            if axis < 0:
                axis += self.dimensions
            if not (0 <= axis < self.dimensions):
                raise IndexError("axis %d is not present in a %d-dimensional MultiIndexable" % (axis, self.dimensions))
            if self._shape[axis] == 0 and op != A.RED_SUM:
                raise EmptyError("Empty enumerable")
            oshape = self._shape[:axis] + self._shape[axis + 1:]
        if out_dtype is None:
            out_dtype = A.I32 if op in (A.RED_ARGMAX, A.RED_ARGMIN) and axis is not None else (
                A.I64 if op in (A.RED_ARGMAX, A.RED_ARGMIN) else self.dtype)
        out = CuNArray.empty(oshape if oshape else [1], out_dtype)
        A.check(lib().phcu_reduce(op, ctypes.byref(src._cview()), -1 if axis is None else axis,
                                  ctypes.byref(out._view())), "phcu_reduce")
        if op == A.RED_SUM and _is_int(self.dtype) and config.eager_errors:
            check_errors()
        if axis is None:
            v = out.to_narr().reshape(-1)[0].item()
            if op in (A.RED_ARGMAX, A.RED_ARGMIN):
                return list(np.unravel_index(int(v), self._shape)) if self._shape else [int(v)]
            return v
        if not oshape:
            return out.to_narr().reshape(-1)[0].item()
        return out

    def sum(self, axis=None, dtype=None):
        """Enumerable#sum (axis=None) or the slices(axis) fold; Float32 sums are
        compensated on the device (pass dtype=Float64 for an FP64 result)."""
        return self._reduce(A.RED_SUM, axis, dtype)

    def max(self, axis=None):
        return self._reduce(A.RED_MAX, axis)

    def min(self, axis=None):
        return self._reduce(A.RED_MIN, axis)

    def argmax(self, axis=None):
        """README.md:56-61 idiom: first maximum wins; axis=None returns its coordinate."""
        return self._reduce(A.RED_ARGMAX, axis)

    def argmin(self, axis=None):
        return self._reduce(A.RED_ARGMIN, axis)

    def __repr__(self):
        return "%s(%s, %s)" % (type(self).__name__, "x".join(map(str, self._shape)), A.DTYPE_NAMES[self.dtype])

    # ---------------------------------------------------------- printing
    def to_s(self, settings=None):
        """MultiIndexable#to_s (formatter/formatter.cr:304-315): only the
        displayed elements are gathered on the device and downloaded."""
        from . import formatter

        return formatter.to_s(self, settings)

    __str__ = to_s

    def to_literal_s(self):
        """MultiIndexable#to_literal_s (formatter/formatter.cr:298-300)."""
        from . import formatter

        return formatter.to_literal_s(self)


_OP_NAMES = {A.OP_ADD: "+", A.OP_SUB: "-", A.OP_MUL: "*", A.OP_DIV: "/", A.OP_FLOORDIV: "//", A.OP_MOD: "%",
             A.OP_POW: "**", A.OP_WADD: "&+", A.OP_WSUB: "&-", A.OP_WMUL: "&*", A.OP_WPOW: "&**",
             A.OP_AND: "&", A.OP_OR: "|", A.OP_XOR: "^", A.OP_GT: ">", A.OP_LT: "<", A.OP_GE: ">=",
             A.OP_LE: "<=", A.OP_CMP: "<=>", A.OP_EQ: "=="}


def _can_raise(op, ta, tb):
    if _is_int(ta) and _is_int(tb):
        return op in (A.OP_ADD, A.OP_SUB, A.OP_MUL, A.OP_FLOORDIV, A.OP_MOD, A.OP_POW, A.OP_WPOW)
    return op == A.OP_MOD


def _after(op, ta, tb):
    if config.eager_errors and _can_raise(op, ta, tb):
        check_errors()


def _copy_into(dst_view, src_view):
    A.check(lib().phcu_copy(ctypes.byref(dst_view), ctypes.byref(src_view)), "phcu_copy")


# ================================================================ CuNArray
class CuNArray(_Indexable):
    """Device-resident NArray (src/n_array.cr:15-913): contiguous row-major buffer."""

    def __init__(self, shape, dtype, buf=None):
        shape = [int(s) for s in shape]
        for s in shape:
            if s < 0:
                raise DimensionError("Cannot create NArray: One or more of the provided dimensions was negative.")
        self._shape = shape
        self.dtype = dtype
        n = shape_to_size(shape) if shape else 1
        self._buf = buf if buf is not None else _Buffer(n * A.DTYPE_SIZE[dtype])

    # --------------------------------------------------------- constructors
    @classmethod
    def empty(cls, shape, dtype=A.F32):
        return cls(list(shape), dtype)

    @classmethod
    def of_buffer(cls, shape, buffer):
        """NArray.of_buffer (n_array.cr:76-79): shape + lexicographic buffer (numpy)."""
        buffer = np.ascontiguousarray(buffer)
        shape = list(shape)
        if shape_to_size(shape) != buffer.size:
            raise ShapeError("Cannot create NArray: Given shape does not match number of elements in buffer.")
        a = cls(shape, dtype_of_numpy(buffer.dtype))
        if buffer.nbytes:
            A.check(lib().phcu_upload(a._buf.ptr, buffer.ctypes.data, buffer.nbytes), "phcu_upload")
            A.call("phcu_sync")
        return a

    @classmethod
    def from_numpy(cls, arr):
        arr = np.asarray(arr)
        return cls.of_buffer(list(arr.shape), arr)

    @classmethod
    def new(cls, nested):
        """NArray.new(nested array) / NArray[...]."""
        return cls.from_numpy(np.asarray(nested))

    @classmethod
    def fill(cls, shape, value, dtype=None):
        """NArray.fill (n_array.cr:230-232)."""
        t = dtype if dtype is not None else scalar_dtype(value)
        a = cls(list(shape), t)
        a._fill_view(a._view(), value)
        return a

    @classmethod
    def build(cls, shape, fn):
        """NArray.build (n_array.cr:111-116): the block runs on the host, then uploads."""
        shape = list(shape)
        vals = [fn(list(c), i) for i, c in enumerate(np.ndindex(*shape))] if shape_to_size(shape) else []
        arr = np.array(vals).reshape(shape) if vals else np.zeros(shape, dtype=np.int32)
        return cls.of_buffer(shape, arr)

    def clone(self):
        out = CuNArray.empty(self._shape, self.dtype)
        _copy_into(out._view(), self._view())
        return out

    # ------------------------------------------------------- serialisation
    def to_json(self):
        """NArray#to_json (n_array.cr:807-817): one bulk download."""
        from . import serial
        return serial.to_json(self.to_narr())

    def to_yaml(self):
        """NArray#to_yaml (n_array.cr:854-868): one bulk download."""
        from . import serial
        return serial.to_yaml(self.to_narr())

    @classmethod
    def from_json(cls, text, dtype):
        """NArray(T).from_json (n_array.cr:819-852): parse, then one upload."""
        from . import serial
        return cls.from_numpy(serial.from_json(text, _NP[dtype]))

    @classmethod
    def from_yaml(cls, text, dtype):
        """NArray(T).from_yaml (n_array.cr:870-911): parse, then one upload."""
        from . import serial
        return cls.from_numpy(serial.from_yaml(text, _NP[dtype]))

    @classmethod
    def tile(cls, source, counts):
        """NArray.tile (n_array.cr:242-252): repeats source counts[i] times along
        axis i.  One strided copy: the output seen as [c0, s0, c1, s1, ...]
        receives the source read with stride 0 along every c axis (split into
        several copies when that view would exceed the device's rank limit)."""
        if isinstance(source, CuProcView):
            source = source.to_cu()
        sshape = list(source.shape)
        counts = [int(c) for c in counts]
        if len(counts) < len(sshape):
            raise IndexError("tile: %d counts for a %d-dimensional source" % (len(counts), len(sshape)))
        if any(c < 0 for c in counts[:len(sshape)]):
            raise ValueError("tile: negative count")
        shape = [n * c for n, c in zip(sshape, counts)]
        out = cls(shape, source.dtype)
        if shape_to_size(shape) == 0:
            return out
        sbuf, soff, _, sst = source._desc()
        ost = _row_major(shape)
        R = len(sshape)
        # leading axes that a rank-8 descriptor cannot pair (lead + 2 (R - lead) <= 8) are walked on the host
        lead = max(0, 2 * R - A.MAX_RANK)
        for prefix in np.ndindex(*counts[:lead]) if lead else [()]:
            dshape, dst, sshape2, sst2 = [], [], [], []
            doff = 0
            for i in range(R):
                if i < lead:
                    doff += prefix[i] * sshape[i] * ost[i]
                    dshape.append(sshape[i])
                    dst.append(ost[i])
                    sshape2.append(sshape[i])
                    sst2.append(sst[i])
                else:
                    dshape += [counts[i], sshape[i]]
                    dst += [sshape[i] * ost[i], ost[i]]
                    sshape2 += [counts[i], sshape[i]]
                    sst2 += [0, sst[i]]
            _copy_into(_make_view(out._buf, out.dtype, doff, dshape, dst),
                       _make_view(sbuf, source.dtype, soff, sshape2, sst2))
        return out

    @classmethod
    def concatenate(cls, *narrs, axis=0):
        """NArray.concatenate (n_array.cr:719-749): one strided copy of each
        operand into its slab of the output along `axis`."""
        if len(narrs) == 1 and isinstance(narrs[0], (list, tuple)):
            narrs = tuple(narrs[0])
        narrs = [n.to_cu() if isinstance(n, CuProcView) else n for n in narrs]
        first = narrs[0]
        rank = first.dimensions
        ax = axis + rank if axis < 0 else axis
        for n in narrs[1:]:
            if n.dimensions != rank or any(a != b for i, (a, b) in enumerate(zip(first.shape, n.shape)) if i != ax):
                raise DimensionError("Cannot concatenate these arrays along axis %d: shapes do not match" % axis)
            if n.dtype != first.dtype:
                raise TypeError("Cannot concatenate arrays of different element types")
        if not 0 <= ax < rank:
            raise IndexError("axis %d is not present in a %d-dimensional MultiIndexable" % (axis, rank))
        shape = list(first.shape)
        shape[ax] = sum(n.shape[ax] for n in narrs)
        out = cls(shape, first.dtype)
        ost = _row_major(shape)
        pos = 0
        for n in narrs:
            k = n.shape[ax]
            if k and n.size:
                sub = list(shape)
                sub[ax] = k
                _copy_into(_make_view(out._buf, out.dtype, pos * ost[ax], sub, ost), n._cview())
            pos += k
        return out

    def push(self, *others, axis=0):
        """NArray#push / #<< (n_array.cr:682-712): appends others along axis 0
        in place (the buffer is replaced by the concatenation)."""
        if axis != 0:
            raise ValueError("push appends along axis 0 only")
        cat = CuNArray.concatenate(self, *others, axis=0)
        self._buf, self._shape = cat._buf, cat._shape
        return self

    def __lshift__(self, other):
        return self.push(other)

    # ------------------------------------------------------------- layout
    def _desc(self):
        return self._buf, 0, list(self._shape), _row_major(self._shape)

    def _view(self):
        return _make_view(self._buf, self.dtype, 0, self._shape, _row_major(self._shape))

    @property
    def buffer(self):
        return self.to_narr().reshape(-1)

    def reshape(self, *new_shape):
        """NArray#reshape (n_array.cr:429-437): same buffer, new shape."""
        new_shape = normalise_literal(new_shape)
        if shape_to_size(new_shape) != self.size:
            raise ShapeError("Cannot create NArray: Given shape does not match number of elements in buffer.")
        return CuNArray(new_shape, self.dtype, self._buf)

    def flatten(self):
        return self.reshape(self.size)

    # ------------------------------------------------------------ writing
    def _fill_view(self, view, value):
        s = A.Scalar()
        s.dtype = self.dtype
        v = _cast_scalar(value, self.dtype)
        if _is_float(self.dtype):
            s.v.f = float(v)
        else:
            s.v.i = int(v)
        A.check(lib().phcu_fill(ctypes.byref(view), ctypes.byref(s)), "phcu_fill")

    def set_chunk(self, *args):
        """MultiWritable#set_chunk / #[]= (multi_writable.cr:55-84)."""
        *lits, src = args
        lits = normalise_literal(lits)
        if len(lits) == 1 and isinstance(lits[0], IndexRegion):
            region = lits[0]
        else:
            region = IndexRegion.new(lits, self._shape)
        _write_region(self, region, src)

    def __setitem__(self, key, value):
        if not isinstance(key, tuple):
            key = (key,)
        if len(key) == 1 and isinstance(key[0], _Indexable) and key[0].dtype == A.BOOL:
            # NArray#[]=(mask, value) (n_array.cr:510-551)
            if key[0].shape != self._shape:
                raise DimensionError("Cannot perform masking: mask shape does not match array shape.")
            return _masked_write(self, key[0], value)
        self.set_chunk(*key, value)

    def set_element(self, coord, value):
        from .region import canonicalize_index

        coord = [canonicalize_index(c, n) for c, n in zip(coord, self._shape)]
        if len(coord) != self.dimensions:
            raise DimensionError("coordinate rank mismatch")
        reg = IndexRegion.new(coord, self._shape, drop=False)
        _write_region(self, reg, value)

    def set_mask(self, mask, value):
        """MultiWritable#set_mask (multi_writable.cr:155-172): writes value (a
        scalar or a same-shaped MultiIndexable) where mask is true."""
        if isinstance(value, _Indexable) and value.shape != self._shape:
            raise ShapeError("Cannot perform masking: source shape %r does not match array shape %r."
                             % (value.shape, self._shape))
        if mask.shape != self._shape:
            raise ShapeError("Cannot perform masking: mask shape %r does not match array shape %r."
                             % (mask.shape, self._shape))
        _masked_write(self, mask, value)

    def mutable_view(self, *region):
        """MultiIndexable::Mutable#mutable_view (mutable.cr:6-12)."""
        v = CuMutableView(self, self._buf, self.dtype, 0, list(self._shape), _row_major(self._shape))
        lits = normalise_literal(region)
        return v._restrict(lits) if lits else v



# Above this many elements, an overlapping write is classified by the
# address-order rule only (the exact check walks every element on the host).
_ALIAS_EXACT_LIMIT = 1 << 22


def _lex_addresses(off, shape, stride):
    """Element offsets of an affine view in lexicographic order (int64)."""
    a = np.full([1], off, dtype=np.int64)
    for n, st in zip(shape, stride):
        a = (a[:, None] + np.arange(n, dtype=np.int64)[None, :] * st).reshape(-1)
    return a


def _sequential_order_differs(dst, src):
    """Whether writing `src` into `dst` element by element in lexicographic
    order (MultiWritable#unsafe_set_chunk, multi_writable.cr:29-44; Mutable#map_with!,
    mutable.cr:54-67) can give other results than reading every source
    element first, which is what the device does (it stages an overlapping
    source).  dst and src are (buffer, offset, shape, stride) of one element
    size with equal element counts.  They differ when some element is read at
    step i after a step j < i changed it: S(i) = D(j) with S(j) != D(j) (a
    step that reads and writes the same element changes nothing; a
    destination that writes an element twice is always refused).  Above
    _ALIAS_EXACT_LIMIT elements the answer is conservative: False only when
    the destination is walked in increasing address order and every read
    stays at or ahead of the write of its step."""
    dbuf, doff, dshape, dstride = dst
    sbuf, soff, sshape, sstride = src
    if dbuf is None or sbuf is None or dbuf.ptr != sbuf.ptr:
        return False
    dsh = [(n, st) for n, st in zip(dshape, dstride) if n != 1]
    ssh = [(n, st) for n, st in zip(sshape, sstride) if n != 1]
    n = shape_to_size(list(dshape))
    if n == 0:
        return False
    if doff == soff and dsh == ssh:
        return False  # the same mapping: each step reads the element it writes
    lo_d = doff + sum(min(0, (k - 1) * st) for k, st in dsh)
    hi_d = doff + sum(max(0, (k - 1) * st) for k, st in dsh)
    lo_s = soff + sum(min(0, (k - 1) * st) for k, st in ssh)
    hi_s = soff + sum(max(0, (k - 1) * st) for k, st in ssh)
    if hi_s < lo_d or hi_d < lo_s:
        return False  # disjoint
    if n <= _ALIAS_EXACT_LIMIT:
        d = _lex_addresses(doff, [x[0] for x in dsh], [x[1] for x in dsh])
        s_ = _lex_addresses(soff, [x[0] for x in ssh], [x[1] for x in ssh])
        order = np.argsort(d, kind="stable")
        ds = d[order]
        if ds.size > 1 and np.any(ds[1:] == ds[:-1]):
            return True  # the destination writes some element twice
        pos = np.minimum(np.searchsorted(ds, s_), ds.size - 1)
        hit = ds[pos] == s_
        j = order[pos]
        changed = s_[j] != d[j]
        return bool(np.any(hit & (j < np.arange(n)) & changed))
    # large views: a destination walked in increasing address order (positive
    # strides, each larger than the span of the axes inside it) whose every
    # read S(i) is at or past D(i) never reads an element already written
    monotone = all(st > 0 for _, st in dsh)
    inner = 0
    for k, st in reversed(dsh):
        monotone = monotone and st > inner
        inner += (k - 1) * st
    if not monotone or [x[0] for x in dsh] != [x[0] for x in ssh]:
        return True
    gap = soff - doff + sum(min(0, (k - 1) * (ss - ds)) for (k, ds), (_, ss) in zip(dsh, ssh))
    return gap < 0


def _refuse_reordered_alias(dst, src, what):
    if _sequential_order_differs(dst, src):
        raise NotImplementedError(
            "%s: the source overlaps the destination in another element order, so the reference's "
            "element-by-element write would read elements it has already written, while the device reads "
            "the whole source first; write a copy of the source (clone) instead" % what)


def _write_region(target, region, src):
    """unsafe_set_chunk (n_array.cr:484-500; multi_writable.cr:29-44) with a
    device source (gather/scatter kernel) or a scalar (fill kernel)."""
    buf, off, shape, stride = target._desc()
    o, s, st = _affine_region(off, shape, stride, region)
    if isinstance(src, CuProcView):
        # the reference reads the ProcView's operands element by element while
        # it writes: an operand aliasing the region in another order is refused
        for leaf in src._leaves:
            if not isinstance(leaf, CuIndexView):
                _refuse_reordered_alias((buf, o, s, st), leaf._desc(), "set_chunk")
        src = src.to_cu()
    dview = _make_view(buf, target.dtype, o, s, st)
    if isinstance(src, _Indexable):
        if not compatible_shapes(src.shape, region.shape):
            raise ShapeError("Cannot substitute %s: the given %s has shape %r, but region %r has shape %r."
                             % (type(src).__name__, type(src).__name__, src.shape, region, region.shape))
        if src.dtype != target.dtype:
            src = src.to_cu()._astype(target.dtype)
        _refuse_reordered_alias((buf, o, s, st), src._desc(), "set_chunk")
        _copy_into(dview, src._cview())
    else:
        sv = A.Scalar()
        sv.dtype = target.dtype
        v = _cast_scalar(src, target.dtype)
        if _is_float(target.dtype):
            sv.v.f = float(v)
        else:
            sv.v.i = int(v)
        A.check(lib().phcu_fill(ctypes.byref(dview), ctypes.byref(sv)), "phcu_fill")


def _astype(self, t):
    if t == self.dtype:
        return self
    out = CuNArray.empty(self._shape, t)
    pv = CuProcView._leaf(self)
    pv._expr = ("cvt", t, pv._expr)
    pv.dtype = t
    pv._eval_into(out._view(), t)
    return out


CuNArray._astype = _astype


# ================================================================== CuView
class CuView(_Indexable):
    """Lazy aliasing view over a device buffer (src/view.cr): the transform
    chain is folded into one affine map (offset, shape, stride)."""

    def __init__(self, src, buf, dtype, offset, shape, stride):
        self._src = src
        self._buf = buf
        self.dtype = dtype
        self._off = int(offset)
        self._shape = [int(x) for x in shape]
        self._stride = [int(x) for x in stride]

    def _desc(self):
        return self._buf, self._off, list(self._shape), list(self._stride)

    def _base(self):
        return self._src

    def _new(self, off, shape, stride):
        return type(self)(self._src, self._buf, self.dtype, off, shape, stride)

    def clone(self):
        return self._new(self._off, self._shape, self._stride)

    def _restrict(self, lits):
        """View#restrict_to (view.cr:43-56) with a literal or an IndexRegion."""
        if len(lits) == 1 and isinstance(lits[0], IndexRegion):
            region = lits[0]
        else:
            region = IndexRegion.new(lits, self._shape)
        o, s, st = _affine_region(self._off, self._shape, self._stride, region)
        return self._new(o, s, st)

    def view(self, *region):
        """View#view (view.cr:36-40): a new view composed with `region`."""
        lits = normalise_literal(region)
        v = CuView(self._src, self._buf, self.dtype, self._off, self._shape, self._stride)
        return v._restrict(lits) if lits else v

    def _unsafe_fetch_chunk(self, region):
        """View#unsafe_fetch_chunk (view.cr:105-107): another view, no copy."""
        o, s, st = _affine_region(self._off, self._shape, self._stride, region)
        return CuView(self._src, self._buf, self.dtype, o, s, st)

    def permute(self, *order):
        """View#permute (view.cr:72-89); no argument reverses the axis order."""
        order = normalise_literal(order)
        if not order:
            order = list(range(self.dimensions - 1, -1, -1))
        bad = [a for a in order if a < 0 or a >= self.dimensions]
        if bad:
            raise IndexError("Could not use pattern %r to permute: Axis %d is not present in a %d-dimensional "
                             "MultiIndexable" % (order, bad[0], self.dimensions))
        return self._new(*_affine_permute(self._off, self._shape, self._stride, order))

    def reverse(self):
        """View#reverse (view.cr:96-103): every axis reversed."""
        return self._new(*_affine_reverse(self._off, self._shape, self._stride))

    def reshape(self, *new_shape):
        """View#reshape (view.cr:58-70)."""
        new_shape = [int(x) for x in normalise_literal(new_shape)]
        if shape_to_size(new_shape) != self.size:
            raise ShapeError("Cannot change shape from %s (%d elements) to %s (%d elements) because reshape cannot "
                             "add or remove elements." % ("x".join(map(str, self._shape)), self.size,
                                                          "x".join(map(str, new_shape)), shape_to_size(new_shape)))
        r = _affine_reshape(self._off, self._shape, self._stride, new_shape)
        if r is not None:
            return self._new(*r)
        if isinstance(self, CuMutableView):
            raise NotImplementedError("a writable reshape of this strided view is not affine")
        # the layout cannot express the new shape: materialise (reads now, not lazily)
        mat = self.to_cu().reshape(new_shape)
        return CuView(mat, mat._buf, self.dtype, 0, new_shape, _row_major(new_shape))

    def to_narr(self):
        return self.to_cu().to_narr()


def _masked_write(self, mask, value):
    """One in-place select kernel over a writable target (an array or a
    mutable view): self = mask ? value : self.  Program: S0 = IN0 (the mask);
    ACC = IN2 (self); ACC = S0 ? B : ACC with B the source view IN1 or an
    immediate."""
    if isinstance(value, CuProcView):
        value = value.to_cu()
    src = value._cview() if isinstance(value, _Indexable) else None
    if src is not None and value.dtype != self.dtype:
        raise TypeError("masked write of a %s source into a %s array" % (np_dtype(value.dtype), np_dtype(self.dtype)))
    me = self._cview()
    ins = (A.View * 3)()
    ins[0] = mask._cview()
    ins[1] = src if src is not None else me
    ins[2] = me
    P = A.Program()
    P.n_instr = 4
    P.out_type = self.dtype
    code = [(A.I_LD, 0, A.BOOL, A.BOOL, 0), (A.I_ST0, 0, A.BOOL, 0, 0), (A.I_LD, 2, self.dtype, self.dtype, 0),
            (A.I_SEL, 1, self.dtype, self.dtype, 0) if src is not None else
            (A.I_SEL, A.SRC_IMM, self.dtype, self.dtype, _slot_bits(_cast_scalar(value, self.dtype), self.dtype))]
    for i, (op, sr, t, bt, imm) in enumerate(code):
        c = P.code[i]
        c.op, c.src, c.type, c.btype, c.flags = op, sr, t, bt, 0
        c.imm.i = int(imm) if imm < 2 ** 63 else int(imm) - 2 ** 64
    A.check(lib().phcu_eval(ctypes.byref(P), ins, 3, ctypes.byref(me)), "phcu_eval")


class CuMutableView(CuView):
    """Writable view (src/mutable_view.cr): writes land in the source buffer."""

    def view(self, *region):
        """MutableView#view (mutable_view.cr:20-24) returns a read-only view."""
        v = CuView(self._src, self._buf, self.dtype, self._off, self._shape, self._stride)
        lits = normalise_literal(region)
        return v._restrict(lits) if lits else v

    def mutable_view(self, *region):
        lits = normalise_literal(region)
        v = self.clone()
        return v._restrict(lits) if lits else v

    def set_chunk(self, *args):
        *lits, src = args
        lits = normalise_literal(lits)
        if len(lits) == 1 and isinstance(lits[0], IndexRegion):
            region = lits[0]
        else:
            region = IndexRegion.new(lits, self._shape)
        _write_region(self, region, src)

    def __setitem__(self, key, value):
        if not isinstance(key, tuple):
            key = (key,)
        if len(key) == 1 and isinstance(key[0], _Indexable) and key[0].dtype == A.BOOL:
            return self.set_mask(key[0], value)  # MultiWritable#[]=(mask, value) (multi_writable.cr:127-129)
        self.set_chunk(*key, value)

    set_mask = CuNArray.set_mask


class CuIndexView(CuView):
    """An index operand: a read-only Int32 "array" whose element at coordinate
    c is offset + sum c_i * stride_i, computed on the device (PHCU_INDEX) and
    never stored.  CuIndexView.lex(shape) holds every element's lexicographic
    index, CuIndexView.axis(shape, d) its coordinate along axis d.  Views of it
    (regions, permutations, reversals) fold into the affine map like any view,
    so an index keeps naming the element it was computed for."""

    def __init__(self, offset, shape, stride):
        super().__init__(None, None, A.I32, offset, shape, stride)

    @classmethod
    def lex(cls, shape):
        return cls(0, list(shape), _row_major(list(shape)))

    @classmethod
    def axis(cls, shape, d):
        return cls(0, list(shape), [1 if i == d else 0 for i in range(len(shape))])

    def _new(self, off, shape, stride):
        return CuIndexView(off, shape, stride)

    def _as_leaf(self):
        return self.clone()

    def _cview(self):
        return _make_view(None, A.INDEX, self._off, self._shape, self._stride)

    def view(self, *region):
        lits = normalise_literal(region)
        v = self.clone()
        return v._restrict(lits) if lits else v

    def _unsafe_fetch_chunk(self, region):
        return self._new(*_affine_region(self._off, self._shape, self._stride, region))

    def reshape(self, *new_shape):
        new_shape = [int(x) for x in normalise_literal(new_shape)]
        r = _affine_reshape(self._off, self._shape, self._stride, new_shape)
        if r is None or shape_to_size(new_shape) != self.size:
            return self.to_cu().reshape(new_shape)
        return self._new(*r)

    def to_cu(self):
        return CuProcView._leaf(self).to_cu()


# ============================================================= CuProcView
class _Sym:
    """Symbolic element handed to process() blocks."""

    __slots__ = ("expr", "dtype")

    def __init__(self, expr, dtype):
        self.expr, self.dtype = expr, dtype

    def _bin(self, op, other, reflected=False):
        if isinstance(other, _Sym):
            oe, ot = other.expr, other.dtype
        else:
            ot = scalar_dtype(other)
            oe = ("const", other, ot)
        a, ta, b, tb = (oe, ot, self.expr, self.dtype) if reflected else (self.expr, self.dtype, oe, ot)
        t = result_dtype(op, ta, tb)
        return _Sym(("bin", op, a, b, ta, tb, t), t)

    def __add__(self, o): return self._bin(A.OP_ADD, o)
    def __radd__(self, o): return self._bin(A.OP_ADD, o, True)
    def __sub__(self, o): return self._bin(A.OP_SUB, o)
    def __rsub__(self, o): return self._bin(A.OP_SUB, o, True)
    def __mul__(self, o): return self._bin(A.OP_MUL, o)
    def __rmul__(self, o): return self._bin(A.OP_MUL, o, True)
    def __truediv__(self, o): return self._bin(A.OP_DIV, o)
    def __rtruediv__(self, o): return self._bin(A.OP_DIV, o, True)
    def __floordiv__(self, o): return self._bin(A.OP_FLOORDIV, o)
    def __mod__(self, o): return self._bin(A.OP_MOD, o)
    def __pow__(self, o): return self._bin(A.OP_POW, o)
    def __and__(self, o): return self._bin(A.OP_AND, o)
    def __or__(self, o): return self._bin(A.OP_OR, o)
    def __xor__(self, o): return self._bin(A.OP_XOR, o)
    def __gt__(self, o): return self._bin(A.OP_GT, o)
    def __lt__(self, o): return self._bin(A.OP_LT, o)
    def __ge__(self, o): return self._bin(A.OP_GE, o)
    def __le__(self, o): return self._bin(A.OP_LE, o)

    def __neg__(self):
        return _Sym(("un", A.I_NEG, self.expr, self.dtype), self.dtype)


class CuProcView(_Indexable):
    """Lazy elementwise program over up to four aliasing operand views
    (src/proc_view.cr).  process() composes blocks (proc_view.cr:32-35); infix
    operators with views, arrays or scalars extend the program; the whole chain
    runs as ONE kernel when it is materialised (to_cu / to_narr / a reduction)."""

    def __init__(self, leaves, expr, dtype, shape):
        self._leaves = leaves  # list of CuView
        self._expr = expr
        self.dtype = dtype
        self._shape = list(shape)

    @classmethod
    def _leaf(cls, x):
        if isinstance(x, CuProcView):
            return x
        return cls([x._as_leaf()], ("in", 0, x.dtype), x.dtype, x.shape)

    @classmethod
    def _of_result(cls, leaves, out, shape):
        """The program whose result is `out` (a symbol, or a constant the block
        returned), keeping only the leaves it reads."""
        if isinstance(out, _Sym):
            pv = cls(leaves, out.expr, out.dtype, shape)
        else:
            t = scalar_dtype(out)
            pv = cls(leaves, ("const", out, t), t, shape)
        return pv._prune()._dedupe()

    def _prune(self):
        used = sorted(_leaf_ids(self._expr))
        remap = {old: new for new, old in enumerate(used)}
        self._expr = _remap(self._expr, remap)
        self._leaves = [self._leaves[i] for i in used]
        return self

    def _desc(self):
        raise NotImplementedError("a CuProcView has no storage; materialise it with to_cu()")

    def _cview(self):
        # a temporary CuNArray would be freed (stream-ordered) before its use
        raise NotImplementedError("materialise a CuProcView with to_cu() before passing it to a kernel")

    def _fetch_element(self, coord):
        return self.to_cu()._fetch_element(coord)

    def process(self, fn):
        sym = fn(_Sym(self._expr, self.dtype))
        if not isinstance(sym, _Sym):
            # constant block: broadcast the constant
            t = scalar_dtype(sym)
            return CuProcView(self._leaves, ("const", sym, t), t, self._shape)
        return CuProcView(self._leaves, sym.expr, sym.dtype, self._shape)

    # elementwise programs commute with index transforms: apply to every leaf
    def _map_leaves(self, f):
        leaves = [f(l) for l in self._leaves]
        shape = leaves[0].shape if leaves else self._shape
        return CuProcView(leaves, self._expr, self.dtype, shape)

    def view(self, *region):
        lits = normalise_literal(region)
        return self._map_leaves(lambda l: l.view(*lits))

    def permute(self, *order):
        return self._map_leaves(lambda l: l.permute(*order))

    def reverse(self):
        return self._map_leaves(lambda l: l.reverse())

    def _unsafe_fetch_chunk(self, region):
        return self._map_leaves(lambda l: l._unsafe_fetch_chunk(region))

    def _binary(self, op, other, reflected=False):
        leaves = list(self._leaves)
        if isinstance(other, CuProcView):
            if other._shape != self._shape:
                raise ShapeError("The shape of this MultiIndexable (%r) does not match the shape of the one provided "
                                 "(%r), so '%s' cannot be applied element-wise." % (self._shape, other._shape,
                                                                                     _OP_NAMES.get(op)))
            base = len(leaves)
            leaves += other._leaves
            oe = _shift(other._expr, base)
            ot = other.dtype
        elif isinstance(other, _Indexable):
            if other.shape != self._shape:
                raise ShapeError("The shape of this MultiIndexable (%r) does not match the shape of the one provided "
                                 "(%r), so '%s' cannot be applied element-wise." % (self._shape, other.shape,
                                                                                     _OP_NAMES.get(op)))
            leaves.append(other._as_leaf())
            oe = ("in", len(leaves) - 1, other.dtype)
            ot = other.dtype
        else:
            ot = scalar_dtype(other)
            oe = ("const", other, ot)
        a, ta, b, tb = (oe, ot, self._expr, self.dtype) if reflected else (self._expr, self.dtype, oe, ot)
        t = result_dtype(op, ta, tb)
        pv = CuProcView(leaves, ("bin", op, a, b, ta, tb, t), t, self._shape)
        return pv._dedupe()

    def _dedupe(self):
        # identical leaf views share one input slot
        keys, remap, leaves = {}, {}, []
        for i, l in enumerate(self._leaves):
            k = ("index" if isinstance(l, CuIndexView) else l._buf.ptr if l._buf else 0, l.dtype, l._off,
                 tuple(l._shape), tuple(l._stride))
            if k not in keys:
                keys[k] = len(leaves)
                leaves.append(l)
            remap[i] = keys[k]
        self._expr = _remap(self._expr, remap)
        self._leaves = leaves
        return self

    def _unary(self, uop):
        op = {A.UOP_NEG: A.I_NEG, A.UOP_NOT: A.I_NOT, A.UOP_POS: A.I_POS}[uop]
        return CuProcView(self._leaves, ("un", op, self._expr, self.dtype), self.dtype, self._shape)

    # ------------------------------------------------------------- evaluate
    def _eval_into(self, out_view, out_dtype):
        """Runs the program into out_view.  An expression the device program
        cannot hold in one piece (more than MAX_INPUTS distinct views, more
        than MAX_INSTR instructions, or nesting deeper than the two stash
        registers) is split: its largest sub-expression that fits is
        materialised into a temporary array of its own type, which becomes a
        leaf, until the rest fits (ProcView composes without limit,
        proc_view.cr:32-35).  Every operation still runs once per element in
        its own type, so the results are those of the unsplit expression."""
        expr, leaves, temps, can_raise = _split_to_fit(self._expr, list(self._leaves), self._shape, out_dtype)
        prog, raises = compile_program(expr, out_dtype)
        ins = (A.View * max(1, len(leaves)))()
        for k, l in enumerate(leaves):
            ins[k] = l._cview()
        A.check(lib().phcu_eval(ctypes.byref(prog), ins, len(leaves), ctypes.byref(out_view)), "phcu_eval")
        del temps  # freed stream-ordered, after the launch that reads them
        if (can_raise or raises) and config.eager_errors:
            check_errors()

    def to_cu(self):
        out = CuNArray.empty(self._shape, self.dtype)
        self._eval_into(out._view(), self.dtype)
        return out

    def to_narr(self):
        return self.to_cu().to_narr()

    def _reduce(self, op, axis, out_dtype=None):
        return self.to_cu()._reduce(op, axis, out_dtype)


def _shift(e, base):
    k = e[0]
    if k == "in":
        return ("in", e[1] + base, e[2])
    if k == "const":
        return e
    if k == "bin":
        return ("bin", e[1], _shift(e[2], base), _shift(e[3], base)) + tuple(e[4:])
    if k == "un":
        return ("un", e[1], _shift(e[2], base), e[3])
    if k == "cvt":
        return ("cvt", e[1], _shift(e[2], base))
    return e


def _fits(expr, nleaves, out_dtype):
    if nleaves > A.MAX_INPUTS:
        return False
    try:
        compile_program(expr, out_dtype)
    except NotImplementedError:
        return False
    return True


def _subtrees(e, acc):
    """Every operator node below the root (with repeats)."""
    k = e[0]
    if k == "bin":
        for c in (e[2], e[3]):
            if c[0] in ("bin", "un", "cvt"):
                acc.append(c)
            _subtrees(c, acc)
    elif k in ("un", "cvt"):
        c = e[2]
        if c[0] in ("bin", "un", "cvt"):
            acc.append(c)
        _subtrees(c, acc)
    return acc


def _size(e):
    k = e[0]
    if k == "bin":
        return 1 + _size(e[2]) + _size(e[3])
    if k in ("un", "cvt"):
        return 1 + _size(e[2])
    return 0


def _replace(e, old, new):
    if e == old:
        return new
    k = e[0]
    if k == "bin":
        return ("bin", e[1], _replace(e[2], old, new), _replace(e[3], old, new)) + tuple(e[4:])
    if k == "un":
        return ("un", e[1], _replace(e[2], old, new), e[3])
    if k == "cvt":
        return ("cvt", e[1], _replace(e[2], old, new))
    return e


def _split_to_fit(expr, leaves, shape, out_dtype):
    """Materialises sub-expressions of `expr` until it fits one device program.
    Returns (expr, leaves, temporaries, can_raise)."""
    temps = []
    can_raise = False
    while not _fits(expr, len(_leaf_ids(expr)), out_dtype):
        best = None
        for sub in _subtrees(expr, []):
            ids = _leaf_ids(sub)
            if _fits(sub, len(ids), _etype(sub)) and (best is None or _size(sub) > _size(best)):
                best = sub
        if best is None:  # cannot happen: an operator over two leaves always fits
            raise NotImplementedError("expression cannot be split into device programs")
        piece = CuProcView(leaves, best, _etype(best), shape)._prune()
        tmp = CuNArray.empty(shape, piece.dtype)
        prog, raises = compile_program(piece._expr, piece.dtype)
        can_raise = can_raise or raises
        ins = (A.View * max(1, len(piece._leaves)))()
        for k, l in enumerate(piece._leaves):
            ins[k] = l._cview()
        A.check(lib().phcu_eval(ctypes.byref(prog), ins, len(piece._leaves), ctypes.byref(tmp._view())),
                "phcu_eval")
        temps.append(tmp)
        leaves = leaves + [tmp._as_leaf()]
        expr = _replace(expr, best, ("in", len(leaves) - 1, piece.dtype))
        used = sorted(_leaf_ids(expr))
        remap = {old: new for new, old in enumerate(used)}
        expr = _remap(expr, remap)
        leaves = [leaves[i] for i in used]
    return expr, leaves, temps, can_raise


def _leaf_ids(e, acc=None):
    acc = set() if acc is None else acc
    k = e[0]
    if k == "in":
        acc.add(e[1])
    elif k == "bin":
        _leaf_ids(e[2], acc)
        _leaf_ids(e[3], acc)
    elif k in ("un", "cvt"):
        _leaf_ids(e[2], acc)
    return acc


def _remap(e, m):
    k = e[0]
    if k == "in":
        return ("in", m[e[1]], e[2])
    if k == "bin":
        return ("bin", e[1], _remap(e[2], m), _remap(e[3], m)) + tuple(e[4:])
    if k == "un":
        return ("un", e[1], _remap(e[2], m), e[3])
    if k == "cvt":
        return ("cvt", e[1], _remap(e[2], m))
    return e


def _etype(e):
    k = e[0]
    if k == "in":
        return e[2]
    if k == "const":
        return e[2]
    if k == "bin":
        return e[6]
    if k == "un":
        return e[3]
    if k == "cvt":
        return e[1]
    raise ValueError(e)


# ------------------------------------------------------- program compiler
def compile_program(expr, out_dtype):
    """Compiles an expression tree into the library's accumulator program.
    Returns (Program, can_raise)."""
    code = []
    flags = {"raise": False}

    def emit(op, src=0, t=0, bt=0, imm=0, fl=0):
        if len(code) >= A.MAX_INSTR:
            raise NotImplementedError("fused program longer than %d instructions" % A.MAX_INSTR)
        code.append((op, src, t, bt, imm, fl))

    def simple(e):
        return e[0] in ("in", "const")

    def src_of(e):
        if e[0] == "in":
            return e[1], e[2], 0
        return A.SRC_IMM, e[2], _slot_bits(e[1], e[2])

    def gen(e, depth):
        k = e[0]
        if k in ("in", "const"):
            s, t, imm = src_of(e)
            emit(A.I_LD, s, t, t, imm)
            return
        if k == "cvt":
            gen(e[2], depth)
            emit(A.I_CVT, 0, _etype(e[2]), 0, e[1])
            return
        if k == "un":
            gen(e[2], depth)
            if e[1] == A.I_NEG and _is_int(e[3]):
                flags["raise"] = True
            emit(e[1], 0, e[3])
            return
        _, op, l, r, ta, tb, tout = e
        T = _compute_type(op, ta, tb)
        int_exp = op == A.OP_POW and _is_float(ta) and _is_int(tb)
        if _can_raise(op, ta, tb):
            flags["raise"] = True
        if ta == A.BOOL and tb != A.BOOL or tb == A.BOOL and ta != A.BOOL:
            emit(A.I_LD, A.SRC_IMM, A.BOOL, A.BOOL, 0)  # Bool == number: false
            return
        if simple(r):
            gen(l, depth)
            if ta != T:
                emit(A.I_CVT, 0, ta, 0, T)
            s, st, imm = src_of(r)
            emit(op, s, T, st, imm)
        elif simple(l) and not int_exp and op != A.OP_POW:
            gen(r, depth)
            if tb != T:
                emit(A.I_CVT, 0, tb, 0, T)
            s, st, imm = src_of(l)
            emit(op, s, T, st, imm, 1)
        else:
            if depth >= 2:
                raise NotImplementedError("expression too deep for the two stash registers")
            gen(r, depth)
            emit(A.I_ST0 if depth == 0 else A.I_ST1, 0, tb)
            gen(l, depth + 1)
            if ta != T:
                emit(A.I_CVT, 0, ta, 0, T)
            emit(op, A.SRC_S0 if depth == 0 else A.SRC_S1, T, tb, 0)
        rt = T
        if op in (A.OP_GT, A.OP_LT, A.OP_GE, A.OP_LE, A.OP_EQ):
            rt = A.BOOL
        elif op == A.OP_CMP:
            rt = A.I32
        elif op == A.OP_DIV and _is_int(T):
            rt = A.F64
        if rt != tout:
            emit(A.I_CVT, 0, rt, 0, tout)

    gen(expr, 0)
    et = _etype(expr)
    if et != out_dtype:
        emit(A.I_CVT, 0, et, 0, out_dtype)
    P = A.Program()
    P.n_instr = len(code)
    P.out_type = out_dtype
    for i, (op, src, t, bt, imm, fl) in enumerate(code):
        c = P.code[i]
        c.op, c.src, c.type, c.btype, c.flags = op, src, t, bt, fl
        c.imm.i = int(imm) if imm < 2 ** 63 else int(imm) - 2 ** 64
    return P, flags["raise"]
