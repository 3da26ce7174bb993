"""ctypes wrapper of liboracle.so -- TEST INFRASTRUCTURE ONLY.

The CPU restatement of the reference semantics (phase_oracle.c) is the checker
for the CUDA path and the timed CPU baseline.  Only tests/, the smoke test
and bench.py's CPU-baseline / reference legs import this module; the product
(libphcuda.so and the phase_cu package) never does.

View operands are described abstractly, in the reference's own vocabulary,
as a base array plus the transforms applied to it oldest first:
    ("region", [literal...])   View#view / restrict_to  (view.cr:43-56)
    ("permute", [order] | None) View#permute!           (view.cr:72-81)
    ("reverse",)               View#reverse!            (view.cr:96-99)
    ("reshape", [shape])       View#reshape!            (view.cr:58-66)
Literals are ints, Python slices, or any object with first/last/step/exclusive
attributes (Crystal ranges).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
MAXR = 8
MAXTF = 16

BOOL, I32, I64, F32, F64 = 0, 1, 2, 3, 4
NP = {BOOL: np.bool_, I32: np.int32, I64: np.int64, F32: np.float32, F64: np.float64}
FROM_NP = {np.dtype(v): k for k, v in NP.items()}

OK, ERR_SHAPE, ERR_DIM, ERR_INDEX, ERR_OVERFLOW, ERR_DIVZERO, ERR_ARGUMENT, ERR_UNBOUNDED, ERR_EMPTY, \
    ERR_UNSUPPORTED = range(10)
ST_OVERFLOW, ST_DIVZERO, ST_ARGUMENT = 1, 2, 4
(OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_FLOORDIV, OP_MOD, OP_POW, OP_WADD, OP_WSUB, OP_WMUL, OP_WPOW,
 OP_AND, OP_OR, OP_XOR, OP_GT, OP_LT, OP_GE, OP_LE, OP_CMP, OP_EQ) = range(20)
UOP_POS, UOP_NEG, UOP_NOT = 0, 1, 2
RED_SUM, RED_MAX, RED_MIN, RED_ARGMAX, RED_ARGMIN = range(5)
TF_REGION, TF_PERMUTE, TF_REVERSE, TF_RESHAPE = range(4)


class Lit(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("has_first", ctypes.c_int32), ("has_last", ctypes.c_int32),
                ("has_step", ctypes.c_int32), ("exclusive", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("first", ctypes.c_int64), ("last", ctypes.c_int64), ("step", ctypes.c_int64)]


class Range(ctypes.Structure):
    _fields_ = [("first", ctypes.c_int64), ("step", ctypes.c_int64), ("last", ctypes.c_int64),
                ("size", ctypes.c_int64)]


class Region(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_int32), ("drop", ctypes.c_int32), ("reduced_rank", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("first", ctypes.c_int64 * MAXR), ("step", ctypes.c_int64 * MAXR),
                ("last", ctypes.c_int64 * MAXR), ("shape", ctypes.c_int64 * MAXR),
                ("degeneracy", ctypes.c_int32 * MAXR), ("reduced_shape", ctypes.c_int64 * MAXR)]

    def as_dict(self):
        n = self.rank
        return {"first": list(self.first[:n]), "step": list(self.step[:n]), "last": list(self.last[:n]),
                "proper_shape": list(self.shape[:n]), "degeneracy": [bool(x) for x in self.degeneracy[:n]],
                "shape": list(self.reduced_shape[:self.reduced_rank]), "drop": bool(self.drop)}


class Xf(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("in_rank", ctypes.c_int32), ("out_rank", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("region", Region), ("pattern", ctypes.c_int32 * MAXR),
                ("shape", ctypes.c_int64 * MAXR), ("new_shape", ctypes.c_int64 * MAXR)]


class Operand(ctypes.Structure):
    _fields_ = [("buf", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("base_rank", ctypes.c_int32),
                ("base_shape", ctypes.c_int64 * MAXR), ("ntf", ctypes.c_int32), ("rank", ctypes.c_int32),
                ("shape", ctypes.c_int64 * MAXR), ("tf", Xf * MAXTF)]


_lib = None


def build():
    """Compiles liboracle.so with its Makefile (gcc, -ffp-contract=off)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_P = ctypes.POINTER
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_I64A = _P(ctypes.c_int64)


def _sigs():
    return {
        "ora_get_size": [_i64, _i64, _i64, _I64A],
        "ora_infer_range": [_P(Lit), _i64, _P(Range)],
        "ora_canonicalize_range": [_P(Lit), _i64, _P(Range)],
        "ora_canonicalize_index": [_i64, _i64, _I64A],
        "ora_compatible_shapes": [_I64A, _i32, _I64A, _i32],
        "ora_region_new": [_P(Lit), _i32, _I64A, _i32, _i32, _P(Region)],
        "ora_region_new_absolute": [_P(Lit), _i32, _i32, _P(Region)],
        "ora_region_new_trim": [_P(Lit), _i32, _I64A, _I64A, _i32, _i32, _P(Region)],
        "ora_region_cover": [_I64A, _i32, _P(Region)],
        "ora_region_trim": [_P(Region), _I64A, _i32],
        "ora_region_fits_in": [_P(Region), _I64A, _i32, _P(_i32)],
        "ora_region_reverse": [_P(Region)],
        "ora_region_translate": [_P(Region), _I64A, _i32],
        "ora_region_includes": [_P(Region), _I64A, _i32],
        "ora_region_local_to_absolute": [_P(Region), _I64A, _I64A],
        "ora_xf_apply": [_P(Xf), _I64A, _I64A],
        "ora_gather": [_P(Operand), _vp, _i32],
        "ora_gather_range": [_P(Operand), _vp, _i64, _i64, _i32],
        "ora_map_binary_range": [_i32, _P(Operand), _P(Operand), _vp, _i64, _i64, _P(ctypes.c_uint32), _i32],
        "ora_scatter_range": [_P(Operand), _P(Operand), _i64, _i64, _i32],
        "ora_narray_fetch_chunk": [_vp, _i32, _I64A, _i32, _P(Region), _vp, _i32],
        "ora_narray_set_chunk": [_vp, _i32, _I64A, _i32, _P(Region), _vp],
        "ora_narray_set_chunk_scalar": [_vp, _i32, _I64A, _i32, _P(Region), _vp],
        "ora_scatter": [_P(Operand), _P(Operand)],
        "ora_scatter_scalar": [_P(Operand), _vp],
        "ora_result_dtype": [_i32, _i32, _i32, _P(_i32)],
        "ora_map_binary": [_i32, _P(Operand), _P(Operand), _vp, _P(ctypes.c_uint32), _i32],
        "ora_map_binary_scalar": [_i32, _P(Operand), _vp, _i32, _i32, _vp, _P(ctypes.c_uint32), _i32],
        "ora_map_unary": [_i32, _P(Operand), _vp, _P(ctypes.c_uint32)],
        "ora_reduce": [_i32, _vp, _i32, _I64A, _i32, _i32, _vp, _i32],
        "ora_reduce_f64": [_vp, _i32, _I64A, _i32, _i32, _vp],
        "ora_heat_run_f32": [_vp, _vp, _i64, _i64, ctypes.c_float, _i32, _i32],
        "ora_heat_run_f64": [_vp, _vp, _i64, _i64, ctypes.c_double, _i32, _i32],
        "ora_mlp_forward_backward": [_vp, _i32, _i32, _i32, _vp, _vp, _i32, _P(ctypes.c_double), _vp],
    }


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        l = ctypes.CDLL(LIB)
        for name, args in _sigs().items():
            f = getattr(l, name)
            f.argtypes = args
            f.restype = ctypes.c_int32
        _lib = l
    return _lib


class OracleError(Exception):
    def __init__(self, code, what=""):
        super().__init__("oracle status %d %s" % (code, what))
        self.code = code


def _chk(rc, what=""):
    if rc != OK:
        raise OracleError(rc, what)


def _i64arr(xs):
    a = (ctypes.c_int64 * max(MAXR, len(xs)))()
    for i, x in enumerate(xs):
        a[i] = int(x)
    return a


# ------------------------------------------------------------------ literals
def lit(x):
    """Region literal element -> Lit (RangeSyntax.parse_range, range_syntax.cr:42-68)."""
    l = Lit()
    if isinstance(x, (int, np.integer)) and not isinstance(x, bool):
        l.kind = 0
        l.first = int(x)
        return l
    l.kind = 1
    if x is Ellipsis:
        return l
    if isinstance(x, slice):
        f, la, st, ex = x.start, x.stop, x.step, x.stop is not None
    else:
        f, la, st, ex = x.first, x.last, x.step, x.exclusive
    if f is not None:
        l.has_first, l.first = 1, int(f)
    if la is not None:
        l.has_last, l.last = 1, int(la)
    if st is not None:
        l.has_step, l.step = 1, int(st)
    l.exclusive = 1 if ex else 0
    return l


def _lits(xs):
    arr = (Lit * max(1, len(xs)))()
    for i, x in enumerate(xs):
        arr[i] = lit(x)
    return arr


def infer_range(x, bound):
    r = Range()
    _chk(lib().ora_infer_range(ctypes.byref(lit(x)), bound, ctypes.byref(r)), "infer_range")
    return (r.first, r.step, r.last, r.size)


def canonicalize_range(x, bound):
    r = Range()
    _chk(lib().ora_canonicalize_range(ctypes.byref(lit(x)), bound, ctypes.byref(r)),
         "canonicalize_range")
    return (r.first, r.step, r.last, r.size)


def get_size(first, last, step):
    s = ctypes.c_int64()
    _chk(lib().ora_get_size(first, last, step, ctypes.byref(s)))
    return s.value


def canonicalize_index(i, n):
    o = ctypes.c_int64()
    _chk(lib().ora_canonicalize_index(i, n, ctypes.byref(o)))
    return o.value


def compatible_shapes(a, b):
    return bool(lib().ora_compatible_shapes(_i64arr(a), len(a), _i64arr(b), len(b)))


def region_new(lits, bound, drop=True):
    r = Region()
    _chk(lib().ora_region_new(_lits(lits), len(lits), _i64arr(bound), len(bound), int(drop), ctypes.byref(r)),
         "region_new")
    return r


def region_absolute(lits, drop=True):
    r = Region()
    _chk(lib().ora_region_new_absolute(_lits(lits), len(lits), int(drop), ctypes.byref(r)), "region_absolute")
    return r


def region_trimmed(lits, trim_to, bound=None, drop=True):
    r = Region()
    b = _i64arr(bound) if bound is not None else None
    _chk(lib().ora_region_new_trim(_lits(lits), len(lits), b, _i64arr(trim_to), len(trim_to), int(drop),
                                   ctypes.byref(r)), "region_trimmed")
    return r


def region_cover(shape):
    r = Region()
    _chk(lib().ora_region_cover(_i64arr(shape), len(shape), ctypes.byref(r)))
    return r


def region_trim(r, bound):
    _chk(lib().ora_region_trim(ctypes.byref(r), _i64arr(bound), len(bound)), "trim")
    return r


def region_fits_in(r, bound):
    f = ctypes.c_int32()
    _chk(lib().ora_region_fits_in(ctypes.byref(r), _i64arr(bound), len(bound), ctypes.byref(f)), "fits_in")
    return bool(f.value)


def region_reverse(r):
    lib().ora_region_reverse(ctypes.byref(r))
    return r


def region_translate(r, offset):
    _chk(lib().ora_region_translate(ctypes.byref(r), _i64arr(offset), len(offset)), "translate")
    return r


def region_includes(r, coord):
    return bool(lib().ora_region_includes(ctypes.byref(r), _i64arr(coord), len(coord)))


def region_local_to_absolute(r, local):
    out = (ctypes.c_int64 * MAXR)()
    lib().ora_region_local_to_absolute(ctypes.byref(r), _i64arr(local), out)
    return list(out[:r.rank])


def xf_apply(kind, in_coord, **kw):
    """Applies one transform to one coordinate (transform KATs)."""
    t = Xf()
    t.kind = kind
    t.in_rank = len(in_coord)
    if kind == TF_PERMUTE:
        for i, p in enumerate(kw["pattern"]):
            t.pattern[i] = p
        t.out_rank = len(in_coord)
    elif kind == TF_REVERSE:
        t.shape = _i64arr(kw["shape"])
        t.out_rank = len(in_coord)
    elif kind == TF_RESHAPE:
        t.shape = _i64arr(kw["src_shape"])
        t.new_shape = _i64arr(kw["new_shape"])
        t.out_rank = len(kw["src_shape"])
    out = (ctypes.c_int64 * MAXR)()
    _chk(lib().ora_xf_apply(ctypes.byref(t), _i64arr(in_coord), out))
    return list(out[:t.out_rank])


# ------------------------------------------------------------------ operands
class ViewOperand:
    """Keeps the numpy buffer alive next to the C operand."""

    def __init__(self, arr, transforms=()):
        self.arr = np.ascontiguousarray(arr)
        op = Operand()
        op.buf = self.arr.ctypes.data
        op.dtype = FROM_NP[self.arr.dtype]
        op.base_rank = self.arr.ndim
        op.base_shape = _i64arr(self.arr.shape)
        shape = list(self.arr.shape)
        tfs = []
        for t in transforms:
            x = Xf()
            k = t[0]
            if k == "region":
                r = region_new(list(t[1]), shape, True)
                x.kind = TF_REGION
                x.region = r
                x.in_rank = r.reduced_rank
                x.out_rank = len(shape)
                shape = list(r.reduced_shape[:r.reduced_rank])
            elif k == "permute":
                order = list(t[1]) if len(t) > 1 and t[1] is not None else list(range(len(shape) - 1, -1, -1))
                if any(o < 0 or o >= len(shape) for o in order):
                    raise OracleError(ERR_INDEX, "permute")
                x.kind = TF_PERMUTE
                for i, p in enumerate(order):
                    x.pattern[i] = p
                x.in_rank = x.out_rank = len(shape)
                shape = [shape[p] for p in order]
            elif k == "reverse":
                x.kind = TF_REVERSE
                x.shape = _i64arr(shape)
                x.in_rank = x.out_rank = len(shape)
            elif k == "reshape":
                new = list(t[1])
                if int(np.prod(new)) != int(np.prod(shape)):
                    raise OracleError(ERR_SHAPE, "reshape")
                x.kind = TF_RESHAPE
                x.shape = _i64arr(shape)
                x.new_shape = _i64arr(new)
                x.in_rank = len(new)
                x.out_rank = len(shape)
                shape = new
            else:
                raise ValueError(k)
            tfs.append(x)
        # ComposedTransform#compose! unshifts: newest first (transforms.cr:46-48)
        for i, x in enumerate(reversed(tfs)):
            op.tf[i] = x
        op.ntf = len(tfs)
        op.rank = len(shape)
        op.shape = _i64arr(shape)
        self.shape = shape
        self.dtype = op.dtype
        self.op = op

    @property
    def size(self):
        return int(np.prod(self.shape)) if self.shape else 0


def gather(v, nthreads=1):
    """View#to_narr (view.cr:123-126)."""
    out = np.empty(v.shape, dtype=NP[v.dtype])
    _chk(lib().ora_gather(ctypes.byref(v.op), out.ctypes.data, nthreads), "gather")
    return out


def gather_range(v, out, lo, hi, nthreads=1):
    """Elements [lo, hi) of gather(v), written into `out` (a bounded sample of
    the full-size gather)."""
    _chk(lib().ora_gather_range(ctypes.byref(v.op), out.ctypes.data, lo, hi, nthreads), "gather_range")
    return out


def map_binary_range(op, a, b, out, lo, hi, nthreads=1):
    """Elements [lo, hi) of map_binary(op, a, b), written into `out`."""
    st = ctypes.c_uint32()
    _chk(lib().ora_map_binary_range(op, ctypes.byref(a.op), ctypes.byref(b.op), out.ctypes.data, lo, hi,
                                    ctypes.byref(st), nthreads), "map_binary_range")
    return out, st.value


def scatter_range(dst, src, lo, hi, nthreads=1):
    """Writes [lo, hi) of scatter(dst, src), for a source that does not alias dst."""
    _chk(lib().ora_scatter_range(ctypes.byref(dst.op), ctypes.byref(src.op), lo, hi, nthreads), "scatter_range")
    return dst.arr


def narray_fetch_chunk(arr, lits, drop=True, nthreads=1):
    """NArray#[] via IndexRegion + the buffer-index odometer (n_array.cr:450-453)."""
    arr = np.ascontiguousarray(arr)
    r = region_new(list(lits), list(arr.shape), drop)
    out = np.empty(list(r.reduced_shape[:r.reduced_rank]), dtype=arr.dtype)
    _chk(lib().ora_narray_fetch_chunk(arr.ctypes.data, FROM_NP[arr.dtype], _i64arr(arr.shape), arr.ndim,
                                      ctypes.byref(r), out.ctypes.data, nthreads), "fetch_chunk")
    return out


def narray_set_chunk(arr, lits, src):
    """NArray#[]= (n_array.cr:484-500); arr is modified in place."""
    r = region_new(list(lits), list(arr.shape), True)
    if np.isscalar(src) or (isinstance(src, np.ndarray) and src.ndim == 0):
        v = np.array(src, dtype=arr.dtype)
        _chk(lib().ora_narray_set_chunk_scalar(arr.ctypes.data, FROM_NP[arr.dtype], _i64arr(arr.shape), arr.ndim,
                                               ctypes.byref(r), v.ctypes.data), "set_chunk")
    else:
        s = np.ascontiguousarray(src, dtype=arr.dtype)
        if s.size != int(np.prod(r.reduced_shape[:r.reduced_rank])):
            raise OracleError(ERR_SHAPE, "set_chunk")
        _chk(lib().ora_narray_set_chunk(arr.ctypes.data, FROM_NP[arr.dtype], _i64arr(arr.shape), arr.ndim,
                                        ctypes.byref(r), s.ctypes.data), "set_chunk")
    return arr


def scatter(dst, src):
    """MultiWritable#unsafe_set_chunk through a MutableView (multi_writable.cr:29-36)."""
    _chk(lib().ora_scatter(ctypes.byref(dst.op), ctypes.byref(src.op)), "scatter")
    return dst.arr


def scatter_scalar(dst, value):
    v = np.array(value, dtype=NP[dst.dtype])
    _chk(lib().ora_scatter_scalar(ctypes.byref(dst.op), v.ctypes.data), "scatter_scalar")
    return dst.arr


def set_mask(arr, mask, value):
    """NArray#[]=(mask, value) / MultiWritable#set_mask (n_array.cr:510-551,
    multi_writable.cr:155-172): walks the coordinates in lexicographic order
    and writes value (a scalar, or the element of a same-shaped source at the
    coordinate) where the mask holds true.  arr is modified in place.  A
    Python loop: for the small cases of the parity tests."""
    mask = np.asarray(mask)
    if tuple(mask.shape) != tuple(arr.shape):
        raise OracleError(ERR_DIM, "set_mask")
    src = None
    if not np.isscalar(value) and not (isinstance(value, np.ndarray) and value.ndim == 0):
        src = np.asarray(value)
        if tuple(src.shape) != tuple(arr.shape):
            raise OracleError(ERR_SHAPE, "set_mask")
    for coord in np.ndindex(*arr.shape):
        if mask[coord]:
            arr[coord] = src[coord] if src is not None else value
    return arr


def tile(src, counts):
    """NArray.tile (n_array.cr:242-252 with TilingLexIterator,
    multi_indexable/tiling_lex_iterator.cr): the output walks its coordinates
    in lexicographic order and element c takes source element c mod shape.
    A Python loop for small cases."""
    src = np.asarray(src)
    shape = [n * int(c) for n, c in zip(src.shape, counts)]
    out = np.empty(shape, dtype=src.dtype)
    for coord in np.ndindex(*shape):
        out[coord] = src[tuple(c % n for c, n in zip(coord, src.shape))]
    return out


def concatenate(narrs, axis=0):
    """NArray.concatenate_to_slice (n_array.cr:726-749): for each chunk of the
    axes before `axis`, the next shape[axis] * stride[axis] elements of every
    operand in turn, each read in lexicographic order."""
    narrs = [np.asarray(n) for n in narrs]
    first = narrs[0]
    for n in narrs:
        if n.ndim != first.ndim or any(a != b for i, (a, b) in enumerate(zip(first.shape, n.shape)) if i != axis):
            raise OracleError(ERR_DIM, "concatenate")
    shape = list(first.shape)
    shape[axis] = sum(n.shape[axis] for n in narrs)
    partial = int(np.prod(first.shape[axis + 1:], dtype=np.int64))
    num_chunks = int(np.prod(shape[:axis], dtype=np.int64))
    flats = [n.reshape(-1) for n in narrs]
    pos = [0] * len(narrs)
    values = []
    for _ in range(num_chunks):
        for i, n in enumerate(narrs):
            size = n.shape[axis] * partial
            values.extend(flats[i][pos[i]:pos[i] + size].tolist())
            pos[i] += size
    return np.array(values, dtype=first.dtype).reshape(shape)


def lex_index(shape):
    """The index NArray#map_with_index hands its block (n_array.cr:605-611,
    `@buffer.map_with_index`): the buffer position of every element, which for
    the row-major buffer is its lexicographic position (Int32)."""
    n = int(np.prod(shape, dtype=np.int64))
    return np.arange(n, dtype=np.int32).reshape(shape)


def coords(shape):
    """The coordinates LexIterator.cover(shape) yields in lexicographic order
    (n_array.cr:641-650; MultiIndexable#map_with_coord builds over them,
    multi_indexable.cr:708-712): one Int32 array per axis."""
    return [np.ascontiguousarray(c.astype(np.int32)) for c in np.indices(shape, dtype=np.int64)]


def result_dtype(op, ta, tb):
    t = ctypes.c_int32()
    _chk(lib().ora_result_dtype(op, ta, tb, ctypes.byref(t)), "result_dtype")
    return t.value


def map_binary(op, a, b, nthreads=1):
    """a <op> b with Crystal semantics -> (numpy result, status bits)."""
    a = a if isinstance(a, ViewOperand) else ViewOperand(a)
    b = b if isinstance(b, ViewOperand) else ViewOperand(b)
    t = result_dtype(op, a.dtype, b.dtype)
    out = np.empty(a.shape, dtype=NP[t])
    st = ctypes.c_uint32()
    _chk(lib().ora_map_binary(op, ctypes.byref(a.op), ctypes.byref(b.op), out.ctypes.data, ctypes.byref(st),
                              nthreads), "map_binary")
    return out, st.value


def map_binary_scalar(op, a, scalar, scalar_dtype, scalar_left=False, nthreads=1):
    a = a if isinstance(a, ViewOperand) else ViewOperand(a)
    t = result_dtype(op, scalar_dtype, a.dtype) if scalar_left else result_dtype(op, a.dtype, scalar_dtype)
    out = np.empty(a.shape, dtype=NP[t])
    s = np.array(scalar, dtype=NP[scalar_dtype])
    st = ctypes.c_uint32()
    _chk(lib().ora_map_binary_scalar(op, ctypes.byref(a.op), s.ctypes.data, scalar_dtype, int(scalar_left),
                                     out.ctypes.data, ctypes.byref(st), nthreads), "map_binary_scalar")
    return out, st.value


def map_unary(uop, a):
    a = a if isinstance(a, ViewOperand) else ViewOperand(a)
    out = np.empty(a.shape, dtype=NP[a.dtype])
    st = ctypes.c_uint32()
    _chk(lib().ora_map_unary(uop, ctypes.byref(a.op), out.ctypes.data, ctypes.byref(st)), "map_unary")
    return out, st.value


def reduce(op, arr, axis=None, out_dtype=None):
    """Reference-path reduction (sequential fold / scan)."""
    arr = np.ascontiguousarray(arr)
    t = FROM_NP[arr.dtype]
    if out_dtype is None:
        out_dtype = I64 if op in (RED_ARGMAX, RED_ARGMIN) else t
    shape = list(arr.shape)
    oshape = [1] if axis is None else shape[:axis] + shape[axis + 1:]
    out = np.empty(oshape if oshape else [1], dtype=NP[out_dtype])
    _chk(lib().ora_reduce(op, arr.ctypes.data, t, _i64arr(shape), len(shape), -1 if axis is None else axis,
                          out.ctypes.data, out_dtype), "reduce")
    return out if (axis is not None and oshape) else out.reshape(-1)[0]


def reduce_f64(arr, axis=None):
    """FP64 oracle for sums."""
    arr = np.ascontiguousarray(arr)
    shape = list(arr.shape)
    oshape = [1] if axis is None else shape[:axis] + shape[axis + 1:]
    out = np.empty(oshape if oshape else [1], dtype=np.float64)
    _chk(lib().ora_reduce_f64(arr.ctypes.data, FROM_NP[arr.dtype], _i64arr(shape), len(shape),
                              -1 if axis is None else axis, out.ctypes.data), "reduce_f64")
    return out if (axis is not None and oshape) else out.reshape(-1)[0]


def heat_run(u, steps, coef=0.2, nthreads=1, f64=False):
    """`steps` explicit heat steps (Phase program in phase_oracle.c)."""
    if f64:
        a = np.ascontiguousarray(u, dtype=np.float64).copy()
        tmp = np.empty_like(a)
        fn = lib().ora_heat_run_f64
    else:
        a = np.ascontiguousarray(u, dtype=np.float32).copy()
        tmp = np.empty_like(a)
        fn = lib().ora_heat_run_f32
    _chk(fn(a.ctypes.data, tmp.ctypes.data, a.shape[0], a.shape[1], coef, steps, nthreads), "heat_run")
    return a


def mlp_forward_backward(params, x, y, in_dim=24, h1=64, h2=64):
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    grad = np.zeros(params.size, dtype=np.float64)
    loss = ctypes.c_double()
    _chk(lib().ora_mlp_forward_backward(params.ctypes.data, in_dim, h1, h2, x.ctypes.data, y.ctypes.data,
                                        len(y), ctypes.byref(loss), grad.ctypes.data), "mlp")
    return loss.value, grad
