"""Region literals, RangeSyntax and IndexRegion: host-side validation.

The reference keeps all index validation on the host (src/range_syntax/,
src/index_region.cr, src/coord_util.cr); so does this backend.  A region
literal is a sequence with one entry per leading axis:

  * an int            -- an integer index (the axis is dropped when drop=True)
  * R(first, last, step=None, exclusive=False)
                      -- Crystal's `first..last`, `first...last`,
                         `first..step..last`; any of first/last/step may be None
  * a Python slice    -- `a:b:s` means R(a, b, s, exclusive=b is not None)
  * slice(None) / ... -- the full axis (Crystal `..`)

Canonical regions follow RangeSyntax.infer_range / canonicalize_range
(src/range_syntax/range_syntax.cr:84-153) and IndexRegion
(src/index_region.cr:192-702).
"""
from .errors import DimensionError, ShapeError


class R:
    """A Crystal range literal: `first..last`, `first...last` or `first..step..last`."""

    __slots__ = ("first", "last", "step", "exclusive")

    def __init__(self, first=None, last=None, step=None, exclusive=False):
        self.first, self.last, self.step, self.exclusive = first, last, step, bool(exclusive)

    def __repr__(self):
        f = "" if self.first is None else str(self.first)
        l = "" if self.last is None else str(self.last)
        dots = "..." if self.exclusive else ".."
        if self.step is None:
            return "%s%s%s" % (f, dots, l)
        return "%s..%d%s%s" % (f, self.step, dots, l)


def parse_literal(lit):
    """RangeSyntax.parse_range (range_syntax.cr:42-68): -> dict or int."""
    if isinstance(lit, bool):
        raise TypeError("a Bool is not a region literal")
    if isinstance(lit, int):
        return int(lit)
    if lit is Ellipsis:
        return {"first": None, "last": None, "step": None, "exclusive": False}
    if isinstance(lit, slice):
        return {"first": lit.start, "last": lit.stop, "step": lit.step, "exclusive": lit.stop is not None}
    if isinstance(lit, R):
        return {"first": lit.first, "last": lit.last, "step": lit.step, "exclusive": lit.exclusive}
    if hasattr(lit, "__index__"):
        return int(lit.__index__())
    raise TypeError("poorly formatted range literal: %r" % (lit,))


def _sign(x):
    return (x > 0) - (x < 0)


def get_size(first, last, step):
    """RangeSyntax.get_size (range_syntax.cr:7-17)."""
    if last != first and _sign(step) != _sign(last - first):
        raise IndexError("Could not get size of range - step direction disagrees with first and last.")
    if step == 0:
        raise IndexError("Could not get size of range - zero step.")
    if last >= first:
        return (last - first) // step + 1
    return (first - last) // (-step) + 1


def _canon_unsafe(index, size):
    return size + index if index < 0 else index


def canonicalize_index(index, size):
    """CoordUtil.canonicalize_index (coord_util.cr:43-48)."""
    if not (index < size and index >= -size):
        raise IndexError("Could not canonicalize index: %d is not a valid index for an axis of length %d."
                         % (index, size))
    return _canon_unsafe(index, size)


def infer_range(lit, bound):
    """RangeSyntax.infer_range (range_syntax.cr:84-136) -> (first, step, last, size)."""
    p = parse_literal(lit)
    if isinstance(p, int):
        c = _canon_unsafe(p, bound)
        return (c, 1, c, 1)
    f, l, step = p["first"], p["last"], p["step"]
    if step is None:
        first = 0 if f is None else _canon_unsafe(f, bound)
        temp_last = bound - 1 if l is None else _canon_unsafe(l, bound)
        step = 1 if temp_last >= first else -1
    else:
        first = (0 if step > 0 else bound - 1) if f is None else _canon_unsafe(f, bound)
        temp_last = (bound - 1 if step > 0 else 0) if l is None else _canon_unsafe(l, bound)
    if l is not None and p["exclusive"]:
        if temp_last == first:
            return (0, 0, 0, 0)
        temp_last -= _sign(step)
    if first < 0 or temp_last < 0:
        raise IndexError("Invalid index: At least one endpoint of %r is negative after canonicalization." % (lit,))
    try:
        size = get_size(first, temp_last, step)
    except IndexError:
        raise IndexError("Could not canonicalize range: Conflict between implicit direction of %r and provided "
                         "step %s" % (lit, step))
    return (first, step, first + step * (size - 1), size)


def canonicalize_range(lit, bound):
    """RangeSyntax.canonicalize_range (range_syntax.cr:145-153)."""
    r = infer_range(lit, bound)
    first, _, last, _ = r
    if not (0 <= last < bound and 0 <= first < bound):
        raise IndexError("Could not canonicalize range: %r is not a sensible index range for axis of length %d."
                         % (lit, bound))
    return r


def shape_to_size(shape):
    """ShapeUtil.shape_to_size (shape_util.cr:41-50)."""
    if len(shape) == 0:
        return 0
    n = 1
    for s in shape:
        n *= s
    return n


def compatible_shapes(s1, s2):
    """ShapeUtil.compatible_shapes? (shape_util.cr:6-32)."""
    if len(s1) == 0 or len(s2) == 0:
        return list(s1) == list(s2)
    larger, shared = (s1, len(s2)) if len(s1) > len(s2) else (s2, len(s1))
    for i in range(shared):
        if s1[i] != s2[i]:
            return False
    return all(larger[i] == 1 for i in range(shared, len(larger)))


class IndexRegion:
    """Canonical region: per proper axis {first, step, last, size}, degeneracy, drop."""

    def __init__(self, first, step, last, proper_shape, drop=True, degeneracy=None):
        self.first = list(first)
        self.step = list(step)
        self.last = list(last)
        self.proper_shape = list(proper_shape)
        self.drop = bool(drop)
        self.degeneracy = list(degeneracy) if degeneracy is not None else [False] * len(self.proper_shape)
        self._reduce()

    def _reduce(self):
        # IndexRegion.compute_reduced_shape (index_region.cr:304-317)
        if self.drop:
            red = [s for s, d in zip(self.proper_shape, self.degeneracy) if not d]
            if not red:
                red = [shape_to_size(self.proper_shape)]
            self.reduced_shape = red
        else:
            self.reduced_shape = list(self.proper_shape)

    # --------------------------------------------------------- constructors
    @classmethod
    def new(cls, region_literal, bound_shape, drop=True):
        """IndexRegion.new(region_literal, bound_shape, drop) (index_region.cr:192-224)."""
        lits = list(region_literal)
        n = len(bound_shape)
        if len(lits) > n:
            raise DimensionError("The region literal %r had more dimensions than its bound shape %r"
                                 % (lits, list(bound_shape)))
        first, step, last, shape, degen = [0] * n, [1] * n, [0] * n, [0] * n, [False] * n
        for i, lit in enumerate(lits):
            f, s, l, sz = canonicalize_range(lit, bound_shape[i])
            first[i], step[i], last[i], shape[i] = f, s, l, sz
            if isinstance(parse_literal(lit), int):
                degen[i] = drop
        for a in range(len(lits), n):
            last[a] = bound_shape[a] - 1
            shape[a] = bound_shape[a]
        return cls(first, step, last, shape, drop, degen)

    @classmethod
    def absolute(cls, region_literal, drop=True):
        """IndexRegion.new(region_literal, drop) without a bound (index_region.cr:255-283)."""
        lits = list(region_literal)
        n = len(lits)
        first, step, last, shape, degen = [0] * n, [0] * n, [0] * n, [0] * n, [False] * n
        for i, lit in enumerate(lits):
            p = parse_literal(lit)
            if isinstance(p, int):
                if p < 0:
                    raise IndexError("Negative indices have no meaning when a bounding shape is not provided.")
                degen[i] = True
            else:
                for e in (p["first"], p["last"]):
                    if e is not None and e < 0:
                        raise IndexError("Negative indices have no meaning when a bounding shape is not provided.")
                st = p["step"]
                bounded = (p["last"] is not None) if (st is None or st >= 0) else (p["first"] is not None)
                if not bounded:
                    raise ValueError("Cannot create IndexRegion without an explicit upper bound unless you provide "
                                     "a bounding shape")
            f, s, l, sz = infer_range(lit, 0)
            first[i], step[i], last[i], shape[i] = f, s, l, sz
        return cls(first, step, last, shape, drop, degen)

    @classmethod
    def trimmed(cls, region_literal, trim_to, bound_shape=None, drop=True):
        """IndexRegion.new(region_literal, bound_shape?, drop, trim_to:) (index_region.cr:137-169)."""
        lits = list(region_literal)
        n = len(trim_to)
        allow_relative = bound_shape is not None
        bs = list(bound_shape) if bound_shape is not None else list(trim_to)
        first, step, last, shape, degen = [0] * n, [1] * n, [0] * n, [0] * n, [False] * n
        for i, lit in enumerate(lits):
            p = parse_literal(lit)
            if not allow_relative:
                ends = [p] if isinstance(p, int) else [p["first"], p["last"]]
                if any(e is not None and e < 0 for e in ends):
                    raise IndexError("Negative indices have no meaning when a bounding shape is not provided.")
            f, s, l, sz = infer_range(lit, bs[i])
            first[i], step[i], last[i], shape[i] = f, s, l, sz
            if isinstance(p, int):
                degen[i] = drop
        for a in range(len(lits), n):
            last[a] = bs[a] - 1
            shape[a] = bs[a]
        return cls(first, step, last, shape, drop, degen).trim(trim_to)

    @classmethod
    def cover(cls, bound_shape, drop=True):
        """IndexRegion.cover (index_region.cr:232-238)."""
        return cls([0] * len(bound_shape), [0 if x == 0 else 1 for x in bound_shape],
                   [max(0, x - 1) for x in bound_shape], list(bound_shape), drop, None)

    # ----------------------------------------------------------- queries
    @property
    def shape(self):
        return list(self.reduced_shape)

    @property
    def size(self):
        return shape_to_size(self.reduced_shape)

    @property
    def proper_dimensions(self):
        return len(self.proper_shape)

    def clone(self):
        return IndexRegion(self.first, self.step, self.last, self.proper_shape, self.drop, self.degeneracy)

    def fits_in(self, bound_shape):
        """IndexRegion#fits_in? (index_region.cr:468-478)."""
        if len(bound_shape) != self.proper_dimensions:
            raise DimensionError("The bound shape provided had a different number of dimensions than this "
                                 "IndexRegion, so fits_in? is meaningless.")
        return all(b > max(f, l) for b, f, l in zip(bound_shape, self.first, self.last))

    def trim(self, bound_shape):
        """IndexRegion#trim! (index_region.cr:502-515, trim_axis :684-702); in place, returns self."""
        if len(bound_shape) != self.proper_dimensions:
            raise DimensionError("Cannot trim a %d-dimensional region to a %d-dimensional shape"
                                 % (self.proper_dimensions, len(bound_shape)))
        for a, nb in enumerate(bound_shape):
            f, s, l, sz = self.first[a], self.step[a], self.last[a], self.proper_shape[a]
            if f >= nb:
                if l >= nb:
                    f, s, l, sz = 0, 0, 0, 0
                elif s < 0:
                    span = (nb - 1) - l
                    sz = span // abs(s) + 1
                    span -= span % abs(s)
                    f = l + span
            elif s > 0 and l >= nb:
                span = (nb - 1) - f
                span -= span % abs(s)
                sz = span // abs(s) + 1
                l = f + span
            self.first[a], self.step[a], self.last[a], self.proper_shape[a] = f, s, l, sz
        self._reduce()
        return self

    def reverse(self):
        """IndexRegion#reverse! (index_region.cr:533-537); in place, returns self."""
        self.first, self.last = self.last, self.first
        self.step = [-s for s in self.step]
        return self

    def translate(self, offset):
        """IndexRegion#translate! (index_region.cr:577-585); in place, returns self."""
        for a, amt in enumerate(offset):
            if amt < 0 and (self.first[a] < -amt or self.last[a] < -amt):
                raise IndexError("Can't translate to negative indices")
        for a, amt in enumerate(offset):
            self.first[a] += amt
            self.last[a] += amt
        return self

    def includes(self, coord):
        """IndexRegion#includes? (index_region.cr:445-458)."""
        if len(coord) != self.proper_dimensions:
            return False
        for i, o in enumerate(coord):
            lo, hi = (self.first[i], self.last[i]) if self.step[i] > 0 else (self.last[i], self.first[i])
            if not (lo <= o <= hi) or self.step[i] == 0:
                return False
            if (o - self.first[i]) % self.step[i] != 0:
                return False
        return True

    def local_to_absolute(self, coord):
        """IndexRegion#local_to_absolute_unsafe (index_region.cr:621-637)."""
        if self.drop:
            out, la = [], 0
            for i, d in enumerate(self.degeneracy):
                if d:
                    out.append(self.first[i])
                else:
                    out.append(self.first[i] + coord[la] * self.step[i])
                    la += 1
            return out
        return [f + c * s for f, c, s in zip(self.first, coord, self.step)]

    def __eq__(self, other):
        return (isinstance(other, IndexRegion) and self.first == other.first and self.step == other.step
                and self.last == other.last and self.degeneracy == other.degeneracy and self.drop == other.drop)

    def __repr__(self):
        parts = []
        for i in range(self.proper_dimensions):
            if self.degeneracy[i]:
                parts.append(str(self.first[i]))
            elif abs(self.step[i]) == 1:
                parts.append("%d..%d" % (self.first[i], self.last[i]))
            else:
                parts.append("%d..%d..%d" % (self.first[i], self.step[i], self.last[i]))
        return "IndexRegion[%s]" % ", ".join(parts)


def normalise_literal(args):
    """Accepts region literals written as a tuple/list or as splatted arguments."""
    if len(args) == 1 and isinstance(args[0], (list, tuple)):
        return list(args[0])
    return list(args)


def check_region_fits(region, shape):
    """MultiIndexable#get_chunk(region) checks (multi_indexable.cr:337-348)."""
    if region.proper_dimensions != len(shape):
        raise DimensionError("'region' was %d-dimensional, but this MultiIndexable is %d-dimensional."
                             % (region.proper_dimensions, len(shape)))
    if not region.fits_in(shape):
        raise ShapeError("'region' (%r) cannot fit into a MultiIndexable with shape %r." % (region, list(shape)))
