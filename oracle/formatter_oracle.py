"""TEST INFRASTRUCTURE ONLY: a literal CPU restatement of the reference's
Formatter walk over a whole host array, used to check the product's
formatter (which gathers only the displayed elements on the device).

It follows src/multi_indexable/formatter/formatter.cr step by step:
- the element source is a lexicographic coordinate iterator that holds the
  last coordinate it yielded and yields its first coordinate without advancing
  (src/iterators/stride_iterator.cr:71-127, lex_iterator.cr:13-25);
- capped_iterator (formatter.cr:65-95) skips an over-long axis by adding
  size - (max_count - 1) to that axis' coordinate, exactly as the reference
  does, so the displayed elements are whatever that jump selects;
- walk_n_measure / walk_n_print / walk_n_print_flat / open / close / newline
  (formatter.cr:123-294) and format_element (formatter.cr:220-280).
Colours are left out (the product's tests switch them off).  Settings are
passed as a plain dict with the keys of settings.cr's constructor.
"""
import math
import re

import numpy as np

DEFAULT = {"indent_width": 4, "max_element_width": 15, "omit_after": [10, 5], "brackets": [("[", "]")],
           "collapse_brackets_after": 5, "integer_format": "%d", "decimal_format": "%.3g"}


def _fmt(fmt, v):
    if not re.search(r"%[-+ #0]*\d*(\.\d+)?[a-zA-Z]", fmt.replace("%%", "")):
        return fmt.replace("%%", "%")
    s = fmt % v
    if isinstance(v, float) and math.isnan(v) and math.copysign(1.0, v) < 0:
        s = s.replace("nan", "-nan")
    return s


class _Lex:
    """LexIterator.cover(shape) with the reference's hold flag."""

    def __init__(self, shape):
        self.last = [n - 1 for n in shape]
        self.coord = [0] * len(shape)
        self.hold = True

    def next(self):
        if self.hold:
            self.hold = False
            return list(self.coord)
        for i in range(len(self.coord) - 1, -1, -1):
            if self.coord[i] == self.last[i]:
                self.coord[i] = 0
                if i == 0:
                    raise StopIteration
            else:
                self.coord[i] += 1
                break
        return list(self.coord)

    def reset(self):
        self.coord = [0] * len(self.coord)
        self.hold = True


class OracleFormatter:
    ELEM, SKIP, LAST, EMPTY = range(4)

    def __init__(self, arr, settings=None):
        self.a = np.asarray(arr)
        self.s = dict(DEFAULT, **(settings or {}))
        self.shape = list(self.a.shape)
        self.it = _Lex(self.shape)
        self.out = []
        self.ind = 0
        self.just = 0
        if self.a.dtype == np.bool_:
            self.kind = "bool"
        elif np.issubdtype(self.a.dtype, np.integer):
            self.kind = "int"
        else:
            self.kind = "float"

    def _next(self):
        return self.a[tuple(self.it.next())]

    def _limit(self, height):
        lim = self.s["omit_after"]
        return lim[min(len(lim) - 1, height)]

    def capped(self, depth, max_count):
        size = self.shape[depth]
        if size > max_count:
            left = max_count // 2
            right = max_count - left - 1
            for idx in range(left):
                yield self.ELEM, idx
            self.it.coord[depth] += size - (max_count - 1)  # the reference's coordinate jump
            yield self.SKIP, -1
            for idx in range(right - 1):
                yield self.ELEM, size - right + idx
        elif size > 0:
            for idx in range(size - 1):
                yield self.ELEM, idx
        else:
            yield self.EMPTY, -1
            return
        yield self.LAST, size - 1

    def format_element(self, el):
        if self.kind == "int":
            s = _fmt(self.s["integer_format"], int(el))
            if len(s) > self.just:
                return self._float(float(int(el)))
            return s
        if self.kind == "float":
            return self._float(float(el))
        s = "true" if bool(el) else "false"
        if len(s) > self.just:
            s = s[:max(0, self.just - 3)] + "..."
        return s

    def _float(self, v):
        s = _fmt(self.s["decimal_format"], v)
        if len(s) > self.just:
            m = [i for i, c in enumerate(s) if c in "pePE"]
            if not m:
                s = _fmt("%e", v)
                m = [i for i, c in enumerate(s) if c in "pePE"]
            sep = m[-1]
            trunc = len(s) - self.just
            s = (s[0] if sep - trunc < 3 else s[:sep - trunc]) + s[sep:]
        return s

    def measure(self, depth=0):
        if int(np.prod(self.shape)) == 0:
            return 0
        height = len(self.shape) - depth - 1
        best = 0
        for flag, _ in self.capped(depth, self._limit(height)):
            if flag == self.SKIP:
                continue
            if depth < len(self.shape) - 1:
                best = max(best, self.measure(depth + 1))
            else:
                best = max(best, len(self.format_element(self._next())))
        return best

    def newline(self, change=0):
        self.out.append("\n")
        self.ind += change * self.s["indent_width"]
        self.out.append(" " * self.ind)

    def compact(self, height):
        return height > self.s["collapse_brackets_after"] or height == 1

    def open(self, height, idx):
        b = self.s["brackets"][height % len(self.s["brackets"])]
        t = _fmt(b[0], idx)
        self.out.append(t)
        if self.compact(height):
            self.ind += len(t)
        elif height != 0:
            self.newline(1)

    def close(self, height, idx):
        b = self.s["brackets"][height % len(self.s["brackets"])]
        if self.compact(height):
            self.ind -= len(_fmt(b[0], idx))
        elif height != 0:
            self.newline(-1)
        self.out.append(_fmt(b[1], idx))

    def walk(self, depth=0, idx=0):
        height = len(self.shape) - depth - 1
        maxc = self._limit(height)
        if self.shape[depth] == 0:
            self.open(height, idx)
            self.close(height, idx)
            return
        self.open(height, idx)
        extra = lambda: height == 2 or (self.s["collapse_brackets_after"] < 2 and height != 1)  # noqa: E731
        if height > 0:
            for flag, i in self.capped(depth, maxc):
                if flag == self.SKIP:
                    self.out.append(" ⋮ %d total, %d shown" % (self.shape[depth], maxc - 1))
                    self.newline()
                    if extra():
                        self.newline()
                else:
                    self.walk(depth + 1, i)
                    if flag == self.ELEM:
                        self.out.append(",")
                        self.newline()
                        if extra():
                            self.newline()
        else:
            for flag, _ in self.capped(depth, maxc):
                if flag == self.SKIP:
                    self.out.append("..., ")
                elif flag in (self.ELEM, self.LAST):
                    self.out.append(self.format_element(self._next()).rjust(self.just))
                    if flag != self.LAST:
                        self.out.append(", ")
        self.close(height, idx)


def format_body(arr, settings=None):
    """Formatter#print after the header line (formatter.cr:103-107)."""
    f = OracleFormatter(arr, settings)
    f.just = f.s["max_element_width"]
    f.just = f.measure()
    f.it.reset()
    f.walk()
    return "".join(f.out)


def _inspect(v, kind):
    """Crystal #inspect of a number or Bool: shortest round-trip float text,
    scientific below 1e-4 and from 1e16 on, with ".0" and a signed exponent."""
    if kind == "bool":
        return "true" if bool(v) else "false"
    if kind == "int":
        return str(int(v))
    f = float(v)
    if math.isnan(f):
        return "NaN"
    if math.isinf(f):
        return "Infinity" if f > 0 else "-Infinity"
    single = isinstance(v, np.float32)
    x = np.float32(v) if single else np.float64(v)
    if f == 0 or 1e-4 <= abs(f) < 1e16:
        t = np.format_float_positional(x, unique=True, trim="0")
        return t if "." in t else t + ".0"
    t = np.format_float_scientific(x, unique=True, trim="0")
    mant, exp = t.split("e")
    if "." not in mant:
        mant += ".0"
    return "%se%s%d" % (mant, "-" if exp.startswith("-") else "+", abs(int(exp)))


def format_literal(arr):
    """Formatter#print_literal (formatter.cr:109-112, 152-168): every element,
    nested square brackets, elements as #inspect prints them."""
    f = OracleFormatter(arr)

    def flat(depth):
        f.out.append("[")
        n = f.shape[depth]
        for i in range(n):
            if len(f.shape) - 1 > depth:
                flat(depth + 1)
            else:
                f.out.append(_inspect(f._next(), f.kind))
            if i != n - 1:
                f.out.append(", ")
        f.out.append("]")

    flat(0)
    return "".join(f.out)
