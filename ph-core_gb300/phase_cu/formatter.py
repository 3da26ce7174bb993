"""Pretty-printing of device arrays: the reference's Formatter and its
Settings (src/multi_indexable/formatter/formatter.cr, settings.cr), with only
the displayed elements brought to the host.

Which elements are displayed.  Along an axis of length n whose display limit
M (settings.display_limit, indexed by the axis' height above the innermost
axis) is below n, the reference shows the first M // 2 indices, a skip marker
and the last M - M // 2 - 1 indices (formatter.cr:65-95, capped_iterator,
whose coordinate jump lands on n - (M - M // 2 - 1) because the reference's
lexicographic iterator holds the last coordinate it yielded,
src/iterators/stride_iterator.cr:110-127).  The displayed elements are
therefore a product of per-axis index sets: gather_displayed() copies each
corner block of that product into one compact device array (one strided copy
per block) and downloads it in a single transfer.  The layout walk then reads
those elements in lexicographic order, the order in which the reference's
ElemIterator visits them during both its measuring and printing passes.
Display limits below 3 are refused: with them the reference's coordinate
jump leaves the axis (right part of length 0).

Element text follows the reference: `integer_format % e` for integers,
`decimal_format % e` for floats (C printf semantics, "-nan" for a NaN with its
sign bit set, as glibc prints it), shortened to the column width through
scientific notation (formatter.cr:233-262); Bool prints true/false.  Colours
are ANSI escapes as Crystal's Colorize writes them (ESC[<code>m text ESC[0m),
switched off globally with `Colorize.enabled = False`.
"""
import math
import os
import re

import numpy as np

from . import _abi as A


class FormatterError(ValueError):
    """YAML::ParseException / ArgumentError of the reference's settings loader."""


# ------------------------------------------------------------------ colours
class Colorize:
    """Crystal's Colorize switch and colour codes (ANSI foreground)."""

    enabled = True
    CODES = {"default": 39, "black": 30, "red": 31, "green": 32, "yellow": 33, "blue": 34, "magenta": 35,
             "cyan": 36, "light_gray": 37, "dark_gray": 90, "light_red": 91, "light_green": 92,
             "light_yellow": 93, "light_blue": 94, "light_magenta": 95, "light_cyan": 96, "white": 97}

    @classmethod
    def wrap(cls, text, color):
        if not cls.enabled or color == "default":
            return text
        if isinstance(color, tuple):
            code = "38;2;%d;%d;%d" % color
        else:
            code = str(cls.CODES[color])
        return "\x1b[%sm%s\x1b[0m" % (code, text)


# ----------------------------------------------------------------- settings
def _crystal_sprintf(fmt, value):
    """`fmt % value` in Crystal: a format without a conversion ignores the
    argument ("[" % 3 == "[")."""
    if not re.search(r"%[-+ #0]*\d*(\.\d+)?[a-zA-Z]", fmt.replace("%%", "")):
        return fmt.replace("%%", "%")
    return fmt % value


class Settings:
    """Formatter::Settings (settings.cr:4-212)."""

    USER_CONFIG_FILENAME = "formatter.yaml"
    project_settings = None
    _cached_user_settings = None
    _disable_user_settings = False

    def __init__(self, indent_width, max_element_width, omit_after, brackets, colors, collapse_brackets_after,
                 integer_format, decimal_format):
        self.indent_width = int(indent_width)
        self.max_element_width = int(max_element_width)
        self.display_limit = [int(x) for x in omit_after]
        self.brackets = [(str(a), str(b)) for a, b in brackets]
        self.colors = list(colors)
        self.collapse_height = int(collapse_brackets_after)
        self.integer_format = integer_format
        self.decimal_format = decimal_format

    @classmethod
    def new(cls):
        """project settings, else user settings, else the defaults (settings.cr:117-119)."""
        return cls.project_settings or cls.user_settings() or cls.default()

    @classmethod
    def default(cls):
        """settings.cr:158-169."""
        return cls(indent_width=4, max_element_width=15, omit_after=[10, 5], brackets=[("[", "]")],
                   colors=["red", "yellow", "blue"], collapse_brackets_after=5, integer_format="%d",
                   decimal_format="%.3g")

    @classmethod
    def user_settings(cls):
        """formatter.yaml from $PHASE_CONFIG_DIR, then $XDG_CONFIG_DIR/phase and
        ~/.config/phase; a failed search is remembered (settings.cr:126-156)."""
        if cls._disable_user_settings:
            return None
        if cls._cached_user_settings is not None:
            return cls._cached_user_settings
        cands = []
        if os.environ.get("PHASE_CONFIG_DIR"):
            cands.append(os.path.join(os.environ["PHASE_CONFIG_DIR"], cls.USER_CONFIG_FILENAME))
        for d in (os.environ.get("XDG_CONFIG_DIR"), "~/.config"):
            if d:
                cands.append(os.path.join(d, "phase", cls.USER_CONFIG_FILENAME))
        for path in cands:
            path = os.path.expanduser(path)
            if os.path.isfile(path):
                with open(path) as f:
                    cls._cached_user_settings = cls.from_yaml(f.read())
                return cls._cached_user_settings
        cls._disable_user_settings = True
        return None

    @classmethod
    def from_yaml(cls, text):
        """The settings mapping (keys as settings.cr names them: omit_after,
        collapse_brackets_after, ...).  Colours are Colorize names or 6-digit
        RGB hex strings (settings.cr:171-210)."""
        d = _parse_yaml_mapping(text)
        need = ["indent_width", "max_element_width", "omit_after", "brackets", "colors", "collapse_brackets_after",
                "integer_format", "decimal_format"]
        for k in need:
            if k not in d:
                raise FormatterError("Missing YAML attribute: %s" % k)
        colors = [_parse_color(c) for c in d["colors"]]
        brackets = []
        for b in d["brackets"]:
            if not isinstance(b, list) or len(b) != 2:
                raise FormatterError("Expected a pair of brackets, not %r" % (b,))
            brackets.append((b[0], b[1]))
        return cls(d["indent_width"], d["max_element_width"], d["omit_after"], brackets, colors,
                   d["collapse_brackets_after"], d["integer_format"], d["decimal_format"])

    def to_yaml(self):
        """The settings as from_yaml reads them.  RGB colours are written as
        plain hex ("12ABFF"): the reference writes "#12ABFF", which its own
        loader then refuses."""
        def color(c):
            return "\"%02X%02X%02X\"" % c if isinstance(c, tuple) else c

        def q(s):
            return '"%s"' % s.replace("\\", "\\\\").replace('"', '\\"')

        lines = ["---",
                 "indent_width: %d" % self.indent_width,
                 "max_element_width: %d" % self.max_element_width,
                 "omit_after: [%s]" % ", ".join(str(x) for x in self.display_limit),
                 "brackets:"] + ["- [%s, %s]" % (q(a), q(b)) for a, b in self.brackets] + [
                 "colors: [%s]" % ", ".join(color(c) for c in self.colors),
                 "collapse_brackets_after: %d" % self.collapse_height,
                 "integer_format: %s" % q(self.integer_format),
                 "decimal_format: %s" % q(self.decimal_format)]
        return "\n".join(lines) + "\n"


def _parse_color(c):
    if isinstance(c, str):
        if c in Colorize.CODES:
            return c
        h = c[1:] if c.startswith("#") else c
        if re.fullmatch(r"[0-9a-fA-F]{6}", h) and not c.startswith("#"):
            return tuple(int(h[i:i + 2], 16) for i in (0, 2, 4))
    raise FormatterError("Expected %s, or an RGB hex string, not %r" % (", ".join('"%s"' % k for k in Colorize.CODES),
                                                                       c))


def _yaml_token(tok):
    tok = tok.strip()
    if len(tok) >= 2 and tok[0] == tok[-1] and tok[0] in "\"'":
        body = tok[1:-1]
        return body.replace('\\"', '"').replace("\\\\", "\\") if tok[0] == '"' else body.replace("''", "'")
    if re.fullmatch(r"[-+]?\d+", tok):
        return int(tok)
    return tok


def _split_flow(body):
    """Items of a flow sequence body, respecting quotes and nested brackets."""
    items, cur, depth, quote = [], "", 0, None
    for ch in body:
        if quote:
            cur += ch
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        elif ch == "," and depth == 0:
            items.append(cur)
            cur = ""
            continue
        cur += ch
    if cur.strip():
        items.append(cur)
    return items


def _yaml_value(text):
    text = text.strip()
    if text.startswith("["):
        if not text.endswith("]"):
            raise FormatterError("unterminated flow sequence: %s" % text)
        return [_yaml_value(t) for t in _split_flow(text[1:-1])]
    return _yaml_token(text)


def _strip_comment(line):
    quote = None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _parse_yaml_mapping(text):
    """The block mapping of scalars, flow sequences and block sequences that a
    settings file holds."""
    out, key = {}, None
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        s = line.strip()
        if s.startswith("- "):
            if key is None or not isinstance(out.get(key), list):
                raise FormatterError("sequence item outside a sequence: %s" % raw)
            out[key].append(_yaml_value(s[2:]))
            continue
        m = re.match(r"^([A-Za-z_][A-Za-z0-9_]*)\s*:(.*)$", s)
        if not m or line[0] in " \t":
            raise FormatterError("unsupported settings line: %s" % raw)
        key, rest = m.group(1), m.group(2).strip()
        out[key] = _yaml_value(rest) if rest else []
    return out


# ------------------------------------------------------- displayed elements
def _limit(settings, height):
    return settings.display_limit[min(len(settings.display_limit) - 1, height)]


def displayed_ranges(shape, settings):
    """Per axis, the index ranges [(start, stop), ...] the formatter shows."""
    rank = len(shape)
    out = []
    for d, n in enumerate(shape):
        m = _limit(settings, rank - d - 1)
        if m < 3:
            raise ValueError("display limit %d below 3: the reference's skip leaves the axis" % m)
        if n > m:
            left = m // 2
            right = m - left - 1
            out.append([(0, left), (n - right, n)])
        else:
            out.append([(0, n)])
    return out


def _compact_on_device(arr, ranges):
    """A new device array holding the elements of the device view `arr` at the
    product of the per-axis index ranges: one strided copy per corner block."""
    from .narray import CuNArray, _copy_into, _make_view, _row_major

    kshape = [sum(b - a for a, b in r) for r in ranges]
    out = CuNArray.empty(kshape, arr.dtype)
    if any(n == 0 for n in kshape):
        return out
    buf, off, _, stride = arr._desc()
    ostride = _row_major(kshape)
    combos = [[]]
    for d in range(len(ranges)):
        combos = [c + [(d, i)] for c in combos for i in range(len(ranges[d]))]
    for combo in combos:
        soff, doff, bshape = off, 0, []
        for d, i in combo:
            a, b = ranges[d][i]
            pos = sum(y - x for x, y in ranges[d][:i])  # where this range starts in the compact axis
            soff += a * stride[d]
            doff += pos * ostride[d]
            bshape.append(b - a)
        _copy_into(_make_view(out._buf, arr.dtype, doff, bshape, ostride),
                   _make_view(buf, arr.dtype, soff, bshape, stride))
    return out


def gather_displayed(arr, settings):
    """The displayed elements of a device array as a compact host array: one
    strided device copy per corner block of the displayed index product, then
    one download.  A lazy CuProcView gathers the displayed elements of each of
    its operand views and runs its fused program on those alone, as the
    reference's ProcView computes only the elements it is asked for."""
    from .narray import CuNArray, CuProcView

    shape = list(arr.shape)
    ranges = displayed_ranges(shape, settings)
    kshape = [sum(b - a for a, b in r) for r in ranges]
    if any(n == 0 for n in kshape):
        return np.empty(kshape, dtype=arr.np_dtype)
    if isinstance(arr, CuProcView):
        leaves = [CuProcView._leaf(_compact_on_device(v, ranges)) for v in arr._leaves]
        compact = CuProcView([x._leaves[0] for x in leaves], arr._expr, arr.dtype, kshape)
        return compact.to_narr()
    if kshape == shape and isinstance(arr, CuNArray):
        return arr.to_narr()
    return _compact_on_device(arr, ranges).to_narr()


# ---------------------------------------------------------- element text
def _c_format(fmt, v):
    """C printf of a double (glibc writes "-nan" for a NaN with the sign bit)."""
    s = _crystal_sprintf(fmt, v)
    if isinstance(v, float) and math.isnan(v) and math.copysign(1.0, v) < 0:
        s = s.replace("nan", "-nan").replace("NAN", "-NAN")
    return s


class Formatter:
    """MultiIndexable::Formatter (formatter.cr:15-296) over a compact array of
    the displayed elements, walked with the full shape."""

    ELEM, SKIP, LAST, EMPTY = range(4)

    def __init__(self, shape, displayed, kind, settings):
        self.settings = settings
        self.shape = list(shape)
        self.kind = kind  # "int", "float" or "bool"
        self.elems = np.asarray(displayed).reshape(-1)
        self.pos = 0
        self.out = []
        self.current_indentation = 0
        self.justify_length = 0

    # ------------------------------------------------------------ entry
    @classmethod
    def print(cls, arr, settings=None, class_name=None):
        """Formatter.print (formatter.cr:40-56): header line, then the layout."""
        settings = settings or Settings.new()
        shape = list(arr.shape)
        dims = len(shape)
        disp = []
        for i, n in enumerate(shape):
            color = settings.colors[(dims - i + 1) % len(settings.colors)] if i < dims - 1 else "default"
            disp.append(Colorize.wrap(str(n), color))
        head = "%s %s%s\n" % ("x".join(disp), "element " if dims == 1 else "", class_name or _class_name(arr))
        f = cls(shape, _displayed(arr, settings), _kind(arr), settings)
        f.measure()
        f.walk_n_print(0, 0)
        return head + "".join(f.out)

    @classmethod
    def print_literal(cls, arr):
        """Formatter.print_literal (formatter.cr:58-61): every element, nested brackets."""
        f = cls(list(arr.shape), _host(arr), _kind(arr), Settings.new())
        f.walk_n_print_flat(0)
        return "".join(f.out)

    # ------------------------------------------------------------ walk
    def _next(self):
        v = self.elems[self.pos]
        self.pos += 1
        return v

    def capped(self, depth, max_count):
        size = self.shape[depth]
        if size > max_count:
            left = max_count // 2
            right = max_count - left - 1
            for idx in range(left):
                yield self.ELEM, idx
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

    def measure(self):
        self.justify_length = self.settings.max_element_width
        self.justify_length = self.walk_n_measure(0)
        self.pos = 0

    def walk_n_measure(self, depth):
        if any(n == 0 for n in self.shape):
            return 0
        height = len(self.shape) - depth - 1
        maxc = _limit(self.settings, height)
        best = 0
        for flag, _ in self.capped(depth, maxc):
            if flag == self.SKIP:
                continue
            if depth < len(self.shape) - 1:
                best = max(best, self.walk_n_measure(depth + 1))
            else:
                best = max(best, len(self.format_element(self._next())))
        return best

    def walk_n_print_flat(self, depth):
        self.out.append("[")
        n = self.shape[depth]
        for i in range(n):
            if len(self.shape) - 1 > depth:
                self.walk_n_print_flat(depth + 1)
            else:
                self.out.append(_inspect(self._next(), self.kind))
            if i != n - 1:
                self.out.append(", ")
        self.out.append("]")

    def walk_n_print(self, depth, idx):
        height = len(self.shape) - depth - 1
        maxc = _limit(self.settings, height)
        if self.shape[depth] == 0:
            self.open(height, idx)
            self.close(height, idx)
            return
        self.open(height, idx)
        if height > 0:
            for flag, i in self.capped(depth, maxc):
                if flag == self.SKIP:
                    self.color_print(" ⋮ %d total, %d shown" % (self.shape[depth], maxc - 1), height)
                    self.newline()
                    if height == 2 or (self.settings.collapse_height < 2 and height != 1):
                        self.newline()
                else:
                    self.walk_n_print(depth + 1, i)
                    if flag == self.ELEM:
                        self.color_print(",", height)
                        self.newline()
                        if height == 2 or (self.settings.collapse_height < 2 and height != 1):
                            self.newline()
        else:
            for flag, _ in self.capped(depth, maxc):
                if flag == self.SKIP:
                    self.out.append("..., ")
                elif flag in (self.ELEM, self.LAST):
                    self.out.append(self.format_element(self._next()).rjust(self.justify_length, " "))
                    if flag != self.LAST:
                        self.out.append(", ")
        self.close(height, idx)

    # -------------------------------------------------------- elements
    def format_element(self, el):
        if self.kind == "int":
            s = _crystal_sprintf(self.settings.integer_format, int(el))
            if len(s) > self.justify_length:
                return self._format_float(float(int(el)))
            return s
        if self.kind == "float":
            return self._format_float(float(el))
        s = "true" if bool(el) else "false"
        if len(s) > self.justify_length:
            s = s[:max(0, self.justify_length - 3)] + "..."
        return s

    def _format_float(self, v):
        s = _c_format(self.settings.decimal_format, v)
        if len(s) > self.justify_length:
            sep = _rindex_pe(s)
            if sep is None:
                s = _c_format("%e", v)
                sep = _rindex_pe(s)
            trunc = len(s) - self.justify_length
            mantissa = s[0] if sep - trunc < 3 else s[:sep - trunc]
            s = mantissa + s[sep:]
        return s

    # ----------------------------------------------------------- layout
    def color_print(self, text, height):
        self.out.append(Colorize.wrap(text, self.settings.colors[height % len(self.settings.colors)]))

    def compact(self, height):
        return height > self.settings.collapse_height or height == 1

    def newline(self, indent_change=0):
        self.out.append("\n")
        self.current_indentation += indent_change * self.settings.indent_width
        self.out.append(" " * self.current_indentation)

    def open(self, height, idx):
        b = self.settings.brackets[height % len(self.settings.brackets)]
        text = _crystal_sprintf(b[0], idx)
        self.color_print(text, height)
        if self.compact(height):
            self.current_indentation += len(text)
        elif height != 0:
            self.newline(1)

    def close(self, height, idx):
        b = self.settings.brackets[height % len(self.settings.brackets)]
        if self.compact(height):
            self.current_indentation -= len(_crystal_sprintf(b[0], idx))
        elif height != 0:
            self.newline(-1)
        self.color_print(_crystal_sprintf(b[1], idx), height)


def _rindex_pe(s):
    for i in range(len(s) - 1, -1, -1):
        if s[i] in "pePE":
            return i
    return None


def _inspect(v, kind):
    """Crystal #inspect of one element (print_literal)."""
    if kind == "bool":
        return "true" if bool(v) else "false"
    if kind == "int":
        return str(int(v))
    from .serial import _float_text

    f = float(v)
    if math.isnan(f):
        return "NaN"
    if math.isinf(f):
        return "Infinity" if f > 0 else "-Infinity"
    return _float_text(v, isinstance(v, np.float32), False)


# -------------------------------------------------- device / host sources
def _kind(arr):
    t = getattr(arr, "dtype", None)
    if t in (A.F32, A.F64):
        return "float"
    if t in (A.I32, A.I64):
        return "int"
    if t == A.BOOL:
        return "bool"
    dt = np.asarray(arr).dtype
    if dt == np.bool_:
        return "bool"
    return "int" if np.issubdtype(dt, np.integer) else "float"


def _class_name(arr):
    t = getattr(arr, "dtype", None)
    if t in A.DTYPE_NAMES:
        return "Phase::%s(%s)" % (type(arr).__name__, A.DTYPE_NAMES[t])
    dt = np.asarray(arr).dtype
    names = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.int32): "Int32",
             np.dtype(np.int64): "Int64", np.dtype(np.bool_): "Bool"}
    return "Phase::NArray(%s)" % names.get(dt, str(dt))


def _displayed(arr, settings):
    if hasattr(arr, "_desc"):
        return gather_displayed(arr, settings)
    a = np.asarray(arr)
    ranges = displayed_ranges(list(a.shape), settings)
    idx = np.ix_(*[np.concatenate([np.arange(x, y) for x, y in r]).astype(np.int64) for r in ranges])
    return a[idx] if a.ndim else a


def _host(arr):
    return arr.to_narr() if hasattr(arr, "_desc") else np.asarray(arr)


def to_s(arr, settings=None):
    """MultiIndexable#to_s (formatter.cr:304-315)."""
    return Formatter.print(arr, settings)


def to_literal_s(arr):
    """MultiIndexable#to_literal_s (formatter.cr:298-300)."""
    return Formatter.print_literal(arr)
