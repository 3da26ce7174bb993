"""JSON and YAML forms of an NArray (src/n_array.cr:807-912): an object with
"shape" and "elements" (row-major), written after one bulk download and read
before one bulk upload.

Scalars print as Crystal prints them: integers in decimal, booleans as
true/false, floats in the shortest form that reads back to the same value
(Float32 at Float32 precision), with ".0" on integral values and an exponent
written as "e+N" / "e-N" after a mantissa that always has a decimal point;
non-finite floats are refused in JSON and written .nan / .inf / -.inf in YAML.
"""
import json

import numpy as np


class SerialError(ValueError):
    """JSON::Error / YAML::Error of the reference."""


def _float_text(x, single, yaml):
    v = float(x)
    if v != v or v in (float("inf"), float("-inf")):
        if not yaml:  # JSON::Builder refuses non-finite numbers
            raise SerialError("%s not allowed in JSON" % ("NaN" if v != v else "Infinity"))
        return ".nan" if v != v else (".inf" if v > 0 else "-.inf")
    if single:  # shortest text that reads back to the same Float32
        f = np.float32(x)
        if v == 0 or 1e-4 <= abs(v) < 1e16:
            s = np.format_float_positional(f, unique=True, trim="0")
        else:
            s = np.format_float_scientific(f, unique=True, trim="0")
    else:
        s = repr(v)
    if "e" in s:
        mant, exp = s.split("e")
        if "." not in mant:
            mant += ".0"
        return "%se%s%d" % (mant, "-" if exp.startswith("-") else "+", abs(int(exp)))
    return s if "." in s else s + ".0"


def _scalar_text(x, dt, yaml=False):
    if dt == np.bool_:
        return "true" if bool(x) else "false"
    if np.issubdtype(dt, np.integer):
        return str(int(x))
    return _float_text(x, dt == np.float32, yaml)


def to_json(arr):
    """NArray#to_json (n_array.cr:807-817)."""
    arr = np.asarray(arr)
    shape = ",".join(str(int(n)) for n in arr.shape)
    elems = ",".join(_scalar_text(v, arr.dtype.type) for v in arr.reshape(-1))
    return '{"shape":[%s],"elements":[%s]}' % (shape, elems)


def to_yaml(arr):
    """NArray#to_yaml (n_array.cr:854-868): flow sequences for numbers."""
    arr = np.asarray(arr)
    shape = ", ".join(str(int(n)) for n in arr.shape)
    elems = ", ".join(_scalar_text(v, arr.dtype.type, True) for v in arr.reshape(-1))
    return "---\nshape: [%s]\nelements: [%s]\n" % (shape, elems)


def _coerce(values, dtype):
    dt = np.dtype(dtype)
    try:
        if dt == np.bool_:
            if not all(isinstance(v, bool) for v in values):
                raise TypeError
            return np.array(values, dtype=np.bool_)
        if np.issubdtype(dt, np.integer):
            if not all(isinstance(v, int) and not isinstance(v, bool) for v in values):
                raise TypeError
            info = np.iinfo(dt)
            if any(v < info.min or v > info.max for v in values):
                raise TypeError
            return np.array(values, dtype=dt)
        return np.array([float(v) for v in values], dtype=dt)
    except (TypeError, ValueError):
        raise SerialError("element of the wrong type for %s" % dt.name) from None


def _build(shape, elements, dtype, what):
    if shape is None or elements is None:
        raise SerialError("Could not read NArray from %s: 'shape' and/or 'elements' were missing." % what)
    if not isinstance(shape, list) or not all(isinstance(n, int) and not isinstance(n, bool) for n in shape):
        raise SerialError("Could not read NArray from %s: shape must be a list of Int32" % what)
    size = int(np.prod(shape, dtype=np.int64)) if shape else 1
    if size != len(elements):
        raise SerialError("Could not read NArray from %s: wrong number of elements for shape %s" % (what, shape))
    return _coerce(elements, dtype).reshape(shape)


def from_json(text, dtype):
    """NArray(T).new(JSON::PullParser) (n_array.cr:819-852)."""
    try:
        obj = json.loads(text, parse_constant=lambda c: {"NaN": float("nan"), "Infinity": float("inf"),
                                                          "-Infinity": float("-inf")}[c])
    except json.JSONDecodeError as e:
        raise SerialError(str(e)) from None
    if not isinstance(obj, dict):
        raise SerialError("Could not read NArray from JSON: expected an object")
    return _build(obj.get("shape"), obj.get("elements"), dtype, "JSON")


def _yaml_scalar(tok):
    t = tok.strip()
    if t in ("true", "false"):
        return t == "true"
    for conv in (int, float):
        try:
            return conv(t)
        except ValueError:
            pass
    low = t.lower()
    if low in (".nan", "nan"):
        return float("nan")
    if low in (".inf", "+.inf", "infinity"):
        return float("inf")
    if low in ("-.inf", "-infinity"):
        return float("-inf")
    raise SerialError("Could not read NArray from YAML: unexpected scalar %r" % t)


def from_yaml(text, dtype):
    """NArray(T).new(YAML::ParseContext, node) (n_array.cr:870-911) for the
    mapping the writer produces: flow ([a, b]) or block (- a) sequences."""
    fields = {}
    key = None
    for raw in text.splitlines():
        line = raw.split(" #")[0].rstrip()
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        s = line.strip()
        if s.startswith("- "):
            if key is None or not isinstance(fields.get(key), list):
                raise SerialError("Could not read NArray from YAML: sequence item outside a key")
            fields[key].append(_yaml_scalar(s[2:]))
            continue
        if ":" not in s:
            raise SerialError("Could not read NArray from YAML: expected mapping, found %r" % s)
        key, val = s.split(":", 1)
        key, val = key.strip(), val.strip()
        if val == "":
            fields[key] = []
        elif val.startswith("[") and val.endswith("]"):
            inner = val[1:-1].strip()
            fields[key] = [_yaml_scalar(t) for t in inner.split(",")] if inner else []
        else:
            raise SerialError("Could not read NArray from YAML: Expected sequence, found %r" % val)
    return _build(fields.get("shape"), fields.get("elements"), dtype, "YAML")
