"""The C++ host mirror (ph-core_gb300/host/phase.hpp): its RangeSyntax /
IndexRegion logic (canonicalisation, absolute regions, fits_in?, trim!,
reverse!, translate!, includes?, local_to_absolute) against the reference's
TestRanges and IndexRegion KATs, and against the Python mirror (itself pinned
by those KATs) on 3,000 random regions and operations; its affine reshape of
views against the Python mirror's on 4,000 random layouts.  Host logic only:
compiled with g++, no GPU."""
import os
import random
import shutil
import subprocess

import pytest

from phase_cu import region as reg
from phase_cu.errors import DimensionError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("hostcpp") / "host_cpp_regions")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-o", out, os.path.join(ROOT, "tests", "host_cpp_regions.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "host")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def _tok(v):
    return "n" if v is None else str(int(v))


def _ints(v):
    return [str(len(v))] + [str(int(x)) for x in v]


def _encode(bound, lits, op=("none",)):
    """bound None = an absolute region (no bounding shape)."""
    parts = ["A"] if bound is None else ["N", str(len(bound))] + [str(b) for b in bound]
    parts.append(str(len(lits)))
    for x in lits:
        if isinstance(x, int):
            parts += ["I", str(x)]
        else:
            parts += ["R", _tok(x.first), _tok(x.last), _tok(x.step), "1" if x.exclusive else "0"]
    parts.append(op[0])
    if len(op) > 1:
        parts += _ints(op[1])
    return " ".join(parts)


def _region_text(r):
    axes = " ".join("%d %d %d %d" % t for t in zip(r.first, r.step, r.last, r.proper_shape))
    return "OK %d %s | %s" % (len(r.shape), " ".join(str(v) for v in r.shape), axes)


def _python(bound, lits, op=("none",)):
    try:
        r = reg.IndexRegion.absolute(lits) if bound is None else reg.IndexRegion.new(lits, bound)
        if op[0] == "fits":
            return "BOOL %d" % r.fits_in(op[1])
        if op[0] == "incl":
            return "BOOL %d" % r.includes(op[1])
        if op[0] == "l2a":
            return "COORD " + " ".join(str(v) for v in r.local_to_absolute(op[1]))
        if op[0] == "trim":
            r.trim(op[1])
        elif op[0] == "rev":
            r.reverse()
        elif op[0] == "trans":
            r.translate(op[1])
        return _region_text(r)
    except DimensionError:
        return "ERR DimensionError"
    except IndexError:
        return "ERR IndexError"
    except ValueError:
        return "ERR ArgumentError"


def _run(exe, cases):
    text = "\n".join(_encode(*c) for c in cases) + "\n"
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    assert len(out) == len(cases)
    return [" ".join(o.split()) for o in out]


def _lit(x):
    return x["i"] if "i" in x else reg.R(x["f"], x["l"], x["s"], x["x"])


def test_test_ranges_kats(exe, kats):
    tr = kats["test_ranges"]
    b = tr["bound"]
    good = [(lit, exp) for key in ("fully_defined", "negative_indices", "implicit_bounds") for lit, exp in tr[key]]
    out = _run(exe, [([b], [_lit(lit)]) for lit, _ in good])
    for (lit, (f, s, l)), o in zip(good, out):
        size = (l - f) // s + 1
        assert o == "OK 1 %d | %d %d %d %d" % (size, f, s, l, size), (lit, o)
    bad = tr["out_of_bounds"] + tr["step_conflict"]
    assert all(o == "ERR IndexError" for o in _run(exe, [([b], [_lit(lit)]) for lit in bad]))
    for o in _run(exe, [([b], [_lit(lit)]) for lit in tr["empty"]]):
        assert o.startswith("OK 1 0 |"), o
    # absolute regions (spec/spec_helper.cr TestRanges without a bound)
    out = _run(exe, [(None, [_lit(lit)]) for lit, _ in tr["fully_defined"]])
    for (lit, (f, s, l)), o in zip(tr["fully_defined"], out):
        assert o.split("|")[1].split()[:3] == [str(f), str(s), str(l)], (lit, o)
    assert all(o.startswith("ERR") for o in _run(exe, [(None, [_lit(lit)]) for lit, _ in tr["implicit_bounds"]]))
    assert all(o == "ERR IndexError" for o in _run(exe, [(None, [_lit(lit)]) for lit, _ in tr["negative_indices"]]))


def test_index_region_kats(exe, kats):
    k = kats["region_multi_axis"]
    o = _run(exe, [(k["bound"], [_lit(x) for x in k["literal"]]), (k["bound"], [_lit(x) for x in k["bad_literal"]])])
    axes = " ".join("%d %d %d %d" % t for t in zip(k["first"], k["step"], k["last"], k["shape"]))
    assert o[0] == "OK 2 %s | %s" % (" ".join(map(str, k["shape"])), axes)
    assert o[1] == "ERR IndexError"
    k = kats["region_absolute"]
    o = _run(exe, [(None, [_lit(x) for x in k["literal"]])])[0]
    axes = " ".join("%d %d %d %d" % t for t in zip(k["first"], k["step"], k["last"], k["shape"]))
    assert o == "OK 2 %s | %s" % (" ".join(map(str, k["shape"])), axes)
    k = kats["region_includes"]
    lits = [_lit(x) for x in k["literal"]]
    assert all(o == "BOOL 1" for o in _run(exe, [(None, lits, ("incl", c)) for c in k["included"]]))
    assert all(o == "BOOL 0" for o in _run(exe, [(None, lits, ("incl", c)) for c in k["excluded"]]))
    k = kats["region_fits_in"]
    lits = [_lit(x) for x in k["literal"]]
    assert all(o == "BOOL 1" for o in _run(exe, [(None, lits, ("fits", b)) for b in k["fits"]]))
    assert all(o == "BOOL 0" for o in _run(exe, [(None, lits, ("fits", b)) for b in k["not_fits"]]))
    k = kats["region_translate"]
    lits = [_lit(x) for x in k["literal"]]
    base, moved = _run(exe, [(None, lits), (None, lits, ("trans", k["offset"]))])
    firsts = lambda o: [int(v) for v in o.split("|")[1].split()[0::4]]  # noqa: E731
    assert firsts(moved) == [f + d for f, d in zip(firsts(base), k["offset"])]
    assert all(o == "ERR IndexError" for o in _run(exe, [(None, lits, ("trans", off)) for off in k["raises"]]))
    k = kats["region_reverse"]
    o = _run(exe, [(None, [_lit(x) for x in k["literal"]], ("rev",))])[0]
    assert firsts(o) == k["first_after"]


def test_random_regions_and_operations_match_the_python_mirror(exe):
    rnd = random.Random(5)
    cases = []
    for _ in range(3000):
        rank = rnd.randint(1, 4)
        bound = [rnd.randint(0, 12) for _ in range(rank)]
        lits = []
        for a in range(rnd.randint(0, rank + (1 if rnd.random() < 0.05 else 0))):
            if rnd.random() < 0.25:
                lits.append(rnd.randint(-14, 14))
            else:
                pick = lambda: None if rnd.random() < 0.3 else rnd.randint(-14, 14)  # noqa: E731
                step = None if rnd.random() < 0.4 else rnd.choice([-3, -2, -1, 1, 2, 3])
                lits.append(reg.R(pick(), pick(), step, rnd.random() < 0.3))
        kind = rnd.choice(["none", "rev", "trim", "trans", "incl", "fits", "l2a"])
        n = rank if rnd.random() < 0.9 else rank + 1
        if kind in ("trim", "fits"):
            op = (kind, [rnd.randint(0, 14) for _ in range(n)])
        elif kind == "trans":
            op = (kind, [rnd.randint(-4, 4) for _ in range(rank)])
        elif kind == "incl":
            op = (kind, [rnd.randint(-1, 13) for _ in range(n)])
        elif kind == "l2a":
            try:
                shape = reg.IndexRegion.new(lits, bound).shape
            except (IndexError, DimensionError):
                shape = []
            if not shape or min(shape) == 0:
                op = ("none",)
            else:
                op = (kind, [rnd.randint(0, s - 1) for s in shape])
        else:
            op = (kind,)
        cases.append((bound, lits, op))
    out = _run(exe, cases)
    for (bound, lits, op), o in zip(cases, out):
        assert o == " ".join(_python(bound, lits, op).split()), (bound, lits, op, o)


def test_affine_reshape_matches_python_mirror(tmp_path):
    """View#reshape as strides (the C++ mirror's affine_reshape) gives the
    Python mirror's answer on random layouts: row-major arrays seen through
    random regions with steps, reversals and permutations, reshaped to random
    factorisations of their element count (some expressible with strides,
    some not).  Where both give strides, the lexicographic element addresses
    of the new view equal those of the old one."""
    import itertools

    import numpy as np

    from phase_cu import narray

    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "host_cpp_reshape")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-o", exe, os.path.join(ROOT, "tests", "host_cpp_reshape.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "host")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    rng = random.Random(11)

    def factorisation(n, rank):
        dims = []
        for _ in range(rank - 1):
            divs = [d for d in range(1, n + 1) if n % d == 0]
            d = rng.choice(divs)
            dims.append(d)
            n //= d
        dims.append(n)
        rng.shuffle(dims)
        return dims

    def addresses(off, shape, stride):
        return [off + sum(c * s for c, s in zip(idx, stride)) for idx in itertools.product(*map(range, shape))]

    cases = []
    for _ in range(4000):
        base = [rng.randint(1, 6) for _ in range(rng.randint(1, 4))]
        st = narray._row_major(base)
        off, shape, stride = 0, [], []
        for n, s in zip(base, st):  # a region with a step, maybe reversed
            step = rng.choice([1, 1, 1, 2, 3])
            k = (n - 1) // step + 1
            if rng.random() < 0.3:
                off += (n - 1) * s
                shape.append(k)
                stride.append(-step * s)
            else:
                shape.append(k)
                stride.append(step * s)
        perm = list(range(len(shape)))
        if rng.random() < 0.4:
            rng.shuffle(perm)
        shape = [shape[p] for p in perm]
        stride = [stride[p] for p in perm]
        n = int(np.prod(shape))
        new = factorisation(n, rng.randint(1, 4))
        cases.append((off, shape, stride, new))
    lines = []
    for off, shape, stride, new in cases:
        lines.append(" ".join(map(str, [off, len(shape)] + shape + stride + [len(new)] + new)))
    p = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    out = p.stdout.splitlines()
    assert len(out) == len(cases)
    affine = 0
    for (off, shape, stride, new), got in zip(cases, out):
        exp = narray._affine_reshape(off, shape, stride, new)
        if exp is None:
            assert got == "NONE", (off, shape, stride, new, got)
            continue
        eoff, _, est = exp
        assert got == "OK " + " ".join(str(int(v)) for v in [eoff] + list(est)), (off, shape, stride, new, got)
        assert addresses(eoff, new, est) == addresses(off, shape, stride)
        affine += 1
    assert 1000 < affine < len(cases)  # both outcomes are exercised
