"""The C++ host mirror (ph-core_gb300/host/phase.hpp): its RangeSyntax /
IndexRegion canonicalisation against the reference's TestRanges and region
KATs, and against the Python mirror (itself pinned by those KATs) on 3,000
random region literals.  Host logic only: compiled with g++, no GPU."""
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


def _encode(bound, lits):
    parts = [str(len(bound))] + [str(b) for b in bound] + [str(len(lits))]
    for x in lits:
        if isinstance(x, int):
            parts += ["I", str(x)]
        else:
            parts += ["R", _tok(x.first), _tok(x.last), _tok(x.step), "1" if x.exclusive else "0"]
    return " ".join(parts)


def _python(bound, lits):
    try:
        r = reg.IndexRegion.new(lits, bound)
    except DimensionError:
        return "ERR DimensionError"
    except IndexError:
        return "ERR IndexError"
    axes = " ".join("%d %d %d %d" % t for t in zip(r.first, r.step, r.last, r.proper_shape))
    return "OK %d %s | %s" % (len(r.shape), " ".join(str(v) for v in r.shape), axes)


def _run(exe, cases):
    text = "\n".join(_encode(b, l) for b, l in cases) + "\n"
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


def test_region_multi_axis_kat(exe, kats):
    k = kats["region_multi_axis"]
    o = _run(exe, [(k["bound"], [_lit(x) for x in k["literal"]]),
                   (k["bound"], [_lit(x) for x in k["bad_literal"]])])
    axes = " ".join("%d %d %d %d" % t for t in zip(k["first"], k["step"], k["last"], k["shape"]))
    assert o[0] == "OK 2 %s | %s" % (" ".join(map(str, k["shape"])), axes)
    assert o[1] == "ERR IndexError"


def test_random_literals_match_the_python_mirror(exe):
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
        cases.append((bound, lits))
    out = _run(exe, cases)
    for (bound, lits), o in zip(cases, out):
        assert o == " ".join(_python(bound, lits).split()), (bound, lits, o)
