"""The C++ host mirror's fused expressions (ph-core_gb300/host/phase.hpp: Sym,
CuProcView and its program compiler) hand the device the same programs as
the Python mirror's compile_program: instruction by instruction, immediates
bit for bit, on fixed chains (the fused chain, stash use, Crystal's result
types, checked and wrapping integer operators) and 4,000 random expression
trees; CuProcView's operand views (sharing, index transforms) against
hand-computed layouts; the documented public surface compiles without
warnings.  Host logic only: compiled with g++, no GPU."""
import os
import random
import shutil
import subprocess

import numpy as np
import pytest

from phase_cu import _abi as A
from phase_cu import narray as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F32, F64, I32, I64 = A.F32, A.F64, A.I32, A.I64
f32 = np.float32


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("hostcpp_prog") / "host_cpp_programs")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-o", out, os.path.join(ROOT, "tests", "host_cpp_programs.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "host")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def _run(exe, mode, text=""):
    p = subprocess.run([exe, mode], input=text, capture_output=True, text=True, check=True)
    return [" ".join(o.split()) for o in p.stdout.splitlines()]


def _fmt(prog, raises):
    body = "".join(" %d %d %d %d %d %d;" % (c.op, c.src, c.type, c.btype, c.flags, c.imm.i)
                   for c in prog.code[:prog.n_instr])
    return " ".join(("P %d %d %d |%s" % (raises, prog.n_instr, prog.out_type, body)).split())


def _python(sym, out=None):
    try:
        prog, raises = N.compile_program(sym.expr, sym.dtype if out is None else out)
        return _fmt(prog, raises)
    except NotImplementedError:
        return "ERR NotImplementedError"


def _sym(slot, t):
    return N._Sym(("in", slot, t), t)


def test_fixed_expressions_match_the_python_compiler(exe):
    x, y, z, w = (_sym(k, F32) for k in range(4))
    a, b = _sym(0, I32), _sym(1, I32)
    d, l = _sym(2, F64), _sym(3, I64)
    expected = [
        (x + 4) ** 2 * y - z,
        (x + y + z - w * 4) * f32(0.2),
        a / b,
        a * f32(0.5) + x,
        x * y - z * w,
        (x * y - z * w) * ((x + y) - (z + w)),
        7 - x * 3,
        -a + b,
        x ** 3,
        a ** x,
        a ** b,
        a._bin(A.OP_WPOW, 3),
        a._bin(A.OP_WADD, b) - a._bin(A.OP_WMUL, 5),
        (a // 3) % 7,
        (a & b) ^ (a | 12),
        d * x + 1.5,
        l + a,
        a + l,
        x / f32(0.0),
        x % f32(2.5),
        (x * y) ** (z - w),
        2 - (x - (y - (z - w))),
        ((x * y - z * w) * (x - y * z)) - ((x + y) * (z - w * x)),
    ]
    out = _run(exe, "sym")
    assert len(out) == len(expected)
    for k, (e, o) in enumerate(zip(expected, out)):
        assert o == _python(e), (k, o)
    assert out[-1] == "ERR NotImplementedError"  # three nested stashes
    assert out[0].split("|")[1].split(";")[2].split() == ["6", "8", "3", "1", "0", "2"]  # ** Int32 2 in Float32


def test_proc_view_chains(exe):
    out = _run(exe, "proc")
    x, y, z = _sym(0, F32), _sym(1, F32), _sym(2, F32)
    chain = _python((x + 4) ** 2 * y - z)
    assert out[0:4] == [chain, "L 0 4 3 2 : 6 2 1", "L 1000 4 3 2 : 6 2 1", "L 2000 4 3 2 : 6 2 1"]
    # permute(2, 0, 1) then reverse axis 1: the program is unchanged, every operand view moves
    assert out[4:8] == [chain, "L 18 2 4 3 : 1 -6 2", "L 1018 2 4 3 : 1 -6 2", "L 2018 2 4 3 : 1 -6 2"]
    x0 = _sym(0, F32)
    assert out[8:10] == [_python(x0 * x0 + x0), "L 0 4 3 2 : 6 2 1"]  # one operand view, one slot
    x1 = _sym(1, F32)
    assert out[10:13] == [_python((x0 - x1) * (x1 - x0)), "L 0 4 3 2 : 6 2 1", "L 1000 4 3 2 : 6 2 1"]
    a0 = _sym(0, I32)
    assert out[13:16] == [_python(a0 * 2 / a0 + x1), "L 3000 4 3 2 : 6 2 1", "L 0 4 3 2 : 6 2 1"]
    const = N._Sym(("const", f32(1.5), F32), F32)
    assert out[16:18] == [_python(const), "L 0 4 3 2 : 6 2 1"]
    assert out[18:20] == [_python(-(a0 * 3)), "L 3000 4 3 2 : 6 2 1"]
    assert out[20:23] == [_python(x0 + x1), "L 6 3 2 : 2 1", "L 1012 3 2 : 2 1"]  # x[1] + y[2]
    assert out[23:25] == [_python(x0 * 2.0), "L 23 4 3 2 : -6 -2 -1"]
    assert out[25] == ("ERR ShapeError The shape of this MultiIndexable ([4, 3, 2]) does not match the shape of "
                       "the one provided ([3, 3, 2]), so '+' cannot be applied element-wise.")
    assert out[26] == "N 5"
    assert len(out) == 27


_OPS = [A.OP_ADD, A.OP_SUB, A.OP_MUL, A.OP_DIV, A.OP_FLOORDIV, A.OP_MOD, A.OP_POW,
        A.OP_WADD, A.OP_WSUB, A.OP_WMUL, A.OP_WPOW, A.OP_AND, A.OP_OR, A.OP_XOR]
_TYPES = [I32, I64, F32, F64]


def _random_tree(rnd, depth):
    """(prefix text for the C++ driver, expression tuple for compile_program)."""
    if depth == 0 or rnd.random() < (0.3 if depth < 3 else 0.05):
        t = rnd.choice(_TYPES)
        if rnd.random() < 0.6:
            k = rnd.randrange(4)
            return "i %d %d" % (k, t), ("in", k, t)
        if t == I32:
            v = rnd.randint(-2 ** 31, 2 ** 31 - 1) if rnd.random() < 0.3 else rnd.randint(-9, 9)
            return "c %d %d" % (t, v), ("const", v, t)
        if t == I64:
            v = rnd.randint(-2 ** 63, 2 ** 63 - 1) if rnd.random() < 0.5 else rnd.randint(-9, 9)
            return "c %d %d" % (t, v), ("const", v, t)
        v = rnd.choice([0.0, -0.0, 0.5, 3.0, 1e-30, float("inf")]) if rnd.random() < 0.3 else rnd.uniform(-1e3, 1e3)
        if t == F32:
            v = f32(v)
        return "c %d %s" % (t, float(v).hex()), ("const", v, t)
    if rnd.random() < 0.15:
        s, e = _random_tree(rnd, depth - 1)
        return "u %d %s" % (A.I_NEG, s), ("un", A.I_NEG, e, N._etype(e))
    op = rnd.choice(_OPS) if rnd.random() < 0.4 else rnd.choice(_OPS[:7])
    sl, el = _random_tree(rnd, depth - 1)
    sr, er = _random_tree(rnd, depth - 1)
    ta, tb = N._etype(el), N._etype(er)
    try:
        t = N.result_dtype(op, ta, tb)
    except NotImplementedError:
        t = None
    return "b %d %s %s" % (op, sl, sr), ("bin", op, el, er, ta, tb, t)


def _valid(e):
    if e[0] == "bin":
        return e[6] is not None and _valid(e[2]) and _valid(e[3])
    if e[0] == "un":
        return _valid(e[2])
    return True


def test_random_expressions_match_the_python_compiler(exe):
    rnd = random.Random(11)
    lines, expected = [], []
    for _ in range(4000):
        text, e = _random_tree(rnd, rnd.randint(0, 6))
        out_t = N._etype(e) if rnd.random() < 0.7 or not _valid(e) else rnd.choice(_TYPES)
        lines.append("%d %s" % (-1 if out_t is None else out_t, text))
        if not _valid(e):
            expected.append("ERR NotImplementedError")
            continue
        try:
            prog, raises = N.compile_program(e, out_t)
            expected.append(_fmt(prog, raises))
        except NotImplementedError:
            expected.append("ERR NotImplementedError")
    out = _run(exe, "expr", "\n".join(lines) + "\n")
    assert len(out) == len(expected)
    for line, o, x in zip(lines, out, expected):
        assert o == x, line
    kinds = {x.split()[0] + ("" if x.startswith("ERR") else str(min(int(x.split()[2]), 8))) for x in expected}
    assert {"ERR", "P1", "P4", "P8"} <= kinds, kinds  # errors, single loads and long programs all occur
    assert sum(" 66 0 " in x for x in expected) > 50  # second stash register used


@pytest.mark.parametrize("std", ["c++17", "c++20"])
def test_public_surface_compiles_without_warnings(std):
    """tests/host_cpp_api.cpp uses the C++ host mirror's public surface as a
    caller does; its static assertions pin Crystal's result types of fused
    chains."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    cmd = [gxx, "-std=" + std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
           os.path.join(ROOT, "tests", "host_cpp_api.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "host")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
