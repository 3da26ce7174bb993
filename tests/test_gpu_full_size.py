"""The benchmark's workloads at their full sizes, checked against the oracle
(its multithreaded restatement of the reference loops), bit-exact except the
Float32 sums (1e-6 relative to the FP64 oracle):
- 512x512x256 Float32 and Int32: permuted and reversed gathers, + - * / on
  both view kinds (Int32 * wrapping; Int32 / Int32 -> Float64 exact), and the
  MutableView scatter;
- 64x128x128x64 Float32 lognormal: the fused chain ((x + 4) ** 2) * y - z and
  sum / max / argmax along every axis;
- 4096x4096 Float32 heat: 20 steps (five four-step launches)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = max(1, min(16, os.cpu_count() or 1))


def test_strided_views_512x512x256(cu, ora):
    from phase_cu import synth

    shape = [512, 512, 256]
    n = int(np.prod(shape))
    perm = [("permute", [2, 0, 1])]
    rev = [("region", [slice(None), cu.R(None, None, -1), slice(None)])]
    for dt in ("f32", "i32"):
        if dt == "f32":
            a = synth.uniform_f32(shape, seed=0)
            b = synth.uniform_f32(shape, seed=0, start=n)
        else:
            a = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20)
            b = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20, start=n)
        A, B = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
        for chain in (perm, rev):
            oa, ob = ora.ViewOperand(a, chain), ora.ViewOperand(b, chain)
            av, bv = A.view(), B.view()
            for t in chain:
                av = av.permute(*t[1]) if t[0] == "permute" else av.view(*t[1])
                bv = bv.permute(*t[1]) if t[0] == "permute" else bv.view(*t[1])
            assert np.array_equal(av.to_narr(), ora.gather(oa, NT)), (dt, chain)
            ops = [(ora.OP_ADD, lambda p, q: p + q), (ora.OP_SUB, lambda p, q: p - q),
                   (ora.OP_DIV, lambda p, q: p / q)]
            ops.append((ora.OP_MUL, lambda p, q: p * q) if dt == "f32" else (ora.OP_WMUL, lambda p, q: p.wmul(q)))
            for op, fn in ops:
                exp, _ = ora.map_binary(op, oa, ob, NT)
                got = fn(av, bv).to_narr()
                assert got.dtype == exp.dtype
                assert np.array_equal(got, exp, equal_nan=True), (dt, chain, op)
                del exp, got
        c = np.zeros([256, 512, 512], dtype=a.dtype)
        C = cu.CuNArray.from_numpy(c)
        M = C.mutable_view(slice(None), cu.R(None, None, -1), slice(None))
        M[slice(None), slice(None), slice(None)] = A.view().permute(2, 0, 1)
        od = ora.ViewOperand(c, [("region", [slice(None), cu.R(None, None, -1), slice(None)])])
        ora.scatter(od, ora.ViewOperand(a, perm))
        assert np.array_equal(C.to_narr(), od.arr), dt


def test_fused_chain_and_reductions_64x128x128x64(cu, ora):
    from phase_cu import synth

    shape = [64, 128, 128, 64]
    x, y, z = (synth.lognormal_f32(shape, s) for s in (0, 1, 2))
    X, Y, Z = (cu.CuNArray.from_numpy(v) for v in (x, y, z))
    R = (X.process(lambda e: (e + 4) ** 2) * Y - Z).to_cu()
    t, _ = ora.map_binary_scalar(ora.OP_ADD, x, 4, ora.I32, nthreads=NT)
    t, _ = ora.map_binary_scalar(ora.OP_POW, t, 2, ora.I32, nthreads=NT)
    t, _ = ora.map_binary(ora.OP_MUL, t, y, NT)
    t, _ = ora.map_binary(ora.OP_SUB, t, z, NT)
    assert np.array_equal(R.to_narr(), t)
    for k in range(4):
        s = R.sum(axis=k).to_narr()
        ref = ora.reduce_f64(t, k)
        assert np.max(np.abs(s - ref) / np.abs(ref)) <= 1e-6, k  # tolerance: 1e-6 relative vs FP64
        assert np.array_equal(R.max(axis=k).to_narr(), ora.reduce(ora.RED_MAX, t, k)), k
        assert np.array_equal(R.argmax(axis=k).to_narr(), ora.reduce(ora.RED_ARGMAX, t, k, ora.I32)), k
    full, ref_full = R.sum(), ora.reduce_f64(t)
    assert abs(full - ref_full) <= 1e-6 * abs(ref_full)


def test_heat_4096_twenty_steps(cu, ora):
    from phase_cu import stencil, synth

    u0 = synth.gaussian_bumps_f32(4096, 4096, bumps=16, seed=0)
    h = stencil.Heat(u0)
    h.run(20, use_graph=True)
    assert np.array_equal(h.get(), ora.heat_run(u0, 20, nthreads=NT))
