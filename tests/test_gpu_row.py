"""Parity of the ROW launch shape (operands sharing a unit-stride inner axis)
against the oracle: row lengths that do and do not divide the vector width,
reversed row and batch axes, one long merged row, every element size on input
and output (Bool, 4- and 8-byte, and mixed), and fused programs with several
inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (base shape, region literal builder): the inner axis kept whole and forward
CASES = [
    ([6, 37, 300], lambda R: [slice(None), R(None, None, -1), slice(None)]),    # W = 300
    ([512, 64], lambda R: [R(None, None, -1), slice(None)]),                     # row axis reversed
    ([3, 5, 9, 256], lambda R: [R(None, None, -1), slice(None), R(None, None, -2), slice(None)]),
    ([2, 4, 3, 40], lambda R: [slice(None), R(1, None, 1), slice(None), slice(None)]),  # offset start
    ([70000], lambda R: [slice(None)]),                                          # one long row
    ([4, 65536], lambda R: [slice(None), slice(None)]),                          # merges into one row
    ([33, 9], lambda R: [R(None, None, -1), slice(None)]),                       # W = 9: scalar accesses
]


def _data(rng, shape, dt):
    if dt == np.bool_:
        return rng.integers(0, 2, shape).astype(np.bool_)
    if np.issubdtype(dt, np.integer):
        return rng.integers(-1000, 1000, shape).astype(dt)
    return (rng.standard_normal(shape) * 8).astype(dt)


@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64, np.int64, np.bool_])
def test_row_gathers(cu, ora, dt):
    rng = np.random.default_rng(61)
    for shape, lits in CASES:
        x = _data(rng, shape, dt)
        X = cu.CuNArray.from_numpy(x)
        L = lits(cu.R)
        v = X.view(*L)
        ov = ora.ViewOperand(x, [("region", L)])
        assert np.array_equal(v.to_narr(), ora.gather(ov)), (shape, dt)


@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64, np.int64])
def test_row_binary_operators(cu, ora, dt):
    import phase_cu._abi as A

    rng = np.random.default_rng(62)
    ops = [A.OP_ADD, A.OP_SUB, A.OP_DIV, A.OP_GT, A.OP_EQ]
    ops.append(A.OP_MUL if np.issubdtype(dt, np.floating) else A.OP_WMUL)
    for shape, lits in CASES:
        a = _data(rng, shape, dt)
        b = _data(rng, shape, dt)
        if np.issubdtype(dt, np.integer):
            b[b == 0] = 3
        L = lits(cu.R)
        av = cu.CuNArray.from_numpy(a).view(*L)
        bv = cu.CuNArray.from_numpy(b).view(*L)
        oa = ora.ViewOperand(a, [("region", L)])
        ob = ora.ViewOperand(b, [("region", L)])
        for op in ops:
            exp, st = ora.map_binary(op, oa, ob)
            assert st == 0
            got = av._binary(op, bv).to_narr()
            assert got.dtype == exp.dtype
            assert np.array_equal(got, exp, equal_nan=True), (shape, op, dt)


def test_row_bool_and_mixed_programs(cu, ora):
    import phase_cu._abi as A

    rng = np.random.default_rng(63)
    for shape, lits in CASES:
        L = lits(cu.R)
        p = _data(rng, shape, np.bool_)
        q = _data(rng, shape, np.bool_)
        pv = cu.CuNArray.from_numpy(p).view(*L)
        qv = cu.CuNArray.from_numpy(q).view(*L)
        op_, oq = ora.ViewOperand(p, [("region", L)]), ora.ViewOperand(q, [("region", L)])
        for op in (A.OP_AND, A.OP_XOR, A.OP_EQ):
            exp, _ = ora.map_binary(op, op_, oq)
            assert np.array_equal(pv._binary(op, qv).to_narr(), exp), (shape, op)
        # Float32 x Float64 mix and a three-input fused chain
        x = _data(rng, shape, np.float32)
        y = _data(rng, shape, np.float64)
        z = _data(rng, shape, np.float32)
        xv, yv, zv = (cu.CuNArray.from_numpy(t).view(*L) for t in (x, y, z))
        ox, oy, oz = (ora.ViewOperand(t, [("region", L)]) for t in (x, y, z))
        exp, _ = ora.map_binary(A.OP_MUL, ox, oy)
        assert np.array_equal((xv * yv).to_narr(), exp), shape
        r = xv.process(lambda e: (e + 4) ** 2) * zv - xv
        t, _ = ora.map_binary_scalar(ora.OP_ADD, ox, 4, ora.I32)
        t, _ = ora.map_binary_scalar(ora.OP_POW, t, 2, ora.I32)
        t, _ = ora.map_binary(ora.OP_MUL, t, oz)
        t, _ = ora.map_binary(ora.OP_SUB, t, ox)
        assert np.array_equal(r.to_narr(), t), shape
