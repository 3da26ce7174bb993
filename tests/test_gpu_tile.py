"""Parity of the transposing (TILE) launch shape against the oracle, at sizes
with full and partial 64x64 tiles: permuted gathers, infix operators with two
staged inputs or a staged and a direct input, fused chains, 64-bit results
and MutableView scatters.  Shapes whose strides are multiples of 16 bytes
take the tensor-map (TMA) fetch; the unaligned ones take the register /
cp.async staging; both must give the oracle's bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (base shape, permutation): full + partial tiles, a 4-axis plan, unaligned strides
CASES = [
    ([80, 72, 136], [2, 0, 1]),     # R = 136 (64 + 64 + 8), W = 72 (64 + 8), 80 batches
    ([3, 4, 24, 68], [3, 1, 0, 2]),  # two batch axes that do not merge
    ([130, 96, 64], [2, 0, 1]),     # R = 64 exactly, W = 96 (64 + 32), 130 batches
    ([40, 66, 37], [2, 0, 1]),      # a W stride of 37 elements (148 bytes): no tensor map
    ([33, 65, 12], [1, 2, 0]),      # R = 12: a single partial box
    ([5, 7, 9], [2, 0, 1]),         # too small to tile
]


def _data(rng, shape, dt):
    if dt == np.float32:
        return (rng.standard_normal(shape) * 8).astype(np.float32)
    return rng.integers(-1000, 1000, shape).astype(np.int32)


def _perm(cu, ora, x, order):
    X = cu.CuNArray.from_numpy(x)
    return X, X.view().permute(*order), ora.ViewOperand(x, [("permute", order)])


@pytest.mark.parametrize("dt", [np.float32, np.int32])
def test_permuted_gathers(cu, ora, dt):
    rng = np.random.default_rng(20)
    for shape, order in CASES:
        x = _data(rng, shape, dt)
        _, v, ov = _perm(cu, ora, x, order)
        assert np.array_equal(v.to_narr(), ora.gather(ov)), (shape, order)
    # a reversed batch axis (the tensor map walks it forwards from its last element)
    x = _data(rng, [80, 72, 136], dt)
    X = cu.CuNArray.from_numpy(x)
    lits = [cu.R(None, None, -1), slice(None), slice(None)]
    v = X.view(*lits).permute(2, 0, 1)
    ov = ora.ViewOperand(x, [("region", lits), ("permute", [2, 0, 1])])
    assert np.array_equal(v.to_narr(), ora.gather(ov))
    # a region whose first element is not 16-byte aligned
    x = _data(rng, [70, 66, 40], dt)
    X = cu.CuNArray.from_numpy(x)
    v = X.view(slice(None), slice(None), cu.R(1, None, 1)).permute(2, 0, 1)
    ov = ora.ViewOperand(x, [("region", [slice(None), slice(None), cu.R(1, None, 1)]), ("permute", [2, 0, 1])])
    assert np.array_equal(v.to_narr(), ora.gather(ov))


@pytest.mark.parametrize("dt", [np.float32, np.int32])
def test_permuted_binary_operators(cu, ora, dt):
    import phase_cu._abi as A

    rng = np.random.default_rng(21)
    ops = [A.OP_ADD, A.OP_SUB, A.OP_DIV, A.OP_MUL if dt == np.float32 else A.OP_WMUL]
    if dt == np.int32:
        ops += [A.OP_FLOORDIV, A.OP_MOD, A.OP_CMP]
    for shape, order in CASES:
        a = _data(rng, shape, dt)
        b = _data(rng, shape, dt)
        b[b == 0] = 7  # // and % by zero raise; the tile edges must not see zeros either
        _, av, oa = _perm(cu, ora, a, order)
        _, bv, ob = _perm(cu, ora, b, order)
        for op in ops:
            exp, st = ora.map_binary(op, oa, ob)
            assert st == 0
            got = av._binary(op, bv).to_narr()
            assert got.dtype == exp.dtype
            assert np.array_equal(got, exp, equal_nan=True), (shape, order, op)
        # a staged input and a direct one (contiguous in the output's order)
        c = _data(rng, av.shape, dt)
        C = cu.CuNArray.from_numpy(c)
        exp, _ = ora.map_binary(A.OP_SUB, oa, c)
        assert np.array_equal((av - C).to_narr(), exp), (shape, order)
        exp, _ = ora.map_binary(A.OP_SUB, c, oa)
        assert np.array_equal((C - av).to_narr(), exp), (shape, order)


def test_permuted_fused_chain(cu, ora):
    rng = np.random.default_rng(22)
    for shape, order in CASES:
        x = (rng.standard_normal(shape) * 2).astype(np.float32)
        y = (rng.standard_normal(shape) * 2).astype(np.float32)
        _, xv, ox = _perm(cu, ora, x, order)
        _, yv, oy = _perm(cu, ora, y, order)
        r = xv.process(lambda e: (e + 4) ** 2) * yv - xv
        t, _ = ora.map_binary_scalar(ora.OP_ADD, ox, 4, ora.I32)
        t, _ = ora.map_binary_scalar(ora.OP_POW, t, 2, ora.I32)
        t, _ = ora.map_binary(ora.OP_MUL, t, oy)
        t, _ = ora.map_binary(ora.OP_SUB, t, ox)
        assert np.array_equal(r.to_narr(), t), (shape, order)


def test_permuted_scatter(cu, ora):
    rng = np.random.default_rng(23)
    for shape, order in CASES:
        a = _data(rng, shape, np.int32)
        _, av, oa = _perm(cu, ora, a, order)
        out_shape = av.shape
        for rev in (0, 1):  # reversing output axis 0 (the R axis here) or 1 (a batch axis)
            c = np.zeros(out_shape, np.int32)
            C = cu.CuNArray.from_numpy(c)
            lits = [slice(None)] * len(out_shape)
            lits[rev] = cu.R(None, None, -1)
            M = C.mutable_view(*lits)
            M[tuple(slice(None) for _ in out_shape)] = av
            od = ora.ViewOperand(c, [("region", lits)])
            ora.scatter(od, oa)
            assert np.array_equal(C.to_narr(), od.arr), (shape, order, rev)
