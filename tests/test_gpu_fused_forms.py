"""Fused programs made only of pre-decoded operator forms (the reduced
interpreter): every Float32 and Int32 form, operands swapped by a scalar on
the left, Int32 immediates of Float32 operators, three and four inputs,
checked Int32 overflow, on ROW (reversed view), TMA tile (permuted view) and
staged tile (permuted view of an odd shape) launches.  Each chain is checked against the oracle applied one reference
operation at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = [24, 40, 36]
# an odd innermost length: the permuted view's strides are not 16-byte
# multiples, so its tiles are staged without the Tensor Memory Accelerator
ODD_SHAPE = [24, 40, 37]


def _view(cu, X, kind):
    if kind == "reverse":
        return X.view(slice(None), cu.R(None, None, -1), slice(None))
    return X.view().permute(2, 0, 1)


def _shape(kind):
    return ODD_SHAPE if kind == "permute_odd" else SHAPE


def _host(x, kind):
    return np.ascontiguousarray(x[:, ::-1, :] if kind == "reverse" else np.transpose(x, (2, 0, 1)))


@pytest.mark.parametrize("kind", ["reverse", "permute", "permute_odd"])
def test_float32_forms(cu, ora, kind):
    rng = np.random.default_rng(2)
    a, b, c, d = [(rng.standard_normal(_shape(kind)) * 5).astype(np.float32) for _ in range(4)]
    A, B, C, D = (_view(cu, cu.CuNArray.from_numpy(x), kind) for x in (a, b, c, d))
    ha, hb, hc, hd = (_host(x, kind) for x in (a, b, c, d))
    # ((a + 3) * b - c) / d, then 2.5f - acc, then 0.75f / acc, then + a
    pv = ((((A.process(lambda e: e + 3) * B - C) / D).__rsub__(np.float32(2.5))).__rtruediv__(np.float32(0.75))) + A
    assert isinstance(pv, cu.CuProcView)
    t, _ = ora.map_binary_scalar(ora.OP_ADD, ha, 3, ora.I32)
    t, _ = ora.map_binary(ora.OP_MUL, t, hb)
    t, _ = ora.map_binary(ora.OP_SUB, t, hc)
    t, _ = ora.map_binary(ora.OP_DIV, t, hd)
    t, _ = ora.map_binary_scalar(ora.OP_SUB, t, np.float32(2.5), ora.F32, scalar_left=True)
    t, _ = ora.map_binary_scalar(ora.OP_DIV, t, np.float32(0.75), ora.F32, scalar_left=True)
    t, _ = ora.map_binary(ora.OP_ADD, t, ha)
    assert np.array_equal(pv.to_narr(), t)
    # an input on the left of a longer expression: swapped subtraction and division
    sw = D / (C - A.process(lambda e: e * 2))
    t, _ = ora.map_binary_scalar(ora.OP_MUL, ha, 2, ora.I32)
    t, _ = ora.map_binary(ora.OP_SUB, hc, t)
    t, _ = ora.map_binary(ora.OP_DIV, hd, t)
    assert np.array_equal(sw.to_narr(), t)
    # powers with an immediate exponent stay in the reduced interpreter
    pw = A.process(lambda e: (e - 1) ** 3) * B
    t, _ = ora.map_binary_scalar(ora.OP_SUB, ha, 1, ora.I32)
    t, _ = ora.map_binary_scalar(ora.OP_POW, t, 3, ora.I32)
    t, _ = ora.map_binary(ora.OP_MUL, t, hb)
    assert np.array_equal(pw.to_narr(), t)


@pytest.mark.parametrize("kind", ["reverse", "permute", "permute_odd"])
def test_int32_forms(cu, ora, kind):
    rng = np.random.default_rng(3)
    a, b, c, d = [rng.integers(-1000, 1000, _shape(kind)).astype(np.int32) for _ in range(4)]
    A, B, C, D = (_view(cu, cu.CuNArray.from_numpy(x), kind) for x in (a, b, c, d))
    ha, hb, hc, hd = (_host(x, kind) for x in (a, b, c, d))
    pv = (((((A.process(lambda e: e + 7) * B) - C).__rsub__(5)).wadd(D).wmul(B).wsub(C) & A) | B) ^ D
    t, _ = ora.map_binary_scalar(ora.OP_ADD, ha, 7, ora.I32)
    t, _ = ora.map_binary(ora.OP_MUL, t, hb)
    t, _ = ora.map_binary(ora.OP_SUB, t, hc)
    t, _ = ora.map_binary_scalar(ora.OP_SUB, t, 5, ora.I32, scalar_left=True)
    for op, y in ((ora.OP_WADD, hd), (ora.OP_WMUL, hb), (ora.OP_WSUB, hc), (ora.OP_AND, ha), (ora.OP_OR, hb),
                  (ora.OP_XOR, hd)):
        t, _ = ora.map_binary(op, t, y)
    assert np.array_equal(pv.to_narr(), t)
    # an input on the left of a longer expression: swapped checked and wrapping subtraction
    ws = B - A.process(lambda e: e * 3)
    t, _ = ora.map_binary_scalar(ora.OP_MUL, ha, 3, ora.I32)
    t, _ = ora.map_binary(ora.OP_SUB, hb, t)
    assert np.array_equal(ws.to_narr(), t)
    rw = C.wsub(A.process(lambda e: e * 3))
    t, _ = ora.map_binary_scalar(ora.OP_MUL, ha, 3, ora.I32)
    t, _ = ora.map_binary(ora.OP_WSUB, hc, t)
    assert np.array_equal(rw.to_narr(), t)


def test_int32_overflow_in_fused_chain_raises(cu, ora):
    big = np.full(SHAPE, 2 ** 30, dtype=np.int32)
    X = cu.CuNArray.from_numpy(big)
    old = cu.config.eager_errors
    cu.config.eager_errors = True
    try:
        pv = X.view().process(lambda e: e + 5) * X.view()
        with pytest.raises(OverflowError):
            pv.to_cu()
            cu.check_errors()
        # the wrapping forms never raise and equal the oracle's wrapped result
        w = X.view().process(lambda e: e + 5).wmul(X.view())
        t, st = ora.map_binary_scalar(ora.OP_ADD, big, 5, ora.I32)
        t, st2 = ora.map_binary(ora.OP_WMUL, t, big)
        assert st2 == 0
        assert np.array_equal(w.to_narr(), t)
        cu.check_errors()
    finally:
        cu.config.eager_errors = old
