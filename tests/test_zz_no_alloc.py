"""phcu_reduce_noalloc: the reduction entry point for callers that cannot
allocate device memory (their memory is owned by another pool, or they run
where cudaMalloc is not allowed).  Its split-reduction partials live in a
static device array; the results must equal phcu_reduce's, call after call.

This file is collected last on purpose, and passes alone in a fresh process
as well as after the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reduce(lib, A, fn, op, view, axis, out):
    return getattr(lib, fn)(op, ctypes.byref(view), axis, ctypes.byref(out._view()))


CASES = [
    # (shape, op, axis): a full sum split over thousands of blocks, a split
    # column reduction, a split group argmax, an unsplit reduction
    ([1 << 22], "SUM", None),
    ([64, 1 << 16], "SUM", 0),
    ([1000, 5000], "ARGMAX", 1),
    ([37, 129, 65], "MAX", 2),
]


@pytest.mark.parametrize("shape,opname,axis", CASES)
def test_noalloc_matches_phcu_reduce_twice(cu, shape, opname, axis):
    from phase_cu import _abi as A

    lib = A.load()
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) * 3).astype(np.float32)
    X = cu.CuNArray.from_numpy(x)
    view = X.view().reverse()._cview()  # a strided input
    op = getattr(A, "RED_" + opname)
    oshape = [1] if axis is None else (shape[:axis] + shape[axis + 1:])
    odt = cu.Int32 if opname == "ARGMAX" else cu.Float32
    ax = -1 if axis is None else axis
    ref = cu.CuNArray.empty(oshape, odt)
    A.check(_reduce(lib, A, "phcu_reduce", op, view, ax, ref), "phcu_reduce")
    expected = ref.to_narr()
    mag = None
    if opname == "SUM":
        absx = cu.CuNArray.from_numpy(np.abs(x)[tuple(slice(None, None, -1) for _ in shape)].copy())
        m = cu.CuNArray.empty(oshape, cu.Float64)
        A.check(_reduce(lib, A, "phcu_reduce", op, absx._view(), ax, m), "phcu_reduce")
        mag = m.to_narr()
    for call in range(2):
        out = cu.CuNArray.empty(oshape, odt)
        A.check(_reduce(lib, A, "phcu_reduce_noalloc", op, view, ax, out), "phcu_reduce_noalloc")
        got = out.to_narr()
        if opname == "SUM":
            # tolerance of the reduction tests: 1e-6 of the sum of magnitudes
            assert np.all(np.abs(got.astype(np.float64) - expected) <= 1e-6 * mag + 1e-30), call
        else:
            assert np.array_equal(got, expected), call


def test_noalloc_rejects_reductions_beyond_its_scratch(cu):
    """A reduction whose partials exceed the static array is refused with a
    clear error (phcu_reduce, which may allocate, still handles it)."""
    from phase_cu import _abi as A

    lib = A.load()
    x = np.ones([256, 150000], dtype=np.float32)
    X = cu.CuNArray.from_numpy(x)
    out = cu.CuNArray.empty([150000], cu.Float32)
    rc = _reduce(lib, A, "phcu_reduce_noalloc", A.RED_SUM, X._view(), 0, out)
    assert rc == A.ERR_UNSUPPORTED
    assert "partials" in A.last_error()
    A.check(_reduce(lib, A, "phcu_reduce", A.RED_SUM, X._view(), 0, out))
    assert np.all(out.to_narr() == 256.0)
