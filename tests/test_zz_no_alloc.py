"""phcu_reduce_noalloc: the reduction entry point for callers that cannot
allocate device memory (their device memory belongs to another pool, or they
run where cudaMalloc must not be called).  Its split-reduction partials live
in a static device array.  Its results must equal phcu_reduce's and the
oracle's, call after call, and no call may take memory from the device's
stream-ordered pool (the pool phcu_reduce's scratch comes from).

This file is collected last on purpose, and passes alone in a fresh process
as well as after the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# cuMemPoolGetAttribute / cuMemPoolSetAttribute attributes (cuda.h)
CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7
CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8


class _Pool:
    """The default memory pool of device 0, read through the driver API: the
    pool the library's cudaMallocAsync scratch comes from."""

    def __init__(self):
        self.drv = ctypes.CDLL("libcuda.so.1")
        self.pool = ctypes.c_void_p()
        rc = self.drv.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), ctypes.c_int(0))
        assert rc == 0, "cuDeviceGetDefaultMemPool: %d" % rc

    def get(self, attr):
        v = ctypes.c_uint64()
        rc = self.drv.cuMemPoolGetAttribute(self.pool, ctypes.c_int(attr), ctypes.byref(v))
        assert rc == 0, "cuMemPoolGetAttribute: %d" % rc
        return v.value

    def reset_high(self):
        z = ctypes.c_uint64(0)  # the high watermark can only be reset to zero
        rc = self.drv.cuMemPoolSetAttribute(self.pool, ctypes.c_int(CU_MEMPOOL_ATTR_USED_MEM_HIGH), ctypes.byref(z))
        assert rc == 0, "cuMemPoolSetAttribute: %d" % rc


def _reduce(lib, fn, op, view, axis, out):
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
def test_noalloc_matches_phcu_reduce_and_oracle_twice(cu, ora, shape, opname, axis):
    from phase_cu import _abi as A

    lib = A.load()
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) * 3).astype(np.float32)
    X = cu.CuNArray.from_numpy(x)
    view = X.view().reverse()._cview()  # a strided input: every axis reversed
    xr = np.ascontiguousarray(x[tuple(slice(None, None, -1) for _ in shape)])
    op = getattr(A, "RED_" + opname)
    oshape = [1] if axis is None else (shape[:axis] + shape[axis + 1:])
    odt = cu.Int32 if opname == "ARGMAX" else cu.Float32
    ax = -1 if axis is None else axis
    ref = cu.CuNArray.empty(oshape, odt)
    A.check(_reduce(lib, "phcu_reduce", op, view, ax, ref), "phcu_reduce")
    expected = ref.to_narr()
    if opname == "SUM":
        exact = np.asarray(ora.reduce_f64(xr, axis), dtype=np.float64).reshape(oshape)
        mag = np.asarray(ora.reduce_f64(np.abs(xr), axis), dtype=np.float64).reshape(oshape)
    else:
        rop = ora.RED_ARGMAX if opname == "ARGMAX" else ora.RED_MAX
        exact = np.asarray(ora.reduce(rop, xr, axis, ora.I32 if opname == "ARGMAX" else None)).reshape(oshape)
    outs = [cu.CuNArray.empty(oshape, odt) for _ in range(2)]  # allocated before the pool is watched
    A.call("phcu_sync")
    pool = _Pool()
    used_before = pool.get(CU_MEMPOOL_ATTR_USED_MEM_CURRENT)
    pool.reset_high()
    for call, out in enumerate(outs):
        A.check(_reduce(lib, "phcu_reduce_noalloc", op, view, ax, out), "phcu_reduce_noalloc")
    A.call("phcu_sync")
    assert pool.get(CU_MEMPOOL_ATTR_USED_MEM_HIGH) <= used_before, "the pool grew during phcu_reduce_noalloc"
    for call, out in enumerate(outs):
        got = out.to_narr()
        if opname == "SUM":
            # tolerance of the reduction tests: 1e-6 of the sum of magnitudes
            # (the FP64 oracle), and phcu_reduce's result within the same bound
            assert np.all(np.abs(got.astype(np.float64) - exact) <= 1e-6 * mag + 1e-30), call
            assert np.all(np.abs(got.astype(np.float64) - expected) <= 1e-6 * mag + 1e-30), call
        else:
            assert np.array_equal(got, exact), call
            assert np.array_equal(got, expected), call


def test_noalloc_rejects_reductions_beyond_its_scratch(cu):
    """A reduction whose partials exceed the static array is refused with a
    clear error (phcu_reduce, which may allocate, still handles it).  The
    shape is derived from the device: a column reduction of O < sm_count*1024
    outputs splits its reduced axis into ceil(sm_count*1024 / O) parts."""
    from phase_cu import _abi as A

    lib = A.load()
    sm = ctypes.c_int32()
    l2 = ctypes.c_int64()
    smem = ctypes.c_int32()
    clk = ctypes.c_int32()
    A.check(lib.phcu_device_info(ctypes.byref(sm), ctypes.byref(l2), ctypes.byref(smem), ctypes.byref(clk)))
    target = sm.value * 1024
    O = target - 1  # two splits of the reduced axis
    if 2 * O <= (1 << 18):
        pytest.skip("a device with %d SMs never needs more than 2^18 partials in this shape" % sm.value)
    K = 256
    X = cu.CuNArray.from_numpy(np.ones([K, O], dtype=np.float32))
    out = cu.CuNArray.empty([O], cu.Float32)
    rc = _reduce(lib, "phcu_reduce_noalloc", A.RED_SUM, X._view(), 0, out)
    assert rc == A.ERR_UNSUPPORTED
    assert "partials" in A.last_error()
    A.check(_reduce(lib, "phcu_reduce", A.RED_SUM, X._view(), 0, out))
    assert np.all(out.to_narr() == float(K))
