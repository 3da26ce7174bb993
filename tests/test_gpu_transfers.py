"""Overlapped transfers: phcu_upload_async / phcu_download_async /
phcu_transfer_wait.  Results downloaded behind later kernels must equal the
synchronous path, and an upload must not overtake kernels that still read its
destination."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(lib, A, nbytes):
    p = ctypes.c_void_p()
    A.check(lib.phcu_host_alloc(nbytes, ctypes.byref(p)))
    return p.value


def test_pipelined_downloads_match_the_oracle(cu, ora):
    from phase_cu import _abi as A

    lib = A.load()
    shape = [64, 256, 128]
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape).astype(np.float32)
    b = rng.standard_normal(shape).astype(np.float32)
    X = cu.CuNArray.from_numpy(a)
    Y = cu.CuNArray.from_numpy(b)
    ops = [A.OP_ADD, A.OP_SUB, A.OP_MUL, A.OP_DIV] * 3
    xv = X.view().permute(2, 0, 1)._cview()
    yv = Y.view(slice(None), cu.R(None, None, -1), slice(None)).permute(2, 0, 1)._cview()
    outs, hosts = [], []
    nbytes = a.nbytes
    for op in ops:
        o = cu.CuNArray.empty([128, 64, 256], cu.Float32)
        A.check(lib.phcu_binary(op, ctypes.byref(xv), ctypes.byref(yv), ctypes.byref(o._view())))
        h = _pinned(lib, A, nbytes)
        A.check(lib.phcu_download_async(h, o._buf.ptr, nbytes))
        outs.append(o)
        hosts.append(h)
    A.check(lib.phcu_transfer_wait())
    at = np.ascontiguousarray(np.transpose(a, (2, 0, 1)))
    bt = np.ascontiguousarray(np.transpose(b[:, ::-1, :], (2, 0, 1)))
    for op, h in zip(ops, hosts):
        got = np.frombuffer((ctypes.c_char * nbytes).from_address(h), dtype=np.float32).reshape(128, 64, 256)
        exp, _ = ora.map_binary(op, at, bt)
        assert np.array_equal(got, exp)
        lib.phcu_host_free(h)


def test_upload_waits_for_kernels_reading_its_destination(cu):
    from phase_cu import _abi as A

    lib = A.load()
    n = 1 << 24
    first = np.arange(n, dtype=np.int32)
    second = np.full(n, 7, dtype=np.int32)
    X = cu.CuNArray.from_numpy(first)
    hs = _pinned(lib, A, second.nbytes)
    ctypes.memmove(hs, second.ctypes.data, second.nbytes)
    outs = []
    for _ in range(4):  # several kernels read X before the upload replaces it
        o = cu.CuNArray.empty([n], cu.Int32)
        A.check(lib.phcu_binary(A.OP_WADD, ctypes.byref(X._view()), ctypes.byref(X._view()),
                                ctypes.byref(o._view())))
        outs.append(o)
    A.check(lib.phcu_upload_async(X._buf.ptr, hs, second.nbytes))
    after = cu.CuNArray.empty([n], cu.Int32)
    A.check(lib.phcu_binary(A.OP_WADD, ctypes.byref(X._view()), ctypes.byref(X._view()), ctypes.byref(after._view())))
    A.check(lib.phcu_transfer_wait())
    for o in outs:
        assert np.array_equal(o.to_narr(), first + first)
    assert np.array_equal(after.to_narr(), second + second)
    lib.phcu_host_free(hs)
