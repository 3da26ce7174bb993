"""Overlapping writes on the device: a source (or an in-place map's operand)
that aliases its destination gives the reference's result whenever the
reference's element-by-element order (src/multi_writable.cr:29-44,
src/multi_indexable/mutable.cr:54-67) reads no element it already wrote,
checked against the oracle's sequential scatter; the other cases raise."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _seq_scatter(ora, cu, arr, dst_lits, src_lits):
    seq = arr.copy()
    ora.scatter(ora.ViewOperand(seq, [("region", dst_lits)]), ora.ViewOperand(seq, [("region", src_lits)]))
    return seq


def test_set_chunk_with_an_aliasing_source(cu, ora):
    R = cu.R
    a = np.arange(100, 100 + 6 * 9, dtype=np.int32).reshape(6, 9)
    all_ = slice(None)
    # the source ahead of the destination: the reference's result
    for dst, src in (([R(0, 3), all_], [R(2, 5), all_]),
                     ([all_, R(0, 5)], [all_, R(3, 8)]),
                     ([R(0, 4, 2), all_], [R(1, 5, 2), all_])):
        C = cu.CuNArray.from_numpy(a)
        C[tuple(dst)] = C.view(*src)
        assert np.array_equal(C.to_narr(), _seq_scatter(ora, cu, a, dst, src)), (dst, src)
    # behind, reversed in place, transposed in place: refused
    C = cu.CuNArray.from_numpy(a)
    with pytest.raises(NotImplementedError):
        C[R(2, 5), all_] = C.view(R(0, 3), all_)
    with pytest.raises(NotImplementedError):
        C[all_, all_] = C.view(all_, R(None, None, -1))
    S = cu.CuNArray.from_numpy(a[:, :6].copy())
    with pytest.raises(NotImplementedError):
        S[all_, all_] = S.view().permute(1, 0)
    with pytest.raises(NotImplementedError):  # a lazy source reading the rows it writes
        C[R(1, 5), all_] = C.view(R(0, 4), all_).process(lambda e: e * 2)
    assert np.array_equal(C.to_narr(), a)  # nothing was written by the refused calls


def test_in_place_map_with_an_aliasing_operand(cu, ora):
    R = cu.R
    a = np.arange(1, 1 + 64, dtype=np.int32)
    X = cu.CuNArray.from_numpy(a)
    M = X.mutable_view(R(0, 59))
    M.map_with_inplace(X.view(R(4, 63)), lambda e, y: e + y)  # reads ahead: allowed
    exp = a.copy()
    for i in range(60):  # Mutable#map_with! order
        exp[i] = exp[i] + exp[i + 4]
    assert np.array_equal(X.to_narr(), exp)
    Y = cu.CuNArray.from_numpy(a)
    with pytest.raises(NotImplementedError):
        Y.mutable_view(R(4, 63)).map_with_inplace(Y.view(R(0, 59)), lambda e, y: e + y)
