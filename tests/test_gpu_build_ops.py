"""Device constructors around the hot path: NArray.tile, NArray.concatenate
and NArray#push, each one or a few strided copies, against the oracle's
restatement of the reference loops."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tile(cu, ora):
    rng = np.random.default_rng(41)
    src = np.array([[1, 2], [3, 4]], np.int32)
    t = cu.CuNArray.tile(cu.CuNArray.from_numpy(src), [2, 1]).to_narr()
    # counts[i] multiplies axis i (n_array.cr:242-243), so [2, 1] doubles axis 0
    assert t.tolist() == [[1, 2], [3, 4], [1, 2], [3, 4]]
    assert np.array_equal(t, ora.tile(src, [2, 1]))
    for rank in (1, 2, 3, 4, 5):
        shape = [int(rng.integers(1, 5)) for _ in range(rank)]
        counts = [int(rng.integers(1, 4)) for _ in range(rank)]
        x = rng.integers(-100, 100, shape).astype(np.int32)
        got = cu.CuNArray.tile(cu.CuNArray.from_numpy(x), counts).to_narr()
        assert np.array_equal(got, ora.tile(x, counts)), (shape, counts)
    # a strided view as the source
    x = rng.standard_normal([6, 7]).astype(np.float32)
    X = cu.CuNArray.from_numpy(x)
    v = X.view(cu.R(None, None, -2), cu.R(1, None, 3))
    got = cu.CuNArray.tile(v, [3, 2]).to_narr()
    assert np.array_equal(got, ora.tile(np.ascontiguousarray(x[::-2, 1::3]), [3, 2]))


def test_concatenate_and_push(cu, ora):
    rng = np.random.default_rng(42)
    for axis in (0, 1, 2):
        parts = []
        for k in range(3):
            shape = [4, 5, 6]
            shape[axis] = int(rng.integers(0, 4))
            parts.append(rng.integers(-9, 9, shape).astype(np.int32))
        got = cu.CuNArray.concatenate(*[cu.CuNArray.from_numpy(p) for p in parts], axis=axis).to_narr()
        assert np.array_equal(got, ora.concatenate(parts, axis)), axis
    a = rng.standard_normal([3, 4]).astype(np.float32)
    b = rng.standard_normal([2, 4]).astype(np.float32)
    A_ = cu.CuNArray.from_numpy(a)
    B_ = cu.CuNArray.from_numpy(b)
    v = B_.view(cu.R(None, None, -1), slice(None))  # a view operand
    A_.push(v)
    assert A_.shape == [5, 4]
    assert np.array_equal(A_.to_narr(), ora.concatenate([a, b[::-1]], 0))
    A_ << B_
    assert np.array_equal(A_.to_narr(), ora.concatenate([a, b[::-1], b], 0))
    with pytest.raises(cu.DimensionError):
        cu.CuNArray.concatenate(cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b), axis=1)


def test_serialisation_on_device_arrays(cu, kats):
    """spec/n_array_spec.cr:520-557 through device arrays (one download / upload)."""
    k = kats["serialization"]
    stock = cu.CuNArray.from_numpy(np.array(kats["narray_ops"]["stock"], np.int32))
    assert stock.to_json() == k["stock_json"]
    assert stock.to_yaml() == k["stock_yaml"]
    assert cu.CuNArray.from_json(k["stock_json"], cu.Int32) == stock
    assert cu.CuNArray.from_yaml(k["stock_yaml"], cu.Int32) == stock
    assert cu.CuNArray.fill([0], 0).to_json() == k["empty_json"]
    assert cu.CuNArray.from_yaml(k["empty_yaml"], cu.Int32).shape == [0]
    x = np.random.default_rng(3).standard_normal([4, 5]).astype(np.float32)
    X = cu.CuNArray.from_numpy(x)
    assert np.array_equal(cu.CuNArray.from_json(X.to_json(), cu.Float32).to_narr(), x)
