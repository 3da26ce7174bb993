"""Masked writes (NArray#[]=(mask, value), MultiWritable#set_mask) and
whole-array equality, both evaluated on the device, against the oracle and
the reference's known answers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mask_kats_on_device(cu, kats):
    k = kats["narray_ops"]
    stock = np.array(k["stock"], np.int32)
    mask = np.array(k["mask"], np.bool_)
    S = cu.CuNArray.from_numpy(stock)
    M = cu.CuNArray.from_numpy(mask)
    a = S.clone()
    a[M] = 6
    assert a.to_narr().tolist() == k["mask_scalar_6"]
    a = S.clone()
    a[M] = S + 10
    assert a.to_narr().tolist() == k["mask_src_plus_10"]
    # a generic mask: a Bool view (here the mask read through a double reversal)
    gm = M.view(cu.R(None, None, -1), cu.R(None, None, -1)).view(cu.R(None, None, -1), cu.R(None, None, -1))
    a = S.clone()
    a.set_mask(gm, S + 10)
    assert a.to_narr().tolist() == k["mask_src_plus_10"]
    with pytest.raises(cu.DimensionError):
        a[cu.CuNArray.from_numpy(mask[:, :2])] = 1
    with pytest.raises(cu.ShapeError):
        a.set_mask(M, cu.CuNArray.from_numpy(stock[:, :2]))


@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64, np.int64, np.bool_])
def test_random_masked_writes(cu, ora, dt):
    rng = np.random.default_rng(31)
    for trial in range(12):
        rank = int(rng.integers(1, 5))
        shape = [int(rng.integers(1, 40)) for _ in range(rank)]
        base = (rng.standard_normal(shape) * 50).astype(dt)
        mask = rng.random(shape) < 0.4
        B = cu.CuNArray.from_numpy(base)
        Mk = cu.CuNArray.from_numpy(mask)
        if trial % 3 == 0:
            value = dt(7) if dt != np.bool_ else True
            V = value
        else:
            src = (rng.standard_normal(shape) * 50).astype(dt)
            S = cu.CuNArray.from_numpy(src)
            if trial % 3 == 1:
                value, V = src, S
            else:  # a reversed view of a reversed copy reads like src
                rev = src[tuple(slice(None, None, -1) for _ in shape)].copy()
                R = cu.CuNArray.from_numpy(rev)
                V = R.view(*[cu.R(None, None, -1) for _ in shape])
                value = src
        exp = ora.set_mask(base.copy(), mask, value)
        B[Mk] = V
        assert np.array_equal(B.to_narr(), exp), (trial, shape)


def test_masked_write_through_mutable_view(cu, ora):
    rng = np.random.default_rng(32)
    base = rng.integers(-100, 100, [12, 30, 9]).astype(np.int32)
    B = cu.CuNArray.from_numpy(base)
    lits = [cu.R(None, None, -1), cu.R(2, 20, 3), slice(None)]
    MV = B.mutable_view(*lits)
    mask = rng.random(MV.shape) < 0.5
    src = rng.integers(-100, 100, MV.shape).astype(np.int32)
    MV[cu.CuNArray.from_numpy(mask)] = cu.CuNArray.from_numpy(src)
    exp = base.copy()
    ora.set_mask(exp[::-1, 2:21:3, :], mask, src)
    assert np.array_equal(B.to_narr(), exp)
    MV.set_mask(cu.CuNArray.from_numpy(~mask), -5)
    ora.set_mask(exp[::-1, 2:21:3, :], ~mask, -5)
    assert np.array_equal(B.to_narr(), exp)


def test_equality_on_device(cu):
    rng = np.random.default_rng(33)
    x = rng.standard_normal([33, 70]).astype(np.float32)
    X, Y = cu.CuNArray.from_numpy(x), cu.CuNArray.from_numpy(x.copy())
    assert X == Y and X.equals(Y)
    y = x.copy()
    y[32, 69] += 1
    assert not X.equals(cu.CuNArray.from_numpy(y))
    assert not X.equals(cu.CuNArray.from_numpy(x.reshape(70, 33)))
    n = x.copy()
    n[0, 0] = np.nan
    Nn = cu.CuNArray.from_numpy(n)
    assert not Nn.equals(cu.CuNArray.from_numpy(n.copy()))  # NaN == NaN is false
    # a view compares element by element with its materialised copy
    v = X.view(cu.R(None, None, -1), cu.R(1, None, 2))
    assert v.equals(cu.CuNArray.from_numpy(np.ascontiguousarray(x[::-1, 1::2])))
    assert cu.CuNArray.from_numpy(np.zeros([0, 3], np.int32)).equals(cu.CuNArray.from_numpy(np.zeros([0, 3], np.int32)))
