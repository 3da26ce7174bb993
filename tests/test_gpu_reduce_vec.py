"""Reductions over forward-strided (unit-stride) inputs, which take the
16-byte-load kernels: GROUP along a contiguous reduced axis and COLUMN across
a contiguous run of outputs, with and without split partials, for every
element type, against the oracle.  Ties and NaNs are placed inside vectors
and across lanes to pin the first-index rule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# [4099, 48] and [4097, 61] along axis 1: an odd number of outputs whose rows
# one pass of a group covers (the extremum takes two outputs per group), the
# second with a partial last vector
SHAPES = [[64, 8, 8, 64], [3, 1000], [1000, 3], [7, 4097], [2, 3, 5, 8], [1, 300001], [300000, 1], [16, 4096],
          [4096, 16], [5, 6, 7], [4099, 48], [4097, 61]]


def _arr(x):
    return x.to_narr() if hasattr(x, "to_narr") else np.array(x)


@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64, np.int64])
def test_vector_reductions(cu, ora, dt):
    rng = np.random.default_rng(51)
    for shape in SHAPES:
        if np.issubdtype(dt, np.integer):
            x = rng.integers(-50, 50, shape).astype(dt)  # many ties
        else:
            x = (rng.standard_normal(shape) * 10).astype(dt)
            x.reshape(-1)[::97] = 3.0   # ties
            x.reshape(-1)[5::1013] = np.nan
        X = cu.CuNArray.from_numpy(x)
        out_i = ora.I32
        for k in range(len(shape)):
            assert np.array_equal(_arr(X.argmax(axis=k)), ora.reduce(ora.RED_ARGMAX, x, k, out_i)), (shape, k)
            assert np.array_equal(_arr(X.argmin(axis=k)), ora.reduce(ora.RED_ARGMIN, x, k, out_i)), (shape, k)
            assert np.array_equal(_arr(X.max(axis=k)), ora.reduce(ora.RED_MAX, x, k), equal_nan=True), (shape, k)
            if np.issubdtype(dt, np.integer):
                assert np.array_equal(_arr(X.sum(axis=k)), ora.reduce(ora.RED_SUM, x, k)), (shape, k)
            else:
                xs = np.nan_to_num(x, nan=1.0)
                Xs = cu.CuNArray.from_numpy(xs)
                s = _arr(Xs.sum(axis=k))
                ref = ora.reduce_f64(xs, k)
                mag = ora.reduce_f64(np.abs(xs), k)
                # tolerance: 1e-6 of the sum of magnitudes (values of both signs)
                assert np.all(np.abs(s - ref) <= 1e-6 * mag + 1e-30), (shape, k)
        assert X.argmax() == list(np.unravel_index(int(ora.reduce(ora.RED_ARGMAX, x)), shape))


def test_vector_reductions_config3_shape(cu, ora):
    """The 64x128x128x64 layout at 1/16 of its size: every axis, sum/max/argmax."""
    from phase_cu import synth

    shape = [16, 32, 32, 64]
    x = synth.lognormal_f32(shape, seed=3)
    X = cu.CuNArray.from_numpy(x)
    for k in range(4):
        s = X.sum(axis=k).to_narr()
        ref = ora.reduce_f64(x, k)
        assert np.max(np.abs(s - ref) / np.abs(ref)) <= 1e-6  # tolerance: 1e-6 relative vs FP64
        assert np.array_equal(X.max(axis=k).to_narr(), ora.reduce(ora.RED_MAX, x, k))
        assert np.array_equal(X.argmax(axis=k).to_narr(), ora.reduce(ora.RED_ARGMAX, x, k, ora.I32))
    full = X.sum()
    assert abs(full - ora.reduce_f64(x)) <= 1e-6 * abs(ora.reduce_f64(x))
