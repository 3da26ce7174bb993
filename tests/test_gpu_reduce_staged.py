"""Reductions against the oracle: the two single-launch paths, and COLUMN
layouts over contiguous arrays:

- short contiguous rows laid back to back (the innermost axis of a contiguous
  array, 32-96 four-byte elements, enough rows for every SM), staged into
  shared memory by bulk copies and reduced one row per thread;
- the full reduction of one contiguous run, block partials folded by the
  block that finishes last (no second launch).

Ties, zeros of both signs, NaNs (also as the first element) and integer
overflow are placed to pin the reference's scan rule (first extreme wins,
strict comparison, NaNs skipped unless first) and the checked Int32 sum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rows(rng, shape, dt):
    if np.issubdtype(dt, np.integer):
        x = rng.integers(-60, 60, shape).astype(dt)
    else:
        x = (rng.standard_normal(shape) * 10).astype(dt)
        flat = x.reshape(-1)
        flat[::97] = 3.0          # ties
        flat[7::389] = np.nan     # NaNs inside rows
        x[5, 0] = np.nan          # a NaN first element
        x[6, :] = np.nan          # a row of NaNs
        x[8, :] = -0.0
        x[8, 3] = 0.0             # zeros of both signs: the first one wins
    return x


@pytest.mark.parametrize("dt", [np.float32, np.int32])
@pytest.mark.parametrize("k", [32, 64, 96])
def test_staged_rows(cu, ora, dt, k):
    rng = np.random.default_rng(k)
    x = _rows(rng, [40000, k], dt)
    X = cu.CuNArray.from_numpy(x)
    oi = ora.I32
    assert np.array_equal(X.argmax(axis=1).to_narr(), ora.reduce(ora.RED_ARGMAX, x, 1, oi))
    assert np.array_equal(X.argmin(axis=1).to_narr(), ora.reduce(ora.RED_ARGMIN, x, 1, oi))
    mx, mn = X.max(axis=1).to_narr(), X.min(axis=1).to_narr()
    omx, omn = ora.reduce(ora.RED_MAX, x, 1), ora.reduce(ora.RED_MIN, x, 1)
    # bit patterns: the sign of a zero and NaN must match
    assert np.array_equal(mx.view(np.uint32), omx.view(np.uint32))
    assert np.array_equal(mn.view(np.uint32), omn.view(np.uint32))
    s = X.sum(axis=1).to_narr()
    if dt == np.int32:
        assert np.array_equal(s, ora.reduce(ora.RED_SUM, x, 1))
    else:
        ref = ora.reduce_f64(x, 1)
        mag = ora.reduce_f64(np.abs(x), 1)
        fin = np.isfinite(ref)
        # tolerance: 1e-6 of the sum of magnitudes vs the FP64 oracle
        assert np.all(np.abs(s[fin] - ref[fin]) <= 1e-6 * mag[fin] + 1e-30)
        assert np.all(np.isnan(s[~fin]))


def test_staged_rows_checked_int32_sum(cu):
    x = np.full([40000, 64], 1 << 26, dtype=np.int32)  # each row sums to 2^32: overflows Int32
    X = cu.CuNArray.from_numpy(x)
    with pytest.raises(OverflowError):
        X.sum(axis=1)
    cu.check_errors()


@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64, np.int64])
@pytest.mark.parametrize("n", [1 << 16, (1 << 22) + 3, 3 * (1 << 20) + 1])
def test_full_run(cu, ora, dt, n):
    rng = np.random.default_rng(n % 1000)
    if np.issubdtype(dt, np.integer):
        x = rng.integers(-1000, 1000, n).astype(dt)
    else:
        x = (rng.standard_normal(n) * 3).astype(dt)
        x[::1001] = 7.5  # ties of the maximum
        x[n // 3] = 9.0
        x[2 * n // 3] = 9.0
    X = cu.CuNArray.from_numpy(x)
    assert X.argmax() == [ora.reduce(ora.RED_ARGMAX, x)]  # axis=None: the coordinate
    assert X.argmin() == [ora.reduce(ora.RED_ARGMIN, x)]
    assert X.max() == ora.reduce(ora.RED_MAX, x)
    if np.issubdtype(dt, np.integer):
        assert X.sum() == ora.reduce(ora.RED_SUM, x)
    else:
        ref, mag = ora.reduce_f64(x), ora.reduce_f64(np.abs(x))
        assert abs(X.sum() - ref) <= 1e-6 * mag  # tolerance: 1e-6 of the sum of magnitudes
    # twice in a row: the arrival counter is reset by the launch that used it
    assert X.argmax() == [ora.reduce(ora.RED_ARGMAX, x)]


# COLUMN layouts over contiguous arrays (kept outputs in runs of 64 whose
# reduced positions lie back to back, runs of 4096, one run)
@pytest.mark.parametrize("dt", [np.float32, np.int32])
@pytest.mark.parametrize("shape,axis", [([38, 64, 40, 64], 2), ([40, 33, 4096], 1), ([37, 262144], 0)])
def test_column_layouts(cu, ora, dt, shape, axis):
    rng = np.random.default_rng(sum(shape))
    if np.issubdtype(dt, np.integer):
        x = rng.integers(-60, 60, shape).astype(dt)
    else:
        x = (rng.standard_normal(shape) * 10).astype(dt)
        flat = x.reshape(-1)
        flat[::89] = 3.0
        flat[11::997] = np.nan
    X = cu.CuNArray.from_numpy(x)
    oi = ora.I32
    assert np.array_equal(X.argmax(axis=axis).to_narr(), ora.reduce(ora.RED_ARGMAX, x, axis, oi))
    assert np.array_equal(X.argmin(axis=axis).to_narr(), ora.reduce(ora.RED_ARGMIN, x, axis, oi))
    mx = X.max(axis=axis).to_narr()
    assert np.array_equal(mx.view(np.uint32), ora.reduce(ora.RED_MAX, x, axis).view(np.uint32))
    s = X.sum(axis=axis).to_narr()
    if dt == np.int32:
        assert np.array_equal(s, ora.reduce(ora.RED_SUM, x, axis))
    else:
        ref, mag = ora.reduce_f64(x, axis), ora.reduce_f64(np.abs(x), axis)
        fin = np.isfinite(ref)
        assert np.all(np.abs(s[fin] - ref[fin]) <= 1e-6 * mag[fin] + 1e-30)  # 1e-6 of the sum of magnitudes
        assert np.all(np.isnan(s[~fin]))


# SLAB sums: the reduced axis directly outside the innermost kept axis, the
# two contiguous (one K x L slab per outer index), L / (16 / element size) a
# power of two up to 256, one split (at least 1024 outputs per SM) and enough
# slabs for every SM.  Odd K leaves tails after the eight-in-flight batches;
# L = 8 gives 128 row sets per block, L = 1024 a single one (Float64: COLUMN;
# extrema of Float64 always COLUMN).
@pytest.mark.parametrize("dt", [np.float32, np.int32, np.float64])
@pytest.mark.parametrize("shape", [[2500, 37, 64], [20000, 33, 8], [160, 20, 1024], [3, 820, 9, 64]])
def test_slab_sums(cu, ora, dt, shape):
    axis = len(shape) - 2
    rng = np.random.default_rng(sum(shape))
    if np.issubdtype(dt, np.integer):
        x = rng.integers(-1000, 1000, shape).astype(dt)
    else:
        x = (rng.standard_normal(shape) * 10).astype(dt)
        flat = x.reshape(-1)
        flat[13::1009] = np.nan
        flat[::4099] = 1e30  # large terms next to small ones: the compensation matters
    X = cu.CuNArray.from_numpy(x)
    s = X.sum(axis=axis).to_narr()
    if dt == np.int32:
        assert np.array_equal(s, ora.reduce(ora.RED_SUM, x, axis))
    else:
        ref, mag = ora.reduce_f64(x, axis), ora.reduce_f64(np.abs(x), axis)
        fin = np.isfinite(ref)
        assert np.all(np.abs(s[fin] - ref[fin]) <= 1e-6 * mag[fin] + 1e-30)  # 1e-6 of the sum of magnitudes
        assert np.all(np.isnan(s[~fin]))
    # extrema of the same layouts (slabs for 4-byte elements): first index of
    # the extreme, NaNs skipped unless first, both zeros equal
    if dt == np.float32:
        xs = np.moveaxis(x, axis, 0)  # [K, ...]: row k of every output
        xs[3][..., ::5] = 77.0
        xs[6][..., ::5] = 77.0   # ties of the maximum: index 3 wins
        xs[0][..., 1::7] = np.nan  # NaN first element: index 0 wins
        xs[1][..., 2::11] = -0.0
        xs[2][..., 2::11] = 0.0
        X = cu.CuNArray.from_numpy(x)
    oi = ora.I32
    assert np.array_equal(X.argmax(axis=axis).to_narr(), ora.reduce(ora.RED_ARGMAX, x, axis, oi))
    assert np.array_equal(X.argmin(axis=axis).to_narr(), ora.reduce(ora.RED_ARGMIN, x, axis, oi))
    bits = np.uint64 if dt == np.float64 else np.uint32
    assert np.array_equal(X.max(axis=axis).to_narr().view(bits), ora.reduce(ora.RED_MAX, x, axis).view(bits))
    assert np.array_equal(X.min(axis=axis).to_narr().view(bits), ora.reduce(ora.RED_MIN, x, axis).view(bits))
