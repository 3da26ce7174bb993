"""Parity of the device path (libphcuda.so through the phase_cu host mirror)
against the CPU oracle: gather/scatter through views, every infix operator,
fused ProcView chains, reductions and the heat stencil.  Bit-exact unless a
tolerance is written next to the assertion."""
import numpy as np
import pytest

from conftest import lit_from_json as L

pytestmark = pytest.mark.gpu


def _views(cu, ora, base, chain):
    """Builds the same view chain on the device and in the oracle."""
    dev = cu.CuNArray.from_numpy(base)
    v = dev.view()
    for t in chain:
        if t[0] == "region":
            v = v.view(*t[1])
        elif t[0] == "permute":
            v = v.permute(*(t[1] or []))
        elif t[0] == "reverse":
            v = v.reverse()
        elif t[0] == "reshape":
            v = v.reshape(t[1])
    return dev, v, ora.ViewOperand(base, chain)


def _random_chain(rng, shape):
    from phase_cu.region import R

    chain = []
    cur = list(shape)
    for _ in range(int(rng.integers(1, 4))):
        k = int(rng.integers(0, 4))
        if k == 0 and all(c > 0 for c in cur):
            lits = []
            for n in cur:
                f = int(rng.integers(0, n))
                l = int(rng.integers(0, n))
                s = int(rng.integers(1, 4)) * (1 if l >= f else -1)
                lits.append(R(f, l, s))
            chain.append(("region", lits))
            from phase_cu.region import IndexRegion
            cur = IndexRegion.new(lits, cur).shape
        elif k == 1:
            order = [int(x) for x in rng.permutation(len(cur))]
            chain.append(("permute", order))
            cur = [cur[o] for o in order]
        elif k == 2:
            chain.append(("reverse",))
        else:
            # View#reshape: a random factorisation of the element count (an
            # affine fold where the layout allows it, a materialised copy else)
            n = int(np.prod(cur)) if cur else 1
            new = []
            for _ in range(int(rng.integers(1, 4)) - 1):
                divs = [d for d in range(1, n + 1) if n % d == 0]
                d = divs[int(rng.integers(0, len(divs)))]
                new.append(d)
                n //= d
            new.append(n)
            chain.append(("reshape", new))
            cur = new
    return chain


@pytest.mark.parametrize("dtype", [np.float32, np.int32, np.float64, np.int64, np.bool_])
def test_random_view_gathers(cu, ora, dtype):
    rng = np.random.default_rng(10)
    for _ in range(40):
        rank = int(rng.integers(1, 5))
        shape = [int(rng.integers(1, 9)) for _ in range(rank)]
        base = (rng.standard_normal(shape) * 100).astype(dtype)
        chain = _random_chain(rng, shape)
        _, v, ov = _views(cu, ora, base, chain)
        assert v.shape == ov.shape
        assert np.array_equal(v.to_narr(), ora.gather(ov)), chain


def test_kats_on_device(cu, kats):
    stock = np.array(kats["narray_ops"]["stock"], dtype=np.int32)
    s = cu.CuNArray.from_numpy(stock)
    for case in kats["narray_fetch_chunk"]:
        got = s.get_chunk(*[L(x) for x in case["literal"]]).to_narr()
        if "expected" in case:
            assert got.tolist() == case["expected"]
        else:
            assert list(got.shape) == case["expected_shape"]
    for case in kats["narray_set_chunk"]:
        a = s.clone()
        if "src" in case:
            a.set_chunk(*[L(x) for x in case["literal"]], cu.CuNArray.from_numpy(np.array(case["src"], np.int32)))
        else:
            a.set_chunk(*[L(x) for x in case["literal"]], case["scalar"])
        assert a.to_narr().tolist() == case["expected"]
    k = kats["narray_ops"]
    assert (s + 10).to_narr().tolist() == k["plus_10"]
    assert (s ** 2).to_narr().tolist() == k["pow_2"]
    assert (s * 2).to_narr().tolist() == k["times_2"]
    assert (s * 3).to_narr().tolist() == k["times_3"]
    r = kats["readme"]
    a = cu.CuNArray.from_numpy(np.array(r["narr"], np.int32))
    b = cu.CuNArray.from_numpy(np.array(r["narr2"], np.int32))
    assert (a + b).to_narr().tolist() == r["sum"]
    assert (a * b).to_narr().tolist() == r["prod"]
    assert b.argmax() == r["argmax_narr2"] and b.max() == r["max_narr2"]
    assert [x.to_narr().tolist() for x in b.slices(1)] == r["slices_axis1"]
    m = kats["multi_writable"]
    w = cu.CuNArray.from_numpy(np.array(m["buffer"], np.int32).reshape(m["shape"]))
    w[tuple(L(x) for x in m["literal"])] = m["scalar"]
    exp = np.array(m["buffer"], np.int32)
    exp[m["scalar_indices"]] = m["scalar"]
    assert w.to_narr().reshape(-1).tolist() == exp.tolist()
    with pytest.raises(cu.ShapeError):
        w.set_chunk(*[L(x) for x in m["bad_literal"]], cu.CuNArray.from_numpy(np.array(m["chunk"], np.int32)))


def test_config1_plain(cu, ora):
    """1024x1024 Float32/Int32: a+b, a*b, a[.., 1..2..-1], bit-exact."""
    from phase_cu import synth

    a = synth.uniform_f32([1024, 1024], seed=0)
    b = synth.uniform_f32([1024, 1024], seed=0, start=1024 * 1024)
    ai = synth.uniform_i32([1024, 1024], seed=0)
    bi = synth.uniform_i32([1024, 1024], seed=0, start=1024 * 1024)
    for x, y in ((a, b), (ai, bi)):
        X, Y = cu.CuNArray.from_numpy(x), cu.CuNArray.from_numpy(y)
        assert np.array_equal((X + Y).to_narr(), ora.map_binary(ora.OP_ADD, x, y)[0])
        assert np.array_equal((X * Y).to_narr(), ora.map_binary(ora.OP_MUL, x, y)[0])
        lit = [slice(None), cu.R(1, -1, 2)]
        got = X[tuple(lit)]
        assert got.shape == [1024, 512]
        assert np.array_equal(got.to_narr(), ora.narray_fetch_chunk(x, lit))


def test_config2_strided_small(cu, ora):
    """Config-2 program at a size the oracle finishes quickly (64x32x16)."""
    from phase_cu import synth

    shape = [64, 32, 16]
    for dt in ("f32", "i32"):
        if dt == "f32":
            a = synth.uniform_f32(shape, seed=0)
            b = synth.uniform_f32(shape, seed=0, start=a.size)
        else:
            a = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20)
            b = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20, start=a.size)
        A, B = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
        perm = [("permute", [2, 0, 1])]
        rev = [("region", [slice(None), cu.R(None, None, -1), slice(None)])]
        for chain in (perm, rev):
            _, av, oa = _views(cu, ora, a, chain)
            _, bv, ob = _views(cu, ora, b, chain)
            av = A.view()
            bv = B.view()
            for t in chain:
                av = av.permute(*t[1]) if t[0] == "permute" else av.view(*t[1])
                bv = bv.permute(*t[1]) if t[0] == "permute" else bv.view(*t[1])
            assert np.array_equal(av.to_narr(), ora.gather(oa))
            ops = [(ora.OP_ADD, lambda p, q: p + q), (ora.OP_SUB, lambda p, q: p - q),
                   (ora.OP_DIV, lambda p, q: p / q)]
            if dt == "f32":
                ops.append((ora.OP_MUL, lambda p, q: p * q))
            else:
                ops.append((ora.OP_WMUL, lambda p, q: p.wmul(q)))
            for op, fn in ops:
                exp, st = ora.map_binary(op, oa, ob)
                got = fn(av, bv).to_narr()
                assert got.dtype == exp.dtype
                assert np.array_equal(got, exp, equal_nan=True), (dt, chain, op)
            if dt == "i32":
                with pytest.raises(OverflowError):
                    av * bv
        # scatter: C.mutable_view(.., ..-1.., ..)[..] = A.view.permute(2,0,1)
        c = np.zeros([16, 64, 32], dtype=a.dtype)
        C = cu.CuNArray.from_numpy(c)
        M = C.mutable_view(slice(None), cu.R(None, None, -1), slice(None))
        M[slice(None), slice(None), slice(None)] = A.view().permute(2, 0, 1)
        od = ora.ViewOperand(c, [("region", [slice(None), cu.R(None, None, -1), slice(None)])])
        os_ = ora.ViewOperand(a, [("permute", [2, 0, 1])])
        ora.scatter(od, os_)
        assert np.array_equal(C.to_narr(), od.arr)


BIN_OPS = ["ADD", "SUB", "MUL", "DIV", "FLOORDIV", "MOD", "POW", "WADD", "WSUB", "WMUL", "WPOW",
           "AND", "OR", "XOR", "GT", "LT", "GE", "LE", "CMP", "EQ"]


def _operand(rng, t, n):
    if t == np.bool_:
        return rng.integers(0, 2, n).astype(np.bool_)
    if np.issubdtype(t, np.integer):
        return rng.integers(-50, 50, n).astype(t)
    x = (rng.standard_normal(n) * 4).astype(t)
    x[::7] = np.round(x[::7])
    return x


@pytest.mark.parametrize("opname", BIN_OPS)
def test_every_binary_operator(cu, ora, opname):
    """Each infix operator on every dtype pair the reference defines, with a
    strided (reversed, stepped) left operand, against the oracle."""
    import phase_cu._abi as A

    op = getattr(A, "OP_" + opname)
    rng = np.random.default_rng(hash(opname) % 2 ** 32)
    types = [np.bool_, np.int32, np.int64, np.float32, np.float64]
    for ta in types:
        for tb in types:
            try:
                ora.result_dtype(op, ora.FROM_NP[np.dtype(ta)], ora.FROM_NP[np.dtype(tb)])
            except ora.OracleError:
                continue
            a = _operand(rng, ta, 2 * 37)
            b = _operand(rng, tb, 37)
            if opname in ("POW", "WPOW") and np.issubdtype(tb, np.integer):
                b = np.abs(b) % 5
                b = b.astype(tb)
            if opname in ("FLOORDIV", "MOD") and np.issubdtype(tb, np.integer):
                b[b == 0] = 3
            if opname in ("FLOORDIV", "MOD", "DIV") and np.issubdtype(tb, np.floating):
                b[b == 0] = 1.5
            A_ = cu.CuNArray.from_numpy(a)
            B_ = cu.CuNArray.from_numpy(b)
            av = A_.view(cu.R(None, None, -2))  # reversed, stepped
            oa = ora.ViewOperand(a, [("region", [cu.R(None, None, -2)])])
            exp, st = ora.map_binary(op, oa, b)
            if st:
                continue  # the error paths have their own test
            got = av._binary(op, B_).to_narr()
            assert got.dtype == exp.dtype, (opname, ta, tb)
            _same(got, exp, opname, np.issubdtype(tb, np.floating))
            # scalar right and scalar left
            for s in (3, 2.5, np.float32(1.25)):
                sd = cu.scalar_dtype(s)
                try:
                    e2, st2 = ora.map_binary_scalar(op, oa, s, sd)
                except ora.OracleError:
                    continue
                if st2:
                    continue
                _same(av._binary(op, s).to_narr(), e2, opname, isinstance(s, (float, np.floating)))
                try:
                    e3, st3 = ora.map_binary_scalar(op, oa, s, sd, scalar_left=True)
                except ora.OracleError:
                    continue
                if st3:
                    continue
                _same(av._binary(op, s, True).to_narr(), e3, opname, np.issubdtype(ta, np.floating))


def _same(got, exp, opname, float_exponent):
    """Bit-exact, except `**` with a floating-point exponent: that is libm pow
    (CUDA's and glibc's may differ in the last bit), tolerance 2 ulp."""
    if opname == "POW" and float_exponent:
        tol = 2 * np.finfo(exp.dtype).eps
        assert np.allclose(got, exp, rtol=tol, atol=0, equal_nan=True), (got, exp)
    else:
        assert np.array_equal(got, exp, equal_nan=True), (opname, got, exp)


def test_unary_and_errors(cu, ora):
    x = np.array([3, -4, 0, 2 ** 31 - 1], dtype=np.int32)
    X = cu.CuNArray.from_numpy(x)
    assert np.array_equal((-X).to_narr(), ora.map_unary(ora.UOP_NEG, x)[0])
    assert np.array_equal((~X).to_narr(), ora.map_unary(ora.UOP_NOT, x)[0])
    with pytest.raises(OverflowError):
        X + 1
    assert (X.wadd(1)).to_narr()[-1] == -2 ** 31
    with pytest.raises(ZeroDivisionError):
        X // cu.CuNArray.from_numpy(np.zeros(4, np.int32))
    with pytest.raises(ValueError):
        X ** -1
    with pytest.raises(OverflowError):
        -cu.CuNArray.from_numpy(np.array([-2 ** 31], np.int32))
    f = cu.CuNArray.from_numpy(np.array([1.5, -2.0], np.float32))
    assert np.array_equal((-f).to_narr(), np.array([-1.5, 2.0], np.float32))
    with pytest.raises(cu.ShapeError):
        X + f
    with pytest.raises(IndexError):
        X[5]
    with pytest.raises(cu.DimensionError):
        X[0, 0]


def test_fused_chain_config3_small(cu, ora):
    """((x + 4) ** 2) * y - z in ONE kernel equals four reference passes."""
    from phase_cu import synth

    shape = [8, 16, 16, 8]
    x = synth.lognormal_f32(shape, seed=0)
    y = synth.lognormal_f32(shape, seed=1)
    z = synth.lognormal_f32(shape, seed=2)
    X, Y, Z = (cu.CuNArray.from_numpy(v) for v in (x, y, z))
    r = X.process(lambda e: (e + 4) ** 2) * Y - Z
    assert isinstance(r, cu.CuProcView)
    t, _ = ora.map_binary_scalar(ora.OP_ADD, x, 4, ora.I32)
    t, _ = ora.map_binary_scalar(ora.OP_POW, t, 2, ora.I32)
    t, _ = ora.map_binary(ora.OP_MUL, t, y)
    t, _ = ora.map_binary(ora.OP_SUB, t, z)
    R = r.to_cu()
    assert np.array_equal(R.to_narr(), t)
    # eager infix on arrays gives the same bits
    E = ((X + 4) ** 2) * Y - Z
    assert np.array_equal(E.to_narr(), t)
    # a lazy chain viewed through a permutation = the permuted result
    assert np.array_equal(r.permute(3, 1, 0, 2).to_narr(), t.transpose(3, 1, 0, 2))
    for k in range(4):
        s = R.sum(axis=k).to_narr()
        ref = ora.reduce_f64(t, k)
        assert np.max(np.abs(s - ref) / np.abs(ref)) <= 1e-6  # tolerance: 1e-6 relative vs FP64
        assert np.array_equal(R.max(axis=k).to_narr(), ora.reduce(ora.RED_MAX, t, k))
        assert np.array_equal(R.argmax(axis=k).to_narr(), ora.reduce(ora.RED_ARGMAX, t, k, ora.I32))
        assert np.array_equal(R.min(axis=k).to_narr(), ora.reduce(ora.RED_MIN, t, k))
        assert np.array_equal(R.argmin(axis=k).to_narr(), ora.reduce(ora.RED_ARGMIN, t, k, ora.I32))
    full = R.sum()
    assert abs(full - ora.reduce_f64(t)) <= 1e-6 * abs(ora.reduce_f64(t))
    assert R.argmax() == list(np.unravel_index(int(ora.reduce(ora.RED_ARGMAX, t)), shape))


def _arr(x):
    """A reduction of a rank-1 array along its axis is a scalar."""
    return x.to_narr() if hasattr(x, "to_narr") else np.array(x)


def test_reductions_edge_cases(cu, ora):
    rng = np.random.default_rng(5)
    # ties -> first index; NaN rule
    t = np.array([[1, 5, 5, 2], [7, 7, 1, 7]], np.float32)
    T = cu.CuNArray.from_numpy(t)
    assert T.argmax(axis=1).to_narr().tolist() == [1, 0]
    assert T.argmax(axis=0).to_narr().tolist() == [1, 1, 0, 1]
    n = np.array([[np.nan, 1, 3], [1, np.nan, 3]], np.float32)
    N = cu.CuNArray.from_numpy(n)
    assert N.argmax(axis=1).to_narr().tolist() == [0, 2]
    assert np.isnan(N.max(axis=1).to_narr()[0]) and N.max(axis=1).to_narr()[1] == 3
    # strided / reversed / permuted inputs, many shapes, with split-K paths
    for shape in ([3], [1000], [5, 70000], [70000, 3], [2, 3, 5, 7], [1, 1, 300000], [64, 4096]):
        x = (rng.standard_normal(shape) * 10).astype(np.float32)
        X = cu.CuNArray.from_numpy(x)
        vx = X.view().reverse()
        xr = x[tuple(slice(None, None, -1) for _ in shape)]
        for k in range(len(shape)):
            assert np.array_equal(_arr(vx.argmax(axis=k)), ora.reduce(ora.RED_ARGMAX, xr.copy(), k, ora.I32))
            assert np.array_equal(_arr(vx.max(axis=k)), ora.reduce(ora.RED_MAX, xr.copy(), k))
            s = _arr(vx.sum(axis=k, dtype=cu.Float64))
            ref = ora.reduce_f64(xr.copy(), k)
            # tolerance: 1e-6 of the sum of magnitudes (values of both signs)
            mag = ora.reduce_f64(np.abs(xr).copy(), k)
            assert np.all(np.abs(s - ref) <= 1e-6 * mag + 1e-30)
        assert vx.argmax() == list(np.unravel_index(int(ora.reduce(ora.RED_ARGMAX, xr.copy())), shape))
    xi = rng.integers(-1000, 1000, [33, 517]).astype(np.int32)
    XI = cu.CuNArray.from_numpy(xi)
    for k in (0, 1):
        assert np.array_equal(XI.sum(axis=k).to_narr(), ora.reduce(ora.RED_SUM, xi, k))
        assert np.array_equal(XI.argmin(axis=k).to_narr(), ora.reduce(ora.RED_ARGMIN, xi, k, ora.I32))
    assert XI.sum() == int(ora.reduce(ora.RED_SUM, xi))
    with pytest.raises(OverflowError):
        cu.CuNArray.from_numpy(np.full(3, 2 ** 30, np.int32)).sum()
    with pytest.raises(cu.EmptyError):
        cu.CuNArray.from_numpy(np.zeros((0,), np.float32)).max()
    assert cu.CuNArray.from_numpy(np.zeros((0, 3), np.float32)).sum(axis=0).to_narr().tolist() == [0, 0, 0]


def test_heat_small_bit_exact(cu, ora):
    from phase_cu import synth

    u0 = synth.gaussian_bumps_f32(130, 257, bumps=4, seed=0, wmin=5, wmax=20)
    for steps in (1, 2, 4, 7, 9):  # whole and partial groups of the 4 steps one launch takes
        U = cu.CuNArray.from_numpy(u0)
        T = cu.CuNArray.empty([130, 257], cu.Float32)
        for use_graph in (0, 1):
            U = cu.CuNArray.from_numpy(u0)
            from phase_cu import _abi
            _abi.call("phcu_heat_run", U._buf.ptr, T._buf.ptr, 130, 257, 0.2, steps, use_graph)
            assert np.array_equal(U.to_narr(), ora.heat_run(u0, steps, 0.2)), (steps, use_graph)


def test_empty_and_degenerate(cu, ora):
    a = np.arange(12, dtype=np.int32).reshape(3, 4)
    A = cu.CuNArray.from_numpy(a)
    e = A[cu.R(0, 0, exclusive=True), slice(None)]
    assert e.shape == [0, 4] and e.to_narr().shape == (0, 4)
    assert A[1, 2].to_narr().tolist() == [6]
    assert A[cu.R(2, 0, -1), 3].to_narr().tolist() == [11, 7, 3]
    assert A.get(-1, -1) == 11
    assert A.get_available(cu.R(1, 5), 1).to_narr().tolist() == [5, 9]
    big_step = A[cu.R(0, 2, 7), slice(None)]
    assert big_step.to_narr().tolist() == [[0, 1, 2, 3]]
    B = A.clone()
    B[slice(None), cu.R(None, None, -1)] = A
    assert B.to_narr().tolist() == a[:, ::-1].tolist()
    # overlapping source and destination are staged
    C = A.clone()
    C[cu.R(0, 1), slice(None)] = C.view(cu.R(1, 2), slice(None))
    assert C.to_narr()[:2].tolist() == a[1:3].tolist()


@pytest.mark.parametrize("view", ["plain", "reverse", "permute"])
def test_int32_division_kernel(cu, view):
    """Int32 / Int32 -> Float64 through its own kernel kind (ROW for plain and
    reversed views, TMA tiles for permuted ones), bit-exact against IEEE
    division on the host, with zero divisors and dividends, Int32::MIN and
    exact quotients among random pairs."""
    rng = np.random.default_rng(7)
    shape = [96, 130, 72]
    a = rng.integers(-2 ** 31, 2 ** 31, shape, dtype=np.int64).astype(np.int32)
    b = rng.integers(-2 ** 31, 2 ** 31, shape, dtype=np.int64).astype(np.int32)
    fa, fb = a.reshape(-1), b.reshape(-1)
    fb[::7] = rng.integers(-1000, 1000, fb[::7].size)
    fb[3::101] = 0
    fa[5::103] = 0
    fa[11::211] = -2 ** 31
    fb[17::223] = -2 ** 31
    fa[19::97] = fb[19::97] * 3  # exact quotients (wrapping is fine: still Int32 pairs)
    A_, B_ = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
    if view == "reverse":
        A_, B_, a, b = A_.reverse(), B_.reverse(), a[::-1, ::-1, ::-1], b[::-1, ::-1, ::-1]
    elif view == "permute":
        A_, B_, a, b = A_.permute(2, 0, 1), B_.permute(2, 0, 1), a.transpose(2, 0, 1), b.transpose(2, 0, 1)
    got = (A_ / B_).to_narr()
    with np.errstate(divide="ignore", invalid="ignore"):
        exp = a.astype(np.float64) / b.astype(np.float64)
    assert got.dtype == np.float64
    nan = np.isnan(exp)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint64), exp[~nan].view(np.uint64))


def test_integer_power_by_scalar(cu, ora):
    """Int32 ** n and Int32 &** n with a scalar exponent run in the reduced
    interpreter (binary exponentiation, checked or wrapping) and match the
    oracle; a checked overflow raises, a negative exponent is refused."""
    x = np.array([2, -3, 1000, 0, 1, -1, 46340, 7], dtype=np.int32)
    X = cu.CuNArray.from_numpy(x)
    for e in (0, 1, 2, 3):
        exp, err = ora.map_binary_scalar(ora.OP_POW, x if e < 3 else x[:4], e, ora.I32)
        got = ((X if e < 3 else cu.CuNArray.from_numpy(x[:4])) ** e).to_narr()
        assert np.array_equal(got, exp), e
    w = X.wpow(5).to_narr()
    assert np.array_equal(w, ora.map_binary_scalar(ora.OP_WPOW, x, 5, ora.I32)[0])
    with pytest.raises(OverflowError):
        cu.CuNArray.from_numpy(np.array([46341, 2], np.int32)) ** 2
    with pytest.raises(ValueError):
        X ** -2
    cu.check_errors()


@pytest.mark.parametrize("dtype", [np.float32, np.int32, np.float64, np.int64, np.bool_])
def test_set_element(cu, dtype):
    """MultiWritable#unsafe_set_element through set_element (negative
    coordinates canonicalised as the reference's CoordUtil does); the other
    elements keep their values; out-of-range and rank errors raise."""
    rng = np.random.default_rng(3)
    base = (rng.standard_normal([5, 7, 3]) * 50).astype(dtype)
    X = cu.CuNArray.from_numpy(base)
    exp = base.copy()
    for coord in ([0, 0, 0], [4, 6, 2], [-1, 3, -2], [2, -7, 1]):
        val = dtype(1) if dtype == np.bool_ else dtype(-17)
        X.set_element(coord, val)
        exp[tuple(coord)] = val
    assert np.array_equal(X.to_narr(), exp)
    with pytest.raises(IndexError):
        X.set_element([5, 0, 0], dtype(1))
    with pytest.raises(IndexError):
        X.set_element([0, -8, 0], dtype(1))
    with pytest.raises(cu.DimensionError):
        X.set_element([0, 0], dtype(1))
    cu.check_errors()
