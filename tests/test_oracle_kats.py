"""Pins the CPU oracle to the reference's own known-answer tests (spec/ of
in-phase/ph-core, transcribed in tests/golden/reference_kats.json)."""
import numpy as np
import pytest

from conftest import lit_from_json as L


def _check(r, v):
    f, s, l = v
    assert (r.first[0], r.step[0], r.last[0]) == (f, s, l)
    assert r.reduced_shape[0] == (l - f) // s + 1


def test_test_ranges_valid(ora, kats):
    tr = kats["test_ranges"]
    b = tr["bound"]
    for key in ("fully_defined", "negative_indices", "implicit_bounds"):
        for lit, v in tr[key]:
            r = ora.region_new([L(lit)], [b])
            _check(r, v)


def test_test_ranges_errors(ora, kats):
    tr = kats["test_ranges"]
    b = tr["bound"]
    for lit in tr["out_of_bounds"] + tr["step_conflict"]:
        with pytest.raises(ora.OracleError) as e:
            ora.region_new([L(lit)], [b])
        assert e.value.code == ora.ERR_INDEX
    for lit in tr["empty"]:
        r = ora.region_new([L(lit)], [b])
        assert r.reduced_shape[0] == 0


def test_test_ranges_absolute(ora, kats):
    """index_region_spec.cr:93-128: the bound-free constructor."""
    tr = kats["test_ranges"]
    for lit, v in tr["fully_defined"]:
        _check(ora.region_absolute([L(lit)]), v)
    for lit, _ in tr["implicit_bounds"]:
        with pytest.raises(ora.OracleError):
            ora.region_absolute([L(lit)])
    for lit, _ in tr["negative_indices"]:
        with pytest.raises(ora.OracleError) as e:
            ora.region_absolute([L(lit)])
        assert e.value.code == ora.ERR_INDEX
    for lit in tr["step_conflict"]:
        with pytest.raises(ora.OracleError):
            ora.region_absolute([L(lit)])


def test_region_copy_and_fits(ora, kats):
    """index_region_spec.cr:140-170, 248-256: fits_in? of every valid literal."""
    tr = kats["test_ranges"]
    b = tr["bound"]
    for key in ("fully_defined", "negative_indices", "implicit_bounds"):
        for lit, v in tr[key]:
            r = ora.region_new([L(lit)], [b])
            assert ora.region_fits_in(r, [b])
            assert not ora.region_fits_in(r, [max(v[0], v[2])])


def test_region_trim_valid(ora, kats):
    """index_region_spec.cr:266-294."""
    tr = kats["test_ranges"]
    b = tr["bound"]
    for key in ("fully_defined", "negative_indices", "implicit_bounds"):
        for lit, (f, s, l) in tr[key]:
            r = ora.region_trim(ora.region_new([L(lit)], [b]), [b])
            _check(r, (f, s, l))
            r = ora.region_new([L(lit)], [b])
            if l > f:
                ora.region_trim(r, [l])
                _check(r, (f, s, l - s))
            elif f > l:
                ora.region_trim(r, [f])
                _check(r, (f + s, s, l))
            else:
                ora.region_trim(r, [l])
                assert r.reduced_shape[0] == 0


def test_region_multi_axis(ora, kats):
    k = kats["region_multi_axis"]
    r = ora.region_new([L(x) for x in k["literal"]], k["bound"])
    d = r.as_dict()
    assert d["shape"] == k["shape"] and d["first"] == k["first"]
    assert d["last"] == k["last"] and d["step"] == k["step"]
    with pytest.raises(ora.OracleError) as e:
        ora.region_new([L(x) for x in k["bad_literal"]], k["bound"])
    assert e.value.code == ora.ERR_INDEX
    a = kats["region_absolute"]
    d = ora.region_absolute([L(x) for x in a["literal"]]).as_dict()
    assert d["shape"] == a["shape"] and d["first"] == a["first"] and d["last"] == a["last"]


def test_region_includes_fits_translate_reverse(ora, kats):
    k = kats["region_includes"]
    r = ora.region_absolute([L(x) for x in k["literal"]])
    for c in k["excluded"]:
        assert not ora.region_includes(r, c)
    for c in k["included"]:
        assert ora.region_includes(r, c)
    k = kats["region_fits_in"]
    r = ora.region_absolute([L(x) for x in k["literal"]])
    assert all(ora.region_fits_in(r, s) for s in k["fits"])
    assert not any(ora.region_fits_in(r, s) for s in k["not_fits"])
    k = kats["region_translate"]
    r = ora.region_absolute([L(x) for x in k["literal"]])
    d0 = r.as_dict()
    loc = ora.region_local_to_absolute(r, [3, 1])
    t = ora.region_translate(ora.region_absolute([L(x) for x in k["literal"]]), k["offset"])
    d1 = t.as_dict()
    assert d1["shape"] == d0["shape"]
    assert d1["first"] == [a + o for a, o in zip(d0["first"], k["offset"])]
    assert d1["last"] == [a + o for a, o in zip(d0["last"], k["offset"])]
    assert ora.region_local_to_absolute(t, [3, 1]) == [a + o for a, o in zip(loc, k["offset"])]
    for off in k["raises"]:
        with pytest.raises(ora.OracleError):
            ora.region_translate(ora.region_absolute([L(x) for x in k["literal"]]), off)
    k = kats["region_reverse"]
    r = ora.region_absolute([L(x) for x in k["literal"]])
    d0 = r.as_dict()
    d1 = ora.region_reverse(r).as_dict()
    assert d1["first"] == k["first_after"] == d0["last"] and d1["last"] == d0["first"]
    assert d1["step"] == [-s for s in d0["step"]] and d1["shape"] == d0["shape"]
    k = kats["region_trim_cover"]
    r = ora.region_trim(ora.region_cover(k["cover"]), k["trim_to"])
    assert ora.region_fits_in(r, k["fits"][0]) and not ora.region_fits_in(r, k["not_fits"][0])


def test_narray_chunks(ora, kats):
    stock = np.array(kats["narray_ops"]["stock"], dtype=np.int32)
    for case in kats["narray_fetch_chunk"]:
        got = ora.narray_fetch_chunk(stock, [L(x) for x in case["literal"]])
        if "expected" in case:
            assert got.tolist() == case["expected"]
        else:
            assert list(got.shape) == case["expected_shape"]
    for case in kats["narray_set_chunk"]:
        a = stock.copy()
        src = case.get("src", case.get("scalar"))
        ora.narray_set_chunk(a, [L(x) for x in case["literal"]],
                             np.array(src, dtype=np.int32) if "src" in case else src)
        assert a.tolist() == case["expected"]


def test_narray_ops(ora, kats):
    k = kats["narray_ops"]
    stock = np.array(k["stock"], dtype=np.int32)
    out, st = ora.map_binary_scalar(ora.OP_ADD, stock, 10, ora.I32)
    assert out.tolist() == k["plus_10"] and st == 0
    out, _ = ora.map_binary_scalar(ora.OP_POW, stock, 2, ora.I32)
    assert out.tolist() == k["pow_2"]
    out, _ = ora.map_binary_scalar(ora.OP_MUL, stock, 2, ora.I32)
    assert out.tolist() == k["times_2"]
    out, _ = ora.map_binary_scalar(ora.OP_MUL, stock, 3, ora.I32)
    assert out.tolist() == k["times_3"]
    r = kats["readme"]
    a = np.array(r["narr"], dtype=np.int32)
    b = np.array(r["narr2"], dtype=np.int32)
    assert ora.map_binary(ora.OP_ADD, a, b)[0].tolist() == r["sum"]
    assert ora.map_binary(ora.OP_MUL, a, b)[0].tolist() == r["prod"]
    idx = ora.reduce(ora.RED_ARGMAX, b)
    assert list(np.unravel_index(int(idx), b.shape)) == r["argmax_narr2"]
    assert ora.reduce(ora.RED_MAX, b) == r["max_narr2"]


def test_mask_writes(ora, kats):
    """spec/n_array_spec.cr:297-333: narr[mask] = 6 and narr[mask] = stock + 10."""
    k = kats["narray_ops"]
    stock = np.array(k["stock"], dtype=np.int32)
    mask = np.array(k["mask"], dtype=np.bool_)
    assert ora.set_mask(stock.copy(), mask, 6).tolist() == k["mask_scalar_6"]
    assert ora.set_mask(stock.copy(), mask, stock + 10).tolist() == k["mask_src_plus_10"]
    with pytest.raises(ora.OracleError):
        ora.set_mask(stock.copy(), mask[:, :2], 6)


def test_transforms(ora, kats):
    t = kats["transforms"]
    assert ora.xf_apply(ora.TF_PERMUTE, t["permute"]["coord"], pattern=t["permute"]["pattern"]) == \
        t["permute"]["expected"]
    assert ora.xf_apply(ora.TF_RESHAPE, t["reshape"]["coord"], src_shape=t["reshape"]["src_shape"],
                        new_shape=t["reshape"]["new_shape"]) == t["reshape"]["expected"]
    assert ora.xf_apply(ora.TF_REVERSE, t["reverse"]["coord"], shape=t["reverse"]["shape"]) == t["reverse"]["expected"]


def test_elem_iterators(ora, kats):
    """The lexicographic and colexicographic iteration orders of the reference's
    element iterators (spec/multi_indexable/elem_iterator_spec.cr,
    elem_coord_iterator_spec.cr): every bulk operation writes its output in
    lexicographic order, so the gather of the array is the lexicographic
    sequence, the gather of its transpose the colexicographic one, and the
    gather of its reversal the reversed sequence (reverse_each); the
    coordinate operands (map_with_coord) give the coordinates in the same
    orders."""
    k = kats["elem_iterators"]
    narr = np.array(k["narr"], dtype=np.int32)
    from phase_cu.region import R

    assert ora.gather(ora.ViewOperand(narr)).reshape(-1).tolist() == k["lex"]
    assert ora.gather(ora.ViewOperand(narr, [("permute", [1, 0])])).reshape(-1).tolist() == k["colex"]
    rev = [("region", [R(None, None, -1), R(None, None, -1)])]
    assert ora.gather(ora.ViewOperand(narr, rev)).reshape(-1).tolist() == k["lex"][::-1]
    c0, c1 = ora.coords(narr.shape)
    lex = [[int(a), int(b)] for a, b in zip(c0.reshape(-1), c1.reshape(-1))]
    assert lex == k["lex_coords"]
    t0 = ora.gather(ora.ViewOperand(c0, [("permute", [1, 0])])).reshape(-1)
    t1 = ora.gather(ora.ViewOperand(c1, [("permute", [1, 0])])).reshape(-1)
    assert [[int(a), int(b)] for a, b in zip(t0, t1)] == k["colex_coords"]


def test_narray_maps(ora, kats):
    """NArray#map, #map_with_coord and #map_with_index (spec/n_array_spec.cr:
    444-518) on the oracle: the block evaluated per element with the
    coordinates / lexicographic index operands, Crystal Int32 arithmetic."""
    k = kats["narray_maps"]
    stock = np.array(k["stock"], dtype=np.int32)
    sq, _ = ora.map_binary_scalar(ora.OP_POW, stock, 2, ora.I32)
    assert sq.tolist() == k["map_pow_2"]
    c0, c1 = ora.coords(stock.shape)
    t, _ = ora.map_binary_scalar(ora.OP_MUL, c0, 10, ora.I32, scalar_left=True)
    t, _ = ora.map_binary(ora.OP_ADD, t, c1)
    t, _ = ora.map_binary(ora.OP_ADD, t, stock)
    assert t.tolist() == k["map_with_coord"]
    twice, _ = ora.map_binary_scalar(ora.OP_MUL, stock, 2, ora.I32)
    t, _ = ora.map_binary(ora.OP_ADD, ora.lex_index(stock.shape), twice)
    assert t.tolist() == k["map_with_index_of_times_2"]


def test_multi_writable(ora, kats):
    k = kats["multi_writable"]
    buf = np.array(k["buffer"], dtype=np.int32).reshape(k["shape"])
    a = buf.copy()
    ora.narray_set_chunk(a, [L(x) for x in k["literal"]], k["scalar"])
    exp = buf.reshape(-1).copy()
    exp[k["scalar_indices"]] = k["scalar"]
    assert a.reshape(-1).tolist() == exp.tolist()
    a = buf.copy()
    ora.narray_set_chunk(a, [L(x) for x in k["literal"]], np.array(k["chunk"], dtype=np.int32))
    exp = buf.reshape(-1).copy()
    exp[k["scalar_indices"]] = np.array(k["chunk"]).reshape(-1)
    assert a.reshape(-1).tolist() == exp.tolist()
    with pytest.raises(ora.OracleError):
        r = ora.region_new([L(x) for x in k["bad_literal"]], k["shape"])
        if list(r.reduced_shape[:r.reduced_rank]) != [2, 3]:
            raise ora.OracleError(ora.ERR_SHAPE)


def test_coord_and_shape_utils(ora, kats):
    k = kats["canonicalize_index"]
    for i, n, exp in k["ok"]:
        assert ora.canonicalize_index(i, n) == exp
    for i, n in k["raises"] + k["has_index_false"]:
        with pytest.raises(ora.OracleError):
            ora.canonicalize_index(i, n)
    c = kats["compatible_shapes"]
    for a, b in zip(c["base"], c["compatible"]):
        assert ora.compatible_shapes(a, b) and ora.compatible_shapes(b, a)
    for a, b in zip(c["base"], c["incompatible"]):
        assert not ora.compatible_shapes(a, b)


def test_views_compose_like_the_reference(ora):
    """View transform chains applied per element (view.cr:109-117) equal
    numpy's strided reading of the same chain."""
    a = np.arange(4 * 5 * 6, dtype=np.int32).reshape(4, 5, 6)
    from phase_cu.region import R

    v = ora.ViewOperand(a, [("region", [slice(None), R(None, None, -1), R(1, None, 2)]), ("permute", [2, 0, 1])])
    got = ora.gather(v)
    exp = a[:, ::-1, 1::2].transpose(2, 0, 1)
    assert got.tolist() == exp.tolist()
    v = ora.ViewOperand(a, [("reverse",), ("region", [1]), ("reshape", [3, 10])])
    assert ora.gather(v).tolist() == a[::-1, ::-1, ::-1][1].reshape(3, 10).tolist()
    v = ora.ViewOperand(a, [("permute", None)])
    assert ora.gather(v).tolist() == a.transpose(2, 1, 0).tolist()


def test_crystal_int_semantics(ora):
    a = np.array([7, -7, 7, -7, 2 ** 31 - 1, -2 ** 31], dtype=np.int32)
    b = np.array([2, 2, -2, -2, 1, -1], dtype=np.int32)
    q, st = ora.map_binary(ora.OP_FLOORDIV, a[:4], b[:4])
    assert q.tolist() == [3, -4, -4, 3] and st == 0
    m, st = ora.map_binary(ora.OP_MOD, a[:4], b[:4])
    assert m.tolist() == [1, 1, -1, -1] and st == 0
    _, st = ora.map_binary(ora.OP_ADD, a[4:5], b[4:5])
    assert st & ora.ST_OVERFLOW
    w, st = ora.map_binary(ora.OP_WADD, a[4:5], b[4:5])
    assert w.tolist() == [-2 ** 31] and st == 0
    _, st = ora.map_binary(ora.OP_FLOORDIV, a[5:], b[5:])
    assert st & ora.ST_OVERFLOW
    d, st = ora.map_binary(ora.OP_DIV, a[:2], b[:2])
    assert d.dtype == np.float64 and d.tolist() == [3.5, -3.5]
    _, st = ora.map_binary(ora.OP_FLOORDIV, a[:1], np.zeros(1, dtype=np.int32))
    assert st & ora.ST_DIVZERO
    _, st = ora.map_binary_scalar(ora.OP_POW, a[:1], -1, ora.I32)
    assert st & ora.ST_ARGUMENT


def test_float32_semantics(ora):
    x = np.array([1.5, -2.25, 3.0], dtype=np.float32)
    out, _ = ora.map_binary_scalar(ora.OP_POW, x, 2, ora.I32)
    assert out.dtype == np.float32 and out.tolist() == (x * x).tolist()
    out, _ = ora.map_binary_scalar(ora.OP_ADD, x, 4, ora.I32)
    assert out.dtype == np.float32 and out.tolist() == (x + np.float32(4)).tolist()
    out, _ = ora.map_binary_scalar(ora.OP_ADD, x, 4.0, ora.F64)
    assert out.dtype == np.float64
    fm, st = ora.map_binary(ora.OP_MOD, np.array([5.5, -5.5], np.float32), np.array([2, 2], np.float32))
    assert fm.tolist() == [1.5, 0.5]


def test_reduce_semantics(ora):
    x = np.array([[1, 5, 5], [7, 2, 7]], dtype=np.float32)
    assert ora.reduce(ora.RED_ARGMAX, x, 1).tolist() == [1, 0]
    assert ora.reduce(ora.RED_ARGMAX, x, 0).tolist() == [1, 0, 1]
    assert ora.reduce(ora.RED_SUM, x, 0).tolist() == [8, 7, 12]
    nan = np.array([np.nan, 1.0, 3.0], dtype=np.float32)
    assert int(ora.reduce(ora.RED_ARGMAX, nan)) == 0
    n2 = np.array([1.0, np.nan, 3.0], dtype=np.float32)
    assert int(ora.reduce(ora.RED_ARGMAX, n2)) == 2
    with pytest.raises(ora.OracleError):
        ora.reduce(ora.RED_MAX, np.zeros((0,), np.float32))
    big = np.full(3, 2 ** 30, dtype=np.int32)
    with pytest.raises(ora.OracleError) as e:
        ora.reduce(ora.RED_SUM, big)
    assert e.value.code == ora.ERR_OVERFLOW
    assert abs(ora.reduce_f64(np.full(1000, 0.1, np.float32)) - 1000 * float(np.float32(0.1))) < 1e-9


def test_heat_oracle_small(ora):
    u = np.zeros((6, 7), dtype=np.float32)
    u[2, 3] = 1.0
    one = ora.heat_run(u, 1)
    assert one[2, 3] == np.float32(1.0) + np.float32(-4.0) * np.float32(0.2)
    assert one[1, 3] == np.float32(0.0) + np.float32(1.0) * np.float32(0.2)
    assert one[0].tolist() == [0.0] * 7
    f64 = ora.heat_run(u, 10, f64=True)
    f32 = ora.heat_run(u, 10)
    assert np.max(np.abs(f64 - f32)) < 1e-6


def test_mlp_grad_matches_finite_differences(ora):
    rng = np.random.default_rng(0)
    n = 64 * 24 + 64 + 64 * 64 + 64 + 64 + 1
    p = (rng.standard_normal(n) * 0.1).astype(np.float32)
    x = rng.standard_normal((8, 24)).astype(np.float32)
    y = rng.standard_normal(8).astype(np.float32)
    loss, g = ora.mlp_forward_backward(p, x, y)
    for idx in [0, 100, 64 * 24 + 3, n - 1, n - 10]:
        e = 1e-2
        pp = p.copy()
        pp[idx] += e
        lp, _ = ora.mlp_forward_backward(pp, x, y)
        pm = p.copy()
        pm[idx] -= e
        lm, _ = ora.mlp_forward_backward(pm, x, y)
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[idx]) < 1e-3 + 1e-2 * abs(g[idx])
