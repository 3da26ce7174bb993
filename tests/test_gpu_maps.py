"""Element-index and coordinate maps, in-place maps and expressions longer
than one device program, on the device, bit-exact against the oracle:

- NArray#map / #map_with_index / #map_with_coord and their in-place forms
  (src/n_array.cr:589-650), MultiIndexable#map_with_coord and #map_with
  (src/multi_indexable.cr:708-712, 1026-1078), Mutable#map!, #map_with_coord!
  and #map_with! (src/multi_indexable/mutable.cr:16-67): the index and the
  coordinates are index operands computed on the device, never stored;
- ProcView composition without limit (src/proc_view.cr:32-35): expressions
  with more distinct views, instructions or nesting than one device program
  holds are split into materialised pieces, with unchanged results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f32(shape, seed):
    return (np.random.default_rng(seed).uniform(-4, 4, shape)).astype(np.float32)


def _i32(shape, seed):
    return np.random.default_rng(seed).integers(-1000, 1000, shape).astype(np.int32)


def test_reference_map_kats_on_device(cu, kats):
    """NArray#map, #map_with_coord, #map_with_index and the in-place forms
    map!, map_with_coord!, map_with_index! on the spec's stock array
    (spec/n_array_spec.cr:444-518), on the device."""
    k = kats["narray_maps"]
    stock = np.array(k["stock"], dtype=np.int32)
    S = cu.CuNArray.from_numpy(stock)
    assert S.map(lambda x: x ** 2).to_narr().tolist() == k["map_pow_2"]
    assert S.map_with_coord(lambda el, c: 10 * c[0] + c[1] + el).to_narr().tolist() == k["map_with_coord"]
    T = cu.CuNArray.from_numpy(stock * 2)
    assert T.map_with_index(lambda el, idx: idx + el).to_narr().tolist() == k["map_with_index_of_times_2"]
    M = S.clone()
    assert M.map_inplace(lambda x: x ** 2) is M
    assert M.to_narr().tolist() == k["map_pow_2"]
    C = S.clone()
    assert C.map_with_coord_inplace(lambda el, c: 10 * c[0] + c[1] + el) is C
    assert C.to_narr().tolist() == k["map_with_coord"]
    I = cu.CuNArray.from_numpy(stock * 2)  # noqa: E741
    assert I.map_with_index_inplace(lambda el, idx: idx + el) is I
    assert I.to_narr().tolist() == k["map_with_index_of_times_2"]


def test_map_with_index(cu, ora):
    shape = [6, 33, 17]
    a = _f32(shape, 0)
    A = cu.CuNArray.from_numpy(a)
    idx = ora.lex_index(shape)
    exp, _ = ora.map_binary(ora.OP_MUL, a, idx)  # Float32 * Int32 -> Float32
    exp, _ = ora.map_binary_scalar(ora.OP_ADD, exp, 1, ora.I32)
    got = A.map_with_index(lambda e, i: e * i + 1)
    assert got.dtype == cu.Float32
    assert np.array_equal(got.to_narr(), exp)
    ai = _i32(shape, 1)
    Ai = cu.CuNArray.from_numpy(ai)
    e3, _ = ora.map_binary_scalar(ora.OP_MUL, ai, 3, ora.I32)
    exp, st = ora.map_binary(ora.OP_SUB, e3, idx)
    assert st == 0
    assert np.array_equal(Ai.map_with_index(lambda e, i: e * 3 - i).to_narr(), exp)


def test_map_with_coord_on_a_permuted_view(cu, ora):
    shape = [9, 14, 11]
    a = _f32(shape, 2)
    A = cu.CuNArray.from_numpy(a)
    V = A.view().permute(2, 0, 1)
    v = np.ascontiguousarray(np.transpose(a, (2, 0, 1)))
    c = ora.coords(v.shape)
    m, _ = ora.map_binary_scalar(ora.OP_MUL, c[0], 100, ora.I32)
    exp, _ = ora.map_binary(ora.OP_ADD, v, m)
    exp, _ = ora.map_binary(ora.OP_ADD, exp, c[2])
    got = V.map_with_coord(lambda e, coord: e + coord[0] * 100 + coord[2])
    assert np.array_equal(got.to_narr(), exp)


def test_map_with_coord_rank4_splits(cu, ora):
    """Element and four coordinates: five operands, one more than a device
    program reads, so the expression runs as two programs."""
    shape = [5, 6, 7, 8]
    a = _f32(shape, 3)
    A = cu.CuNArray.from_numpy(a)
    c = ora.coords(shape)
    s01, _ = ora.map_binary(ora.OP_ADD, c[0], c[1])
    p, _ = ora.map_binary(ora.OP_MUL, a, s01)
    q, _ = ora.map_binary(ora.OP_MUL, c[2], c[3])
    exp, _ = ora.map_binary(ora.OP_SUB, p, q)
    got = A.map_with_coord(lambda e, k: e * (k[0] + k[1]) - k[2] * k[3])
    assert np.array_equal(got.to_narr(), exp)
    # the idiom of MultiIndexable#map_with_coord's example: el + coord.sum
    # (Enumerable#sum folds from 0 in Int32: (((0 + c0) + c1) + c2) + c3)
    tot = np.zeros(shape, dtype=np.int32)
    for k in range(4):
        tot, _ = ora.map_binary(ora.OP_ADD, tot, c[k])
    exp2, _ = ora.map_binary(ora.OP_ADD, a, tot)
    got2 = A.map_with_coord(lambda e, k: e + sum(k))
    assert np.array_equal(got2.to_narr(), exp2)


def test_index_operands_follow_views(cu, ora):
    """A lazy map_with_index viewed through a region and a reversal: each
    element keeps the index it was computed for."""
    shape = [12, 40]
    a = _f32(shape, 4)
    A = cu.CuNArray.from_numpy(a)
    P = A.process_with_index(lambda e, i: e + i)
    full, _ = ora.map_binary(ora.OP_ADD, a, ora.lex_index(shape))
    got = P.view(cu.R(2, -1), cu.R(None, None, -1)).to_narr()
    assert np.array_equal(got, full[2:, ::-1])
    assert np.array_equal(P.permute(1, 0).to_narr(), np.ascontiguousarray(full.T))


def test_map_and_map_with(cu, ora):
    shape = [7, 129]
    a, b = _f32(shape, 5), _f32(shape, 6)
    A, B = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
    exp, _ = ora.map_binary_scalar(ora.OP_MUL, a, np.float32(2.5), ora.F32)
    assert np.array_equal(A.map(lambda e: e * np.float32(2.5)).to_narr(), exp)
    # map_with(b, 3) { |x, y, s| x * s - y }
    t, _ = ora.map_binary_scalar(ora.OP_MUL, a, 3, ora.I32)
    exp, _ = ora.map_binary(ora.OP_SUB, t, b)
    assert np.array_equal(A.map_with(B, 3, lambda x, y, s: x * s - y).to_narr(), exp)
    with pytest.raises(cu.ShapeError):
        A.map_with(cu.CuNArray.from_numpy(_f32([7, 128], 7)), lambda x, y: x + y)


def test_in_place_maps(cu, ora):
    shape = [10, 24, 9]
    a, b = _f32(shape, 8), _f32(shape, 9)
    B = cu.CuNArray.from_numpy(b)
    # NArray#map_with_index!
    X = cu.CuNArray.from_numpy(a)
    X.map_with_index_inplace(lambda e, i: e - i)
    exp, _ = ora.map_binary(ora.OP_SUB, a, ora.lex_index(shape))
    assert np.array_equal(X.to_narr(), exp)
    # Mutable#map! and #map_with! on an array
    X = cu.CuNArray.from_numpy(a)
    X.map_inplace(lambda e: e * e)
    sq, _ = ora.map_binary(ora.OP_MUL, a, a)
    assert np.array_equal(X.to_narr(), sq)
    X.map_with_inplace(B, np.float32(0.5), lambda e, y, s: e * s + y)
    t, _ = ora.map_binary_scalar(ora.OP_MUL, sq, np.float32(0.5), ora.F32)
    exp, _ = ora.map_binary(ora.OP_ADD, t, b)
    assert np.array_equal(X.to_narr(), exp)
    # Mutable#map_with_coord! through a MutableView (region + reversed axis)
    C = cu.CuNArray.from_numpy(a)
    M = C.mutable_view(cu.R(1, -2), slice(None), cu.R(None, None, -1))
    M.map_with_coord_inplace(lambda e, k: e + k[0] - k[2])
    c = a.copy()
    reg = np.ascontiguousarray(c[1:-1, :, ::-1])
    kk = ora.coords(reg.shape)
    t, _ = ora.map_binary(ora.OP_ADD, reg, kk[0])
    t, _ = ora.map_binary(ora.OP_SUB, t, kk[2])
    c[1:-1, :, ::-1] = t
    assert np.array_equal(C.to_narr(), c)
    # a read-only view has no in-place forms
    with pytest.raises(NotImplementedError):
        C.view().map_inplace(lambda e: e + 1)


def test_six_operand_depth_four_chain(cu, ora):
    """(((a*b) + (c*d)) * ((e - f) * (a + c))) - ((b * e) + (d * f)) over six
    distinct views: six inputs, nesting below the second stash level."""
    shape = [16, 31, 9]
    arrs = [_f32(shape, 10 + k) for k in range(6)]
    a, b, c, d, e, f = arrs
    D = [cu.CuNArray.from_numpy(x) for x in arrs]
    # view operands: two reversed, one permuted back and forth
    A_, B_, C_, D_, E_, F_ = D
    rev = (slice(None), cu.R(None, None, -1), slice(None))
    Av = A_.view(*rev)
    av = np.ascontiguousarray(a[:, ::-1, :])
    Ev = E_.view().permute(2, 1, 0).permute(2, 1, 0)
    P = Av.process()
    expr = (((P * B_) + (C_.process() * D_)) * ((Ev.process() - F_) * (P + C_))) - ((B_.process() * Ev) + (D_.process() * F_))
    got = expr.to_narr()
    M = lambda op, x, y: ora.map_binary(op, x, y)[0]
    exp = M(ora.OP_SUB,
            M(ora.OP_MUL, M(ora.OP_ADD, M(ora.OP_MUL, av, b), M(ora.OP_MUL, c, d)),
              M(ora.OP_MUL, M(ora.OP_SUB, e, f), M(ora.OP_ADD, av, c))),
            M(ora.OP_ADD, M(ora.OP_MUL, b, e), M(ora.OP_MUL, d, f)))
    assert np.array_equal(got, exp)
    # and a chain longer than one program: 30 operators over two arrays
    t = A_.process()
    ex = a
    for k in range(30):
        t = t * np.float32(0.5) + B_ if k % 2 == 0 else t - B_
        ex = (M(ora.OP_ADD, ora.map_binary_scalar(ora.OP_MUL, ex, np.float32(0.5), ora.F32)[0], b) if k % 2 == 0
              else M(ora.OP_SUB, ex, b))
    assert np.array_equal(t.to_narr(), ex)
