"""Overlapping writes: the host rule that decides whether writing a source that
aliases its destination element by element in lexicographic order (the
reference's MultiWritable#unsafe_set_chunk, src/multi_writable.cr:29-44, and
Mutable#map_with!, src/multi_indexable/mutable.cr:54-67) can differ from
reading the whole source first (what the device does).

Checked on the CPU: random region / reverse / permute views of one 2-D array
are scattered into each other by the oracle's sequential scatter (the
reference's element order) and by a staged copy; whenever the rule says
"same", the two results are equal (the rule is sound), with the exact
per-element check and with the address-order rule used for large views.  The
classic differing patterns are recognised."""
import numpy as np
import pytest

BASE = [8, 9]


class _Buf:
    def __init__(self, ptr):
        self.ptr = ptr


def _rand_lits(rng, shape):
    """A region literal per axis, or None when the draw is empty."""
    lits, out = [], []
    for n in shape:
        step = int(rng.choice([-3, -2, -1, 1, 2, 3]))
        first = int(rng.integers(0, n))
        room = first if step < 0 else n - 1 - first
        count = int(rng.integers(1, room // abs(step) + 2))
        lits.append((first, first + (count - 1) * step, step))
        out.append(count)
    return lits, out


def _transforms(cu, lits, permute, reverse):
    tf = [("region", [cu.R(f, l, s) for f, l, s in lits])]
    if permute:
        tf.append(("permute", [1, 0]))
    if reverse:
        tf.append(("reverse",))
    return tf


def _affine(cu, tf):
    """The descriptor the product folds the same chain into."""
    from phase_cu import narray
    from phase_cu.region import IndexRegion

    off, shape, stride = 0, list(BASE), [BASE[1], 1]
    for t in tf:
        if t[0] == "region":
            off, shape, stride = narray._affine_region(off, shape, stride, IndexRegion.new(t[1], shape))
        elif t[0] == "permute":
            off, shape, stride = narray._affine_permute(off, shape, stride, t[1])
        else:
            off, shape, stride = narray._affine_reverse(off, shape, stride)
    return off, shape, stride


def _draw(cu, rng):
    lits, shape = _rand_lits(rng, BASE)
    perm = bool(rng.integers(0, 2))
    rev = bool(rng.integers(0, 2))
    return _transforms(cu, lits, perm, rev), (shape[::-1] if perm else shape)


@pytest.mark.parametrize("exact", [True, False])
def test_rule_is_sound_against_the_sequential_order(ora, exact, monkeypatch):
    import phase_cu as cu
    from phase_cu import narray

    if not exact:
        monkeypatch.setattr(narray, "_ALIAS_EXACT_LIMIT", 0)
    rng = np.random.default_rng(11)
    base = np.arange(100, 100 + BASE[0] * BASE[1], dtype=np.int32).reshape(BASE)
    B = _Buf(0x1000)
    tried = flagged = 0
    while tried < 1500:
        tf_d, shape_d = _draw(cu, rng)
        tf_s, shape_s = _draw(cu, rng)
        if shape_d != shape_s:
            continue
        tried += 1
        # the reference's order: both views over one buffer, written in place
        seq = base.copy()
        ora.scatter(ora.ViewOperand(seq, tf_d), ora.ViewOperand(seq, tf_s))
        # the device's order: the whole source read first
        staged = base.copy()
        src_vals = ora.gather(ora.ViewOperand(base, tf_s))
        ora.scatter(ora.ViewOperand(staged, tf_d), ora.ViewOperand(src_vals))
        od, sd, std = _affine(cu, tf_d)
        os_, ss, sts = _affine(cu, tf_s)
        differs = narray._sequential_order_differs((B, od, sd, std), (B, os_, ss, sts))
        if differs:
            flagged += 1
        else:
            assert np.array_equal(seq, staged), (tf_d, tf_s)
    assert flagged >= 10  # the draws exercise both outcomes


def test_classic_patterns():
    from phase_cu import narray

    B = _Buf(0x1000)
    rows = (B, 8, [3, 8], [8, 1])  # rows 1..3 of a 4x8 array
    # a source one row before the destination: the reference propagates row 0
    assert narray._sequential_order_differs(rows, (B, 0, [3, 8], [8, 1]))
    # one row after: every read comes before the write that reaches it
    assert not narray._sequential_order_differs((B, 0, [3, 8], [8, 1]), rows)
    # the same region reversed
    assert narray._sequential_order_differs((B, 0, [10], [1]), (B, 9, [10], [-1]))
    # an in-place transpose of a square block
    assert narray._sequential_order_differs((B, 0, [4, 4], [4, 1]), (B, 0, [4, 4], [1, 4]))
    # identical mappings and disjoint views
    assert not narray._sequential_order_differs((B, 3, [5, 2], [2, 1]), (B, 3, [5, 2], [2, 1]))
    assert not narray._sequential_order_differs((B, 0, [5], [1]), (B, 5, [5], [1]))
    # different buffers never alias
    assert not narray._sequential_order_differs((B, 0, [5], [1]), (_Buf(0x2000), 0, [5], [-1]))
