"""The C++ host mirror (ph-core_gb300/host/phase.hpp) on the device: views,
infix operators with Crystal's result types, fused chains (CuProcView: one
program per materialisation), reductions, chunk reads and writes, element
access, slices, comparisons, masked writes, equality, in-place maps and the
reference's exceptions, checked against the oracle on 16x12x10 Float32 and
Int32 arrays (bit-exact; sums within 1e-6 relative of the FP64 oracle)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE = (16, 12, 10)


def _cuda_lib_dir():
    """The directory holding libcudart.so of the toolkit nvcc belongs to."""
    import glob

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for d in [os.path.join(home, "lib64")] + sorted(glob.glob(os.path.join(home, "targets", "*", "lib"))):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(home, "lib64")


@pytest.fixture(scope="module")
def built(tmp_path_factory, cu):
    """(driver executable, work directory, input arrays)."""
    from phase_cu import synth

    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("hostcpp_dev")
    lib = os.path.join(ROOT, "ph-core_gb300", "phase_cu", "_lib")
    exe = str(d / "host_cpp_device")
    cmd = [gxx, "-std=c++17", "-O1", "-o", exe, os.path.join(ROOT, "tests", "host_cpp_device.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "host"),
           "-L", lib, "-lphcuda", "-Wl,-rpath," + lib, "-L", _cuda_lib_dir(), "-Wl,-rpath," + _cuda_lib_dir()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    n = int(np.prod(SHAPE))
    arrays = {
        "f32": (synth.uniform_f32(list(SHAPE), seed=4), synth.uniform_f32(list(SHAPE), seed=4, start=n)),
        "i32": (synth.uniform_i32(list(SHAPE), seed=4, lo=-1000, hi=1000),
                synth.uniform_i32(list(SHAPE), seed=4, lo=-1000, hi=1000, start=n)),
    }
    for tag, (a, b) in arrays.items():
        a.tofile(str(d / ("a." + tag)))
        b.tofile(str(d / ("b." + tag)))
    return exe, d, arrays


def _drive(built, *mode):
    exe, d, arrays = built
    p = subprocess.run([exe, str(d)] + list(mode), capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    lines = p.stdout.splitlines()

    def load(name, dtype):
        return np.fromfile(str(d / (name + ".bin")), dtype=dtype)

    return arrays, lines, load


@pytest.fixture(scope="module")
def run(built):
    return _drive(built)


@pytest.fixture(scope="module")
def run_proc(built):
    return _drive(built, "proc")


@pytest.fixture(scope="module")
def run_more(built):
    return _drive(built, "more")


@pytest.mark.parametrize("tag", ["f32", "i32"])
def test_element_access_slices_masks_equality_and_inplace_maps(run_more, ora, cu, tag):
    """get / set_element, slices(axis), the elementwise comparison as a Bool
    array, set_mask with a value and with a source view, equals? and the
    in-place maps map! and map_with! of the C++ mirror, against the oracle
    (bit-exact)."""
    arrays, lines, load = run_more
    a, b = arrays[tag]
    dt = a.dtype
    rb = np.ascontiguousarray(b[:, ::-1, :])
    m, _ = ora.map_binary_scalar(ora.OP_MUL, a, 3, ora.I32)
    m, _ = ora.map_binary_scalar(ora.OP_ADD, m, 1, ora.I32)
    assert m.dtype == dt
    assert np.array_equal(load(tag + "_map_inplace", dt), m.reshape(-1))
    w, _ = ora.map_binary_scalar(ora.OP_MUL, rb, 2, ora.I32)
    w, _ = ora.map_binary(ora.OP_SUB, a, w)
    assert np.array_equal(load(tag + "_map_with_inplace", dt), w.reshape(-1))
    assert np.array_equal(load(tag + "_get", dt), np.array([a[3, -1, 2], a[-16, 0, -1]], dtype=dt))
    f = a.copy()
    f[0, 0, 0] = 42
    f[-1, -1, -1] = -7
    assert np.array_equal(load(tag + "_set_element", dt), f.reshape(-1))
    assert "raised %s_get_index IndexError" % tag in lines
    assert "raised %s_get_dim DimensionError" % tag in lines
    assert "nslices %s 12" % tag in lines
    assert np.array_equal(load(tag + "_slice5", dt), ora.narray_fetch_chunk(a, [slice(None), 5]).reshape(-1))
    gt, _ = ora.map_binary(ora.OP_GT, a, b)
    mask = np.asarray(gt).reshape(-1).astype(bool)
    assert np.array_equal(load(tag + "_gt", np.uint8).astype(bool), mask)
    assert np.array_equal(load(tag + "_mask_value", dt), np.where(mask, dt.type(0), a.reshape(-1)))
    assert np.array_equal(load(tag + "_mask_src", dt), np.where(mask, rb.reshape(-1), a.reshape(-1)))
    assert "raised %s_mask_shape ShapeError" % tag in lines
    for what, expected in (("same", 1), ("other", 0), ("reversed", 1), ("shape", 0)):
        assert "equals %s %s %d" % (tag, what, expected) in lines


@pytest.mark.parametrize("tag", ["f32", "i32"])
def test_reshape_tile_concatenate_push_and_index_maps(run_more, ora, cu, tag):
    """View#reshape (affine, or copied first where strides cannot express the
    new shape), NArray#reshape, NArray.tile, NArray.concatenate, #push and the
    in-place maps with the element's index and coordinates of the C++ mirror,
    against the oracle (bit-exact)."""
    arrays, lines, load = run_more
    a, b = arrays[tag]
    dt = a.dtype
    rev = lambda x: np.ascontiguousarray(x[:, ::-1, :])  # noqa: E731
    assert np.array_equal(load(tag + "_reshape_perm", dt), np.transpose(a, (2, 0, 1)).reshape(-1))
    assert np.array_equal(load(tag + "_reshape_rows", dt), a[2:10].reshape(-1))
    assert np.array_equal(load(tag + "_reshape_rev", dt), rev(a).reshape(-1))
    assert np.array_equal(load(tag + "_reshape_array", dt), a.reshape(-1))
    assert "raised %s_reshape_size ShapeError" % tag in lines
    s = ora.narray_fetch_chunk(a, [cu.R(0, 3), cu.R(0, 4), cu.R(0, 5)])
    assert s.shape == (4, 5, 6)
    assert np.array_equal(load(tag + "_tile", dt), ora.tile(rev(s), [2, 3, 1]).reshape(-1))
    assert np.array_equal(load(tag + "_concat", dt), ora.concatenate([rev(a), b], 1).reshape(-1))
    assert "raised %s_concat_dim DimensionError" % tag in lines
    assert np.array_equal(load(tag + "_push", dt), ora.concatenate([a, b], 0).reshape(-1))
    index = np.arange(a.size, dtype=np.int32).reshape(a.shape)
    mi, _ = ora.map_binary(ora.OP_ADD, a, index)
    assert mi.dtype == dt
    assert np.array_equal(load(tag + "_map_with_index", dt), mi.reshape(-1))
    c0 = np.broadcast_to(np.arange(a.shape[0], dtype=np.int32)[:, None, None], a.shape).copy()
    c2 = np.broadcast_to(np.arange(a.shape[2], dtype=np.int32)[None, None, :], a.shape).copy()
    mc, _ = ora.map_binary(ora.OP_MUL, a, c0)
    mc, _ = ora.map_binary(ora.OP_SUB, mc, c2)
    assert np.array_equal(load(tag + "_map_with_coord", dt), mc.reshape(-1))


@pytest.mark.parametrize("tag", ["f32", "i32"])
def test_views_operators_and_chunks(run, ora, cu, tag):
    arrays, lines, load = run
    a, b = arrays[tag]
    dt = a.dtype
    perm, rev = [("permute", [2, 0, 1])], [("region", [slice(None), cu.R(None, None, -1), slice(None)])]
    oap, obp = ora.ViewOperand(a, perm), ora.ViewOperand(b, perm)
    oar, obr = ora.ViewOperand(a, rev), ora.ViewOperand(b, rev)
    assert np.array_equal(load(tag + "_perm", dt), ora.gather(oap).reshape(-1))
    assert np.array_equal(load(tag + "_rev", dt), ora.gather(oar).reshape(-1))
    assert np.array_equal(load(tag + "_add_perm", dt), ora.map_binary(ora.OP_ADD, oap, obp)[0].reshape(-1))
    assert np.array_equal(load(tag + "_sub_rev", dt), ora.map_binary(ora.OP_SUB, oar, obr)[0].reshape(-1))
    div = ora.map_binary(ora.OP_DIV, oap, obp)[0]
    assert div.dtype == (np.float32 if tag == "f32" else np.float64)  # Int32 / Int32 is Float64
    assert np.array_equal(load(tag + "_div_perm", div.dtype), div.reshape(-1), equal_nan=True)
    mul_op = ora.OP_MUL if tag == "f32" else ora.OP_WMUL
    assert np.array_equal(load(tag + "_mul_rev", dt), ora.map_binary(mul_op, oar, obr)[0].reshape(-1))
    t, _ = ora.map_binary_scalar(ora.OP_MUL, ora.gather(oap), dt.type(3), ora.F32 if tag == "f32" else ora.I32)
    t, _ = ora.map_binary_scalar(ora.OP_SUB, t, dt.type(7), ora.F32 if tag == "f32" else ora.I32, scalar_left=True)
    assert np.array_equal(load(tag + "_scal", dt), t.reshape(-1))
    chunk = ora.narray_fetch_chunk(a, [1, cu.R(0, 10, 3, True), cu.R(-1, 2)])
    assert chunk.shape == (4, 8)
    assert np.array_equal(load(tag + "_chunk", dt), chunk.reshape(-1))
    c = np.full([10, 16, 12], 5, dtype=dt)
    od = ora.ViewOperand(c, rev)
    ora.scatter(od, oap)
    c = od.arr
    c[2, 0:4, :] = -1
    assert np.array_equal(load(tag + "_scatter", dt), c.reshape(-1))
    for name, exc in (("_shape", "ShapeError"), ("_index", "IndexError"), ("_dim", "DimensionError")):
        assert "raised %s%s %s" % (tag, name, exc) in lines


@pytest.mark.parametrize("tag", ["f32", "i32"])
def test_reductions(run, ora, tag):
    arrays, _, load = run
    a, _ = arrays[tag]
    dt = a.dtype
    ap = np.ascontiguousarray(np.transpose(a, (2, 0, 1)))
    ar = np.ascontiguousarray(a[:, ::-1, :])
    for k in range(3):
        s = load(tag + "_sum%d" % k, dt)
        if tag == "f32":
            ref = ora.reduce_f64(ap, k).reshape(-1)
            mag = ora.reduce_f64(np.abs(ap), k).reshape(-1)
            assert np.all(np.abs(s - ref) <= 1e-6 * mag + 1e-30), k  # tolerance: 1e-6 of the sum of magnitudes
        else:
            assert np.array_equal(s, ora.reduce(ora.RED_SUM, ap, k).reshape(-1))
        assert np.array_equal(load(tag + "_max%d" % k, dt), ora.reduce(ora.RED_MAX, ar, k).reshape(-1))
        assert np.array_equal(load(tag + "_argmax%d" % k, np.int32),
                              ora.reduce(ora.RED_ARGMAX, ap, k, ora.I32).reshape(-1))
    full = load(tag + "_sumall", dt)[0]
    ref = ora.reduce_f64(a)
    if tag == "f32":
        assert abs(full - ref) <= 1e-6 * float(np.abs(a.astype(np.float64)).sum())
    else:
        assert full == int(ref)
    coord = load(tag + "_argmaxall", np.int64)
    assert list(coord) == list(np.unravel_index(int(ora.reduce(ora.RED_ARGMAX, ar)), ar.shape))


def test_checked_and_wrapping_int32(run):
    _, lines, load = run
    assert "raised overflow OverflowError" in lines
    assert np.all(load("wrapped", np.int32) == np.int32(-2 ** 31))


@pytest.mark.parametrize("tag", ["f32", "i32"])
def test_fused_chains(run_proc, ora, tag):
    """CuProcView: ((x + 4) ** 2) * y - z as one program, checked against the
    reference's one pass per operator; its permuted / reversed / chunked
    forms, reductions and writes."""
    arrays, lines, load = run_proc
    a, b = arrays[tag]
    dt = a.dtype
    t = ora.I32
    rev = lambda x: np.ascontiguousarray(x[:, ::-1, :])  # noqa: E731
    chain, _ = ora.map_binary_scalar(ora.OP_ADD, a, 4, t)
    chain, _ = ora.map_binary_scalar(ora.OP_POW, chain, 2, t)
    chain, _ = ora.map_binary(ora.OP_MUL, chain, rev(b))
    chain, _ = ora.map_binary(ora.OP_SUB, chain, rev(a))
    assert chain.dtype == dt
    assert np.array_equal(load(tag + "_proc_chain", dt), chain.reshape(-1))
    perm = np.transpose(chain, (2, 0, 1))[::-1, ::-1, ::-1]
    assert np.array_equal(load(tag + "_proc_chain_perm", dt), perm.reshape(-1))
    assert np.array_equal(load(tag + "_proc_chain_chunk", dt), chain[3, 0:10:3, :].reshape(-1))
    assert np.array_equal(load(tag + "_proc_chain_max1", dt), ora.reduce(ora.RED_MAX, chain, 1).reshape(-1))
    assert np.array_equal(load(tag + "_proc_chain_argmax0", np.int32),
                          ora.reduce(ora.RED_ARGMAX, chain, 0, ora.I32).reshape(-1))
    lin, _ = ora.map_binary_scalar(ora.OP_MUL, a, 3, t)
    lin, _ = ora.map_binary(ora.OP_SUB, lin, rev(b))
    s1 = load(tag + "_proc_sum1", dt)
    if tag == "f32":
        ref = ora.reduce_f64(lin, 1).reshape(-1)
        mag = ora.reduce_f64(np.abs(lin), 1).reshape(-1)
        assert np.all(np.abs(s1 - ref) <= 1e-6 * mag + 1e-30)  # tolerance: 1e-6 of the sum of magnitudes
    else:
        assert np.array_equal(s1, ora.reduce(ora.RED_SUM, lin, 1).reshape(-1))
    c = np.zeros_like(a)
    c[:, ::-1, :] = ora.map_binary(ora.OP_ADD, a, b)[0]
    assert np.array_equal(load(tag + "_proc_set", dt), c.reshape(-1))
    d = a.copy()
    d[:-1] = ora.map_binary_scalar(ora.OP_MUL, np.ascontiguousarray(a[1:]), 2, t)[0]
    assert np.array_equal(load(tag + "_proc_overlap", dt), d.reshape(-1))
    # the reference's element order would read rows already written: refused
    assert "raised %s_proc_overlap_behind NotImplementedError" % tag in lines
    assert np.all(load(tag + "_proc_const", np.float32) == np.float32(2.5))
    # five operand views: split into two device programs, same results
    five, _ = ora.map_binary(ora.OP_ADD, a, b)
    five, _ = ora.map_binary(ora.OP_MUL, five, ora.map_binary(ora.OP_SUB, rev(a), rev(b))[0])
    five, _ = ora.map_binary(ora.OP_ADD, five, np.ascontiguousarray(a[::-1, ::-1, ::-1]))
    assert np.array_equal(load(tag + "_proc_five", dt), five.reshape(-1))


def test_fused_mixed_types_and_checked_int32(run_proc, ora):
    arrays, lines, load = run_proc
    a, _ = arrays["f32"]
    ai, bi = arrays["i32"]
    m, _ = ora.map_binary_scalar(ora.OP_MUL, ai, 0.5, ora.F32)  # Int32 * Float32 -> Float32
    m, _ = ora.map_binary(ora.OP_ADD, m, a)
    m, _ = ora.map_binary_scalar(ora.OP_DIV, m, 3.0, ora.F64)  # Float32 / Float64 -> Float64
    assert m.dtype == np.float64
    assert np.array_equal(load("proc_mixed", np.float64), m.reshape(-1))
    ap = np.ascontiguousarray(np.transpose(ai, (2, 0, 1)))
    bp = np.ascontiguousarray(np.transpose(bi, (2, 0, 1)))
    q, _ = ora.map_binary(ora.OP_DIV, ap, bp)  # Int32 / Int32 -> Float64, zero divisors give Inf / NaN
    assert np.array_equal(load("proc_div", np.float64), q.reshape(-1), equal_nan=True)
    assert "raised proc_overflow OverflowError" in lines
    assert np.all(load("proc_wrapped", np.int32) == np.int32(2 ** 30))
