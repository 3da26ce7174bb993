"""Formatter of device arrays (src/multi_indexable/formatter/): layout and
element text against the reference's printed examples and against the oracle's
literal restatement of the reference's walk (which reads the whole array and
reproduces the reference's coordinate jump), and on the GPU the device gather
of the displayed elements."""
import os

import numpy as np
import pytest

from phase_cu import formatter as F

import formatter_oracle as FO


@pytest.fixture(autouse=True)
def _no_colour():
    old = F.Colorize.enabled
    F.Colorize.enabled = False
    yield
    F.Colorize.enabled = old


def _settings(**kw):
    s = F.Settings.default()
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _oracle_settings(s):
    return {"indent_width": s.indent_width, "max_element_width": s.max_element_width, "omit_after": s.display_limit,
            "brackets": s.brackets, "collapse_brackets_after": s.collapse_height, "integer_format": s.integer_format,
            "decimal_format": s.decimal_format}


def test_readme_examples(kats):
    for key in ("readme_narr", "readme_narr2"):
        k = kats["formatter"][key]
        a = np.array(k["elements"], dtype=np.int32)
        assert F.Formatter.print(a, F.Settings.default()) == k["text"]
        assert "2x3 Phase::NArray(Int32)\n" + FO.format_body(a) == k["text"]


def test_bracket_settings_example(kats):
    k = kats["formatter"]["brackets_4d"]
    a = np.arange(16, dtype=np.int32).reshape(k["shape"])
    s = _settings(brackets=[tuple(b) for b in k["brackets"]])
    text = F.Formatter.print(a, s)
    assert text.split("\n", 1)[1] == k["body"]
    assert FO.format_body(a, _oracle_settings(s)) == k["body"]


def _random_case(rng):
    rank = int(rng.integers(1, 5))
    shape = [int(rng.choice([0, 1, 2, 3, 5, 7, 11, 13, 40])) if rng.random() < 0.9 else 0 for _ in range(rank)]
    kind = rng.choice(["f32", "f64", "i32", "i64", "bool"])
    n = int(np.prod(shape))
    if kind in ("f32", "f64"):
        vals = rng.standard_normal(n) * 10.0 ** rng.integers(-6, 9, n)
        vals[rng.random(n) < 0.05] = np.nan
        vals[rng.random(n) < 0.03] = -np.inf
        a = vals.astype(np.float32 if kind == "f32" else np.float64)
    elif kind == "bool":
        a = rng.random(n) < 0.5
    else:
        a = rng.integers(-10 ** 9, 10 ** 9, n).astype(np.int32 if kind == "i32" else np.int64)
    a = a.reshape(shape)
    limits = [int(x) for x in rng.integers(3, 12, int(rng.integers(1, 4)))]
    s = _settings(display_limit=limits, collapse_height=int(rng.integers(0, 6)),
                  max_element_width=int(rng.integers(4, 16)), indent_width=int(rng.integers(1, 5)),
                  brackets=[("[", "]"), ("(%d:", ")")][: int(rng.integers(1, 3))])
    return a, s


def test_host_formatter_matches_oracle_walk():
    rng = np.random.default_rng(7)
    for _ in range(300):
        a, s = _random_case(rng)
        body = F.Formatter.print(a, s).split("\n", 1)[1]
        assert body == FO.format_body(a, _oracle_settings(s)), (a.shape, a.dtype, s.display_limit)


def test_displayed_ranges_are_what_the_reference_walk_reads():
    """The oracle walk reads elements one at a time through the reference's
    iterator; record which coordinates it visits and compare with the ranges
    the device gather copies."""
    rng = np.random.default_rng(3)
    for _ in range(100):
        a, s = _random_case(rng)
        if a.size == 0:
            continue
        f = FO.OracleFormatter(a, _oracle_settings(s))
        seen = []
        nxt = f.it.next

        def spy():
            c = nxt()
            seen.append(tuple(c))
            return c

        f.it.next = spy
        f.just = s.max_element_width
        f.measure()
        ranges = F.displayed_ranges(list(a.shape), s)
        idx = [np.concatenate([np.arange(x, y) for x, y in r]) for r in ranges]
        expect = [tuple(int(v) for v in c) for c in np.stack(np.meshgrid(*idx, indexing="ij"), -1).reshape(-1, a.ndim)]
        assert seen == expect


def test_literal_text():
    a = np.array([[1.5, -0.0, 1e-5], [2e20, np.nan, np.inf]], dtype=np.float64)
    assert F.Formatter.print_literal(a) == FO.format_literal(a)
    assert F.Formatter.print_literal(a) == "[[1.5, -0.0, 1.0e-5], [2.0e+20, NaN, Infinity]]"
    b = np.array([0.1, 3.0], dtype=np.float32)
    assert F.Formatter.print_literal(b) == "[0.1, 3.0]"


def test_colours_follow_heights():
    F.Colorize.enabled = True
    a = np.arange(6, dtype=np.int32).reshape(2, 3)
    text = F.Formatter.print(a, F.Settings.default())
    red, yellow = "\x1b[31m", "\x1b[33m"
    # header: the first dimension takes colors[(2 - 0 + 1) % 3] = red, the last none
    assert text.startswith(red + "2\x1b[0mx3 Phase::NArray(Int32)\n")
    # rows (height 1) yellow, elements' brackets (height 0) red
    assert (yellow + "[\x1b[0m" + red + "[\x1b[0m0, 1, 2" + red + "]\x1b[0m" + yellow + ",\x1b[0m") in text


def test_settings_yaml_and_user_file(tmp_path, monkeypatch):
    s = F.Settings.default()
    s.colors = ["red", (0x12, 0xAB, 0xFF)]
    s.brackets = [("[", "]"), ("<%d|", ">")]
    t = F.Settings.from_yaml(s.to_yaml())
    assert vars(t) == vars(s)
    with pytest.raises(F.FormatterError):
        F.Settings.from_yaml(s.to_yaml().replace("red", "reddish"))
    (tmp_path / "formatter.yaml").write_text(s.to_yaml())
    monkeypatch.setenv("PHASE_CONFIG_DIR", str(tmp_path))
    monkeypatch.setattr(F.Settings, "_cached_user_settings", None)
    monkeypatch.setattr(F.Settings, "_disable_user_settings", False)
    monkeypatch.setattr(F.Settings, "project_settings", None)
    assert vars(F.Settings.new()) == vars(s)
    monkeypatch.setattr(F.Settings, "project_settings", F.Settings.default())
    assert F.Settings.new().brackets == [("[", "]")]


def test_small_display_limits_refused():
    with pytest.raises(ValueError):
        F.displayed_ranges([10], _settings(display_limit=[2]))


# ------------------------------------------------------------------ device
@pytest.mark.gpu
def test_device_to_s_gathers_only_displayed(cu):
    rng = np.random.default_rng(11)
    for _ in range(40):
        a, s = _random_case(rng)
        if a.dtype == np.float64 and a.size == 0:
            continue
        X = cu.CuNArray.from_numpy(np.ascontiguousarray(a))
        text = X.to_s(s)
        name = "Phase::CuNArray(%s)" % {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64",
                                        np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64",
                                        np.dtype(np.bool_): "Bool"}[a.dtype]
        head, body = text.split("\n", 1)
        assert head.endswith(name)
        assert body == FO.format_body(a, _oracle_settings(s))
        got = F.gather_displayed(X, s)
        ranges = F.displayed_ranges(list(a.shape), s)
        assert list(got.shape) == [sum(y - x for x, y in r) for r in ranges]


@pytest.mark.gpu
def test_device_views_print_like_their_host_copy(cu):
    a = (np.random.default_rng(5).standard_normal((30, 17, 12)) * 100).astype(np.float32)
    X = cu.CuNArray.from_numpy(a)
    v = X.view().permute(2, 0, 1).reverse()
    host = np.ascontiguousarray(np.transpose(a, (2, 0, 1))[::-1, ::-1, ::-1])
    s = F.Settings.default()
    assert str(v).split("\n", 1)[1] == FO.format_body(host, _oracle_settings(s))
    assert v.to_literal_s() == FO.format_literal(host)
    assert str(X[cu.R(1, -1, 2), 3]).split("\n", 1)[1] == FO.format_body(a[1::2, 3], _oracle_settings(s))


@pytest.mark.gpu
def test_device_proc_view_prints_its_displayed_elements(cu):
    """A lazy ProcView gathers the displayed elements of its operands and runs
    its fused program on those alone; the text equals the full result's."""
    rng = np.random.default_rng(9)
    a = (rng.standard_normal((40, 33, 21)) * 10).astype(np.float32)
    b = (rng.standard_normal((40, 33, 21)) * 10).astype(np.float32)
    X, Y = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
    pv = X.view().process(lambda e: (e + 4) ** 2) * Y.view().reverse() - X.view()
    full = pv.to_narr()
    s = F.Settings.default()
    assert str(pv).split("\n", 1)[1] == FO.format_body(full, _oracle_settings(s))
    small = X.view(slice(0, 3), 0, slice(0, 4)).process(lambda e: e * 2)
    assert str(small).split("\n", 1)[1] == FO.format_body(small.to_narr(), _oracle_settings(s))
