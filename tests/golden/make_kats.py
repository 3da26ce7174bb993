"""Writes tests/golden/reference_kats.json: the known-answer tests of the
reference's own spec suite (in-phase/ph-core spec/), transcribed as data.

The reference is Crystal and cannot run here, so its expected values are taken
from the spec files themselves (each entry cites spec file:line).  Literals are
encoded as {"i": n} for an integer index or {"f": first, "l": last, "s": step,
"x": exclusive} for a Crystal range (None = omitted endpoint).

Run: python tests/golden/make_kats.py
"""
import json
import os


def I(n):
    return {"i": n}


def Rg(f=None, l=None, s=None, x=False):
    return {"f": f, "l": l, "s": s, "x": x}


def test_ranges(bound):
    """TestRanges (spec/spec_helper.cr:64-193)."""
    mid = bound // 2
    full = [0, 1, bound - 1]
    fully_defined = [  # spec_helper.cr:66-93
        (Rg(mid, mid), [mid, 1, mid]),
        (Rg(None, mid), [0, 1, mid]),
        (Rg(None, mid, x=True), [0, 1, mid - 1]),
        (I(0), [0, 1, 0]),
        (I(bound - 1), [bound - 1, 1, bound - 1]),
        (Rg(mid, 0), [mid, -1, 0]),
        (Rg(mid, None, -1), [mid, -1, 0]),
        (Rg(0, bound, 2, True), [0, 2, bound - 1 - ((bound - 1) % 2)]),
        (Rg(0, bound - 1, 2, True), [0, 2, bound - 2 - (bound % 2)]),
        (Rg(5, 1, -3), [5, -3, 2]),
        (Rg(5, 1, -3), [5, -3, 2]),
        (Rg(bound - 1, 0, -1), [bound - 1, -1, 0]),       # (bound-1).step(by: -1, to: 0)
        (Rg(0, bound, 2, True), [0, 2, bound - 1 - ((bound - 1) % 2)]),
        (Rg(0, bound - 1, 2, True), [0, 2, bound - 2 - (bound % 2)]),
    ]
    implicit_bounds = [  # spec_helper.cr:96-111
        (Rg(), full),
        (Rg(x=True), full),
        (Rg(mid, None), [mid, 1, bound - 1]),
        (Rg(None, None, -1), [bound - 1, -1, 0]),
        (Rg(None, 2, -1, True), [bound - 1, -1, 3]),
        (Rg(None, None, -4), [bound - 1, -4, (bound - 1) % 4]),
        (Rg(None, None, -4), [bound - 1, -4, (bound - 1) % 4]),
    ]
    negative_indices = [  # spec_helper.cr:114-125
        (Rg(-bound, None), full),
        (Rg(None, -bound), [0, 1, 0]),
        (Rg(None, -1), full),
        (Rg(-mid, -mid + 2), [bound - mid, 1, bound - mid + 2]),
        (I(-mid), [bound - mid, 1, bound - mid]),
    ]
    out_of_bounds = [Rg(None, bound), Rg(bound, None), Rg(-bound - 1, None), Rg(None, -bound - 1),
                     Rg(None, bound + 1, x=True)]  # spec_helper.cr:127-135
    empty = [Rg(None, 0, x=True), Rg(3, 3, x=True)]  # spec_helper.cr:137-142
    step_conflict = [Rg(4, 2, 1), Rg(2, 4, -1), Rg(4, 2, 1), Rg(2, 4, -1)]  # spec_helper.cr:144-152
    return {
        "bound": bound,
        "fully_defined": fully_defined,
        "implicit_bounds": implicit_bounds,
        "negative_indices": negative_indices,
        "out_of_bounds": out_of_bounds,
        "empty": empty,
        "step_conflict": step_conflict,
    }


def kats():
    k = {"test_ranges": test_ranges(10)}
    # spec/index_region_spec.cr:64-77: [0..2..8, ..-1..] on [10, 4]
    k["region_multi_axis"] = {
        "literal": [Rg(0, 8, 2), Rg(None, None, -1)], "bound": [10, 4],
        "shape": [5, 4], "first": [0, 3], "last": [8, 0], "step": [2, -1],
        "bad_literal": [Rg(0, 3), Rg(0, 8, 2)],  # :74-76 -> IndexError
    }
    # spec/index_region_spec.cr:131-138 (absolute): [0..2..8, 3..-1..]
    k["region_absolute"] = {"literal": [Rg(0, 8, 2), Rg(3, None, -1)], "shape": [5, 4], "first": [0, 3],
                            "last": [8, 0], "step": [2, -1]}
    # spec/index_region_spec.cr:218-245: includes? on [3..5, 10..-2..2]
    k["region_includes"] = {
        "literal": [Rg(3, 5), Rg(10, 2, -2)],
        "excluded": [[6, 4], [2, 4], [4, 11], [4, 0], [0, 0], [4, 5]],
        "included": [[a, b] for a in range(3, 6) for b in range(10, 1, -2)],
    }
    # spec/index_region_spec.cr:258-263: fits_in? of [0..2..8, 3..-1..]
    k["region_fits_in"] = {"literal": [Rg(0, 8, 2), Rg(3, None, -1)], "fits": [[10, 4]], "not_fits": [[4, 10]]}
    # spec/index_region_spec.cr:308-339: translate! of [3..4..20, 7..-2..] by [-3, 5]
    k["region_translate"] = {"literal": [Rg(3, 20, 4), Rg(7, None, -2)], "offset": [-3, 5],
                             "raises": [[0, -2], [-4, 0]]}
    # spec/index_region_spec.cr:341-371: reverse! of [2..6, 8..-2..1]
    k["region_reverse"] = {"literal": [Rg(2, 6), Rg(8, 1, -2)], "first_after": [6, 2]}
    # spec/index_region_spec.cr:296-304: trim! of cover([20, 20]) to [10, 4]
    k["region_trim_cover"] = {"cover": [20, 20], "trim_to": [10, 4], "fits": [[10, 4]], "not_fits": [[4, 10]]}
    # spec/n_array_spec.cr:8 stock_narr = build(2,3) { |_, i| i }
    stock = [[0, 1, 2], [3, 4, 5]]
    k["narray_fetch_chunk"] = [  # spec/n_array_spec.cr:211-229
        {"literal": [I(1), Rg(0, 2, 2)], "expected": [3, 5]},
        {"literal": [I(-2), Rg(-1, 0)], "expected": [2, 1, 0]},
        {"literal": [Rg(0, 0, x=True), Rg(0, 0, x=True)], "expected_shape": [0, 0]},
    ]
    k["narray_set_chunk"] = [  # spec/n_array_spec.cr:238-295
        {"literal": [I(1), Rg(0, 2, 2)], "src": [6, 7], "expected": [[0, 1, 2], [6, 4, 7]]},
        {"literal": [I(-2), Rg(-1, 0)], "src": [6, 7, 8], "expected": [[8, 7, 6], [3, 4, 5]]},
        {"literal": [I(1), Rg(0, 2, 2)], "scalar": 6, "expected": [[0, 1, 2], [6, 4, 6]]},
        {"literal": [I(-2), Rg(-1, 0)], "scalar": 6, "expected": [[6, 6, 6], [3, 4, 5]]},
        {"literal": [Rg(0, 0, x=True), Rg(0, 0, x=True)], "scalar": 6, "expected": stock},
    ]
    k["narray_ops"] = {  # spec/n_array_spec.cr:297-333 (masks), 317-322, 444-466, 505-509
        "stock": stock,
        "plus_10": [[10, 11, 12], [13, 14, 15]],
        "pow_2": [[0, 1, 4], [9, 16, 25]],
        "times_2": [[0, 2, 4], [6, 8, 10]],
        "times_3": [[0, 3, 6], [9, 12, 15]],
        "mask": [[True, False, True], [False, True, False]],
        "mask_scalar_6": [[6, 1, 6], [3, 6, 5]],
        "mask_src_plus_10": [[10, 1, 12], [3, 14, 5]],
    }
    # spec/n_array_spec.cr:444-518: #map, #map_with_coord, #map_with_index and their in-place forms
    # on stock_narr (map { x ** 2 }; map_with_coord { 10 * c[0] + c[1] + el };
    # (stock_narr * 2).map_with_index { idx + el } == stock_narr * 3)
    k["narray_maps"] = {
        "stock": stock,
        "map_pow_2": [[0, 1, 4], [9, 16, 25]],
        "map_with_coord": [[0, 2, 4], [13, 15, 17]],
        "map_with_index_of_times_2": [[0, 3, 6], [9, 12, 15]],
    }
    k["serialization"] = {  # spec/n_array_spec.cr:520-557
        "stock_json": '{"shape":[2,3],"elements":[0,1,2,3,4,5]}',
        "empty_json": '{"shape":[0],"elements":[]}',
        "stock_yaml": "---\nshape: [2, 3]\nelements: [0, 1, 2, 3, 4, 5]\n",
        "empty_yaml": "---\nshape: [0]\nelements: []\n",
    }
    # README.md:36-61: narr + narr2, narr * narr2, argmax idiom
    k["readme"] = {"narr": [[1, 0, 0], [0, 1, 0]], "narr2": [[0, 1, 2], [10, 11, 12]],
                   "sum": [[1, 1, 2], [10, 12, 12]], "prod": [[0, 0, 0], [0, 11, 0]],
                   "argmax_narr2": [1, 2], "max_narr2": 12,
                   "slices_axis1": [[0, 10], [1, 11], [2, 12]]}
    k["transforms"] = {  # spec/view_util/*_transform_spec.cr
        "permute": {"coord": [3, 5, 2, 1, 0, 9, 4], "pattern": [2, 6, 5, 0, 1, 3, 4],
                    "expected": [1, 0, 3, 9, 4, 2, 5]},
        "reshape": {"src_shape": [3, 4], "new_shape": [6, 2], "coord": [2, 1], "expected": [1, 1]},
        "reverse": {"shape": [5, 3], "coord": [1, 2], "expected": [3, 0]},
    }
    # spec/multi_indexable/elem_iterator_spec.cr:7-67 and elem_coord_iterator_spec.cr:7-59:
    # NArray[[1, 2, 3], [4, 5, 6], [7, 8, 9]] iterated in lexicographic and
    # colexicographic order (elements, and elements with coordinates); reverse_each
    # yields each sequence backwards
    k["elem_iterators"] = {
        "narr": [[1, 2, 3], [4, 5, 6], [7, 8, 9]],
        "lex": [1, 2, 3, 4, 5, 6, 7, 8, 9],
        "lex_coords": [[0, 0], [0, 1], [0, 2], [1, 0], [1, 1], [1, 2], [2, 0], [2, 1], [2, 2]],
        "colex": [1, 4, 7, 2, 5, 8, 3, 6, 9],
        "colex_coords": [[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1], [0, 2], [1, 2], [2, 2]],
    }
    # spec/multi_writable_spec.cr:14-65 (Int32 payload; the spec's buffer mixes types)
    k["multi_writable"] = {"shape": [3, 4], "buffer": list(range(1, 13)), "literal": [Rg(1, None), Rg(1, None)],
                           "scalar": 10, "scalar_indices": [5, 6, 7, 9, 10, 11],
                           "chunk": [[10, 11, 12], [13, 14, 15]], "bad_literal": [Rg(2, None), Rg(2, None)]}
    # spec/coord_util_spec.cr:73-93 canonicalize_index on shape [0, 1, 10, Int32::MAX]
    imax, imin = 2 ** 31 - 1, -2 ** 31
    k["canonicalize_index"] = {
        "ok": [[9, 10, 9], [0, imax, 0], [imin + 1, imax, 0], [-10, 10, 0], [-1, 10, 9], [-1, 1, 0]],
        "raises": [[-2, 1], [0, 0]],
        "has_index_false": [[5, 5], [-6, 5], [0, 0], [imax, imax], [imin, imax]],
    }
    # spec/shape_util_spec.cr:4-52
    k["compatible_shapes"] = {
        "base": [[2, 5, 3], [1, 2, 1], [4, 6, 3, 2], [1, 1, 1], []],
        "compatible": [[2, 5, 3, 1, 1], [1, 2, 1, 1], [4, 6, 3, 2, 1, 1, 1, 1, 1], [1], []],
        "incompatible": [[2, 5], [2, 1, 1], [4, 3, 2, 1, 1, 1, 1, 1], [-2], [1]],
    }
    # Formatter output (colours off).  README.md:29-37: `puts narr`, `puts narr2`
    # (header line and body); src/multi_indexable/formatter/settings.cr:53-79:
    # the body printed for NArray.build([2, 2, 2, 2]) { |_, idx| idx } with
    # brackets [{"<", ">"}, {"begin", "end"}] (the doc comment shows no header).
    k["formatter"] = {
        "readme_narr": {"elements": [[1, 0, 0], [0, 1, 0]],
                        "text": "2x3 Phase::NArray(Int32)\n[[1, 0, 0],\n [0, 1, 0]]"},
        "readme_narr2": {"elements": [[0, 1, 2], [10, 11, 12]],
                         "text": "2x3 Phase::NArray(Int32)\n[[ 0,  1,  2],\n [10, 11, 12]]"},
        "brackets_4d": {
            "shape": [2, 2, 2, 2], "brackets": [["<", ">"], ["begin", "end"]],
            "body": "\n".join([
                "begin",
                "    <",
                "        begin< 0,  1>,",
                "             < 2,  3>end,",
                "        ",
                "        begin< 4,  5>,",
                "             < 6,  7>end",
                "    >,",
                "    <",
                "        begin< 8,  9>,",
                "             <10, 11>end,",
                "        ",
                "        begin<12, 13>,",
                "             <14, 15>end",
                "    >",
                "end"]),
        },
    }
    return k


if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(out, "w") as f:
        json.dump(kats(), f, indent=1)
    print("wrote", out)
