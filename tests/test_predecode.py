"""Host-side pre-decoding of fused programs (program.cuh): which instructions
get a pre-decoded Float32/Int32 form, the conversion of Int32 immediates of
Float32 operators (round to nearest even, as the device converts), and which
programs qualify for the reduced interpreter.  A small host-only program is
compiled with nvcc against the library's header and run; no GPU is used."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cases(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("predecode") / "predecode_check")
    # the header's device code needs sm_103a; only the host main runs
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
           os.path.join(ROOT, "tests", "predecode_check.cu"), "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "ph-core_gb300", "csrc"),
           "--expt-relaxed-constexpr"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    lines = [json.loads(x) for x in out.splitlines() if x.strip()]
    names = lines[0]["names"]
    return names, {c["case"]: c for c in lines[1:]}


def _f32_bits(v):
    return int(np.array([v], dtype=np.int32).astype(np.float32).view(np.uint32)[0])


def test_config3_chain(cases):
    n, c = cases
    ch = c["chain"]
    assert ch["fx"] == [n["FX_F32_LD"], n["FX_F32_ADD"], n["FX_NONE"], n["FX_F32_MUL"], n["FX_F32_SUB"]]
    assert ch["is_fx"] == 1  # the power with an immediate exponent keeps its own path
    assert ch["btype"][1] == 3 and ch["imm"][1] == _f32_bits(4)  # Int32 4 -> Float32 4.0f
    assert ch["btype"][2] == 1 and ch["imm"][2] == 2  # the exponent stays Int32


def test_swapped_and_commutative_forms(cases):
    n, c = cases
    assert c["swapped_f32"]["fx"] == [n["FX_F32_LD"], n["FX_F32_RSUB"], n["FX_F32_RDIV"], n["FX_F32_ADD"],
                                      n["FX_F32_MUL"]]
    assert c["int32_forms"]["fx"] == [n["FX_I32_LD"], n["FX_I32_RSUB"], n["FX_I32_RWSUB"], n["FX_I32_WSUB"],
                                      n["FX_I32_WADD"], n["FX_I32_WMUL"], n["FX_I32_AND"], n["FX_I32_OR"],
                                      n["FX_I32_XOR"], n["FX_I32_MUL"], n["FX_I32_ADD"]]
    assert c["int32_forms"]["is_fx"] == 1


def test_general_instructions_keep_the_interpreter(cases):
    n, c = cases
    for name in ("general", "float64", "stash", "f64_immediate", "conversion", "garbage"):
        assert c[name]["is_fx"] == 0, name
    assert c["general"]["fx"][1] == n["FX_NONE"]
    assert c["float64"]["fx"] == [n["FX_NONE"], n["FX_NONE"]]
    assert c["stash"]["fx"][1] == n["FX_NONE"]
    # only Int32 immediates are converted; a Float64 immediate stays as it is
    assert c["f64_immediate"]["fx"][1] == n["FX_NONE"] and c["f64_immediate"]["btype"][1] == 4
    assert c["swapped_pow"]["is_fx"] == 0
    # caller-provided pad bytes are overwritten
    assert c["conversion"]["fx"] == [n["FX_I32_LD"], n["FX_NONE"]]
    assert c["garbage"]["fx"] == [n["FX_F32_LD"], n["FX_NONE"]]


def test_int32_immediates_round_to_nearest_even(cases):
    _, c = cases
    imm = c["immediates"]
    assert imm["btype"][1:] == [3, 3, 3]
    assert imm["imm"][1:] == [_f32_bits(-3), _f32_bits(16777217), _f32_bits(16777219)]
    assert _f32_bits(16777217) == 0x4B800000 and _f32_bits(16777219) == 0x4B800002
