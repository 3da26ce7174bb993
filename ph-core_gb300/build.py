"""Builds libphcuda.so (every CUDA translation unit, sm_103a only) in-tree.

Usage: python ph-core_gb300/build.py   (or import and call build()).
The library lands in ph-core_gb300/phase_cu/_lib/libphcuda.so.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "phase_cu", "_lib")
BUILDDIR = os.path.join(HERE, "_build")
LIBNAME = "libphcuda.so"

SOURCES = ["runtime.cu", "plan.cu", "eval.cu", "eval_inst_u32_lo.cu", "eval_inst_u32_hi.cu", "eval_inst_u64_lo.cu",
           "eval_inst_u64_hi.cu", "reduce.cu", "stencil.cu", "batch.cu", "batch_k32n2.cu", "batch_k32n4.cu",
           "batch_k64.cu", "tuner.cu"]

# -fmad=false: no FMA contraction anywhere, so single Float32 operations round
# exactly as on the host; IEEE division and square root stay the default.
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
]


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src, extra):
    obj = os.path.join(BUILDDIR, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "phcuda.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc_path(), "-c", srcp, "-o", obj, "-I", os.path.join(ROOT, "include"), "-I", CSRC] + NVCC_FLAGS + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    return obj


def build(verbose=False, extra=None):
    """Compiles and links libphcuda.so; returns its path."""
    extra = list(extra or [])
    os.makedirs(BUILDDIR, exist_ok=True)
    os.makedirs(OUTDIR, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    out = os.path.join(OUTDIR, LIBNAME)
    cmd = [nvcc_path(), "-shared", "-o", out + ".tmp"] + objs + [
        "-gencode", "arch=compute_103a,code=sm_103a", "-lcudart", "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(out + ".tmp", out)
    if verbose:
        print("built", out)
    return out


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
