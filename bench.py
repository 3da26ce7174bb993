"""Benchmark of the device-array hot path (Phase CuNArray on one GB300).

Step (the 512x512x256 "large strided views" workload, Float32 and Int32):
  for each dtype:
    P  = A.view.permute(2, 0, 1).to_narr          gather, 256x512x512
    Rv = A[.., ..-1.., ..]                         gather, reversed axis 1
    for op in (+, -, *, /): A.view.permute(2,0,1) op B.view.permute(2,0,1)
    for op in (+, -, *, /): A[.., ..-1.., ..] op B[.., ..-1.., ..]
    C.mutable_view(.., ..-1.., ..)[..] = A.view.permute(2, 0, 1)   scatter
  Int32 `*` would overflow on these inputs (the reference raises OverflowError);
  the timed Int32 multiply is the wrapping `&*`.  Int32 `/` writes Float64.
value = algorithmic bytes of a step / step time (GB/s, 1e9), inputs resident in
HBM; every operand is 256 MiB or more, larger than L2, so no flush is needed.

Flags: --gpus N --steps K --warmup W [--impl reference] [--no-extra]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ph-core_gb300"))

import numpy as np  # noqa: E402

SHAPE = [512, 512, 256]
METRIC = "HBM GB/s vs ~8 TB/s peak; batched ops/s fused vs per-op launches, same GPU"
WORKLOAD = ("large strided views: Float32+Int32 512x512x256, permute(2,0,1) and reversed-axis-1 views, "
            "+ - * / on both view kinds, MutableView scatter")
CPU_SAMPLE_SHAPE = [128, 128, 64]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        load = [s for s in sm if smax and s > 0.3 * smax] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- device arm
def device_arm(args):
    import phase_cu as cu
    from phase_cu import _abi as A
    from phase_cu import synth

    cu.init(int(os.environ.get("LOCAL_RANK", "0")))
    cu.config.eager_errors = False
    lib = A.load()
    MiB = 1 << 20
    n = int(np.prod(SHAPE))
    arrays = {}
    for dt in ("f32", "i32"):
        if dt == "f32":
            a = synth.uniform_f32(SHAPE, seed=0)
            b = synth.uniform_f32(SHAPE, seed=0, start=n)
        else:
            a = synth.uniform_i32(SHAPE, seed=0, lo=-2 ** 20, hi=2 ** 20)
            b = synth.uniform_i32(SHAPE, seed=0, lo=-2 ** 20, hi=2 ** 20, start=n)
        arrays[dt] = (a, b)

    def build_jobs(dev):
        """Descriptors of every operation of one step (outputs preallocated)."""
        jobs = []
        for dt in ("f32", "i32"):
            A_, B_, C_ = dev[dt]
            es = 4
            ap = A_.view().permute(2, 0, 1)
            bp = B_.view().permute(2, 0, 1)
            ar = A_.view(slice(None), cu.R(None, None, -1), slice(None))
            br = B_.view(slice(None), cu.R(None, None, -1), slice(None))
            out_p = cu.CuNArray.empty([256, 512, 512], A_.dtype)
            out_r = cu.CuNArray.empty(SHAPE, A_.dtype)
            out64_p = cu.CuNArray.empty([256, 512, 512], cu.Float64)
            out64_r = cu.CuNArray.empty(SHAPE, cu.Float64)
            jobs.append(("gather_permute", "copy", (out_p._view(), ap._cview()), 2 * n * es, [out_p]))
            jobs.append(("gather_reverse", "copy", (out_r._view(), ar._cview()), 2 * n * es, [out_r]))
            ops = [A.OP_ADD, A.OP_SUB, A.OP_MUL if dt == "f32" else A.OP_WMUL, A.OP_DIV]
            for kind, (x, y, o, o64) in (("permute", (ap, bp, out_p, out64_p)), ("reverse", (ar, br, out_r, out64_r))):
                for op in ops:
                    out = o64 if (op == A.OP_DIV and dt == "i32") else o
                    nbytes = 2 * n * es + n * (8 if out is o64 else es)
                    jobs.append(("binary_" + kind, "binary", (op, x._cview(), y._cview(), out._view()), nbytes,
                                 [out]))
            mv = C_.mutable_view(slice(None), cu.R(None, None, -1), slice(None))
            jobs.append(("scatter", "copy", (mv._cview(), ap._cview()), 2 * n * es, [C_]))
        return jobs

    def run_job(j):
        name, kind, a, nbytes, _ = j
        if kind == "copy":
            rc = lib.phcu_copy(ctypes.byref(a[0]), ctypes.byref(a[1]))
        else:
            rc = lib.phcu_binary(a[0], ctypes.byref(a[1]), ctypes.byref(a[2]), ctypes.byref(a[3]))
        if rc:
            A.check(rc, name)

    dev = {}
    for dt, (a, b) in arrays.items():
        Ad = cu.CuNArray.from_numpy(a)
        Bd = cu.CuNArray.from_numpy(b)
        Cd = cu.CuNArray.empty([256, 512, 512], Ad.dtype)
        dev[dt] = (Ad, Bd, Cd)
    jobs = build_jobs(dev)
    step_bytes = sum(j[3] for j in jobs)

    def timer():
        t = ctypes.c_void_p()
        A.check(lib.phcu_timer_start(ctypes.byref(t)))
        return t

    def stop(t):
        ms = ctypes.c_float()
        A.check(lib.phcu_timer_stop(t, ctypes.byref(ms)))
        return ms.value

    A.call("phcu_sync")
    for _ in range(args.warmup):
        for j in jobs:
            run_job(j)
    A.call("phcu_sync")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # replicas only: one barrier, a max of times
        dist.init_process_group("nccl" if args.gpus > 1 else "gloo")
        dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    c0 = ctypes.c_uint64()
    lib.phcu_launch_count(ctypes.byref(c0))
    A.call("phcu_sync")
    t = timer()
    for _ in range(args.steps):
        for j in jobs:
            run_job(j)
    ms = stop(t)
    c1 = ctypes.c_uint64()
    lib.phcu_launch_count(ctypes.byref(c1))
    A.call("phcu_sync")
    clk = clocks.stop()
    if dist is not None:
        import torch
        tt = torch.tensor([ms], dtype=torch.float64, device="cuda" if args.gpus > 1 else "cpu")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    ms_per_step = ms / args.steps
    value = step_bytes * world / (ms_per_step * 1e-3) / 1e9

    # per-class kernel timing (same launches, one class at a time) for the roofline
    classes = {}
    for j in jobs:
        classes.setdefault(j[0], []).append(j)
    per_class = {}
    reps = max(3, args.steps)
    for name, js in classes.items():
        t = timer()
        for _ in range(reps):
            for j in js:
                run_job(j)
        cms = stop(t) / reps
        cb = sum(j[3] for j in js)
        per_class[name] = {"ms": cms, "launches": len(js), "bytes": cb, "gbs": cb / (cms * 1e-3) / 1e9}
    dom = max(per_class.items(), key=lambda kv: kv[1]["ms"])
    peak, peak_kind = peaks()
    dom_ms_per_launch = dom[1]["ms"] / dom[1]["launches"]
    dom_bytes_per_launch = dom[1]["bytes"] / dom[1]["launches"]
    achieved = dom_bytes_per_launch / (dom_ms_per_launch * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "bytes_per_launch": int(dom_bytes_per_launch), "ms_per_launch": round(dom_ms_per_launch, 4),
                "traffic": None, "step_frac": round(value / world / peak, 4),
                "per_class_gbs": {k: round(v["gbs"], 1) for k, v in per_class.items()}}

    # ------------------------------------------------------------ e2e
    e2e = e2e_leg(A, lib, arrays, dev, jobs, args, timer, stop, step_bytes)

    result = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (SplitMix64, seed 0)",
        "config": {"workload": WORKLOAD, "shape": SHAPE, "bytes_per_step": step_bytes,
                   "l2": "inputs larger than L2 (256 MiB operands), no flush", "parallelism": "replicas"},
        "gpu_launches": int(c1.value - c0.value), "roofline": roofline, "clocks": clk, "e2e": e2e,
    }
    return result, rank


def e2e_leg(A, lib, arrays, dev_arrays, jobs, args, timer, stop, step_bytes):
    """Same step through the C-ABI with pinned HOST buffers: inputs uploaded and
    every result downloaded inside the timed region."""
    def pinned(nbytes):
        p = ctypes.c_void_p()
        A.check(lib.phcu_host_alloc(nbytes, ctypes.byref(p)))
        return p.value

    host_in = {}
    for dt, (a, b) in arrays.items():
        pa, pb = pinned(a.nbytes), pinned(b.nbytes)
        ctypes.memmove(pa, a.ctypes.data, a.nbytes)
        ctypes.memmove(pb, b.ctypes.data, b.nbytes)
        host_in[dt] = (pa, pb, a.nbytes)
    host_out = pinned(max(j[4][0]._buf.nbytes for j in jobs))

    def one_step(dev_arrays):
        for dt in ("f32", "i32"):
            pa, pb, nb = host_in[dt]
            Ad, Bd, _ = dev_arrays[dt]
            A.check(lib.phcu_upload(Ad._buf.ptr, pa, nb))
            A.check(lib.phcu_upload(Bd._buf.ptr, pb, nb))
        for j in jobs:
            name, kind, a, nbytes, outs = j
            if kind == "copy":
                A.check(lib.phcu_copy(ctypes.byref(a[0]), ctypes.byref(a[1])))
            else:
                A.check(lib.phcu_binary(a[0], ctypes.byref(a[1]), ctypes.byref(a[2]), ctypes.byref(a[3])))
            o = outs[0]
            A.check(lib.phcu_download(host_out, o._buf.ptr, o._buf.nbytes))

    one_step(dev_arrays)
    A.call("phcu_sync")
    steps = max(1, min(args.steps, 5))
    t = timer()
    for _ in range(steps):
        one_step(dev_arrays)
    ms = stop(t) / steps
    h2d = sum(2 * v[2] for v in host_in.values())
    d2h = sum(j[4][0]._buf.nbytes for j in jobs)
    for v in host_in.values():
        lib.phcu_host_free(v[0])
        lib.phcu_host_free(v[1])
    lib.phcu_host_free(host_out)
    return {"value": round(step_bytes / (ms * 1e-3) / 1e9, 1), "unit": "GB/s", "ms_per_step": round(ms, 3),
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps,
            "path": "phcu_upload/phcu_copy/phcu_binary/phcu_download on pinned host buffers"}


# ------------------------------------------------------------ CPU baseline
def cpu_workload(nthreads, shape=CPU_SAMPLE_SHAPE):
    """The same step on the oracle (the reference's loops restated in C): one
    materialised pass per operation, per-element view transforms."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    from phase_cu import synth
    from phase_cu.region import R

    ora.build()
    n = int(np.prod(shape))
    total_bytes = 0
    t0 = time.perf_counter()
    for dt in ("f32", "i32"):
        if dt == "f32":
            a = synth.uniform_f32(shape, seed=0)
            b = synth.uniform_f32(shape, seed=0, start=n)
        else:
            a = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20)
            b = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20, start=n)
        es = 4
        perm = [("permute", [2, 0, 1])]
        rev = [("region", [slice(None), R(None, None, -1), slice(None)])]
        ap, bp = ora.ViewOperand(a, perm), ora.ViewOperand(b, perm)
        ar, br = ora.ViewOperand(a, rev), ora.ViewOperand(b, rev)
        ora.gather(ap, nthreads)
        ora.gather(ar, nthreads)
        total_bytes += 4 * n * es
        ops = [ora.OP_ADD, ora.OP_SUB, ora.OP_MUL if dt == "f32" else ora.OP_WMUL, ora.OP_DIV]
        for x, y in ((ap, bp), (ar, br)):
            for op in ops:
                ora.map_binary(op, x, y, nthreads)
                total_bytes += 2 * n * es + n * (8 if (op == ora.OP_DIV and dt == "i32") else es)
        c = np.zeros([shape[2], shape[0], shape[1]], dtype=a.dtype)
        ora.scatter(ora.ViewOperand(c, rev), ap)
        total_bytes += 2 * n * es
    dt_s = time.perf_counter() - t0
    return total_bytes / dt_s / 1e9, dt_s, total_bytes


def cpu_baseline(nthreads):
    gbs, secs, nbytes = cpu_workload(nthreads)
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": nthreads, "kind": "port",
            "sample": "the same step on Float32+Int32 %s arrays (1/64 of the elements), %.1f s, %d algorithmic bytes"
                      % ("x".join(map(str, CPU_SAMPLE_SHAPE)), secs, nbytes)}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None, rank
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_workload(threads)
    for _ in range(args.steps):
        gbs, secs, nbytes = cpu_workload(threads)
        vals.append((gbs, secs, nbytes))
    gbs = sum(v[2] for v in vals) / sum(v[1] for v in vals) / 1e9
    ms = 1e3 * sum(v[1] for v in vals) / len(vals)
    res = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (SplitMix64, seed 0)",
           "config": {"workload": WORKLOAD, "shape": SHAPE, "sample_shape": CPU_SAMPLE_SHAPE,
                      "l2": "n/a (CPU)", "parallelism": "host threads"},
           "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                            "sample": "each step = the step on %s arrays (1/64 of the elements); the reference is "
                                      "Crystal and cannot be built here, so its loops run as the C oracle"
                                      % "x".join(map(str, CPU_SAMPLE_SHAPE))},
           "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return res, rank


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours")
    p.add_argument("--no-cpu", action="store_true")
    args = p.parse_args()
    if args.impl == "reference":
        res, rank = reference_arm(args)
        if rank == 0 and res:
            print(json.dumps(res), flush=True)
        return
    res, rank = device_arm(args)
    if rank == 0:
        if not args.no_cpu:
            res["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
