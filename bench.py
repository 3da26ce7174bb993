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


def bench_config():
    """The workload both arms measure (the device arm and --impl reference)."""
    return {"workload": WORKLOAD, "shape": SHAPE, "dtypes": ["Float32", "Int32"],
            "l2": "inputs larger than L2 (256 MiB operands), no flush", "parallelism": "replicas"}


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
        return make_jobs(cu, A, dev, n)

    def run_job(j):
        execute_job(lib, A, j)

    dev = {}
    for dt, (a, b) in arrays.items():
        Ad = cu.CuNArray.from_numpy(a)
        Bd = cu.CuNArray.from_numpy(b)
        Cd = cu.CuNArray.empty([256, 512, 512], Ad.dtype)
        dev[dt] = (Ad, Bd, Cd)
    jobs = build_jobs(dev)
    step_bytes = sum(j[3] for j in jobs)
    return _device_timed(args, cu, A, lib, arrays, dev, jobs, run_job, step_bytes)


def make_jobs(cu, A, dev, n, shape=SHAPE):
    """Descriptors of every operation of one step (outputs preallocated).
    dev maps dtype tag -> (A, B, C) device arrays."""
    if True:
        jobs = []
        for dt in dev:
            A_, B_, C_ = dev[dt]
            es = 4
            ap = A_.view().permute(2, 0, 1)
            bp = B_.view().permute(2, 0, 1)
            ar = A_.view(slice(None), cu.R(None, None, -1), slice(None))
            br = B_.view(slice(None), cu.R(None, None, -1), slice(None))
            pshape = [shape[2], shape[0], shape[1]]
            out_p = cu.CuNArray.empty(pshape, A_.dtype)
            out_r = cu.CuNArray.empty(shape, A_.dtype)
            out64_p = cu.CuNArray.empty(pshape, cu.Float64)
            out64_r = cu.CuNArray.empty(shape, cu.Float64)
            jobs.append(("gather_permute", "copy", (out_p._view(), ap._cview()), 2 * n * es, [out_p]))
            jobs.append(("gather_reverse", "copy", (out_r._view(), ar._cview()), 2 * n * es, [out_r]))
            ops = [A.OP_ADD, A.OP_SUB, A.OP_MUL if dt == "f32" else A.OP_WMUL, A.OP_DIV]
            for kind, (x, y, o, o64) in (("permute", (ap, bp, out_p, out64_p)), ("reverse", (ar, br, out_r, out64_r))):
                for op in ops:
                    out = o64 if (op == A.OP_DIV and dt == "i32") else o
                    nbytes = 2 * n * es + n * (8 if out is o64 else es)
                    # Int32 / Int32 -> Float64 runs its own (compute-bound) kernel: its own class
                    cls = "binary_" + kind + ("_div_i32" if out is o64 else "")
                    jobs.append((cls, "binary", (op, x._cview(), y._cview(), out._view()), nbytes, [out]))
            mv = C_.mutable_view(slice(None), cu.R(None, None, -1), slice(None))
            jobs.append(("scatter", "copy", (mv._cview(), ap._cview()), 2 * n * es, [C_]))
        return jobs


def execute_job(lib, A, j):
    name, kind, a, nbytes, _ = j
    if kind == "copy":
        rc = lib.phcu_copy(ctypes.byref(a[0]), ctypes.byref(a[1]))
    else:
        rc = lib.phcu_binary(a[0], ctypes.byref(a[1]), ctypes.byref(a[2]), ctypes.byref(a[3]))
    if rc:
        A.check(rc, name)


def profile_class(args):
    """Runs only the launches of one operation class of the step (Float32 or
    Int32), a few times: the command profiled by ncu."""
    import phase_cu as cu
    from phase_cu import _abi as A
    from phase_cu import synth

    cu.init(0)
    lib = A.load()
    shape = [int(x) for x in args.profile_shape.split("x")] if args.profile_shape else SHAPE
    n = int(np.prod(shape))
    dt = args.profile_dtype
    if dt == "f32":
        a, b = synth.uniform_f32(shape, seed=0), synth.uniform_f32(shape, seed=0, start=n)
    else:
        a = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20)
        b = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20, start=n)
    Ad, Bd = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
    dev = {dt: (Ad, Bd, cu.CuNArray.empty([shape[2], shape[0], shape[1]], Ad.dtype))}
    jobs = [j for j in make_jobs(cu, A, dev, n, shape) if j[0] == args.profile_class]
    for _ in range(args.warmup):
        for j in jobs:
            execute_job(lib, A, j)
    for _ in range(args.steps):
        for j in jobs:
            execute_job(lib, A, j)
    A.call("phcu_sync")
    print("profiled %d launches of %s (%s)" % (len(jobs) * (args.warmup + args.steps), args.profile_class, dt))


def replica_max_ms(ms, dist, device):
    """Replicas only: the job's time is the slowest rank's (an all-reduce MAX;
    it also holds every rank until all have finished the timed region)."""
    import torch

    tt = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_gbs(step_bytes, world, ms_per_step):
    """Whole-job throughput: every rank moves step_bytes per step."""
    return step_bytes * world / (ms_per_step * 1e-3) / 1e9


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# dominant class, binary + - * / on permuted 32-bit views, from one ncu capture
# of four launches on a 256x512x256 case (half the bench's elements; reads and
# writes both scale with the element count, so the figure is doubled):
#   python bench.py --profile-class binary_permute --profile-shape 256x512x256 --steps 1 --warmup 0
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       --clock-control none -k regex:eval -c 4 --csv --log-file traffic_permute.csv <same command>
# Mean per launch there: 268,647,040 B read + 92,249,920 B written.
MEASURED_TRAFFIC = {"binary_permute": 2 * (268647040 + 92249920)}
TRAFFIC_SOURCE = ("ncu, 4 launches of eval_tma_kernel<u32,2> at 256x512x256, scaled x2 "
                  "(profiles/eval_tma_kernel_traffic_binary_permute_256x512x256.md)")


def measured_traffic(cls):
    """DRAM bytes per full-size launch of one operation class from the ncu
    capture; None when no capture covers the class."""
    t = MEASURED_TRAFFIC.get(cls)
    return t, (TRAFFIC_SOURCE if t is not None else None)


def profile_config(args):
    """One untimed pass of a secondary workload, for ncu: c3 (the fused chain
    over 64x128x128x64, then sum/max/argmax along every axis and the full sum),
    c4 (8 heat steps on 4096x4096 without a graph) or c5 (the 10,000-task
    uneven batch: two persistent launches)."""
    import phase_cu as cu
    from phase_cu import _abi as A
    from phase_cu import synth

    cu.init(0)
    lib = A.load()
    if args.profile_config == "c3":
        shape = [64, 128, 128, 64]
        x, y, z = (cu.CuNArray.from_numpy(synth.lognormal_f32(shape, s)) for s in (0, 1, 2))
        r = (x.process(lambda e: (e + 4) ** 2) * y - z).to_cu()
        for k in range(4):
            r.sum(axis=k), r.max(axis=k), r.argmax(axis=k)
        r.sum()
    elif args.profile_config == "c5":
        from phase_cu.batch import Batch, Workload

        wl = Workload(n_tasks=10000, seed=0)
        b = Batch(wl.tasks(), wl.programs)
        b.launch(0)
        b.launch(0)
        A.call("phcu_sync")
        b.close()
    else:
        from phase_cu import stencil

        hs = stencil.Heat(synth.gaussian_bumps_f32(4096, 4096, bumps=16, seed=0))
        hs.run(8, use_graph=False)
    A.call("phcu_sync")
    print("profiled %s" % args.profile_config)


def _device_timed(args, cu, A, lib, arrays, dev, jobs, run_job, step_bytes):
    n = int(np.prod(SHAPE))

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
        import torch
        import torch.distributed as dist  # replicas only: one barrier, a max of times
        if args.gpus > 1:
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if args.gpus > 1 else "gloo")
        dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    # The step's 22 operations are captured once as a CUDA graph (the library's
    # phcu_graph_begin/end: same kernels, same launch shapes, TMA maps and
    # descriptors baked in) and replayed once per step, which removes the
    # per-launch gaps; the same step as direct C-ABI calls is timed too and
    # reported beside it.
    c0 = ctypes.c_uint64()
    lib.phcu_launch_count(ctypes.byref(c0))
    graph = ctypes.c_void_p()
    A.check(lib.phcu_graph_begin())
    for j in jobs:
        run_job(j)
    A.check(lib.phcu_graph_end(ctypes.byref(graph)))
    c1 = ctypes.c_uint64()
    lib.phcu_launch_count(ctypes.byref(c1))
    launches_per_step = int(c1.value - c0.value)
    for _ in range(args.warmup):
        A.check(lib.phcu_graph_launch(graph))
    A.call("phcu_sync")
    t = timer()
    for _ in range(args.steps):
        for j in jobs:
            run_job(j)
    direct_ms = stop(t) / args.steps
    A.call("phcu_sync")
    if dist is not None:
        dist.barrier()
    clocks.start()
    t = timer()
    for _ in range(args.steps):
        A.check(lib.phcu_graph_launch(graph))
    ms = stop(t)
    A.call("phcu_sync")
    clk = clocks.stop()
    lib.phcu_graph_destroy(graph)
    if dist is not None:
        ms = replica_max_ms(ms, dist, "cuda" if args.gpus > 1 else "cpu")
    ms_per_step = ms / args.steps
    value = job_gbs(step_bytes, world, ms_per_step)

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
    traffic, traffic_src = measured_traffic(dom[0])
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "bytes_per_launch": int(dom_bytes_per_launch), "ms_per_launch": round(dom_ms_per_launch, 4),
                "traffic": traffic, "traffic_source": traffic_src, "step_frac": round(value / world / peak, 4),
                "per_class_gbs": {k: round(v["gbs"], 1) for k, v in per_class.items()}}

    # ------------------------------------------------------------ e2e
    e2e = e2e_leg(A, lib, arrays, dev, jobs, args, timer, stop, step_bytes)

    result = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (SplitMix64, seed 0)",
        "config": bench_config(),
        "execution": "step captured once as a CUDA graph, one graph launch per step; %d algorithmic bytes per step"
                     % step_bytes,
        "gpu_launches": launches_per_step * args.steps, "roofline": roofline, "clocks": clk, "e2e": e2e,
        "direct_calls": {"ms_per_step": round(direct_ms, 4),
                         "value": round(job_gbs(step_bytes, 1, direct_ms), 1),
                         "note": "the same step as 22 direct C-ABI calls per step, no graph"},
    }
    return result, rank


def e2e_leg(A, lib, arrays, dev_arrays, jobs, args, timer, stop, step_bytes):
    """Same step through the C-ABI with pinned HOST buffers: inputs uploaded and
    every result downloaded inside the timed region.  Each operation writes its
    own device output; the uploads run on the library's host-to-device stream,
    every download starts behind its operation (phcu_download_async) into one
    of two pinned staging buffers and overlaps the operations after it, and the
    next step's uploads overlap this step's last downloads; every step uploads
    its inputs and downloads all its results inside the timed region."""
    import phase_cu as cu

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
    # one device output per operation; results land in two pinned staging
    # buffers taken in turn (one buffer per result, 6.4 GB of pinned memory,
    # measured slower: 83-92 ms per step against 38.5 ms)
    own = []
    for j in jobs:
        name, kind, a, nbytes, outs = j
        o = outs[0]
        mine = cu.CuNArray.empty(o.shape, o.dtype)
        if kind == "copy" and name == "scatter":  # writes into C through its mutable view
            args_ = (a[0], a[1])
            target = o
        elif kind == "copy":
            args_ = (mine._view(), a[1])
            target = mine
        else:
            args_ = (a[0], a[1], a[2], mine._view())
            target = mine
        own.append((kind, args_, target, None, mine))
    staging_bytes = max(x[2]._buf.nbytes for x in own)
    staging = [pinned(staging_bytes), pinned(staging_bytes)]
    own = [(k, a_, t_, staging[i % 2], m_) for i, (k, a_, t_, _, m_) in enumerate(own)]

    def upload(dev_arrays):
        for dt in ("f32", "i32"):
            pa, pb, nb = host_in[dt]
            Ad, Bd, _ = dev_arrays[dt]
            A.check(lib.phcu_upload_async(Ad._buf.ptr, pa, nb))
            A.check(lib.phcu_upload_async(Bd._buf.ptr, pb, nb))

    def run_steps(dev_arrays, n):
        # Step k's uploads are issued right after step k-1's operations, so they
        # run on the host-to-device engine while step k-1's results are still
        # being downloaded (phcu_upload_async waits for the kernels that read the
        # inputs).  The wait before step k's operations covers those uploads and
        # step k-1's downloads, whose device buffers step k overwrites.
        upload(dev_arrays)
        for k in range(n):
            A.check(lib.phcu_transfer_wait())
            for kind, a, target, hbuf, _ in own:
                if kind == "copy":
                    A.check(lib.phcu_copy(ctypes.byref(a[0]), ctypes.byref(a[1])))
                else:
                    A.check(lib.phcu_binary(a[0], ctypes.byref(a[1]), ctypes.byref(a[2]), ctypes.byref(a[3])))
                A.check(lib.phcu_download_async(hbuf, target._buf.ptr, target._buf.nbytes))
            if k + 1 < n:
                upload(dev_arrays)
        A.check(lib.phcu_transfer_wait())

    run_steps(dev_arrays, 1)
    A.call("phcu_sync")
    # five rounds of up to five steps each, the median round reported: the
    # host link is shared with the rest of the machine, and one round alone
    # has ranged from 35 to 56 ms per step on the same box
    steps = max(1, min(args.steps, 5))
    rounds = []
    for _ in range(5):
        t = timer()
        run_steps(dev_arrays, steps)
        rounds.append(stop(t) / steps)
    ms = statistics.median(rounds)
    check = e2e_check(A, lib, arrays, own, upload, dev_arrays)
    h2d = sum(2 * v[2] for v in host_in.values())
    d2h = sum(x[2]._buf.nbytes for x in own)
    for v in host_in.values():
        lib.phcu_host_free(v[0])
        lib.phcu_host_free(v[1])
    for h in staging:
        lib.phcu_host_free(h)
    return {"value": round(step_bytes / (ms * 1e-3) / 1e9, 1), "unit": "GB/s", "ms_per_step": round(ms, 3),
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps,
            "rounds_ms_per_step": [round(r, 3) for r in rounds],
            "path": ("phcu_upload_async/phcu_copy/phcu_binary/phcu_download_async/phcu_transfer_wait "
                     "on pinned host buffers"), "check": check}


def expected_results(arrays):
    """The step's results computed on the host with numpy, in the order of
    make_jobs (IEEE single operations, Int32 wrapping multiply, Int32 / Int32
    as Float64 division): an independent check of what the e2e leg downloads."""
    for dt, (a, b) in arrays.items():
        ap, bp = np.transpose(a, (2, 0, 1)), np.transpose(b, (2, 0, 1))
        ar, br = a[:, ::-1, :], b[:, ::-1, :]
        yield np.ascontiguousarray(ap)
        yield np.ascontiguousarray(ar)
        for x, y in ((ap, bp), (ar, br)):
            with np.errstate(all="ignore"):
                yield x + y
                yield x - y
                yield x * y
                yield (x.astype(np.float64) / y.astype(np.float64)) if dt == "i32" else x / y
        c = np.empty([256, 512, 512], dtype=a.dtype)
        c[:, ::-1, :] = ap
        yield c


def e2e_check(A, lib, arrays, own, upload, dev_arrays):
    """After the timed steps: (1) the last two pinned staging buffers (the last
    two results of the last timed step) equal the device results; (2) one more
    step through the same upload / operation / async download path, each
    download compared with the numpy result of that operation."""
    def host_view(ptr, nbytes, dtype):
        raw = (ctypes.c_uint8 * nbytes).from_address(ptr)
        return np.frombuffer(raw, dtype=np.uint8).view(dtype)

    def device_bytes(t):
        h = np.empty(t._buf.nbytes, dtype=np.uint8)
        A.check(lib.phcu_download(h.ctypes.data, t._buf.ptr, t._buf.nbytes))
        return h

    last_ok = True
    for i in (len(own) - 2, len(own) - 1):
        t, hbuf = own[i][2], own[i][3]
        last_ok = last_ok and bool(np.array_equal(host_view(hbuf, t._buf.nbytes, np.uint8), device_bytes(t)))
    upload(dev_arrays)
    A.check(lib.phcu_transfer_wait())
    bad = []
    for i, ((kind, a, target, hbuf, _), exp) in enumerate(zip(own, expected_results(arrays))):
        if kind == "copy":
            A.check(lib.phcu_copy(ctypes.byref(a[0]), ctypes.byref(a[1])))
        else:
            A.check(lib.phcu_binary(a[0], ctypes.byref(a[1]), ctypes.byref(a[2]), ctypes.byref(a[3])))
        A.check(lib.phcu_download_async(hbuf, target._buf.ptr, target._buf.nbytes))
        A.check(lib.phcu_transfer_wait())
        got = host_view(hbuf, target._buf.nbytes, exp.dtype).reshape(exp.shape)
        if not np.array_equal(got, exp, equal_nan=exp.dtype.kind == "f"):
            bad.append(i)
    return {"results_checked": len(own), "mismatches": bad, "last_timed_step_equals_device": last_ok,
            "reference": "numpy on the host inputs (IEEE single ops, wrapping Int32 *, Float64 division)"}


# --------------------------------------------------------- other configs
def _ms(A, lib, fn, reps, flush=False):
    """Median device time of fn() over reps (CUDA events on the library stream)."""
    out = []
    for _ in range(reps):
        if flush:
            A.check(lib.phcu_l2_flush())
        t = ctypes.c_void_p()
        A.check(lib.phcu_timer_start(ctypes.byref(t)))
        fn()
        ms = ctypes.c_float()
        A.check(lib.phcu_timer_stop(t, ctypes.byref(ms)))
        out.append(ms.value)
    return statistics.median(out)


C1_REPS = 50


def _flushed_graph_ms(A, lib, fn, reps=C1_REPS):
    """Device time of fn() with a cold L2: a CUDA graph of `reps` (L2 flush,
    fn) pairs and one of `reps` flushes alone are each replayed five times;
    the difference of the median replay times over reps."""
    A.check(lib.phcu_l2_flush())  # allocates the scrub buffer before any capture
    fn()
    A.call("phcu_sync")

    def graph(with_op):
        g = ctypes.c_void_p()
        A.check(lib.phcu_graph_begin())
        for _ in range(reps):
            A.check(lib.phcu_l2_flush())
            if with_op:
                fn()
        A.check(lib.phcu_graph_end(ctypes.byref(g)))
        return g

    g_op, g_fl = graph(True), graph(False)
    t_op, t_fl = [], []
    for _ in range(5):
        t_op.append(_ms(A, lib, lambda: A.check(lib.phcu_graph_launch(g_op)), 1))
        t_fl.append(_ms(A, lib, lambda: A.check(lib.phcu_graph_launch(g_fl)), 1))
    lib.phcu_graph_destroy(g_op)
    lib.phcu_graph_destroy(g_fl)
    return max(1e-6, (statistics.median(t_op) - statistics.median(t_fl)) / reps)


def _ms_batched(A, lib, fn, reps=5, inner=10):
    """Median over reps of the mean device time of `inner` back-to-back calls
    (one event pair around them): the per-launch event and gap overhead is
    spread over `inner` launches.  For kernels whose inputs exceed L2."""
    return _ms(A, lib, lambda: [fn() for _ in range(inner)], reps) / inner


def extra_configs(reps=5):
    """The remaining workloads, each measured on its own (GB/s = algorithmic
    bytes / median device time)."""
    import phase_cu as cu
    from phase_cu import _abi as A
    from phase_cu import synth

    lib = A.load()
    res = {}
    gb = lambda nbytes, ms: round(nbytes / (ms * 1e-3) / 1e9, 1)

    # C1: 1024x1024 a+b, a*b, a[.., 1..2..-1]; 12 MiB fits L2, so L2 is flushed before each rep.
    # One event pair around one such launch reads the launch and event overhead
    # (~9 us for any of these ops), so each op is timed as a CUDA graph of
    # C1_REPS (flush, op) pairs minus a graph of C1_REPS flushes alone.
    c1 = {}
    n = 1024 * 1024
    for dt in ("f32", "i32"):
        a = synth.uniform_f32([1024, 1024], 0) if dt == "f32" else synth.uniform_i32([1024, 1024], 0)
        b = (synth.uniform_f32([1024, 1024], 0, start=n) if dt == "f32"
             else synth.uniform_i32([1024, 1024], 0, start=n))
        X, Y = cu.CuNArray.from_numpy(a), cu.CuNArray.from_numpy(b)
        O = cu.CuNArray.empty([1024, 1024], X.dtype)
        G = cu.CuNArray.empty([1024, 512], X.dtype)
        xv, yv, ov = X._view(), Y._view(), O._view()
        sv = X.view(slice(None), cu.R(1, -1, 2))._cview()
        gv = G._view()
        for name, op in (("add", A.OP_ADD), ("mul", A.OP_MUL if dt == "f32" else A.OP_WMUL)):
            ms = _flushed_graph_ms(A, lib, lambda: A.check(lib.phcu_binary(op, ctypes.byref(xv), ctypes.byref(yv),
                                                                           ctypes.byref(ov))))
            c1["%s_%s" % (name, dt)] = {"ms": round(ms, 5), "gbs": gb(3 * n * 4, ms)}
        ms = _flushed_graph_ms(A, lib, lambda: A.check(lib.phcu_copy(ctypes.byref(gv), ctypes.byref(sv))))
        c1["view_step2_%s" % dt] = {"ms": round(ms, 5), "gbs": gb(2 * (n // 2) * 4, ms)}
    c1["method"] = ("graph of %d (L2 flush, op) pairs minus a graph of %d flushes, median of 5 replays; "
                    "the op reads its inputs from HBM" % (C1_REPS, C1_REPS))
    res["c1_plain_1024sq"] = c1

    # C3: fused ((x+4)**2)*y - z over 64x128x128x64 lognormal, then reductions per axis
    shape = [64, 128, 128, 64]
    n3 = int(np.prod(shape))
    x = cu.CuNArray.from_numpy(synth.lognormal_f32(shape, 0))
    y = cu.CuNArray.from_numpy(synth.lognormal_f32(shape, 1))
    z = cu.CuNArray.from_numpy(synth.lognormal_f32(shape, 2))
    pv = x.process(lambda e: (e + 4) ** 2) * y - z
    prog, _ = cu.compile_program(pv._expr, cu.Float32)
    ins = (A.View * 3)(*[l._cview() for l in pv._leaves])
    r = cu.CuNArray.empty(shape, cu.Float32)
    rv = r._view()
    # every operand is 256 MiB (twice L2): launches are timed ten back to back per event pair
    ms = _ms_batched(A, lib, lambda: A.check(lib.phcu_eval(ctypes.byref(prog), ins, 3, ctypes.byref(rv))), reps)
    c3 = {"fused_chain": {"ms": round(ms, 4), "gbs": gb(4 * n3 * 4, ms), "kernels": 1,
                          "unfused_bytes": 10 * n3 * 4},
          "method": "median of 5 event pairs, each around 10 back-to-back launches (operands 256 MiB > L2)"}
    for k in range(4):
        oshape = shape[:k] + shape[k + 1:]
        for name, op, odt in (("sum", A.RED_SUM, cu.Float32), ("max", A.RED_MAX, cu.Float32),
                              ("argmax", A.RED_ARGMAX, cu.Int32)):
            o = cu.CuNArray.empty(oshape, odt)
            oview = o._view()
            ms = _ms_batched(A, lib, lambda: A.check(lib.phcu_reduce(op, ctypes.byref(rv), k, ctypes.byref(oview))),
                             reps)
            c3["%s_axis%d" % (name, k)] = {"ms": round(ms, 4), "gbs": gb(n3 * 4 + o.size * 4, ms)}
    o1 = cu.CuNArray.empty([1], cu.Float32)
    o1v = o1._view()
    ms = _ms_batched(A, lib, lambda: A.check(lib.phcu_reduce(A.RED_SUM, ctypes.byref(rv), -1, ctypes.byref(o1v))),
                     reps)
    c3["sum_all"] = {"ms": round(ms, 4), "gbs": gb(n3 * 4, ms)}
    res["c3_fused_reduce"] = c3
    del x, y, z, r

    # C4: 4096x4096 heat, 1000 steps captured in one CUDA graph; FP32 error vs an FP64 run
    from phase_cu import stencil

    u0 = synth.gaussian_bumps_f32(4096, 4096, bumps=16, seed=0)
    hs = stencil.Heat(u0)
    ms = _ms(A, lib, lambda: hs.run(1000, use_graph=True), 3)
    c4 = {"steps": 1000, "ms": round(ms, 3), "steps_per_s": round(1000 / (ms * 1e-3), 1),
          "gbs_effective": gb(1000 * 2 * 4094 * 4094 * 4, ms),
          "note": "two 64 MiB grids ping-pong; most of the working set stays in the 126 MB L2"}
    c4["error_vs_fp64"] = stencil.error_vs_fp64(u0, (10, 100, 1000))
    res["c4_heat_4096sq"] = c4

    # C5: 10,000 uneven tasks, one persistent launch vs per-op launches (and a graph of them)
    res["c5_batched"] = batched_leg(reps)
    return res


def batched_leg(reps=5, n_tasks=10000):
    import phase_cu as cu
    from phase_cu import _abi as A
    from phase_cu import tuner
    from phase_cu.batch import Batch, Workload

    lib = A.load()
    wl = Workload(n_tasks=n_tasks, seed=0)
    tasks = wl.tasks()
    b = Batch(tasks, wl.programs)
    info = b.info()
    out = {"tasks": n_tasks, "items": info["items"], "bytes": info["bytes"]}
    c0 = ctypes.c_uint64()
    for mode, name in ((0, "persistent"), (1, "per_op"), (2, "per_op_graph")):
        b.launch(mode)  # warm-up (mode 2 captures its graph here)
        lib.phcu_launch_count(ctypes.byref(c0))
        before = c0.value
        ms = _ms(A, lib, lambda: b.launch(mode), reps)
        lib.phcu_launch_count(ctypes.byref(c0))
        out[name] = {"ms": round(ms, 3), "ops_per_s": round(n_tasks / (ms * 1e-3), 1),
                     "gbs": round(info["bytes"] / (ms * 1e-3) / 1e9, 1),
                     "launches_per_run": (c0.value - before) // max(1, reps)}
    b.close()
    out["speedup_vs_per_op"] = round(out["per_op"]["ms"] / out["persistent"]["ms"], 2)
    # learned tuner: exhaustive timings of a sample train the MLP; it then picks
    # per-task work-item sizes for the whole batch
    rng = np.random.default_rng(0)
    sample = rng.choice(n_tasks, 480, replace=False)
    times = np.stack([tuner.measure(tasks[i], wl.programs, reps=3) for i in sample])
    feats = tuner.feature_matrix([tasks[i] for i in sample])
    half = len(sample) * 3 // 4
    net = tuner.MLP(seed=1)
    net.train(feats[:half].reshape(-1, 24), np.log2(times[:half].reshape(-1)), epochs=200, batch=256, lr=2e-3)
    picks, _ = net.pick(feats[half:])
    out["tuner"] = {"train_tasks": int(half), "test_tasks": int(len(sample) - half),
                    "regret_mlp": round(tuner.regret(times[half:], picks), 4),
                    "regret_default": round(tuner.regret(times[half:], np.full(len(picks), tuner.DEFAULT_CONFIG)),
                                            4)}
    allf = tuner.feature_matrix(tasks)
    allpick, _ = net.pick(allf)
    chunks, layouts = tuner.config_args(allpick)
    bt = Batch(wl.tasks(chunks, layouts), wl.programs)
    bt.launch(0)
    ms = _ms(A, lib, lambda: bt.launch(0), reps)
    bt.close()
    out["persistent_mlp_tuned"] = {"ms": round(ms, 3), "ops_per_s": round(n_tasks / (ms * 1e-3), 1),
                                   "gbs": round(info["bytes"] / (ms * 1e-3) / 1e9, 1)}
    out["speedup_tuned_vs_per_op"] = round(out["per_op"]["ms"] / ms, 2)
    return out


# ------------------------------------------------------------ CPU baseline
CPU_SLABS = 16


class CpuStep:
    """The step on the oracle (the reference's loops restated in C: one
    materialised pass per operation, per-element view transforms) over the
    full-size arrays.  A bounded sample computes one lexicographic slab (1/16)
    of every operation's output with every host thread: the same arrays,
    strides and access pattern as the full step, a sixteenth of its elements."""

    def __init__(self, shape=SHAPE):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as ora
        from phase_cu import synth
        from phase_cu.region import R

        ora.build()
        self.ora = ora
        self.n = n = int(np.prod(shape))
        self.ops = []
        for dt in ("f32", "i32"):
            if dt == "f32":
                a = synth.uniform_f32(shape, seed=0)
                b = synth.uniform_f32(shape, seed=0, start=n)
            else:
                a = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20)
                b = synth.uniform_i32(shape, seed=0, lo=-2 ** 20, hi=2 ** 20, start=n)
            perm = [("permute", [2, 0, 1])]
            rev = [("region", [slice(None), R(None, None, -1), slice(None)])]
            ap, bp = ora.ViewOperand(a, perm), ora.ViewOperand(b, perm)
            ar, br = ora.ViewOperand(a, rev), ora.ViewOperand(b, rev)
            out = np.empty(ap.shape, dtype=a.dtype)
            out64 = np.empty(ap.shape, dtype=np.float64)
            self.ops.append(("gather", ap, None, out, 8))
            self.ops.append(("gather", ar, None, out, 8))
            for x, y in ((ap, bp), (ar, br)):
                for op in (ora.OP_ADD, ora.OP_SUB, ora.OP_MUL if dt == "f32" else ora.OP_WMUL, ora.OP_DIV):
                    wide = op == ora.OP_DIV and dt == "i32"
                    self.ops.append((op, x, y, out64 if wide else out, 16 if wide else 12))
            c = np.zeros([shape[2], shape[0], shape[1]], dtype=a.dtype)
            self.ops.append(("scatter", ora.ViewOperand(c, rev), ap, None, 8))

    def run(self, nthreads, slab=0, slabs=1):
        """Runs slab `slab` of `slabs` of every operation; returns (seconds, algorithmic bytes)."""
        ora, n = self.ora, self.n
        lo, hi = n * slab // slabs, n * (slab + 1) // slabs
        t0 = time.perf_counter()
        for kind, x, y, out, per in self.ops:
            if kind == "gather":
                ora.gather_range(x, out, lo, hi, nthreads)
            elif kind == "scatter":
                ora.scatter_range(x, y, lo, hi, nthreads)
            else:
                ora.map_binary_range(kind, x, y, out, lo, hi, nthreads)
        return time.perf_counter() - t0, sum(o[4] for o in self.ops) * (hi - lo)


def cpu_baseline(nthreads):
    """Two slab samples (1/16 each) of the full-size step on the oracle with
    every host thread, and (for scale) the reference's own single thread on
    one slab."""
    step = CpuStep()
    secs, nbytes = 0.0, 0
    for k in range(2):
        t, b = step.run(nthreads, k, CPU_SLABS)
        secs += t
        nbytes += b
    t1, b1 = step.run(1, 2, CPU_SLABS)
    return {"value": round(nbytes / secs / 1e9, 3), "unit": "GB/s", "cores": nthreads, "kind": "port",
            "sample": "slabs 0-1 of %d of every operation's output on the full-size step (Float32+Int32 %s), "
                      "%.1f s, %d algorithmic bytes" % (CPU_SLABS, "x".join(map(str, SHAPE)), secs, nbytes),
            "single_thread": {"value": round(b1 / t1 / 1e9, 3), "cores": 1,
                              "sample": "slab 2 of %d, %.1f s" % (CPU_SLABS, t1)}}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None, rank
    threads = os.cpu_count() or 1
    step = CpuStep()
    for k in range(args.warmup):
        step.run(threads, k % CPU_SLABS, CPU_SLABS)
    vals = []
    for k in range(args.steps):
        vals.append(step.run(threads, k % CPU_SLABS, CPU_SLABS))
    gbs = sum(v[1] for v in vals) / sum(v[0] for v in vals) / 1e9
    ms = 1e3 * sum(v[0] for v in vals) / len(vals)
    res = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (SplitMix64, seed 0)",
           "config": bench_config(),
           "execution": "oracle port of the reference loops on %d host threads" % threads,
           "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                            "sample": "step k = slab k mod %d (1/%d of the elements, a contiguous lexicographic "
                                      "range) of every operation's output on the full-size arrays (Float32+Int32 "
                                      "%s), every host thread; the reference is Crystal and cannot be built here, "
                                      "so its loops run as the C oracle (one materialised pass per operation, "
                                      "per-element view transforms)" % (CPU_SLABS, CPU_SLABS, "x".join(map(str, SHAPE)))},
           "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return res, rank


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extra", action="store_true")
    p.add_argument("--profile-class", default=None,
                   help="run only one operation class (gather_permute, gather_reverse, binary_permute, "
                        "binary_reverse, binary_permute_div_i32, binary_reverse_div_i32, scatter) for profiling")
    p.add_argument("--profile-dtype", default="f32")
    p.add_argument("--profile-shape", default=None,
                   help="a smaller AxBxC shape for --profile-class (ncu captures of several metrics)")
    p.add_argument("--profile-config", default=None, choices=["c3", "c4", "c5"],
                   help="one untimed pass of the fused-chain/reduction (c3), heat (c4) or batch (c5) workload, "
                        "for profiling")
    args = p.parse_args()
    if args.profile_class:
        profile_class(args)
        return
    if args.profile_config:
        profile_config(args)
        return
    if args.impl == "reference":
        res, rank = reference_arm(args)
        if rank == 0 and res:
            print(json.dumps(res), flush=True)
        return
    res, rank = device_arm(args)
    if rank == 0:
        if not args.no_extra:
            res["extra"] = extra_configs()
        if not args.no_cpu:
            res["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
