"""Batched execution of many small, uneven array operations.

Builds phcu_task_t lists (fused elementwise programs over strided views, or
reductions), prepares them once (phcu_batch_prepare) and replays them as one
persistent launch (mode 0), as one ordinary launch per task (mode 1, the
per-op baseline) or as per-op launches captured in a CUDA graph (mode 2).

`synth_tasks` builds the uneven workload: tasks of rank 1-4 whose element
counts are log-uniform in [2^min_log2, 2^max_log2], Float32/Int32 50/50, each
reading a strided view (per-axis steps 1-4, random axis permutation) of a
base array, with an op drawn from {+, *, ((v+4)**2)*w - v, sum(axis), argmax(axis)};
binary operands take the same view of a paired array w.
"""
import ctypes

import numpy as np

from . import _abi as A
from .narray import _Buffer, compile_program, init, lib

OPS = ("add", "mul", "chain", "sum", "argmax")


def view_struct(base_ptr, dtype, offset, shape, stride):
    v = A.View()
    v.base = base_ptr
    v.dtype = dtype
    v.rank = len(shape)
    v.offset = int(offset)
    for i, (n, s) in enumerate(zip(shape, stride)):
        v.shape[i] = int(n)
        v.stride[i] = int(s)
    return v


def row_major(shape):
    st, s = [0] * len(shape), 1
    for i in range(len(shape) - 1, -1, -1):
        st[i] = s
        s *= shape[i]
    return st


def program_table():
    """Programs of the workload: + , *, ((v+4)**2)*w - v for Float32 and Int32."""
    progs = []
    for t in (A.F32, A.I32):
        v = ("in", 0, t)
        w = ("in", 1, t)
        add = ("bin", A.OP_ADD, v, w, t, t, t)
        mul = ("bin", A.OP_MUL, v, w, t, t, t)
        c = ("bin", A.OP_ADD, v, ("const", 4, A.I32), t, A.I32, t)
        c = ("bin", A.OP_POW, c, ("const", 2, A.I32), t, A.I32, t)
        c = ("bin", A.OP_MUL, c, w, t, t, t)
        c = ("bin", A.OP_SUB, c, v, t, t, t)
        for e in (add, mul, c):
            progs.append(compile_program(e, t)[0])
    table = (A.Program * len(progs))(*progs)
    return table  # index = 3 * (0 for Float32, 1 for Int32) + (0 add, 1 mul, 2 chain)


def eval_task(out, inputs, prog, chunk=0, layout=0):
    t = A.Task()
    t.kind = A.TASK_EVAL
    t.n_inputs = len(inputs)
    t.prog = prog
    t.chunk = chunk
    t.layout = layout
    for k, v in enumerate(inputs):
        t.inp[k] = v
    t.out = out
    return t


def reduce_task(op, inp, axis, out, chunk=0, layout=0):
    t = A.Task()
    t.kind = A.TASK_REDUCE
    t.red_op = op
    t.axis = axis
    t.n_inputs = 1
    t.inp[0] = inp
    t.out = out
    t.chunk = chunk
    t.layout = layout
    return t


class Batch:
    """A prepared task list (device-resident plans and work queue)."""

    def __init__(self, tasks, programs):
        init()
        self._keep = (tasks, programs)
        arr = (A.Task * len(tasks))(*tasks) if not isinstance(tasks, ctypes.Array) else tasks
        self._tasks = arr
        h = ctypes.c_void_p()
        A.check(lib().phcu_batch_prepare(arr, len(arr), programs, len(programs) if programs is not None else 0,
                                         ctypes.byref(h)), "phcu_batch_prepare")
        self.handle = h

    def launch(self, mode=0):
        A.check(lib().phcu_batch_launch(self.handle, mode), "phcu_batch_launch")

    def info(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        A.check(lib().phcu_batch_info(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"tasks": a.value, "items": b.value, "bytes": c.value}

    def close(self):
        if self.handle:
            lib().phcu_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _factor(n, rank, rng):
    """A random shape of `rank` axes whose product is close to n."""
    if rank == 1:
        return [n]
    logs = rng.dirichlet(np.ones(rank)) * np.log2(n)
    shape = [max(1, int(round(2 ** l))) for l in logs]
    return shape


class Workload:
    """Device buffers and task descriptions of the uneven batched workload."""

    def __init__(self, n_tasks=10000, seed=0, min_log2=4, max_log2=20, pool_log2=24):
        from .synth import uniform_f32, uniform_i32

        init()
        rng = np.random.default_rng(seed)
        self.pool_n = 1 << pool_log2
        # read-only input pools; each task's base arrays start at a random offset
        self.host_f = uniform_f32([self.pool_n], seed=seed)
        self.host_i = uniform_i32([self.pool_n], seed=seed, lo=-1000, hi=1000)
        self.pool_f = _Buffer(self.pool_n * 4)
        self.pool_i = _Buffer(self.pool_n * 4)
        A.check(lib().phcu_upload(self.pool_f.ptr, self.host_f.ctypes.data, self.host_f.nbytes))
        A.check(lib().phcu_upload(self.pool_i.ptr, self.host_i.ctypes.data, self.host_i.nbytes))
        self.meta = []
        out_total = 0
        for i in range(n_tasks):
            rank = int(rng.integers(1, 5))
            n = int(round(2 ** rng.uniform(min_log2, max_log2)))
            shape = _factor(n, rank, rng)
            n = int(np.prod(shape))
            dt = A.F32 if rng.random() < 0.5 else A.I32
            steps = [int(rng.integers(1, 5)) for _ in range(rank)]
            perm = [int(x) for x in rng.permutation(rank)]
            op = OPS[int(rng.integers(0, 5))]
            off_v = int(rng.integers(0, self.pool_n - n + 1))
            off_w = int(rng.integers(0, self.pool_n - n + 1))
            # the view: base[::s0, ::s1, ...] then permuted
            vshape = [(d + s - 1) // s for d, s in zip(shape, steps)]
            bst = row_major(shape)
            vst = [b * s for b, s in zip(bst, steps)]
            vshape = [vshape[p] for p in perm]
            vst = [vst[p] for p in perm]
            axis = int(rng.integers(0, rank))
            if op in ("sum", "argmax"):
                oshape = vshape[:axis] + vshape[axis + 1:] or [1]
            else:
                oshape = list(vshape)
            odt = A.I32 if op == "argmax" else dt
            on = int(np.prod(oshape))
            self.meta.append(dict(rank=rank, shape=shape, dtype=dt, steps=steps, perm=perm, op=op, off_v=off_v,
                                  off_w=off_w, vshape=vshape, vstride=vst, axis=axis, oshape=oshape, odtype=odt,
                                  out_off=out_total, out_n=on))
            out_total += on
        self.out_n = out_total
        self.out = _Buffer(max(out_total, 1) * 4)
        self.programs = program_table()

    def tasks(self, chunks=None, layouts=None):
        out = []
        for i, m in enumerate(self.meta):
            pool = self.pool_f if m["dtype"] == A.F32 else self.pool_i
            v = view_struct(pool.ptr, m["dtype"], m["off_v"], m["vshape"], m["vstride"])
            w = view_struct(pool.ptr, m["dtype"], m["off_w"], m["vshape"], m["vstride"])
            o = view_struct(self.out.ptr, m["odtype"], m["out_off"], m["oshape"], row_major(m["oshape"]))
            ch = 0 if chunks is None else int(chunks[i])
            ly = 0 if layouts is None else int(layouts[i])
            if m["op"] in ("add", "mul", "chain"):
                prog = 3 * (0 if m["dtype"] == A.F32 else 1) + OPS.index(m["op"])
                out.append(eval_task(o, [v, w], prog, ch, ly))
            else:
                rop = A.RED_SUM if m["op"] == "sum" else A.RED_ARGMAX
                out.append(reduce_task(rop, v, m["axis"], o, ch, ly))
        return out

    def download_outputs(self):
        host = np.empty(max(self.out_n, 1) * 4, dtype=np.uint8)
        A.check(lib().phcu_download(host.ctypes.data, self.out.ptr, host.nbytes))
        return host

    def task_output(self, host, i):
        m = self.meta[i]
        dt = np.float32 if m["odtype"] == A.F32 else np.int32
        raw = host[m["out_off"] * 4:(m["out_off"] + m["out_n"]) * 4]
        return raw.view(dt).reshape(m["oshape"])

    def task_inputs(self, i):
        """Host copies of the task's views (numpy, same element order)."""
        m = self.meta[i]
        pool = self.host_f if m["dtype"] == A.F32 else self.host_i
        base_v = pool[m["off_v"]:m["off_v"] + int(np.prod(m["shape"]))].reshape(m["shape"])
        base_w = pool[m["off_w"]:m["off_w"] + int(np.prod(m["shape"]))].reshape(m["shape"])
        sl = tuple(slice(None, None, s) for s in m["steps"])
        return base_v[sl].transpose(m["perm"]), base_w[sl].transpose(m["perm"])
