"""The explicit 2-D heat equation on device (config workload of the
reference's examples/heat_equation.cr, generalised to 2-D shifted views).

One step is the Phase program
    c   = u[1..-2, 1..-2]
    lap = u[0..-3, 1..-2] + u[2.., 1..-2] + u[1..-2, 0..-3] + u[1..-2, 2..] - c * 4
    u[1..-2, 1..-2] = c + lap * coef
fused into one kernel; `run` replays many steps as one CUDA graph.
"""
import ctypes

import numpy as np

from . import _abi as A
from .narray import _Buffer, init, lib


class Heat:
    """Two device grids (u and a ping-pong partner) of one dtype."""

    def __init__(self, u0, coef=0.2, f64=False):
        init()
        self.f64 = f64
        self.dtype = np.float64 if f64 else np.float32
        u0 = np.ascontiguousarray(u0, dtype=self.dtype)
        self.n, self.m = u0.shape
        self.coef = coef
        self.u = _Buffer(u0.nbytes)
        self.tmp = _Buffer(u0.nbytes)
        A.check(lib().phcu_upload(self.u.ptr, u0.ctypes.data, u0.nbytes))

    def run(self, steps, use_graph=True):
        fn = lib().phcu_heat_run_f64 if self.f64 else lib().phcu_heat_run
        A.check(fn(self.u.ptr, self.tmp.ptr, self.n, self.m, self.coef, steps, 1 if use_graph else 0), "phcu_heat_run")

    def get(self):
        h = np.empty((self.n, self.m), dtype=self.dtype)
        A.check(lib().phcu_download(h.ctypes.data, self.u.ptr, h.nbytes))
        return h


def error_vs_fp64(u0, checkpoints=(10, 100, 1000), coef=0.2):
    """Max-abs and relative-L2 error of the Float32 run against a Float64 run
    from the same (Float32-rounded) initial field, at each checkpoint."""
    h32 = Heat(u0, coef, f64=False)
    h64 = Heat(u0.astype(np.float64), coef, f64=True)
    done = 0
    out = {}
    for c in checkpoints:
        h32.run(c - done, use_graph=False)
        h64.run(c - done, use_graph=False)
        done = c
        a, b = h32.get().astype(np.float64), h64.get()
        out[str(c)] = {"max_abs": float(np.max(np.abs(a - b))),
                       "rel_l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}
    return out
