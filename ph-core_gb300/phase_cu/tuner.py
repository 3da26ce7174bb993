"""Autotuner and learned tuner for batched tasks.

`measure` times a task under every launch configuration (exhaustive
autotune, phcu_tune_measure).  `MLP` is the 24 -> 64 -> 64 -> 1 network whose
forward, backward and Adam steps run on the GPU (phcu_mlp_*); it is trained
to predict log2(time) of (task, configuration) from `features`, and `pick`
chooses, per task, the configuration with the smallest predicted time.  The
exhaustive timings remain the yardstick: `regret` compares any choice with the best
measured configuration.
"""
import ctypes

import numpy as np

from . import _abi as A
from .narray import _Buffer, init, lib

DEFAULT_CONFIG = 3  # 32768-element work items (the executor's default), planner's launch shape
CHUNKS = (4096, 8192, 16384, 32768)  # work-item sizes (elements) of configurations c % 4


def config_args(picks):
    """(work-item sizes, layouts) of per-task configuration indices: config c
    is work items of CHUNKS[c % 4] elements in layout c // 4 (0 = the
    planner's launch shape, 1 = the alternative)."""
    return [CHUNKS[int(c) % len(CHUNKS)] for c in picks], [int(c) // len(CHUNKS) for c in picks]


def n_configs():
    n = ctypes.c_int32()
    A.check(lib().phcu_tune_n_configs(ctypes.byref(n)))
    return n.value


def features(task, config):
    f = (ctypes.c_float * A.TUNE_FEATURES)()
    A.check(lib().phcu_tune_features(ctypes.byref(task), config, f), "phcu_tune_features")
    return np.frombuffer(f, dtype=np.float32).copy()


def feature_matrix(tasks):
    nc = n_configs()
    return np.stack([np.stack([features(t, c) for c in range(nc)]) for t in tasks])  # [tasks, configs, 24]


def measure(task, programs, reps=3):
    nc = n_configs()
    ms = (ctypes.c_float * nc)()
    A.check(lib().phcu_tune_measure(ctypes.byref(task), programs, reps, ms), "phcu_tune_measure")
    return np.frombuffer(ms, dtype=np.float32).copy()


def regret(times, picks):
    """Mean relative excess time of the picked configurations over the best."""
    best = times.min(axis=1)
    chosen = times[np.arange(len(picks)), picks]
    return float(np.mean((chosen - best) / best))


class _Dev:
    """A float32 device array (upload/download helpers)."""

    def __init__(self, n):
        self.n = int(n)
        self.buf = _Buffer(max(1, self.n) * 4)

    @classmethod
    def of(cls, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float32)
        d = cls(arr.size)
        if arr.nbytes:
            A.check(lib().phcu_upload(d.buf.ptr, arr.ctypes.data, arr.nbytes))
        return d

    def get(self):
        h = np.empty(self.n, dtype=np.float32)
        if h.nbytes:
            A.check(lib().phcu_download(h.ctypes.data, self.buf.ptr, h.nbytes))
        return h


class MLP:
    """24 -> 64 -> 64 -> 1 ReLU network on the GPU (parameters stay on the device)."""

    def __init__(self, seed=0):
        init()
        self.params = _Dev(A.MLP_PARAMS)
        A.check(lib().phcu_mlp_init(self.params.buf.ptr, seed), "phcu_mlp_init")
        self.mu = np.zeros(A.TUNE_FEATURES, np.float32)
        self.sd = np.ones(A.TUNE_FEATURES, np.float32)
        self.ymu = 0.0

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        A.check(lib().phcu_upload(self.params.buf.ptr, p.ctypes.data, p.nbytes))

    def get_params(self):
        return self.params.get()

    def _norm(self, x):
        return ((x - self.mu) / self.sd).astype(np.float32)

    def forward(self, x, normalise=True):
        x = np.ascontiguousarray(self._norm(x) if normalise else x, dtype=np.float32).reshape(-1, A.TUNE_FEATURES)
        dx = _Dev.of(x)
        dy = _Dev(len(x))
        A.check(lib().phcu_mlp_forward(self.params.buf.ptr, dx.buf.ptr, len(x), dy.buf.ptr), "phcu_mlp_forward")
        return dy.get() + (self.ymu if normalise else 0.0)

    def grad(self, x, y):
        """Loss and gradient of mean squared error (no normalisation)."""
        dx, dyv = _Dev.of(x), _Dev.of(y)
        g = _Dev(A.MLP_PARAMS)
        loss = ctypes.c_float()
        A.check(lib().phcu_mlp_grad(self.params.buf.ptr, dx.buf.ptr, dyv.buf.ptr, len(y), g.buf.ptr,
                                    ctypes.byref(loss)), "phcu_mlp_grad")
        return loss.value, g.get()

    def train(self, x, y, epochs=300, batch=256, lr=2e-3, seed=0):
        x = np.asarray(x, np.float32).reshape(-1, A.TUNE_FEATURES)
        y = np.asarray(y, np.float32).reshape(-1)
        self.mu = x.mean(axis=0)
        self.sd = x.std(axis=0) + 1e-3
        self.ymu = float(y.mean())
        rng = np.random.default_rng(seed)
        order = rng.permutation(len(y))
        xs = self._norm(x[order])
        ys = (y[order] - self.ymu).astype(np.float32)
        dx, dy = _Dev.of(xs), _Dev.of(ys)
        loss = ctypes.c_float()
        A.check(lib().phcu_mlp_train(self.params.buf.ptr, dx.buf.ptr, dy.buf.ptr, len(ys), epochs, batch, lr, seed,
                                     ctypes.byref(loss)), "phcu_mlp_train")
        return loss.value

    def pick(self, feats, default=DEFAULT_CONFIG, margin=0.1):
        """feats [tasks, configs, 24] -> the configuration with the smallest
        predicted time, or `default` when the network predicts no gain of at
        least `margin` (relative) over it: many tasks run in a few
        microseconds under every configuration, where a predicted difference
        is mostly timing noise and the default is as good a choice."""
        t, c, f = feats.shape
        pred = self.forward(feats.reshape(-1, f)).reshape(t, c)
        best = np.argmin(pred, axis=1)
        gain = pred[:, default] - pred[np.arange(t), best]  # log2 of the predicted speed-up
        return np.where(gain >= np.log2(1.0 + margin), best, default), pred
