"""The batched and heat workloads at the sizes the benchmark runs them, checked
against the oracle (its multithreaded restatement of the reference loops):

- the uneven batch: 10,000 tasks (seed 0), ranks 1-4, element counts
  log-uniform in [16, 2^20], Float32/Int32, strided permuted views, ops
  {+, *, ((v+4)**2)*w - v, sum(axis), argmax(axis)}; every task compared with
  the oracle after the persistent launch, the per-op launches, the per-op
  graph and a persistent launch in the layout the learned tuner picks
  (the reference computes each task with map_with / the slices fold,
  src/multi_indexable.cr:1026-1102 and :742-786);
- the 4096x4096 Float32 heat equation: 1000 steps in one CUDA graph,
  bit-exact against the Float32 oracle (examples/heat_equation.cr:38-51).

Integer, index and elementwise results are bit-exact; Float32 sums are within
1e-6 of the sum of magnitudes of the FP64 oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = max(1, min(16, os.cpu_count() or 1))


def _oracle_task(ora, wl, i):
    m = wl.meta[i]
    v, w = wl.task_inputs(i)
    v, w = np.ascontiguousarray(v), np.ascontiguousarray(w)
    op = m["op"]
    nt = NT if v.size > 65536 else 1
    if op == "add":
        return ora.map_binary(ora.OP_ADD, v, w, nt)[0], None
    if op == "mul":
        return ora.map_binary(ora.OP_MUL, v, w, nt)[0], None
    if op == "chain":
        t, _ = ora.map_binary_scalar(ora.OP_ADD, v, 4, ora.I32, nthreads=nt)
        t, _ = ora.map_binary_scalar(ora.OP_POW, t, 2, ora.I32, nthreads=nt)
        t, _ = ora.map_binary(ora.OP_MUL, t, w, nt)
        return ora.map_binary(ora.OP_SUB, t, v, nt)[0], None
    if op == "sum":
        if v.dtype == np.int32:
            return ora.reduce(ora.RED_SUM, v, m["axis"]), None
        return ora.reduce_f64(v, m["axis"]), ora.reduce_f64(np.abs(v), m["axis"])
    return ora.reduce(ora.RED_ARGMAX, v, m["axis"], ora.I32), None


@pytest.fixture(scope="module")
def full_batch(cu, ora):
    from phase_cu.batch import Workload

    wl = Workload(n_tasks=10000, seed=0)
    expected = [_oracle_task(ora, wl, i) for i in range(len(wl.meta))]
    return wl, expected


def _check_all(cu, wl, expected, host, what):
    bad = []
    for i, m in enumerate(wl.meta):
        got = np.asarray(wl.task_output(host, i)).reshape(-1)
        exp, mag = expected[i]
        exp = np.asarray(exp).reshape(-1)
        if mag is not None:
            # tolerance: 1e-6 of the sum of magnitudes vs the FP64 oracle
            ok = np.all(np.abs(got.astype(np.float64) - exp) <= 1e-6 * np.asarray(mag).reshape(-1) + 1e-30)
        else:
            ok = np.array_equal(got, exp.astype(got.dtype))
        if not ok:
            bad.append((i, m["op"], m["dtype"], m["vshape"], m["axis"]))
    assert not bad, "%s: %d tasks differ, first %s" % (what, len(bad), bad[:5])


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batch_10000_tasks_every_mode(cu, full_batch, mode):
    from phase_cu import _abi
    from phase_cu.batch import Batch

    wl, expected = full_batch
    _abi.call("phcu_memset", wl.out.ptr, 0xff, wl.out.nbytes)
    b = Batch(wl.tasks(), wl.programs)
    b.launch(mode)
    if mode == 2:
        b.launch(mode)  # a replay of the captured graph
    cu.check_errors()
    host = wl.download_outputs()
    b.close()
    _check_all(cu, wl, expected, host, "mode %d" % mode)


def test_batch_10000_tasks_tuned_layout(cu, full_batch):
    """The learned tuner picks a (work-item size, layout) per task, as the
    benchmark does; the persistent launch of that batch gives the same
    results."""
    from phase_cu import _abi, tuner
    from phase_cu.batch import Batch

    wl, expected = full_batch
    tasks = wl.tasks()
    rng = np.random.default_rng(0)
    sample = rng.choice(len(tasks), 96, replace=False)
    times = np.stack([tuner.measure(tasks[i], wl.programs, reps=2) for i in sample])
    net = tuner.MLP(seed=1)
    feats = tuner.feature_matrix([tasks[i] for i in sample])
    net.train(feats.reshape(-1, 24), np.log2(times.reshape(-1)), epochs=60, batch=256, lr=2e-3)
    picks, _ = net.pick(tuner.feature_matrix(tasks))
    chunks, layouts = tuner.config_args(picks)
    assert len(set(zip(chunks, layouts))) > 1  # the picks are not all one configuration
    _abi.call("phcu_memset", wl.out.ptr, 0xff, wl.out.nbytes)
    b = Batch(wl.tasks(chunks, layouts), wl.programs)
    b.launch(0)
    cu.check_errors()
    host = wl.download_outputs()
    b.close()
    _check_all(cu, wl, expected, host, "tuned")


def test_heat_4096_thousand_steps(cu, ora):
    from phase_cu import stencil, synth

    u0 = synth.gaussian_bumps_f32(4096, 4096, bumps=16, seed=0)
    h = stencil.Heat(u0)
    h.run(1000, use_graph=True)
    assert np.array_equal(h.get(), ora.heat_run(u0, 1000, nthreads=NT))
