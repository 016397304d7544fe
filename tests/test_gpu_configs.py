"""GPU parity at the stated workload sizes.

* The uneven batch at full size (8,192 programs, n log-uniform in [8, 1024],
  d in {2, 3, 5, 7}, 4n gates + MEASURE all, 1-64 shots), run as one batch:
  every program's deterministic flags agree across its shots (the x / z part
  is shot-independent), and every 64th program equals the oracle -- all its
  shots up to n = 256, its first and last shot up to n = 600, its last shot
  above (the C oracle needs about 20 core-seconds per shot at n = 1024).
* Requests drawn from the serving distribution (n log-uniform in
  [16, 2048], d in {2, 3, 5}, 8n gates + MEASURE all, shots log-uniform in
  [1, 10^4]) served together by the continuous-batching loop: each result
  equals the same request run alone, and the oracle for the requests of
  n <= 200 (first 16 shots).
* The odd-d n = 256 workloads at their bench size (4,096 shots, the
  library's default route) against the oracle on the first and last 64
  shots.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from sdim_gb300 import workloads
from sdim_gb300.batch import BatchRunner
from sdim_gb300.encode import DeviceProgram, encode_table
from sdim_gb300.serving import Server
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


def _oracle_tasks(tasks):
    """Runs (spec, seed, shot0, nshots) oracle tasks on a thread pool, one
    OpenMP thread each (the C call releases the interpreter lock)."""
    def one(task):
        spec, seed, shot0, k = task
        prog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
        return oracle.simulate(prog, seed, shot0, k, threads=1)["records"]
    with ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        return list(ex.map(one, tasks))


def test_uneven_batch_full_size_against_oracle():
    items = workloads.uneven_batch(8192, seed=0)
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    outs = br.run()
    assert len(outs) == 8192
    for it, out in zip(items, outs):
        assert out.shape == (it.shots, it.spec.num_qudits)
        flags = out >> 7
        assert np.all(flags == flags[0]), it.spec.name
    tasks, where = [], []
    for k in range(0, len(items), 64):
        it = items[k]
        n, s = it.spec.num_qudits, it.shots
        if n <= 256:
            ranges = [(0, s)]
        elif n <= 600:
            ranges = [(0, 1), (s - 1, 1)] if s > 1 else [(0, 1)]
        else:
            ranges = [(s - 1, 1)]
        for a, c in ranges:
            tasks.append((it.spec, it.seed, a, c))
            where.append((k, a, c))
    refs = _oracle_tasks(tasks)
    assert len(tasks) >= 128
    for (k, a, c), ref in zip(where, refs):
        assert np.array_equal(outs[k][a:a + c], ref), (items[k].spec.name, a)


def _serving_requests(count, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(16), np.log(2048)))))
        d = int((2, 3, 5)[rng.integers(3)])
        shots = max(1, int(round(np.exp(rng.uniform(0.0, np.log(10_000))))))
        table = workloads.random_hpc_table(n, 8 * n, seed=rng)
        out.append((table, n, d, shots, 7000 + i))
    return out


def _alone(table, n, d, shots, seed):
    from sdim_gb300 import _lib
    ctx = _lib.Context.default(0)
    dp = DeviceProgram(ctx, encode_table(table, n, d))
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, 0, shots, out.ctypes.data, 0), ctx.ptr)
    return out


def test_serving_distribution_mixed_equals_alone_and_oracle():
    reqs = _serving_requests(40, seed=7)
    assert max(r[1] for r in reqs) > 1500 and max(r[3] for r in reqs) > 5000
    server = Server(lanes=4)
    try:
        handles = [server.submit(t, n, d, s, seed) for t, n, d, s, seed in reqs]
        results = [h.wait(timeout=900) for h in handles]
    finally:
        server.close()
    for (t, n, d, s, seed), res in zip(reqs, results):
        assert np.array_equal(res, _alone(t, n, d, s, seed)), (n, d, s)
    small = [(r, res) for r, res in zip(reqs, results) if r[1] <= 200]
    assert len(small) >= 10
    refs = _oracle_tasks([(workloads.CircuitSpec(n, d, None, "", t), seed, 0, min(s, 16))
                          for (t, n, d, s, seed), _ in small])
    for ((t, n, d, s, seed), res), ref in zip(small, refs):
        assert np.array_equal(res[:min(s, 16)], ref), (n, d, s)


@pytest.mark.parametrize("d", [5, 7])
def test_odd_d_n256_bench_size(d):
    from sdim_gb300 import Program
    spec = workloads.odd_d(d, seed=0)
    prog = Program(spec.build())
    rec = prog.sample(4096, seed=0)
    flags = rec >> 7
    assert np.all(flags == flags[0])
    refs = _oracle_tasks([(spec, 0, a, 8) for a in list(range(0, 64, 8)) + list(range(4032, 4096, 8))])
    ref = np.concatenate(refs)
    assert np.array_equal(rec[:64], ref[:64])
    assert np.array_equal(rec[4032:], ref[64:])
