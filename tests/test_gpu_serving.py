"""GPU: the continuous-batching request loop.  Requests of uneven n, d and
shot count overlap on the device in several lanes; each result equals the
same request run alone (and the oracle on a subset)."""
import time

import numpy as np
import pytest

from sdim_gb300 import workloads
from sdim_gb300.encode import DeviceProgram, encode_table
from sdim_gb300.serving import Server, replay
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


def _requests(count, seed, n_max=300, shots_max=200):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(4), np.log(n_max)))))
        d = int([2, 3, 5, 7][rng.integers(4)])
        shots = int(rng.integers(1, shots_max + 1))
        table = workloads.random_hpc_table(n, 4 * n, seed=rng, mr_every=max(1, n), mr_fraction=0.1)
        out.append((table, n, d, shots, 1000 + i))
    return out


def _alone(table, n, d, shots, seed):
    from sdim_gb300 import _lib
    ctx = _lib.Context.default(0)
    dp = DeviceProgram(ctx, encode_table(table, n, d))
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, 0, shots, out.ctypes.data, 0), ctx.ptr)
    return out


def test_results_same_alone_and_in_the_mix():
    reqs = _requests(80, seed=5)
    server = Server(lanes=3, max_batch_requests=12)
    try:
        handles = [server.submit(t, n, d, s, seed) for t, n, d, s, seed in reqs]
        results = [h.wait(timeout=600) for h in handles]
        assert server.batches >= 4          # several batches were in flight
    finally:
        server.close()
    for (t, n, d, s, seed), res in zip(reqs, results):
        assert np.array_equal(res, _alone(t, n, d, s, seed))
    for (t, n, d, s, seed), res in list(zip(reqs, results))[:6]:
        spec = workloads.CircuitSpec(n, d, None, "", t)
        assert np.array_equal(res, oracle_run([spec], seed, 0, s)["records"])


def test_open_loop_trace_latency_stats():
    reqs = _requests(120, seed=9, n_max=128, shots_max=64)
    rng = np.random.Generator(np.random.PCG64(1))
    arrivals = np.cumsum(rng.exponential(1 / 400.0, size=len(reqs)))
    trace = [(a, *r) for a, r in zip(arrivals, reqs)]
    server = Server(lanes=4)
    try:
        done = replay(server, trace)
        st = server.stats(done)
    finally:
        server.close()
    assert st["requests"] == len(reqs)
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    assert all(r.launched >= r.arrival and r.done >= r.launched for r in done)


def test_tight_memory_budget_still_serves_everything():
    reqs = _requests(10, seed=2, n_max=64, shots_max=32)
    server = Server(lanes=2, memory_fraction=1e-12)
    try:
        handles = [server.submit(t, n, d, s, seed) for t, n, d, s, seed in reqs]
        results = [h.wait(timeout=600) for h in handles]
    finally:
        server.close()
    for (t, n, d, s, seed), res in zip(reqs, results):
        assert np.array_equal(res, _alone(t, n, d, s, seed))


def test_chp_requests_match_the_circuit_route():
    """Requests given as .chp text (native parser) give the records of the
    same circuit read by read_circuit and sampled through Program."""
    from sdim_gb300 import Program, circuit_io
    texts = []
    for k, (n, d) in enumerate([(5, 2), (9, 3), (17, 5), (4, 7)]):
        spec = workloads.all_gates_random(n, d, 30 * n, seed=50 + k, name="chp")
        texts.append(circuit_io.chp_text(spec.build()))
    server = Server(lanes=2, max_batch_requests=4)
    try:
        reqs = [server.submit_chp(t, shots=40 + 7 * k, seed=300 + k) for k, t in enumerate(texts)]
        got = [r.wait(120) for r in reqs]
    finally:
        server.close()
    for k, (t, rec) in enumerate(zip(texts, got)):
        want = Program(circuit_io.circuit_from_chp(t)).sample(40 + 7 * k, seed=300 + k)
        assert np.array_equal(rec, want), k
