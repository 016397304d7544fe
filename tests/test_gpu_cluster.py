"""GPU: the odd-d x / z pass on a cluster of 8 CTAs (column slices in shared
memory, or streamed from global memory) against the oracle and the other
x / z passes: slices left empty (n < 4), every gate and noise channel,
random outcomes, deterministic outcomes whose factors span every slice, the
largest programs, the default routing of mixed batches, and the layered
stream's gate groups against the gates applied one at a time."""
import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu

CLUSTER = _lib.FLAG_TRACE | _lib.FLAG_CLUSTER_XZ
STREAMED = CLUSTER | _lib.FLAG_FORCE_GMEM


def _run(prog, seed, shot0, shots, flags):
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, shot0, shots, out.ctypes.data, flags)
    _lib.check(rc, ctx.ptr, "odd-d trace pass")
    return out


def _twice_measured(n, d, seed):
    """Random {H, P, CNOT} circuit and MEASURE on every qudit, a layer of
    random X / Z, then MEASURE on every qudit again: the second sweep is all
    deterministic outcomes with factors over every slice."""
    base = workloads.random_hpc(n, d, 4 * n + 10, seed=seed)
    rng = np.random.default_rng(seed)
    ops = list(base.ops)
    ops += [("X" if rng.random() < 0.5 else "Z", int(q), None, {}) for q in rng.integers(n, size=n)]
    ops += [("M", q, None, {}) for q in range(n)]
    return workloads.CircuitSpec(n, d, ops, f"twice_n{n}_d{d}")


@pytest.mark.parametrize("flags", [CLUSTER, STREAMED], ids=["smem", "streamed"])
@pytest.mark.parametrize("d", [3, 5, 7, 11])
@pytest.mark.parametrize("n", [1, 3, 6, 33, 100])
def test_cluster_against_oracle(n, d, flags):
    spec = (workloads.all_gates_random(n, d, 200, seed=5 * d + n, noise_probs=(0.0, 0.3, 1.0)) if n <= 6 else
            workloads.random_hpc(n, d, 5 * n + 20, seed=17 * d + n, mr_every=max(1, n // 2), mr_fraction=0.3))
    rec = _run(Program(spec.build()), d, 3, 70, flags)
    assert np.array_equal(rec, oracle_run([spec], d, 3, 70)["records"]), (n, d)


@pytest.mark.parametrize("flags", [CLUSTER, STREAMED], ids=["smem", "streamed"])
@pytest.mark.parametrize("n,d", [(9, 3), (64, 5), (129, 7), (250, 3)])
def test_deterministic_sweep_across_slices(n, d, flags):
    spec = _twice_measured(n, d, seed=n + d)
    prog = Program(spec.build())
    rec = _run(prog, 11, 0, 40, flags)
    assert np.array_equal(rec[:4], oracle_run([spec], 11, 0, 4)["records"]), (n, d)
    assert np.array_equal(rec, _run(prog, 11, 0, 40, _lib.FLAG_TRACE | _lib.FLAG_SPLIT_XZ)), (n, d)


@pytest.mark.parametrize("n,d", [(400, 7), (642, 5), (643, 3), (1000, 5)])
def test_large_programs_every_odd_d_pass(n, d):
    """Around the shared-memory limit of the cluster's columns (n = 642):
    cluster in shared memory, cluster streamed, one CTA streamed and the
    shot-group engine agree; the oracle checks two shots."""
    spec = workloads.random_hpc(n, d, 2 * n, seed=n, mr_every=n // 2, mr_fraction=0.1)
    prog = Program(spec.build())
    auto = _run(prog, 5, 0, 40, _lib.FLAG_TRACE)
    assert np.array_equal(auto, _run(prog, 5, 0, 40, CLUSTER))
    assert np.array_equal(auto, _run(prog, 5, 0, 40, STREAMED))
    assert np.array_equal(auto, _run(prog, 5, 0, 40, _lib.FLAG_TRACE | _lib.FLAG_FORCE_GMEM))
    assert np.array_equal(auto, prog.sample(40, seed=5, engine="group"))
    assert np.array_equal(auto[:2], oracle_run([spec], 5, 0, 2)["records"])


@pytest.mark.parametrize("large", [False, True], ids=["latency", "throughput"])
def test_mixed_batch_routes_every_mode(large):
    """Default routing in one run, against each program alone on the
    shot-group engine.  Fewer than 76 odd-d trace programs: one CTA
    (n <= 226), clusters in shared memory and streamed clusters.  76 or
    more: one CTA, CTA pairs and single CTAs streaming from global memory."""
    sizes = [(40, 3), (300, 5), (500, 7), (700, 3), (260, 7), (190, 5), (800, 5), (331, 3)]
    if large:
        sizes += [(232 + 3 * i, (3, 5, 7)[i % 3]) for i in range(72)]
    specs = [workloads.random_hpc(n, d, 3 * n, seed=i, mr_every=n, mr_fraction=0.2)
             for i, (n, d) in enumerate(sizes)]
    runner = BatchRunner()
    for i, s in enumerate(specs):
        runner.add_spec(s, 16 + 8 * i, seed=30 + i, shot0=i)
    outs = runner.run()
    for e, s, out in zip(runner.entries, specs, outs):
        prog = Program(s.build())
        assert np.array_equal(out, prog.sample(e.shots, seed=e.seed, shot0=e.shot0, engine="group")), s.name


@pytest.mark.parametrize("flags", [CLUSTER, STREAMED], ids=["smem", "streamed"])
@pytest.mark.parametrize("d", [3, 7, 11])
@pytest.mark.parametrize("kind", ["hpc", "all-gates"])
def test_layered_gate_groups(kind, d, flags):
    """The cluster x / z pass walks the layered stream: gates between
    measurements in groups on disjoint qudits.  Runs of up to 2,000 gates,
    so that groups meet the ends of the 512-word instruction windows; every
    gate kind and N1 between them.  Records equal the gates applied one at a
    time (SDIM_FLAG_UNLAYERED) and the oracle."""
    if kind == "hpc":
        spec = workloads.random_hpc(40, d, 2000, seed=d, mr_every=700, mr_fraction=0.2)
    else:
        spec = workloads.all_gates_random(12, d, 1500, seed=d, noise_probs=(0.0, 0.3, 1.0))
    prog = Program(spec.build())
    rec = _run(prog, 5, 0, 64, flags)
    assert np.array_equal(rec, _run(prog, 5, 0, 64, flags | _lib.FLAG_UNLAYERED)), (kind, d)
    assert np.array_equal(rec[:8], oracle_run([spec], 5, 0, 8)["records"]), (kind, d)
