"""GPU: a batch captured into a CUDA graph (sdim_graph_*) and replayed with
new seeds and shot ranges gives the records of an ordinary sdim_run_batch
with the same values, for batches that use every engine at once: the d = 2
trace engine with its coin pass on a second stream, odd-d trace programs of
two dimensions whose x / z passes fan out over streams (one CTA, an
eight-CTA cluster), and the shot-group engines."""
import numpy as np
import pytest

from sdim_gb300 import _lib, workloads
from sdim_gb300.batch import BatchEntry, BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


def _specs():
    return [
        (workloads.surface_memory(3, 3, prob=0.05), 300),          # d = 2 trace engine + coin pass
        (workloads.random_hpc(40, 3, 160, seed=1), 70),            # shot-group engine, warp teams
        (workloads.random_hpc(240, 5, 960, seed=2, mr_every=120, mr_fraction=0.1), 40),  # odd-d cluster
        (workloads.random_hpc(100, 7, 400, seed=3), 200),          # odd-d trace, one CTA
        (workloads.surface_memory(5, 2, prob=0.01), 64),           # d = 2 shot groups
    ]


def _runner(ctx):
    runner = BatchRunner(ctx)
    for i, (spec, shots) in enumerate(_specs()):
        runner.add_spec(spec, shots=shots, seed=50 + i, shot0=3 * i)
    return runner


def _moved(runner, seeds, shot0):
    return [BatchEntry(e.program, e.shots, s, o) for e, s, o in zip(runner.entries, seeds, shot0)]


@pytest.mark.parametrize("flags", [0, _lib.FLAG_TRACE | _lib.FLAG_CLUSTER_XZ | _lib.FLAG_FORCE_GMEM,
                                   _lib.FLAG_NO_TRACE], ids=["default", "streamed_clusters", "groups"])
def test_graph_replays_equal_batch_runs(cuda_ctx, flags):
    import torch
    runner = _runner(cuda_ctx)
    outs = [torch.empty((e.shots, e.program.num_records), dtype=torch.uint8, device="cuda")
            for e in runner.entries]
    torch.cuda.synchronize()
    run = runner.capture([o.data_ptr() for o in outs], flags=flags)
    try:
        # creation ran the batch once with the captured seeds
        first = runner.run(flags=flags)
        for o, ref in zip(outs, first):
            assert np.array_equal(o.cpu().numpy(), ref)
        info = run.info()
        assert info["kernel_nodes"] >= 2 and info["staging_bytes"] > 0
        for step in range(3):
            seeds = [1000 * step + 7 * i for i in range(len(outs))]
            shot0 = [5000 * step + i for i in range(len(outs))]
            for o in outs:
                o.fill_(0xFF)
            torch.cuda.synchronize()
            run.launch(seeds=seeds, shot0=shot0)
            run.sync()
            ref = runner.run(entries=_moved(runner, seeds, shot0), flags=flags)
            for i, (o, r) in enumerate(zip(outs, ref)):
                assert np.array_equal(o.cpu().numpy(), r), (step, i)
        # the last replay's first shots against the oracle
        spec = _specs()[0][0]
        assert np.array_equal(outs[0][:4].cpu().numpy(), oracle_run([spec], seeds[0], shot0[0], 4)["records"])
        # a replay without new values repeats the last one
        last = [o.cpu().numpy() for o in outs]
        for o in outs:
            o.fill_(0)
        torch.cuda.synchronize()
        run.launch()
        run.sync()
        for o, r in zip(outs, last):
            assert np.array_equal(o.cpu().numpy(), r)
    finally:
        run.close()


def test_graph_refuses_the_plain_form_and_bad_arguments(cuda_ctx):
    import torch
    runner = _runner(cuda_ctx)
    outs = [torch.empty((e.shots, e.program.num_records), dtype=torch.uint8, device="cuda")
            for e in runner.entries]
    with pytest.raises(ValueError, match="plain"):
        runner.capture([o.data_ptr() for o in outs], flags=_lib.FLAG_PLAIN)
    with pytest.raises(ValueError):
        runner.capture([o.data_ptr() for o in outs[:-1]])
    run = runner.capture([o.data_ptr() for o in outs])
    try:
        with pytest.raises(ValueError):
            run.launch(seeds=[1, 2])
    finally:
        run.close()
