"""CPU: the replica split across ranks (world size 2, gloo).  Each rank runs
its shard -- on CPU the oracle stands in for the GPU run -- and the gathered
records equal one run of all shots."""
import os
import socket

import numpy as np
import pytest

from sdim_gb300.distributed import shard_shots


def test_shard_shots_cover_range_exactly():
    for total in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [shard_shots(total, r, world, shot0=5) for r in range(world)]
            assert sum(c for _, c in spans) == total
            pos = 5
            for first, count in spans:
                assert first == pos
                pos += count
    with pytest.raises(ValueError):
        shard_shots(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    import oracle
    from sdim_gb300 import workloads
    from sdim_gb300.distributed import gather_records, run_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = workloads.surface_memory(3, 2, prob=0.05)
    prog = oracle.OracleProgram([spec], spec.num_qudits, 2)

    def sample_fn(p, count, seed, first):
        return oracle.simulate(p, seed, first, count, threads=1)["records"]

    local = run_sharded(prog, 45, 9, rank, world, sample_fn=sample_fn)
    full = gather_records(local)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gather_equals_single_run(tmp_path):
    import torch.multiprocessing as mp

    import oracle
    from sdim_gb300 import workloads

    out = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    spec = workloads.surface_memory(3, 2, prob=0.05)
    ref = oracle.simulate(oracle.OracleProgram([spec], spec.num_qudits, 2), 9, 0, 45)["records"]
    assert np.array_equal(np.load(out), ref)
