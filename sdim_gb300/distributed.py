"""Multi-GPU replicas: shots are independent, so N ranks split a program's
shot range and only the records are gathered on the host.

No collective touches the data path: each rank runs its own contiguous shot
range on its own GPU; ``gather_records`` concatenates the per-rank records on
rank 0 (torch.distributed object gather, any backend).  Because outcomes and
noise are keyed by the global shot index, the gathered records equal a
single-GPU run of all shots.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np


def shard_shots(total: int, rank: int, world: int, shot0: int = 0) -> Tuple[int, int]:
    """(first shot, count) of ``rank``'s contiguous share of ``total`` shots."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(int(total), int(world))
    count = base + (1 if rank < extra else 0)
    first = shot0 + rank * base + min(rank, extra)
    return first, count


def gather_records(local: np.ndarray, group=None, dst: int = 0) -> Optional[np.ndarray]:
    """Concatenates every rank's (shots, records) array on rank ``dst``."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world if dist.get_rank(group) == dst else None
    dist.gather_object(np.ascontiguousarray(local), parts, dst=dst, group=group)
    if parts is None:
        return None
    return np.concatenate(parts, axis=0)


def run_sharded(program, total_shots: int, seed: int, rank: int, world: int, shot0: int = 0,
                sample_fn=None) -> np.ndarray:
    """Records of this rank's shard; ``sample_fn(program, shots, seed, shot0)``
    defaults to ``program.sample`` (the GPU path)."""
    first, count = shard_shots(total_shots, rank, world, shot0)
    if sample_fn is None:
        return program.sample(count, seed=seed, shot0=first)
    return sample_fn(program, count, seed, first)
