"""Batched execution of many programs (uneven n, d, depth and shots).

The reference has no batch API: each program is a ``Program.simulate`` call
(sdim/program.py:206-267).  ``BatchRunner`` encodes every program once and runs
all (program, shot) items through ``sdim_run_batch``: one persistent launch
per engine variant, fed by a device work queue, largest programs first.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .encode import DeviceProgram, encode_program, encode_table


@dataclass
class BatchEntry:
    program: DeviceProgram
    shots: int
    seed: int
    shot0: int = 0


class BatchRunner:
    def __init__(self, ctx: Optional[_lib.Context] = None):
        self.ctx = ctx or _lib.Context.default(0)
        self.entries: List[BatchEntry] = []

    def add_spec(self, spec, shots: int, seed: int, shot0: int = 0, noise: bool = True) -> BatchEntry:
        if getattr(spec, "table", None) is not None:
            enc = encode_table(spec.table, spec.num_qudits, spec.dimension)
        else:
            enc = encode_program([spec.build()], spec.num_qudits, spec.dimension, noise=noise)
        e = BatchEntry(DeviceProgram(self.ctx, enc), int(shots), int(seed), int(shot0))
        self.entries.append(e)
        return e

    def add_program(self, program: DeviceProgram, shots: int, seed: int, shot0: int = 0) -> BatchEntry:
        e = BatchEntry(program, int(shots), int(seed), int(shot0))
        self.entries.append(e)
        return e

    @staticmethod
    def _arrays(entries):
        k = len(entries)
        circs = (C.c_void_p * k)(*[e.program.ptr.value for e in entries])
        seeds = (C.c_uint64 * k)(*[e.seed & 0xFFFFFFFFFFFFFFFF for e in entries])
        shot0 = (C.c_int64 * k)(*[e.shot0 for e in entries])
        nshots = (C.c_int64 * k)(*[e.shots for e in entries])
        return circs, seeds, shot0, nshots

    @staticmethod
    def _flags(plain=False, per_shot=False, time_kernels=False, asynchronous=False, device=False, engine=None):
        return ((_lib.FLAG_PLAIN if plain else 0) | (_lib.FLAG_PER_SHOT if per_shot else 0)
                | (_lib.FLAG_TIME if time_kernels else 0) | (_lib.FLAG_ASYNC if asynchronous else 0)
                | (_lib.FLAG_OUT_DEVICE if device else 0) | _lib.engine_flags(engine))

    def run(self, plain: bool = False, per_shot: bool = False, time_kernels: bool = False,
            entries: Optional[Sequence[BatchEntry]] = None,
            outs: Optional[Sequence[np.ndarray]] = None, engine: Optional[str] = None,
            flags: int = 0) -> List[np.ndarray]:
        """Runs every entry; returns one (shots, records) uint8 array each
        (into ``outs`` when given, e.g. views of a pinned buffer).

        ``engine="tuned"`` runs the route the autotuner picked for this
        batch's composition (timing the routes on the first call);
        ``flags`` adds raw SDIM_FLAG_* route flags."""
        entries = list(self.entries if entries is None else entries)
        if engine == "tuned":
            from .autotune import default_tuner
            flags |= default_tuner(self.ctx).flags_for_batch(BatchRunner._view(self.ctx, entries))
            engine = None
        if outs is None:
            outs = [np.empty((e.shots, e.program.num_records), dtype=np.uint8) for e in entries]
        ptrs = (C.c_void_p * len(entries))(*[o.ctypes.data for o in outs])
        circs, seeds, shot0, nshots = self._arrays(entries)
        rc = self.ctx.lib.sdim_run_batch(self.ctx.ptr, len(entries), circs, seeds, shot0, nshots, ptrs, None,
                                         self._flags(plain, per_shot, time_kernels, engine=engine) | int(flags))
        _lib.check(rc, self.ctx.ptr, "batch")
        return list(outs)

    def run_device(self, outs_dev: Sequence[int], stream: Optional[int] = None, plain: bool = False,
                   per_shot: bool = False, time_kernels: bool = False, asynchronous: bool = False,
                   entries: Optional[Sequence[BatchEntry]] = None, engine: Optional[str] = None):
        """Same with device output pointers (e.g. ``tensor.data_ptr()``)."""
        entries = list(self.entries if entries is None else entries)
        ptrs = (C.c_void_p * len(entries))(*[int(p) for p in outs_dev])
        circs, seeds, shot0, nshots = self._arrays(entries)
        rc = self.ctx.lib.sdim_run_batch(self.ctx.ptr, len(entries), circs, seeds, shot0, nshots, ptrs,
                                         C.c_void_p(stream) if stream else None,
                                         self._flags(plain, per_shot, time_kernels, asynchronous, True, engine))
        _lib.check(rc, self.ctx.ptr, "batch")

    def capture(self, outs_dev: Sequence[int], engine: Optional[str] = None, flags: int = 0,
                entries: Optional[Sequence[BatchEntry]] = None):
        """The batch as a CUDA graph (graph.CapturedRun) with device outputs;
        creating it runs the batch once."""
        from .graph import CapturedRun
        entries = list(self.entries if entries is None else entries)
        return CapturedRun(self.ctx, entries, outs_dev, self._flags(engine=engine) | int(flags))

    @staticmethod
    def _view(ctx, entries) -> "BatchRunner":
        r = BatchRunner(ctx)
        r.entries = list(entries)
        return r

    def total_shots(self) -> int:
        return sum(e.shots for e in self.entries)

    def total_gate_updates(self) -> int:
        return sum(e.shots * e.program.num_instructions for e in self.entries)
