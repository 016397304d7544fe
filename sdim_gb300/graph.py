"""A batch run captured once into a CUDA graph and replayed.

``sdim_graph_create`` records the whole shot loop of a batch (descriptor
upload, work-queue resets, the x / z, coin and phase passes of the trace
engines on their streams, the shot-group kernels) as one CUDA graph on a
private context; each ``launch`` is one graph launch.  New seeds or first
shot indices go in through the graph's pinned descriptor copy, so a loop of
steps over fresh shots replays the same graph.  Records are those of
``BatchRunner.run`` with the same seeds and shot ranges.

The reference runs every shot in a Python loop (sdim/program.py:269-365)
and has no graph form.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

from . import _lib


class CapturedRun:
    """Graph of one batch with device outputs (``outs_dev``: one device
    pointer per entry, each holding shots x records bytes).  The entries'
    programs and the output buffers must outlive this object."""

    def __init__(self, ctx: _lib.Context, entries: Sequence, outs_dev: Sequence[int], flags: int = 0):
        self.ctx = ctx
        self.entries = list(entries)
        self._keep = [e.program for e in self.entries]  # programs stay encoded while the graph lives
        k = len(self.entries)
        if len(outs_dev) != k:
            raise ValueError(f"{k} entries but {len(outs_dev)} output pointers")
        circs = (C.c_void_p * k)(*[e.program.ptr.value for e in self.entries])
        seeds = (C.c_uint64 * k)(*[e.seed & 0xFFFFFFFFFFFFFFFF for e in self.entries])
        shot0 = (C.c_int64 * k)(*[e.shot0 for e in self.entries])
        nshots = (C.c_int64 * k)(*[e.shots for e in self.entries])
        outs = (C.c_void_p * k)(*[int(p) for p in outs_dev])
        ptr = C.c_void_p()
        rc = ctx.lib.sdim_graph_create(ctx.ptr, k, circs, seeds, shot0, nshots, outs, int(flags), C.byref(ptr))
        _lib.check(rc, ctx.ptr, "graph capture")
        self.ptr = ptr

    def _check(self, rc: int, what: str):
        if rc == _lib.SDIM_OK:
            return
        raw = self.ctx.lib.sdim_graph_last_error(self.ptr)
        msg = raw.decode() if raw else ""
        if rc == _lib.SDIM_EINVAL:
            raise ValueError(f"{what}: {msg}")
        raise _lib.SdimError(f"{what}: {msg} (status {rc})")

    def launch(self, seeds: Optional[Sequence[int]] = None, shot0: Optional[Sequence[int]] = None,
               stream: Optional[int] = None) -> None:
        """Queues one replay; ``seeds`` / ``shot0`` (one per entry) replace
        the programs' seeds and first shot indices from this replay on."""
        k = len(self.entries)
        s = None
        if seeds is not None:
            if len(seeds) != k:
                raise ValueError(f"{k} entries but {len(seeds)} seeds")
            s = (C.c_uint64 * k)(*[int(v) & 0xFFFFFFFFFFFFFFFF for v in seeds])
        o = None
        if shot0 is not None:
            if len(shot0) != k:
                raise ValueError(f"{k} entries but {len(shot0)} shot offsets")
            o = (C.c_int64 * k)(*[int(v) for v in shot0])
        self._check(self.ctx.lib.sdim_graph_launch(self.ptr, s, o, C.c_void_p(stream) if stream else None),
                    "graph launch")

    def sync(self) -> None:
        """Waits for the last replay; raises on a device-side error."""
        self._check(self.ctx.lib.sdim_graph_sync(self.ptr), "graph replay")

    def info(self) -> dict:
        buf = (C.c_int64 * 3)()
        self._check(self.ctx.lib.sdim_graph_info(self.ptr, buf), "graph info")
        return {"nodes": int(buf[0]), "kernel_nodes": int(buf[1]), "staging_bytes": int(buf[2])}

    def close(self) -> None:
        if getattr(self, "ptr", None):
            self.ctx.lib.sdim_graph_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
