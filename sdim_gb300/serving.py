"""Continuous-batching request loop for simulate requests.

The reference serves one ``Program.simulate`` call at a time
(sdim/program.py:206-267).  ``Server`` accepts requests of any qudit count,
dimension and shot count, and keeps several batches in flight on the GPU:

* a *lane* is one library context with its own CUDA stream, device buffers
  (records, slots, instruction arena) and pinned host buffer; one batch runs
  per lane;
* the scheduler thread admits pending requests into a free lane in arrival
  order while the lane's batch stays within a shot budget and the server's
  device-memory budget (records plus one shot-group slot per program,
  checked against ``cudaMemGetInfo`` at start-up), then launches the whole
  batch with one ``sdim_run_tables`` call (asynchronous, records copied to
  pinned host memory on the lane's stream);
* requests that arrive while other batches run are admitted as soon as a lane
  and memory are free, so their kernels overlap with the running ones;
* every request records its arrival, launch and completion times, from
  which ``stats()`` reports p50 / p99 latency and throughput.

Results are bit-identical to running the request alone: outcomes and noise
come from the (seed, shot, ordinal) Philox stream, independent of batching.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib


@dataclass
class Request:
    table: np.ndarray          # int32 rows (gate id, qudit, target, channel)
    n: int
    d: int
    shots: int
    seed: int
    probs: Optional[np.ndarray] = None
    shot0: int = 0
    ident: int = 0
    nmeas: int = 0
    arrival: float = 0.0
    launched: float = 0.0
    done: float = 0.0
    records: Optional[np.ndarray] = None
    error: Optional[str] = None
    solo: bool = False         # run alone: its batch was refused, so each request is retried by itself
    event: threading.Event = field(default_factory=threading.Event)

    def wait(self, timeout: Optional[float] = None) -> np.ndarray:
        if not self.event.wait(timeout):
            raise TimeoutError(f"request {self.ident} not done")
        if self.error:
            raise RuntimeError(self.error)
        return self.records

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class _PinnedBuffer:
    def __init__(self, lib):
        self.lib, self.ptr, self.cap = lib, C.c_void_p(), 0

    def ensure(self, nbytes: int):
        if nbytes <= self.cap:
            return
        if self.ptr.value:
            self.lib.sdim_host_free(self.ptr)
        cap = max(nbytes, self.cap + self.cap // 2, 1 << 20)
        rc = self.lib.sdim_host_alloc(cap, C.byref(self.ptr))
        if rc != 0:
            raise MemoryError("pinned host allocation failed")
        self.cap = cap

    def view(self, offset: int, nbytes: int) -> np.ndarray:
        return np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(self.ptr.value + offset))

    def free(self):
        if self.ptr.value:
            self.lib.sdim_host_free(self.ptr)
            self.ptr = C.c_void_p()
            self.cap = 0


class _Lane:
    def __init__(self, device: int, context=_lib.Context):
        self.ctx = context(device)
        self.buf = _PinnedBuffer(self.ctx.lib)
        self.requests: List[Request] = []
        self.offsets: List[int] = []
        self.bytes = 0
        self.busy = False


class Server:
    def __init__(self, device: int = 0, lanes: int = 4, max_batch_requests: int = 1024,
                 max_batch_shots: int = 1 << 20, memory_fraction: float = 0.5, context=_lib.Context):
        # context: the class that opens a lane's library context (a test passes a fake)
        self.lanes = [_Lane(device, context) for _ in range(max(1, lanes))]
        self.max_batch_requests = max_batch_requests
        self.max_batch_shots = max_batch_shots
        info = (C.c_int64 * 3)()
        _lib.check(self.lanes[0].ctx.lib.sdim_memory_info(self.lanes[0].ctx.ptr, info), self.lanes[0].ctx.ptr)
        self.mem_budget = int(info[0] * memory_fraction)
        self.mem_in_use = 0
        self._pending: deque = deque()
        self._lock = threading.Lock()
        self._wake = threading.Condition(self._lock)
        self._stop = False
        self._next_id = 0
        self.completed: List[Request] = []
        self.batches = 0
        self._thread = threading.Thread(target=self._loop, name="sdim-serving", daemon=True)
        self._thread.start()

    # ------------------------------------------------------------------
    def submit(self, table: np.ndarray, n: int, d: int, shots: int, seed: int,
               probs: Optional[np.ndarray] = None, shot0: int = 0) -> Request:
        table = np.ascontiguousarray(table, dtype=np.int32).reshape(-1, 4)
        nmeas = int(np.isin(table[:, 0], (14, 15, 16)).sum())
        req = Request(table, int(n), int(d), int(shots), int(seed), probs, int(shot0), nmeas=nmeas)
        with self._wake:
            req.ident = self._next_id
            self._next_id += 1
            req.arrival = time.perf_counter()
            self._pending.append(req)
            self._wake.notify()
        return req

    def submit_chp(self, text, shots: int, seed: int, shot0: int = 0) -> Request:
        """A request given as .chp text, parsed natively into its op table
        (``circuit_io.read_chp_table``) with no Circuit objects."""
        from .circuit_io import read_chp_table
        table, probs, n, d = read_chp_table(text)
        return self.submit(table, n, d, shots, seed, probs=probs, shot0=shot0)

    def close(self):
        with self._wake:
            self._stop = True
            self._wake.notify()
        self._thread.join()
        for lane in self.lanes:
            lane.buf.free()
            lane.ctx.close()

    def drain(self, timeout: float = 600.0):
        """Waits until every submitted request is done."""
        t0 = time.perf_counter()
        while True:
            with self._lock:
                idle = not self._pending and not any(l.busy for l in self.lanes)
            if idle:
                return
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")
            time.sleep(0.001)

    # ------------------------------------------------------------------
    @staticmethod
    def _cost(req: Request) -> int:
        # device records + a generous bound on slots and instruction arena
        return 2 * req.shots * max(req.nmeas, 1) + 64 * req.table.shape[0] + 8 * req.n * req.n

    def _error_text(self, lane: _Lane, rc: int) -> str:
        raw = lane.ctx.lib.sdim_last_error(lane.ctx.ptr)
        return (raw.decode() if raw else "") or f"status {rc}"

    def _retire(self, lane: _Lane, err: Optional[str] = None):
        """Hands the lane's records to its requests.  ``err``: the batch
        failed before it reached the device (its records were never written)."""
        rc = lane.ctx.lib.sdim_sync(lane.ctx.ptr)
        now = time.perf_counter()
        if err is None and rc != 0:
            err = self._error_text(lane, rc)
        for req, off in zip(lane.requests, lane.offsets):
            if err is None:
                nb = req.shots * req.nmeas
                req.records = lane.buf.view(off, nb).copy().reshape(req.shots, req.nmeas) if nb else \
                    np.zeros((req.shots, req.nmeas), np.uint8)
            req.error = err
            req.done = now
            req.event.set()
        with self._lock:
            self.mem_in_use -= sum(self._cost(r) for r in lane.requests)
            self.completed.extend(lane.requests)
            lane.requests, lane.offsets, lane.busy = [], [], False

    def _launch(self, lane: _Lane, batch: List[Request]):
        """Launches a batch on a free lane.  A batch that the library refuses
        (one request with a bad gate, qudit or dimension fails the whole call)
        goes back to the head of the queue with every request marked to run
        alone, so only the bad request fails."""
        try:
            rc = self._start(lane, batch)
        except Exception as exc:  # the scheduler thread must outlive any one batch
            lane.requests, lane.offsets, lane.busy = batch, [0] * len(batch), True
            self._retire(lane, f"{type(exc).__name__}: {exc}")
            return
        if rc == 0:
            return
        err = self._error_text(lane, rc)
        if len(batch) > 1:
            with self._lock:
                self.mem_in_use -= sum(self._cost(r) for r in batch)
                for r in reversed(batch):
                    r.solo = True
                    self._pending.appendleft(r)
                lane.requests, lane.offsets, lane.busy = [], [], False
            return
        self._retire(lane, err)

    def _start(self, lane: _Lane, batch: List[Request]) -> int:
        k = len(batch)
        rows = np.concatenate([r.table for r in batch], axis=0)
        row_begin = np.zeros(k + 1, dtype=np.int64)
        row_begin[1:] = np.cumsum([r.table.shape[0] for r in batch])
        if any(r.probs is not None for r in batch):
            probs = np.concatenate([r.probs if r.probs is not None else np.zeros(r.table.shape[0])
                                    for r in batch]).astype(np.float64)
        else:
            probs = None
        ns = np.asarray([r.n for r in batch], dtype=np.int32)
        ds = np.asarray([r.d for r in batch], dtype=np.int32)
        seeds = (C.c_uint64 * k)(*[r.seed & 0xFFFFFFFFFFFFFFFF for r in batch])
        shot0 = (C.c_int64 * k)(*[r.shot0 for r in batch])
        nshots = (C.c_int64 * k)(*[r.shots for r in batch])
        offs, total = [], 0
        for r in batch:
            offs.append(total)
            total += r.shots * r.nmeas
        lane.buf.ensure(total)
        outs = (C.c_void_p * k)(*[lane.buf.ptr.value + o for o in offs])
        now = time.perf_counter()
        for r in batch:
            r.launched = now
        lane.requests, lane.offsets, lane.busy = batch, offs, True
        rc = lane.ctx.lib.sdim_run_tables(lane.ctx.ptr, k, rows.ctypes.data, row_begin.ctypes.data,
                                          probs.ctypes.data if probs is not None else None, ns.ctypes.data,
                                          ds.ctypes.data, seeds, shot0, nshots, outs, None, _lib.FLAG_ASYNC)
        self.batches += 1
        return rc

    def _admit(self) -> List[Request]:
        batch, shots = [], 0
        while self._pending and len(batch) < self.max_batch_requests:
            req = self._pending[0]
            cost = self._cost(req)
            if batch and (req.solo or batch[0].solo or shots + req.shots > self.max_batch_shots
                          or self.mem_in_use + cost > self.mem_budget):
                break
            if not batch and self.mem_in_use + cost > self.mem_budget and any(l.busy for l in self.lanes):
                break  # wait for memory to free up
            self._pending.popleft()
            batch.append(req)
            shots += req.shots
            self.mem_in_use += cost
        return batch

    def _loop(self):
        while True:
            for lane in self.lanes:
                if lane.busy and lane.ctx.lib.sdim_query(lane.ctx.ptr) != 0:
                    self._retire(lane)
            with self._wake:
                if self._stop and not self._pending and not any(l.busy for l in self.lanes):
                    return
                free = [l for l in self.lanes if not l.busy]
                batch = self._admit() if (free and self._pending) else []
                if batch:
                    free[0].busy = True  # under the lock: drain() never sees the batch in neither place
                elif not any(l.busy for l in self.lanes):
                    self._wake.wait(timeout=0.01)
                    continue
            if batch:
                self._launch(free[0], batch)
            else:
                time.sleep(0.0002)

    # ------------------------------------------------------------------
    def stats(self, requests: Optional[List[Request]] = None) -> dict:
        reqs = requests if requests is not None else self.completed
        done = [r for r in reqs if r.done and not r.error]
        if not done:
            return {"requests": 0}
        lat = np.array([r.latency for r in done]) * 1e3
        t0 = min(r.arrival for r in done)
        t1 = max(r.done for r in done)
        shots = sum(r.shots for r in done)
        updates = sum(r.shots * r.table.shape[0] for r in done)
        return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "span_s": t1 - t0, "shots_per_s": shots / (t1 - t0), "gate_updates_per_s": updates / (t1 - t0),
                "batches": self.batches}


def replay(server: Server, trace, time_scale: float = 1.0) -> List[Request]:
    """Open-loop replay: submits each (arrival_s, table, n, d, shots, seed)
    at its arrival time (scaled) and waits for all of them."""
    t0 = time.perf_counter()
    reqs = []
    for arrival, table, n, d, shots, seed in trace:
        target = t0 + arrival * time_scale
        delay = target - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        reqs.append(server.submit(table, n, d, shots, seed))
    for r in reqs:
        r.wait(timeout=3600)
    return reqs
