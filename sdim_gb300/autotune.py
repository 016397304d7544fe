"""Autotuner: picks the route of a run by timing the alternatives on the device.

The library routes every run by fixed rules over (n, d, shots, batch size,
the device's shared memory); each rule has a run flag that overrides it.  The
tuner times those overrides on the caller's own workload and keeps the
fastest.  Its knobs:

* engine and tableaux per CTA: the trace engines (one x / z pass per
  program), the shot-group engine with one 32-shot group per warp (many
  tableaux per CTA) or one per CTA, or one warp per shot;
* residency: tableaux in shared memory where they fit, or in global memory
  (``FLAG_FORCE_GMEM``);
* the odd-d x / z pass form: one CTA, a CTA pair, an eight-CTA cluster, and
  the packed tableau (bit planes for d = 3, 4-bit lanes for d = 5, 7) or
  residue bytes (``sdim_trace_xz_mode``
  tells which flags change the form, so equal forms are timed once);
* for d = 2 the N1 coins in their own pass or inside the phase pass, and
  one or two shots per phase-pass lane.

Rows in flight per thread are fixed per kernel form at compile time (16 for a
tableau streamed from global memory, 8 for a CTA team, 4 in shared memory)
and are not a run-time knob.

Every candidate runs the same seeds and shot ranges.  Random streams are
keyed by (seed, shot, ordinal), so every route gives the same records; the
tuner checks that bit for bit against the library's default route and
raises on a difference.  A candidate whose first timed run is
``abort_factor`` times slower than the best so far is not repeated.

Choices are cached per device (SM count and shared memory), keyed by the
program's class: d, n and shots by half-octave, the noise flag.  A batch is
keyed by its exact composition.  The cache is in memory, and in a JSON file
when a path is given (or ``SDIM_GB300_AUTOTUNE_CACHE`` names one).

The reference has no counterpart: it runs one Python shot loop
(sdim/program.py:269-365).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
import os
import threading
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np

from . import _lib

# limits of the library's routes (abi.cu: trace_words, kTraceU8MaxQudits,
# kCtaTeamQudits, kColumnMaxWords); candidates outside them would fall back to
# another route
TRACE_BITS_MAX_QUDITS = 2048
TRACE_U8_MAX_QUDITS = 2048
COLUMN_MAX_QUDITS = 512
CTA_TEAM_QUDITS = 160
# the per-shot engine is a candidate for runs of fewer shots than this: a
# partial 32-shot group leaves lanes of the shot-group engine idle
PER_SHOT_MAX_SHOTS = 64
# shots of one timed program run; larger requests are tuned at this size
TUNE_MAX_SHOTS = 1 << 17

_XZ_FORM = {0: "one CTA", 1: "CTA pair", 2: "one CTA, global memory", 3: "8-CTA cluster",
            4: "8-CTA cluster, global memory", 5: "one CTA, bit planes", 6: "one CTA, bit planes in global memory",
            7: "one CTA, 4-bit lanes", 8: "one CTA, 4-bit lanes in global memory"}


@dataclass(frozen=True)
class Candidate:
    name: str
    flags: int


@dataclass
class TuneResult:
    key: str
    best: Candidate
    times_ms: Dict[str, float] = field(default_factory=dict)
    aborted: List[str] = field(default_factory=list)

    def to_json(self) -> dict:
        return {"best": self.best.name, "flags": self.best.flags, "times_ms": self.times_ms,
                "aborted": self.aborted}

    @classmethod
    def from_json(cls, key: str, obj: dict) -> "TuneResult":
        return cls(key, Candidate(obj["best"], int(obj["flags"])), dict(obj.get("times_ms", {})),
                   list(obj.get("aborted", [])))


def _xz_mode(n: int, d: int, programs: int, flags: int, smem_optin: int, num_sms: int) -> int:
    rc = _lib.load().sdim_trace_xz_mode(int(n), int(d), int(programs), int(flags), int(smem_optin), int(num_sms))
    if rc < 0:
        raise ValueError(f"no odd-d x / z pass form for n = {n}")
    return rc


def program_candidates(d: int, n: int, shots: int, smem_optin: int, num_sms: int) -> List[Candidate]:
    """Routes worth timing for one program of n qudits, dimension d."""
    out = [Candidate("default", 0)]
    trace_ok = n <= (TRACE_BITS_MAX_QUDITS if d == 2 else TRACE_U8_MAX_QUDITS)
    if trace_ok:
        out.append(Candidate("trace", _lib.FLAG_TRACE))
        if d == 2:
            if n <= COLUMN_MAX_QUDITS:
                out.append(Candidate("trace, record columns", _lib.FLAG_TRACE | _lib.FLAG_COLUMNS))
            replay = _lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY
            out.append(Candidate("trace, phase replay", replay))
            out.append(Candidate("trace, coins in the phase pass", _lib.FLAG_TRACE | _lib.FLAG_NO_COIN_PASS))
            out.append(Candidate("trace, phase replay, one shot per lane", replay | _lib.FLAG_LANE_SHOTS_1))
            out.append(Candidate("trace, global memory", _lib.FLAG_TRACE | _lib.FLAG_FORCE_GMEM))
        else:
            seen = {_xz_mode(n, d, 1, 0, smem_optin, num_sms)}
            for extra in (_lib.FLAG_SPLIT_XZ, _lib.FLAG_CLUSTER_XZ, _lib.FLAG_FORCE_GMEM,
                          _lib.FLAG_CLUSTER_XZ | _lib.FLAG_FORCE_GMEM, _lib.FLAG_U8_XZ,
                          _lib.FLAG_U8_XZ | _lib.FLAG_FORCE_GMEM, _lib.FLAG_PACKED_XZ,
                          _lib.FLAG_PACKED_XZ | _lib.FLAG_FORCE_GMEM):
                mode = _xz_mode(n, d, 1, extra, smem_optin, num_sms)
                if mode not in seen:
                    seen.add(mode)
                    out.append(Candidate(f"trace, x/z pass on {_XZ_FORM[mode]}", _lib.FLAG_TRACE | extra))
    out.append(Candidate("shot groups", _lib.FLAG_NO_TRACE))
    if n >= CTA_TEAM_QUDITS:
        out.append(Candidate("shot groups, one per warp", _lib.FLAG_TEAM_WARP))
    else:
        out.append(Candidate("shot groups, one per CTA", _lib.FLAG_TEAM_CTA))
    out.append(Candidate("shot groups, global memory", _lib.FLAG_NO_TRACE | _lib.FLAG_FORCE_GMEM))
    if shots < PER_SHOT_MAX_SHOTS:
        out.append(Candidate("one warp per shot", _lib.FLAG_PER_SHOT))
    return out


def batch_candidates() -> List[Candidate]:
    """Routes worth timing for a batch: one flag word applies to every program."""
    return [Candidate("default", 0),
            Candidate("trace engines at any shot count", _lib.FLAG_TRACE),
            Candidate("shot groups only", _lib.FLAG_NO_TRACE),
            Candidate("odd-d x/z passes on CTA pairs", _lib.FLAG_SPLIT_XZ),
            Candidate("odd-d x/z passes on 8-CTA clusters", _lib.FLAG_CLUSTER_XZ),
            Candidate("odd-d x/z passes on residue bytes", _lib.FLAG_U8_XZ),
            Candidate("odd-d packed x/z passes whatever the batch size", _lib.FLAG_PACKED_XZ),
            Candidate("d=2 coins in the phase pass", _lib.FLAG_NO_COIN_PASS),
            Candidate("d=2 one shot per phase-pass lane", _lib.FLAG_LANE_SHOTS_1)]


def _octave(v: int) -> int:
    """Half-octave bucket of a positive count."""
    return int(round(2 * math.log2(max(int(v), 1))))


# (flags) -> (records, kernel milliseconds)
Measure = Callable[[int], Tuple[np.ndarray, float]]


def tune(key: str, candidates: List[Candidate], measure: Measure, reps: int = 3,
         abort_factor: float = 4.0) -> TuneResult:
    """Times every candidate (one warm-up run, then ``reps`` timed runs,
    median) and returns the fastest.  Raises when a candidate's records
    differ from the first candidate's."""
    if not candidates:
        raise ValueError("no candidates to tune")
    ref = None
    times: Dict[str, float] = {}
    aborted: List[str] = []
    best: Optional[Candidate] = None
    for cand in candidates:
        rec, _ = measure(cand.flags)
        if ref is None:
            ref = np.array(rec, copy=True)
        elif not np.array_equal(rec, ref):
            raise RuntimeError(f"autotune: route {cand.name!r} gave records that differ from {candidates[0].name!r}")
        runs = []
        for _ in range(max(1, reps)):
            _, ms = measure(cand.flags)
            runs.append(float(ms))
            if best is not None and ms > abort_factor * times[best.name]:
                aborted.append(cand.name)
                break
        times[cand.name] = float(np.median(runs))
        if best is None or times[cand.name] < times[best.name]:
            best = cand
    return TuneResult(key, best, times, aborted)


class Autotuner:
    """Per-device cache of tuned routes, filled by timing on first use."""

    def __init__(self, ctx: Optional[_lib.Context] = None, cache_path: Optional[str] = None, reps: int = 3,
                 abort_factor: float = 4.0):
        self._ctx = ctx
        env = os.environ.get("SDIM_GB300_AUTOTUNE_CACHE")
        self.cache_path = Path(cache_path) if cache_path else (Path(env) if env else None)
        self.reps = reps
        self.abort_factor = abort_factor
        self._lock = threading.Lock()
        self.results: Dict[str, TuneResult] = {}
        if self.cache_path is not None and self.cache_path.exists():
            self.load(self.cache_path)

    @property
    def ctx(self) -> _lib.Context:
        if self._ctx is None:
            self._ctx = _lib.Context.default(0)
        return self._ctx

    # -- keys ----------------------------------------------------------
    def device_key(self) -> str:
        return f"sm{self.ctx.num_sms}-smem{self.ctx.smem_optin}"

    def program_key(self, d: int, n: int, shots: int, noise: bool = True) -> str:
        return f"{self.device_key()}/program/d{d}/n{_octave(n)}/s{_octave(shots)}/noise{int(bool(noise))}"

    def batch_key(self, items: List[Tuple[int, int, int, int]]) -> str:
        """items: (d, n, instructions, shots) of every program in the batch."""
        h = hashlib.sha1(json.dumps(sorted(items)).encode()).hexdigest()[:16]
        return f"{self.device_key()}/batch/{len(items)}/{h}"

    # -- cache ---------------------------------------------------------
    def load(self, path) -> None:
        data = json.loads(Path(path).read_text())
        for key, obj in data.items():
            self.results[key] = TuneResult.from_json(key, obj)

    def save(self, path=None) -> None:
        path = Path(path) if path else self.cache_path
        if path is None:
            return
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(path.suffix + ".tmp")
        tmp.write_text(json.dumps({k: r.to_json() for k, r in sorted(self.results.items())}, indent=1))
        os.replace(tmp, path)

    def _remember(self, res: TuneResult) -> TuneResult:
        self.results[res.key] = res
        self.save()
        return res

    # -- programs ------------------------------------------------------
    def _program_measure(self, dp, shots: int, seed: int) -> Measure:
        ctx = self.ctx
        out = np.empty((shots, max(dp.num_records, 1)), dtype=np.uint8)

        def measure(flags: int):
            rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, 0, shots, out.ctypes.data if dp.num_records else None,
                                  flags | _lib.FLAG_TIME)
            _lib.check(rc, ctx.ptr, "autotune")
            return out[:, :dp.num_records], ctx.last_kernel_ms()
        return measure

    def tune_program(self, dp, shots: int, seed: int = 0, noise: bool = True) -> TuneResult:
        """Times every route for this device program at ``shots`` shots
        (at most TUNE_MAX_SHOTS) and caches the choice for its class."""
        shots = int(min(max(int(shots), 1), TUNE_MAX_SHOTS))
        enc = dp.enc
        key = self.program_key(enc.d, enc.n, shots, noise)
        cands = program_candidates(enc.d, enc.n, shots, self.ctx.smem_optin, self.ctx.num_sms)
        with self._lock:
            res = tune(key, cands, self._program_measure(dp, shots, int(seed) & 0xFFFFFFFFFFFFFFFF), self.reps,
                       self.abort_factor)
            return self._remember(res)

    def flags_for_program(self, dp, shots: int, noise: bool = True) -> int:
        """Run flags of the tuned route for this program's class (tuned now on a miss)."""
        enc = dp.enc
        key = self.program_key(enc.d, enc.n, min(max(int(shots), 1), TUNE_MAX_SHOTS), noise)
        res = self.results.get(key)
        if res is None:
            res = self.tune_program(dp, shots, noise=noise)
        return res.best.flags

    # -- batches -------------------------------------------------------
    def _batch_items(self, runner) -> List[Tuple[int, int, int, int]]:
        return [(e.program.enc.d, e.program.enc.n, e.program.num_instructions, e.shots) for e in runner.entries]

    def tune_batch(self, runner) -> TuneResult:
        """Times every batch-wide route for the entries of a BatchRunner."""
        key = self.batch_key(self._batch_items(runner))
        outs = [np.empty((e.shots, e.program.num_records), dtype=np.uint8) for e in runner.entries]

        def measure(flags: int):
            runner.run(time_kernels=True, outs=outs, flags=flags)
            flat = np.concatenate([o.reshape(-1) for o in outs]) if outs else np.empty(0, np.uint8)
            return flat, self.ctx.last_kernel_ms()
        with self._lock:
            res = tune(key, batch_candidates(), measure, self.reps, self.abort_factor)
            return self._remember(res)

    def flags_for_batch(self, runner) -> int:
        res = self.results.get(self.batch_key(self._batch_items(runner)))
        if res is None:
            res = self.tune_batch(runner)
        return res.best.flags


_default: Dict[int, Autotuner] = {}
_default_lock = threading.Lock()


def default_tuner(ctx: Optional[_lib.Context] = None) -> Autotuner:
    """The process-wide tuner of a context's device."""
    ctx = ctx or _lib.Context.default(0)
    with _default_lock:
        t = _default.get(ctx.device)
        if t is None:
            t = _default[ctx.device] = Autotuner(ctx)
        return t
