"""CPU: the autotuner's candidate routes, its choice and its cache, with a
fake device (the GPU test of the same code is tests/test_gpu_autotune.py)."""
import numpy as np
import pytest

from sdim_gb300 import _lib, autotune

OPTIN, SMS = 232448, 152


def _names(cands):
    return [c.name for c in cands]


def test_candidates_d2_within_the_trace_limit():
    c = autotune.program_candidates(2, 97, 100_000, OPTIN, SMS)
    flags = {x.name: x.flags for x in c}
    assert flags["default"] == 0
    assert flags["trace"] == _lib.FLAG_TRACE
    assert flags["trace, coins in the phase pass"] == _lib.FLAG_TRACE | _lib.FLAG_NO_COIN_PASS
    assert flags["trace, record columns"] == _lib.FLAG_TRACE | _lib.FLAG_COLUMNS
    assert flags["trace, phase replay"] == _lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY
    assert flags["trace, phase replay, one shot per lane"] == (_lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY
                                                                | _lib.FLAG_LANE_SHOTS_1)
    assert flags["shot groups, one per CTA"] == _lib.FLAG_TEAM_CTA
    assert "one warp per shot" not in flags
    assert len(set(flags.values())) == len(flags)


def test_record_columns_only_within_their_row_limit():
    assert "trace, record columns" in _names(autotune.program_candidates(2, 512, 4096, OPTIN, SMS))
    c = _names(autotune.program_candidates(2, 513, 4096, OPTIN, SMS))
    assert "trace, record columns" not in c and "trace, phase replay" in c


def test_candidates_past_the_d2_trace_limit_and_large_n_teams():
    c = _names(autotune.program_candidates(2, 2100, 20, OPTIN, SMS))
    assert not any(name.startswith("trace") for name in c)
    assert "shot groups, one per warp" in c and "one warp per shot" in c


def test_odd_d_xz_forms_are_deduplicated_by_the_library_query():
    # d = 11, n = 256 does not fit one CTA in bytes: a lone program's default
    # x / z pass is the 8-CTA cluster in shared memory; the pair, the streamed
    # single CTA and the streamed cluster are the other forms, each timed once
    c = _names(autotune.program_candidates(11, 256, 4096, OPTIN, SMS))
    forms = [x for x in c if x.startswith("trace, x/z")]
    assert forms == ["trace, x/z pass on CTA pair", "trace, x/z pass on one CTA, global memory",
                     "trace, x/z pass on 8-CTA cluster, global memory"]
    # n = 100 fits one CTA: every override is a different form
    small = [x for x in _names(autotune.program_candidates(11, 100, 4096, OPTIN, SMS)) if x.startswith("trace, x/z")]
    assert len(small) == 4
    # a lone d = 5, n = 256 program runs on the byte cluster; the 4-bit-lane
    # forms are timed beside the byte ones
    d5 = [x for x in _names(autotune.program_candidates(5, 256, 4096, OPTIN, SMS)) if x.startswith("trace, x/z")]
    assert d5 == ["trace, x/z pass on CTA pair", "trace, x/z pass on one CTA, global memory",
                  "trace, x/z pass on 8-CTA cluster, global memory", "trace, x/z pass on one CTA, 4-bit lanes",
                  "trace, x/z pass on one CTA, 4-bit lanes in global memory"]
    # a lone d = 3 program runs on bytes by default; the bit-plane forms are
    # two of the six others
    d3 = [x for x in _names(autotune.program_candidates(3, 100, 4096, OPTIN, SMS)) if x.startswith("trace, x/z")]
    assert len(d3) == 6 and "trace, x/z pass on one CTA, bit planes" in d3
    assert "trace, x/z pass on one CTA, bit planes in global memory" in d3
    # past the odd-d trace engine's limit only the group engines remain
    big = _names(autotune.program_candidates(5, 2049, 64, OPTIN, SMS))
    assert not any(x.startswith("trace") for x in big)


def _fake(times, records=None):
    """measure(flags) -> (records, ms) from a table of per-flag time lists."""
    calls = []
    rec = np.arange(12, dtype=np.uint8).reshape(3, 4) if records is None else records

    def measure(flags):
        calls.append(flags)
        seq = times[flags]
        ms = seq[min(len([c for c in calls if c == flags]) - 1, len(seq) - 1)]
        r = rec(flags) if callable(rec) else rec
        return r, ms
    return measure, calls


def test_tune_picks_the_fastest_median_and_aborts_slow_routes():
    cands = [autotune.Candidate("a", 0), autotune.Candidate("b", 1), autotune.Candidate("c", 2)]
    # first entry of each list is the untimed warm-up run
    times = {0: [9.0, 5.0, 5.2, 4.9], 1: [9.0, 3.0, 3.1, 2.9], 2: [9.0, 40.0, 1.0, 1.0]}
    measure, calls = _fake(times)
    res = autotune.tune("k", cands, measure, reps=3, abort_factor=4.0)
    assert res.best.name == "b"
    assert res.times_ms["a"] == pytest.approx(5.0)
    assert res.times_ms["b"] == pytest.approx(3.0)
    # c's first timed run is 40 ms > 4 x 3 ms: one timed run only
    assert res.aborted == ["c"] and res.times_ms["c"] == pytest.approx(40.0)
    assert calls.count(2) == 2


def test_tune_rejects_a_route_with_different_records():
    cands = [autotune.Candidate("a", 0), autotune.Candidate("b", 1)]
    base = np.zeros((2, 3), dtype=np.uint8)
    bad = base.copy()
    bad[1, 2] = 1
    measure, _ = _fake({0: [1.0], 1: [0.5]}, records=lambda f: bad if f == 1 else base)
    with pytest.raises(RuntimeError, match="differ"):
        autotune.tune("k", cands, measure)


class _Ctx:
    num_sms, smem_optin, device = SMS, OPTIN, 0


class _Enc:
    def __init__(self, n, d):
        self.n, self.d = n, d


class _Prog:
    def __init__(self, n, d):
        self.enc = _Enc(n, d)


def test_cache_keys_round_trip_and_reuse(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    t = autotune.Autotuner(ctx=_Ctx(), cache_path=str(path), reps=2)
    timed = []

    def fake_measure(dp, shots, seed):
        timed.append((dp.enc.n, shots))
        fast = _lib.FLAG_TRACE
        return lambda flags: (np.zeros((shots, 2), np.uint8), 1.0 if flags == fast else 2.0)
    monkeypatch.setattr(t, "_program_measure", fake_measure)
    assert t.flags_for_program(_Prog(97, 2), 100_000) == _lib.FLAG_TRACE
    n_timed = len(timed)
    # same class (n and shots within half an octave): cached, nothing timed
    assert t.flags_for_program(_Prog(100, 2), 110_000) == _lib.FLAG_TRACE
    assert len(timed) == n_timed
    # shots are tuned at most at TUNE_MAX_SHOTS
    t.flags_for_program(_Prog(40, 3), 10 ** 7)
    assert timed[-1] == (40, autotune.TUNE_MAX_SHOTS)
    # the file holds both classes and a new tuner reads them back
    t2 = autotune.Autotuner(ctx=_Ctx(), cache_path=str(path))
    assert set(t2.results) == set(t.results)
    key = t.program_key(2, 97, 100_000)
    assert key.startswith("sm152-smem232448/program/d2/")
    assert t2.results[key].best.flags == _lib.FLAG_TRACE
    assert t.program_key(2, 97, 100_000) != t.program_key(2, 97, 100_000, noise=False)


def test_batch_key_depends_on_composition_only():
    t = autotune.Autotuner(ctx=_Ctx())
    a = [(2, 97, 4921, 64), (3, 40, 160, 1)]
    assert t.batch_key(a) == t.batch_key(list(reversed(a)))
    assert t.batch_key(a) != t.batch_key(a[:1])
    assert [c.flags for c in autotune.batch_candidates()][0] == 0


class _BatchProgram:
    def __init__(self, n, d, records):
        self.enc = _Enc(n, d)
        self.num_instructions = 4 * n
        self.num_records = records


class _Entry:
    def __init__(self, prog, shots):
        self.program, self.shots = prog, shots


class _FakeRunner:
    """Writes records that depend only on the entry, as every route does,
    and reports a kernel time per route."""

    def __init__(self, ctx, times, wrong_flags=None):
        self.ctx, self.times, self.wrong_flags = ctx, times, wrong_flags
        self.entries = [_Entry(_BatchProgram(8, 3, 2), 5), _Entry(_BatchProgram(200, 2, 3), 70)]
        self.calls = []

    def run(self, time_kernels=False, outs=None, flags=0):
        self.calls.append(flags)
        for i, o in enumerate(outs):
            o[:] = i + 1 + (1 if flags == self.wrong_flags else 0)
        self.ctx.last_ms = self.times.get(flags, 10.0)
        return outs


class _TimedCtx(_Ctx):
    last_ms = 0.0

    def last_kernel_ms(self):
        return self.last_ms


def test_tune_batch_picks_the_fastest_route_and_caches_it():
    ctx = _TimedCtx()
    runner = _FakeRunner(ctx, {0: 5.0, _lib.FLAG_SPLIT_XZ: 3.0, _lib.FLAG_TRACE: 50.0})
    t = autotune.Autotuner(ctx=ctx, reps=2)
    assert t.flags_for_batch(runner) == _lib.FLAG_SPLIT_XZ
    res = t.results[t.batch_key(t._batch_items(runner))]
    assert "trace engines at any shot count" in res.aborted
    n_calls = len(runner.calls)
    assert t.flags_for_batch(runner) == _lib.FLAG_SPLIT_XZ and len(runner.calls) == n_calls


def test_tune_batch_rejects_a_route_that_changes_records():
    ctx = _TimedCtx()
    runner = _FakeRunner(ctx, {}, wrong_flags=_lib.FLAG_NO_TRACE)
    with pytest.raises(RuntimeError, match="shot groups only"):
        autotune.Autotuner(ctx=ctx, reps=1).tune_batch(runner)
