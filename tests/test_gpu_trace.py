"""GPU: the d = 2 trace engine (one x / z pass per program, one lane per shot
replaying its phase deltas) against the oracle and the other engines, for
every trace-row width, both x / z pass teams, partial shot groups, every
noise channel (including p = 0 and p = 1), mixed batches and global-memory
x / z slots."""
import ctypes

import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("distance,rounds,prob,shots,shot0", [(3, 3, 0.05, 200, 5), (5, 2, 0.02, 100, 0),
                                                              (7, 2, 0.01, 65, 31)])
def test_surface_codes_match_oracle(distance, rounds, prob, shots, shot0):
    spec = workloads.surface_memory(distance, rounds, prob=prob)
    prog = Program(spec.build())
    rec = prog.sample(shots, seed=4, shot0=shot0, engine="trace")
    assert np.array_equal(rec, oracle_run([spec], 4, shot0, shots)["records"])
    assert np.array_equal(rec, prog.sample(shots, seed=4, shot0=shot0, engine="group"))


@pytest.mark.parametrize("n", [1, 2, 5, 31, 32, 33, 64, 65, 97, 128, 129, 159])
def test_every_row_width_small_n_against_oracle(n):
    spec = workloads.random_hpc(n, 2, 6 * n + 20, seed=700 + n, mr_every=max(1, n // 2), mr_fraction=0.3)
    prog = Program(spec.build())
    rec = prog.sample(70, seed=n, engine="trace")
    assert np.array_equal(rec, oracle_run([spec], n, 0, 70)["records"]), n


@pytest.mark.parametrize("n", [160, 200, 256, 257, 400, 512])
def test_cta_pass_and_wide_rows_against_group_engine(n):
    spec = workloads.random_hpc(n, 2, 4 * n, seed=900 + n, mr_every=n, mr_fraction=0.2)
    prog = Program(spec.build())
    rec = prog.sample(96, seed=n, engine="trace")
    assert np.array_equal(rec, prog.sample(96, seed=n, engine="group")), n
    if n <= 200:
        assert np.array_equal(rec, oracle_run([spec], n, 0, 96)["records"]), n


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_all_gates_and_noise_channels(seed):
    spec = workloads.all_gates_random(7, 2, 300, seed=seed, noise_probs=(0.0, 0.35, 1.0))
    prog = Program(spec.build())
    rec = prog.sample(130, seed=seed, shot0=11, engine="trace")
    assert np.array_equal(rec, oracle_run([spec], seed, 11, 130)["records"])


def test_records_do_not_depend_on_the_split():
    spec = workloads.surface_memory(5, 3, prob=0.03)
    prog = Program(spec.build())
    whole = prog.sample(150, seed=8, engine="trace")
    parts = np.concatenate([prog.sample(37, seed=8, engine="trace"),
                            prog.sample(113, seed=8, shot0=37, engine="trace")])
    assert np.array_equal(whole, parts)
    assert np.array_equal(whole[:20], prog.sample(20, seed=8))        # group engine below 128 shots
    assert np.array_equal(whole[:3], prog.sample(3, seed=8, per_shot=True))


def test_mixed_batch_routes_each_program():
    """d = 2 programs with many shots run on the trace engine, the others on
    their group engines, all in one call; every result equals the oracle."""
    rng = np.random.default_rng(3)
    specs = [workloads.surface_memory(3, 2, prob=0.04), workloads.random_hpc(40, 2, 200, seed=5, mr_every=20),
             workloads.random_hpc(12, 3, 120, seed=6, mr_every=6), workloads.random_hpc(300, 2, 900, seed=7,
                                                                                        mr_every=300),
             workloads.random_hpc(70, 2, 300, seed=8, mr_every=35)]
    shots = [300, 10, 80, 128, 129]
    runner = BatchRunner()
    for i, (s, k) in enumerate(zip(specs, shots)):
        runner.add_spec(s, k, seed=int(rng.integers(1 << 30)), shot0=i)
    outs = runner.run()
    for e, s, out in zip(runner.entries, specs, outs):
        if s.num_qudits <= 70:
            assert np.array_equal(out, oracle_run([s], e.seed, e.shot0, e.shots)["records"]), s.name
    alone = Program(specs[3].build()).sample(128, seed=runner.entries[3].seed, shot0=3, engine="group")
    assert np.array_equal(outs[3], alone)


@pytest.mark.parametrize("prob", [1e-3, 0.05, 0.5])
def test_coins_in_the_phase_pass_match_the_coin_pass(prob):
    """SDIM_FLAG_NO_COIN_PASS draws the N1 coins inside the phase pass; both
    paths give the oracle's records."""
    spec = workloads.surface_memory(5, 3, prob=prob)
    prog = Program(spec.build())
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((130, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 12, 7, 130, out.ctypes.data, _lib.FLAG_TRACE | _lib.FLAG_NO_COIN_PASS)
    _lib.check(rc, ctx.ptr, "trace without coin pass")
    assert np.array_equal(out, prog.sample(130, seed=12, shot0=7, engine="trace"))
    assert np.array_equal(out, oracle_run([spec], 12, 7, 130)["records"])


def test_two_shots_per_lane_partial_groups_with_and_without_masks():
    """From 77,824 shots per launch the phase pass carries two shots per lane.
    An odd shot count leaves a partial last 64-shot group. Run without the
    coin pass, each group replays its two 32-shot halves in turn. Both forms
    give the group engine's records, and the ends of the range give the
    oracle's."""
    spec = workloads.surface_memory(3, 2, prob=0.05)
    prog = Program(spec.build())
    dp = prog.compile(True)
    ctx = prog.context
    nshots = 80_017
    ref = prog.sample(nshots, seed=3, shot0=5, engine="group")
    for flags in (_lib.FLAG_TRACE, _lib.FLAG_TRACE | _lib.FLAG_NO_COIN_PASS):
        out = np.empty((nshots, dp.num_records), dtype=np.uint8)
        _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, 3, 5, nshots, out.ctypes.data, flags), ctx.ptr, "trace")
        assert np.array_equal(out, ref), flags
    assert np.array_equal(ref[-40:], oracle_run([spec], 3, 5 + nshots - 40, 40)["records"])


def test_xz_pass_in_global_memory():
    spec = workloads.random_hpc(300, 2, 1200, seed=31, mr_every=150, mr_fraction=0.2)
    prog = Program(spec.build())
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((72, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 6, 0, 72, out.ctypes.data, _lib.FLAG_TRACE | _lib.FLAG_FORCE_GMEM)
    _lib.check(rc, ctx.ptr, "trace, x / z in global memory")
    assert np.array_equal(out, prog.sample(72, seed=6, engine="group"))


def test_full_size_noisy_surface_against_group_engine_and_oracle():
    """The bench workload at full size (distance 7, 7 rounds, p = 1e-3,
    100k shots): trace and group engines agree on every record, and the
    first and last 64 shots equal the oracle."""
    spec = workloads.surface_memory(7, 7, prob=1e-3)
    prog = Program(spec.build())
    rec = prog.sample(100_000, seed=2, engine="trace")
    assert np.array_equal(rec, prog.sample(100_000, seed=2, engine="group"))
    assert np.array_equal(rec[:64], oracle_run([spec], 2, 0, 64)["records"])
    assert np.array_equal(rec[-64:], oracle_run([spec], 2, 100_000 - 64, 64)["records"])


# ---------------------------------------------------------------- odd d


def test_pr1_fixture_on_the_odd_d_trace_engine(golden):
    """PR1 (d = 3, n = 32, 1,024 shots): every record equals the reference's."""
    from tests.conftest import program_of
    cases, arrays = golden
    name = next(k for k in cases if k.startswith("pr1"))
    prog = program_of(cases[name])
    rec = prog.sample(cases[name]["nshots"], seed=cases[name]["seed"], engine="trace")
    assert np.array_equal(rec, arrays[f"{name}__records"])


@pytest.mark.parametrize("d", [3, 5, 7, 11])
@pytest.mark.parametrize("n", [1, 5, 33, 100])
def test_odd_d_small_n_against_oracle(d, n):
    spec = workloads.random_hpc(n, d, 5 * n + 20, seed=31 * d + n, mr_every=max(1, n // 2), mr_fraction=0.3)
    prog = Program(spec.build())
    rec = prog.sample(70, seed=d + n, shot0=3, engine="trace")
    assert np.array_equal(rec, oracle_run([spec], d + n, 3, 70)["records"]), (d, n)


@pytest.mark.parametrize("d", [3, 5, 7, 13])
@pytest.mark.parametrize("n", [170, 256, 700])
def test_odd_d_large_n_against_group_engine(d, n):
    # n >= 230 puts the x / z pass's tableau in global memory
    spec = workloads.random_hpc(n, d, 3 * n, seed=17 * d + n, mr_every=n, mr_fraction=0.1)
    prog = Program(spec.build())
    rec = prog.sample(66, seed=n, engine="trace")
    assert np.array_equal(rec, prog.sample(66, seed=n, engine="group")), (d, n)


@pytest.mark.parametrize("d", [3, 5])
def test_odd_d_all_gates_and_noise_channels(d):
    spec = workloads.all_gates_random(6, d, 250, seed=7 * d, noise_probs=(0.0, 0.35, 1.0))
    prog = Program(spec.build())
    rec = prog.sample(100, seed=d, shot0=5, engine="trace")
    assert np.array_equal(rec, oracle_run([spec], d, 5, 100)["records"])


def test_mixed_dimensions_in_one_batch():
    specs = [workloads.random_hpc(30, 3, 150, seed=1, mr_every=15), workloads.random_hpc(40, 2, 200, seed=2,
                                                                                          mr_every=20),
             workloads.random_hpc(64, 5, 300, seed=3, mr_every=32), workloads.random_hpc(20, 7, 90, seed=4,
                                                                                        mr_every=10),
             workloads.random_hpc(12, 3, 60, seed=5, mr_every=6)]
    shots = [200, 130, 150, 128, 10]
    runner = BatchRunner()
    for i, (s, k) in enumerate(zip(specs, shots)):
        runner.add_spec(s, k, seed=100 + i, shot0=2 * i)
    outs = runner.run()
    for e, s, out in zip(runner.entries, specs, outs):
        assert np.array_equal(out, oracle_run([s], e.seed, e.shot0, e.shots)["records"]), s.name


@pytest.mark.parametrize("d", [3, 5, 7, 11])
@pytest.mark.parametrize("n", [1, 6, 33, 100])
def test_odd_d_cta_pair_against_oracle(d, n):
    """SDIM_FLAG_SPLIT_XZ runs the odd-d x / z pass on a CTA pair (stabilizer
    and destabilizer columns in the two blocks' shared memory) even where one
    CTA would do; records equal the oracle's, noise included."""
    spec = (workloads.all_gates_random(n, d, 200, seed=3 * d + n, noise_probs=(0.0, 0.3, 1.0)) if n <= 6 else
            workloads.random_hpc(n, d, 5 * n + 20, seed=13 * d + n, mr_every=max(1, n // 2), mr_fraction=0.3))
    prog = Program(spec.build())
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((70, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, d, 2, 70, out.ctypes.data, _lib.FLAG_TRACE | _lib.FLAG_SPLIT_XZ)
    _lib.check(rc, ctx.ptr, "odd-d trace on a CTA pair")
    assert np.array_equal(out, oracle_run([spec], d, 2, 70)["records"]), (d, n)


@pytest.mark.parametrize("n", [513, 700, 1024, 1025, 1500, 2048])
def test_wide_rows_past_512_qudits(n):
    """Trace rows of 64 and 128 words (n up to 2048, x / z tableau in global
    memory, one shot per phase-pass lane) with MEASURE+RESET rounds and
    depolarizing noise: all 70 shots against the shot-group engine, and up
    to n = 1025 the first two against the oracle (about 20 core-seconds a
    shot at n = 1024)."""
    base = workloads.random_hpc(n, 2, 3 * n, seed=950 + n, mr_every=n, mr_fraction=0.1)
    ops = []
    for op in base.ops:
        ops.append(op)
        if op[0] in ("H", "CNOT"):
            ops.append(("N1", op[1], None, {"noise_channel": "d", "prob": 0.01}))
    spec = workloads.CircuitSpec(n, 2, ops, f"wide_n{n}")
    prog = Program(spec.build())
    rec = prog.sample(70, seed=n, engine="trace")
    assert np.array_equal(rec, prog.sample(70, seed=n, engine="group")), n
    if n <= 1025:
        assert np.array_equal(rec[:2], oracle_run([spec], n, 0, 2)["records"]), n


def test_kept_xz_trace_replays_for_fresh_seeds_and_shot_ranges():
    """keep_xz: the first call writes the program's x / z trace, later calls
    replay it without the x / z pass; every call matches a cold run, and a
    second program (and an edited one) keeps a trace of its own."""
    spec = workloads.surface_memory(5, 3, prob=0.02)
    prog = Program(spec.build())
    other = Program(workloads.surface_memory(3, 4, prob=0.05).build())
    for seed, shot0, shots in [(1, 0, 300), (2, 300, 129), (3, 7, 1000), (1, 0, 300)]:
        warm = prog.sample(shots, seed=seed, shot0=shot0, engine="trace", keep_xz=True)
        assert np.array_equal(warm, prog.sample(shots, seed=seed, shot0=shot0, engine="trace")), (seed, shot0)
        w2 = other.sample(shots, seed=seed, shot0=shot0, engine="trace", keep_xz=True)
        assert np.array_equal(w2, other.sample(shots, seed=seed, shot0=shot0, engine="trace")), (seed, shot0)
    assert np.array_equal(prog.sample(200, seed=9, shot0=3, engine="trace", keep_xz=True),
                          oracle_run([spec], 9, 3, 200)["records"])
    # an edited program is a new encoded program: its trace is written afresh
    prog.circuits[-1].add_gate("H", 0)
    prog.circuits[-1].add_gate("MEASURE", 0)
    cold = prog.sample(200, seed=5, engine="trace")
    assert np.array_equal(prog.sample(200, seed=5, engine="trace", keep_xz=True), cold)
    assert np.array_equal(prog.sample(200, seed=5, engine="trace", keep_xz=True), cold)


def test_kept_xz_trace_with_coins_in_the_phase_pass():
    spec = workloads.surface_memory(5, 2, prob=0.03)
    prog = Program(spec.build())
    dp = prog.compile()
    ctx = prog.context
    cold = prog.sample(500, seed=4, engine="trace")
    out = np.empty_like(cold)
    for flags in (_lib.FLAG_TRACE | _lib.FLAG_REUSE_XZ,
                  _lib.FLAG_TRACE | _lib.FLAG_REUSE_XZ | _lib.FLAG_NO_COIN_PASS):
        out[:] = 0
        _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, 4, 0, 500, out.ctypes.data, flags), ctx.ptr, "run")
        assert np.array_equal(out, cold)
        state = (ctypes.c_int32 * 2)()
        _lib.check(ctx.lib.sdim_circuit_kept(dp.ptr, state), ctx.ptr, "kept")
        assert state[0] == 1, "the x / z trace was not kept"


def test_snapshot_slots_run_out_on_a_wide_program():
    """n = 2048: a deterministic snapshot is 1 MB, so the 64 MB budget holds
    64; 80 runs of deterministic measurements (each measured qudit measured
    again right after its random outcome) use them up and the x / z pass
    sums the rest's cross terms itself.  Records equal the shot-group
    engine's."""
    n = 2048
    ops = [("H", q, None, {}) for q in range(0, 160)]
    ops += [("CNOT", q, q + 1, {}) for q in range(0, 159, 2)]
    ops += [("P", q, None, {}) for q in range(1, 160, 3)]
    for q in range(80):
        ops += [("M", 2 * q, None, {}), ("M", 2 * q, None, {})]
    spec = workloads.CircuitSpec(n, 2, ops)
    prog = Program(spec.build())
    rec = prog.sample(64, seed=3, engine="trace")
    det = rec[0] >> 7
    assert det[1::2].all() and not det[0::2].any(), "the pairs should alternate random / deterministic"
    assert np.array_equal(rec, prog.sample(64, seed=3, engine="group"))
