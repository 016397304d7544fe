"""GPU: record columns of the d = 2 trace engine (trace_cols.cuh) -- each
shot's records as the constant column XOR the columns of its outcome draws and
N1 fires -- against the phase replay and the oracle: every record-word count
(column words 2 to 32), programs with and without N1 before the last
measurement, N1 after it, RESET, every noise channel at p = 0 and p = 1,
partial shot groups, and a kept trace and column table."""
import ctypes

import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.workloads import CircuitSpec
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu

COLS = _lib.FLAG_TRACE | _lib.FLAG_COLUMNS
REPLAY = _lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY


def kept(prog):
    """(trace valid, columns valid) of the program's kept device state."""
    out = (ctypes.c_int32 * 2)()
    _lib.check(prog.context.lib.sdim_circuit_kept(prog.compile().ptr, out), prog.context.ptr, "kept")
    return tuple(out)


def run(prog, shots, seed, shot0, flags):
    dp = prog.compile()
    ctx = prog.context
    out = np.zeros((shots, max(dp.num_records, 1)), dtype=np.uint8)
    _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, shot0, shots, out.ctypes.data, flags | _lib.FLAG_TIME),
               ctx.ptr, "run")
    return out[:, :dp.num_records], ctx.last_passes_ms()


@pytest.mark.parametrize("distance,rounds,prob,shots,shot0", [(3, 3, 0.05, 200, 5), (5, 2, 0.02, 1000, 0),
                                                              (7, 2, 0.01, 65, 31)])
def test_surface_codes_columns_match_replay_and_oracle(distance, rounds, prob, shots, shot0):
    spec = workloads.surface_memory(distance, rounds, prob=prob)
    prog = Program(spec.build())
    rec, passes = run(prog, shots, 4, shot0, COLS)
    assert passes[2] > 0.0, "the column pass did not run"
    assert np.array_equal(rec, run(prog, shots, 4, shot0, REPLAY)[0])
    assert np.array_equal(rec, oracle_run([spec], 4, shot0, shots)["records"])


@pytest.mark.parametrize("n,mr_every,words", [(1, 1, 2), (5, 4, 2), (16, 8, 4), (20, 6, 8), (64, 20, 16),
                                              (97, 40, 32), (128, 40, 32), (300, 300, 32), (512, 800, 32),
                                              (400, 400, 0)])
def test_record_word_counts_against_replay(n, mr_every, words):
    """Measurement counts across 2 .. 32 column words (random gates with
    measure-and-reset blocks, then MEASURE all); past 1,024 measurements
    (words 0) the run keeps the replay."""
    spec = workloads.random_hpc(n, 2, 6 * n + 20, seed=1100 + n, mr_every=mr_every, mr_fraction=0.3)
    prog = Program(spec.build())
    rec, passes = run(prog, 97, n, 3, COLS)
    assert (passes[2] > 0.0) == (words > 0), n
    assert np.array_equal(rec, run(prog, 97, n, 3, REPLAY)[0]), n
    if n <= 128:
        assert np.array_equal(rec, oracle_run([spec], n, 3, 97)["records"]), n


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_all_gates_and_noise_channels(seed):
    spec = workloads.all_gates_random(9, 2, 400, seed=seed, noise_probs=(0.0, 0.35, 1.0))
    prog = Program(spec.build())
    rec, _ = run(prog, 130, seed, 11, COLS)
    assert np.array_equal(rec, run(prog, 130, seed, 11, REPLAY)[0])
    assert np.array_equal(rec, oracle_run([spec], seed, 11, 130)["records"])


def test_n1_after_the_last_measurement_and_none_before():
    """Fires after the last measurement change no record; a program whose N1
    all come after it has no fire columns at all."""
    ops = [("H", 0, None, {}), ("CNOT", 0, 1, {}), ("H", 2, None, {})]
    ops += [("M", q, None, {}) for q in range(3)]
    ops += [("N1", q, None, {"prob": 1.0, "noise_channel": "d"}) for q in range(3)]
    spec = CircuitSpec(3, 2, ops)
    prog = Program(spec.build())
    rec, _ = run(prog, 300, 7, 0, COLS)
    assert np.array_equal(rec, run(prog, 300, 7, 0, REPLAY)[0])
    assert np.array_equal(rec, oracle_run([spec], 7, 0, 300)["records"])
    ops2 = [("N1", 0, None, {"prob": 0.5, "noise_channel": "f"})] + ops
    spec2 = CircuitSpec(3, 2, ops2)
    prog2 = Program(spec2.build())
    rec2, _ = run(prog2, 300, 7, 0, COLS)
    assert np.array_equal(rec2, oracle_run([spec2], 7, 0, 300)["records"])


def test_default_route_takes_columns_for_many_shots():
    spec = workloads.surface_memory(5, 3, prob=0.01)
    prog = Program(spec.build())
    shots = 20000
    rec, passes = run(prog, shots, 2, 0, 0)
    assert passes[2] > 0.0, "the default route did not take the record columns"
    assert np.array_equal(rec, run(prog, shots, 2, 0, REPLAY)[0])
    assert np.array_equal(rec[:300], oracle_run([spec], 2, 0, 300)["records"])


def test_kept_trace_and_columns():
    spec = workloads.surface_memory(5, 3, prob=0.02)
    prog = Program(spec.build())
    cold, _ = run(prog, 700, 3, 0, REPLAY)
    keep = COLS | _lib.FLAG_REUSE_XZ
    assert kept(prog) == (0, 0)
    first, p1 = run(prog, 700, 3, 0, keep)
    assert kept(prog) == (1, 1)
    again, p2 = run(prog, 700, 3, 0, keep)
    assert p1[2] > 0.0 and p2[2] == 0.0, "the kept column table was not reused"
    assert np.array_equal(first, cold) and np.array_equal(again, cold)
    other, _ = run(prog, 321, 9, 40, keep)
    assert np.array_equal(other, run(prog, 321, 9, 40, REPLAY)[0])
    # a kept trace written by a replay run gets its columns on the next column run
    prog2 = Program(spec.build())
    run(prog2, 100, 1, 0, REPLAY | _lib.FLAG_REUSE_XZ)
    assert kept(prog2) == (1, 0)
    rec, p = run(prog2, 700, 3, 0, keep)
    assert p[2] > 0.0 and np.array_equal(rec, cold) and kept(prog2) == (1, 1)
    # an asynchronous call never makes a kept trace valid; the next
    # synchronous one does
    torch = pytest.importorskip("torch")
    prog3 = Program(spec.build())
    dp3, ctx = prog3.compile(), prog3.context
    dev = torch.zeros((700, dp3.num_records), dtype=torch.uint8, device="cuda")
    _lib.check(ctx.lib.sdim_run_device(ctx.ptr, dp3.ptr, 3, 0, 700, dev.data_ptr(), None, keep | _lib.FLAG_ASYNC),
               ctx.ptr, "run")
    ctx.sync()
    assert kept(prog3) == (0, 0)
    assert np.array_equal(dev.cpu().numpy(), cold)
    _lib.check(ctx.lib.sdim_run_device(ctx.ptr, dp3.ptr, 3, 0, 700, dev.data_ptr(), None, keep), ctx.ptr, "run")
    assert kept(prog3) == (1, 1)


@pytest.mark.parametrize("shots", [1024, 4113, 20000])
def test_records_copied_down_in_chunks(shots):
    """sdim_run into page-locked host memory: the record pass runs in chunks
    and each chunk is copied down while the next one is written (partial last
    chunk and group included); the records equal the device-side run's."""
    torch = pytest.importorskip("torch")
    spec = workloads.surface_memory(5, 3, prob=0.02)
    prog = Program(spec.build())
    dp, ctx = prog.compile(), prog.context
    host = torch.zeros((shots, dp.num_records), dtype=torch.uint8, pin_memory=True)
    _lib.check(ctx.lib.sdim_run(ctx.ptr, dp.ptr, 6, 3, shots, host.data_ptr(), COLS), ctx.ptr, "run")
    dev = torch.zeros((shots, dp.num_records), dtype=torch.uint8, device="cuda")
    _lib.check(ctx.lib.sdim_run_device(ctx.ptr, dp.ptr, 6, 3, shots, dev.data_ptr(), None, COLS), ctx.ptr, "run")
    assert np.array_equal(host.numpy(), dev.cpu().numpy())
    assert np.array_equal(host.numpy(), run(prog, shots, 6, 3, REPLAY)[0])
