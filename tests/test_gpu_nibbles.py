"""GPU: the d = 5 and d = 7 x / z pass on 4-bit residue lanes
(trace_n4.cuh) against the oracle and against the byte-residue passes
(SDIM_FLAG_U8_XZ), bit for bit: every gate and noise channel on tiny
programs, qudit counts at the 8-lane word boundaries, deterministic sweeps,
MEASURE+RESET rounds, the tableau in shared memory (to n = 320) and
streamed from global memory (SDIM_FLAG_FORCE_GMEM, and n = 321 up in
batches), and uneven batches whose programs take both forms."""
import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu

LANES = _lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ
LANES_GMEM = _lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ | _lib.FLAG_FORCE_GMEM
BYTES = _lib.FLAG_TRACE | _lib.FLAG_U8_XZ


def _run(prog, seed, shot0, shots, flags):
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, shot0, shots, out.ctypes.data, flags)
    _lib.check(rc, ctx.ptr, "d = 5 / 7 trace pass")
    return out


def _twice_measured(n, d, seed):
    base = workloads.random_hpc(n, d, 4 * n + 10, seed=seed)
    rng = np.random.default_rng(seed)
    ops = list(base.ops)
    ops += [("X" if rng.random() < 0.5 else "Z", int(q), None, {}) for q in rng.integers(n, size=n)]
    ops += [("M", q, None, {}) for q in range(n)]
    return workloads.CircuitSpec(n, d, ops, f"twice_n{n}_d{d}")


@pytest.mark.parametrize("flags", [LANES, LANES_GMEM], ids=["smem", "gmem"])
@pytest.mark.parametrize("d", [5, 7])
@pytest.mark.parametrize("n", [1, 2, 5, 9])
def test_every_gate_and_channel_against_oracle(n, d, flags):
    spec = workloads.all_gates_random(n, d, 300, seed=60 + n + d, noise_probs=(0.0, 0.3, 1.0))
    prog = Program(spec.build())
    rec = _run(prog, 7, 2, 130, flags)
    assert np.array_equal(rec, oracle_run([spec], 7, 2, 130)["records"]), (n, d)
    assert np.array_equal(rec, _run(prog, 7, 2, 130, BYTES)), (n, d)


@pytest.mark.parametrize("flags", [LANES, LANES_GMEM], ids=["smem", "gmem"])
@pytest.mark.parametrize("d", [5, 7])
@pytest.mark.parametrize("n", [7, 8, 9, 16, 17, 100, 160])
def test_word_boundaries_with_measure_reset_rounds(n, d, flags):
    spec = workloads.random_hpc(n, d, 6 * n, seed=n + d, mr_every=max(1, n // 2), mr_fraction=0.3)
    prog = Program(spec.build())
    rec = _run(prog, 5, 0, 64, flags)
    assert np.array_equal(rec[:16], oracle_run([spec], 5, 0, 16)["records"]), (n, d)
    assert np.array_equal(rec, _run(prog, 5, 0, 64, BYTES)), (n, d)


@pytest.mark.parametrize("n,d", [(40, 5), (97, 7), (250, 5)])
def test_deterministic_sweeps(n, d):
    spec = _twice_measured(n, d, seed=n)
    prog = Program(spec.build())
    rec = _run(prog, 11, 0, 40, LANES)
    assert np.array_equal(rec[:4], oracle_run([spec], 11, 0, 4)["records"]), (n, d)
    assert np.array_equal(rec, _run(prog, 11, 0, 40, LANES_GMEM)), (n, d)
    assert np.array_equal(rec, _run(prog, 11, 0, 40, BYTES)), (n, d)


@pytest.mark.parametrize("n,d", [(256, 5), (320, 7), (321, 5), (600, 7)])
def test_shared_memory_limit_and_streamed(n, d):
    spec = workloads.random_hpc(n, d, 4 * n, seed=n + d)
    prog = Program(spec.build())
    rec = _run(prog, 3, 0, 2, LANES)
    assert np.array_equal(rec, oracle_run([spec], 3, 0, 2)["records"]), (n, d)
    assert np.array_equal(rec, _run(prog, 3, 0, 2, LANES_GMEM)), (n, d)
    assert np.array_equal(rec, _run(prog, 3, 0, 2, BYTES)), (n, d)


def test_odd_d_workload_n256_against_oracle():
    """The d = 5 and 7, n = 256 bench workload (MEASURE+RESET rounds, then
    MEASURE all) on 4-bit lanes in one CTA, 256 shots against the oracle."""
    for d in (5, 7):
        spec = workloads.odd_d(d, seed=0)
        prog = Program(spec.build())
        rec = _run(prog, 0, 0, 256, LANES)
        assert np.array_equal(rec[:16], oracle_run([spec], 0, 0, 16)["records"]), d
        assert np.array_equal(rec, _run(prog, 0, 0, 256, BYTES)), d


def test_uneven_batch_forms_agree():
    """A batch of d = 5 and 7 programs from 8 to 900 qudits (4-bit lanes in
    shared memory and streamed) equals the byte passes and, on its smaller
    programs, the oracle."""
    items = workloads.uneven_batch(160, seed=23, n_min=8, n_max=900, dims=(5, 7), shots_max=6)
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    lanes = br.run(flags=_lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ)
    bytes_ = br.run(flags=_lib.FLAG_TRACE | _lib.FLAG_U8_XZ)
    for it, a, b in zip(items, lanes, bytes_):
        assert np.array_equal(a, b), it.spec.name
    checked = 0
    for it, a in zip(items, lanes):
        if it.spec.num_qudits <= 120:
            assert np.array_equal(a, oracle_run([it.spec], it.seed, 0, it.shots)["records"]), it.spec.name
            checked += 1
    assert checked >= 20
