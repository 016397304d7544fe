"""GPU: the d = 3 x / z pass on the two-bit-plane tableau (trace_p3.cuh)
against the oracle and against the byte-residue passes (SDIM_FLAG_U8_XZ),
bit for bit: every gate and noise channel on tiny programs, qudit counts at
the 32-lane word boundaries, deterministic sweeps, MEASURE+RESET rounds,
the tableau in shared memory (to n = 448) and streamed from global memory
(SDIM_FLAG_FORCE_GMEM, and n = 449 up), and uneven batches whose d = 3
programs take both forms."""
import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu

PLANES = _lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ
PLANES_GMEM = _lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ | _lib.FLAG_FORCE_GMEM
BYTES = _lib.FLAG_TRACE | _lib.FLAG_U8_XZ


def _run(prog, seed, shot0, shots, flags):
    dp = prog.compile(True)
    ctx = prog.context
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, seed, shot0, shots, out.ctypes.data, flags)
    _lib.check(rc, ctx.ptr, "d = 3 trace pass")
    return out


def _twice_measured(n, seed):
    base = workloads.random_hpc(n, 3, 4 * n + 10, seed=seed)
    rng = np.random.default_rng(seed)
    ops = list(base.ops)
    ops += [("X" if rng.random() < 0.5 else "Z", int(q), None, {}) for q in rng.integers(n, size=n)]
    ops += [("M", q, None, {}) for q in range(n)]
    return workloads.CircuitSpec(n, 3, ops, f"twice_n{n}")


@pytest.mark.parametrize("flags", [PLANES, PLANES_GMEM], ids=["smem", "gmem"])
@pytest.mark.parametrize("n", [1, 2, 5, 9])
def test_every_gate_and_channel_against_oracle(n, flags):
    spec = workloads.all_gates_random(n, 3, 300, seed=40 + n, noise_probs=(0.0, 0.3, 1.0))
    prog = Program(spec.build())
    rec = _run(prog, 7, 2, 130, flags)
    assert np.array_equal(rec, oracle_run([spec], 7, 2, 130)["records"]), n
    assert np.array_equal(rec, _run(prog, 7, 2, 130, BYTES)), n


@pytest.mark.parametrize("flags", [PLANES, PLANES_GMEM], ids=["smem", "gmem"])
@pytest.mark.parametrize("n", [31, 32, 33, 64, 65, 100, 160])
def test_word_boundaries_with_measure_reset_rounds(n, flags):
    spec = workloads.random_hpc(n, 3, 6 * n, seed=n, mr_every=max(1, n // 2), mr_fraction=0.3)
    prog = Program(spec.build())
    rec = _run(prog, 5, 0, 64, flags)
    assert np.array_equal(rec[:16], oracle_run([spec], 5, 0, 16)["records"]), n
    assert np.array_equal(rec, _run(prog, 5, 0, 64, BYTES)), n


@pytest.mark.parametrize("n", [40, 97, 250])
def test_deterministic_sweeps(n):
    spec = _twice_measured(n, seed=n)
    prog = Program(spec.build())
    rec = _run(prog, 11, 0, 40, PLANES)
    assert np.array_equal(rec[:4], oracle_run([spec], 11, 0, 4)["records"]), n
    assert np.array_equal(rec, _run(prog, 11, 0, 40, PLANES_GMEM)), n
    assert np.array_equal(rec, _run(prog, 11, 0, 40, BYTES)), n


@pytest.mark.parametrize("n", [448, 449, 700])
def test_shared_memory_limit_and_streamed(n):
    spec = workloads.random_hpc(n, 3, 4 * n, seed=n)
    prog = Program(spec.build())
    rec = _run(prog, 3, 0, 2, PLANES)
    assert np.array_equal(rec, oracle_run([spec], 3, 0, 2)["records"]), n
    assert np.array_equal(rec, _run(prog, 3, 0, 2, BYTES)), n


def test_uneven_batch_d3_forms_agree():
    """A batch of d = 3 programs from 8 to 900 qudits (bit planes in shared
    memory and streamed, in one launch each) equals the byte passes and, on
    its smaller programs, the oracle."""
    items = workloads.uneven_batch(120, seed=21, n_min=8, n_max=900, dims=(3,), shots_max=6)
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    planes = br.run(flags=_lib.FLAG_TRACE | _lib.FLAG_PACKED_XZ)
    bytes_ = br.run(flags=_lib.FLAG_TRACE | _lib.FLAG_U8_XZ)
    for it, a, b in zip(items, planes, bytes_):
        assert np.array_equal(a, b), it.spec.name
    checked = 0
    for it, a in zip(items, planes):
        if it.spec.num_qudits <= 120:
            assert np.array_equal(a, oracle_run([it.spec], it.seed, 0, it.shots)["records"]), it.spec.name
            checked += 1
    assert checked >= 20
