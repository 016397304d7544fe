"""GPU: shot-group engines (32 shots share x/z, per-shot phase deltas) for
every dimension, warp teams (n < 160) and CTA teams (n >= 160), against the
oracle: records, and the full tableau of individual shots inside a group."""
import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [3, 5, 7, 11])
def test_warp_team_every_lane_tableau(d):
    spec = workloads.all_gates_random(6, d, 150, seed=40 + d, noise_probs=(0.0, 0.35, 1.0))
    prog = Program(spec.build())
    for shot in (0, 9, 31, 40):
        snaps, rec = prog.snapshot(5, shot, _lib.SNAP_EVERY_INSTRUCTION)
        ref = oracle_run([spec], 5, shot, 1, snapshots=True)
        assert np.array_equal(rec, ref["records"][0]), (d, shot)
        assert np.array_equal(snaps, ref["snapshots"]), (d, shot)
    rec = prog.sample(77, seed=5, shot0=3)
    assert np.array_equal(rec, oracle_run([spec], 5, 3, 77)["records"])


@pytest.mark.parametrize("d", [3, 7])
def test_warp_team_resets_and_exponentiation(d):
    # odd d: pivots with x != 1 (exponentiate) and RESET corrections k in 1..d-1
    spec = workloads.random_hpc(40, d, 400, seed=d, weights=(0.3, 0.2, 0.5), mr_every=40, mr_fraction=0.25)
    prog = Program(spec.build())
    rec = prog.sample(96, seed=12)
    assert np.array_equal(rec, oracle_run([spec], 12, 0, 96)["records"])
    for shot in (2, 65):
        snaps, _ = prog.snapshot(12, shot, _lib.SNAP_AT_MEASUREMENT)
        ref, _ = prog.snapshot(12, shot, _lib.SNAP_AT_MEASUREMENT, per_shot=True)
        assert np.array_equal(snaps, ref)


@pytest.mark.parametrize("d", [2, 3, 5])
def test_cta_team_large_n(d):
    # n >= 160: one CTA per group; n = 170 puts odd-d slots in global memory
    spec = workloads.random_hpc(170, d, 700, seed=100 + d, mr_every=170, mr_fraction=0.1)
    prog = Program(spec.build())
    rec = prog.sample(40, seed=3)
    ref = oracle_run([spec], 3, 0, 40, final=True)
    assert np.array_equal(rec, ref["records"])
    for shot in (0, 17, 33):
        snap, _ = prog.snapshot(3, shot, _lib.SNAP_FINAL)
        assert np.array_equal(snap[0], ref["final"][shot]), (d, shot)


def test_cta_team_surface_code_d2():
    # distance 9: 81 data + 80 ancillas = 161 qubits, noisy, CTA team, shared-memory slot
    spec = workloads.surface_memory(9, 2, prob=0.02)
    prog = Program(spec.build())
    rec = prog.sample(70, seed=9)
    assert np.array_equal(rec, oracle_run([spec], 9, 0, 70)["records"])
    snaps, _ = prog.snapshot(9, 44, _lib.SNAP_AT_MEASUREMENT)
    ref, _ = prog.snapshot(9, 44, _lib.SNAP_AT_MEASUREMENT, per_shot=True)
    assert np.array_equal(snaps, ref)


def test_group_and_per_shot_engines_agree_on_uneven_programs():
    items = workloads.uneven_batch(40, seed=21, n_max=400, shots_max=40)
    for it in items[:12]:
        prog = Program(it.spec.build())
        a = prog.sample(it.shots, seed=it.seed)
        b = prog.sample(it.shots, seed=it.seed, per_shot=True)
        assert np.array_equal(a, b), it.spec.name
