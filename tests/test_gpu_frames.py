"""GPU: the Pauli-frame sampler (the reference's multi-shot route) against
the reference's own route (frame fixtures), the frame oracle at larger sizes,
and size-independent properties at the full surface-code size."""
import json

import numpy as np
import pytest

from sdim_gb300 import Circuit, Program, workloads
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _frame_oracle(specs, seed, nshots):
    import oracle
    from oracle import frame
    n, d = specs[0].num_qudits, specs[0].dimension
    return frame.simulate(oracle.OracleProgram(specs, n, d), seed, nshots)


def _program(specs):
    prog = Program(specs[0].build())
    for s in specs[1:]:
        prog.append_circuit(s.build())
    return prog


def test_frames_match_reference_route_fixtures():
    cases = json.loads((GOLDEN / "frames.json").read_text())["cases"]
    arrays = np.load(GOLDEN / "frames.npz")
    for case in cases:
        specs = [workloads.CircuitSpec.from_json(c) for c in case["circuits"]]
        rec = _program(specs).sample_frames(case["nshots"], seed=case["seed"])
        assert np.array_equal(rec, arrays[case["name"] + "__records"]), case["name"]


@pytest.mark.parametrize("d", [2, 3, 5, 7, 11])
@pytest.mark.parametrize("n", [1, 4, 19])
def test_random_programs_match_oracle(d, n):
    spec = workloads.all_gates_random(n, d, 40 * n + 30, seed=40 * d + n, name="r")
    nshots = 77  # two full 32-shot blocks and a partial one after shot 0
    rec = _program([spec]).sample_frames(nshots, seed=d * 100 + n)
    assert np.array_equal(rec, _frame_oracle([spec], d * 100 + n, nshots))


@pytest.mark.parametrize("d,n", [(2, 300), (3, 300), (5, 700)])
def test_large_n_matches_oracle(d, n):
    spec = workloads.all_gates_random(n, d, 3 * n, seed=n + d, name="big")
    rec = _program([spec]).sample_frames(40, seed=3)
    assert np.array_equal(rec, _frame_oracle([spec], 3, 40))


def test_shot_counts_one_two_and_block_edges():
    spec = workloads.surface_memory(3, 2, prob=0.05)
    prog = _program([spec])
    full = _frame_oracle([spec], 8, 130)
    for nshots in (1, 2, 32, 33, 65, 130):
        assert np.array_equal(prog.sample_frames(nshots, seed=8), full[:nshots]), nshots


def test_surface_L7_rows_match_oracle_and_properties_at_full_size():
    """100,000 shots of the distance-7 memory: the first 300 rows equal the
    oracle (draws are keyed by the absolute shot index), every RESET column
    repeats shot 0, and every deterministic flag is shot 0's."""
    spec = workloads.surface_memory(7, 7, prob=1e-3)
    prog = _program([spec])
    rec = prog.sample_frames(100_000, seed=21)
    assert np.array_equal(rec[:300], _frame_oracle([spec], 21, 300))
    enc = prog.compile(True).enc
    ids = [int(r[0]) for r in enc.ops if int(r[0]) in (14, 15, 16)]
    resets = [j for j, g in enumerate(ids) if g == 16]
    assert np.all(rec[:, resets] == rec[0, resets])
    assert np.all((rec >> 7) == (rec[0] >> 7))


@pytest.mark.parametrize("d", [2, 3, 5])
def test_ghz_outcomes_agree_in_every_shot(d):
    """H on qudit 0 and CNOTs from it to every other qudit: in every shot all
    n outcomes are equal, and across shots every residue occurs."""
    n = 97
    c = Circuit(n, d)
    c.add_gate("H", 0)
    for q in range(1, n):
        c.add_gate("CNOT", 0, q)
    for q in range(n):
        c.add_gate("M", q)
    rec = Program(c).sample_frames(20_000, seed=6) & 0x7F
    assert np.all(rec == rec[:, :1])
    assert set(np.unique(rec[:, 0]).tolist()) == set(range(d))


def test_simulate_routes_like_the_reference():
    spec = workloads.surface_memory(3, 2, prob=0.05)
    prog = _program([spec])
    nested = prog.simulate(shots=50, seed=5)
    rec = prog.sample_frames(50, seed=5)
    enc = prog.compile(True).enc
    for j in range(enc.num_records):
        q, r = int(enc.meas_qudit[j]), int(enc.meas_round[j])
        got = [m.measurement_value | (0x80 if m.deterministic else 0) for m in nested[q][r]]
        assert got == rec[:, j].tolist()
    # shot 0 is the noiseless tableau shot
    assert np.array_equal(rec[0], prog.sample(1, seed=5, noise=False)[0])
    # force_tableau and record_tableau keep every shot on the tableau
    tab = prog.simulate(shots=50, seed=5, force_tableau=True)
    trec = prog.sample(50, seed=5)
    q, r = int(enc.meas_qudit[0]), int(enc.meas_round[0])
    assert [m.measurement_value for m in tab[q][r]] == (trec[:, 0] & 0x7F).tolist()


def test_frame_route_errors_match_the_reference():
    c = Circuit(2, 2)
    c.add_gate("H", 0)
    c.add_gate("N1", 0, prob=0.1)  # 'channel' but no 'noise_channel': the route reads the latter
    c.add_gate("M", 0)
    with pytest.raises(KeyError):
        Program(c).simulate(shots=4, seed=1)
    Program(c).simulate(shots=4, seed=1, force_tableau=True)  # the tableau route does not read it
    c2 = Circuit(2, 3)
    c2.add_gate("H", 1)
    c2.add_gate("M", 1)  # qudit 0 never measured
    with pytest.raises(ValueError):
        Program(c2).simulate(shots=3, seed=1)
