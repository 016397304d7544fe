"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
fixtures and the oracle, bit for bit."""
import numpy as np
import pytest

import oracle
from sdim_gb300 import MeasurementResult, Program, _lib, workloads
from tests.conftest import oracle_run, program_of, specs_of

pytestmark = pytest.mark.gpu


def test_golden_records_every_case(golden):
    cases, arrays = golden
    for name, case in cases.items():
        prog = program_of(case)
        rec = prog.sample(case["nshots"], seed=case["seed"], noise=case["noise"])
        assert np.array_equal(rec, arrays[f"{name}__records"]), name


def test_golden_records_plain_form(golden):
    cases, arrays = golden
    for name, case in cases.items():
        if case["nshots"] > 64:
            continue
        prog = program_of(case)
        rec = prog.sample(case["nshots"], seed=case["seed"], noise=case["noise"], plain=True)
        assert np.array_equal(rec, arrays[f"{name}__records"]), name


def test_golden_tableau_after_every_instruction(golden):
    cases, arrays = golden
    checked = 0
    for name, case in cases.items():
        key = f"{name}__snapshots"
        if key not in arrays.files:
            continue
        prog = program_of(case)
        snaps, rec = prog.snapshot(case["seed"], 0, _lib.SNAP_EVERY_INSTRUCTION, noise=case["noise"])
        assert np.array_equal(snaps, arrays[key]), name
        assert np.array_equal(rec, arrays[f"{name}__records"][0]), name
        checked += 1
    assert checked > 80


def test_golden_final_tableaux(golden):
    cases, arrays = golden
    for name, case in cases.items():
        key = f"{name}__final"
        if key not in arrays.files:
            continue
        ref = arrays[key]
        prog = program_of(case)
        for shot in range(ref.shape[0]):
            snap, _ = prog.snapshot(case["seed"], shot, _lib.SNAP_FINAL, noise=case["noise"])
            assert np.array_equal(snap[0], ref[shot]), (name, shot)


def test_golden_record_tableau(golden):
    cases, arrays = golden
    names = [n for n in cases if f"{n}__record_tableau" in arrays.files]
    assert names
    for name in names:
        case = cases[name]
        prog = program_of(case)
        res = prog.simulate(seed=case["seed"], record_tableau=True)
        ref = arrays[f"{name}__record_tableau"]
        enc = prog.compile().enc
        for j in range(enc.num_records):
            q, r = int(enc.meas_qudit[j]), int(enc.meas_round[j])
            # shots == 1: flat list in (qudit, round) order
            pos = sum(1 for jj in range(enc.num_records)
                      if (enc.meas_qudit[jj], enc.meas_round[jj]) < (q, r))
            t = res[pos].stabilizer_tableau
            flat = np.concatenate([t.x_block.ravel(), t.z_block.ravel(), t.phase_vector,
                                   t.destab_x_block.ravel(), t.destab_z_block.ravel(), t.destab_phase_vector])
            assert np.array_equal(flat.astype(np.int8), ref[j]), (name, j)


def test_known_answers_through_simulate(golden):
    cases, _ = golden
    for name, case in cases.items():
        if "expected" not in case:
            continue
        prog = program_of(case)
        res = prog.simulate(seed=case["seed"])
        assert res == [MeasurementResult(*e) for e in case["expected"]], name
        # shots > 1: nested [qudit][round][shot]
        res2 = prog.simulate(shots=3, seed=case["seed"], force_tableau=True)
        assert [[len(r) for r in q] for q in res2] == [[3] * len(q) for q in res2]
        assert prog.measurement_results == res2


def test_pr1_all_shots_and_per_instruction_tableau():
    spec = workloads.pr1(0)
    prog = Program(spec.build())
    rec = prog.sample(1024, seed=0)
    ref = oracle_run([spec], 0, 0, 1024)
    assert np.array_equal(rec, ref["records"])
    snaps, _ = prog.snapshot(0, 0, _lib.SNAP_EVERY_INSTRUCTION)
    ref0 = oracle_run([spec], 0, 0, 1, snapshots=True)
    assert np.array_equal(snaps, ref0["snapshots"])


def test_surface_distance7_full_size_sample():
    spec = workloads.surface_memory(7, 7, prob=1e-3)
    prog = Program(spec.build())
    rec = prog.sample(2048, seed=0)
    ref = oracle_run([spec], 0, 0, 2048)["records"]
    assert np.array_equal(rec, ref)
    # shot ranges are position-stable: a sub-range run alone gives the same records
    part = prog.sample(100, seed=0, shot0=1000)
    assert np.array_equal(part, rec[1000:1100])


@pytest.mark.parametrize("d", [5, 7])
def test_odd_d_n256_sample(d):
    spec = workloads.odd_d(d, seed=0)
    prog = Program(spec.build())
    rec = prog.sample(32, seed=0)
    ref = oracle_run([spec], 0, 0, 32)["records"]
    assert np.array_equal(rec, ref)


@pytest.mark.parametrize("d", [2, 3, 11])
def test_global_memory_slots_match_shared(d):
    spec = workloads.all_gates_random(9, d, 300, seed=d)
    prog = Program(spec.build())
    dp = prog.compile()
    a = prog.sample(64, seed=4)
    out = np.empty_like(a)
    rc = prog.context.lib.sdim_run(prog.context.ptr, dp.ptr, 4, 0, 64, out.ctypes.data, _lib.FLAG_FORCE_GMEM)
    _lib.check(rc, prog.context.ptr)
    assert np.array_equal(a, out)
    assert np.array_equal(a, oracle_run([spec], 4, 0, 64)["records"])


def test_large_n_global_memory_path():
    # n = 700 at d = 3 needs a 1 MB slot: global-memory tableaux
    spec = workloads.random_hpc(700, 3, 1400, seed=9)
    prog = Program(spec.build())
    assert prog.compile().slot_bytes > prog.context.smem_optin
    rec = prog.sample(4, seed=1)
    assert np.array_equal(rec, oracle_run([spec], 1, 0, 4)["records"])


def test_errors_map_to_python_exceptions():
    from sdim_gb300 import Circuit
    c = Circuit(2, 3)
    c.add_gate("H", 5)
    with pytest.raises(IndexError):
        Program(c).simulate(seed=1)
    c = Circuit(2, 3)
    c.add_gate("CNOT", 0, 7)
    with pytest.raises(IndexError):
        Program(c).simulate(seed=1)


def test_stabilizer_tableau_after_simulate(golden):
    cases, arrays = golden
    case = cases["kat_deutsch_d3"]
    prog = program_of(case)
    prog.simulate(seed=case["seed"])
    t = prog.stabilizer_tableau
    ref = arrays["kat_deutsch_d3__final"][0]
    flat = np.concatenate([t.x_block.ravel(), t.z_block.ravel(), t.phase_vector, t.destab_x_block.ravel(),
                           t.destab_z_block.ravel(), t.destab_phase_vector]).astype(np.int8)
    assert np.array_equal(flat, ref)


# ---------------------------------------------------------------------------
# shot-group engine (d = 2): 32 shots per warp share x/z; phases = c + delta_s
# ---------------------------------------------------------------------------
def test_group_engine_every_lane_tableau_after_every_instruction():
    """Noisy small surface code: the full tableau of several shots inside one
    group (and across groups) equals the oracle's after every instruction."""
    spec = workloads.surface_memory(3, 2, prob=0.08)
    prog = Program(spec.build())
    for shot in (0, 5, 31, 33, 70):
        snaps, rec = prog.snapshot(17, shot, _lib.SNAP_EVERY_INSTRUCTION)
        ref = oracle_run([spec], 17, shot, 1, snapshots=True)
        assert np.array_equal(rec, ref["records"][0]), shot
        assert np.array_equal(snaps, ref["snapshots"]), shot


def test_group_engine_random_circuits_every_lane():
    for d, seed in ((2, 1), (2, 2)):
        spec = workloads.all_gates_random(6, d, 160, seed=seed, noise_probs=(0.0, 0.4, 1.0))
        prog = Program(spec.build())
        for shot in (0, 7, 30):
            snaps, rec = prog.snapshot(3, shot, _lib.SNAP_EVERY_INSTRUCTION)
            ref = oracle_run([spec], 3, shot, 1, snapshots=True)
            assert np.array_equal(snaps, ref["snapshots"]), (d, seed, shot)
        snaps, _ = prog.snapshot(3, 9, _lib.SNAP_AT_MEASUREMENT)
        per_shot, _ = prog.snapshot(3, 9, _lib.SNAP_AT_MEASUREMENT, per_shot=True)
        assert np.array_equal(snaps, per_shot)


@pytest.mark.parametrize("nshots", [1, 31, 45, 97])
def test_group_engine_partial_groups(nshots):
    spec = workloads.surface_memory(3, 3, prob=0.05)
    prog = Program(spec.build())
    rec = prog.sample(nshots, seed=8, shot0=13)
    assert np.array_equal(rec, oracle_run([spec], 8, 13, nshots)["records"])


def test_group_engine_equals_per_shot_engine_full_size():
    spec = workloads.surface_memory(7, 7, prob=1e-3)
    prog = Program(spec.build())
    a = prog.sample(4096, seed=3)
    b = prog.sample(4096, seed=3, per_shot=True)
    assert np.array_equal(a, b)


def test_noiseless_surface_code_properties_100k_shots():
    """Size-independent properties at full size: without noise, round-1
    Z-check outcomes are 0 and every later round repeats round 1; the
    deterministic flags are identical in every shot."""
    spec = workloads.surface_memory(7, 7, noise=False)
    prog = Program(spec.build())
    rec = prog.sample(100_000, seed=0)
    det = rec >> 7
    assert np.all(det == det[0])
    vals = (rec & 0x7F).astype(np.int64)
    n_anc = 48
    rounds = vals[:, :7 * n_anc].reshape(-1, 7, n_anc)
    assert np.all(rounds[:, 1:, :] == rounds[:, :1, :])
    assert np.all(rounds[:, 0, 24:] == 0)          # Z checks start at +1
    assert np.all(det[0, n_anc:7 * n_anc] == 1)     # later rounds are deterministic
    frac_one = rounds[:, 0, :24].mean()
    assert 0.48 < frac_one < 0.52                    # X checks start random


def test_simulate_follows_circuit_mutations_against_oracle():
    """A live Program whose circuit is changed between calls (last
    instruction popped and a different one added, an instruction edited in
    place) simulates the circuit as it now stands: every call's records
    equal the oracle's on the same circuit object (the reference re-reads
    circuit.operations on every simulate, sdim/program.py:311-320)."""
    spec = workloads.random_hpc(6, 3, 60, seed=21)
    c = spec.build()
    prog = Program(c)
    for r in range(40):
        if r:
            c.operations.pop()
            c.add_gate("M" if r % 2 else "P", r % 6)
        if r % 7 == 3 and c.operations[r].target_index is None:
            c.operations[r].qudit_index = (c.operations[r].qudit_index + 1) % 6
        got = prog.sample(64, seed=100 + r)
        ref = oracle.simulate(oracle.OracleProgram([c], 6, 3), 100 + r, 0, 64)["records"]
        assert np.array_equal(got, ref), r
        res = prog.simulate(shots=4, force_tableau=True, seed=100 + r)
        flat = [[m.measurement_value for m in rounds] for per_q in res for rounds in per_q]
        assert sum(len(f) for f in flat) == 4 * ref.shape[1]


def test_apply_gate_continues_the_last_shot_against_oracle():
    """apply_gate steps the tableau of the last simulated shot
    (sdim/program.py:367-385): its measurement results and the resulting
    stabilizer_tableau equal the oracle run of the program with the applied
    instructions appended (RESET applied alone only measures, N1 is the
    identity, as the reference's gate functions do)."""
    from sdim_gb300 import Circuit
    from sdim_gb300.circuit import CircuitInstruction
    spec = workloads.random_hpc(5, 3, 40, seed=12)
    c = spec.build()
    prog = Program(c)
    prog.simulate(shots=1, force_tableau=True, seed=77)
    gd = c.gate_data
    steps = [("H", 0, None), ("CNOT", 0, 2), ("M", 0, None), ("P", 2, None), ("RESET", 2, None),
             ("N1", 1, None), ("M", 2, None), ("M_X", 1, None)]
    extra = Circuit(5, 3)
    got = []
    for name, q, t in steps:
        got.append(prog.apply_gate(CircuitInstruction(gd, name, q, t)))
        ref_name = {"RESET": "M", "N1": "I"}.get(name, name)
        if t is None:
            extra.add_gate(ref_name, q)
        else:
            extra.add_gate(ref_name, q, t)
    ref = oracle.simulate(oracle.OracleProgram([c, extra], 5, 3), 77, 0, 1, final=True)
    recs = ref["records"][0]
    meas = [r for r in got if r is not None]
    assert [r.qudit_index for r in meas] == [0, 2, 2, 1]
    assert [(int(r.measurement_value) | (int(r.deterministic) << 7)) for r in meas] == [int(v) for v in recs[-4:]]
    assert [r is None for r in got] == [True, True, False, True, False, True, False, False]
    snap, _ = prog.snapshot(77, 0, _lib.SNAP_FINAL)
    assert np.array_equal(snap[0], ref["final"][0])
    assert prog.stabilizer_tableau.x_block.shape == (5, 5)
    # simulate starts afresh: the applied instructions are dropped
    from sdim_gb300.encode import encode_program
    from sdim_gb300.program import flatten_single_shot, records_to_nested
    again = prog.simulate(shots=1, force_tableau=True, seed=77)
    first = oracle.simulate(oracle.OracleProgram([c], 5, 3), 77, 0, 1)["records"]
    assert again == flatten_single_shot(records_to_nested(first, encode_program([c], 5, 3), 5))
