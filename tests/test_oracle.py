"""CPU: the oracle is pinned to the reference (golden fixtures) and to the
published Philox known-answer vectors."""
import numpy as np
import pytest

import oracle
from oracle import philox
from tests.conftest import oracle_run, specs_of


@pytest.mark.parametrize("ctr,key,expected", philox.KAT)
def test_philox_known_answers(ctr, key, expected):
    got = [int(v) for v in philox.philox4x32_10(*ctr, *key)]
    assert got == list(expected)
    assert [int(v) for v in oracle.c_philox(ctr, key)] == list(expected)


def test_philox_c_matches_numpy_stream():
    rng = np.random.default_rng(5)
    for _ in range(200):
        ctr = [int(v) for v in rng.integers(0, 2**32, 4)]
        key = [int(v) for v in rng.integers(0, 2**32, 2)]
        a = [int(v) for v in philox.philox4x32_10(*ctr, *key)]
        assert a == [int(v) for v in oracle.c_philox(ctr, key)]


def test_noise_threshold_edges():
    assert philox.noise_threshold(0.0) == 1 << 32
    assert philox.noise_threshold(1.0) == 0
    assert philox.noise_threshold(1.5) == 0
    assert philox.noise_threshold(0.5) == 1 << 31
    assert philox.noise_threshold(1e-3) == int(np.floor((1 - 1e-3) * 2**32))


def test_residue_map_uniform_range():
    w = np.array([0, 1, 2**31, 2**32 - 1], dtype=np.uint64)
    assert philox.residue(w, 3).tolist() == [0, 0, 1, 2]


def test_every_golden_case_is_present(golden):
    cases, arrays = golden
    assert len(cases) >= 100
    for name in cases:
        assert f"{name}__records" in arrays.files


def test_oracle_matches_reference_records_and_tableaux(golden):
    """The C restatement reproduces the reference bit for bit: every record,
    the tableau after every instruction of the first shot, final tableaux."""
    cases, arrays = golden
    for name, case in cases.items():
        specs = specs_of(case)
        snaps = f"{name}__snapshots" in arrays.files
        fin = f"{name}__final" in arrays.files
        res = oracle_run(specs, case["seed"], 0, case["nshots"], noise=case["noise"], final=fin, snapshots=snaps)
        assert np.array_equal(res["records"], arrays[f"{name}__records"]), name
        if snaps:
            assert np.array_equal(res["snapshots"], arrays[f"{name}__snapshots"]), name
        if fin:
            ref = arrays[f"{name}__final"]
            assert np.array_equal(res["final"][:ref.shape[0]], ref), name


def test_known_answers_hold_in_fixtures(golden):
    cases, arrays = golden
    kat = [c for c in cases.values() if "expected" in c]
    assert len(kat) > 40
    for c in kat:
        rec = arrays[f"{c['name']}__records"][0]
        # expected is in the reference's flat (qudit, round) order
        specs = specs_of(c)
        prog = oracle.OracleProgram(specs, specs[0].num_qudits, specs[0].dimension)
        order = sorted(range(len(prog.meas_qudit)), key=lambda j: (prog.meas_qudit[j], j))
        flat = [(prog.meas_qudit[j], bool(rec[j] >> 7), int(rec[j] & 0x7F)) for j in order]
        assert flat == [tuple(e) for e in c["expected"]], c["name"]


def test_oracle_plants_detected():
    """A mistake planted in the oracle's input (one flipped gate) changes the
    records, so the comparison has teeth."""
    from sdim_gb300.workloads import pr1
    s = pr1(0)
    base = oracle_run([s], 0, 0, 16)["records"]
    ops = list(s.ops)
    k = next(i for i, o in enumerate(ops) if o[0] == "H")
    ops[k] = ("P", ops[k][1], None, {})
    s2 = type(s)(s.num_qudits, s.dimension, ops, "planted")
    other = oracle_run([s2], 0, 0, 16)["records"]
    assert not np.array_equal(base, other)


def test_oracle_independent_of_threads():
    from sdim_gb300.workloads import surface_memory
    s = surface_memory(3, 2, prob=0.05)
    a = oracle.simulate(oracle.OracleProgram([s], s.num_qudits, 2), 3, 0, 40, threads=1)["records"]
    b = oracle.simulate(oracle.OracleProgram([s], s.num_qudits, 2), 3, 0, 40, threads=4)["records"]
    c = oracle.simulate(oracle.OracleProgram([s], s.num_qudits, 2), 3, 20, 20, threads=2)["records"]
    assert np.array_equal(a, b)
    assert np.array_equal(a[20:], c)
