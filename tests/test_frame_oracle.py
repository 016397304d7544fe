"""The frame-route oracle (oracle/frame.py) against the reference's own
multi-shot route (fixtures by tests/golden/make_golden.py --frames)."""
import json

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def frame_golden():
    cases = json.loads((GOLDEN / "frames.json").read_text())["cases"]
    arrays = np.load(GOLDEN / "frames.npz")
    return cases, arrays


def _oracle_program(case):
    import oracle
    from sdim_gb300 import workloads as W
    specs = [W.CircuitSpec.from_json(c) for c in case["circuits"]]
    return oracle.OracleProgram(specs, specs[0].num_qudits, specs[0].dimension)


def test_frame_oracle_matches_reference_route(frame_golden):
    from oracle import frame
    cases, arrays = frame_golden
    assert len(cases) >= 15
    for case in cases:
        prog = _oracle_program(case)
        got = frame.simulate(prog, case["seed"], case["nshots"])
        want = arrays[case["name"] + "__records"]
        assert got.shape == want.shape, case["name"]
        assert np.array_equal(got, want), case["name"]


def test_frame_oracle_reset_records_reference_value(frame_golden):
    """RESET rows repeat shot 0's value in every frame shot
    (sdim/program.py:146-155), measurement rows vary with the frame."""
    from oracle import frame
    cases, _ = frame_golden
    case = next(c for c in cases if c["name"] == "frame_surface_L3_r3")
    prog = _oracle_program(case)
    rec = frame.simulate(prog, case["seed"], case["nshots"])
    resets = [j for j, row in enumerate(r for r in prog.ops if r[0] in (14, 15, 16)) if row[0] == 16]
    assert resets
    assert np.all(rec[:, resets] == rec[0, resets])
    measured = [j for j, row in enumerate(r for r in prog.ops if r[0] in (14, 15, 16)) if row[0] != 16]
    assert np.any(rec[1:, measured] != rec[0, measured])


def test_frame_draw_layout():
    """Frame event e uses word e & 3 of the domain-3 block e >> 2."""
    from oracle import frame, philox
    shots = np.arange(1, 9, dtype=np.uint64)
    for e in (0, 1, 2, 3, 4, 7, 9):
        block = philox.stream_words(11, shots, e >> 2, 3)
        assert np.array_equal(frame.frame_residues(11, shots, e, 5), philox.residue(block[e & 3], 5))
