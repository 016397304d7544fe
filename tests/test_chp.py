"""The .chp reader / writer and the native fast path, against fixtures made
by the reference's own sdim/circuit_io.py (tests/golden/make_golden.py --chp).
CPU only: the parser is host code of the library."""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from sdim_gb300 import circuit_io, workloads
from sdim_gb300.encode import encode_program


@pytest.fixture(scope="module")
def chp_cases():
    return json.loads((GOLDEN / "chp.json").read_text())["cases"]


def _parsed(circ):
    return [[ins.gate_name, int(ins.gate_id), int(ins.qudit_index),
             -1 if ins.target_index is None else int(ins.target_index),
             None if ins.params is None else {k: str(v) for k, v in ins.params.items()}]
            for ins in circ.operations]


def test_reader_matches_reference(chp_cases):
    seen = 0
    for case in chp_cases:
        if "parsed" not in case:
            continue
        circ = circuit_io.circuit_from_chp(case["text"])
        assert (circ.num_qudits, circ.dimension) == (case["parsed"]["n"], case["parsed"]["d"]), case["name"]
        assert _parsed(circ) == case["parsed"]["ops"], case["name"]
        seen += 1
    assert seen >= 9


def test_native_table_matches_reader(chp_cases):
    for case in chp_cases:
        if "parsed" not in case:
            continue
        circ = circuit_io.circuit_from_chp(case["text"])
        enc = encode_program([circ], circ.num_qudits, circ.dimension)
        table, probs, n, d = circuit_io.read_chp_table(case["text"])
        assert (n, d) == (circ.num_qudits, circ.dimension), case["name"]
        assert np.array_equal(table, enc.ops), case["name"]
        assert np.array_equal(probs, enc.probs), case["name"]


def test_errors_match_reference(chp_cases):
    errors = [c for c in chp_cases if "error" in c]
    assert len(errors) >= 5
    for case in errors:
        with pytest.raises(Exception) as info:
            circuit_io.circuit_from_chp(case["text"])
        assert type(info.value).__name__ == case["error"], case["name"]
        with pytest.raises(ValueError):
            circuit_io.read_chp_table(case["text"])


def test_writer_matches_reference(chp_cases, tmp_path, capsys):
    written = [c for c in chp_cases if "written_from" in c]
    assert len(written) == 4
    for case in written:
        circ = workloads.CircuitSpec.from_json(case["written_from"]).build()
        path = circuit_io.write_circuit(circ, output_file=case["name"] + ".chp", comment=case["comment"],
                                        directory=str(tmp_path))
        assert open(path).read() == case["text"], case["name"]
        back = circuit_io.read_circuit(path)  # an absolute path stands as it is
        assert _parsed(back) == case["parsed"]["ops"], case["name"]
    assert "Gate is " in capsys.readouterr().out  # the reference echoes every gate


def test_native_parser_sizes_and_long_text():
    spec = workloads.all_gates_random(40, 5, 20_000, seed=9, name="long")
    text = circuit_io.chp_text(spec.build())
    table, probs, n, d = circuit_io.read_chp_table(text.encode())
    circ = circuit_io.circuit_from_chp(text)
    enc = encode_program([circ], circ.num_qudits, circ.dimension)
    assert (n, d) == (circ.num_qudits, 5)
    assert np.array_equal(table, enc.ops) and np.array_equal(probs, enc.probs)
