"""CPU: drop-in API behaviour (Circuit, GateData, encoder, result nesting,
error conventions) and the C ABI library's exports."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from sdim_gb300 import Circuit, GateData, MeasurementResult, Program
from sdim_gb300.encode import encode_program
from sdim_gb300.program import flatten_single_shot, records_to_nested

ROOT = Path(__file__).resolve().parent.parent


def test_gate_ids_and_aliases():
    g = GateData(3)
    expected = ["I", "X", "X_INV", "Z", "Z_INV", "H", "H_INV", "P", "P_INV", "CNOT", "CNOT_INV", "CZ",
                "CZ_INV", "SWAP", "M", "M_X", "RESET", "N1"]
    assert [g.get_gate_name(i) for i in range(18)] == expected
    for alias, gid in [("DFT", 5), ("R_DAG", 6), ("S", 7), ("S_INV", 8), ("CX", 9), ("SUM_INV", 10),
                       ("MEASURE", 14), ("MX", 15), ("MR", 16), ("NOISE1", 17)]:
        assert g.get_gate_id(alias) == gid
    assert g.get_gate_id("NOPE") is None
    with pytest.raises(ValueError):
        g.get_gate_name(99)


def test_add_gate_fan_out_rules():
    c = Circuit(4, 3)
    c.add_gate("cnot", 0, [1, 2, 3])
    assert [(o.qudit_index, o.target_index) for o in c.operations] == [(0, 1), (0, 2), (0, 3)]
    c = Circuit(4, 3)
    c.add_gate("CX", [1, 2], 0)
    assert [(o.qudit_index, o.target_index) for o in c.operations] == [(1, 0), (2, 0)]
    c = Circuit(4, 3)
    c.add_gate("CZ", [0, 1], [2, 3])
    assert [(o.qudit_index, o.target_index, o.name) for o in c.operations] == [(0, 2, "CZ"), (1, 3, "CZ")]
    with pytest.raises(ValueError):
        c.add_gate("CNOT", [0, 1], [1, 2, 3])
    c = Circuit(3, 5)
    c.add_gate("measure", [0, 1, 2])
    assert [o.gate_id for o in c.operations] == [14, 14, 14]
    assert c.operations[0].gate_name == "MEASURE" and c.operations[0].name == "M"
    c.add_gate("N1", 0)
    assert c.operations[-1].params == {"channel": "d", "prob": 0.01}
    with pytest.raises(ValueError):
        c.add_gate("FOO", 0)


def test_circuit_validation_and_arithmetic():
    with pytest.raises(ValueError):
        Circuit(0, 2)
    with pytest.raises(ValueError):
        Circuit(2, 1)
    a = Circuit(2, 3)
    a.add_gate("H", 0)
    b = Circuit(3, 3)
    b.add_gate("X", 2)
    c = a + b
    assert c.num_qudits == 3 and len(c.operations) == 2
    with pytest.raises(ValueError):
        a + Circuit(2, 5)
    a *= 3
    assert len(a.operations) == 3
    d = Circuit.from_operation_list([("H", [0]), ("CNOT", [0, 1])], 2, 3)
    assert [o.gate_id for o in d.operations] == [5, 9]


def test_encoder_rows_and_noise_rule():
    c = Circuit(3, 3)
    c.add_gate("H", 0)
    c.add_gate("CNOT", 0, 1)
    c.add_gate("N1", 1, prob=0.25, noise_channel="f")
    c.add_gate("N1", 2, channel="p", prob=0.5)
    c.add_gate("N1", 2)
    c.add_gate("MX", 2)
    c.add_gate("M", 0)
    c.add_gate("RESET", 2)
    enc = encode_program([c], 3, 3)
    assert enc.ops.tolist() == [[5, 0, -1, 0], [9, 0, 1, 0], [17, 1, -1, 2], [17, 2, -1, 3], [17, 2, -1, 1],
                                [15, 2, -1, 0], [14, 0, -1, 0], [16, 2, -1, 0]]
    assert enc.probs.tolist()[2:5] == [0.25, 0.5, 0.01]
    assert enc.meas_qudit.tolist() == [2, 0, 2]
    assert enc.meas_round.tolist() == [0, 0, 1]
    off = encode_program([c], 3, 3, noise=False)
    assert off.ops[2:5, 0].tolist() == [0, 0, 0]
    bad = Circuit(1, 3)
    bad.add_gate("N1", 0, noise_channel="q")
    with pytest.raises(ValueError):
        encode_program([bad], 1, 3)


def test_records_to_nested_shapes():
    c = Circuit(2, 3)
    c.add_gate("M", [0, 1])
    c.add_gate("M", [0, 1])
    enc = encode_program([c], 2, 3)
    rec = np.array([[0x80 | 1, 2, 0x80, 1], [0x80 | 2, 0, 0x80, 1]], dtype=np.uint8)
    nested = records_to_nested(rec, enc, 2)
    assert nested[0][0] == [MeasurementResult(0, True, 1), MeasurementResult(0, True, 2)]
    assert nested[0][1] == [MeasurementResult(0, True, 0), MeasurementResult(0, True, 0)]
    assert nested[1][0] == [MeasurementResult(1, False, 2), MeasurementResult(1, False, 0)]
    assert nested[1][1] == [MeasurementResult(1, False, 1), MeasurementResult(1, False, 1)]
    flat = flatten_single_shot(records_to_nested(rec[:1], enc, 2))
    assert flat == [MeasurementResult(0, True, 1), MeasurementResult(0, True, 0), MeasurementResult(1, False, 2),
                    MeasurementResult(1, False, 1)]


def test_composite_dimension_rejected_without_gpu():
    with pytest.raises(NotImplementedError):
        Program(Circuit(2, 4))
    with pytest.raises(NotImplementedError):
        Program(Circuit(2, 6))


def test_measurement_result_strings():
    r = MeasurementResult(3, False, 2)
    assert str(r) == "Measured qudit (3) as (2) and was random"
    with pytest.raises(ValueError):
        r.get_tableau()


def _header_symbols():
    text = (ROOT / "include" / "sdim_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|double|const char\*)\s+(sdim_\w+)\s*\(", text, re.M)))


def test_library_builds_and_exports_every_header_symbol():
    from sdim_gb300 import _lib, build
    path = build.build_library()
    lib = ctypes.CDLL(str(path))
    syms = _header_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(_lib.SIGNATURES)


def test_ctypes_bindings_match_header_arity():
    """Every prototype of the header is bound with as many ctypes argument
    types as it has parameters."""
    from sdim_gb300 import _lib
    text = (ROOT / "include" / "sdim_gb300.h").read_text()
    protos = re.findall(r"^(?:int|double|const char\*)\s+(sdim_\w+)\s*\(([^;]*?)\);", text, re.M | re.S)
    assert len(protos) == len(_header_symbols())
    for name, params in protos:
        params = " ".join(params.split())
        arity = 0 if params in ("", "void") else len(params.split(","))
        assert len(_lib.SIGNATURES[name][1]) == arity, name


def test_library_without_device_reports_error_not_fallback():
    """With no CUDA device the context cannot be created: the API raises."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from sdim_gb300 import _lib
    with pytest.raises(_lib.SdimError):
        _lib.Context(0)


def test_odd_d_xz_routing_and_its_bench_mirror():
    """sdim_trace_xz_mode (host-only) on GB300's limits.  Residue bytes
    (d >= 11, or SDIM_FLAG_U8_XZ): one CTA to n = 226; for batches of 76+
    programs a CTA pair to n = 330, then one streaming CTA; for smaller
    batches an eight-CTA cluster, in shared memory to n = 642.  d = 3: one
    CTA on the bit-plane tableau, in shared memory to n = 448, then
    streamed.  d = 5, 7: one CTA on 4-bit lanes, in shared memory to n = 320,
    then streamed in batches of 76+ and the byte cluster in smaller ones.
    The bench's roofline model (bench.u8_xz_layout) agrees with it at every
    n."""
    import bench
    from sdim_gb300 import _lib
    lib = _lib.load()
    optin, sms = 232448, 152
    mode = lambda n, progs, flags=0, d=11: lib.sdim_trace_xz_mode(n, d, progs, flags, optin, sms)  # noqa: E731
    assert [mode(n, 1000) for n in (1, 226, 227, 330, 331, 2048)] == [0, 0, 1, 1, 2, 2]
    assert [mode(n, 75) for n in (226, 227, 642, 643, 2048)] == [0, 3, 3, 4, 4]
    assert mode(100, 1000, _lib.FLAG_CLUSTER_XZ) == 3
    assert mode(100, 1, _lib.FLAG_CLUSTER_XZ | _lib.FLAG_FORCE_GMEM) == 4
    assert mode(100, 1, _lib.FLAG_FORCE_GMEM) == 2
    assert mode(100, 1, _lib.FLAG_SPLIT_XZ) == 1
    # the bench names the x / z kernel of its lone programs from the same routing
    assert bench.xz_kernel_name(mode(32, 1, 0, 3)) == "k_trace_pass_u8"  # PR1
    assert bench.xz_kernel_name(mode(256, 1, 0, 5)) == "k_trace_pass_cluster"  # oddd5
    assert bench.xz_kernel_name(mode(200, 1, 0, 3)) == "k_trace_pass_p3"
    assert bench.xz_kernel_name(mode(200, 1, 0, 7)) == "k_trace_pass_n4"
    assert mode(0, 1) == _lib.SDIM_EINVAL and mode(2049, 1) == _lib.SDIM_EINVAL
    assert mode(10, 1, 0, 4) == _lib.SDIM_EINVAL
    packed = _lib.FLAG_PACKED_XZ
    assert [mode(n, 1000, 0, 3) for n in (1, 448, 449, 2048)] == [5, 5, 6, 6]
    assert [mode(n, 75, 0, 3) for n in (1, 127, 128, 226, 227, 2048)] == [0, 0, 5, 5, 3, 4]
    assert [mode(n, 75, packed, 3) for n in (1, 448, 449, 2048)] == [5, 5, 6, 6]
    assert mode(100, 1000, _lib.FLAG_FORCE_GMEM, 3) == mode(100, 1, packed | _lib.FLAG_FORCE_GMEM, 3) == 6
    assert mode(300, 1000, _lib.FLAG_U8_XZ, 3) == mode(300, 1000, _lib.FLAG_U8_XZ, 5) == mode(300, 1000) == 1
    assert mode(300, 1, _lib.FLAG_CLUSTER_XZ | packed, 3) == 3
    # a batch's CTAs have about one thread per qudit, a lone program's 1024
    # (more room for its row-group sums), so the shared-memory limits differ
    for d, batch_max, lone_max in ((5, 324, 315), (7, 320, 310)):
        assert [mode(n, 1000, 0, d) for n in (1, 256, batch_max, batch_max + 1, 2048)] == [7, 7, 7, 8, 8]
        assert [mode(n, 75, 0, d) for n in (127, 128, 226, 227, 642, 643)] == [0, 7, 7, 3, 3, 4]
        assert [mode(n, 1, packed, d) for n in (256, lone_max, lone_max + 1)] == [7, 7, 8]
        assert mode(100, 1, packed | _lib.FLAG_FORCE_GMEM, d) == 8
    forms = {0: (1, "smem"), 1: (2, "smem"), 2: (1, "hbm"), 3: (8, "smem"), 4: (8, "l2"), 5: (1, "smem"),
             6: (1, "hbm"), 7: (1, "smem"), 8: (1, "hbm")}
    for d in (3, 5, 7, 11):
        for progs in (1, 75, 76, 5000):
            for n in range(1, 2049):
                assert bench.u8_xz_layout(n, progs, optin, sms, d) == forms[mode(n, progs, 0, d)], (n, progs, d)


def test_bench_hbm_view_of_the_trace_step():
    """The headline roofline's HBM view: ncu DRAM bytes of one step over the
    step's kernel time, against the measured copy bandwidth."""
    import bench
    traffic = bench.read_traffic("trace_engine_surface_L7.md")
    assert traffic and traffic > 0
    v = bench.hbm_view(traffic, 0.5)
    assert v["achieved"] == pytest.approx(traffic / 0.5e-3 / 1e9)
    assert v["frac"] == pytest.approx(v["achieved"] / bench.hbm_peak())
    assert bench.hbm_view(None, 0.5) is None and bench.hbm_view(traffic, 0) is None


def test_tableau_properties_as_the_reference_defines_them():
    """sdim/tableau/dataclasses.py:48-119: coprime sets, primality, order."""
    from sdim_gb300.tableau import ExtendedTableau, Tableau
    t = ExtendedTableau(3, 2)
    assert (t.order, t.phase_order, t.pauli_size) == (4, 2, 7)
    assert t.coprime_order == {1, 3} and t.coprime_dimension == {1} and t.prime
    t = Tableau(2, 9)
    assert t.order == 9 and t.coprime_order == {1, 2, 4, 5, 7, 8} and not t.prime
    assert Tableau(1, 7).coprime_dimension == {1, 2, 3, 4, 5, 6}


def test_gatedata_registration_as_the_reference():
    """sdim/gatedata.py:55-122: add_gate takes the next id, aliases resolve,
    get_gate_matrix fails for every id (no gate has a matrix)."""
    from sdim_gb300 import Circuit, GateData
    g = GateData(3)
    g.add_gate("FOO", 1)
    g.add_gate_alias("FOO", ["BAR"])
    assert g.get_gate_id("FOO") == 18 and g.get_gate_id("BAR") == 18 and g.get_gate_name(18) == "FOO"
    assert g.get_gate_name(9) == "CNOT" and g.get_gate_id("SUM") == 9
    with pytest.raises(ValueError):
        g.get_gate_name(19)
    with pytest.raises(AttributeError):
        g.get_gate_matrix(5)
    with pytest.raises(ValueError):
        g.get_gate_matrix(40)
    c = Circuit(2, 3)
    c.gate_data.add_gate("FOO", 1)
    c.add_gate("foo", [0, 1])
    assert [op.gate_id for op in c.operations] == [18, 18]


def test_table_encoder_equals_circuit_encoder():
    """encode_table (arrays, the batch and serving path) gives the op table,
    record qudits, record rounds and gate counts of encode_program (Circuit
    objects) for the same program."""
    from sdim_gb300 import workloads
    from sdim_gb300.encode import encode_table
    for n, d, seed in ((5, 3, 1), (40, 7, 2), (97, 2, 3)):
        spec = workloads.random_hpc(n, d, 6 * n, seed=seed, mr_every=n, mr_fraction=0.3)
        a = encode_table(spec.table, n, d)
        b = encode_program([spec.build()], n, d)
        assert np.array_equal(a.ops, b.ops)
        assert np.array_equal(a.meas_qudit, b.meas_qudit) and np.array_equal(a.meas_round, b.meas_round)
        assert a.gate_counts == b.gate_counts
        assert a.num_records == b.num_records > n


def test_program_cache_key_follows_the_instructions():
    """Replacing, adding or reordering instructions changes the key under
    which the encoded program is cached (no device needed)."""
    from sdim_gb300 import Program
    from sdim_gb300.circuit import CircuitInstruction
    c = Circuit(2, 3)
    c.add_gate("H", 0)
    c.add_gate("M", 0)
    prog = Program(c)
    k0 = prog._program_key(True)
    assert prog._program_key(True) == k0 and prog._program_key(False) != k0
    c.operations[0] = CircuitInstruction(c.gate_data, "P", 0)
    k1 = prog._program_key(True)
    assert k1 != k0
    c.operations.reverse()
    assert prog._program_key(True) != k1
    c.add_gate("M", 1)
    assert len(prog._program_key(True)[0][0][1]) == 3
    # an instruction edited in place changes the key too
    k2 = prog._program_key(True)
    c.operations[-1].qudit_index = 0
    assert prog._program_key(True) != k2


class _FakeDeviceProgram:
    """Stands in for DeviceProgram: records what compile() encoded."""
    made = 0

    def __init__(self, ctx, enc):
        _FakeDeviceProgram.made += 1
        self.enc = enc


def test_program_recompiles_after_pop_and_add_gate(monkeypatch):
    """1,000 rounds of operations.pop() + add_gate() on a live Program: each
    round's compile() encodes the circuit as it now stands (the freed
    instruction's address is reused by CPython within a few rounds, so a key
    built on object ids would hand back the stale program)."""
    import sdim_gb300.program as P
    monkeypatch.setattr(P, "DeviceProgram", _FakeDeviceProgram)
    c = Circuit(3, 3)
    c.add_gate("H", 0)
    c.add_gate("CNOT", 0, 1)
    c.add_gate("M", 0)
    prog = P.Program(c)
    prog._ctx = object()
    dp = prog.compile()
    assert prog.compile() is dp  # unchanged circuit: cached
    _FakeDeviceProgram.made = 0
    prev_key = prog._program_key(True)
    for r in range(1000):
        c.operations.pop()
        c.add_gate("M", (r + 1) % 3)
        key = prog._program_key(True)
        assert key != prev_key
        prev_key = key
        dp = prog.compile()
        assert int(dp.enc.ops[-1, 0]) == 14 and int(dp.enc.ops[-1, 1]) == (r + 1) % 3
        assert prog.compile() is dp
    assert _FakeDeviceProgram.made == 1000
    # the same content again is a cache hit, also with fresh instruction objects
    c.operations.pop()
    c.add_gate("M", 1000 % 3)
    assert prog.compile() is dp and _FakeDeviceProgram.made == 1000


def test_header_flags_match_the_bindings():
    """Every SDIM_FLAG_* of include/sdim_gb300.h has the same value in _lib."""
    import re
    from sdim_gb300 import _lib
    text = (Path(__file__).resolve().parent.parent / "include" / "sdim_gb300.h").read_text()
    flags = dict(re.findall(r"#define SDIM_FLAG_(\w+) (\d+)u", text))
    assert len(flags) >= 14
    for name, v in flags.items():
        assert getattr(_lib, "FLAG_" + name) == int(v), name


def test_apply_gate_validates_before_any_device_call():
    """Program.apply_gate raises ValueError for an unknown gate id and
    IndexError for a qudit out of range (sdim/program.py:381-382; NumPy's
    IndexError in the reference), without touching the device."""
    from sdim_gb300 import Program
    from sdim_gb300.circuit import CircuitInstruction
    c = Circuit(2, 3)
    c.add_gate("H", 0)
    prog = Program(c)
    bad = CircuitInstruction(c.gate_data, "H", 0)
    bad.gate_id = 42
    with pytest.raises(ValueError):
        prog.apply_gate(bad)
    with pytest.raises(IndexError):
        prog.apply_gate(CircuitInstruction(c.gate_data, "CNOT", 0, 5))
    assert prog._applied == [] and prog._ctx is None
