"""Gate table of the tableau path: names, ids and aliases.

The ids, canonical names and aliases must equal sdim's (sdim/gatedata.py:55-102)
because programs are exchanged by name and the ids appear in sdim's IR
(sdim/program.py:13-32); the table is therefore kept identical.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Optional

# (canonical name, qudit count, aliases), in id order
_GATES = (
    ("I", 1, ()),
    ("X", 1, ()),
    ("X_INV", 1, ()),
    ("Z", 1, ()),
    ("Z_INV", 1, ()),
    ("H", 1, ("R", "DFT")),
    ("H_INV", 1, ("R_INV", "DFT_INV", "H_DAG", "R_DAG", "DFT_DAG")),
    ("P", 1, ("PHASE", "S")),
    ("P_INV", 1, ("PHASE_INV", "S_INV")),
    ("CNOT", 2, ("SUM", "CX", "C")),
    ("CNOT_INV", 2, ("SUM_INV", "CX_INV", "C_INV")),
    ("CZ", 2, ()),
    ("CZ_INV", 2, ()),
    ("SWAP", 2, ()),
    ("M", 1, ("MEASURE", "COLLAPSE", "MZ")),
    ("M_X", 1, ("MEASURE_X", "MX")),
    ("RESET", 1, ("MR", "MEASURE_RESET", "MEASURE_R")),
    ("N1", 1, ("NOISE1",)),
)

GATE_ID = {name: gid for gid, (name, _, _) in enumerate(_GATES)}
TWO_QUDIT_IDS = frozenset(gid for gid, (_, k, _) in enumerate(_GATES) if k == 2)
MEASUREMENT_IDS = frozenset((GATE_ID["M"], GATE_ID["M_X"], GATE_ID["RESET"]))
NOISE_ID = GATE_ID["N1"]
RESET_ID = GATE_ID["RESET"]
# N1 parameter defaults attached by add_gate (sdim/gatedata.py:102)
N1_DEFAULTS = {"channel": "d", "prob": 0.01}
NOISE_CHANNEL_CODE = {"d": 1, "f": 2, "p": 3}


@dataclass
class Gate:
    name: str
    arg_count: int
    gate_id: int
    defaults: Optional[dict] = None

    def __str__(self):
        return f"{self.name} {self.gate_id}"


class GateData:
    """Name/alias -> gate lookup, with the same attribute names as sdim's."""

    def __init__(self, dimension: int = 2):
        self.dimension = dimension
        self.gateMap: Dict[str, Gate] = {}
        self.aliasMap: Dict[str, str] = {}
        for gid, (name, count, aliases) in enumerate(_GATES):
            self.gateMap[name] = Gate(name, count, gid)
            for a in aliases:
                self.aliasMap[a] = name
        self.gateMap["N1"].defaults = dict(N1_DEFAULTS)
        self.num_gates = len(_GATES)

    def __str__(self):
        return "\n".join(str(g) for g in self.gateMap.values())

    def add_gate(self, name: str, arg_count: int):
        """Registers a gate under the next id (sdim/gatedata.py:55-59).  A
        program that uses an id outside 0-17 is refused when it is encoded,
        as the reference's apply_gate refuses it (sdim/program.py:381-382)."""
        self.gateMap[name] = Gate(name, arg_count, self.num_gates)
        self.num_gates += 1

    def add_gate_alias(self, name: str, list_alias):
        for alias in list_alias:
            self.aliasMap[alias] = name

    def get_gate_id(self, gate_name: str) -> Optional[int]:
        if gate_name in self.gateMap:
            return self.gateMap[gate_name].gate_id
        if gate_name in self.aliasMap:
            return self.gateMap[self.aliasMap[gate_name]].gate_id
        return None

    def get_gate_name(self, gate_id: int) -> str:
        for name, gate in self.gateMap.items():
            if gate.gate_id == gate_id:
                return name
        raise ValueError(f"Gate ID {gate_id} not found")

    def get_gate_matrix(self, gate_id: int):
        """The gate's ``unitary_matrix`` (sdim/gatedata.py:118-122).  No gate
        carries one, in the reference or here, so a known id raises
        AttributeError and an unknown one ValueError, as there."""
        for gate in self.gateMap.values():
            if gate.gate_id == gate_id:
                return gate.unitary_matrix
        raise ValueError(f"Gate ID {gate_id} not found")
