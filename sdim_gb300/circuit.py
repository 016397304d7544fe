"""Circuit builder with sdim's API (sdim/circuit.py:5-242).

``Circuit.add_gate(name, control, target=None, **kwargs)`` follows the
reference's rules: names are upper-cased and resolved through the alias
table; single-qudit gates fan out over a list of qudits and keep ``kwargs``
(N1 gets ``channel='d', prob=0.01`` defaults); two-qudit gates pair one
control with many targets, many controls with one target, or zip equal-length
lists, and drop ``kwargs`` (sdim/circuit.py:95-126).
"""
from __future__ import annotations

import numbers
from dataclasses import dataclass
from typing import List, Optional, Union

from .gatedata import GateData


@dataclass
class CircuitInstruction:
    gate_data: GateData
    gate_name: str
    qudit_index: int
    target_index: Optional[int] = None
    gate_id: Optional[int] = None
    name: Optional[str] = None
    params: Optional[dict] = None

    def __post_init__(self):
        self.gate_id = self.gate_data.get_gate_id(self.gate_name)
        if self.gate_id is None:
            raise ValueError(f"Gate {self.gate_name} not found")
        self.name = self.gate_data.get_gate_name(self.gate_id)

    def __str__(self):
        return f"{self.gate_id} {self.qudit_index} {self.target_index}"


def _as_list(v):
    if v is None:
        return None
    if isinstance(v, numbers.Integral):
        return [int(v)]
    return [int(x) for x in v]


@dataclass
class Circuit:
    num_qudits: int
    dimension: int = 2
    operations: list = None
    gate_data: GateData = None

    def __post_init__(self):
        if self.num_qudits < 1:
            raise ValueError("Number of qudits must be greater than 0")
        if self.dimension < 2:
            raise ValueError("Dimension must be greater than 1")
        self.operations = self.operations or []
        self.gate_data = self.gate_data or GateData(self.dimension)

    def add_gate(self, gate_name: str, control: Union[int, List[int]],
                 target: Union[int, List[int], None] = None, **kwargs):
        controls = _as_list(control)
        targets = _as_list(target)
        upper = gate_name.upper()
        primary = self.gate_data.aliasMap.get(upper, upper)
        gate = self.gate_data.gateMap.get(primary)
        if gate and gate.defaults:
            for k, v in gate.defaults.items():
                kwargs.setdefault(k, v)
        if targets is None:
            for c in controls:
                self.operations.append(CircuitInstruction(self.gate_data, upper, c, None, params=kwargs))
            return
        if len(controls) == 1:
            pairs = [(controls[0], t) for t in targets]
        elif len(targets) == 1:
            pairs = [(c, targets[0]) for c in controls]
        elif len(controls) == len(targets):
            pairs = list(zip(controls, targets))
        else:
            raise ValueError("Invalid combination of control and target qubits")
        for c, t in pairs:
            self.operations.append(CircuitInstruction(self.gate_data, upper, c, t))

    def __mul__(self, repetitions: int):
        original = list(self.operations)
        for _ in range(repetitions - 1):
            self.operations.extend(original)
        return self

    def __imul__(self, repetitions: int):
        return self.__mul__(repetitions)

    def __add__(self, other):
        if self.dimension != other.dimension:
            raise ValueError("Cannot add circuits with different dimensions")
        out = Circuit(max(self.num_qudits, other.num_qudits), self.dimension)
        out.operations = list(self.operations) + list(other.operations)
        return out

    def __iadd__(self, other):
        if self.dimension != other.dimension:
            raise ValueError("Cannot add circuits with different dimensions")
        self.num_qudits = max(self.num_qudits, other.num_qudits)
        self.operations.extend(other.operations)
        return self

    def __str__(self):
        return "\n".join(str(op) for op in self.operations)

    def print_gateData(self):  # noqa: N802 - sdim's name
        print(self.gate_data)

    @classmethod
    def from_operation_list(cls, operation_list, num_qudits, dimension):
        circuit = cls(num_qudits, dimension)
        for op in operation_list:
            if isinstance(op, tuple):
                name, qudits = op[0], op[1]
                if len(qudits) == 1:
                    circuit.add_gate(name, qudits[0])
                elif len(qudits) == 2:
                    circuit.add_gate(name, qudits[0], qudits[1])
                else:
                    raise ValueError(f"Unsupported number of qudits for gate {name}")
            elif isinstance(op, CircuitInstruction):
                circuit.add_gate(op.gate_name, op.qudit_index, op.target_index)
            else:
                raise ValueError(f"Unsupported operation type: {type(op)}")
        return circuit
