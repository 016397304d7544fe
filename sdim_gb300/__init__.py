"""sdim_gb300: GB300-native prime-dimension stabilizer-tableau simulator.

Drop-in for sdim's tableau path: ``from sdim_gb300 import Circuit, Program,
MeasurementResult`` replaces ``from sdim import ...`` for prime dimensions.
All shots run in CUDA kernels (sm_103a) behind the C ABI in
``include/sdim_gb300.h``.
"""
from .circuit import Circuit, CircuitInstruction
from .circuit_io import read_chp_table, read_circuit, write_circuit
from .gatedata import Gate, GateData
from .program import Program, SimulationOptions
from .tableau import ExtendedTableau, MeasurementResult, Tableau

__all__ = ["Circuit", "CircuitInstruction", "Gate", "GateData", "Program", "SimulationOptions",
           "MeasurementResult", "Tableau", "ExtendedTableau", "read_circuit", "write_circuit", "read_chp_table"]
