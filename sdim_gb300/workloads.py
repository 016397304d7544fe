"""Seeded synthetic circuits for the tableau path.

Every generator draws from ``numpy.random.Generator(PCG64(seed))`` and returns
a :class:`CircuitSpec`: qudit count, dimension and a flat list of
``(gate_name, qudit, target, params)`` tuples.  A spec builds into a drop-in
:class:`sdim_gb300.Circuit` (or any class with sdim's ``add_gate`` signature,
sdim/circuit.py:76) with :meth:`CircuitSpec.build`.

The reference ships no generators for these shapes (its random-circuit helper,
sdim/random_circuit.py:9-68, seeds Python's global ``random`` and draws from a
different gate set), so these are written from the workload descriptions:

* :func:`random_hpc` -- i.i.d. gates from {H, P, CNOT} with given weights,
  uniform qudits, CNOT on a uniform ordered pair of distinct qudits,
  optionally MEASURE+RESET on a random subset every ``mr_every`` gates, then
  MEASURE on all qudits.
* :func:`surface_memory` -- rotated-lattice surface-code memory circuit with
  noise after every gate.
* :func:`uneven_batch` -- many random circuits of log-uniform size.
* :func:`serving_stream` -- Poisson arrival trace of simulate requests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence, Tuple

import numpy as np

Op = Tuple[str, int, Optional[int], dict]


@dataclass
class CircuitSpec:
    num_qudits: int
    dimension: int
    ops_list: Optional[List[Op]] = None
    name: str = ""
    table: Optional[np.ndarray] = None  # int32 op table, when generated as arrays

    @property
    def ops(self) -> List[Op]:
        if self.ops_list is None:
            self.ops_list = table_to_ops(self.table) if self.table is not None else []
        return self.ops_list

    def op_table(self) -> np.ndarray:
        """int32 rows (gate id, qudit, target, channel); N1 probabilities are
        not part of the table (tables are only generated for N1-free programs)."""
        if self.table is None:
            from .gatedata import GateData
            gd = GateData(self.dimension)
            rows = []
            for name, q, t, params in self.ops:
                gid = gd.get_gate_id(gd.aliasMap.get(name.upper(), name.upper()))
                if gid == 17:
                    raise ValueError("op_table() holds no noise parameters; build a Circuit instead")
                rows.append((gid, q, -1 if t is None else t, 0))
            self.table = np.asarray(rows, dtype=np.int32).reshape(-1, 4)
        return self.table

    def build(self, circuit_cls=None):
        """Circuit object with every op added through ``add_gate``."""
        if circuit_cls is None:
            from .circuit import Circuit as circuit_cls  # noqa: N813
        c = circuit_cls(self.num_qudits, self.dimension)
        for name, q, t, params in self.ops:
            if t is None:
                c.add_gate(name, q, **params)
            else:
                c.add_gate(name, q, t, **params)
        return c

    def num_measurements(self) -> int:
        return sum(1 for op in self.ops if op[0] in ("M", "MEASURE", "M_X", "MX", "RESET", "MR"))

    def to_json(self) -> dict:
        return {"n": self.num_qudits, "d": self.dimension, "name": self.name,
                "ops": [[o[0], o[1], o[2], o[3]] for o in self.ops]}

    @staticmethod
    def from_json(obj: dict) -> "CircuitSpec":
        return CircuitSpec(obj["n"], obj["d"],
                           [(o[0], int(o[1]), None if o[2] is None else int(o[2]), dict(o[3]))
                            for o in obj["ops"]], obj.get("name", ""))


def _rng(seed) -> np.random.Generator:
    return seed if isinstance(seed, np.random.Generator) else np.random.Generator(np.random.PCG64(seed))


def _pair(rng: np.random.Generator, n: int) -> Tuple[int, int]:
    c = int(rng.integers(n))
    t = int(rng.integers(n - 1))
    if t >= c:
        t += 1
    return c, t


_GID_NAME = {5: "H", 7: "P", 9: "CNOT", 14: "M", 16: "RESET"}


def random_hpc_table(n: int, num_gates: int, seed=0, weights=(1 / 3, 1 / 3, 1 / 3), mr_every: int = 0,
                     mr_fraction: float = 0.0, final_measure: bool = True) -> np.ndarray:
    """Op table (int32 rows gate id, qudit, target, channel) of a random
    {H, P, CNOT} circuit: kinds drawn with ``weights``, single-qudit targets
    uniform, CNOT on a uniform ordered pair of distinct qudits; MEASURE+RESET
    on a uniformly random ``mr_fraction`` of the qudits after every
    ``mr_every`` gates; MEASURE on all qudits at the end."""
    rng = _rng(seed)
    cum = np.cumsum(np.asarray(weights, dtype=np.float64))
    cum /= cum[-1]
    kinds = np.searchsorted(cum, rng.random(num_gates), side="right")
    q = rng.integers(n, size=num_gates)
    t = rng.integers(max(n - 1, 1), size=num_gates)
    t = t + (t >= q)
    if n < 2:
        kinds[kinds == 2] = 1
    gid = np.where(kinds == 0, 5, np.where(kinds == 1, 7, 9))
    gates = np.stack([gid, q, np.where(gid == 9, t, -1), np.zeros_like(gid)], axis=1).astype(np.int32)
    mr_count = int(round(mr_fraction * n)) if mr_every else 0
    parts = []
    if mr_every and mr_count > 0:
        for start in range(0, num_gates, mr_every):
            stop = min(start + mr_every, num_gates)
            parts.append(gates[start:stop])
            if stop - start == mr_every:
                sel = np.sort(rng.choice(n, size=mr_count, replace=False))
                parts.append(np.stack([np.full(mr_count, 16), sel, np.full(mr_count, -1), np.zeros(mr_count)],
                                      axis=1).astype(np.int32))
    else:
        parts.append(gates)
    if final_measure:
        parts.append(np.stack([np.full(n, 14), np.arange(n), np.full(n, -1), np.zeros(n)], axis=1).astype(np.int32))
    return np.concatenate(parts, axis=0) if parts else np.zeros((0, 4), np.int32)


def table_to_ops(table: np.ndarray) -> List[Op]:
    return [(_GID_NAME[g], q, None if t < 0 else t, {}) for g, q, t, _ in table.tolist()]


def random_hpc(n: int, d: int, num_gates: int, seed=0, weights=(1 / 3, 1 / 3, 1 / 3),
               mr_every: int = 0, mr_fraction: float = 0.0, final_measure: bool = True,
               name: str = "") -> CircuitSpec:
    """Random {H, P, CNOT} circuit, optional periodic MEASURE+RESET, final
    MEASURE (the spec of :func:`random_hpc_table`)."""
    table = random_hpc_table(n, num_gates, seed, weights, mr_every, mr_fraction, final_measure)
    return CircuitSpec(n, d, None, name, table)


def pr1(seed: int = 0) -> CircuitSpec:
    """d=3, n=32, 640 gates i.i.d. from {H, P, CNOT}, then MEASURE on all 32."""
    return random_hpc(32, 3, 640, seed=seed, name="pr1_d3_n32_g640")


def odd_d(d: int, seed: int = 0, n: int = 256, num_gates: int = 2560) -> CircuitSpec:
    """Odd prime d, H 25% / P 25% / CNOT 50%; MEASURE+RESET on a random 10%
    of the qudits after every 256 gates; final MEASURE on all."""
    return random_hpc(n, d, num_gates, seed=seed, weights=(0.25, 0.25, 0.5),
                      mr_every=256 if num_gates >= 256 else num_gates, mr_fraction=0.1,
                      name=f"oddd_d{d}_n{n}_g{num_gates}")


# --------------------------------------------------------------------------
# rotated surface code memory
# --------------------------------------------------------------------------
def surface_layout(distance: int):
    """Rotated-lattice layout: data qubits on a distance x distance grid,
    one ancilla per plaquette.  Returns (x_checks, z_checks), each a list of
    data-index lists ordered [NW, NE, SW, SE] with None for missing corners."""
    L = distance
    x_checks, z_checks = [], []
    for i in range(-1, L):
        for j in range(-1, L):
            corners = []
            for (di, dj) in ((0, 0), (0, 1), (1, 0), (1, 1)):
                r, c = i + di, j + dj
                corners.append(r * L + c if 0 <= r < L and 0 <= c < L else None)
            present = sum(v is not None for v in corners)
            is_x = (i + j) % 2 == 0
            bulk = 0 <= i < L - 1 and 0 <= j < L - 1
            if bulk:
                (x_checks if is_x else z_checks).append(corners)
            elif present == 2:
                top_bottom = i in (-1, L - 1) and 0 <= j < L - 1
                left_right = j in (-1, L - 1) and 0 <= i < L - 1
                if top_bottom and is_x:
                    x_checks.append(corners)
                elif left_right and not is_x:
                    z_checks.append(corners)
    return x_checks, z_checks


def surface_memory(distance: int = 7, rounds: int = 7, prob: float = 1e-3,
                   channel: str = "d", noise: bool = True) -> CircuitSpec:
    """Rotated surface-code memory circuit on qubits (d=2).

    Data qubits 0..L*L-1, then X-type ancillas, then Z-type ancillas.  Each
    round: H on X ancillas, four CNOT layers (X checks: ancilla->data in
    NW, NE, SW, SE order; Z checks: data->ancilla in NW, SW, NE, SE order),
    H on X ancillas, RESET (measure + reset, one record each) on all
    ancillas.  With ``noise``, N1 follows every gate on every qudit it
    touches.  After the last round, MEASURE on every data qubit.
    For distance 7: 49 data + 48 ancillas = 97 qubits, 168 CNOTs per round.
    """
    L = distance
    x_checks, z_checks = surface_layout(L)
    nd = L * L
    xa = list(range(nd, nd + len(x_checks)))
    za = list(range(nd + len(x_checks), nd + len(x_checks) + len(z_checks)))
    n = nd + len(xa) + len(za)
    ops: List[Op] = []
    nparams = {"prob": prob, "noise_channel": channel}

    def noisy(q):
        if noise:
            ops.append(("N1", q, None, dict(nparams)))

    x_order = (0, 1, 2, 3)   # NW, NE, SW, SE
    z_order = (0, 2, 1, 3)   # NW, SW, NE, SE
    for _ in range(rounds):
        for a in xa:
            ops.append(("H", a, None, {}))
            noisy(a)
        for step in range(4):
            for a, corners in zip(xa, x_checks):
                dq = corners[x_order[step]]
                if dq is not None:
                    ops.append(("CNOT", a, dq, {}))
                    noisy(a)
                    noisy(dq)
            for a, corners in zip(za, z_checks):
                dq = corners[z_order[step]]
                if dq is not None:
                    ops.append(("CNOT", dq, a, {}))
                    noisy(dq)
                    noisy(a)
        for a in xa:
            ops.append(("H", a, None, {}))
            noisy(a)
        for a in xa + za:
            ops.append(("RESET", a, None, {}))
            noisy(a)
    for q in range(nd):
        ops.append(("M", q, None, {}))
    return CircuitSpec(n, 2, ops, f"surface_L{L}_r{rounds}_p{prob:g}")


# --------------------------------------------------------------------------
# batches and request streams
# --------------------------------------------------------------------------
@dataclass
class BatchItem:
    spec: CircuitSpec
    shots: int
    seed: int


def uneven_batch(num_circuits: int = 8192, seed: int = 0, n_min: int = 8, n_max: int = 1024,
                 dims: Sequence[int] = (2, 3, 5, 7), shots_max: int = 64,
                 gates_per_qudit: int = 4) -> List[BatchItem]:
    """Independent circuits: n = round(exp(U[ln n_min, ln n_max])), d uniform
    over ``dims``, ``gates_per_qudit * n`` gates from {H, P, CNOT}, MEASURE on
    all; shots uniform in [1, shots_max]."""
    rng = _rng(seed)
    items = []
    for i in range(num_circuits):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        d = int(dims[int(rng.integers(len(dims)))])
        shots = int(rng.integers(1, shots_max + 1))
        spec = random_hpc(n, d, gates_per_qudit * n, seed=rng, name=f"uneven{i}_n{n}_d{d}")
        items.append(BatchItem(spec, shots, seed * 1_000_003 + i))
    return items


@dataclass
class Request:
    arrival_s: float
    item: BatchItem


def serving_stream(rate_hz: float = 2000.0, duration_s: float = 60.0, seed: int = 0,
                   n_min: int = 16, n_max: int = 2048, dims: Sequence[int] = (2, 3, 5),
                   shots_min: int = 1, shots_max: int = 10_000, gates_per_qudit: int = 8,
                   max_requests: Optional[int] = None) -> List[Request]:
    """Poisson arrival trace: n and shots log-uniform, d uniform over ``dims``,
    ``gates_per_qudit * n`` random {H, P, CNOT} gates then MEASURE on all."""
    rng = _rng(seed)
    out: List[Request] = []
    t = 0.0
    i = 0
    while True:
        t += float(rng.exponential(1.0 / rate_hz))
        if t >= duration_s or (max_requests is not None and i >= max_requests):
            break
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        d = int(dims[int(rng.integers(len(dims)))])
        shots = int(round(math.exp(rng.uniform(math.log(shots_min), math.log(shots_max)))))
        spec = random_hpc(n, d, gates_per_qudit * n, seed=rng, name=f"req{i}_n{n}_d{d}")
        out.append(Request(t, BatchItem(spec, max(1, shots), seed * 7_919 + i)))
        i += 1
    return out


def all_gates_random(n: int, d: int, num_ops: int, seed=0, noise_probs=(0.0, 0.3, 1.0),
                     name: str = "") -> CircuitSpec:
    """Random circuit over every gate of the prime path (ids 0-17): I, X, X_INV,
    Z, Z_INV, H, H_INV, P, P_INV, CNOT, CNOT_INV, CZ, CZ_INV, SWAP, M, M_X,
    RESET and N1 with all three channels."""
    rng = _rng(seed)
    singles = ["I", "X", "X_INV", "Z", "Z_INV", "H", "H_INV", "P", "P_INV", "M", "M_X", "RESET", "N1"]
    pairs = ["CNOT", "CNOT_INV", "CZ", "CZ_INV", "SWAP"]
    ops: List[Op] = []
    for _ in range(num_ops):
        if n >= 2 and rng.random() < 0.35:
            c, t = _pair(rng, n)
            ops.append((pairs[int(rng.integers(len(pairs)))], c, t, {}))
        else:
            g = singles[int(rng.integers(len(singles)))]
            q = int(rng.integers(n))
            if g == "N1":
                p = float(noise_probs[int(rng.integers(len(noise_probs)))])
                ch = "dfp"[int(rng.integers(3))]
                ops.append(("N1", q, None, {"prob": p, "noise_channel": ch}))
            else:
                ops.append((g, q, None, {}))
    for q in range(n):
        ops.append(("M", q, None, {}))
    return CircuitSpec(n, d, ops, name)


def total_shots(items: Iterable[BatchItem]) -> int:
    return sum(it.shots for it in items)
