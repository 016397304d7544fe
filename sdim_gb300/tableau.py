"""Result and tableau value types with sdim's field names.

``MeasurementResult`` keeps sdim's dataclass fields and equality
(sdim/tableau/dataclasses.py:166-209).  ``Tableau`` / ``ExtendedTableau`` are
host-side views of a GPU tableau export in the reference's int64 block layout
(sdim/tableau/dataclasses.py:8-163, sdim/tableau/tableau_prime.py:8-95); gates
run on the GPU, so these carry state and printing only.
"""
from __future__ import annotations

from dataclasses import dataclass
from math import gcd
from typing import Optional

import numpy as np


@dataclass
class Tableau:
    num_qudits: int = 1
    dimension: int = 2
    phase_vector: Optional[np.ndarray] = None
    z_block: Optional[np.ndarray] = None
    x_block: Optional[np.ndarray] = None

    def __post_init__(self):
        n = self.num_qudits
        if self.phase_vector is None:
            self.phase_vector = np.zeros(n, dtype=np.int64)
        if self.z_block is None:
            self.z_block = np.eye(n, dtype=np.int64)
        if self.x_block is None:
            self.x_block = np.zeros((n, n), dtype=np.int64)

    @property
    def coprime_order(self) -> set:
        """Integers in [1, order) coprime to the order (sdim/tableau/dataclasses.py:48-56)."""
        return {i for i in range(1, self.order) if gcd(i, self.order) == 1}

    @property
    def coprime_dimension(self) -> set:
        """Integers in [1, d) coprime to d (sdim/tableau/dataclasses.py:58-66)."""
        return {i for i in range(1, self.dimension) if gcd(i, self.dimension) == 1}

    @property
    def prime(self) -> bool:
        """Whether d is prime, by the reference's trial division (sdim/tableau/dataclasses.py:68-76)."""
        return not any(self.dimension % i == 0 for i in range(2, self.dimension))

    @property
    def even(self) -> bool:
        return self.dimension % 2 == 0

    @property
    def order(self) -> int:
        return 2 * self.dimension if self.even else self.dimension

    @property
    def phase_order(self) -> int:
        return 2 if self.even else 1

    @property
    def pauli_size(self) -> int:
        return 2 * self.num_qudits + 1

    @property
    def stab_tableau(self) -> np.ndarray:
        return np.vstack((self.phase_vector, self.z_block, self.x_block))

    def modulo(self):
        self.z_block %= self.dimension
        self.x_block %= self.dimension
        self.phase_vector %= self.order

    @staticmethod
    def _print_labeled_matrix(label, matrix):
        print(f"{label}:")
        print(matrix)

    def print_phase_vector(self):
        self._print_labeled_matrix("Phase Vector", self.phase_vector)

    def print_z_block(self):
        self._print_labeled_matrix("Z Block", self.z_block)

    def print_x_block(self):
        self._print_labeled_matrix("X Block", self.x_block)

    def print_tableau(self):
        self.print_phase_vector()
        self.print_z_block()
        self.print_x_block()


@dataclass
class ExtendedTableau(Tableau):
    destab_phase_vector: Optional[np.ndarray] = None
    destab_z_block: Optional[np.ndarray] = None
    destab_x_block: Optional[np.ndarray] = None

    def __post_init__(self):
        super().__post_init__()
        n = self.num_qudits
        if self.destab_z_block is None:
            self.destab_z_block = np.zeros((n, n), dtype=np.int64)
        if self.destab_x_block is None:
            self.destab_x_block = np.eye(n, dtype=np.int64)
        if self.destab_phase_vector is None:
            self.destab_phase_vector = np.zeros(n, dtype=np.int64)

    @property
    def destab_tableau(self) -> np.ndarray:
        return np.vstack((self.destab_phase_vector, self.destab_z_block, self.destab_x_block))

    @property
    def tableau(self) -> np.ndarray:
        return np.hstack((self.stab_tableau, self.destab_tableau))

    def modulo(self):
        super().modulo()
        self.destab_x_block %= self.dimension
        self.destab_z_block %= self.dimension
        self.destab_phase_vector %= self.order

    def print_tableau(self):
        super().print_tableau()
        self._print_labeled_matrix("Destabilizer Phase Vector", self.destab_phase_vector)
        self._print_labeled_matrix("Destabilizer Z Block", self.destab_z_block)
        self._print_labeled_matrix("Destabilizer X Block", self.destab_x_block)

    @classmethod
    def from_export(cls, flat: np.ndarray, n: int, d: int) -> "ExtendedTableau":
        """Builds a tableau from one export record (x, z, ph, dx, dz, dph int8)."""
        flat = np.asarray(flat, dtype=np.int64)
        nn = n * n
        x = flat[0:nn].reshape(n, n).copy()
        z = flat[nn:2 * nn].reshape(n, n).copy()
        ph = flat[2 * nn:2 * nn + n].copy()
        o = 2 * nn + n
        dx = flat[o:o + nn].reshape(n, n).copy()
        dz = flat[o + nn:o + 2 * nn].reshape(n, n).copy()
        dph = flat[o + 2 * nn:o + 2 * nn + n].copy()
        return cls(n, d, ph, z, x, dph, dz, dx)


@dataclass
class MeasurementResult:
    qudit_index: int
    deterministic: bool
    measurement_value: int
    stabilizer_tableau: Optional[Tableau] = None

    def __str__(self) -> str:
        kind = "deterministic" if self.deterministic else "random"
        return f"Measured qudit ({self.qudit_index}) as ({self.measurement_value}) and was {kind}"

    def __repr__(self) -> str:
        return str(self)

    def get_tableau(self):
        if self.stabilizer_tableau is None:
            raise ValueError("Stabilizer tableau not recorded during measurement")
        return self.stabilizer_tableau
