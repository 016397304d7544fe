"""Oracle for the prime-dimension tableau path -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker or the timed CPU
baseline; the product (``sdim_gb300``) never does.

* ``philox``          -- Philox4x32-10 stream (Salmon et al., SC'11), pinned
                         to the published known-answer vectors.
* ``tableau_oracle.c``-- plain-C restatement of sdim's ExtendedTableau and
                         shot loop (unreduced int64, lazy modulo, gate
                         compositions as in the reference); see its header.
* ``frame``           -- NumPy restatement of the reference's Pauli-frame
                         route (multi-shot ``simulate``), with its draws on
                         the same Philox stream.

The restatements are pinned against fixtures produced by the reference
itself (``tests/golden/make_golden.py`` imports sdim, injects this Philox
stream and records outcomes, tableaux and frame-route records).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path
from typing import Iterable, List, Optional, Sequence

import numpy as np

from . import philox  # noqa: F401

HERE = Path(__file__).resolve().parent
SRC = HERE / "tableau_oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

# sdim/gatedata.py:55-102 -- canonical names, aliases and ids
GATE_IDS = {"I": 0, "X": 1, "X_INV": 2, "Z": 3, "Z_INV": 4, "H": 5, "H_INV": 6, "P": 7, "P_INV": 8,
            "CNOT": 9, "CNOT_INV": 10, "CZ": 11, "CZ_INV": 12, "SWAP": 13, "M": 14, "M_X": 15,
            "RESET": 16, "N1": 17}
ALIASES = {"R": "H", "DFT": "H", "R_INV": "H_INV", "DFT_INV": "H_INV", "H_DAG": "H_INV", "R_DAG": "H_INV",
           "DFT_DAG": "H_INV", "PHASE": "P", "S": "P", "PHASE_INV": "P_INV", "S_INV": "P_INV",
           "SUM": "CNOT", "CX": "CNOT", "C": "CNOT", "SUM_INV": "CNOT_INV", "CX_INV": "CNOT_INV",
           "C_INV": "CNOT_INV", "MEASURE": "M", "COLLAPSE": "M", "MZ": "M", "MEASURE_X": "M_X", "MX": "M_X",
           "MR": "RESET", "MEASURE_RESET": "RESET", "MEASURE_R": "RESET", "NOISE1": "N1"}
CHANNELS = {"d": 1, "f": 2, "p": 3}
MEASUREMENT_IDS = (14, 15, 16)

_lib = None


def build(force: bool = False) -> Path:
    """Compiles the C oracle (OpenMP when the compiler has it)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    base = [cc, "-O2", "-std=c11", "-fPIC", "-shared", str(SRC), "-o", str(tmp)]
    res = subprocess.run(base[:2] + ["-fopenmp"] + base[2:], capture_output=True, text=True)
    if res.returncode != 0:
        res = subprocess.run(base, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.oracle_simulate.restype = C.c_int
        lib.oracle_simulate.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_uint64,
                                        C.c_int64, C.c_int64, C.c_int, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int]
        lib.oracle_philox.restype = None
        lib.oracle_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


def resolve(name: str) -> int:
    up = name.upper()
    up = ALIASES.get(up, up)
    if up not in GATE_IDS:
        raise ValueError(f"Gate {name} not found")
    return GATE_IDS[up]


def noise_rule(params) -> tuple:
    """(channel code, probability): 'noise_channel', then 'channel', then 'd';
    probability 'prob', default 0.01."""
    params = params or {}
    ch = params.get("noise_channel", params.get("channel", "d"))
    return CHANNELS[ch], float(params.get("prob", 0.01))


class OracleProgram:
    """Rows for oracle_simulate built from one or more circuits.

    ``circuits``: a sequence of either specs (objects with ``ops`` of
    (name, qudit, target, params) tuples) or circuit objects (with
    ``operations`` of instructions carrying gate_id / qudit_index /
    target_index / params).  ``time`` restarts at every circuit, as the
    reference's enumerate does (sdim/program.py:311-318).
    """

    def __init__(self, circuits: Sequence, n: int, d: int):
        rows, thr = [], []
        self.meas_qudit: List[int] = []
        for circ in circuits:
            if hasattr(circ, "ops"):
                items = [(resolve(o[0]), o[1], o[2], o[3]) for o in circ.ops]
            else:
                items = [(int(i.gate_id), i.qudit_index, i.target_index, i.params) for i in circ.operations]
            for time, (gid, q, t, params) in enumerate(items):
                ch, th = 0, 0
                if gid == 17:
                    ch, p = noise_rule(params)
                    th = philox.noise_threshold(p)
                if gid in MEASUREMENT_IDS:
                    self.meas_qudit.append(int(q))
                rows.append((gid, int(q), -1 if t is None else int(t), time, ch))
                thr.append(th)
        self.n, self.d = int(n), int(d)
        self.ops = np.asarray(rows, dtype=np.int64).reshape(-1, 5)
        self.thr = np.asarray(thr, dtype=np.int64)
        self.nmeas = len(self.meas_qudit)

    @property
    def tableau_bytes(self) -> int:
        return 4 * self.n * self.n + 2 * self.n


def simulate(prog: OracleProgram, seed: int, shot0: int = 0, nshots: int = 1, noise: bool = True,
             final: bool = False, snapshots: bool = False, threads: int = 0):
    """Runs the C oracle.  Returns dict(records=(nshots, nmeas) uint8,
    final=(nshots, tb) int8 or None, snapshots=(nops, tb) int8 or None)."""
    lib = load()
    if threads <= 0:
        threads = max(1, min(os.cpu_count() or 1, 64))
    tb = prog.tableau_bytes
    rec = np.zeros((nshots, max(prog.nmeas, 1)), dtype=np.uint8)
    fin = np.zeros((nshots, tb), dtype=np.int8) if final else None
    snp = np.zeros((max(prog.ops.shape[0], 1), tb), dtype=np.int8) if snapshots else None
    rc = lib.oracle_simulate(prog.n, prog.d, prog.ops.shape[0], prog.ops.ctypes.data, prog.thr.ctypes.data,
                             int(seed) & 0xFFFFFFFFFFFFFFFF, int(shot0), int(nshots), 1 if noise else 0,
                             prog.nmeas, rec.ctypes.data, fin.ctypes.data if fin is not None else None,
                             snp.ctypes.data if snp is not None else None, int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_simulate failed with status {rc}")
    return {"records": rec[:, :prog.nmeas], "final": fin,
            "snapshots": None if snp is None else snp[:prog.ops.shape[0]]}


def c_philox(ctr, key):
    lib = load()
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib.oracle_philox(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out
