"""The .chp circuit format: ``read_circuit`` / ``write_circuit`` as the
reference has them (sdim/circuit_io.py:6-139), and ``read_chp_table``, the
fast path from .chp text straight to the op table the engines take.

``read_circuit(filename)`` builds a ``Circuit`` with the reference's rules:
the path is taken relative to the directory above the package (an absolute
path stands as it is); the comment block ends at the first line that is "#"
after stripping; a first line "d <dim>" (any case) sets the dimension
(default 2); the circuit has one qudit more than the largest all-digit token;
each non-blank line is ``NAME idx [idx] [key=value ...]`` and goes through
``Circuit.add_gate`` with its all-digit tokens as indices and its
``key=value`` tokens as (string) parameters.

``write_circuit`` writes the comment (or the reference's default one), "#",
"d <dim>" and one ``NAME q [t] [key=value ...]`` line per instruction into
``directory`` (default: ``circuits/`` beside the package), prints each gate
as it goes, as the reference does, and returns the path.

``read_chp_table(text)`` parses the same text with the library's native
parser (``sdim_parse_chp``) into ``(table, probs, n, d)``: int32 rows
(gate id, qudit, target or -1, N1 channel) and N1 probabilities, ready for
``Server.submit`` or ``encode_table``, with no Python object per gate.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Iterable, Optional, Tuple, Union

import numpy as np

from . import _lib
from .circuit import Circuit

_BASE = Path(__file__).resolve().parent.parent


def _lines_to_circuit(lines: Iterable[str]) -> Circuit:
    lines = list(lines)
    start = next(i for i, line in enumerate(lines) if line.strip() == "#")
    body = lines[start + 1:]
    dimension = 2
    head = body[0].split()
    if head[0].upper() == "D":
        dimension = int(head[1])
        body = body[1:]
    largest = max(int(tok) for line in body for tok in line.split() if tok.isdigit())
    circuit = Circuit(largest + 1, dimension)
    for line in body:
        toks = line.split()
        if not toks:
            continue
        name = toks[0].upper()
        indices = [int(tok) for tok in toks[1:] if tok.isdigit()]
        params = None
        for tok in toks[1:]:
            if "=" not in tok:
                continue
            kv = tok.split("=")
            if len(kv) != 2:
                raise ValueError("Extra parameter doesn't have the correct format.")
            params = {} if params is None else params
            params[kv[0]] = kv[1]
        if len(indices) == 1:
            circuit.add_gate(name, indices[0], **(params or {}))
        elif len(indices) == 2:
            circuit.add_gate(name, indices[0], indices[1], **(params or {}))
        else:
            raise ValueError(f"Unexpected number of arguments for gate {name}")
    return circuit


def read_circuit(filename: Union[str, os.PathLike]) -> Circuit:
    """Circuit from a .chp file (sdim/circuit_io.py:6-83)."""
    with open(os.path.join(_BASE, filename), "r") as fh:
        return _lines_to_circuit(fh.readlines())


def circuit_from_chp(text: str) -> Circuit:
    """Circuit from .chp text, by the rules of ``read_circuit``."""
    return _lines_to_circuit(text.splitlines(keepends=True))


def chp_text(circuit: Circuit, comment: str = "", echo: bool = False) -> str:
    """The .chp text ``write_circuit`` writes for ``circuit``."""
    out = [f"{comment}\n#\n" if comment else "Randomly-generated Clifford group quantum circuit\n#\n",
           f"d {circuit.dimension}\n"]
    for gate in circuit.operations:
        line = gate.gate_name
        if echo:
            print("Gate is " + line)
        line += f" {gate.qudit_index}" if gate.target_index is None else f" {gate.qudit_index} {gate.target_index}"
        if gate.params is not None:
            for key, value in gate.params.items():
                line += f" {key}={value}"
        out.append(line + "\n")
    return "".join(out)


def write_circuit(circuit: Circuit, output_file: str = "random_circuit.chp", comment: str = "",
                  directory: Optional[str] = None) -> str:
    """Writes ``circuit`` as .chp (sdim/circuit_io.py:85-139); returns the path."""
    text = chp_text(circuit, comment, echo=True)
    if directory is None:
        directory = os.path.join(_BASE, "circuits")
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, output_file)
    with open(path, "w") as fh:
        fh.write(text)
    return path


def read_chp_table(text: Union[str, bytes]) -> Tuple[np.ndarray, np.ndarray, int, int]:
    """(table, probs, n, d) of .chp text, parsed natively (``sdim_parse_chp``)."""
    raw = text.encode() if isinstance(text, str) else bytes(text)
    lib = _lib.load()
    nrows, n, d = C.c_int64(0), C.c_int32(0), C.c_int32(0)
    err = C.create_string_buffer(512)
    rc = lib.sdim_parse_chp(raw, len(raw), None, None, 0, C.byref(nrows), C.byref(n), C.byref(d), err, 512)
    if rc != _lib.SDIM_OK:
        raise ValueError(err.value.decode())
    table = np.zeros((nrows.value, 4), dtype=np.int32)
    probs = np.zeros(nrows.value, dtype=np.float64)
    rc = lib.sdim_parse_chp(raw, len(raw), table.ctypes.data, probs.ctypes.data, nrows.value, C.byref(nrows),
                            C.byref(n), C.byref(d), err, 512)
    if rc != _lib.SDIM_OK:
        raise ValueError(err.value.decode())
    return table, probs, int(n.value), int(d.value)
