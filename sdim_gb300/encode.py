"""Host encoder: Circuit objects -> the op table of ``sdim_encode_circuit``.

The reference walks ``circuit.operations`` for every shot and dispatches
through GATE_FUNCTIONS (sdim/program.py:311-320, 367-385).  Here the walk
happens once per program: each instruction becomes one int32 row
``(gate_id, qudit, target, channel)`` plus an N1 probability, and the C
encoder turns the table into the device instruction stream.

N1 parameters: the channel is ``params['noise_channel']`` when present (the
key the reference's noise code reads, sdim/program.py:486 and
sdim/tableau/tableau_gates.py:374), else ``params['channel']`` (the key
add_gate fills by default, sdim/gatedata.py:102), else 'd'; the probability is
``params['prob']`` (default 0.01).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, List, Sequence

import numpy as np

from . import _lib
from .gatedata import MEASUREMENT_IDS, NOISE_CHANNEL_CODE, NOISE_ID, TWO_QUDIT_IDS


@dataclass
class EncodedProgram:
    n: int
    d: int
    ops: np.ndarray            # int32 [nops, 4]: gate id, qudit, target, channel
    probs: np.ndarray          # float64 [nops]
    meas_qudit: np.ndarray     # int64 [records]: qudit of each measurement record
    meas_round: np.ndarray     # int64 [records]: index of the record among that qudit's
    gate_counts: Dict[int, int] = field(default_factory=dict)

    @property
    def num_records(self) -> int:
        return int(self.meas_qudit.shape[0])

    @property
    def num_instructions(self) -> int:
        return int(self.ops.shape[0])


def noise_params(params) -> tuple:
    params = params or {}
    channel = params.get("noise_channel", params.get("channel", "d"))
    prob = float(params.get("prob", 0.01))
    if channel not in NOISE_CHANNEL_CODE:
        raise ValueError("Must specify a valid noise channel.")
    return NOISE_CHANNEL_CODE[channel], prob


def encode_program(circuits: Sequence, n: int, d: int, noise: bool = True) -> EncodedProgram:
    """Flattens the circuits of a program into the ABI op table.

    With ``noise=False`` every N1 becomes the identity, which is what the
    reference's tableau path does (sdim/program.py:31).
    """
    rows: List[tuple] = []
    probs: List[float] = []
    meas_q: List[int] = []
    counts: Dict[int, int] = {}
    for circuit in circuits:
        for ins in circuit.operations:
            gid = int(ins.gate_id)
            q = int(ins.qudit_index)
            t = -1 if ins.target_index is None else int(ins.target_index)
            if gid in TWO_QUDIT_IDS and ins.target_index is None:
                raise ValueError(f"gate {ins.name} needs a target qudit")
            ch, p = 0, 0.0
            if gid == NOISE_ID:
                if noise:
                    ch, p = noise_params(ins.params)
                else:
                    gid = 0
            if gid in MEASUREMENT_IDS:
                meas_q.append(q)
            rows.append((gid, q, t, ch))
            probs.append(p)
            counts[gid] = counts.get(gid, 0) + 1
    ops = np.asarray(rows, dtype=np.int32).reshape(-1, 4)
    mq = np.asarray(meas_q, dtype=np.int64)
    mr = np.zeros_like(mq)
    seen: Dict[int, int] = {}
    for j, q in enumerate(meas_q):
        mr[j] = seen.get(q, 0)
        seen[q] = mr[j] + 1
    return EncodedProgram(n, d, ops, np.asarray(probs, dtype=np.float64), mq, mr, counts)


def encode_table(table: np.ndarray, n: int, d: int, probs: np.ndarray = None) -> EncodedProgram:
    """EncodedProgram straight from an op table (rows gate id, qudit, target,
    channel) -- the path for callers that generate programs as arrays."""
    ops = np.ascontiguousarray(table, dtype=np.int32).reshape(-1, 4)
    if probs is None:
        probs = np.zeros(ops.shape[0], dtype=np.float64)
    meas = np.isin(ops[:, 0], (14, 15, 16))
    mq = ops[meas, 1].astype(np.int64)
    # round of each record: how many earlier records the same qudit has
    order = np.argsort(mq, kind="stable")
    sq = mq[order]
    starts = np.r_[0, np.flatnonzero(np.diff(sq)) + 1]
    counts = np.diff(np.r_[starts, len(sq)])
    rr = np.arange(len(sq)) - np.repeat(starts, counts)
    mr = np.empty_like(mq)
    mr[order] = rr
    gids, cnt = np.unique(ops[:, 0], return_counts=True)
    return EncodedProgram(int(n), int(d), ops, np.ascontiguousarray(probs, dtype=np.float64), mq, mr,
                          {int(g): int(c) for g, c in zip(gids, cnt)})


class DeviceProgram:
    """An encoded program resident on the device (``sdim_circuit``)."""

    def __init__(self, ctx: "_lib.Context", enc: EncodedProgram):
        self.ctx = ctx
        self.enc = enc
        lib = ctx.lib
        ptr = C.c_void_p()
        ops = np.ascontiguousarray(enc.ops)
        probs = np.ascontiguousarray(enc.probs)
        rc = lib.sdim_encode_circuit(ctx.ptr, ops.ctypes.data_as(C.c_void_p), int(ops.shape[0]),
                                     probs.ctypes.data_as(C.c_void_p) if probs.size else None,
                                     int(enc.n), int(enc.d), C.byref(ptr))
        _lib.check(rc, ctx.ptr, "encode")
        self.ptr = ptr
        info = (C.c_int64 * 8)()
        _lib.check(lib.sdim_circuit_info(ptr, info), ctx.ptr)
        (self.n, self.d, self.num_records, self.num_instructions, self.num_device_ops,
         self.backend, self.slot_bytes, self.group_slot_bytes) = (int(v) for v in info)

    def close(self):
        if getattr(self, "ptr", None):
            self.ctx.lib.sdim_circuit_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
