"""Drop-in ``Program`` for sdim's prime-dimension tableau path.

Mirrors sdim/program.py:167-573: ``Program(circuit)``,
``simulate(shots, show_measurement, record_tableau, force_tableau, verbose,
show_gate, exact, options)``, ``append_circuit``, ``measurement_results`` and
the return shapes (flat list for one shot, ``[qudit][round][shot]``
otherwise, sdim/program.py:355-365).  Every shot of every call runs on the
GPU through the C ABI; there is no CPU path.

Differences from the reference, by design:
* outcomes of random measurements come from the Philox stream keyed by
  (seed, shot, measurement ordinal) instead of Python's ``random``
  (sdim/tableau/tableau_prime.py:332); ``seed`` is a keyword of ``simulate``;
* on the tableau route N1 noise acts on the tableau (X^a then Z^b after the
  instruction); the reference's tableau path treats N1 as the identity
  (sdim/program.py:31) and samples noise only in its Pauli-frame route.
  ``noise=False`` reproduces the identity behaviour;
* composite dimensions raise NotImplementedError (the reference switches to
  WeylTableau, sdim/program.py:196-199).

Routes, as in sdim/program.py:244-265: ``shots > 1`` without
``record_tableau`` or ``force_tableau`` runs the Pauli-frame sampler on the
GPU (``sample_frames``: shot 0 is a noiseless tableau shot, the others
propagate frames against it); every other call runs every shot on the
tableau (``sample``).  The frame draws and N1 samples come from the Philox
stream, keyed by shot index, instead of ``np.random``.
"""
from __future__ import annotations

import copy
import gc
import secrets
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _lib
from .circuit import Circuit
from .encode import DeviceProgram, EncodedProgram, encode_program
from .gatedata import RESET_ID, GateData
from .tableau import ExtendedTableau, MeasurementResult


@dataclass
class SimulationOptions:
    shots: int = 1
    show_measurement: bool = False
    record_tableau: bool = False
    force_tableau: bool = False
    verbose: bool = False
    show_gate: bool = False
    exact: bool = False


def _is_prime(d: int) -> bool:
    return d >= 2 and all(d % k for k in range(2, int(d ** 0.5) + 1))


def records_to_nested(records: np.ndarray, enc: EncodedProgram, num_qudits: int) -> list:
    """(shots, records) bytes -> [qudit][round][shot] MeasurementResult lists.

    The cyclic garbage collector is paused while the objects are made: they
    hold only ints, bools and None, so they form no cycles, and without the
    pause the collector's repeated passes over millions of new objects take
    about two thirds of the time."""
    records = np.asarray(records, dtype=np.uint8).reshape(-1, enc.num_records)
    vals = (records & 0x7F).astype(np.int64)
    dets = (records >> 7).astype(bool)
    out: List[list] = [[] for _ in range(num_qudits)]
    collecting = gc.isenabled()
    gc.disable()
    try:
        for j in range(enc.num_records):
            q = int(enc.meas_qudit[j])
            col_v = vals[:, j].tolist()
            col_d = dets[:, j].tolist()
            out[q].append([MeasurementResult(q, dd, vv) for vv, dd in zip(col_v, col_d)])
    finally:
        if collecting:
            gc.enable()
    return out


def flatten_single_shot(nested: list) -> list:
    flat = []
    for per_qudit in nested:
        for shots_list in per_qudit:
            flat.append(shots_list[0])
    return flat


class Program:
    def __init__(self, circuit: Circuit, tableau=None, *, device: int = 0, seed: Optional[int] = None):
        if tableau is not None:
            raise NotImplementedError("a custom initial tableau is not supported on the GPU path")
        if not _is_prime(circuit.dimension):
            raise NotImplementedError(
                f"dimension {circuit.dimension} is composite: only prime dimensions have a GPU tableau path")
        self.num_qudits = circuit.num_qudits
        self.dimension = circuit.dimension
        self.circuits = [circuit]
        self.measurement_results: list = []
        self.device = device
        self.seed = seed
        self._ctx = None
        self._cache = {}
        self._last = None  # (seed, shot, noise) of the last simulated shot
        self._applied: list = []  # instructions applied by apply_gate since then

    # ------------------------------------------------------------------
    @property
    def context(self) -> _lib.Context:
        if self._ctx is None:
            self._ctx = _lib.Context.default(self.device)
        return self._ctx

    @staticmethod
    def _instruction_content(ins) -> tuple:
        """What the encoder reads from one instruction: gate id, qudit,
        target, and for N1 the channel keys and probability."""
        gid = ins.gate_id
        if gid == 17:
            p = ins.params or {}
            return (gid, ins.qudit_index, ins.target_index,
                    (p.get("noise_channel"), p.get("channel"), p.get("prob")))
        return (gid, ins.qudit_index, ins.target_index)

    def _program_key(self, noise: bool):
        """Cache key of the encoded program: the content of every instruction
        of every circuit (and each circuit's qudit count), read afresh on
        every call as the reference re-reads ``circuit.operations`` on every
        simulate (sdim/program.py:311-320).  Added, removed, replaced,
        reordered or edited-in-place instructions all change it; object
        identities play no part, so a new instruction that reuses a freed
        object's address cannot alias an old one."""
        content = self._instruction_content
        circuits = self.circuits + ([self._applied_circuit()] if self._applied else [])
        return (tuple((c.num_qudits, tuple([content(o) for o in c.operations])) for c in circuits),
                bool(noise))

    def _applied_circuit(self) -> Circuit:
        c = Circuit(self.num_qudits, self.dimension)
        c.operations = list(self._applied)
        return c

    def compile(self, noise: bool = True) -> DeviceProgram:
        """Encoded program on the device (cached while the circuits' content
        stays the same)."""
        key = self._program_key(noise)
        hit = self._cache.get(key[1])
        if hit is not None and hit[0] == key[0]:
            return hit[1]
        # apply_gate's instructions run after the circuits
        circuits = self.circuits + ([self._applied_circuit()] if self._applied else [])
        enc = encode_program(circuits, self.num_qudits, self.dimension, noise=noise)
        dp = DeviceProgram(self.context, enc)
        # keep the other noise setting only while it encodes the same circuits
        # (the frame route uses both)
        self._cache = {k: v for k, v in self._cache.items() if v[0] == key[0]}
        self._cache[key[1]] = (key[0], dp)
        return dp

    def _seed(self, seed):
        if seed is not None:
            return int(seed) & 0xFFFFFFFFFFFFFFFF
        if self.seed is not None:
            return int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return secrets.randbits(63)

    # ------------------------------------------------------------------
    def sample(self, shots: int, seed: Optional[int] = None, shot0: int = 0, noise: bool = True,
               plain: bool = False, out: Optional[np.ndarray] = None, per_shot: bool = False,
               engine: Optional[str] = None, keep_xz: bool = False) -> np.ndarray:
        """Records of shots [shot0, shot0 + shots) as a (shots, records) uint8
        array, value | deterministic << 7 -- the fast path without Python objects.

        ``engine`` picks the batched engine: None (by shot count and d),
        "trace" (d = 2: one x / z pass, one lane per shot), "group" (32-shot
        groups), "per_shot" (one warp per shot; same as ``per_shot=True``),
        "tuned" (the route the autotuner timed fastest for this program's
        class of d, n and shots; the first call of a class times them).

        ``keep_xz`` (d = 2 trace engine): the first call keeps the program's
        x / z trace on the device and later calls with ``keep_xz=True`` replay
        it without the x / z pass; it depends on the program alone, so a
        sampling loop over fresh seeds or shot ranges gets the same records
        as without it."""
        dp = self.compile(noise)
        s = self._seed(seed)
        if out is None:
            out = np.empty((int(shots), dp.num_records), dtype=np.uint8)
        flags = (_lib.FLAG_PLAIN if plain else 0) | (_lib.FLAG_PER_SHOT if per_shot else 0)
        flags |= _lib.FLAG_REUSE_XZ if keep_xz else 0
        if engine == "tuned":
            from .autotune import default_tuner
            if shots > 0:
                flags |= default_tuner(self.context).flags_for_program(dp, int(shots), noise)
        else:
            flags |= _lib.engine_flags(engine)
        if shots > 0 and dp.num_records > 0:
            rc = self.context.lib.sdim_run(self.context.ptr, dp.ptr, s, int(shot0), int(shots),
                                           out.ctypes.data, flags)
            _lib.check(rc, self.context.ptr, "simulate")
        elif shots > 0:
            rc = self.context.lib.sdim_run(self.context.ptr, dp.ptr, s, int(shot0), int(shots), None, flags)
            _lib.check(rc, self.context.ptr, "simulate")
        self._last = (s, int(shot0) + int(shots) - 1, noise)
        return out

    def _check_frame_noise_params(self):
        """The frame route reads ``params['noise_channel']`` and
        ``params['prob']`` of every N1 and raises KeyError without them
        (sdim/program.py:486, 502)."""
        for circ in self.circuits:
            for ins in circ.operations:
                if ins.gate_id == 17:
                    params = ins.params if ins.params is not None else {}
                    for key in ("noise_channel", "prob"):
                        if key not in params:
                            raise KeyError(key)

    def sample_frames(self, shots: int, seed: Optional[int] = None, out: Optional[np.ndarray] = None,
                      noise: bool = True) -> np.ndarray:
        """Records of the reference's multi-shot route as a (shots, records)
        uint8 array (value | deterministic << 7): row 0 is the noiseless
        tableau shot 0, rows 1 .. shots-1 are Pauli-frame shots
        (sdim/program.py:45-165, 244-265); ``noise=False`` leaves N1 out of
        the frames too."""
        ref = self.compile(False)
        dp = self.compile(noise)
        s = self._seed(seed)
        if out is None:
            out = np.empty((int(shots), dp.num_records), dtype=np.uint8)
        if shots > 0:
            rc = self.context.lib.sdim_frame_run(self.context.ptr, dp.ptr, ref.ptr, s, int(shots),
                                                 out.ctypes.data if dp.num_records else None, 0)
            _lib.check(rc, self.context.ptr, "simulate")
        self._last = (s, 0, False)
        return out

    def snapshot(self, seed: int, shot: int = 0, mode: int = _lib.SNAP_EVERY_INSTRUCTION, noise: bool = True,
                 per_shot: bool = False):
        """Tableau exports (int8, reference block order) and the shot's records.

        ``per_shot`` selects the one-warp-per-shot engine; by default the
        batched engine of the program (the shot-group engine for d = 2) runs."""
        dp = self.compile(noise)
        n = self.num_qudits
        tb = 4 * n * n + 2 * n
        count = {_lib.SNAP_EVERY_INSTRUCTION: dp.num_instructions,
                 _lib.SNAP_AT_MEASUREMENT: dp.num_records, _lib.SNAP_FINAL: 1}[mode]
        buf = np.empty((max(count, 1), tb), dtype=np.int8)
        rec = np.empty(max(dp.num_records, 1), dtype=np.uint8)
        rc = self.context.lib.sdim_snapshot(self.context.ptr, dp.ptr, int(seed) & 0xFFFFFFFFFFFFFFFF, int(shot),
                                            int(mode), buf.ctypes.data, rec.ctypes.data,
                                            _lib.FLAG_PER_SHOT if per_shot else 0)
        _lib.check(rc, self.context.ptr, "snapshot")
        return buf[:count], rec[:dp.num_records]

    # ------------------------------------------------------------------
    def simulate(self, shots: int = 1, show_measurement: bool = False, record_tableau: bool = False,
                 force_tableau: bool = False, verbose: bool = False, show_gate: bool = False,
                 exact: bool = False, options: Optional[SimulationOptions] = None, *,
                 seed: Optional[int] = None, noise: bool = True, plain: bool = False):
        if options is None:
            options = SimulationOptions(shots, show_measurement, record_tableau, force_tableau, verbose,
                                        show_gate, exact)
        shots = int(options.shots)
        s = self._seed(seed)
        if self._applied:
            self._applied = []
            self._cache = {}
        frame = shots > 1 and not options.record_tableau and not options.force_tableau and not plain
        if frame:
            # the reference's frame route (sdim/program.py:244-265); verbose and
            # show_gate cover its tableau shot only, which has no noise
            self._check_frame_noise_params()
            dp = self.compile(noise)
            records = self.sample_frames(shots, seed=s, noise=noise)
            shown, shown_noise = 1, False
        else:
            dp = self.compile(noise)
            records = self.sample(shots, seed=s, noise=noise, plain=plain)
            shown, shown_noise = shots, noise
        enc = dp.enc
        nested = records_to_nested(records, enc, self.num_qudits)
        if options.record_tableau or options.verbose:
            n, d = self.num_qudits, self.dimension
            for shot in range(shown):
                if options.record_tableau:
                    snaps, _ = self.snapshot(s, shot, _lib.SNAP_AT_MEASUREMENT, shown_noise)
                    for j in range(enc.num_records):
                        q, r = int(enc.meas_qudit[j]), int(enc.meas_round[j])
                        nested[q][r][shot].stabilizer_tableau = ExtendedTableau.from_export(snaps[j], n, d)
                if options.verbose:
                    snaps, _ = self.snapshot(s, shot, _lib.SNAP_EVERY_INSTRUCTION, shown_noise)
                    print("Initial state")
                    ExtendedTableau(n, d).print_tableau()
                    print("\n")
                    for t in range(enc.num_instructions):
                        self._show_gate(t, enc) if options.show_gate else None
                        ExtendedTableau.from_export(snaps[t], n, d).print_tableau()
                        print("\n")
        elif options.show_gate:
            for _ in range(shown):
                for t in range(enc.num_instructions):
                    self._show_gate(t, enc)
        self.measurement_results = nested
        self._last = (s, 0, False) if frame else (s, shots - 1, noise)
        if frame and not nested[0]:
            # sdim/program.py:398-399: the route needs a measurement on qudit 0
            raise ValueError("Empty or invalid measurement results format")
        if options.show_measurement:
            self.print_measurements()
        if shots == 1:
            return flatten_single_shot(nested)
        return nested

    @staticmethod
    def _show_gate(t: int, enc: EncodedProgram):
        from .gatedata import GateData
        gid, q, tgt, _ = (int(v) for v in enc.ops[t])
        name = GateData().get_gate_name(gid)
        info = tgt if tgt >= 0 else ""
        label = "Time step" if t < enc.num_instructions - 1 else "Final step"
        print(label, t, "\t", name, q, info)

    # ------------------------------------------------------------------
    def apply_gate(self, instruc) -> Optional[MeasurementResult]:
        """Applies one instruction to the current stabilizer tableau, as
        sdim/program.py:367-385 does: the tableau after the last simulated
        shot (the initial tableau before any), changed by every instruction
        applied since.  Returns the MeasurementResult of M, M_X and RESET,
        else None.

        There is no host tableau here: the current state is the last shot
        replayed on the GPU (same seed and shot index, so the same outcomes)
        with the applied instructions appended, and its outcome stream
        continues at the next measurement ordinal.  Each call replays the
        whole program, so it is meant for stepping, not for throughput.
        ``simulate`` starts afresh and drops the applied instructions."""
        gid = getattr(instruc, "gate_id", None)
        if gid is None or not 0 <= int(gid) <= 17:
            raise ValueError("Invalid gate value")
        q = int(instruc.qudit_index)
        t = instruc.target_index
        if not 0 <= q < self.num_qudits or (t is not None and not 0 <= int(t) < self.num_qudits):
            raise IndexError("qudit index out of range")
        if self._last is None:
            self._last = (self._seed(None), 0, True)
        # sdim/tableau/tableau_gates.py:331-346: applied alone, RESET only
        # measures (the shot loop applies the X corrections), and N1 is the
        # identity (sdim/program.py:31)
        if int(gid) in (16, 17):
            from .circuit import CircuitInstruction
            instruc = CircuitInstruction(GateData(self.dimension), "M" if int(gid) == 16 else "I", q)
        self._applied.append(instruc)
        self._cache = {}
        if int(gid) not in (14, 15, 16):
            return None
        s, shot, noise = self._last
        dp = self.compile(noise)
        _, rec = self.snapshot(s, max(shot, 0), _lib.SNAP_FINAL, noise)
        v = int(rec[dp.num_records - 1])
        return MeasurementResult(q, bool(v >> 7), v & 0x7F)

    @property
    def stabilizer_tableau(self) -> ExtendedTableau:
        """Final tableau of the last simulated shot (initial state before any run)."""
        if self._last is None and not self._applied:
            return ExtendedTableau(self.num_qudits, self.dimension)
        s, shot, noise = self._last
        snaps, _ = self.snapshot(s, max(shot, 0), _lib.SNAP_FINAL, noise)
        return ExtendedTableau.from_export(snaps[0], self.num_qudits, self.dimension)

    @property
    def initial_tableau(self) -> ExtendedTableau:
        return ExtendedTableau(self.num_qudits, self.dimension)

    def append_circuit(self, circuit: Circuit):
        """Same bookkeeping as sdim/program.py:528-545; the tableau keeps the
        qudit count of the first circuit."""
        if self.circuits[-1].num_qudits < circuit.num_qudits:
            self.circuits[-1].num_qudits = circuit.num_qudits
        else:
            circuit.num_qudits = self.circuits[-1].num_qudits
        if self.circuits[-1].dimension != circuit.dimension:
            raise ValueError("Circuits must have the same dimension")
        self.circuits.append(circuit)
        self._cache = {}

    def print_measurements(self):
        shot_count = 0
        for per_qudit in self.measurement_results:
            for group in per_qudit:
                shot_count = max(shot_count, len(group))
        if shot_count == 0:
            print("No measurements recorded.")
            return
        for shot_index in range(shot_count):
            if shot_count > 1:
                print(f"Shot {shot_index + 1}:")
            for per_qudit in self.measurement_results:
                for number, shots_list in enumerate(per_qudit):
                    if shot_count > 1:
                        print(f"{shots_list[shot_index]} during measurement {number}")
                    else:
                        print(shots_list[0])
            if shot_count > 1:
                print()

    def __str__(self) -> str:
        return "\n".join(str(c) for c in self.circuits)

    def __deepcopy__(self, memo):
        other = Program.__new__(Program)
        other.__dict__.update({k: copy.deepcopy(v, memo) for k, v in self.__dict__.items()
                               if k not in ("_ctx", "_cache")})
        other._ctx = self._ctx
        other._cache = {}
        return other
