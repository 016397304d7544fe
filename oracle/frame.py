"""Pauli-frame sampler restated in NumPy -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker.

It restates the reference's multi-shot route (``Program.simulate(shots > 1)``
without ``record_tableau`` / ``force_tableau``, sdim/program.py:244-265):

* shot 0 is one tableau shot with every N1 as the identity
  (sdim/program.py:246-247, 31); here it comes from the C oracle with the
  noise off;
* shots 1 .. S-1 propagate a Pauli frame (x, z residues per qudit and shot)
  through the instruction list (``simulate_frame``, sdim/program.py:45-165):
  - x starts at 0 and z at a uniform residue per qudit and shot (:63-64);
  - X / X_INV / Z / Z_INV leave the frame alone (:82-89); H, H_INV, P,
    P_INV, CNOT, CNOT_INV, CZ, CZ_INV and SWAP act on (x, z) as at :90-120;
  - M_X first maps (x, z) to (z, -x) (:128-131); M and M_X record
    ``(ref + x_q) mod d`` with the reference shot's deterministic flag
    (:133-140), then draw a fresh z_q (:144);
  - RESET records the reference shot's value unchanged, sets x_q = 0 and
    draws a fresh z_q (:146-157);
  - N1 adds its (a, b) sample to (x_q, z_q) (:159-162), with (a, b) drawn
    per shot as ``_build_ir`` does (sdim/program.py:484-509).

Random draws (the reference's ``np.random`` calls) come from the Philox
stream of ``philox.py``:

* frame draws, domain 3: event e of a shot is the initial z of qudit e for
  e < n and the z drawn after measurement ordinal k (M, M_X and RESET in
  program order) for e = n + k; word e & 3 of the block with counter ordinal
  e >> 2 gives the residue ``(w * d) >> 32``;
* N1 samples: ``philox.noise_pauli`` (domains 1 and 2), keyed by the shot
  index and the N1 ordinal, as in the tableau route;
* the reference shot's outcomes: domain 0 at shot 0.

Shot s of the frame route (s >= 1) uses stream shot index s.
"""
from __future__ import annotations

import numpy as np

from . import philox

DOMAIN_FRAME = 3
CHANNEL_NAMES = {1: "d", 2: "f", 3: "p"}


def frame_residues(seed: int, shots, event: int, d: int) -> np.ndarray:
    """Residues in [0, d) of frame event ``event`` for the given shot indices."""
    block = philox.stream_words(seed, shots, int(event) >> 2, DOMAIN_FRAME)
    return philox.residue(block[int(event) & 3], d)


def simulate_frame(prog, ref_records: np.ndarray, seed: int, nshots: int) -> np.ndarray:
    """Records of frame shots 1 .. nshots-1 of ``prog`` (an ``OracleProgram``),
    given the reference shot's records (value | deterministic << 7, one byte
    per measurement in program order).  Returns (nshots - 1, nmeas) uint8."""
    n, d = prog.n, prog.d
    S = int(nshots) - 1
    out = np.zeros((max(S, 0), prog.nmeas), dtype=np.uint8)
    if S <= 0:
        return out
    shots = np.arange(1, nshots, dtype=np.uint64)
    x = np.zeros((n, S), dtype=np.int64)
    z = np.stack([frame_residues(seed, shots, q, d) for q in range(n)]) if n else np.zeros((0, S), np.int64)
    ref = np.asarray(ref_records, dtype=np.uint8).reshape(-1)
    k = 0  # measurement ordinal
    j = 0  # N1 ordinal
    for row, thr in zip(prog.ops, prog.thr):
        gid, q, t, ch = int(row[0]), int(row[1]), int(row[2]), int(row[4])
        if gid == 5:  # H
            x[q], z[q] = (-z[q]) % d, x[q].copy()
        elif gid == 6:  # H_INV
            x[q], z[q] = z[q].copy(), (-x[q]) % d
        elif gid == 7:  # P
            z[q] = (z[q] + x[q]) % d
        elif gid == 8:  # P_INV
            z[q] = (z[q] - x[q]) % d
        elif gid == 9:  # CNOT
            x[t] = (x[t] + x[q]) % d
            z[q] = (z[q] - z[t]) % d
        elif gid == 10:  # CNOT_INV
            x[t] = (x[t] - x[q]) % d
            z[q] = (z[q] + z[t]) % d
        elif gid == 11:  # CZ
            z[t] = (z[t] + x[q]) % d
            z[q] = (z[q] + x[t]) % d
        elif gid == 12:  # CZ_INV
            z[t] = (z[t] - x[q]) % d
            z[q] = (z[q] - x[t]) % d
        elif gid == 13:  # SWAP
            x[[q, t]] = x[[t, q]]
            z[[q, t]] = z[[t, q]]
        elif gid in (14, 15):
            if gid == 15:
                x[q], z[q] = z[q].copy(), (-x[q]) % d
            value, det = int(ref[k] & 0x7F), int(ref[k] & 0x80)
            out[:, k] = (((value + x[q]) % d) | det).astype(np.uint8)
            z[q] = frame_residues(seed, shots, n + k, d)
            k += 1
        elif gid == 16:
            out[:, k] = ref[k]
            x[q] = 0
            z[q] = frame_residues(seed, shots, n + k, d)
            k += 1
        elif gid == 17:
            a, b = philox.noise_pauli(seed, shots, j, d, CHANNEL_NAMES[ch], int(thr))
            x[q] = (x[q] + a) % d
            z[q] = (z[q] + b) % d
            j += 1
        # I, X, X_INV, Z, Z_INV: the frame is unchanged
    return out


def simulate(prog, seed: int, nshots: int, threads: int = 0) -> np.ndarray:
    """The whole route: row 0 is the noiseless tableau shot 0 (C oracle),
    rows 1 .. nshots-1 the frame shots.  Returns (nshots, nmeas) uint8."""
    from . import simulate as tableau_simulate

    ref = tableau_simulate(prog, seed, 0, 1, noise=False, threads=threads or 1)["records"]
    rows = [ref] + ([simulate_frame(prog, ref[0], seed, nshots)] if nshots > 1 else [])
    return np.concatenate(rows, axis=0)[:nshots]
