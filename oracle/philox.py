"""Philox4x32-10 counter-based generator in NumPy (test infrastructure only).

This module is part of the oracle: only the tests, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` use it, as the checker.

Written from the published description in J. K. Salmon, M. A. Moraes,
R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3",
SC'11: a 4x32-bit counter block, a 2x32-bit key, ten rounds of two 32x32->64
multiplies with the round constants below, and a Weyl-sequence key schedule.
The known-answer vectors in ``KAT`` come from the same publication's
reference implementation.

Stream layout used by both the GPU kernels and the oracle
(the reference draws with ``random.choice(range(d))`` at
sdim/tableau/tableau_prime.py:332; the drop-in replaces that draw):

* key     = (seed & 0xffffffff, seed >> 32)
* counter = (ordinal, shot & 0xffffffff, shot >> 32, domain)
* domain 0: measurement outcome, ordinal = index of the measurement among the
  M / M_X / RESET instructions of the program, word 0 gives the residue
  ``(w0 * d) >> 32``;
* domain 1: N1 coins.  For the N1 instruction with ordinal j (its index among
  all N1 instructions of the program) the block with counter ordinal j >> 2
  gives the coin in word j & 3: the Pauli is the identity iff
  ``coin < threshold``;
* domain 2: N1 Pauli choice, drawn only when the coin fires: word 0 of the
  block with counter ordinal j picks the Pauli.
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

DOMAIN_MEASURE = 0
DOMAIN_COIN = 1
DOMAIN_CHOICE = 2

# (counter, key, expected output) from the Random123 known-answer tests.
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10. All inputs broadcast; returns four uint32 arrays."""
    c0 = np.asarray(c0, dtype=np.uint64) & MASK32
    c1 = np.asarray(c1, dtype=np.uint64) & MASK32
    c2 = np.asarray(c2, dtype=np.uint64) & MASK32
    c3 = np.asarray(c3, dtype=np.uint64) & MASK32
    k0 = np.asarray(k0, dtype=np.uint64) & MASK32
    k1 = np.asarray(k1, dtype=np.uint64) & MASK32
    c0, c1, c2, c3, k0, k1 = np.broadcast_arrays(c0, c1, c2, c3, k0, k1)
    c0, c1, c2, c3 = c0.copy(), c1.copy(), c2.copy(), c3.copy()
    k0, k1 = k0.copy(), k1.copy()
    for rnd in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        n0 = hi1 ^ c1 ^ k0
        n1 = lo1
        n2 = hi0 ^ c3 ^ k1
        n3 = lo0
        c0, c1, c2, c3 = n0, n1, n2, n3
        if rnd != 9:
            k0 = (k0 + np.uint64(W0)) & MASK32
            k1 = (k1 + np.uint64(W1)) & MASK32
    return (c0.astype(np.uint32), c1.astype(np.uint32),
            c2.astype(np.uint32), c3.astype(np.uint32))


def stream_words(seed: int, shot, ordinal, domain: int):
    """Philox block for (seed, shot, ordinal, domain); shot/ordinal may be arrays."""
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    shot = np.asarray(shot, dtype=np.uint64)
    return philox4x32_10(ordinal, shot & MASK32, shot >> np.uint64(32), domain,
                         seed & 0xFFFFFFFF, seed >> 32)


def residue(word, d: int):
    """Multiply-shift map of a uint32 word onto [0, d)."""
    return ((np.asarray(word, dtype=np.uint64) * np.uint64(d)) >> np.uint64(32)).astype(np.int64)


def measurement_outcome(seed: int, shot, ordinal: int, d: int):
    """Outcome drawn for a random measurement (domain 0)."""
    w0, _, _, _ = stream_words(seed, shot, ordinal, DOMAIN_MEASURE)
    return residue(w0, d)


def noise_threshold(prob: float) -> int:
    """Integer coin threshold: the Pauli is the identity iff word0 < threshold.

    Returns 2**32 for a channel that never fires and 0 for one that always does.
    """
    t = np.floor((1.0 - float(prob)) * 4294967296.0)
    if t >= 4294967296.0:
        return 1 << 32
    if t <= 0.0:
        return 0
    return int(t)


def noise_pauli(seed: int, shot, ordinal: int, d: int, channel: str, threshold: int):
    """(a, b) exponents of X^a Z^b for one N1 instruction (domain 1).

    Channel semantics follow the frame sampler's draw (sdim/program.py:486-507):
    'd' draws r in [1, d^2) with a = r % d, b = r // d; 'f' draws a in [1, d);
    'p' draws b in [1, d); the draw is replaced by the identity when the coin
    says so.
    """
    block = stream_words(seed, shot, int(ordinal) >> 2, DOMAIN_COIN)
    w0 = np.asarray(block[int(ordinal) & 3], dtype=np.uint64)
    w1 = stream_words(seed, shot, ordinal, DOMAIN_CHOICE)[0]
    fire = w0 >= np.uint64(threshold) if threshold < (1 << 32) else np.zeros_like(w0, dtype=bool)
    if channel == 'd':
        r = 1 + residue(w1, d * d - 1)
        a, b = r % d, r // d
    elif channel == 'f':
        a = 1 + residue(w1, d - 1)
        b = np.zeros_like(a)
    elif channel == 'p':
        b = 1 + residue(w1, d - 1)
        a = np.zeros_like(b)
    else:
        raise ValueError(f"unknown noise channel {channel!r}")
    a = np.where(fire, a, 0)
    b = np.where(fire, b, 0)
    return a.astype(np.int64), b.astype(np.int64)
