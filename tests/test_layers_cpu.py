"""CPU: the layered instruction stream the odd-d cluster x / z pass walks
(abi.cu: append_layers_u8), read through the host-only sdim_program_words.
Against the program's own device words: the same measurements, RESETs and
N1 in the same order; between two of them the same gates, with every qudit's
gates in their original order; groups of 2 to 8 gates on pairwise disjoint
qudits, none across a 512-word window; each run of gates behind an OP_RUN
header that counts its words."""
import ctypes as C

import numpy as np
import pytest

from sdim_gb300 import _lib, workloads
from sdim_gb300.encode import encode_program

OP_NOP, OP_CNOT, OP_CNOT_INV, OP_GROUP, OP_RUN = 0, 9, 10, 21, 22
GATES = set(range(1, 11))
WINDOW = 512


def words(enc, layered):
    lib = _lib.load()
    ops = np.ascontiguousarray(enc.ops)
    probs = np.ascontiguousarray(enc.probs)
    count = C.c_int64()
    args = (ops.ctypes.data_as(C.c_void_p), int(ops.shape[0]), probs.ctypes.data_as(C.c_void_p) if probs.size else None,
            int(enc.n), int(enc.d), int(layered))
    assert lib.sdim_program_words(*args, None, 0, C.byref(count)) in (_lib.SDIM_OK, _lib.SDIM_ENOMEM)
    out = np.zeros(2 * max(count.value, 1), dtype=np.uint32)
    rc = lib.sdim_program_words(*args, out.ctypes.data_as(C.c_void_p), count.value, C.byref(count))
    assert rc == _lib.SDIM_OK
    return out[:2 * count.value].reshape(-1, 2)


def touched(w):
    op, q = int(w[0]) & 0x7F, int(w[0]) >> 8
    return (q, int(w[1])) if op in (OP_CNOT, OP_CNOT_INV) else (q,)


def segments(ws):
    """(gate words, the non-gate word that ends the segment or None) in order."""
    segs, cur = [], []
    for w in ws:
        op = int(w[0]) & 0x7F
        if op == OP_NOP:
            continue
        if op in GATES:
            cur.append((int(w[0]) & ~0x80, int(w[1])))
        else:
            segs.append((cur, (int(w[0]), int(w[1]))))
            cur = []
    segs.append((cur, None))
    return segs


def check_layered(plain, lay):
    # headers: runs and groups
    i, body = 0, []
    while i < len(lay):
        op = int(lay[i][0]) & 0x7F
        if op == OP_RUN:
            end = i + 1 + int(lay[i][1])
            assert end <= len(lay)
            for w in lay[i + 1:end]:
                assert (int(w[0]) & 0x7F) in GATES | {OP_GROUP, OP_NOP}, "a run holds gates, groups and padding only"
            assert end == len(lay) or (int(lay[end][0]) & 0x7F) not in GATES | {OP_GROUP}, "the run ends at a non-gate"
            i += 1
            continue
        if op == OP_GROUP:
            cnt = int(lay[i][1])
            assert 2 <= cnt <= 8
            assert i // WINDOW == (i + cnt) // WINDOW, "a group straddles an instruction window"
            members = lay[i + 1:i + 1 + cnt]
            qs = [q for w in members for q in touched(w)]
            assert all((int(w[0]) & 0x7F) in GATES for w in members)
            assert len(qs) == len(set(qs)), "a group's gates share a qudit"
            body.extend(members)
            i += 1 + cnt
            continue
        body.append(lay[i])
        i += 1
    a, b = segments(plain), segments(np.array(body).reshape(-1, 2))
    assert len(a) == len(b)
    for (ga, ea), (gb, eb) in zip(a, b):
        assert ea == eb, "measurements, RESETs and N1 keep their order"
        assert sorted(ga) == sorted(gb), "a segment keeps its gates"
        per_q = lambda g: {q: [w for w in g if q in touched(w)] for w in g for q in touched(w)}  # noqa: E731
        assert per_q(ga) == per_q(gb), "every qudit's gates keep their order"


@pytest.mark.parametrize("d", [3, 5, 7, 11])
@pytest.mark.parametrize("n,gates,mr", [(2, 300, 0), (40, 2000, 700), (256, 2560, 256)])
def test_layered_stream_keeps_the_program(n, gates, mr, d):
    spec = workloads.random_hpc(n, d, gates, seed=n + d, mr_every=mr, mr_fraction=0.1)
    enc = encode_program([spec.build()], n, d)
    check_layered(words(enc, 0), words(enc, 1))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_layered_stream_every_gate_and_noise(seed):
    spec = workloads.all_gates_random(9, 5, 1500, seed=seed, noise_probs=(0.0, 0.3, 1.0))
    enc = encode_program([spec.build()], 9, 5)
    check_layered(words(enc, 0), words(enc, 1))


def test_layered_stream_groups_the_oddd5_program():
    """The lone d = 5, n = 256 workload: most gates travel in full groups."""
    spec = workloads.odd_d(5, seed=0)
    enc = encode_program([spec.build()], spec.num_qudits, 5)
    lay = words(enc, 1)
    ops = lay[:, 0] & 0x7F
    grouped = int(lay[ops == OP_GROUP, 1].sum())
    assert grouped >= 0.9 * 2560
    assert (ops == OP_RUN).sum() == 10  # one run per block of 256 gates
    check_layered(words(enc, 0), lay)


def test_program_words_rejects_layered_d2_and_short_buffers():
    spec = workloads.random_hpc(5, 3, 20, seed=1)
    enc = encode_program([spec.build()], 5, 3)
    lib = _lib.load()
    ops = np.ascontiguousarray(enc.ops)
    count = C.c_int64()
    assert lib.sdim_program_words(ops.ctypes.data_as(C.c_void_p), int(ops.shape[0]), None, 5, 2, 1, None, 0,
                                  C.byref(count)) == _lib.SDIM_EINVAL
    assert lib.sdim_program_words(ops.ctypes.data_as(C.c_void_p), int(ops.shape[0]), None, 5, 3, 0, None, 0,
                                  C.byref(count)) == _lib.SDIM_ENOMEM
    assert count.value >= 20
