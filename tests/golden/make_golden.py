"""Generates the golden fixtures by running the reference sdim itself.

Run in a container that holds the reference source, with its path in
$SDIM_REFERENCE (required; there is no default):

    SDIM_REFERENCE=<path to the sdim source tree> PYTHONDONTWRITEBYTECODE=1 \
        python tests/golden/make_golden.py

It imports sdim from the reference tree (with import-time stand-ins for
numba, cirq and Diophantine from ``_stubs``, none of which the
prime-dimension path calls), never writes into that tree, and drives the
reference's own ``Program.simulate(force_tableau=True)`` with two injections:

* outcomes: ``sdim.tableau.tableau_prime.random`` is replaced by an object
  whose ``choice(seq)`` returns ``seq[(word0 * d) >> 32]`` of the Philox block
  (seed, shot, measurement ordinal, domain 0) -- the only random draw on the
  path (sdim/tableau/tableau_prime.py:332);
* noise: after every N1 instruction the reference's own ``apply_X`` /
  ``apply_Z`` (sdim/tableau/tableau_gates.py:27, 85) are applied a and b
  times, with (a, b) drawn from the Philox block (seed, shot, N1 ordinal,
  domain 1), as its deprecated tableau noise function orders them
  (sdim/tableau/tableau_gates.py:387-391).

Outputs (beside this script): ``cases.json`` (programs, seeds, expected
known answers) and ``arrays.npz`` (records, per-instruction tableaux of the
first shot, final tableaux, record_tableau exports; int8/uint8).

With ``--frames`` it drives the reference's multi-shot route instead
(``run_reference_frames``: the Pauli-frame sampler of sdim/program.py:45-165,
with ``np.random`` answered from the same Philox stream) and writes
``frames.json`` / ``frames.npz``; with ``--chp`` it runs the reference's
.chp reader and writer (sdim/circuit_io.py:6-139) on corner-case texts and
on circuits it writes itself, and writes ``chp.json``.  With ``--stats``
it runs the reference's ``Program.simulate(shots)`` with its own random
number generators (seeded ``random`` and ``np.random``, no injection) on the
circuits of ``stat_cases`` and writes the outcome histograms to
``stats.json``: the counts that the chi-square tests compare runs with
different random streams against.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = os.environ.get("SDIM_REFERENCE", "")


def _setup_paths():
    if not REF or not (Path(REF) / "sdim").is_dir():
        raise SystemExit("set SDIM_REFERENCE to the reference sdim source tree (the directory holding sdim/)")
    sys.dont_write_bytecode = True
    for p in (str(ROOT), REF, str(HERE / "_stubs")):
        if p not in sys.path:
            sys.path.insert(0, p)


_setup_paths()

from oracle import philox  # noqa: E402
from sdim_gb300 import workloads as W  # noqa: E402

MEAS = (14, 15, 16)


def _reduce(tab, n, d):
    order = 2 * d if d % 2 == 0 else d
    parts = [tab.x_block % d, tab.z_block % d, tab.phase_vector % order,
             tab.destab_x_block % d, tab.destab_z_block % d, tab.destab_phase_vector % order]
    return np.concatenate([np.asarray(p, dtype=np.int64).ravel() for p in parts]).astype(np.int8)


def run_reference(specs, seed, shot0, nshots, noise=True, snapshots=False, final=False,
                  record_tableau=False, want_nested=False):
    """Runs the reference on the programs in ``specs`` (list of CircuitSpec,
    appended in order) and returns records and tableaux."""
    import sdim.tableau.tableau_prime as tp
    from sdim.circuit import Circuit
    from sdim.program import Program
    from sdim.tableau.tableau_gates import apply_X, apply_Z

    n, d = specs[0].num_qudits, specs[0].dimension
    circuits = [s.build(Circuit) for s in specs]
    prog = Program(circuits[0])
    for c in circuits[1:]:
        prog.append_circuit(c)
    nops = sum(len(c.operations) for c in circuits)

    class Shim:
        shot = 0
        mord = 0

        def choice(self, seq):
            m = int(philox.measurement_outcome(seed, self.shot, self.mord, len(seq)))
            return seq[m]

    shim = Shim()
    tp.random = shim
    st = {"idx": 0, "mord": 0, "nord": 0, "rec": [], "snaps": [], "objs": []}
    orig = prog.apply_gate

    def wrapped(ins):
        if snapshots and st["idx"] > 0:
            st["snaps"].append(_reduce(prog.stabilizer_tableau, n, d))
        if ins.gate_id in MEAS:
            shim.mord = st["mord"]
            st["mord"] += 1
        res = orig(ins)
        if ins.gate_id == 17:
            if noise:
                params = ins.params or {}
                ch = params.get("noise_channel", params.get("channel", "d"))
                thr = philox.noise_threshold(float(params.get("prob", 0.01)))
                a, b = philox.noise_pauli(seed, shim.shot, st["nord"], d, ch, thr)
                for _ in range(int(a)):
                    apply_X(prog.stabilizer_tableau, ins.qudit_index, None)
                for _ in range(int(b)):
                    apply_Z(prog.stabilizer_tableau, ins.qudit_index, None)
            st["nord"] += 1
        if res is not None:
            st["rec"].append(int(res.measurement_value) | (0x80 if res.deterministic else 0))
            st["objs"].append(res)
        st["idx"] += 1
        return res

    prog.apply_gate = wrapped
    records, finals, snaps, rts, nested = [], [], None, [], None
    for s in range(nshots):
        shim.shot = shot0 + s
        st.update(idx=0, mord=0, nord=0, rec=[], snaps=[], objs=[])
        out = prog.simulate(shots=1, force_tableau=True, record_tableau=record_tableau)
        if snapshots and s == 0:
            st["snaps"].append(_reduce(prog.stabilizer_tableau, n, d))
            snaps = np.stack(st["snaps"]) if st["snaps"] else np.zeros((0, 4 * n * n + 2 * n), np.int8)
            assert snaps.shape[0] == nops
        if final:
            finals.append(_reduce(prog.stabilizer_tableau, n, d))
        if record_tableau and s == 0:
            for r in st["objs"]:  # program order; set by the reference after apply_gate
                rts.append(_reduce(r.stabilizer_tableau, n, d))
        if want_nested and s == 0:
            nested = [[(r.qudit_index, bool(r.deterministic), int(r.measurement_value)) for r in out]]
        records.append(st["rec"])
    rec = np.asarray(records, dtype=np.uint8).reshape(nshots, -1)
    return {"records": rec, "snapshots": snaps, "final": np.stack(finals) if finals else None,
            "record_tableau": np.stack(rts) if rts else None, "nested": nested}


def run_reference_frames(specs, seed, nshots):
    """Runs the reference's multi-shot route, ``Program.simulate(nshots)``
    (sdim/program.py:244-265), with its draws taken from the Philox stream:

    * shot 0's outcomes: ``tableau_prime.random`` as in ``run_reference``
      (shot 0, measurement ordinal); N1 stays the identity there, as the
      reference's tableau shot has it;
    * ``np.random`` of sdim/program.py (``_build_ir`` and ``simulate_frame``)
      is replaced by an object that answers, in call order,
      ``randint(1, hi, S)`` of N1 ordinal j with ``1 + residue(word 0 of the
      domain-2 block j, hi - 1)``, ``uniform(0, 1, S)`` of N1 ordinal j with
      1.0 where the domain-1 coin fires and 0.0 elsewhere (so the
      reference's ``roll < 1 - prob`` test keeps exactly the fired shots),
      ``randint(0, d, (n, S))`` with the frame events 0 .. n-1 and the k-th
      ``randint(0, d, S)`` with frame event n + k (oracle/frame.py);
      frame shot s (1 .. S) uses stream shot index s.
    Returns (nshots, records) uint8: value | deterministic << 7, program order.
    """
    import sdim.program as sp
    import sdim.tableau.tableau_prime as tp
    from sdim.circuit import Circuit
    from sdim.program import Program
    from oracle import frame as oframe

    n, d = specs[0].num_qudits, specs[0].dimension
    circuits = [s.build(Circuit) for s in specs]
    prog = Program(circuits[0])
    for c in circuits[1:]:
        prog.append_circuit(c)
    instrs = [ins for c in circuits for ins in c.operations]
    thresholds = [philox.noise_threshold(float(ins.params["prob"])) for ins in instrs if ins.gate_id == 17]
    S = nshots - 1
    shots = np.arange(1, nshots, dtype=np.uint64)

    class Outcomes:
        mord = 0

        def choice(self, seq):
            m = int(philox.measurement_outcome(seed, 0, self.mord, len(seq)))
            return seq[m]

    class Draws:
        choice_j = coin_j = frame_k = 0

        def randint(self, low, high=None, size=None):
            if low == 1:
                j = self.choice_j
                self.choice_j += 1
                w1 = philox.stream_words(seed, shots, j, philox.DOMAIN_CHOICE)[0]
                return (1 + philox.residue(w1, int(high) - 1)).astype(np.int64)
            assert low == 0 and high == d
            if isinstance(size, tuple):
                return np.stack([oframe.frame_residues(seed, shots, q, d) for q in range(size[0])])
            k = self.frame_k
            self.frame_k += 1
            return oframe.frame_residues(seed, shots, n + k, d)

        def uniform(self, low, high, size=None):
            j = self.coin_j
            self.coin_j += 1
            thr = thresholds[j]
            coin = philox.stream_words(seed, shots, j >> 2, philox.DOMAIN_COIN)[j & 3].astype(np.uint64)
            fire = coin >= np.uint64(thr) if thr < (1 << 32) else np.zeros(S, dtype=bool)
            return np.where(fire, 1.0, 0.0)

    class NumpyWithDraws:
        def __init__(self, real, draws):
            self._real = real
            self.random = draws

        def __getattr__(self, name):
            return getattr(self._real, name)

    outcomes = Outcomes()
    tp.random = outcomes
    orig = prog.apply_gate
    st = {"mord": 0}

    def wrapped(ins):
        if ins.gate_id in MEAS:
            outcomes.mord = st["mord"]
            st["mord"] += 1
        return orig(ins)

    prog.apply_gate = wrapped
    real_np = sp.np
    sp.np = NumpyWithDraws(real_np, Draws())
    try:
        nested = prog.simulate(shots=nshots)
    finally:
        sp.np = real_np
    counts = [0] * n
    cols = []
    for ins in instrs:
        if ins.gate_id in MEAS:
            q = ins.qudit_index
            group = nested[q][counts[q]]
            counts[q] += 1
            cols.append([int(r.measurement_value) | (0x80 if r.deterministic else 0) for r in group])
    return np.asarray(cols, dtype=np.uint8).T.reshape(nshots, len(cols))


def frame_cases():
    out = []
    for s, _ in kat_cases()[:3]:
        out.append((s, 6))
    k = 0
    for d in (2, 3, 5, 7):
        for n in (2, 3, 5):
            out.append((W.all_gates_random(n, d, 60 if n == 2 else 120, seed=3000 + k,
                                           name=f"frame_rand_d{d}_n{n}"), 24))
            k += 1
    for d in (2, 5):
        ops = [("H", 0, None, {}), ("CZ", 1, 1, {}), ("CZ_INV", 0, 0, {}), ("SWAP", 1, 1, {}),
               ("CNOT", 0, 0, {}), ("N1", 0, None, {"prob": 0.5, "noise_channel": "d"}), ("P", 1, None, {}),
               ("M_X", 1, None, {}), ("M", 0, None, {}), ("RESET", 1, None, {}), ("M", 1, None, {})]
        out.append((W.CircuitSpec(2, d, ops, f"frame_aliased_d{d}"), 24))
    out.append((W.surface_memory(3, 3, prob=0.02), 64))
    out[-1][0].name = "frame_surface_L3_r3"
    out.append((W.random_hpc(12, 5, 120, seed=5, weights=(0.25, 0.25, 0.5), mr_every=12, mr_fraction=0.25,
                             name="frame_oddd_d5"), 32))
    return out


def stat_cases():
    """Circuits of the statistical tests, each with its shot count.  The
    first five restate the reference's own statistical tests
    (tests/test_noise_and_io.py:101-186, tests/test_reset.py:11-37) at fixed
    dimensions and probabilities; the last two correlate several records
    (a GHZ state under depolarizing noise; a mid-circuit MEASURE + RESET)."""
    def c(n, d, ops, name):
        return W.CircuitSpec(n, d, ops, name)

    nz = lambda q, p, ch: ("N1", q, None, {"prob": p, "noise_channel": ch})  # noqa: E731
    m = lambda q: ("M", q, None, {})  # noqa: E731
    out = [
        (c(1, 3, [nz(0, 0.55, "d"), m(0)], "stat_depolarizing_d3"), 100_000),
        (c(1, 7, [nz(0, 0.8, "d"), m(0)], "stat_depolarizing_d7"), 100_000),
        (c(1, 5, [nz(0, 0.37, "f"), m(0)], "stat_flip_d5"), 100_000),
        (c(1, 11, [("H", 0, None, {}), nz(0, 0.42, "p"), ("H_INV", 0, None, {}), m(0)], "stat_phase_d11"), 100_000),
        (c(1, 5, [nz(0, 24 / 25, "d"), ("RESET", 0, None, {})] + [("X", 0, None, {})] * 3 + [m(0)],
           "stat_reset_skip_d5"), 100_000),
        (c(3, 3, [("H", 0, None, {}), ("CNOT", 0, 1, {}), ("CNOT", 1, 2, {})]
           + [nz(q, 0.3, "d") for q in range(3)] + [m(q) for q in range(3)], "stat_ghz_d3"), 100_000),
        (c(3, 2, [("H", 0, None, {}), ("CNOT", 0, 1, {}), nz(1, 0.2, "d"), m(1), ("RESET", 1, None, {}),
                  ("CNOT", 0, 1, {}), ("CNOT", 1, 2, {}), nz(2, 0.1, "f"), m(0), m(1), m(2)],
           "stat_midcircuit_reset_d2"), 100_000),
    ]
    return out


def main_stats():
    import random as pyrandom

    from sdim.circuit import Circuit
    from sdim.program import Program

    cases = []
    for k, (spec_, shots) in enumerate(stat_cases()):
        seed = 1000 + k
        pyrandom.seed(seed)
        np.random.seed(seed)
        nested = Program(spec_.build(Circuit)).simulate(shots=shots)
        counts = [0] * spec_.num_qudits
        cols, kinds = [], []
        for op in spec_.ops:
            if op[0] in ("M", "RESET"):
                q = op[1]
                cols.append([int(r.measurement_value) for r in nested[q][counts[q]]])
                kinds.append(op[0])
                counts[q] += 1
        vals = np.asarray(cols, dtype=np.int64).T
        d = spec_.dimension
        # the reference's frame route gives every shot shot 0's value at a
        # RESET (sdim/program.py:146-157), so RESET records are left out of
        # the joint histogram: it is over the M records, first record in the
        # lowest digit
        keep = [j for j, k in enumerate(kinds) if k == "M"]
        index = (vals[:, keep] * (d ** np.arange(len(keep)))).sum(axis=1)
        hist = np.bincount(index, minlength=d ** len(keep))
        resets = [sorted(set(vals[:, j].tolist())) for j, k in enumerate(kinds) if k == "RESET"]
        cases.append({"name": spec_.name, "shots": shots, "reference_seed": seed, "circuit": spec_.to_json(),
                      "record_kinds": kinds, "histogram": hist.tolist(), "reset_values": resets})
        print(spec_.name, hist[:8].tolist(), resets, flush=True)
    (HERE / "stats.json").write_text(json.dumps({"cases": cases}, indent=0))
    print("wrote", len(cases), "statistical cases")


def main_frames():
    cases, arrays = [], {}
    for s, nshots in frame_cases():
        seed = 17
        rec = run_reference_frames([s], seed, nshots)
        arrays[f"{s.name}__records"] = rec
        cases.append({"name": s.name, "seed": seed, "nshots": nshots, "circuits": [s.to_json()]})
        print(s.name, rec.shape, flush=True)
    (HERE / "frames.json").write_text(json.dumps({"cases": cases}, indent=0))
    np.savez_compressed(HERE / "frames.npz", **arrays)
    print("wrote", len(cases), "frame-route cases")


CHP_TEXTS = {
    # hand-written texts for the reader's corner cases
    "chp_comment_and_upper_d": "two lines\nof comment\n#\nD 5\nh 0\ncx 0 3\n\nmr 2\nN1 1 prob=0.25 noise_channel=p\n"
                               "M 3\n",
    "chp_default_dimension": "#\nH 0\nCNOT 0 1\nMEASURE 1\nnoise1 0 channel=f prob=1e-3\nM 0\n",
    "chp_crlf_and_tabs": "c\r\n#\r\nd 3\r\n\tS 1\r\nSUM  1\t2\r\nM_X 2\r\nMZ 1\r\n",
    "chp_two_qudit_params_dropped": "#\nd 7\nN1 0 1 prob=0.5 noise_channel=p\nCZ 1 0 x=1\nM 1\n",
    "chp_junk_tokens": "#\nd 2\nH 0 junk\nCX 0 1 -3 more\nM 1 tail=end\n",
}
CHP_ERRORS = {
    "chp_err_no_hash": "H 0\nM 0\n",
    "chp_err_param": "#\nN1 0 prob=0.1=0.2\n",
    "chp_err_three_indices": "#\nCNOT 0 1 2\n",
    "chp_err_unknown_gate": "#\nFOO 0\n",
    "chp_err_no_index": "#\nH\nM 0\n",
}


def main_chp():
    """Fixtures of the reference's .chp reader and writer (sdim/circuit_io.py:6-139)."""
    import tempfile
    from sdim.circuit import Circuit
    from sdim.circuit_io import read_circuit, write_circuit

    def parsed(circ):
        return {"n": circ.num_qudits, "d": circ.dimension,
                "ops": [[ins.gate_name, int(ins.gate_id), int(ins.qudit_index),
                         -1 if ins.target_index is None else int(ins.target_index),
                         None if ins.params is None else {k: str(v) for k, v in ins.params.items()}]
                        for ins in circ.operations]}

    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, text in CHP_TEXTS.items():
            path = os.path.join(tmp, name + ".chp")
            Path(path).write_text(text)
            cases.append({"name": name, "text": text, "parsed": parsed(read_circuit(path))})
        for name, text in CHP_ERRORS.items():
            path = os.path.join(tmp, name + ".chp")
            Path(path).write_text(text)
            try:
                read_circuit(path)
                raise AssertionError(name + " parsed")
            except Exception as e:  # the type the reference raises
                cases.append({"name": name, "text": text, "error": type(e).__name__})
        for k, (n, d, nops) in enumerate([(3, 2, 40), (6, 3, 90), (4, 5, 70), (9, 7, 150)]):
            spec = W.all_gates_random(n, d, nops, seed=7000 + k, name=f"chp_written_d{d}")
            circ = spec.build(Circuit)
            comment = "" if k % 2 else f"written by the reference, case {k}"
            path = write_circuit(circ, output_file=spec.name + ".chp", comment=comment, directory=tmp)
            text = Path(path).read_text()
            cases.append({"name": spec.name, "written_from": spec.to_json(), "comment": comment, "text": text,
                          "parsed": parsed(read_circuit(path))})
    (HERE / "chp.json").write_text(json.dumps({"cases": cases}, indent=0))
    print("wrote", len(cases), ".chp cases")


def _worker(args):
    specs_json, seed, shot0, nshots, noise = args
    _setup_paths()
    specs = [W.CircuitSpec.from_json(s) for s in specs_json]
    return run_reference(specs, seed, shot0, nshots, noise=noise)["records"]


def run_parallel(specs, seed, nshots, noise=True, procs=8, chunk=32):
    jobs = [([s.to_json() for s in specs], seed, a, min(chunk, nshots - a), noise)
            for a in range(0, nshots, chunk)]
    with mp.get_context("spawn").Pool(procs) as pool:
        parts = pool.map(_worker, jobs)
    return np.concatenate(parts, axis=0)


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------
def spec(n, d, ops, name):
    return W.CircuitSpec(n, d, [(o[0], o[1], o[2] if len(o) > 2 else None, o[3] if len(o) > 3 else {})
                                for o in ops], name)


def kat_cases():
    """Known-answer circuits of the reference's tests (tests/test_circuit.py:9-263,
    tests/test_program.py:14-47) with their expected outcomes."""
    out = []
    out.append((spec(2, 2, [("H", 1), ("P", 1), ("H", 0), ("CNOT", 0, 1), ("H", 1), ("CNOT", 0, 1), ("H", 1),
                            ("P", 0), ("H", 0), ("M", 0), ("P", 1), ("H", 1), ("M", 1)], "kat_phase_kickback"),
                [(0, True, 1), (1, True, 1)]))
    out.append((spec(2, 2, [("H", 0), ("P", 0), ("P", 0), ("H", 0), ("M", 0), ("X", 1), ("M", 1)],
                     "kat_qubit_flip"), [(0, True, 1), (1, True, 1)]))
    out.append((spec(2, 3, [("X", 0), ("M", 0)], "kat_qutrit_flip"), [(0, True, 1)]))
    for d in (2, 3, 5):
        for x0 in range(d):
            for x1 in range(d):
                ops = [("X", 0)] * x0 + [("X", 1)] * x1 + [("SWAP", 0, 1), ("M", 0), ("M", 1)]
                out.append((spec(2, d, ops, f"kat_swap_d{d}_{x0}{x1}"), [(0, True, x1), (1, True, x0)]))
                ops = [("X", 0)] * x0 + [("X", 1)] * x1 + [("SWAP", 0, 1), ("SWAP", 0, 1), ("M", 0), ("M", 1)]
                out.append((spec(2, d, ops, f"kat_double_swap_d{d}_{x0}{x1}"), [(0, True, x0), (1, True, x1)]))
    for a in range(3):
        for b in range(3):
            ops = [("X", 0)] * a + [("DFT", 0)] + [("X", 1)] * b + [("DFT", 1), ("SWAP", 0, 1), ("MX", 0),
                                                                     ("MX", 1)]
            out.append((spec(2, 3, ops, f"kat_xswap_{a}{b}"), [(0, True, b), (1, True, a)]))
    for s0 in (0, 1):
        for s1 in (0, 1):
            ops = [("H", 0), ("X", 1), ("H", 1)]
            if s0:
                ops += [("CNOT", 0, 1), ("X", 1)]
            if s1:
                ops += [("CNOT", 0, 1)]
            ops += [("H", 0), ("M", 0)]
            out.append((spec(2, 2, ops, f"kat_qubit_deutsch_{s0}{s1}"), [(0, True, 0 if s0 == s1 else 1)]))
    ops = [("X", 2), ("X", 3), ("X", 4), ("H", 0), ("CZ", 0, 2), ("CZ", 0, 3), ("CZ_INV", 0, 4), ("H_INV", 0),
           ("H", 1), ("CZ_INV", 1, 2), ("CZ_INV", 1, 3), ("CZ", 1, 4), ("H_INV", 1), ("M", 0), ("M", 1)]
    out.append((spec(5, 3, ops, "kat_z_stabilizer_extraction"), [(0, True, 1), (1, True, 2)]))
    ops = [("H", 2), ("H", 3), ("H", 4), ("Z", 2), ("H", 0), ("CX", 0, 2), ("CX", 0, 3), ("CX_INV", 0, 4),
           ("H_INV", 0), ("H", 1), ("CX_INV", 1, 2), ("CX_INV", 1, 3), ("CX", 1, 4), ("H_INV", 1), ("M", 0),
           ("M", 1)]
    out.append((spec(5, 3, ops, "kat_x_stabilizer_extraction"), [(0, True, 2), (1, True, 1)]))
    out.append((spec(2, 3, [("H", 0), ("X", 1), ("H", 1), ("CNOT", 0, 1), ("H_INV", 0), ("M", 0)],
                     "kat_deutsch_d3"), [(0, True, 2)]))
    out.append((spec(2, 3, [("M", 0), ("M", 1)], "kat_measurement_format_1"), [(0, True, 0), (1, True, 0)]))
    out.append((spec(2, 3, [("M", 0), ("M", 1), ("M", 0), ("M", 1)], "kat_measurement_format_2"),
                [(0, True, 0), (0, True, 0), (1, True, 0), (1, True, 0)]))
    return out


def random_cases():
    out = []
    k = 0
    for d in (2, 3, 5, 7, 11, 13):
        for n in (1, 2, 3, 5, 8):
            nops = 50 if n <= 2 else 110
            s = W.all_gates_random(n, d, nops, seed=1000 + k, name=f"rand_d{d}_n{n}")
            out.append(s)
            k += 1
    # long runs of additive gates between reductions (lazy modulo, large intermediates)
    rng = np.random.Generator(np.random.PCG64(77))
    for d in (3, 7):
        ops = []
        for _ in range(300):
            g = ["CNOT", "CNOT_INV", "P", "P_INV", "H"][int(rng.integers(5))]
            if g.startswith("CNOT"):
                c, t = rng.choice(4, 2, replace=False)
                ops.append((g, int(c), int(t), {}))
            else:
                ops.append((g, int(rng.integers(4)), None, {}))
        ops += [("M", q, None, {}) for q in range(4)] + [("RESET", q, None, {}) for q in range(4)]
        out.append(W.CircuitSpec(4, d, ops, f"long_additive_d{d}"))
    # aliased two-qudit gates (control == target) are accepted by the reference
    for d in (2, 5):
        ops = [("H", 0, None, {}), ("CNOT", 1, 0, {}), ("P", 1, None, {}), ("CNOT", 1, 1, {}), ("H", 1, None, {}),
               ("CZ", 0, 0, {}), ("M", 0, None, {}), ("M", 1, None, {}), ("RESET", 0, None, {}),
               ("CNOT_INV", 0, 0, {}), ("M", 0, None, {}), ("M", 1, None, {})]
        out.append(W.CircuitSpec(3, d, ops, f"aliased_pairs_d{d}"))
    return out


def main():
    cases, arrays = [], {}

    def add(name, specs, seed, nshots, noise=True, snapshots=False, final=False, record_tableau=False,
            expected=None, parallel=False):
        if parallel:
            rec = run_parallel(specs, seed, nshots, noise=noise)
            res = run_reference(specs, seed, 0, min(4, nshots), noise=noise, final=final)
            assert np.array_equal(res["records"], rec[:res["records"].shape[0]])
        else:
            res = run_reference(specs, seed, 0, nshots, noise=noise, snapshots=snapshots, final=final,
                                record_tableau=record_tableau, want_nested=expected is not None)
            rec = res["records"]
        arrays[f"{name}__records"] = rec
        if res.get("snapshots") is not None and snapshots:
            arrays[f"{name}__snapshots"] = res["snapshots"]
        if res.get("final") is not None:
            arrays[f"{name}__final"] = res["final"]
        if res.get("record_tableau") is not None:
            arrays[f"{name}__record_tableau"] = res["record_tableau"]
        entry = {"name": name, "seed": seed, "nshots": nshots, "noise": noise,
                 "circuits": [s.to_json() for s in specs]}
        if expected is not None:
            got = res["nested"][0]
            assert got == [tuple(e) for e in expected], (name, got, expected)
            entry["expected"] = [list(e) for e in expected]
        cases.append(entry)
        print(name, rec.shape, flush=True)

    for s, exp in kat_cases():
        add(s.name, [s], 7, 1, snapshots=True, final=True, expected=exp)
    for s in random_cases():
        add(s.name, [s], 4242, 3, snapshots=True, final=True)
    for d in (3, 5):
        s = W.all_gates_random(3, d, 40, seed=555 + d, name=f"record_tableau_d{d}")
        add(s.name, [s], 99, 1, final=True, record_tableau=True)
    a = W.all_gates_random(3, 3, 70, seed=31, name="program_part_a")
    b = W.all_gates_random(3, 3, 70, seed=32, name="program_part_b")
    add("appended_program_d3", [a, b], 5, 3, snapshots=True, final=True)
    add("noise_off_d5", [W.all_gates_random(4, 5, 90, seed=71, name="noise_off_d5")], 11, 3, noise=False,
        snapshots=True, final=True)
    add("no_measurement_d3", [W.CircuitSpec(3, 3, [("H", 0, None, {}), ("CNOT", 0, 1, {})], "nm")], 1, 2,
        snapshots=True, final=True)
    add("pr1_d3_n32", [W.pr1(0)], 0, 1024, final=True, parallel=True)
    add("surface_L3_r3", [W.surface_memory(3, 3, prob=0.02)], 0, 128, final=True, parallel=True)
    for d in (5, 7):
        s = W.random_hpc(24, d, 240, seed=d, weights=(0.25, 0.25, 0.5), mr_every=24, mr_fraction=0.1,
                         name=f"oddd_small_d{d}")
        add(s.name, [s], 0, 64, final=True, parallel=True)
    (HERE / "cases.json").write_text(json.dumps({"cases": cases}, indent=0))
    np.savez_compressed(HERE / "arrays.npz", **arrays)
    print("wrote", len(cases), "cases")


if __name__ == "__main__":
    if "--frames" in sys.argv:
        main_frames()
    elif "--stats" in sys.argv:
        main_stats()
    elif "--chp" in sys.argv:
        main_chp()
    else:
        main()
