"""CPU: the synthetic workloads have the shapes the benchmark configs name,
and the surface-code schedule measures its stabilizers (checked with the
oracle)."""
import math

import numpy as np
import pytest

import oracle
from sdim_gb300 import workloads


def test_pr1_shape():
    s = workloads.pr1(0)
    assert (s.num_qudits, s.dimension, len(s.ops)) == (32, 3, 672)
    gates = s.ops[:640]
    assert {g[0] for g in gates} == {"H", "P", "CNOT"}
    assert all(g[1] != g[2] for g in gates if g[0] == "CNOT")
    assert [g[1] for g in s.ops[640:]] == list(range(32))
    assert workloads.pr1(0).ops == s.ops  # seeded


def test_odd_d_shape():
    s = workloads.odd_d(5, seed=0)
    assert (s.num_qudits, s.dimension) == (256, 5)
    kinds = [o[0] for o in s.ops]
    assert kinds.count("RESET") == 10 * 26
    assert kinds.count("M") == 256
    gates = [k for k in kinds if k in ("H", "P", "CNOT")]
    assert len(gates) == 2560
    assert 0.45 < gates.count("CNOT") / 2560 < 0.55


@pytest.mark.parametrize("L", [3, 5, 7])
def test_surface_layout_counts(L):
    xc, zc = workloads.surface_layout(L)
    assert len(xc) == len(zc) == (L * L - 1) // 2
    s = workloads.surface_memory(L, 1, noise=False)
    cnots = sum(1 for o in s.ops if o[0] == "CNOT")
    assert cnots == 4 * (L - 1) ** 2 + 2 * 2 * (L - 1)
    if L == 7:
        assert s.num_qudits == 97 and cnots == 168


def test_surface_memory_noise_placement():
    s = workloads.surface_memory(7, 7, prob=1e-3)
    ops = s.ops
    n1 = [o for o in ops if o[0] == "N1"]
    assert len(n1) == 7 * (24 + 2 * 168 + 24 + 48)
    assert all(o[3] == {"prob": 1e-3, "noise_channel": "d"} for o in n1)
    assert len(ops) == 4921 and s.num_measurements() == 385


@pytest.mark.parametrize("L", [3, 5])
def test_surface_schedule_measures_stabilizers(L):
    """Noiseless: Z checks start at 0, every round repeats round 1, later
    rounds are deterministic (oracle, 64 shots)."""
    spec = workloads.surface_memory(L, 3, noise=False)
    nanc = spec.num_qudits - L * L
    nx = len(workloads.surface_layout(L)[0])
    rec = oracle.simulate(oracle.OracleProgram([spec], spec.num_qudits, 2), 0, 0, 64)["records"]
    vals = (rec & 0x7F).astype(int)
    rounds = vals[:, :3 * nanc].reshape(-1, 3, nanc)
    assert np.all(rounds[:, 1:] == rounds[:, :1])
    assert np.all(rounds[:, 0, nx:] == 0)
    assert np.all((rec[0, nanc:3 * nanc] >> 7) == 1)


def test_uneven_batch_distribution():
    items = workloads.uneven_batch(2000, seed=0)
    ns = np.array([it.spec.num_qudits for it in items])
    assert ns.min() >= 8 and ns.max() <= 1024
    med = float(np.median(np.log(ns)))
    assert abs(med - 0.5 * (math.log(8) + math.log(1024))) < 0.15
    assert {it.spec.dimension for it in items} == {2, 3, 5, 7}
    shots = np.array([it.shots for it in items])
    assert shots.min() >= 1 and shots.max() <= 64
    it = items[0]
    assert len(it.spec.ops) == 5 * it.spec.num_qudits


def test_serving_stream_rate():
    reqs = workloads.serving_stream(rate_hz=2000.0, duration_s=1.0, seed=1, n_max=64, shots_max=100)
    assert 1800 < len(reqs) < 2200
    t = [r.arrival_s for r in reqs]
    assert all(a < b for a, b in zip(t, t[1:]))
    assert {r.item.spec.dimension for r in reqs} <= {2, 3, 5}
