"""GPU: outcome statistics of both routes where the random streams differ.

The tableau route (``Program.sample``) and the Pauli-frame route
(``Program.sample_frames``) run 100,000 shots of each circuit of
tests/golden/stats.json with the Philox seed the CPU statistical tests use.
The first 4,096 shots must equal the oracle's bit for bit; the histograms
of all shots go through the same chi-square tests against the reference's
own histograms (its native random number generators) and the closed forms.
Collected after the other GPU tests (and before tests/test_zz_no_alloc.py).
"""
import numpy as np
import pytest

import oracle
from oracle import frame
from sdim_gb300 import Program
from sdim_gb300.workloads import CircuitSpec
from tests import stats_util as su

pytestmark = pytest.mark.gpu

CASES = su.cases()
SEED = 2026
EXACT = 4096


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_routes_match_reference_statistics(case):
    spec = CircuitSpec.from_json(case["circuit"])
    shots = case["shots"]
    prog = Program(spec.build())
    oprog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
    tab = prog.sample(shots, seed=SEED)
    frm = prog.sample_frames(shots, seed=SEED)
    assert np.array_equal(tab[:EXACT], oracle.simulate(oprog, SEED, 0, EXACT)["records"])
    assert np.array_equal(frm[:EXACT], frame.simulate(oprog, SEED, EXACT))
    su.check_statistics(case, tab, "tableau")
    su.check_statistics(case, frm, "frame")
