"""CPU: outcome statistics where the random streams differ.

Both routes of the oracle (the tableau shot loop and the Pauli-frame route),
drawing from the Philox stream, against histograms of the reference's own
``Program.simulate`` with its native random number generators
(chi-square homogeneity), and against the closed-form distributions of the
reference's statistical tests (chi-square goodness of fit and the
reference's own 0.01 criterion).  The GPU runs the same seeds in
tests/test_gpu_z_statistics.py.
"""
import numpy as np
import pytest

import oracle
from oracle import frame
from sdim_gb300.workloads import CircuitSpec
from tests import stats_util as su

CASES = su.cases()
SEED = 2026


def _runs(case):
    spec = CircuitSpec.from_json(case["circuit"])
    prog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
    shots = case["shots"]
    return spec, {"tableau": oracle.simulate(prog, SEED, 0, shots)["records"],
                  "frame": frame.simulate(prog, SEED, shots)}


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_routes_match_reference_statistics(case):
    _, runs = _runs(case)
    for route, rec in runs.items():
        su.check_statistics(case, rec, route)
    ideal = su.ideal_distribution(case)
    if ideal is not None:
        # the reference's own histogram passes the same tests
        assert su.goodness_of_fit_pvalue(np.asarray(case["histogram"]), ideal) > su.P_MIN


@pytest.mark.parametrize("case", [c for c in CASES if "RESET" in c["record_kinds"]],
                         ids=[c["name"] for c in CASES if "RESET" in c["record_kinds"]])
def test_reset_records_per_route(case):
    """Frame route: every shot records shot 0's value at a RESET, as the
    reference's does (sdim/program.py:146-157; its fixture holds one value).
    Tableau route: RESET measures, so it repeats an M just before it."""
    spec, runs = _runs(case)
    kinds = case["record_kinds"]
    resets = [j for j, k in enumerate(kinds) if k == "RESET"]
    fr, tb = runs["frame"] & 0x7F, runs["tableau"] & 0x7F
    for j, ref_vals in zip(resets, case["reset_values"]):
        assert len(ref_vals) == 1
        assert np.all(fr[:, j] == fr[0, j])
    ops = [o for o in spec.ops if o[0] in ("M", "RESET")]
    for j in resets:
        if j > 0 and ops[j - 1][0] == "M" and ops[j - 1][1] == ops[j][1]:
            assert np.array_equal(tb[:, j], tb[:, j - 1])
    if case["name"].startswith("stat_reset_skip"):
        # after maximal mixing the tableau route's RESET outcome is uniform
        d = spec.dimension
        counts = np.bincount(tb[:, resets[0]], minlength=d)
        assert su.goodness_of_fit_pvalue(counts, np.full(d, 1.0 / d)) > su.P_MIN
