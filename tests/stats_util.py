"""Helpers of the statistical tests: joint outcome histograms, the
closed-form outcome distributions of the reference's statistical tests, and
chi-square comparisons.

``tests/golden/stats.json`` holds the reference's own histograms
(``make_golden.py --stats``: sdim's ``Program.simulate(shots)`` with its
native random number generators).  Runs here draw from the Philox stream,
so shots differ one by one; the distributions must not.
"""
import json

import numpy as np
from scipy import stats

from tests.conftest import GOLDEN

# Significance floor of every chi-square test.  Seeds are fixed, so each test
# is deterministic; the floor only says how unlikely a pass must be to fail.
P_MIN = 1e-4
# The reference's own criterion (tests/test_noise_and_io.py:127, 154):
# every outcome frequency within 0.01 of the ideal probability.
FUZZ = 0.01


def cases():
    return json.loads((GOLDEN / "stats.json").read_text())["cases"]


def joint_histogram(records: np.ndarray, kinds, d: int) -> np.ndarray:
    """Counts of the joint outcome of the M records (first record in the
    lowest base-d digit); RESET records are left out, as in the fixtures."""
    vals = (np.asarray(records, dtype=np.int64) & 0x7F)
    keep = [j for j, k in enumerate(kinds) if k == "M"]
    index = (vals[:, keep] * (d ** np.arange(len(keep)))).sum(axis=1)
    return np.bincount(index, minlength=d ** len(keep))


def homogeneity_pvalue(a: np.ndarray, b: np.ndarray) -> float:
    """Chi-square test that two histograms come from one distribution
    (categories empty in both are dropped; one category left is a match)."""
    a, b = np.asarray(a), np.asarray(b)
    used = (a + b) > 0
    if used.sum() <= 1:
        return 1.0
    return float(stats.chi2_contingency(np.stack([a[used], b[used]]))[1])


def ideal_distribution(case):
    """Closed-form outcome distribution of the single-qudit cases
    (tests/test_noise_and_io.py:101-186, tests/test_reset.py:11-37), or None."""
    circ = case["circuit"]
    d = circ["d"]
    ops = circ["ops"]
    name = case["name"]
    p = next((o[3]["prob"] for o in ops if o[0] == "N1"), None)
    if name.startswith("stat_depolarizing"):
        p0 = (1 - p) + (d - 1) * p / (d * d - 1)
        return np.array([p0] + [d * p / (d * d - 1)] * (d - 1))
    if name.startswith(("stat_flip", "stat_phase")):
        return np.array([1 - p] + [p / (d - 1)] * (d - 1))
    if name.startswith("stat_reset_skip"):
        k = sum(1 for o in ops if o[0] == "X")
        return np.eye(d)[k % d]
    return None


def goodness_of_fit_pvalue(hist: np.ndarray, probs: np.ndarray) -> float:
    used = probs > 0
    if np.any(hist[~used]):
        return 0.0
    if used.sum() <= 1:
        return 1.0
    expected = probs[used] * hist.sum()
    return float(stats.chisquare(hist[used], expected)[1])


def check_statistics(case, records: np.ndarray, route: str) -> None:
    """The histogram of one route's M records against the reference's
    (homogeneity) and, for the single-qudit cases, against the closed form
    (goodness of fit and the reference's 0.01 criterion)."""
    d = case["circuit"]["d"]
    h = joint_histogram(records, case["record_kinds"], d)
    assert h.sum() == case["shots"], route
    p = homogeneity_pvalue(h, np.asarray(case["histogram"]))
    assert p > P_MIN, (route, p)
    ideal = ideal_distribution(case)
    if ideal is not None:
        assert goodness_of_fit_pvalue(h, ideal) > P_MIN, route
        assert np.all(np.abs(h / h.sum() - ideal) < FUZZ), route
