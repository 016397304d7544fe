"""GPU: the largest programs each engine takes, against the oracle and the
other engines.  Each program is 2n random {H, P, CNOT} gates, a MEASURE+RESET
sweep and MEASURE on every 32nd qudit, so the oracle stays quick at n = 2048:
- n = 2048 is the odd-d trace engine's limit, with the x/z columns of a
  lone program streamed from global memory by a cluster of 8 CTAs, and
  beyond the d = 2 trace engine's 512;
- n = 2049 sends odd d back to the shot-group engine."""
import numpy as np
import pytest

from sdim_gb300 import Program, workloads
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


def _big(n, d, seed):
    base = workloads.random_hpc(n, d, 2 * n, seed=seed, final_measure=False)
    ops = list(base.ops)
    ops += [("RESET", q, None, {}) for q in range(5, n, 97)]
    ops += [("M", q, None, {}) for q in range(0, n, 32)]
    return workloads.CircuitSpec(n, d, ops, f"big_n{n}_d{d}")


@pytest.mark.parametrize("n,d", [(2048, 2), (2048, 3), (2049, 5)])
def test_largest_programs(n, d):
    spec = _big(n, d, seed=n + d)
    prog = Program(spec.build())
    auto = prog.sample(40, seed=7)
    assert np.array_equal(auto, prog.sample(40, seed=7, engine="group"))
    assert np.array_equal(auto[:8], prog.sample(8, seed=7, engine="per_shot"))
    if d != 2 and n <= 2048:
        assert np.array_equal(auto, prog.sample(40, seed=7, engine="trace"))
    assert np.array_equal(auto[:2], oracle_run([spec], 7, 0, 2)["records"])
