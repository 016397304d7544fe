import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def golden():
    cases = json.loads((GOLDEN / "cases.json").read_text())["cases"]
    arrays = np.load(GOLDEN / "arrays.npz")
    return {c["name"]: c for c in cases}, arrays


@pytest.fixture(scope="session")
def cuda_ctx():
    from sdim_gb300 import _lib
    return _lib.Context.default(0)


def specs_of(case):
    from sdim_gb300.workloads import CircuitSpec
    return [CircuitSpec.from_json(s) for s in case["circuits"]]


def program_of(case, **kw):
    """Drop-in Program built from a golden case (appending extra circuits)."""
    from sdim_gb300 import Program
    specs = specs_of(case)
    prog = Program(specs[0].build(), **kw)
    for s in specs[1:]:
        prog.append_circuit(s.build())
    return prog


def oracle_run(specs, seed, shot0=0, nshots=1, noise=True, **kw):
    import oracle
    n, d = specs[0].num_qudits, specs[0].dimension
    return oracle.simulate(oracle.OracleProgram(specs, n, d), seed, shot0, nshots, noise=noise, **kw)
