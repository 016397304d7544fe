"""GPU: records written straight into page-locked host memory.

With SDIM_FLAG_DIRECT_HOST and a page-locked host output buffer the kernels
store the records into it directly (no device buffer, no copy); otherwise
they go through a device buffer and a copy.  Both routes must give the same
records, bit for bit, for every engine, and equal the oracle."""
import numpy as np
import pytest

import oracle
from sdim_gb300 import Program, _lib, workloads
from sdim_gb300.batch import BatchRunner

pytestmark = pytest.mark.gpu


def _pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.uint8, pin_memory=True).numpy()


@pytest.mark.parametrize("spec,shots,engine", [
    (workloads.surface_memory(3, 3, prob=0.02), 300, None),        # d = 2 trace engine
    (workloads.surface_memory(3, 3, prob=0.02), 40, None),         # d = 2 shot groups
    (workloads.random_hpc(40, 5, 200, seed=3), 200, None),         # odd-d trace engine
    (workloads.random_hpc(40, 7, 200, seed=4), 50, None),          # odd-d shot groups
    (workloads.random_hpc(20, 3, 120, seed=5), 70, "per_shot"),    # per-shot engine
], ids=["d2_trace", "d2_group", "d5_trace", "d7_group", "d3_per_shot"])
def test_pinned_and_pageable_outputs_agree(spec, shots, engine):
    prog = Program(spec.build())
    n, d = spec.num_qudits, spec.dimension
    ref = oracle.simulate(oracle.OracleProgram([spec], n, d), 9, 5, shots)["records"]
    pageable = prog.sample(shots, seed=9, shot0=5, engine=engine)
    pinned = _pinned(pageable.shape)
    pinned.fill(0xEE)
    dp = prog.compile()
    rc = prog.context.lib.sdim_run(prog.context.ptr, dp.ptr, 9, 5, shots, pinned.ctypes.data,
                                   _lib.FLAG_DIRECT_HOST | _lib.engine_flags(engine))
    _lib.check(rc, prog.context.ptr)
    staged = _pinned(pageable.shape)
    prog.sample(shots, seed=9, shot0=5, engine=engine, out=staged)
    assert np.array_equal(pageable, ref)
    assert np.array_equal(pinned, ref)
    assert np.array_equal(staged, ref)


def test_batch_mixes_pinned_and_pageable_outputs():
    """One batch whose outputs are partly page-locked, partly pageable, run
    with SDIM_FLAG_DIRECT_HOST (the page-locked ones written directly), and
    the same batch staged through the device."""
    specs = [workloads.random_hpc(12, 3, 60, seed=1), workloads.surface_memory(3, 2, prob=0.05),
             workloads.random_hpc(170, 5, 400, seed=2), workloads.random_hpc(30, 2, 100, seed=3)]
    shots = [33, 200, 20, 150]
    br = BatchRunner()
    for i, (s, k) in enumerate(zip(specs, shots)):
        br.add_spec(s, k, seed=40 + i)
    refs = [oracle.simulate(oracle.OracleProgram([s], s.num_qudits, s.dimension), 40 + i, 0, k)["records"]
            for i, (s, k) in enumerate(zip(specs, shots))]
    outs = []
    for i, e in enumerate(br.entries):
        shape = (e.shots, e.program.num_records)
        outs.append(_pinned(shape) if i % 2 == 0 else np.empty(shape, dtype=np.uint8))
    got = br.run(outs=outs, flags=_lib.FLAG_DIRECT_HOST)
    staged = br.run()
    for g, st, r in zip(got, staged, refs):
        assert np.array_equal(g, r)
        assert np.array_equal(st, r)
