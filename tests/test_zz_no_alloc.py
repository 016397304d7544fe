"""GPU: the allocation-free entry point ``sdim_run_noalloc``.

It serves callers that cannot call cudaMalloc themselves -- code running
under another framework's device allocator, or in a process whose device
memory is already reserved -- by keeping all of its scratch in one fixed
device array compiled into the library.  The caller passes the op table and
a device output buffer (here a torch tensor: the test allocates, the entry
point does not).  Its records must equal those of the ordinary entry point
(``sdim_run`` through ``Program.sample``) bit for bit, on consecutive calls
that reuse the shared scratch.

This file is collected last so that a failure here stops a ``-x`` run only
after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from sdim_gb300 import Program, _lib, workloads

pytestmark = pytest.mark.gpu


def _noalloc(enc, seed, shot0, shots, out, stream=0):
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)
    ops = np.ascontiguousarray(enc.ops)
    probs = np.ascontiguousarray(enc.probs)
    rc = lib.sdim_run_noalloc(ops.ctypes.data, int(ops.shape[0]), probs.ctypes.data if probs.size else None,
                              int(enc.n), int(enc.d), int(seed), int(shot0), int(shots),
                              out.data_ptr() if out is not None else None, stream or None, err, 256)
    return rc, err.value.decode()


@pytest.mark.parametrize("spec", [
    workloads.pr1(0),
    workloads.surface_memory(3, 3, prob=0.05),
    workloads.all_gates_random(7, 5, 200, seed=4),
], ids=["pr1_d3", "surface_L3_d2", "all_gates_d5"])
def test_noalloc_equals_run_on_two_calls_in_a_row(spec):
    import torch
    prog = Program(spec.build())
    enc = prog.compile().enc
    shots = 300
    out = torch.empty((shots, enc.num_records), dtype=torch.uint8, device="cuda")
    for call, shot0 in enumerate((0, 1000)):
        ref = prog.sample(shots, seed=21, shot0=shot0)
        out.fill_(0xFF)
        rc, msg = _noalloc(enc, 21, shot0, shots, out)
        assert rc == _lib.SDIM_OK, msg
        assert np.array_equal(out.cpu().numpy(), ref), f"call {call}"


def test_noalloc_rejects_programs_beyond_its_limits():
    import torch
    # tableau too large for shared memory
    big = workloads.random_hpc(400, 7, 10, seed=1)
    enc = Program(big.build()).compile().enc
    out = torch.empty((1, enc.num_records), dtype=torch.uint8, device="cuda")
    rc, msg = _noalloc(enc, 0, 0, 1, out)
    assert rc == _lib.SDIM_EINVAL and "shared memory" in msg
    # more device instructions than the scratch array holds (SWAP expands to 9)
    from sdim_gb300 import Circuit
    c = Circuit(2, 3)
    for _ in range(14600):
        c.add_gate("SWAP", 0, 1)
    c.add_gate("M", 0)
    enc = Program(c).compile().enc
    rc, msg = _noalloc(enc, 0, 0, 1, out)
    assert rc == _lib.SDIM_EINVAL and "131072" in msg
