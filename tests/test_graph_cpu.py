"""CPU: the Python side of graph capture (graph.CapturedRun) against a fake
library: the arrays it passes to sdim_graph_create / sdim_graph_launch, its
argument checks and its error mapping (the GPU test is tests/test_gpu_graph.py)."""
import ctypes as C

import pytest

from sdim_gb300 import _lib
from sdim_gb300.batch import BatchEntry
from sdim_gb300.graph import CapturedRun


class _Prog:
    def __init__(self, addr):
        self.ptr = C.c_void_p(addr)


class FakeLib:
    def __init__(self):
        self.created = None
        self.launches = []
        self.destroyed = 0
        self.fail_launch = False

    def sdim_graph_create(self, ctx, k, circs, seeds, shot0, nshots, outs, flags, out):
        self.created = {"k": k, "circs": [circs[i] for i in range(k)], "seeds": [seeds[i] for i in range(k)],
                        "shot0": [shot0[i] for i in range(k)], "nshots": [nshots[i] for i in range(k)],
                        "outs": [outs[i] for i in range(k)], "flags": flags}
        out._obj.value = 0xABC
        return 0

    def sdim_graph_launch(self, g, seeds, shot0, stream):
        if self.fail_launch:
            return _lib.SDIM_ECUDA
        k = self.created["k"]
        self.launches.append((None if seeds is None else [seeds[i] for i in range(k)],
                              None if shot0 is None else [shot0[i] for i in range(k)],
                              None if stream is None else stream.value))
        return 0

    def sdim_graph_sync(self, g):
        return 0

    def sdim_graph_info(self, g, buf):
        buf[0], buf[1], buf[2] = 6, 3, 768
        return 0

    def sdim_graph_last_error(self, g):
        return b"graph launch: device busy"

    def sdim_graph_destroy(self, g):
        self.destroyed += 1
        return 0


class FakeCtx:
    def __init__(self):
        self.lib = FakeLib()
        self.ptr = C.c_void_p(1)


def test_captured_run_passes_entries_and_replay_values():
    ctx = FakeCtx()
    entries = [BatchEntry(_Prog(0x1000), 64, 7, 3), BatchEntry(_Prog(0x2000), 5, -1, 0)]
    run = CapturedRun(ctx, entries, [0x9000, 0xA000], flags=_lib.FLAG_TRACE)
    c = ctx.lib.created
    assert c["k"] == 2 and c["circs"] == [0x1000, 0x2000] and c["outs"] == [0x9000, 0xA000]
    assert c["seeds"] == [7, 0xFFFFFFFFFFFFFFFF] and c["shot0"] == [3, 0] and c["nshots"] == [64, 5]
    assert c["flags"] == _lib.FLAG_TRACE
    run.launch()
    run.launch(seeds=[1, 2], shot0=[100, 200], stream=0x55)
    assert ctx.lib.launches[0] == (None, None, None)
    assert ctx.lib.launches[1] == ([1, 2], [100, 200], 0x55)
    assert run.info() == {"nodes": 6, "kernel_nodes": 3, "staging_bytes": 768}
    run.sync()
    run.close()
    run.close()
    assert ctx.lib.destroyed == 1


def test_captured_run_argument_checks_and_errors():
    ctx = FakeCtx()
    entries = [BatchEntry(_Prog(0x1000), 64, 7, 3)]
    with pytest.raises(ValueError):
        CapturedRun(ctx, entries, [])
    run = CapturedRun(ctx, entries, [0x9000])
    with pytest.raises(ValueError):
        run.launch(seeds=[1, 2])
    with pytest.raises(ValueError):
        run.launch(shot0=[])
    ctx.lib.fail_launch = True
    with pytest.raises(_lib.SdimError, match="device busy"):
        run.launch()
    run.close()
