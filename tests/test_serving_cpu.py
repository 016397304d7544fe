"""CPU: the serving loop's scheduling and error handling against a fake
library (no device).  A batch that the library refuses is retried one
request at a time, so only the bad request fails; an exception while
launching fails that batch's requests without stopping the scheduler."""
import ctypes as C
import threading

import numpy as np
import pytest

from sdim_gb300.serving import Server


def _expected(seed, shot0, shots, nmeas):
    s = np.arange(shots)[:, None] + shot0
    j = np.arange(nmeas)[None, :]
    return ((seed + 3 * s + 7 * j) % 100).astype(np.uint8)


class FakeLib:
    """Records of request i: (seed + 3 shot + 7 record) mod 100.  A table
    with a gate id above 17 makes the whole call fail, as the library's
    encoder does."""

    def __init__(self):
        self.err = b""
        self.pinned = {}
        self.calls = []
        self.idle = threading.Event()
        self.idle.set()
        self.raise_on = None

    def sdim_memory_info(self, ptr, info):
        info[0], info[1], info[2] = 1 << 34, 1 << 35, 0
        return 0

    def sdim_host_alloc(self, cap, pptr):
        buf = (C.c_uint8 * int(cap))()
        self.pinned[C.addressof(buf)] = buf
        pptr._obj.value = C.addressof(buf)
        return 0

    def sdim_host_free(self, ptr):
        self.pinned.pop(ptr.value, None)
        return 0

    def sdim_run_tables(self, ctx, k, rows, row_begin, probs, ns, ds, seeds, shot0, nshots, outs, stream, flags):
        rb = np.ctypeslib.as_array((C.c_int64 * (k + 1)).from_address(row_begin)).copy()
        table = np.ctypeslib.as_array((C.c_int32 * (4 * int(rb[-1]))).from_address(rows)).reshape(-1, 4)
        self.calls.append(k)
        if self.raise_on is not None and int(seeds[0]) == self.raise_on:
            raise RuntimeError("launch failed on the host")
        if (table[:, 0] > 17).any():
            self.err = b"unknown gate id"
            return -1
        for i in range(k):
            t = table[rb[i]:rb[i + 1]]
            nmeas = int(np.isin(t[:, 0], (14, 15, 16)).sum())
            nb = int(nshots[i]) * nmeas
            if nb:
                dst = np.ctypeslib.as_array((C.c_uint8 * nb).from_address(outs[i]))
                dst[:] = _expected(int(seeds[i]), int(shot0[i]), int(nshots[i]), nmeas).reshape(-1)
        return 0

    def sdim_query(self, ctx):
        return 1 if self.idle.is_set() else 0

    def sdim_sync(self, ctx):
        self.idle.wait(10)
        return 0

    def sdim_last_error(self, ctx):
        return self.err


def _context(lib):
    class FakeContext:
        def __init__(self, device):
            self.ptr = C.c_void_p(1)
            self.lib = lib

        def close(self):
            pass
    return FakeContext


def _table(nmeas, bad=False):
    rows = [(5, 0, -1, 0), (9, 0, 1, 0)] + [(14, q % 2, -1, 0) for q in range(nmeas)]
    if bad:
        rows.insert(1, (99, 0, -1, 0))
    return np.asarray(rows, dtype=np.int32)


def test_refused_batch_is_retried_request_by_request():
    lib = FakeLib()
    server = Server(lanes=1, context=_context(lib))
    try:
        lib.idle.clear()  # the first batch stays in flight until released
        first = server.submit(_table(2), 2, 3, shots=4, seed=1)
        while not lib.calls:
            threading.Event().wait(0.001)
        reqs = [server.submit(_table(3, bad=(i == 2)), 2, 3, shots=5 + i, seed=10 + i, shot0=i) for i in range(5)]
        lib.idle.set()
        assert np.array_equal(first.wait(10), _expected(1, 0, 4, 2))
        for i, r in enumerate(reqs):
            if i == 2:
                with pytest.raises(RuntimeError, match="unknown gate id"):
                    r.wait(10)
            else:
                assert np.array_equal(r.wait(10), _expected(10 + i, i, 5 + i, 3)), i
        # one call for the first request, the refused batch of five, then each alone
        assert lib.calls == [1, 5, 1, 1, 1, 1, 1]
        server.drain(10)
        assert server.mem_in_use == 0
    finally:
        server.close()


def test_host_exception_fails_only_its_batch():
    lib = FakeLib()
    lib.raise_on = 77
    server = Server(lanes=2, context=_context(lib))
    try:
        bad = server.submit(_table(1), 2, 3, shots=3, seed=77)
        with pytest.raises(RuntimeError, match="launch failed on the host"):
            bad.wait(10)
        good = server.submit(_table(2), 2, 3, shots=6, seed=5)
        assert np.array_equal(good.wait(10), _expected(5, 0, 6, 2))
        server.drain(10)
        assert server.mem_in_use == 0
        assert server.stats()["requests"] == 1
    finally:
        server.close()
