"""ctypes binding of ``include/sdim_gb300.h``.

The library is the only execution path: when it cannot be built or loaded,
or no CUDA device is present, every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

SDIM_OK = 0
SDIM_EINVAL = -1
SDIM_ECUDA = -2
SDIM_ENOMEM = -3
SDIM_EDEVICE = -4
SDIM_EUNSUPPORTED = -5

FLAG_PLAIN = 1
FLAG_OUT_DEVICE = 2
FLAG_ASYNC = 4
FLAG_TIME = 8
FLAG_FORCE_GMEM = 16
FLAG_PER_SHOT = 32
FLAG_TEAM_WARP = 64
FLAG_TEAM_CTA = 128
FLAG_TRACE = 256
FLAG_NO_TRACE = 512
FLAG_NO_COIN_PASS = 1024
FLAG_SPLIT_XZ = 2048
FLAG_CLUSTER_XZ = 4096
FLAG_DIRECT_HOST = 8192
FLAG_U8_XZ = 16384
FLAG_PACKED_XZ = 131072
FLAG_LANE_SHOTS_1 = 65536
FLAG_REUSE_XZ = 262144
FLAG_COLUMNS = 524288
FLAG_PHASE_REPLAY = 1048576
FLAG_UNLAYERED = 2097152


def engine_flags(engine) -> int:
    """Run flags that select a batched engine by name (None: the library's
    choice by shot count and dimension)."""
    table = {None: 0, "auto": 0, "trace": FLAG_TRACE, "group": FLAG_NO_TRACE, "per_shot": FLAG_PER_SHOT,
             "group_warp": FLAG_TEAM_WARP, "group_cta": FLAG_TEAM_CTA}
    if engine not in table:
        raise ValueError(f"unknown engine {engine!r}; expected one of {sorted(k for k in table if k)}")
    return table[engine]

SNAP_EVERY_INSTRUCTION = 1
SNAP_AT_MEASUREMENT = 2
SNAP_FINAL = 3

# exported symbol -> (restype, argtypes)
_P = C.c_void_p
SIGNATURES = {
    "sdim_ctx_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "sdim_ctx_destroy": (C.c_int, [_P]),
    "sdim_last_error": (C.c_char_p, [_P]),
    "sdim_device_info": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sdim_memory_info": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sdim_program_bytes": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int64)]),
    "sdim_encode_circuit": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int, C.c_int, C.POINTER(_P)]),
    "sdim_circuit_destroy": (C.c_int, [_P]),
    "sdim_circuit_info": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sdim_circuit_kept": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "sdim_run": (C.c_int, [_P, _P, C.c_uint64, C.c_int64, C.c_int64, _P, C.c_uint]),
    "sdim_run_device": (C.c_int, [_P, _P, C.c_uint64, C.c_int64, C.c_int64, _P, _P, C.c_uint]),
    "sdim_frame_run": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_int64, _P, C.c_uint]),
    "sdim_parse_chp": (C.c_int, [C.c_char_p, C.c_int64, _P, _P, C.c_int64, C.POINTER(C.c_int64),
                               C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_char_p, C.c_size_t]),
    "sdim_run_batch": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P, C.c_uint]),
    "sdim_sync": (C.c_int, [_P]),
    "sdim_query": (C.c_int, [_P]),
    "sdim_run_tables": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_uint]),
    "sdim_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "sdim_host_free": (C.c_int, [_P]),
    "sdim_last_kernel_ms": (C.c_double, [_P]),
    "sdim_last_stage_ms": (C.c_int, [_P, _P]),
    "sdim_last_pass_ms": (C.c_int, [_P, _P]),
    "sdim_last_passes_ms": (C.c_int, [_P, _P, C.c_int]),
    "sdim_snapshot": (C.c_int, [_P, _P, C.c_uint64, C.c_int64, C.c_int, _P, _P, C.c_uint]),
    "sdim_probe_smem_bandwidth": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sdim_probe_l2_bandwidth": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sdim_trace_xz_mode": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_uint, C.c_int32, C.c_int32]),
    "sdim_program_words": (C.c_int, [_P, C.c_int64, _P, C.c_int32, C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "sdim_probe_philox_rate": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sdim_graph_create": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, C.c_uint, C.POINTER(_P)]),
    "sdim_graph_launch": (C.c_int, [_P, _P, _P, _P]),
    "sdim_graph_sync": (C.c_int, [_P]),
    "sdim_graph_info": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sdim_graph_last_error": (C.c_char_p, [_P]),
    "sdim_graph_destroy": (C.c_int, [_P]),
    "sdim_run_noalloc": (C.c_int, [_P, C.c_int64, _P, C.c_int, C.c_int, C.c_uint64, C.c_int64, C.c_int64, _P,
                                   _P, C.c_char_p, C.c_size_t]),
}

_lock = threading.Lock()
_default_lock = threading.Lock()
_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads (building first when needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and not _build.up_to_date():
            _build.build_library()
        path = _build.LIB
        if not path.exists():
            raise RuntimeError(f"sdim_gb300 CUDA library missing at {path}; run sdim_gb300.build.build_library()")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class SdimError(RuntimeError):
    pass


def check(rc: int, ctx_ptr=None, what: str = ""):
    if rc == SDIM_OK:
        return
    msg = ""
    if ctx_ptr:
        raw = load().sdim_last_error(ctx_ptr)
        msg = raw.decode() if raw else ""
    text = f"{what}: {msg}" if what else msg
    if rc == SDIM_EINVAL:
        if "out of range" in msg:
            raise IndexError(text)
        raise ValueError(text)
    if rc == SDIM_EUNSUPPORTED:
        raise NotImplementedError(text)
    raise SdimError(f"{text} (status {rc})")


class Context:
    """One CUDA device: owns the library context (stream, device buffers)."""

    _default = {}

    def __init__(self, device: int = 0):
        lib = load()
        ptr = _P()
        rc = lib.sdim_ctx_create(int(device), C.byref(ptr))
        if rc != SDIM_OK:
            raise SdimError(f"no usable CUDA device {device} for sdim_gb300 (status {rc})")
        self.ptr = ptr
        self.device = int(device)
        self.lib = lib
        info = (C.c_int64 * 4)()
        check(lib.sdim_device_info(ptr, info), ptr)
        self.num_sms, self.smem_optin, self.l2_bytes, self.gmem_bytes = (int(v) for v in info)

    @classmethod
    def default(cls, device: int = 0) -> "Context":
        """The process-wide context of a device (created once, also when
        several threads ask at the same time)."""
        with _default_lock:
            if device not in cls._default:
                cls._default[device] = Context(device)
            return cls._default[device]

    def close(self):
        if self.ptr:
            self.lib.sdim_ctx_destroy(self.ptr)
            self.ptr = None

    def last_kernel_ms(self) -> float:
        return float(self.lib.sdim_last_kernel_ms(self.ptr))

    def last_stage_ms(self):
        """(x / z passes, phase passes, other engines) of the last timed call."""
        buf = (C.c_double * 3)()
        check(self.lib.sdim_last_stage_ms(self.ptr, buf), self.ptr, "sdim_last_stage_ms")
        return tuple(float(v) for v in buf)

    def last_pass_ms(self):
        """(x / z passes alone, d = 2 coin pass alone) of the last timed call."""
        buf = (C.c_double * 2)()
        check(self.lib.sdim_last_pass_ms(self.ptr, buf), self.ptr, "sdim_last_pass_ms")
        return tuple(float(v) for v in buf)

    def last_passes_ms(self):
        """(x / z passes alone, d = 2 coin pass, d = 2 column pass, shot-group
        engines beside the trace engines) of the last timed call."""
        buf = (C.c_double * 4)()
        check(self.lib.sdim_last_passes_ms(self.ptr, buf, 4), self.ptr, "sdim_last_passes_ms")
        return tuple(float(v) for v in buf)

    def sync(self):
        check(self.lib.sdim_sync(self.ptr), self.ptr, "sdim_sync")
