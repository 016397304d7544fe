"""Builds the CUDA library ``sdim_gb300/_build/libsdim_gb300.so`` in-tree.

One nvcc invocation per translation unit, sm_103a only, compiled in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libsdim_gb300.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-diag-suppress", "177"]
UNITS = ["abi.cu", "k_pershot.cu", "k_group.cu", "k_trace.cu", "k_trace_u8.cu", "k_trace_p3.cu", "k_trace_n4.cu",
         "k_frame.cu",
         "noalloc.cu", "chp.cu"]


def _nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the sdim_gb300 CUDA library cannot be built")


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in _sources())


def build_library(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    """Compiles the library unless it is newer than every source."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    flags = list(NVCC_FLAGS) + list(extra_flags or [])
    objs = []

    def compile_unit(unit):
        obj = BUILD / (Path(unit).stem + ".o")
        cmd = [nvcc, *ARCH, *flags, "-c", str(CSRC / unit), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{res.stdout}\n{res.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(UNITS), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *[str(o) for o in objs], "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
