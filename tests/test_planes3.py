"""CPU: the mod-3 bit-plane arithmetic of the d = 3 trace engine
(sdim_gb300/csrc/planes3.cuh), compiled for the host with g++ and checked
exhaustively against integer arithmetic (tests/native/planes3_check.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_planes3_arithmetic(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "planes3_check"
    subprocess.run([cxx, "-O2", "-std=c++17", str(HERE / "native" / "planes3_check.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stdout + res.stderr
