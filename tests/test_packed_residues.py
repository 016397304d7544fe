"""CPU: the packed residue arithmetic of the odd-d trace engine's x / z
passes -- mod-3 bit planes (sdim_gb300/csrc/planes3.cuh) and 4-bit lanes for
d = 5, 7 (sdim_gb300/csrc/nibbles.cuh) -- compiled for the host with g++ and
checked exhaustively against integer arithmetic (tests/native/*_check.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


@pytest.mark.parametrize("name", ["planes3_check", "nibbles_check"])
def test_packed_residue_arithmetic(tmp_path, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / name
    subprocess.run([cxx, "-O2", "-std=c++17", str(HERE / "native" / f"{name}.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stdout + res.stderr
