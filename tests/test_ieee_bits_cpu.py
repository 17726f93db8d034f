"""The FP64 Jacobi's integer-pipe IEEE helpers (csrc/dtk_ieee.cuh), built for
the host, give exactly the host's IEEE results (tests/cpp/ieee_bits.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_ieee_helpers_match_ieee_arithmetic(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "ieee_bits"
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(ROOT / "datatransferkit_gb300" / "csrc"),
           str(ROOT / "tests" / "cpp" / "ieee_bits.cpp"), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip() == "PASS"
