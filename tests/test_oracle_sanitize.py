"""The oracle under AddressSanitizer and UndefinedBehaviorSanitizer
(tests/cpp/oracle_sanitize.cpp): every entry point of oracle/dtk_oracle.h on
small clouds and edge shapes, built with -fsanitize=address,undefined and
halting on the first report."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_oracle_is_clean_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "oracle_san"
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-ffp-contract=off", "-I", str(ROOT / "oracle"),
           str(ROOT / "oracle" / "dtk_oracle.cpp"), str(ROOT / "tests" / "cpp" / "oracle_sanitize.cpp"),
           "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0 and ("asan" in res.stderr.lower() or "ubsan" in res.stderr.lower()):
        pytest.skip("sanitizer runtimes not available: " + res.stderr.strip().splitlines()[-1])
    assert res.returncode == 0, res.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, env=env)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip() == "PASS", run.stdout + run.stderr
    assert "runtime error" not in run.stderr and "Sanitizer" not in run.stderr, run.stderr
