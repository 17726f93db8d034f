"""The C++ drop-in headers compile on the host without a GPU: with and
without the Kokkos stand-in (where PointCloudOperator<DeviceType>::apply
takes the reference's Kokkos::View value types), and the multi-rank test
program with its shared-memory communicator."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("kokkos", [False, True])
def test_dropin_test_program_compiles(kokkos):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    if not (cuda / "include" / "cuda_runtime.h").exists():
        pytest.skip("no CUDA headers")
    cmd = [gxx, "-std=c++17", "-fsyntax-only", "-Wall", str(ROOT / "tests" / "cpp" / "test_dropin.cpp"),
           "-I", str(ROOT / "include"), "-I", str(cuda / "include")] + (["-DDTK_FAKE_KOKKOS"] if kokkos else [])
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.parametrize("mpi", [False, True])
def test_distributed_test_program_compiles(mpi):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    if not (cuda / "include" / "cuda_runtime.h").exists():
        pytest.skip("no CUDA headers")
    cmd = [gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-pthread",
           str(ROOT / "tests" / "cpp" / "test_distributed.cpp"), "-I", str(ROOT / "include"),
           "-I", str(cuda / "include")] + (["-DDTK_FAKE_MPI"] if mpi else [])
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
