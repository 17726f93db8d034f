"""The C++ drop-in's multi-rank path (tests/cpp/test_distributed.cpp): two
ranks as two host threads on one GPU, against the one-rank operator over the
union of the clouds and the reference's grid case; with a shared-memory
communicator, and through the MPI_Comm path over a test stand-in for MPI."""
import os
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("mpi", [False, True])
def test_cpp_distributed(dtk_lib, tmp_path, mpi):
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    exe = tmp_path / "test_distributed"
    lib_dir = ROOT / "datatransferkit_gb300"
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", str(ROOT / "tests" / "cpp" / "test_distributed.cpp"),
           "-I", str(ROOT / "include"), "-I", str(cuda / "include"), "-L", str(lib_dir), "-ldtk_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)] + \
        (["-DDTK_FAKE_MPI"] if mpi else [])
    subprocess.run(cmd, check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("PASS")
