"""The reference's MLS operator tests in C++ against the header-only drop-in
(include/dtk/DTK_MovingLeastSquaresOperator.hpp) linked to libdtk_gb300.so,
built without Kokkos and with a Kokkos stand-in (the virtual apply then takes
the reference's Kokkos::View value types)."""
import os
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("kokkos", [False, True])
def test_cpp_dropin(dtk_lib, tmp_path, kokkos):
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    exe = tmp_path / "test_dropin"
    lib_dir = ROOT / "datatransferkit_gb300"
    cmd = ["g++", "-std=c++17", "-O2", str(ROOT / "tests" / "cpp" / "test_dropin.cpp"),
           "-I", str(ROOT / "include"), "-I", str(cuda / "include"), "-L", str(lib_dir),
           "-ldtk_gb300", "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib_dir}",
           "-o", str(exe)] + (["-DDTK_FAKE_KOKKOS"] if kokkos else [])
    subprocess.run(cmd, check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("PASS")
