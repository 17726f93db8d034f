"""Build recipe of the CUDA library ``libdtk_gb300.so`` (in-tree, sm_103a only).

Each ``csrc/*.cu`` compiles in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and the
objects link into one shared library with a C ABI (``include/dtk_gb300.h``)
and the CUDA runtime linked statically.  Objects go to ``_build/``; both are
git-ignored build products.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libdtk_gb300.so"
HEADER = HERE.parent / "include" / "dtk_gb300.h"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", *ARCH]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdtk_gb300.so")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.stem + ".o")
    deps = [src, HEADER, *CSRC.glob("*.cuh")]
    if obj.exists() and all(d.stat().st_mtime <= obj.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(_compile, srcs))
    # drop objects of removed sources
    live = {o.name for o in objs}
    for o in BUILD.glob("*.o"):
        if o.name not in live:
            o.unlink()
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        # -ldl: the NVTX ranges find a profiling tool with dlopen when one is attached
        cmd = [nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-ldl"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv))
