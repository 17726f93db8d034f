"""Build recipe for the CPU oracle (test infrastructure only).

* ``_build/libdtk_oracle.so``: the FP64 restatement (dtk_oracle.cpp), g++
  -O3 -fopenmp -ffp-contract=off.  Built on every machine (here and on the
  GPU host) by ``__graft_entry__.build()``.
* ``_build/libdtk_oracle_contract.so``: the same restatement built with
  multiply-add contraction, to measure the rounding spread of the reference
  algorithm (the parity tolerance of the FP64 form is derived from it).
* ``_ref/libdtk_ref.so``: the reference's own MLS numerics headers compiled
  where they lie in the DataTransferKit tree against the project-written API
  shim in ``ref_shim/`` plus ``ref_driver.cpp``.  Built only when the
  reference sources are present (``DTK_REFERENCE_ROOT``, else a
  ``reference`` directory beside this repository); it never travels as
  source and never ships.

Both use portable flags only (no -march), so results agree between x86-64
and aarch64 hosts.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_SO = BUILD / "libdtk_oracle.so"
ORACLE_CONTRACT_SO = BUILD / "libdtk_oracle_contract.so"
REF_SO = REF_OUT / "libdtk_ref.so"

COMMON = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-std=c++17"]


def reference_root() -> Path:
    """DTK_REFERENCE_ROOT, else the DataTransferKit tree beside this repository."""
    env = os.environ.get("DTK_REFERENCE_ROOT")
    return Path(env) if env else HERE.parent.parent / "reference"


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _contract_flags():
    # Same sources with multiply-add contraction on: the build that a compiler
    # for another backend (an FMA-contracting GPU or Arm build) would make.
    # The distance between the two builds measures how far the reference
    # algorithm itself moves under equally valid roundings.
    flags = ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    return flags


def build_oracle(force: bool = False, contract: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = ORACLE_CONTRACT_SO if contract else ORACLE_SO
    deps = [HERE / "dtk_oracle.cpp", HERE / "dtk_oracle.h"]
    if force or _stale(out, deps):
        flags = [f for f in COMMON if f != "-ffp-contract=off"] + _contract_flags() if contract else COMMON
        cmd = ["g++", *flags, str(HERE / "dtk_oracle.cpp"), "-o", str(out)]
        subprocess.run(cmd, check=True)
    return out


def build_ref(force: bool = False) -> Path | None:
    root = reference_root()
    meshfree = root / "packages" / "Meshfree" / "src"
    utils = root / "packages" / "Utils" / "src"
    if not (meshfree / "DTK_DetailsSVDImpl.hpp").exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    deps = [HERE / "ref_driver.cpp", *sorted((HERE / "ref_shim").glob("*.hpp"))]
    if force or _stale(REF_SO, deps):
        cmd = ["g++", *COMMON, "-I", str(HERE / "ref_shim"), "-I", str(meshfree),
               "-I", str(utils), str(HERE / "ref_driver.cpp"), "-o", str(REF_SO)]
        subprocess.run(cmd, check=True)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_oracle(force="--force" in sys.argv, contract=True))
    print(build_ref(force="--force" in sys.argv))
