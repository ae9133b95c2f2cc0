"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the CPU restatement (numa_oracle.cpp), g++ + OpenMP,
  floating-point contraction off.  Built wherever the tests or bench.py's CPU baseline run.
* ``oracle/_ref/libnuma_ref.so`` — ref_driver.cpp compiled against the reference's own headers
  where they lie: the reference checkout named by the environment variable ``NUMA_REFERENCE_ROOT``,
  or else a checkout called ``reference`` beside this repository's directory.  Built only where
  the reference is present; it generates the golden fixtures under tests/golden/.

Run ``python oracle/build.py`` to build both.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"


def reference_root() -> Path | None:
    """The reference checkout: $NUMA_REFERENCE_ROOT, else ``../reference`` beside this repository.

    None when neither holds the reference's headers (as on a machine that only runs the tests)."""
    env = os.environ.get("NUMA_REFERENCE_ROOT")
    cands = [Path(env)] if env else [ROOT.parent / "reference"]
    for c in cands:
        if (c / "include" / "numa" / "problems" / "bratu3d.hpp").is_file():
            return c
    return None


COMMON = ["-O3", "-DNDEBUG", "-std=c++20", "-fopenmp", "-fPIC", "-shared"]


def _cxx() -> str:
    return os.environ.get("CXX", shutil.which("g++") or "g++")


def _stale(out: Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU restatement into oracle/_build/liboracle.so."""
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    srcs = [HERE / "numa_oracle.cpp", ROOT / "include" / "numa_gpu.h"]
    if force or _stale(out, srcs):
        cmd = [_cxx(), *COMMON, "-ffp-contract=off", str(HERE / "numa_oracle.cpp"), "-o", str(out)]
        subprocess.run(cmd, check=True)
    return out


def reference_available() -> bool:
    return reference_root() is not None


def build_ref(force: bool = False) -> Path | None:
    """Compile ref_driver.cpp against the reference headers (None if they are absent).

    Flags follow the reference's Release build (CMakeLists.txt: -O3, C++20, OpenMP with
    NUMA_HAS_OPENMP=1, no -march), so x86-64 code has no FMA contraction, like the oracle.
    """
    root = reference_root()
    if root is None:
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libnuma_ref.so"
    srcs = [HERE / "ref_driver.cpp", ROOT / "include" / "numa_gpu.h"]
    if force or _stale(out, srcs):
        cmd = [_cxx(), *COMMON, "-DNUMA_HAS_OPENMP=1", f"-I{root / 'include'}",
               str(HERE / "ref_driver.cpp"), "-o", str(out)]
        subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
