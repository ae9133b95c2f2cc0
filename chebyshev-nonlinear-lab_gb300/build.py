"""Build libnuma_gpu.so in place (sm_103a only).

    python chebyshev-nonlinear-lab_gb300/build.py [--force]

Each translation unit under csrc/ is compiled by nvcc in parallel, then linked into
chebyshev-nonlinear-lab_gb300/libnuma_gpu.so with the CUDA runtime linked statically, so the
library loads on a machine without a GPU (the symbol-export tests) and needs only the driver
where it runs.  Objects go to csrc/_build/ (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OBJ = CSRC / "_build"
LIB = HERE / "libnuma_gpu.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH, "-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC,-ffp-contract=off", "-fmad=false",
    "--extended-lambda", "-Xptxas", "-warn-spills", f"-I{INCLUDE}",
]
SOURCES = [
    "context.cu", "bratu3d.cu", "ops.cu", "poisson_mg.cu", "hmg2d.cu", "brusselator.cu", "gmres.cu", "drivers.cu", "capi.cu", "diag.cu",
    "mg_noalloc.cu", "learned.cu", "learned_net.cu", "batch.cu", "batch_solver.cu",
]
HEADERS = ["common.cuh", "numa_internal.hpp", "mg_kernels.cuh", "learned_conv.cuh", "batch_kernels.cuh"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _mtime(p: Path) -> float:
    return p.stat().st_mtime if p.exists() else -1.0


APPS = {"run_campaign_gpu": HERE / "apps" / "run_campaign_gpu.cpp"}


def build_apps(force: bool = False) -> list[Path]:
    """C++ applications over the C++ adaptor (include/numa/gpu/numa_gpu.hpp), linked to the library."""
    outs = []
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    for name, src in APPS.items():
        exe = HERE / name
        if force or _mtime(exe) < max(_mtime(src), _mtime(LIB), _mtime(INCLUDE / "numa" / "gpu" / "numa_gpu.hpp")):
            cmd = [cxx, "-std=c++20", "-O2", "-ffp-contract=off", f"-I{INCLUDE}", str(src), "-o", str(exe), f"-L{HERE}", "-lnuma_gpu",
                   f"-Wl,-rpath,{HERE}"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"building {name} failed:\n{r.stderr}")
        outs.append(exe)
    return outs


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    deps = [CSRC / h for h in HEADERS] + [INCLUDE / "numa_gpu.h"]
    dep_time = max(_mtime(d) for d in deps)

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = OBJ / (Path(src).stem + ".o")
        if force or _mtime(o) < max(_mtime(s), dep_time):
            cmd = [nvcc(), *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd))
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _mtime(LIB) < max(_mtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(*build_apps(force="--force" in sys.argv))
