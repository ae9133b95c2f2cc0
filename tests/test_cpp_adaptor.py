"""The C++20 adaptor (include/numa/gpu/numa_gpu.hpp) from the reference's side.

* CPU: where the reference headers are present, the reference's own templates (newton_krylov,
  chebyshev_inexact, tf_chebyshev_2018, gmres) compile unchanged against the GPU operator and
  provider; the adaptor header compiles on its own.
* GPU: a C++ program using only the adaptor runs the native drivers at 31^3 and reproduces the
  reference's counts."""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import PKG, ROOT



def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_adaptor_header_compiles():
    r = subprocess.run([_gxx(), "-std=c++20", "-fsyntax-only", f"-I{ROOT / 'include'}", "-x", "c++", "-"],
                       input='#include "numa/gpu/numa_gpu.hpp"\nint main(){return 0;}\n', text=True,
                       capture_output=True)
    assert r.returncode == 0, r.stderr


def _ref_include():
    from oracle.build import reference_root
    root = reference_root()  # $NUMA_REFERENCE_ROOT, or ../reference beside the repository
    if root is None:
        pytest.skip("reference headers not present on this machine (set NUMA_REFERENCE_ROOT)")
    return root / "include"


def test_reference_templates_build_against_gpu_types(lib_path, tmp_path):
    """The reference's templates compile against the GPU types and the program links against
    libnuma_gpu.so (it cannot run here: the reference's headers exist only where there is no GPU)."""
    REF_INCLUDE = _ref_include()
    exe = tmp_path / "dropin_reference_templates"
    r = subprocess.run([_gxx(), "-std=c++20", "-O1", f"-I{REF_INCLUDE}", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "cpp" / "dropin_reference_templates.cpp"), "-o", str(exe),
                        f"-L{PKG}", "-lnuma_gpu", f"-Wl,-rpath,{PKG}"], text=True, capture_output=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


@pytest.mark.gpu
def test_native_driver_program(lib_path, tmp_path, ref_counts):
    exe = tmp_path / "native_driver"
    r = subprocess.run([_gxx(), "-std=c++20", "-O2", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "cpp" / "native_driver.cpp"), "-o", str(exe), f"-L{PKG}",
                        "-lnuma_gpu", f"-Wl,-rpath,{PKG}"], text=True, capture_output=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), "31"], text=True, capture_output=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    nk = out.stdout.split("\n")[0].split()
    ch = out.stdout.split("\n")[1].split()
    ref = {c["method"]: c["result"] for c in ref_counts if c["tag"] == "lambda6_n31"}
    assert [int(v) for v in nk[1:5]] == [ref["nk"]["iters"], ref["nk"]["n_F"], ref["nk"]["n_JVP"], ref["nk"]["n_prec"]]
    assert [int(v) for v in ch[1:6]] == [ref["cheb"]["iters"], ref["cheb"]["n_F"], ref["cheb"]["n_JVP"],
                                         ref["cheb"]["n_D2"], ref["cheb"]["n_prec"]]
    mx = out.stdout.split("\n")[2].split()
    assert mx[0] == "mixed" and int(mx[3]) == 1 and abs(int(mx[1]) - ref["nk"]["iters"]) <= 1
    assert float(mx[4]) < 1e-8
