"""CPU-only checks of the boundary: the C-ABI library loads without a GPU and exports every
declared entry point, the Python structs match the C layout, host-only functions agree with
the oracle, and GPU calls fail loudly (no CPU fallback) when there is no device."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions() -> list[str]:
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?(?:int|double|void|char)\s*\*?\s*(numa_[a-z0-9_]+)\s*\(", text, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(str(lib_path))
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(lib_path):
    import numa_gpu
    assert set(declared_functions()) <= set(numa_gpu.SIGNATURES)


def test_struct_layouts_agree():
    import numa_gpu
    from oracle import oracle_lib
    for a, b in ((numa_gpu.KrylovParams, oracle_lib.KrylovParams),
                 (numa_gpu.KrylovResult, oracle_lib.KrylovResult),
                 (numa_gpu.GmresResult, oracle_lib.GmresResult)):
        assert C.sizeof(a) == C.sizeof(b)
        assert [(n, getattr(a, n).offset) for n, _ in a._fields_] == [(n, getattr(b, n).offset) for n, _ in b._fields_]
    assert C.sizeof(numa_gpu.KrylovParams) == 136
    assert C.sizeof(numa_gpu.KrylovResult) == 128


def test_default_params_match_reference(lib_path):
    import numa_gpu
    from oracle.oracle_lib import default_params
    a, b = numa_gpu.default_params(), default_params()
    for name, _ in a._fields_:
        if name == "reserved":
            continue
        assert getattr(a, name) == getattr(b, name), name


def test_forcing_matches_oracle(lib_path, oracle, ref_small):
    """detail::forcing (krylov_newton.hpp:54-65) runs on the host: no GPU needed."""
    import numa_gpu
    from oracle.oracle_lib import default_params
    rng = np.random.default_rng(3)
    for rtol in (1e-8, 1e-10):
        pg, po = numa_gpu.default_params(rtol_nl=rtol), default_params(rtol_nl=rtol)
        for _ in range(500):
            k = int(rng.integers(0, 4))
            rn, rp, ep, r0 = 10.0 ** rng.uniform(-10, 2, 4)
            assert numa_gpu.forcing(pg, k, rn, rp, ep, r0) == oracle.forcing(po, k, rn, rp, ep, r0)
    pg = numa_gpu.default_params(rtol_nl=1e-10)
    for k, rn, rp, ep, r0, expect in ref_small["forcing_rtol1e-10_res0_100"]:
        assert numa_gpu.forcing(pg, int(k), rn, rp, ep, r0) == expect


def test_status_strings(lib_path):
    import numa_gpu
    lib = numa_gpu.load()
    assert lib.numa_gpu_abi_version() == 1
    assert lib.numa_gpu_status_string(0) == b"ok"
    assert lib.numa_gpu_status_string(6) == b"no CUDA device"
    assert lib.numa_gpu_status_string(99) == b"unknown status"


def test_no_device_fails_loudly(lib_path):
    """Without a GPU the library reports NUMA_GPU_ERR_NO_DEVICE; nothing falls back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numa_gpu
    with pytest.raises(numa_gpu.NumaGPUError) as e:
        numa_gpu.Context(0)
    assert e.value.code == 6
    lib = numa_gpu.load()
    assert lib.numa_gpu_vec_create(None, 4, C.byref(C.c_void_p())) == 1
    res = numa_gpu.KrylovResult()
    assert lib.numa_gpu_solve_bratu3d_host(None, 8, 1.0, 0, 1, 0, None, None, None, C.byref(res)) == 1


def test_missing_library_is_an_import_error(tmp_path):
    import numa_gpu
    with pytest.raises(ImportError):
        numa_gpu.load(tmp_path / "nope.so")


def test_child_finalised_after_its_context_makes_no_c_call(lib_path):
    """Objects close before their context, except when the context and its children become garbage
    together: the collector clears the context's weak references to its children before it runs any
    finaliser, so a child can be finalised after the context's C handle is destroyed.  Such a child
    must drop its handle without calling its C destroy function (which would read the destroyed
    context); with the context open it calls it once."""
    import numa_gpu

    calls = []

    class RecordingLib:
        def __getattr__(self, name):
            return lambda *args: calls.append(name) or 0

    class FakeContext:
        def __init__(self, h):
            self.h = h

    kinds = [(numa_gpu.Vec, {"owned": True}), (numa_gpu.Bratu3D, {}), (numa_gpu.Burgers2D, {}),
             (numa_gpu.Brusselator2D, {}), (numa_gpu.HelmholtzMG2D, {}),
             (numa_gpu.LearnedNet, {}), (numa_gpu.PoissonMG, {}), (numa_gpu.Provider, {}),
             (numa_gpu.KrylovSpace, {}), (numa_gpu.BatchSolver, {})]
    for ctx_open in (False, True):
        calls.clear()
        for cls, extra in kinds:
            obj = object.__new__(cls)
            obj.__dict__.update(h=C.c_void_p(1), ctx=FakeContext(C.c_void_p(1) if ctx_open else None),
                                lib=RecordingLib(), **extra)
            obj.close()
            assert obj.h is None, cls.__name__
            obj.close()  # a second close (the finaliser's) does nothing
        assert len(calls) == (len(kinds) if ctx_open else 0), calls
        assert all(c.endswith("_destroy") for c in calls)
