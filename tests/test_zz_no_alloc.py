"""The V-cycle entry point that allocates nothing (numa_gpu_mg_apply_noalloc).

It exists for callers that cannot allocate device memory when they apply the preconditioner:
another library's solver callback that must not allocate or free on every application, and
programs with a device-memory budget fixed up front.  These tests call it through the C ABI and
hold it to the existing entry point numa_gpu_mg_apply: the FP64 V-cycle has no reductions, so
the two must agree bit for bit (the tolerance the V-cycle tests use), on two calls in a row.
This file is collected last; it also passes when run alone in a fresh process.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle_lib import make_point

pytestmark = pytest.mark.gpu


def _G():
    import numa_gpu
    return numa_gpu


@pytest.mark.parametrize("n,pre,post", [(63, 2, 2), (31, 2, 2), (15, 1, 3), (7, 0, 2), (16, 2, 2), (64, 2, 2), (1, 2, 2)])
def test_noalloc_matches_mg_apply_twice(gpu, n, pre, post):
    G = _G()
    N = n ** 3
    mg = G.PoissonMG(gpu, n, pre, post)
    rng = np.random.default_rng(n)
    for call, r in enumerate((make_point(N, 1.0), rng.uniform(-1.0, 1.0, N))):
        dr = gpu.from_numpy(r)
        z_ref, z_na = gpu.vec(N), gpu.vec(N)
        z_na.fill(-7.0)  # whatever the output held must not matter
        mg(dr, z_ref)
        rc = G.mg_apply_noalloc(n, dr, z_na, pre, post)
        assert rc == 0, (call, rc)
        gpu.sync()
        assert np.array_equal(z_na.numpy(), z_ref.numpy()), (n, call)


def test_noalloc_allocates_nothing_after_set_up(gpu):
    import torch
    G = _G()
    n = 63
    N = n ** 3
    dr, dz = gpu.from_numpy(make_point(N, 1.0)), gpu.vec(N)
    assert G.mg_apply_noalloc(n, dr, dz) == 0  # first call on the device: set-up
    gpu.sync()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert G.mg_apply_noalloc(n, dr, dz) == 0
    gpu.sync()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_what_does_not_fit(gpu):
    G = _G()
    lib = G.load()
    TOO_LARGE, INVALID = 9, 1
    big = gpu.vec(8)
    # 65^3 needs 2*65^3 + 3*32^3 doubles > NUMA_GPU_NOALLOC_MAX_DOUBLES; 127^3 and 255^3 too
    for n in (65, 127, 255, 5000):
        assert G.mg_apply_noalloc(n, big, gpu.vec(8)) == TOO_LARGE
    assert lib.numa_gpu_status_string(TOO_LARGE) == b"too large for the fixed scratch array"
    v = gpu.vec(27)
    assert G.mg_apply_noalloc(0, v, gpu.vec(27)) == INVALID
    assert G.mg_apply_noalloc(3, v, v) == INVALID  # r and z must differ
    assert G.mg_apply_noalloc(3, v, gpu.vec(27), pre=-1) == INVALID


@pytest.mark.parametrize("n,pre,post", [(31, 2, 2), (15, 0, 2)])
def test_noalloc_captured_in_a_graph(gpu, n, pre, post):
    """One uncaptured call, then one call captured into a CUDA graph on a side stream (global
    capture mode, which fails the capture on any forbidden runtime call); two replays of the graph
    on fresh right-hand sides give the V-cycle bit for bit, the pre = 0 case through the memset node."""
    import torch
    G = _G()
    N = n ** 3
    mg = G.PoissonMG(gpu, n, pre, post)
    rng = np.random.default_rng(100 + n)
    r = torch.zeros(N, dtype=torch.float64, device="cuda")
    z = torch.full((N,), -3.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    lib = G.load()
    assert lib.numa_gpu_mg_apply_noalloc(n, pre, post, r.data_ptr(), z.data_ptr(), None) == 0
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="global"):
        rc = lib.numa_gpu_mg_apply_noalloc(n, pre, post, r.data_ptr(), z.data_ptr(), side.cuda_stream)
    assert rc == 0
    for rep in range(2):
        rh = rng.uniform(-1.0, 1.0, N)
        r.copy_(torch.from_numpy(rh))
        z.fill_(5.0)
        graph.replay()
        torch.cuda.synchronize()
        dr, z_ref = gpu.from_numpy(rh), gpu.vec(N)
        mg(dr, z_ref)
        gpu.sync()
        assert np.array_equal(z.cpu().numpy(), z_ref.numpy()), (n, pre, rep)
