"""Batched solves (numa_gpu_solve_batch): instances of uneven grid size and lambda solved concurrently
by worker threads must give each instance exactly the counts of solving it alone (the kernels are
deterministic for a given grid), whatever the number of workers."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _G():
    import numa_gpu
    return numa_gpu


def test_batch_matches_individual_solves(gpu):
    G = _G()
    rng = np.random.default_rng(42)
    inst = [(int(n), float(lam)) for n, lam in zip(rng.choice([15, 31], 10), rng.uniform(1.0, 6.5, 10))]
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1)
    res4, wall4 = G.solve_batch(inst, "nk", G.FP32, p, workers=4)
    res1, _ = G.solve_batch(inst, "nk", G.FP32, p, workers=1)
    assert wall4 > 0.0
    keys = ("converged", "iters", "n_F", "n_JVP", "n_lin_iters", "n_prec")
    for (n, lam), a, b in zip(inst, res4, res1):
        assert a["converged"] == 1 and a["res_rel"] <= 1e-10
        assert all(a[k] == b[k] for k in keys)
        op = G.Bratu3D(gpu, n, lam)
        x = gpu.vec(n ** 3)
        r = G.newton_krylov(op, x, p, G.Provider.poisson_mg(gpu, n, precision=G.FP32))
        assert all(a[k] == r[k] for k in keys), (n, lam)


def test_batch_rejects_bad_input():
    G = _G()
    with pytest.raises(G.NumaGPUError):
        G.solve_batch([(0, 1.0)])
    with pytest.raises(G.NumaGPUError):
        G.solve_batch([(15, 1.0)], workers=0)


def test_batch_executor_reuses_state_across_batches(gpu):
    """numa_gpu_batch_*: the same executor solving two batches (the second one after its workers have
    set up their grid sizes) returns the counts of the one-shot call, and the methods other than NK run
    through it too."""
    G = _G()
    inst = [(15, 2.0), (31, 5.5), (15, 6.0), (23, 1.0), (31, 3.3)]
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1)
    keys = ("converged", "iters", "n_F", "n_JVP", "n_lin_iters", "n_prec")
    ref, _ = G.solve_batch(inst, "nk", G.FP32, p, workers=3)
    ex = G.BatchExecutor(workers=3)
    try:
        for _ in range(2):
            got, wall = ex.solve(inst, "nk", G.FP32, p)
            assert wall > 0.0
            for a, b in zip(got, ref):
                assert all(a[k] == b[k] for k in keys)
        for method in ("cheb", "rec", "tf2018"):
            got, _ = ex.solve([(15, 2.0), (31, 3.3), (23, 1.0)], method, G.FP64, G.default_params(rtol_nl=1e-8))
            assert all(r["converged"] == 1 for r in got), method
    finally:
        ex.close()


def test_batch_autotune(gpu):
    """The schedule autotuner tries each worker count on the batch, keeps the fastest, and the
    executor then solves with it; counts do not depend on the schedule."""
    G = _G()
    inst = [(15, 2.0), (31, 5.5), (15, 6.0), (23, 1.0), (31, 3.3), (23, 4.4)]
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1)
    keys = ("converged", "iters", "n_F", "n_JVP", "n_lin_iters", "n_prec")
    ex = G.BatchExecutor(workers=4)
    try:
        chosen, tune = ex.autotune(inst, (1, 2, 4), "nk", G.FP32, p)
        assert chosen in (1, 2, 4) and set(tune) == {1, 2, 4} and all(t > 0 for t in tune.values())
        assert tune[chosen] == min(tune.values())
        got, _ = ex.solve(inst, "nk", G.FP32, p)
        ex.set_workers(1)
        one, _ = ex.solve(inst, "nk", G.FP32, p)
        for a, b in zip(got, one):
            assert all(a[k] == b[k] for k in keys)
        with pytest.raises(G.NumaGPUError):
            ex.set_workers(5)
        with pytest.raises(G.NumaGPUError):
            ex.autotune(inst, (8,), "nk", G.FP32, p)
    finally:
        ex.close()
