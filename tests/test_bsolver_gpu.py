"""The batched solver (numa_gpu_bsolver_*): all instances advanced together, one launch per operation
over a packed instance table, scalar decisions on the device, Arnoldi steps and line-search trials
replayed as CUDA graphs.

Its oracle is the reference solving each instance alone (the campaign runner's per-instance loop,
apps/run_campaign.cpp:344-475): tests/golden/reference_batch.* holds the reference's own run of
every instance of the batched configuration (128 instances, n from {31, 63, 127}, lambda ~ U[1, 6.5],
seed 42; Newton-Krylov, GMRES(30), MG V(2,2), rtol 1e-10).  The batched solver runs the mixed path
(FP32 V-cycle, FP32 Jacobian products and Krylov basis, FP64 residual and updates), so its bar is the
mixed path's: every instance converged, the Newton count within +-1 and the solution within 1e-8.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

pytestmark = pytest.mark.gpu


def _G():
    import numa_gpu
    return numa_gpu


def _mixed(G, **kw):
    return G.default_params(rtol_nl=1e-10, gmres_restart=30, flexible=1, jvp_precision=G.FP32, orth=G.CGS1, **kw)


def _sample_idx(N: int, target: int) -> np.ndarray:
    """The fixture's strided sample (tests/golden/make_golden.py strided_sample)."""
    stride = max(1, N // target) | 1
    return np.arange(stride // 2, N, stride, dtype=np.int64)


@pytest.mark.parametrize("jac", [0, 1])
def test_bsolver_config_matches_reference(gpu, jac):
    G = _G()
    fx = json.loads((GOLDEN / "reference_batch.json").read_text())
    vec = np.load(GOLDEN / "reference_batch.npz")
    inst = G.batch_config_instances(128, seed=42)
    assert [(e["n"], e["lam"]) for e in fx["instances"]] == inst
    bs = G.BatchSolver(gpu, inst, _mixed(G, jvp_tight=jac, coarse_jacobian=jac))
    try:
        res, secs, xs = bs.solve(want_x=True)
    finally:
        bs.close()
    assert secs > 0.0
    for i, e in enumerate(fx["instances"]):
        r, ref = res[i], e["result"]
        assert r["converged"] == 1 and r["res_rel"] <= 1e-10, (i, r)
        assert abs(int(r["iters"]) - int(ref["iters"])) <= 1, (i, r, ref)
        n = e["n"]
        x = xs[i]
        want = vec[f"x_{i}"]
        assert rel_err(x[_sample_idx(n ** 3, 512)], want) < 1e-8, i
        assert float(x.max()) == pytest.approx(e["solution"]["max"], rel=1e-8)


def test_bsolver_matches_single_instance_mixed_path(gpu):
    """Each instance of a small uneven batch against the same instance solved alone by the
    single-instance mixed path: the same Newton count and n_F, linear iterations within 2, and
    solutions within 1e-10 of each other."""
    G = _G()
    inst = [(63, 6.2), (31, 1.5), (127, 4.0), (31, 6.4), (63, 2.5), (31, 3.0)]
    p = _mixed(G)
    bs = G.BatchSolver(gpu, inst, p)
    try:
        res, _, xs = bs.solve(want_x=True)
    finally:
        bs.close()
    for (n, lam), r, xb in zip(inst, res, xs):
        op = G.Bratu3D(gpu, n, lam)
        x = gpu.vec(n ** 3).fill(0.0)
        rs = G.newton_krylov(op, x, p, G.Provider.poisson_mg(gpu, n, precision=G.FP32))
        assert r["converged"] == rs["converged"] == 1
        assert (r["iters"], r["n_F"]) == (rs["iters"], rs["n_F"]), (n, lam, r, rs)
        assert abs(int(r["n_lin_iters"]) - int(rs["n_lin_iters"])) <= 2, (n, lam, r, rs)
        assert rel_err(xb, x.numpy()) < 1e-10, (n, lam)


def test_bsolver_jacobian_tail_and_tight_products(gpu):
    """The benchmark's form of the batched solver: the multigrid tail (levels n <= 15) solving with the
    Jacobian of each iterate (coarse_jacobian) and products of FP32 accuracy in the linear solves with
    forcing terms below 1e-5 (jvp_tight).  Against each instance solved alone by the single-instance path
    with the same settings (the Jacobian-aware provider): the same Newton count and n_F, linear
    iterations within 2, solutions within 1e-10; and fewer Newton steps and linear iterations in total
    than the batched solver with the Poisson tail and FP32 products (the batched configuration's mix)."""
    G = _G()
    inst = [(63, 6.2), (31, 1.5), (127, 4.0), (31, 6.4), (63, 2.5), (127, 6.0), (31, 3.0)]
    p = _mixed(G, jvp_tight=1, coarse_jacobian=1)
    bs = G.BatchSolver(gpu, inst, p)
    try:
        res, _, xs = bs.solve(want_x=True)
    finally:
        bs.close()
    for (n, lam), r, xb in zip(inst, res, xs):
        op = G.Bratu3D(gpu, n, lam)
        x = gpu.vec(n ** 3).fill(0.0)
        rs = G.newton_krylov(op, x, _mixed(G, jvp_tight=1), G.Provider.jacobian_mg(gpu, n))
        assert r["converged"] == rs["converged"] == 1 and r["res_rel"] <= 1e-10
        assert (r["iters"], r["n_F"]) == (rs["iters"], rs["n_F"]), (n, lam, r, rs)
        assert abs(int(r["n_lin_iters"]) - int(rs["n_lin_iters"])) <= 2, (n, lam, r, rs)
        assert rel_err(xb, x.numpy()) < 1e-10, (n, lam)
    bp = G.BatchSolver(gpu, inst, _mixed(G))
    try:
        rp, _, _ = bp.solve()
    finally:
        bp.close()
    assert sum(r["iters"] for r in res) < sum(r["iters"] for r in rp)
    assert sum(r["n_lin_iters"] for r in res) < sum(r["n_lin_iters"] for r in rp)


def test_bsolver_restarted_cycles(gpu):
    """FGMRES(2) forces restarts (the residual r = F - J z recomputed, a new cycle from RN32(r)/||r||):
    the instances still converge, to the FP64 single-instance solution within 1e-8."""
    G = _G()
    inst = [(31, 6.0), (63, 5.0), (31, 2.0)]
    p = G.default_params(rtol_nl=1e-10, gmres_restart=2, gmres_max_iters=500, flexible=1, jvp_precision=G.FP32,
                         orth=G.CGS1)
    bs = G.BatchSolver(gpu, inst, p)
    try:
        res, _, xs = bs.solve(want_x=True)
    finally:
        bs.close()
    for (n, lam), r, xb in zip(inst, res, xs):
        assert r["converged"] == 1 and r["res_rel"] <= 1e-10, r
        assert r["n_lin_iters"] > 2 * r["iters"]  # more iterations than one 2-step cycle per Newton step
        op = G.Bratu3D(gpu, n, lam)
        x = gpu.vec(n ** 3).fill(0.0)
        G.newton_krylov(op, x, G.default_params(rtol_nl=1e-10, gmres_restart=30), G.Provider.poisson_mg(gpu, n))
        assert rel_err(xb, x.numpy()) < 1e-8


def test_bsolver_repeatable_and_tuning_independent(gpu, tmp_path):
    """A second solve repeats the first bit for bit (fixed reduction order); other tile shapes give
    the same counts and solutions within 1e-10; the autotuner keeps the fastest candidate and its
    cache answers the second call.  Another tile shape sums the norms and inner products in another
    order, which moves FP32 roundings of the basis: measured 1e-14 to 2.3e-12 between shapes, against
    8e-13 to 1.2e-11 between the mixed path's solution and the FP64 one for these instances."""
    G = _G()
    inst = [(31, 6.0), (63, 3.5), (31, 1.2), (63, 6.5)]
    bs = G.BatchSolver(gpu, inst, _mixed(G))
    try:
        r1, _, x1 = bs.solve(want_x=True)
        r2, _, x2 = bs.solve(want_x=True)
        assert r1 == [dict(r, seconds=a["seconds"]) for r, a in zip(r2, r1)]
        assert all(np.array_equal(a, b) for a, b in zip(x1, x2))
        bs.set_tuning(2, 4096)
        assert bs.tuning() == {"planes": 2, "elems_per_block": 4096}
        r3, _, x3 = bs.solve(want_x=True)
        keys = ("converged", "iters", "n_F", "n_JVP", "n_lin_iters", "n_prec")
        assert all(all(a[k] == b[k] for k in keys) for a, b in zip(r1, r3))
        assert all(rel_err(a, b) < 1e-10 for a, b in zip(x3, x1))
        cache = tmp_path / "tuning.json"
        t = bs.autotune((4, 8), (8192, 16384), cache=cache)
        assert (t["planes"], t["elems_per_block"]) in {(4, 8192), (4, 16384), (8, 8192), (8, 16384)}
        assert t["seconds"][f"{t['planes']}x{t['elems_per_block']}"] == min(t["seconds"].values())
        again = bs.autotune((4, 8), (8192, 16384), cache=cache)
        assert again["cached"] and (again["planes"], again["elems_per_block"]) == (t["planes"], t["elems_per_block"])
    finally:
        bs.close()


def test_bsolver_rejects_unsupported_input(gpu):
    G = _G()
    for inst in ([(21, 1.0)], [(15, 1.0)], [(2047, 1.0)]):
        with pytest.raises(G.NumaGPUError) as e:
            G.BatchSolver(gpu, inst, _mixed(G))
        assert e.value.code == 8  # NUMA_GPU_ERR_NOT_SUPPORTED
    with pytest.raises(G.NumaGPUError):
        G.BatchSolver(gpu, [(31, 1.0)], G.default_params(gmres_restart=0))
