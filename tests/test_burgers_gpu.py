"""Burgers2D and the 2D Helmholtz multigrid on the GPU, through the C ABI, against the oracle
and the reference's golden vectors (problems/burgers2d.hpp, linalg/helmholtz_mg2d.hpp,
tests/test_burgers.cpp).

Pointwise kernels (F, F'(w)d, F''(w)[d,d], the V-cycle) are bit-exact: the GPU evaluates the
reference's expressions operation for operation.  The manufactured root is formed on the host
with the C library's sin, so it is compared with the oracle built on the same machine, bit for
bit, and with the reference's fixture to 1 ulp.  Solves meet the path's parity bar: counts equal
to the reference's within +-1 (parallel reductions may move a borderline Krylov stop) and the
solution within 1e-12 relative.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.oracle_lib import default_params as oracle_params
from oracle.oracle_lib import make_point

pytestmark = pytest.mark.gpu

COUNTS = ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec")


def _G():
    import numa_gpu
    return numa_gpu


@pytest.mark.parametrize("n", [1, 2, 15, 64, 127])
def test_burgers_pointwise_bit_exact(gpu, oracle, n):
    G = _G()
    nu, dt, amp = 0.05, 0.1, 1.0
    op = G.Burgers2D(gpu, n, nu, dt, amp)
    N = 2 * n * n
    assert op.size() == N
    ex = gpu.vec(N)
    op.exact(ex)
    assert np.array_equal(ex.numpy(), oracle.burgers_exact(n, nu, dt, amp))
    w = make_point(N, 0.7) + oracle.burgers_exact(n, nu, dt, amp)
    d = make_point(N, 1.9)
    wv, dv, out = gpu.from_numpy(w), gpu.from_numpy(d), gpu.vec(N)
    op.eval(wv, out)
    assert np.array_equal(out.numpy(), oracle.burgers_eval(n, nu, dt, amp, w))
    op.jvp(wv, dv, out)
    assert np.array_equal(out.numpy(), oracle.burgers_jvp(n, nu, dt, amp, w, d))
    op.d2(wv, dv, out)
    assert np.array_equal(out.numpy(), oracle.burgers_d2(n, nu, dt, amp, w, d))


def test_burgers_reference_vectors(gpu, ref_vectors):
    """tests/test_burgers.cpp:27-48 at n = 15 against the reference's own outputs."""
    G = _G()
    n, nu, dt, amp = 15, 0.05, 0.1, 1.0
    op = G.Burgers2D(gpu, n, nu, dt, amp)
    N = 2 * n * n
    ex = gpu.vec(N)
    op.exact(ex)
    e = ex.numpy()
    # the root is formed with the host's sin: within 1 ulp of the reference machine's
    assert np.all(np.abs(e - ref_vectors["burgers_n15_exact"]) <= np.spacing(np.abs(ref_vectors["burgers_n15_exact"])))
    F = gpu.vec(N)
    op.eval(ex, F)
    assert np.linalg.norm(F.numpy()) < 1e-10 * (1 + np.linalg.norm(e))
    x, v = ref_vectors["burgers_n15_x"], ref_vectors["burgers_n15_v"]
    xv, vv, out = gpu.from_numpy(x), gpu.from_numpy(v), gpu.vec(N)
    op.jvp(xv, vv, out)
    J = out.numpy()
    op.d2(xv, vv, out)
    D = out.numpy()
    # analytic products do not depend on the root: equal to the reference's bit for bit
    assert np.array_equal(J, ref_vectors["burgers_n15_jvp"])
    assert np.array_equal(D, ref_vectors["burgers_n15_d2"])
    op.jvp(xv, vv, out, G.FD)
    assert rel_err(out.numpy(), J) < 1e-6
    assert rel_err(out.numpy(), ref_vectors["burgers_n15_jvp_fd"]) < 1e-7
    op.d2(xv, vv, out, G.FD)
    assert rel_err(out.numpy(), D) < 2e-4
    assert op.cell_reynolds() == pytest.approx(abs(amp) / (nu * (n + 1)), rel=0, abs=0)


def test_burgers_rejects_bad_arguments(gpu):
    G = _G()
    for args in ((0, 0.05, 0.1), (15, 0.0, 0.1), (15, 0.05, -1.0), (15, float("nan"), 0.1)):
        with pytest.raises(G.NumaGPUError):
            G.Burgers2D(gpu, *args)
    op = G.Burgers2D(gpu, 7, 0.05, 0.1)
    with pytest.raises(G.NumaGPUError):
        op.eval(gpu.vec(98), gpu.vec(97))


def test_hmg2d_levels(gpu, ref_small):
    G = _G()
    for n, lv in ref_small["hmg2d_levels"].items():
        assert G.HelmholtzMG2D(gpu, int(n), 10.0, 0.05).levels() == lv


def test_hmg2d_reference_vectors(gpu, ref_vectors):
    """One V-cycle of alpha I - nu Lap_h equals the reference's output bit for bit."""
    G = _G()
    for n in (15, 31):
        mg = G.HelmholtzMG2D(gpu, n, 10.0, 0.05)
        z = gpu.vec(n * n)
        mg(gpu.from_numpy(make_point(n * n, 1.0)), z)
        assert np.array_equal(z.numpy(), ref_vectors[f"hmg2d_n{n}_z"])


@pytest.mark.parametrize("n,pre,post", [(1, 2, 2), (3, 2, 2), (16, 2, 2), (63, 2, 2), (127, 2, 2),
                                        (255, 2, 2), (31, 0, 2), (31, 2, 0), (31, 1, 1), (31, 3, 1),
                                        (10, 2, 2)])
def test_hmg2d_bit_exact(gpu, oracle, n, pre, post):
    G = _G()
    alpha, nu = 25.0, 0.02
    mg = G.HelmholtzMG2D(gpu, n, alpha, nu, pre, post)
    r = make_point(n * n, 2.3)
    rv, z = gpu.from_numpy(r), gpu.vec(n * n)
    mg(rv, z)
    want = oracle.hmg2d_apply(n, alpha, nu, r, pre, post)
    assert np.array_equal(z.numpy(), want)
    mg(rv, rv)  # r and z aliased
    assert np.array_equal(rv.numpy(), want)


def test_burgers_mg_provider(gpu, oracle):
    """BurgersMGProvider applies the V-cycle of (1/dt) I - nu Lap_h to u and to v."""
    G = _G()
    n, nu, dt = 31, 0.05, 0.1
    pc = G.Provider.burgers_mg(gpu, n, nu, dt)
    r = make_point(2 * n * n, 0.4)
    z = gpu.vec(2 * n * n)
    pc.make(gpu.from_numpy(r))
    pc.apply(gpu.from_numpy(r), z)
    want = np.concatenate([oracle.hmg2d_apply(n, 1.0 / dt, nu, r[: n * n]),
                           oracle.hmg2d_apply(n, 1.0 / dt, nu, r[n * n:])])
    assert np.array_equal(z.numpy(), want)


def test_burgers_solves(gpu, oracle, ref_small, ref_vectors):
    """tests/test_burgers.cpp:55-67: every driver, with and without the multigrid provider, from the
    perturbed manufactured root at 31^2, on device handles."""
    G = _G()
    n, nu, dt, amp = 31, 0.05, 0.1, 1.0
    x0 = oracle.burgers_exact(n, nu, dt, amp) + 0.05 * np.sin(1.3 * np.arange(2 * n * n))
    op = G.Burgers2D(gpu, n, nu, dt, amp)
    for c in ref_small["burgers_solves"]:
        pc = G.Provider.create(gpu, c["precond"], op)
        x = gpu.from_numpy(x0)
        r = G.solve(op, x, c["method"], G.default_params(), pc)
        ref = c["result"]
        for k in COUNTS:
            assert abs(int(r[k]) - int(ref[k])) <= 1, (c["method"], c["precond"], k, r[k], ref[k])
        assert r["converged"] == ref["converged"]
        xo, _ = oracle.solve_burgers(n, nu, dt, amp, c["method"], c["precond"], oracle_params(), x0)
        assert rel_err(x.numpy(), xo) < 1e-12, (c["method"], c["precond"])
        assert np.linalg.norm(x.numpy()) == pytest.approx(c["solution"]["l2"], rel=1e-12)
        if c["method"] == "nk" and c["precond"] == "mg":
            assert rel_err(x.numpy(), ref_vectors["burgers_n31_nk_mg_x"]) < 1e-12


def _calibration_rows(n: int):
    return [r for r in json.loads((GOLDEN / "c1_burgers_mg.json").read_text()) if r["n"] == str(n)]


def _run_rows(gpu, n: int, rows) -> int:
    """Runs the published rows through the host-buffer entry point; returns how many match the
    published counts exactly (every row must match within +-1)."""
    G = _G()
    exact = 0
    for r in rows:
        p = G.default_params(rtol_nl=float(r["rtol"]), max_nl=int(r["max_nl"]), eta_init=float(r["eta_init"]),
                             eta_max=float(r["eta_max"]), gamma=float(r["gamma"]), alpha=float(r["alpha"]),
                             eta2_factor=float(r["eta2_factor"]), eta2_max=float(r["eta2_max"]),
                             gmres_restart=int(r["restart"]), gmres_max_iters=int(r["maxlin"]))
        _, res = G.solve_burgers2d_host(gpu, n, float(r["param"]), float(r["dt"]), float(r["amp"]),
                                        np.zeros(2 * n * n), method=r["method"], precond="mg", params=p)
        got = (res["iters"], res["n_F"], res["n_JVP"], res["n_D2"], res["n_lin_iters"], res["n_prec"])
        want = tuple(int(r[k]) for k in ("nonlinear_iters", "n_F", "n_JVP", "n_D2", "n_lin", "n_prec"))
        assert all(abs(a - b) <= 1 for a, b in zip(got, want)), (n, r["param"], r["dt"], r["method"], got, want)
        assert res["converged"] == int(r["success"])
        exact += got == want
    return exact


def test_burgers_calibration_n63(gpu):
    """The reference's published Burgers2D calibration runs at 63^2 (MG provider, u0 = 0)."""
    rows = _calibration_rows(63)
    assert len(rows) == 108
    exact = _run_rows(gpu, 63, rows)
    assert exact >= 100, f"only {exact} of 108 rows match exactly"


@pytest.mark.parametrize("n", [127, 255, 511])
def test_burgers_calibration_large(gpu, n):
    """The same published campaign at 127^2, 255^2 and 511^2 (up to 522,242 unknowns): sizes the
    CPU oracle does not run in the test suite, checked against the reference's own counts."""
    rows = _calibration_rows(n)
    assert len(rows) == 108
    exact = _run_rows(gpu, n, rows)
    assert exact >= 95, f"only {exact} of 108 rows match exactly at n={n}"
