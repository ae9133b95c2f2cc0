"""The Brusselator family on the GPU, through the C ABI.

Brusselator1DStep and BrusselatorJacobi (problems/brusselator1d.hpp) against the reference's own
fixtures and its 144 published calibration rows: pointwise kernels bit-exact (the previous state
is formed with the C library's sin on the host, so quantities that read it agree to a few ulp
across machines), solves with counts within +-1 and solutions within 1e-12.

The periodic 2D Brusselator and its coupled-block multigrid against the CPU restatement (no
reference code exists for them: parity unpinned): F, J v, F'' and the FP64 V-cycle bit for bit,
every driver's counts within +-1 and solution within 1e-12; the FP32 V-cycle within FP32 rounding
of the FP64 one, and the mixed solve (FP32 multigrid and FP32 Jacobian products inside FGMRES)
within 1e-8 of the FP64 solve.
At the full 2048^2 size, size-independent properties: the steady state is a fixed point of the
time stepping, and a periodic translation of the initial state by a multiple of the coarsest
spacing translates the solution.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.oracle_lib import default_params as oracle_params

pytestmark = pytest.mark.gpu

COUNTS = ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec")
PRM = dict(A=1.0, B=3.4, Du=0.002, Dv=0.002, dt=0.01)


def _G():
    import numa_gpu
    return numa_gpu


@pytest.fixture(scope="module")
def bvec():
    return dict(np.load(GOLDEN / "reference_brusselator.npz"))


def _gparams(G, d: dict):
    p = G.default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _opar(d: dict):
    p = oracle_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


# ------------------------------------------------------------------------------ Brusselator1D
def test_bruss1d_pointwise(gpu, bvec):
    G = _G()
    n, dt = 31, 0.01
    op = G.Brusselator1D(gpu, n, dt)
    assert op.size() == 62
    prev = gpu.vec(62)
    op.previous(prev)
    assert rel_err(prev.numpy(), bvec["prev"]) < 1e-15
    x, d, out = gpu.from_numpy(bvec["x"]), gpu.from_numpy(bvec["d"]), gpu.vec(62)
    op.eval(x, out)
    assert rel_err(out.numpy(), bvec["eval_x"]) < 1e-13
    for mode, tag in ((0, ""), (1, "_fd")):
        op.jvp(x, d, out, mode)
        ref = bvec[f"jvp{tag}"]
        if mode == 0:
            assert np.array_equal(out.numpy(), ref)
        else:
            assert rel_err(out.numpy(), ref) < 1e-8
        op.d2(x, d, out, mode)
        ref = bvec[f"d2{tag}"]
        if mode == 0:
            assert np.array_equal(out.numpy(), ref)
        else:
            assert rel_err(out.numpy(), ref) < 1e-5
    pc = G.Provider.brusselator_jacobi(op)
    z = gpu.vec(62)
    pc.make(x)
    pc.apply(d, z)
    assert np.array_equal(z.numpy(), bvec["jacobi_x_d"])


def test_bruss1d_solves(gpu, bvec):
    G = _G()
    cases = json.loads((GOLDEN / "reference_brusselator.json").read_text())["solves"]
    for c in cases:
        op = G.Brusselator1D(gpu, c["n"], c["dt"])
        x = gpu.vec(op.size())
        op.previous(x)
        pc = G.Provider.create(gpu, c["precond"], op)
        r = G.solve(op, x, c["method"], _gparams(G, c["params"]), pc)
        for k in COUNTS:
            assert abs(int(r[k]) - int(c["result"][k])) <= 1, (c["tag"], c["method"], c["precond"], k, r[k])
        assert r["converged"] == c["result"]["converged"]
        assert np.linalg.norm(x.numpy()) == pytest.approx(c["solution"]["l2"], rel=1e-12)
        if c["precond"] == "jacobi":
            assert rel_err(x.numpy(), bvec[f"x_{c['tag']}_{c['method']}"]) < 1e-12


def test_bruss1d_calibration_rows(gpu):
    """The reference's 144 published Brusselator calibration runs through the host entry point."""
    G = _G()
    rows = json.loads((GOLDEN / "c1_brusselator_jacobi.json").read_text())
    assert len(rows) == 144
    exact = 0
    for r in rows:
        p = G.default_params(rtol_nl=float(r["rtol"]), max_nl=int(r["max_nl"]), eta_init=float(r["eta_init"]),
                             eta_max=float(r["eta_max"]), gamma=float(r["gamma"]), alpha=float(r["alpha"]),
                             eta2_factor=float(r["eta2_factor"]), eta2_max=float(r["eta2_max"]),
                             gmres_restart=int(r["restart"]), gmres_max_iters=int(r["maxlin"]))
        _, res = G.solve_brusselator1d_host(gpu, int(r["n"]), float(r["param"]), None, r["method"], "jacobi", p)
        got = (res["iters"], res["n_F"], res["n_JVP"], res["n_D2"], res["n_lin_iters"], res["n_prec"])
        want = tuple(int(r[k]) for k in ("nonlinear_iters", "n_F", "n_JVP", "n_D2", "n_lin", "n_prec"))
        assert all(abs(a - b) <= 1 for a, b in zip(got, want)), (r["n"], r["param"], r["method"], got, want)
        assert res["converged"] == int(r["success"])
        exact += got == want
    assert exact >= 140, f"only {exact} of 144 rows match exactly"


# ------------------------------------------------------------------------------ Brusselator2D
def _state(n, seed=20261203):
    import numa_gpu
    return numa_gpu.brusselator2d_initial(n, 1.0, 3.4, seed)


def test_bruss2d_initial_state():
    z = _state(64)
    assert z.shape == (2 * 64 * 64,)
    assert abs(z[:4096].mean() - 1.0) < 1e-3 and abs(z[4096:].mean() - 3.4) < 1e-3
    assert 0.009 < z[:4096].std() < 0.011
    assert np.array_equal(z, _state(64))


@pytest.mark.parametrize("n", [3, 16, 33, 64])
def test_bruss2d_pointwise_bit_exact(gpu, oracle, n):
    G = _G()
    prm = G.brusselator_params()
    op = G.Brusselator2D(gpu, n, prm)
    N = 2 * n * n
    prev = _state(n)
    w = prev + 0.02 * np.sin(0.37 * np.arange(N))
    d = np.sin(0.31 * np.arange(N) + 0.2)
    op.set_previous(gpu.from_numpy(prev))
    wv, dv, out = gpu.from_numpy(w), gpu.from_numpy(d), gpu.vec(N)
    op.eval(wv, out)
    assert np.array_equal(out.numpy(), oracle.bruss2d_eval(n, PRM, prev, w))
    op.jvp(wv, dv, out)
    assert np.array_equal(out.numpy(), oracle.bruss2d_jvp(n, PRM, prev, w, d))
    op.d2(wv, dv, out)
    assert np.array_equal(out.numpy(), oracle.bruss2d_d2(n, PRM, prev, w, d))
    op.jvp(wv, dv, out, G.FD)
    assert rel_err(out.numpy(), oracle.bruss2d_jvp(n, PRM, prev, w, d, 1)) < 1e-8
    op.jvp(wv, dv, out, G.ANALYTIC_FP32)  # the mixed path's product: FP32 arithmetic
    assert rel_err(out.numpy(), oracle.bruss2d_jvp(n, PRM, prev, w, d)) < 1e-5
    op.d2(wv, dv, out, G.FD)
    assert rel_err(out.numpy(), oracle.bruss2d_d2(n, PRM, prev, w, d, 1)) < 1e-5


@pytest.mark.parametrize("n", [4, 6, 12, 16, 64, 130, 256])
def test_bmg2d_fp64_bit_exact(gpu, oracle, n):
    """One V-cycle, every level shape: a single level (6, and 130 = 2 x 65 solved by plain sweeps
    on the whole grid), a two-level hierarchy ending at 6, and power-of-two hierarchies."""
    G = _G()
    N = 2 * n * n
    mg = G.BrussMG2D(gpu, n, G.brusselator_params(), G.FP64)
    assert mg.levels() == oracle.bmg2d_levels(n)
    w = _state(n, 3)
    r = np.sin(0.13 * np.arange(N) + 0.3)
    mg.set_state(gpu.from_numpy(w))
    rv, z = gpu.from_numpy(r), gpu.vec(N)
    mg.apply(rv, z)
    zo = oracle.bmg2d_apply(n, PRM, w, r)
    assert np.array_equal(z.numpy(), zo)
    mg.apply(rv, rv)  # aliased r and z
    assert np.array_equal(rv.numpy(), zo)


@pytest.mark.parametrize("n", [16, 128, 512])
def test_bmg2d_fp32(gpu, oracle, n):
    G = _G()
    N = 2 * n * n
    mg = G.BrussMG2D(gpu, n, G.brusselator_params(), G.FP32)
    w = _state(n, 4)
    r = np.cos(0.07 * np.arange(N))
    mg.set_state(gpu.from_numpy(w))
    z = gpu.vec(N)
    mg.apply(gpu.from_numpy(r), z)
    assert rel_err(z.numpy(), oracle.bmg2d_apply(n, PRM, w, r)) < 2e-5


@pytest.mark.parametrize("method", ["nk", "cheb", "rec", "tf2018"])
@pytest.mark.parametrize("precond", ["mg", "none"])
def test_bruss2d_step_parity(gpu, oracle, method, precond):
    G = _G()
    n = 64
    prev = _state(n)
    kp = dict(rtol_nl=1e-10, gmres_restart=40, gmres_max_iters=400)
    xo, ro = oracle.solve_bruss2d(n, PRM, prev, method, precond, oracle_params(**kp))
    op = G.Brusselator2D(gpu, n, G.brusselator_params())
    op.set_previous(gpu.from_numpy(prev))
    x = gpu.from_numpy(prev)
    pc = G.Provider.create(gpu, precond, op)
    r = G.solve(op, x, method, G.default_params(**kp), pc)
    for k in COUNTS:
        assert abs(int(r[k]) - int(ro[k])) <= 1, (method, precond, k, r[k], ro[k])
    assert r["converged"] == 1
    assert rel_err(x.numpy(), xo) < 1e-12


def test_bruss2d_mixed_and_advance(gpu, oracle):
    """Three implicit-Euler steps: FP64 multigrid against the oracle stepping, and the FP32
    multigrid inside FGMRES(40) within 1e-8 of it."""
    G = _G()
    n, steps = 64, 3
    x0 = _state(n)
    kp = dict(rtol_nl=1e-10, gmres_restart=40, gmres_max_iters=400)
    xo = x0.copy()
    for _ in range(steps):
        xo, ro = oracle.solve_bruss2d(n, PRM, xo, "nk", "mg", oracle_params(**kp))
        assert ro["converged"] == 1
    op = G.Brusselator2D(gpu, n, G.brusselator_params())
    x = gpu.from_numpy(x0)
    res = op.advance(x, steps, "nk", G.default_params(**kp), G.Provider.brusselator_mg(op, G.FP64))
    assert len(res) == steps and all(r["converged"] == 1 for r in res)
    assert rel_err(x.numpy(), xo) < 1e-12
    xm, resm = G.brusselator2d_advance_host(gpu, n, x0, steps, mg_precision=G.FP32,
                                            kparams=G.default_params(flexible=1, jvp_precision=G.FP32, **kp))
    assert all(r["converged"] == 1 for r in resm)
    assert rel_err(xm, xo) < 1e-8
    # the state moved (the homogeneous state is unstable for B > 1 + A^2)
    assert rel_err(xo, x0) > 1e-4


def test_bruss2d_full_size_properties(gpu):
    """2048^2 (8.4M unknowns): the steady state is a fixed point, and translating the initial state
    by multiples of 512 points (the coarsest level's spacing, so every level translates with it)
    translates the FP32-multigrid solution."""
    G = _G()
    n = 2048
    nn = n * n
    kp = G.default_params(rtol_nl=1e-10, gmres_restart=40, gmres_max_iters=400, flexible=1, jvp_precision=G.FP32)
    ss = np.concatenate([np.full(nn, 1.0), np.full(nn, 3.4)])
    xs, rs = G.brusselator2d_advance_host(gpu, n, ss, 2, kparams=kp)
    assert np.array_equal(xs, ss) and all(r["iters"] == 0 for r in rs)
    x0 = _state(n)
    x1, r1 = G.brusselator2d_advance_host(gpu, n, x0, 2, kparams=kp)
    assert all(r["converged"] == 1 and r["res"] <= 1e-10 * r["res0"] for r in r1)

    def roll(a):
        return np.roll(a.reshape(2, n, n), (512, -1024), axis=(1, 2)).ravel()

    x2, r2 = G.brusselator2d_advance_host(gpu, n, roll(x0), 2, kparams=kp)
    assert all(r["converged"] == 1 for r in r2)
    assert rel_err(x2, roll(x1)) < 1e-9
