"""The oracle's Brusselator family (CPU).

Brusselator1DStep / BrusselatorJacobi are pinned against the reference: fixtures made by its own
headers (tests/golden/make_golden.py --brusselator) and its published calibration rows
(experiments/c1/amendment01/calibration_combined.csv), every one of which the restatement
reproduces count for count.  The periodic 2D Brusselator and its coupled-block multigrid have no
reference code (parity unpinned): they are checked here through properties of the mathematics —
finite differences against the analytic derivatives, the steady state as an exact root, periodic
translation equivariance, and the V-cycle's contraction.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.oracle_lib import default_params

COUNTS = ("converged", "iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec")
PRM = dict(A=1.0, B=3.4, Du=0.002, Dv=0.002, dt=0.01)


@pytest.fixture(scope="module")
def bvec():
    return dict(np.load(GOLDEN / "reference_brusselator.npz"))


@pytest.fixture(scope="module")
def bsolves():
    return json.loads((GOLDEN / "reference_brusselator.json").read_text())["solves"]


@pytest.fixture(scope="module")
def brows():
    return json.loads((GOLDEN / "c1_brusselator_jacobi.json").read_text())


def kparams(**kw):
    return default_params(**kw)


def test_bruss1d_vectors(oracle, bvec):
    """F, J v, F'' and the block-Jacobi solve on the reference test's point (test_brusselator.cpp:13-53)."""
    n, dt = 31, 0.01
    assert np.array_equal(oracle.bruss1d_previous(n, dt), bvec["prev"])
    assert np.array_equal(oracle.bruss1d_eval(n, dt, bvec["prev"]), bvec["eval_prev"])
    assert np.array_equal(oracle.bruss1d_eval(n, dt, bvec["x"]), bvec["eval_x"])
    x, d = bvec["x"], bvec["d"]
    for mode, tag in ((0, ""), (1, "_fd")):
        assert np.array_equal(oracle.bruss1d_jvp(n, dt, x, d, mode), bvec[f"jvp{tag}"])
        assert np.array_equal(oracle.bruss1d_d2(n, dt, x, d, mode), bvec[f"d2{tag}"])
    assert np.array_equal(oracle.bruss1d_jacobi_apply(n, dt, x, d), bvec["jacobi_x_d"])
    # the reference test's bounds: FD vs analytic J v < 2e-6, F'' < 5e-4 (relative to 1 + ||analytic||)
    jv, dd = bvec["jvp"], bvec["d2"]
    assert np.linalg.norm(bvec["jvp_fd"] - jv) / (1 + np.linalg.norm(jv)) < 2e-6
    assert np.linalg.norm(bvec["d2_fd"] - dd) / (1 + np.linalg.norm(dd)) < 5e-4
    # the previous state is not a root (test_brusselator.cpp:30-38)
    assert np.isfinite(np.linalg.norm(bvec["eval_prev"])) and np.linalg.norm(bvec["eval_prev"]) > 0


def test_bruss1d_solves(oracle, bsolves, bvec):
    """Every method with and without BrusselatorJacobi, from the previous state."""
    for c in bsolves:
        p = default_params()
        for k, v in c["params"].items():
            setattr(p, k, v)
        x, r = oracle.solve_bruss1d(c["n"], c["dt"], c["method"], c["precond"], p)
        for k in COUNTS:
            assert r[k] == c["result"][k], (c["tag"], c["method"], c["precond"], k)
        assert r["res"] == pytest.approx(c["result"]["res"], rel=1e-12)
        assert np.linalg.norm(x) == pytest.approx(c["solution"]["l2"], rel=1e-14)
        if c["precond"] == "jacobi":
            assert np.array_equal(x, bvec[f"x_{c['tag']}_{c['method']}"])
    # NK and Chebyshev converge from the previous state (test_brusselator.cpp:55-67)
    assert all(c["result"]["converged"] for c in bsolves if c["tag"] == "test" and c["method"] in ("nk", "cheb"))


def test_bruss1d_calibration_rows(oracle, brows):
    """The reference's 144 published Brusselator calibration runs (BrusselatorJacobi, natural start)."""
    assert len(brows) == 144
    for r in brows:
        p = kparams(rtol_nl=float(r["rtol"]), max_nl=int(r["max_nl"]), eta_init=float(r["eta_init"]),
                    eta_max=float(r["eta_max"]), gamma=float(r["gamma"]), alpha=float(r["alpha"]),
                    eta2_factor=float(r["eta2_factor"]), eta2_max=float(r["eta2_max"]),
                    gmres_restart=int(r["restart"]), gmres_max_iters=int(r["maxlin"]))
        _, res = oracle.solve_bruss1d(int(r["n"]), float(r["param"]), r["method"], r["precond"], p)
        got = (res["iters"], res["n_F"], res["n_JVP"], res["n_D2"], res["n_lin_iters"], res["n_prec"])
        want = tuple(int(r[k]) for k in ("nonlinear_iters", "n_F", "n_JVP", "n_D2", "n_lin", "n_prec"))
        assert got == want, (r["n"], r["param"], r["method"], r["internal_candidate_id"])
        assert res["converged"] == int(r["success"])
        assert res["res"] / res["res0"] == pytest.approx(float(r["residual_rel"]), rel=1e-6)


def _state(n, seed=20261203):
    z = np.random.default_rng(seed).standard_normal(2 * n * n)
    z[: n * n] = 1.0 + 0.01 * z[: n * n]
    z[n * n:] = 3.4 + 0.01 * z[n * n:]
    return z


def test_bruss2d_derivatives_and_root(oracle):
    n = 32
    prev = _state(n)
    w = prev + 0.02 * np.sin(0.37 * np.arange(2 * n * n))
    d = np.sin(0.31 * np.arange(2 * n * n) + 0.2)
    J = oracle.bruss2d_jvp(n, PRM, prev, w, d)
    assert rel_err(oracle.bruss2d_jvp(n, PRM, prev, w, d, 1), J) < 1e-7
    D = oracle.bruss2d_d2(n, PRM, prev, w, d)
    assert rel_err(oracle.bruss2d_d2(n, PRM, prev, w, d, 1), D) < 1e-6
    # linearity of J in the direction
    assert rel_err(oracle.bruss2d_jvp(n, PRM, prev, w, 3.0 * d), 3.0 * J) < 1e-15
    # the homogeneous steady state u = A, v = B/A with itself as the previous level is an exact root
    ss = np.concatenate([np.full(n * n, 1.0), np.full(n * n, 3.4)])
    assert np.all(oracle.bruss2d_eval(n, PRM, ss, ss) == 0.0)


def test_bruss2d_periodic_equivariance(oracle):
    """Translating the grid periodically commutes with F and J (the stencil sums are in a fixed
    order, so bit for bit)."""
    n = 24
    prev = _state(n, 5)
    w = prev + 0.01 * np.cos(0.7 * np.arange(2 * n * n))
    d = np.sin(0.11 * np.arange(2 * n * n))

    def roll(a, di, dj):
        return np.roll(a.reshape(2, n, n), (di, dj), axis=(1, 2)).ravel()

    for di, dj in ((1, 0), (0, 5), (7, 3)):
        F = oracle.bruss2d_eval(n, PRM, prev, w)
        Fr = oracle.bruss2d_eval(n, PRM, roll(prev, di, dj), roll(w, di, dj))
        assert np.array_equal(Fr, roll(F, di, dj))
        J = oracle.bruss2d_jvp(n, PRM, prev, w, d)
        assert np.array_equal(oracle.bruss2d_jvp(n, PRM, prev, roll(w, di, dj), roll(d, di, dj)), roll(J, di, dj))


def test_bmg2d_levels_and_contraction(oracle):
    assert oracle.bmg2d_levels(2048) == 10
    assert oracle.bmg2d_levels(64) == 5
    assert oracle.bmg2d_levels(12) == 2
    assert oracle.bmg2d_levels(6) == 1
    assert oracle.bmg2d_levels(7) == -1 and oracle.bmg2d_levels(2) == -1
    n = 64
    prev = _state(n)
    e = np.random.default_rng(1).standard_normal(2 * n * n)
    for _ in range(3):
        z = oracle.bmg2d_apply(n, PRM, prev, oracle.bruss2d_jvp(n, PRM, prev, prev, e))
        e2 = e - z
        assert np.linalg.norm(e2) < 0.2 * np.linalg.norm(e)
        e = e2


@pytest.mark.parametrize("method", ["nk", "cheb", "rec", "tf2018"])
def test_bruss2d_step_converges(oracle, method):
    n = 32
    prev = _state(n)
    p = default_params(rtol_nl=1e-10, gmres_restart=40, gmres_max_iters=400)
    x, r = oracle.solve_bruss2d(n, PRM, prev, method, "mg", p)
    assert r["converged"] == 1 and r["res"] <= 1e-10 * r["res0"]
    assert np.linalg.norm(oracle.bruss2d_eval(n, PRM, prev, x)) <= 1e-10 * r["res0"] * 1.01
    x2, r2 = oracle.solve_bruss2d(n, PRM, prev, method, "none", p)
    assert r2["converged"] == 1 and rel_err(x2, x) < 1e-9
    # the multigrid cuts the Krylov work
    assert r["n_lin_iters"] < r2["n_lin_iters"]
