"""The oracle's Burgers2D / HelmholtzMG2D (the second multigrid family) pinned against the
reference: fixtures from the reference's headers (tests/golden/make_golden.py) and the
reference's published Burgers2D calibration rows (experiments/c1/amendment01/calibration_combined.csv)."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.oracle_lib import default_params, make_point

COUNTS = ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec", "converged")


@pytest.fixture(scope="module")
def burgers_rows():
    return json.loads((GOLDEN / "c1_burgers_mg.json").read_text())


def test_burgers_vectors(oracle, ref_vectors):
    n, nu, dt, amp = 15, 0.05, 0.1, 1.0
    exact = oracle.burgers_exact(n, nu, dt, amp)
    assert np.array_equal(exact, ref_vectors["burgers_n15_exact"])
    F = oracle.burgers_eval(n, nu, dt, amp, exact)
    assert np.array_equal(F, ref_vectors["burgers_n15_eval_exact"])
    assert np.linalg.norm(F) < 1e-10 * (1 + np.linalg.norm(exact))  # tests/test_burgers.cpp:27-32
    x, v = ref_vectors["burgers_n15_x"], ref_vectors["burgers_n15_v"]
    J = oracle.burgers_jvp(n, nu, dt, amp, x, v)
    D = oracle.burgers_d2(n, nu, dt, amp, x, v)
    assert np.array_equal(J, ref_vectors["burgers_n15_jvp"])
    assert np.array_equal(D, ref_vectors["burgers_n15_d2"])
    assert rel_err(oracle.burgers_jvp(n, nu, dt, amp, x, v, 1), ref_vectors["burgers_n15_jvp_fd"]) < 1e-12
    # the reference test's FD-vs-analytic bounds (tests/test_burgers.cpp:34-48)
    assert rel_err(oracle.burgers_jvp(n, nu, dt, amp, x, v, 1), J) < 1e-6
    assert rel_err(oracle.burgers_d2(n, nu, dt, amp, x, v, 1), D) < 2e-4


def test_helmholtz_mg2d(oracle, ref_small, ref_vectors):
    for n, lv in ref_small["hmg2d_levels"].items():
        assert oracle.hmg2d_levels(int(n), 10.0, 0.05) == lv
    assert oracle.hmg2d_levels(31, 10.0, 0.05) == 5  # tests/test_burgers.cpp:50-53
    for n in (15, 31):
        z = oracle.hmg2d_apply(n, 10.0, 0.05, make_point(n * n, 1.0))
        assert np.array_equal(z, ref_vectors[f"hmg2d_n{n}_z"])


def test_burgers_solves(oracle, ref_small, ref_vectors):
    """tests/test_burgers.cpp:55-67: NK and Chebyshev converge from the perturbed manufactured
    root; every method with and without the multigrid provider reproduces the reference."""
    x0 = oracle.burgers_exact(31, 0.05, 0.1, 1.0) + 0.05 * np.sin(1.3 * np.arange(2 * 31 * 31))
    for c in ref_small["burgers_solves"]:
        x, r = oracle.solve_burgers(31, 0.05, 0.1, 1.0, c["method"], c["precond"], default_params(), x0)
        for k in COUNTS:
            assert r[k] == c["result"][k], (c["method"], c["precond"], k)
        assert np.linalg.norm(x) == pytest.approx(c["solution"]["l2"], rel=1e-13)
        if c["method"] == "nk" and c["precond"] == "mg":
            assert rel_err(x, ref_vectors["burgers_n31_nk_mg_x"]) < 1e-13


def test_burgers_calibration_n63(oracle, burgers_rows):
    """The reference's published Burgers2D calibration runs at 63^2 (MG provider, u0 = 0)."""
    rows = [r for r in burgers_rows if r["n"] == "63"]
    assert len(rows) == 108
    for r in rows:
        p = default_params(rtol_nl=float(r["rtol"]), max_nl=int(r["max_nl"]), eta_init=float(r["eta_init"]),
                           eta_max=float(r["eta_max"]), gamma=float(r["gamma"]), alpha=float(r["alpha"]),
                           eta2_factor=float(r["eta2_factor"]), eta2_max=float(r["eta2_max"]),
                           gmres_restart=int(r["restart"]), gmres_max_iters=int(r["maxlin"]))
        _, res = oracle.solve_burgers(63, float(r["param"]), float(r["dt"]), float(r["amp"]), r["method"], "mg", p)
        got = (res["iters"], res["n_F"], res["n_JVP"], res["n_D2"], res["n_lin_iters"], res["n_prec"])
        want = tuple(int(r[k]) for k in ("nonlinear_iters", "n_F", "n_JVP", "n_D2", "n_lin", "n_prec"))
        assert got == want, (r["param"], r["dt"], r["method"], r["internal_candidate_id"], got, want)
