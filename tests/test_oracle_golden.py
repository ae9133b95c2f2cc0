"""The oracle (CPU restatement, oracle/numa_oracle.cpp) pinned against the reference.

Three sources of truth, none of them the oracle itself:
* the reference's published count table (docs/research/R1_OPERATOR_INTERFACE.md:113-121);
* fixtures produced by the reference's own headers compiled here (tests/golden/make_golden.py);
* the reference's published calibration rows (experiments/c1/amendment01/calibration_combined.csv).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle_lib import default_params, make_point

COUNT_KEYS = ("converged", "iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec")

# docs/research/R1_OPERATOR_INTERFACE.md:113-121 (n = 16, N = 4096, lambda = 1, default params):
# (precond, method) -> (iter, n_F, n_JVP, n_D2, n_prec, res_rel printed with 2 digits)
PUBLISHED_SMOKE = {
    ("mg", "nk"): (4, 5, 11, 0, 15, 9.9e-11),
    ("mg", "cheb"): (4, 5, 20, 4, 28, 1.0e-10),
    ("mg", "rec"): (4, 5, 18, 4, 30, 1.0e-10),
    ("jacobi", "nk"): (5, 6, 74, 0, 79, 4.8e-09),
    ("jacobi", "cheb"): (5, 6, 123, 5, 133, 4.8e-09),
    ("jacobi", "rec"): (5, 6, 99, 5, 112, 4.8e-09),
}


@pytest.mark.parametrize("key", sorted(PUBLISHED_SMOKE))
def test_published_smoke_table(oracle, key):
    precond, method = key
    _, r = oracle.solve(16, 1.0, method, precond, default_params())
    it, nf, njvp, nd2, nprec, rr = PUBLISHED_SMOKE[key]
    assert (r["iters"], r["n_F"], r["n_JVP"], r["n_D2"], r["n_prec"]) == (it, nf, njvp, nd2, nprec)
    assert f"{r['res'] / r['res0']:.1e}" == f"{rr:.1e}"
    assert r["converged"] == 1


def _cases(ref_counts, cheap=True):
    return [c for c in ref_counts if not cheap or c["n"] <= 31]


def test_reference_counts(oracle, ref_counts):
    """Every nonlinear solve recorded from the reference: identical counts, same solution."""
    for c in ref_counts:
        if c["n"] > 31:
            continue
        p = default_params(**c["params"])
        x, r = oracle.solve(c["n"], c["lam"], c["method"], c["precond"], p)
        for k in COUNT_KEYS:
            assert r[k] == c["result"][k], (c["tag"], c["method"], k, r[k], c["result"][k])
        if not c["count_stable"]:
            continue
        # the final residual is a cancellation-dominated difference: compare loosely
        assert r["res"] == pytest.approx(c["result"]["res"], rel=2e-2)
        s = c["solution"]
        assert np.linalg.norm(x) == pytest.approx(s["l2"], rel=1e-12)
        assert x.sum() == pytest.approx(s["sum"], rel=1e-12, abs=1e-12)


def test_reference_counts_n63(oracle, ref_counts):
    for c in ref_counts:
        if c["n"] != 63 or c["method"] not in ("nk", "cheb"):
            continue
        x, r = oracle.solve(c["n"], c["lam"], c["method"], c["precond"], default_params(**c["params"]))
        for k in COUNT_KEYS:
            assert r[k] == c["result"][k], (c["tag"], c["method"], k)
        assert np.linalg.norm(x) == pytest.approx(c["solution"]["l2"], rel=1e-12)


def test_solution_n31_lambda6(oracle, ref_vectors):
    """31^3, lambda = 6, rtol 1e-10, GMRES(30): the full solution vector to 1e-12."""
    x, r = oracle.solve(31, 6.0, "nk", "mg", default_params(rtol_nl=1e-10, gmres_restart=30))
    assert r["iters"] == 5 and r["n_JVP"] == 12 and r["n_prec"] == 17
    assert rel_err(x, ref_vectors["solution_n31_lambda6_nk"]) < 1e-12


@pytest.mark.parametrize("n", [6, 8])
def test_operator_vectors(oracle, ref_vectors, n):
    u, v = ref_vectors[f"op_n{n}_u"], ref_vectors[f"op_n{n}_v"]
    w = make_point(n ** 3, 0.5)
    assert rel_err(oracle.eval(n, 1.0, u), ref_vectors[f"op_n{n}_eval"]) < 1e-15
    assert rel_err(oracle.jvp(n, 1.0, u, v, 0), ref_vectors[f"op_n{n}_jvp"]) < 1e-15
    assert rel_err(oracle.jvp(n, 1.0, u, v, 1), ref_vectors[f"op_n{n}_jvp_fd"]) < 1e-12
    assert rel_err(oracle.d2(n, 1.0, u, w, 0), ref_vectors[f"op_n{n}_d2"]) < 1e-15
    assert rel_err(oracle.d2(n, 1.0, u, w, 1), ref_vectors[f"op_n{n}_d2_fd"]) < 1e-10
    assert rel_err(oracle.jacobi_diag(n, 1.0, u), ref_vectors[f"op_n{n}_jacobi_diag"]) < 1e-15
    # the reference tests' own tolerances (tests/test_operators.cpp:46, :60)
    assert rel_err(oracle.jvp(n, 1.0, u, v, 1), oracle.jvp(n, 1.0, u, v, 0)) < 1e-6
    assert rel_err(oracle.d2(n, 1.0, u, w, 1), oracle.d2(n, 1.0, u, w, 0)) < 1e-4


def test_vcycle_n15(oracle, ref_vectors):
    b = make_point(15 ** 3, 1.0)
    z = oracle.mg_apply(15, b)
    assert np.array_equal(z, ref_vectors["mg_n15_z"])  # no reductions in a V-cycle: bit-exact


def test_mg_levels(oracle, ref_small):
    for n, lv in ref_small["mg_levels"].items():
        assert oracle.mg_levels(int(n)) == lv
    assert oracle.mg_levels(0) == ref_small["mg_levels_errors"]["n0"] == -1
    assert oracle.mg_levels(7, -1, 2) == ref_small["mg_levels_errors"]["pre_neg"] == -1
    assert oracle.mg_levels(15) == 4  # tests/test_operators.cpp:194


def test_gmres_cases(oracle, ref_small, ref_vectors):
    x, g = oracle.gmres_bratu3d(8, 1.0, np.zeros(512), make_point(512, 1.0), 1e-10, 40, 400, "none")
    assert g == ref_small["gmres_n8"]
    assert rel_err(x, ref_vectors["gmres_n8_x"]) < 1e-13
    for n in (15, 31):
        _, g = oracle.gmres_poisson_mg(n, make_point(n ** 3, 1.0), 1e-8, 50, 200)
        ref = ref_small[f"gmres_poisson_mg_n{n}"]
        assert g["iters"] == ref["iters"] and g["converged"] == ref["converged"]
        assert g["rel_res"] == pytest.approx(ref["rel_res"], rel=1e-8)
    N = 15 ** 3
    b1 = make_point(N, 1.0)
    z, u, k, r1, r2 = oracle.gmres_recycle_pair(15, 1.0, np.full(N, 0.1), b1, b1 * b1, 1e-8, 50, 100, "mg")
    assert k == ref_small["recycle_n15_k"]
    for a, b in ((r1, ref_small["recycle_n15_first"]), (r2, ref_small["recycle_n15_second"])):
        assert (a["iters"], a["matvecs"], a["precs"], a["converged"]) == (b["iters"], b["matvecs"], b["precs"],
                                                                        b["converged"])
    assert rel_err(u, ref_vectors["recycle_n15_u"]) < 1e-12


def test_forcing(oracle, ref_small):
    p = default_params(rtol_nl=1e-10)
    for k, rn, rp, ep, r0, expect in ref_small["forcing_rtol1e-10_res0_100"]:
        assert oracle.forcing(p, int(k), rn, rp, ep, r0) == expect


def test_c1_calibration_n31(oracle, c1_rows):
    """The reference's published calibration runs (Bratu3D, Jacobi, n = 31, four tuning
    candidates, seven lambdas, NK / Cheb / Cheb+recycle): identical counts."""
    rows = [r for r in c1_rows if r["n"] == "31"]
    assert len(rows) == 84
    meth = {"nk": "nk", "cheb": "cheb", "rec": "rec"}
    for r in rows:
        p = default_params(rtol_nl=float(r["rtol"]), max_nl=int(r["max_nl"]), eta_init=float(r["eta_init"]),
                           eta_max=float(r["eta_max"]), gamma=float(r["gamma"]), alpha=float(r["alpha"]),
                           eta2_factor=float(r["eta2_factor"]), eta2_max=float(r["eta2_max"]),
                           gmres_restart=int(r["restart"]), gmres_max_iters=int(r["maxlin"]))
        _, res = oracle.solve(31, float(r["param"]), meth[r["method"]], "jacobi", p)
        got = (res["iters"], res["n_F"], res["n_JVP"], res["n_D2"], res["n_lin_iters"], res["n_prec"])
        want = tuple(int(r[k]) for k in ("nonlinear_iters", "n_F", "n_JVP", "n_D2", "n_lin", "n_prec"))
        assert got == want, (r["param"], r["method"], r["internal_candidate_id"])
        assert res["res"] / res["res0"] == pytest.approx(float(r["residual_rel"]), rel=1e-3)


# ------------------------------------------------------------------ the benchmark's sizes
def test_oracle_matches_reference_at_127(oracle):
    """The oracle port at 127^3 (lambda = 6, rtol 1e-10, GMRES(30), MG V(2,2)) against the reference's
    own run (tests/golden/reference_large.*): equal counts, solution to 1e-12 at the sampled points.
    (The 255^3 fixtures pin the GPU path in tests/test_parity_large_gpu.py; the oracle takes ~10 s
    there on one thread, too long for this suite.)"""
    import json

    from conftest import GOLDEN
    cases = {(c["n"], c["method"]): c for c in json.loads((GOLDEN / "reference_large.json").read_text())}
    vec = np.load(GOLDEN / "reference_large.npz")
    c = cases[(127, "nk")]
    x, r = oracle.solve(127, c["lam"], "nk", "mg", default_params(rtol_nl=1e-10, gmres_restart=30))
    assert all(r[k] == c["result"][k] for k in COUNT_KEYS)
    idx = vec["idx_n127"]
    assert rel_err(x[idx], vec["x_n127_nk"]) < 1e-12
    assert float(x.max()) == pytest.approx(c["solution"]["max"], rel=1e-12)


def test_batch_fixture_instance_table():
    """The batched configuration's instance table (numa_gpu.batch_config_instances: 128 instances,
    n from {31, 63, 127}, lambda ~ U[1, 6.5], seed 42) is the one the reference solved for
    tests/golden/reference_batch.*, and every instance there converged."""
    import json

    import numa_gpu
    from conftest import GOLDEN
    fx = json.loads((GOLDEN / "reference_batch.json").read_text())
    table = numa_gpu.batch_config_instances(128, seed=42)
    assert [(e["n"], e["lam"]) for e in fx["instances"]] == table
    assert all(e["result"]["converged"] == 1 for e in fx["instances"])
    assert {n for n, _ in table} == {31, 63, 127}
