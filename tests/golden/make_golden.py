"""Generate the golden fixtures in this directory from the reference itself.

Run from the repository root, where the reference is present:

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py [--brusselator | --large]

(one thread: OpenMP's reduction order is not fixed across runs with more threads, and the
reference's published calibration runs used one thread).

It compiles oracle/ref_driver.cpp against the reference's own headers (oracle/build.py) and
records what the reference computes:

* ``reference_counts.json`` — nonlinear solves (iteration / call counts, residuals, solution
  statistics) for the reference's published smoke table (n=16, lambda=1), the 31^3 and 63^3
  lambda=6 rtol=1e-10 GMRES(30) MG configuration (analytic and finite-difference derivatives,
  all four methods) and the reference tests' small cases;
* ``reference_vectors.npz`` — operator, V-cycle and GMRES outputs on the reference tests'
  deterministic inputs (make_point, tests/test_operators.cpp:19-23), and the 31^3 lambda=6
  Newton-Krylov solution;
* ``c1_bratu_jacobi.json`` / ``c1_burgers_mg.json`` — the reference's own published calibration
  rows for Bratu3D with the Jacobi preconditioner and for Burgers2D with its multigrid provider
  (experiments/c1/amendment01/calibration_combined.csv, repetition 1), read from the CSV, not
  recomputed; ``c1_csv_header.txt`` — that file's header line.
"""
from __future__ import annotations

import csv
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.build import build_ref, reference_root  # noqa: E402
from oracle.oracle_lib import Oracle, default_params, make_point  # noqa: E402

REFERENCE_ROOT = reference_root()  # $NUMA_REFERENCE_ROOT, or ../reference beside the repository
if REFERENCE_ROOT is None:
    raise SystemExit("the reference checkout was not found: set NUMA_REFERENCE_ROOT")
CALIBRATION_CSV = REFERENCE_ROOT / "experiments/c1/amendment01/calibration_combined.csv"


def solution_stats(x: np.ndarray) -> dict:
    return {"sum": float(x.sum()), "l2": float(np.linalg.norm(x)), "max": float(x.max()),
            "min": float(x.min()), "first": float(x[0]), "center": float(x[len(x) // 2])}


def params_dict(p) -> dict:
    return {name: getattr(p, name) for name, _ in p._fields_ if name != "reserved"}


def counts_cases():
    cases = []
    # Published smoke table (docs/research/R1_OPERATOR_INTERFACE.md:113-121), default params.
    for precond in ("mg", "jacobi"):
        for method in ("nk", "cheb", "rec"):
            cases.append(dict(tag="smoke16", n=16, lam=1.0, method=method, precond=precond, params={}))
    # 31^3 / 63^3, lambda = 6, u0 = 0, rtol 1e-10, GMRES(30), V(2,2) on the full hierarchy.
    north = dict(rtol_nl=1e-10, gmres_restart=30)
    for n in (31, 63):
        for method in ("nk", "cheb", "rec", "tf2018"):
            cases.append(dict(tag=f"lambda6_n{n}", n=n, lam=6.0, method=method, precond="mg", params=north))
    for method in ("nk", "cheb"):
        cases.append(dict(tag="lambda6_n31_fd", n=31, lam=6.0, method=method, precond="mg",
                          params=dict(north, jvp_mode=1, d2_mode=1)))
    # Reference test cases (tests/test_operators.cpp:91-120, :277-297; apps/check_openmp_consistency.cpp).
    for method in ("nk", "cheb"):
        cases.append(dict(tag="test_n8_jacobi", n=8, lam=1.0, method=method, precond="jacobi", params={}))
    cases.append(dict(tag="test_n15_mg_rec", n=15, lam=1.0, method="rec", precond="mg", params={}))
    cases.append(dict(tag="consistency_n17", n=17, lam=1.0, method="rec", precond="mg", params={}))
    # Jacobi-preconditioned 31^3 with C1 tuning candidate t01.
    t01 = dict(rtol_nl=1e-8, eta_init=0.25, gmres_restart=30, gmres_max_iters=200)
    for method in ("nk", "cheb", "rec", "tf2018"):
        cases.append(dict(tag="c1_t01_n31", n=31, lam=6.9305946741898339, method=method,
                          precond="jacobi", params=t01,
                          # tf2018 with Jacobi: the first GMRES stops at its 200-iteration cap at
                          # eta = 1e-8, so rounding decides the outcome (the reference itself gives
                          # different counts from run to run with several threads)
                          count_stable=method != "tf2018"))
    # An odd grid that is not 2^m - 1 (15 -> 7 -> 3 -> 1 vs 21 -> 10: a two-level hierarchy).
    cases.append(dict(tag="odd21", n=21, lam=3.0, method="nk", precond="mg", params=dict(rtol_nl=1e-10)))
    return cases


def main() -> None:
    if os.environ.get("OMP_NUM_THREADS") != "1":
        raise SystemExit("run with OMP_NUM_THREADS=1")
    if build_ref() is None:
        raise SystemExit("reference headers not found; fixtures can only be made where the reference is")
    ref = Oracle.reference()
    out_counts = []
    vectors = {}
    for c in counts_cases():
        c.setdefault("count_stable", True)
        p = default_params(**c["params"])
        x, res = ref.solve(c["n"], c["lam"], c["method"], c["precond"], p)
        entry = dict(c, params=params_dict(p), result={k: res[k] for k in (
            "converged", "iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec",
            "res0", "res")}, solution=solution_stats(x))
        out_counts.append(entry)
        if c["tag"] == "lambda6_n31" and c["method"] == "nk":
            vectors["solution_n31_lambda6_nk"] = x
        print(c["tag"], c["method"], c["precond"], entry["result"]["iters"], entry["result"]["n_JVP"],
              entry["result"]["n_prec"])
    (HERE / "reference_counts.json").write_text(json.dumps(out_counts, indent=1))

    # Operators on make_point inputs (tests/test_operators.cpp:39-61).
    for n in (6, 8):
        N = n ** 3
        u, v = make_point(N, 0.3), make_point(N, 1.0)
        vectors[f"op_n{n}_u"] = u
        vectors[f"op_n{n}_v"] = v
        vectors[f"op_n{n}_eval"] = ref.eval(n, 1.0, u)
        vectors[f"op_n{n}_jvp"] = ref.jvp(n, 1.0, u, v, 0)
        vectors[f"op_n{n}_jvp_fd"] = ref.jvp(n, 1.0, u, v, 1)
        vectors[f"op_n{n}_d2"] = ref.d2(n, 1.0, u, make_point(N, 0.5), 0)
        vectors[f"op_n{n}_d2_fd"] = ref.d2(n, 1.0, u, make_point(N, 0.5), 1)
        vectors[f"op_n{n}_jacobi_diag"] = ref.jacobi_diag(n, 1.0, u)
    # One V-cycle at n = 15 (tests/test_operators.cpp:189-205).
    vectors["mg_n15_z"] = ref.mg_apply(15, make_point(15 ** 3, 1.0))
    # GMRES on the Bratu Jacobian at 0, n = 8 (tests/test_operators.cpp:78-89).
    x, g = ref.gmres_bratu3d(8, 1.0, np.zeros(512), make_point(512, 1.0), 1e-10, 40, 400, "none")
    vectors["gmres_n8_x"] = x
    gm = {"gmres_n8": g}
    # MG-preconditioned GMRES on the Poisson operator (tests/test_operators.cpp:207-233).
    for n in (15, 31):
        x, g = ref.gmres_poisson_mg(n, make_point(n ** 3, 1.0), 1e-8, 50, 200)
        gm[f"gmres_poisson_mg_n{n}"] = g
    # Recycled second solve (tests/test_operators.cpp:235-275).
    N = 15 ** 3
    b1 = make_point(N, 1.0)
    z, u, k, r1, r2 = ref.gmres_recycle_pair(15, 1.0, np.full(N, 0.1), b1, b1 * b1, 1e-8, 50, 100, "mg")
    vectors["recycle_n15_z"], vectors["recycle_n15_u"] = z, u
    gm["recycle_n15_first"], gm["recycle_n15_second"], gm["recycle_n15_k"] = r1, r2, k
    # MG level counts and constructor errors (poisson_mg.hpp:26-64).
    gm["mg_levels"] = {str(n): ref.mg_levels(n) for n in (1, 2, 3, 7, 15, 16, 21, 31, 63, 127, 255)}
    gm["mg_levels_errors"] = {"n0": ref.mg_levels(0), "pre_neg": ref.mg_levels(7, -1, 2)}
    # Forcing term (krylov_newton.hpp:54-65) on a grid of arguments.
    p = default_params(rtol_nl=1e-10)
    forcing = []
    for k_ in (0, 1, 3):
        for rn, rp, ep in ((1.0, 2.0, 0.5), (1e-3, 1e-1, 0.9), (1e-8, 1e-6, 1e-3), (5.0, 5.0, 0.2)):
            forcing.append([k_, rn, rp, ep, 100.0, ref.forcing(p, k_, rn, rp, ep, 100.0)])
    gm["forcing_rtol1e-10_res0_100"] = forcing
    # Burgers2D and HelmholtzMG2D (tests/test_burgers.cpp): the 15^2 manufactured problem, its
    # operators on the test's points, V-cycles, and solves from the test's perturbed start.
    bn, bnu, bdt, bamp = 15, 0.05, 0.1, 1.0
    exact = ref.burgers_exact(bn, bnu, bdt, bamp)
    vectors["burgers_n15_exact"] = exact
    vectors["burgers_n15_eval_exact"] = ref.burgers_eval(bn, bnu, bdt, bamp, exact)
    bx = 0.5 * np.sin(0.37 * np.arange(2 * bn * bn) + 0.5)
    bv = 0.7 * np.sin(0.37 * np.arange(2 * bn * bn) + 1.1)
    vectors["burgers_n15_x"], vectors["burgers_n15_v"] = bx, bv
    for mode, tag in ((0, ""), (1, "_fd")):
        vectors[f"burgers_n15_jvp{tag}"] = ref.burgers_jvp(bn, bnu, bdt, bamp, bx, bv, mode)
        vectors[f"burgers_n15_d2{tag}"] = ref.burgers_d2(bn, bnu, bdt, bamp, bx, bv, mode)
    gm["hmg2d_levels"] = {str(n): ref.hmg2d_levels(n, 10.0, 0.05) for n in (1, 3, 7, 15, 16, 31, 63)}
    for n in (15, 31):
        vectors[f"hmg2d_n{n}_z"] = ref.hmg2d_apply(n, 10.0, 0.05, make_point(n * n, 1.0))
    burgers_solves = []
    x0 = ref.burgers_exact(31, 0.05, 0.1, 1.0) + 0.05 * np.sin(1.3 * np.arange(2 * 31 * 31))
    for method in ("nk", "cheb", "rec", "tf2018"):
        for precond in ("mg", "none"):
            x, res = ref.solve_burgers(31, 0.05, 0.1, 1.0, method, precond, default_params(), x0)
            burgers_solves.append(dict(n=31, nu=0.05, dt=0.1, amp=1.0, method=method, precond=precond,
                                       start="exact+0.05sin(1.3i)", result={k: res[k] for k in (
                                           "converged", "iters", "n_F", "n_JVP", "n_D2", "n_lin_iters",
                                           "n_lin_failures", "n_prec", "res0", "res")},
                                       solution=solution_stats(x)))
            if method == "nk" and precond == "mg":
                vectors["burgers_n31_nk_mg_x"] = x
    gm["burgers_solves"] = burgers_solves
    (HERE / "reference_small.json").write_text(json.dumps(gm, indent=1))
    np.savez_compressed(HERE / "reference_vectors.npz", **vectors)

    # Published calibration rows (read, not recomputed).
    rows = []
    with open(CALIBRATION_CSV) as fh:
        for r in csv.DictReader(fh):
            if r["problem"] != "bratu" or r["repetition"] != "1":
                continue
            rows.append({k: r[k] for k in (
                "n", "param", "method", "precond", "internal_candidate_id", "success", "nonlinear_iters",
                "n_F", "n_JVP", "n_D2", "n_lin", "n_lin_failures", "n_prec", "residual_rel", "rtol",
                "max_nl", "eta_init", "eta_max", "gamma", "alpha", "eta2_factor", "eta2_max", "restart",
                "maxlin", "t_total", "threads")})
    (HERE / "c1_bratu_jacobi.json").write_text(json.dumps(rows, indent=0))
    brows = []
    with open(CALIBRATION_CSV) as fh:
        for r in csv.DictReader(fh):
            if r["problem"] != "burgers" or r["repetition"] != "1":
                continue
            kv = dict(item.split("=") for item in r["instance_id"].split(";"))
            brows.append(dict({k: r[k] for k in (
                "n", "param", "method", "precond", "internal_candidate_id", "success", "nonlinear_iters", "n_F",
                "n_JVP", "n_D2", "n_lin", "n_lin_failures", "n_prec", "residual_rel", "rtol", "max_nl", "eta_init",
                "eta_max", "gamma", "alpha", "eta2_factor", "eta2_max", "restart", "maxlin")},
                dt=kv["dt"], amp=kv["amp"]))
    (HERE / "c1_burgers_mg.json").write_text(json.dumps(brows, indent=0))
    with open(CALIBRATION_CSV) as fh:
        (HERE / "c1_csv_header.txt").write_text(fh.readline())
    print(len(out_counts), "solves,", len(vectors), "vectors,", len(rows), "calibration rows")


def brusselator_main() -> None:
    """Brusselator1DStep / BrusselatorJacobi (problems/brusselator1d.hpp) fixtures:

    * ``reference_brusselator.npz`` — the previous state, F, J v, F'' (analytic and finite
      difference) and a BrusselatorJacobi application on the reference test's point
      (tests/test_brusselator.cpp:13-19, :37-53), n = 31, dt = 0.01;
    * ``reference_brusselator.json`` — every method with and without BrusselatorJacobi from the
      previous state at n = 31, dt = 0.01, rtol 1e-9, GMRES(30), 200 iterations (the test's
      configuration, :55-67), and at n = 127, dt = 0.016 with the calibration campaign's parameters;
    * ``c1_brusselator_jacobi.json`` — the reference's published Brusselator calibration rows
      (experiments/c1/amendment01/calibration_combined.csv, repetition 1), read, not recomputed.
    """
    build_ref(force=True)
    ref = Oracle.reference()
    n, dt = 31, 0.01
    prev = ref.bruss1d_previous(n, dt)
    idx = np.arange(2 * n, dtype=np.float64)
    x = prev + 0.05 * np.sin(0.31 * idx + 0.4)
    d = 0.4 * np.sin(0.31 * idx + 1.2)
    vec = {"prev": prev, "x": x, "d": d, "eval_prev": ref.bruss1d_eval(n, dt, prev), "eval_x": ref.bruss1d_eval(n, dt, x)}
    for mode, tag in ((0, ""), (1, "_fd")):
        vec[f"jvp{tag}"] = ref.bruss1d_jvp(n, dt, x, d, mode)
        vec[f"d2{tag}"] = ref.bruss1d_d2(n, dt, x, d, mode)
    vec["jacobi_x_d"] = ref.bruss1d_jacobi_apply(n, dt, x, d)
    solves = []
    cases = [(31, 0.01, default_params(rtol_nl=1e-9, gmres_restart=30, gmres_max_iters=200), "test"),
             (127, 0.016, default_params(rtol_nl=1e-8, eta_init=0.25, gmres_restart=30, gmres_max_iters=200),
              "calibration")]
    for cn, cdt, p, tag in cases:
        for method in ("nk", "cheb", "rec", "tf2018"):
            for precond in ("jacobi", "none"):
                xs, res = ref.solve_bruss1d(cn, cdt, method, precond, p)
                solves.append(dict(tag=tag, n=cn, dt=cdt, method=method, precond=precond, params=params_dict(p),
                                   result={k: res[k] for k in ("converged", "iters", "n_F", "n_JVP", "n_D2",
                                                               "n_lin_iters", "n_lin_failures", "n_prec", "res0",
                                                               "res")},
                                   solution=solution_stats(xs)))
                if precond == "jacobi":
                    vec[f"x_{tag}_{method}"] = xs
    (HERE / "reference_brusselator.json").write_text(json.dumps({"solves": solves}, indent=1))
    np.savez_compressed(HERE / "reference_brusselator.npz", **vec)
    rows = []
    with open(CALIBRATION_CSV) as fh:
        for r in csv.DictReader(fh):
            if r["problem"] != "brusselator" or r["repetition"] != "1":
                continue
            rows.append({k: r[k] for k in (
                "n", "param", "method", "precond", "internal_candidate_id", "success", "nonlinear_iters", "n_F",
                "n_JVP", "n_D2", "n_lin", "n_lin_failures", "n_prec", "residual_rel", "rtol", "max_nl", "eta_init",
                "eta_max", "gamma", "alpha", "eta2_factor", "eta2_max", "restart", "maxlin")})
    (HERE / "c1_brusselator_jacobi.json").write_text(json.dumps(rows, indent=0))
    print(len(solves), "Brusselator solves,", len(vec), "vectors,", len(rows), "calibration rows")


def strided_sample(N: int, target: int) -> np.ndarray:
    """Deterministic sample indices of an N-vector: every stride-th point from stride/2, stride odd
    and about N/target (an odd stride does not alias with the power-of-two-plus-one grid lines)."""
    stride = max(1, N // target) | 1
    return np.arange(stride // 2, N, stride, dtype=np.int64)


def large_main() -> None:
    """Fixtures at the sizes the benchmark runs (the reference's headers compiled here, one thread):

    * ``reference_large.json`` / ``reference_large.npz`` — Bratu3D lambda = 6, u0 = 0, rtol 1e-10,
      GMRES(30), PoissonMG V(2,2) on the full hierarchy: at 255^3 Newton-Krylov, inexact Chebyshev
      and Chebyshev with Krylov recycling; at 127^3 Newton-Krylov and inexact Chebyshev.  Counts,
      residuals, solution statistics and a strided sample of ~16k solution values with its indices;
    * ``reference_batch.json`` / ``reference_batch.npz`` — every instance of the batched
      configuration (128 instances, n from {31, 63, 127}, lambda ~ U[1, 6.5], numpy PCG64 seed 42;
      numa_gpu.batch_config_instances), each solved alone by Newton-Krylov with the same settings,
      as the reference's campaign runner loops over instances (apps/run_campaign.cpp:344-475):
      counts, residuals, statistics and a strided sample of ~512 values per instance.
    """
    sys.path.insert(0, str(ROOT / "chebyshev-nonlinear-lab_gb300"))
    from numa_gpu import batch_config_instances
    if build_ref() is None:
        raise SystemExit("reference headers not found")
    ref = Oracle.reference()
    north = dict(rtol_nl=1e-10, gmres_restart=30)
    keys = ("converged", "iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_lin_failures", "n_prec", "res0", "res")
    large, lvec = [], {}
    for n, methods in ((127, ("nk", "cheb")), (255, ("nk", "cheb", "rec"))):
        N = n ** 3
        idx = strided_sample(N, 16384)
        lvec[f"idx_n{n}"] = idx
        for method in methods:
            p = default_params(**north)
            x, res = ref.solve(n, 6.0, method, "mg", p)
            large.append(dict(n=n, lam=6.0, method=method, precond="mg", params=params_dict(p),
                              result={k: res[k] for k in keys}, solution=solution_stats(x)))
            lvec[f"x_n{n}_{method}"] = x[idx]
            print("large", n, method, res["iters"], res["n_JVP"], res["n_prec"], flush=True)
    (HERE / "reference_large.json").write_text(json.dumps(large, indent=1))
    np.savez_compressed(HERE / "reference_large.npz", **lvec)

    inst = batch_config_instances()
    batch, bvec = [], {}
    for i, (n, lam) in enumerate(inst):
        p = default_params(**north)
        x, res = ref.solve(n, lam, "nk", "mg", p)
        idx = strided_sample(n ** 3, 512)
        batch.append(dict(index=i, n=n, lam=lam, method="nk", precond="mg", result={k: res[k] for k in keys},
                          solution=solution_stats(x), sample_count=int(idx.size)))
        bvec[f"x_{i}"] = x[idx]
        print("batch", i, n, round(lam, 4), res["iters"], res["n_JVP"], res["n_prec"], flush=True)
    (HERE / "reference_batch.json").write_text(json.dumps({"seed": 42, "params": params_dict(default_params(**north)),
                                                           "instances": batch}, indent=1))
    np.savez_compressed(HERE / "reference_batch.npz", **bvec)


if __name__ == "__main__":
    if os.environ.get("OMP_NUM_THREADS") != "1":
        raise SystemExit("run with OMP_NUM_THREADS=1")
    if "--large" in sys.argv:
        large_main()
    elif "--brusselator" in sys.argv:
        brusselator_main()
    else:
        main()
        brusselator_main()
