"""run_campaign_gpu: the reference's campaign command line and raw CSV schema
(apps/run_campaign.cpp, instrument/csv.hpp) on the GPU path."""
from __future__ import annotations

import csv
import subprocess

import pytest

from conftest import GOLDEN, PKG


@pytest.fixture(scope="module")
def app(lib_path):
    import build
    return build.build_apps()[0]


def test_csv_schema_is_the_references(app):
    ours = subprocess.run([str(app), "--print-header"], capture_output=True, text=True, check=True).stdout.strip()
    published = (GOLDEN / "c1_csv_header.txt").read_text().strip().split(",")
    # the published calibration file carries two columns appended by a later tool
    assert ours.split(",") == published[:-2]
    assert len(ours.split(",")) == 43


def test_bad_arguments_exit_2(app):
    assert subprocess.run([str(app), "--n"], capture_output=True).returncode == 2
    assert subprocess.run([str(app), "--phase", "calibration", "--out", "x.csv"], capture_output=True).returncode == 2
    assert subprocess.run([str(app), "--problem", "chandra", "--out", "x.csv", "--commit", "c"],
                          capture_output=True).returncode == 2


@pytest.mark.gpu
def test_calibration_rows_on_gpu(app, tmp_path, c1_rows):
    """Published calibration runs (Bratu3D 31^3, Jacobi, tuning candidate t01) through the GPU
    campaign runner: one CSV row per method with the published counts."""
    rows = [r for r in c1_rows if r["n"] == "31" and r["internal_candidate_id"] == "t01"]
    lambdas = sorted({r["param"] for r in rows})[:3]
    out = tmp_path / "calib.csv"
    for lam in lambdas:
        r0 = next(r for r in rows if r["param"] == lam)
        cmd = [str(app), "--phase", "calibration", "--problem", "bratu", "--n", "31", "--param", lam,
               "--precond", "jacobi", "--methods", "nk,cheb,rec", "--start", "natural", "--warmup", "0",
               "--reps", "1", "--rtol", r0["rtol"], "--eta-init", r0["eta_init"], "--restart", r0["restart"],
               "--maxlin", r0["maxlin"], "--out", str(out), "--commit", "test"]
        res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        assert res.returncode == 0, res.stderr
    got = list(csv.DictReader(open(out)))
    assert len(got) == 3 * len(lambdas)
    for g in got:
        want = next(r for r in rows if r["method"] == g["method"] and float(r["param"]) == float(g["param"]))
        for k in ("success", "nonlinear_iters", "n_F", "n_D2"):
            assert int(g[k]) == int(want[k]), (g["param"], g["method"], k)
        for k in ("n_JVP", "n_lin", "n_prec"):
            assert abs(int(g[k]) - int(want[k])) <= max(3, 0.02 * int(want[k])), (g["param"], g["method"], k)
        assert float(g["t_total"]) > 0 and float(g["t_prec"]) > 0
